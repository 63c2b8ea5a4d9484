// qs_device.cuh — device-side helpers shared by the engine's kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace qs {

template <typename R>
struct Cplx;
template <>
struct Cplx<double> {
    using T = double2;
};
template <>
struct Cplx<float> {
    using T = float2;
};

// Maps a tuple index t (the free bits of an amplitude index, packed) to the
// base amplitude index: zero bits are inserted at the sorted positions of the
// gate's targets and fixed bits, then the fixed bits' values are ORed in.
struct IndexMap {
    uint64_t fixval;
    int npos;
    uint8_t pos[64];
};

__device__ __forceinline__ uint64_t expand_index(uint64_t t, const IndexMap& m) {
    for (int i = 0; i < m.npos; i++) {
        const uint32_t p = m.pos[i];
        const uint64_t lo = t & ((1ull << p) - 1ull);
        t = ((t >> p) << (p + 1)) | lo;
    }
    return t | m.fixval;
}

// ---- arithmetic in the reference's order --------------------------------
// num-complex Complex<f64> multiply, (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re),
// rounded after every operation; the _rn intrinsics are never contracted into FMAs.
__device__ __forceinline__ double2 cmul_exact(double ur, double ui, double2 x) {
    double2 r;
    r.x = __dsub_rn(__dmul_rn(ur, x.x), __dmul_rn(ui, x.y));
    r.y = __dadd_rn(__dmul_rn(ur, x.y), __dmul_rn(ui, x.x));
    return r;
}
// Same product for a matrix entry whose imaginary part is +-0: the terms
// ui*x are +-0 and do not change the value.
__device__ __forceinline__ double2 cmul_exact_real(double ur, double2 x) {
    double2 r;
    r.x = __dmul_rn(ur, x.x);
    r.y = __dmul_rn(ur, x.y);
    return r;
}
__device__ __forceinline__ double2 cadd_exact(double2 a, double2 b) {
    return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}

// ---- fused multiply-add arithmetic ---------------------------------------
__device__ __forceinline__ double2 cfma(double ur, double ui, double2 x, double2 acc) {
    acc.x = fma(ur, x.x, fma(-ui, x.y, acc.x));
    acc.y = fma(ur, x.y, fma(ui, x.x, acc.y));
    return acc;
}
__device__ __forceinline__ float2 cfma(float ur, float ui, float2 x, float2 acc) {
    acc.x = fmaf(ur, x.x, fmaf(-ui, x.y, acc.x));
    acc.y = fmaf(ur, x.y, fmaf(ui, x.x, acc.y));
    return acc;
}
__device__ __forceinline__ double2 cfma_real(double ur, double2 x, double2 acc) {
    acc.x = fma(ur, x.x, acc.x);
    acc.y = fma(ur, x.y, acc.y);
    return acc;
}
__device__ __forceinline__ float2 cfma_real(float ur, float2 x, float2 acc) {
    acc.x = fmaf(ur, x.x, acc.x);
    acc.y = fmaf(ur, x.y, acc.y);
    return acc;
}

template <typename T>
__device__ __forceinline__ T czero();
template <>
__device__ __forceinline__ double2 czero<double2>() {
    return make_double2(0.0, 0.0);
}
template <>
__device__ __forceinline__ float2 czero<float2>() {
    return make_float2(0.0f, 0.0f);
}

// Value-exact multiplication by 1, -1, i, -i (PfClass 0..3): a move plus sign
// flips, equal in value to the reference's complex product with that entry.
template <typename T>
__device__ __forceinline__ T apply_pf(T x, uint8_t cls) {
    T r = x;
    if (cls == 1) {
        r.x = -x.x;
        r.y = -x.y;
    } else if (cls == 2) {
        r.x = -x.y;
        r.y = x.x;
    } else if (cls == 3) {
        r.x = x.y;
        r.y = -x.x;
    }
    return r;
}

}  // namespace qs

namespace qs {

// ---- double-float arithmetic on the FP32 pipe (QS_ARITH_DF64) ------------
// GB300's FP64 rate (~2 FMA/clk/SM) cannot keep up with HBM for dense gates;
// its FP32 rate can. A double x is carried as floats (h, l) with
// x = h + l + d, |d| <= 2^-47 |x|; sums of products use Dekker/Knuth
// error-free transformations (TwoProduct by FMA, TwoSum), and the result is
// rejoined by one FP64 addition. Valid for 2^-126 <= |x| < 2^128; smaller
// magnitudes are flushed (absolute error < 2^-74 |x|... below 2^-126).

// Split with integer operations only: h is x with its significand truncated
// to 24 bits, l is the remaining 29 bits rounded to 24 bits.
__device__ __forceinline__ void df_split(double x, float& h, float& l) {
    const uint32_t hi = uint32_t(__double2hiint(x)), lo = uint32_t(__double2loint(x));
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t hb = ((__funnelshift_l(lo, hi, 3) - 0xC0000000u) & 0x7fffffffu) | sign;
    const uint32_t sb = (e * 0x800000u - 948u * 0x800000u) | sign;  // +-2^(e-1075), for e >= 949
    const float lf = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu), __uint_as_float(sb));
    h = (e >= 897u) ? __uint_as_float(hb) : 0.0f;
    l = (e >= 949u) ? lf : 0.0f;
}

// Exact float -> double conversion with integer operations for normal floats (the common case);
// zeros keep their sign, and subnormal, infinite and NaN floats take a rare branch through the
// hardware conversion, which is exact as well.
__device__ __forceinline__ double df_f2d(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t mag = b & 0x7fffffffu;
    if (mag - 0x00800000u < 0x7f000000u) {  // normal: 2^-126 <= |f| < inf
        const uint32_t hi = ((mag >> 3) + (896u << 20)) | (b & 0x80000000u);
        return __hiloint2double(int(hi), int(b << 29));
    }
    if (mag == 0u) return __hiloint2double(int(b & 0x80000000u), 0);
    return double(f);
}

// double -> float rounded to nearest even with integer operations when the float lies in the normal
// range (the common case); results in the subnormal range, zeros, overflows, infinities and NaNs
// take a rare branch through the hardware conversion, which rounds the same way.
__device__ __forceinline__ float d2f_int(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
    const int e = int((b >> 52) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 255) return __double2float_rn(v);
    const unsigned long long m = b & 0xfffffffffffffull;
    uint32_t r = (uint32_t(e) << 23) | uint32_t(m >> 29);
    const uint32_t rest = uint32_t(m & 0x1fffffffull);  // the 29 dropped bits
    if (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) r += 1u;  // a carry may bump the exponent
    return __uint_as_float(sign | r);
}

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// sum_{k<NT} (uh_k + ul_k) * (xh_k + xl_k), returned as a double.
template <int NT>
__device__ __forceinline__ double df_dot(const float* uh, const float* ul, const float* xh, const float* xl) {
    float p[NT];
    float c = 0.0f;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        p[k] = __fmul_rn(uh[k], xh[k]);
        c = __fadd_rn(c, __fmaf_rn(uh[k], xh[k], -p[k]));
        c = __fmaf_rn(uh[k], xl[k], c);
        c = __fmaf_rn(ul[k], xh[k], c);
    }
    float s = p[0];
#pragma unroll
    for (int k = 1; k < NT; k++) {
        float t;
        df_two_sum(s, p[k], s, t);
        c = __fadd_rn(c, t);
    }
    return __dadd_rn(df_f2d(s), df_f2d(c));
}

}  // namespace qs

namespace qs {

// As df_dot, but returns the sum as a normalised float pair (h, l) (TwoSum).
template <int NT>
__device__ __forceinline__ void df_dot_pair(const float* uh, const float* ul, const float* xh, const float* xl,
                                            float& h, float& l) {
    float p[NT];
    float c = 0.0f;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        p[k] = __fmul_rn(uh[k], xh[k]);
        c = __fadd_rn(c, __fmaf_rn(uh[k], xh[k], -p[k]));
        c = __fmaf_rn(uh[k], xl[k], c);
        c = __fmaf_rn(ul[k], xh[k], c);
    }
    float s = p[0];
#pragma unroll
    for (int k = 1; k < NT; k++) {
        float t;
        df_two_sum(s, p[k], s, t);
        c = __fadd_rn(c, t);
    }
    df_two_sum(s, c, h, l);
}

}  // namespace qs

namespace qs {

// ---- FP64-accurate fixed-point dot products on the integer pipes (QS_ARITH_FX64) -------------
// A dense gate's output component is S = sum_t c_t v_t over a tuple of amplitude components v_t.
// GB300's FP64 pipe (~2 FMA/clk/SM) caps such sweeps near a third of HBM bandwidth, so this form
// computes S with integer multiply-adds instead and rounds it once to double:
//  * every v_t of the tuple becomes V_t = sign(v_t) * trunc(|v_t| * 2^(1082 - E)), E = the tuple's
//    largest exponent field, so the largest |v| fills bits 52..59 and |V_t| < 2^60; its limbs carry
//    the sign: Vh = sign * (|V| >> 30), Vl = sign * (|V| & (2^30 - 1)), so |Vh| <= 2^30, |Vl| < 2^30;
//  * every coefficient c_t of the row becomes C_t = RN(c_t * 2^(60 - ec)) on the host (ec: frexp
//    exponent of the row's largest |c|), |C_t| < 2^60, in balanced limbs C = Ch * 2^30 + Cl with
//    Cl in [-2^29, 2^29), |Ch| <= 2^30;
//  * A = sum Vh*Ch (|A| <= 2^62) and B = sum (Vh*Cl + Vl*Ch) (|B| < 3 * 2^61) are exact in 64-bit
//    integers for up to 4 terms per output; R = A + (B >> 30) approximates sum V*C / 2^60 and
//    S = R * 2^(E + ec - 1082) is rounded once to double.
// The truncations (B >> 30, the dropped Vl*Cl, V_t, C_t) cost less than 9 units of R, so
// |S_computed - S| <= ulp(S)/2 + 2^-54 * max|v_t| * max|c_t|; an FP64 FMA chain over the same
// four terms has a worst case of about 2^-51 * max|v_t| * max|c_t|.

// Exponent field of a double (0 for zeros and subnormals).
__device__ __forceinline__ uint32_t fx_efield(double x) { return (uint32_t(__double2hiint(x)) >> 20) & 0x7ffu; }

// Tuples whose largest exponent field is at least this take the fast encoding; smaller ones (every
// component below 2^-958) take fx_encode_small.
constexpr uint32_t kFxMinE = 65u;

// d = E - (exponent field of v) >= 0 and the significand with its implicit bit, shifted so that a
// component with d = 0 has its leading bit at 59: V = (m << 7) >> d in sign-carrying 30-bit limbs.
// Zeros and subnormals (exponent field 0) have d = E >= 65 and come out as 0 whatever their
// significand, so the implicit bit is set unconditionally.
__device__ __forceinline__ void fx_encode(double v, uint32_t E, int32_t& h, int32_t& l) {
    const uint32_t hi = uint32_t(__double2hiint(v)), lo = uint32_t(__double2loint(v));
    const uint32_t d = E - ((hi >> 20) & 0x7ffu);
    const uint32_t mh = (hi & 0xfffffu) | 0x100000u;  // 21 significand bits
    const uint32_t h7 = __funnelshift_l(lo, mh, 7), l7 = lo << 7;  // m << 7 = (h7:l7) < 2^60
    uint32_t vl, vh;
    if (d < 32u) {
        vl = __funnelshift_r(l7, h7, d);
        vh = h7 >> d;
    } else {
        vl = d < 64u ? (h7 >> (d - 32u)) : 0u;
        vh = 0u;
    }
    const int32_t sgn = (int32_t(hi) >> 31) | 1;  // -1 or +1
    h = int32_t(__funnelshift_r(vl, vh, 30)) * sgn;  // |V| >> 30 fits in 30 bits
    l = int32_t(vl & 0x3fffffffu) * sgn;
}

// The same for tuples below 2^-958 (E < kFxMinE; E = 0 for an all-zero tuple): subnormals have
// scale exponent 1 and no implicit bit.
__device__ __forceinline__ void fx_encode_small(double v, uint32_t E, int32_t& h, int32_t& l) {
    const uint32_t hi = uint32_t(__double2hiint(v)), lo = uint32_t(__double2loint(v));
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const uint32_t ee = e > 1u ? e : 1u, EE = E > 1u ? E : 1u;
    const uint32_t hm = (hi & 0xfffffu) | (e != 0u ? 0x100000u : 0u);
    const uint64_t m = ((uint64_t(hm) << 32) | lo) << 7;
    const uint32_t d = EE - ee;
    const uint64_t V = d < 64u ? (m >> d) : 0ull;
    const int32_t sgn = (int32_t(hi) >> 31) | 1;
    h = int32_t(uint32_t(V >> 30)) * sgn;
    l = int32_t(uint32_t(V) & 0x3fffffffu) * sgn;
}

// a * b + c for 32-bit a, b and a 64-bit c, as one wide multiply-add.
__device__ __forceinline__ long long fx_mad(int32_t a, int32_t b, long long c) {
    long long d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// R = sum V*C / 2^60 of one output row: A + (B >> 30).
template <int NT>
__device__ __forceinline__ long long fx_row_sum(const int32_t* vh, const int32_t* vl, const int32_t* ch,
                                                const int32_t* cl) {
    static_assert(NT <= 4, "64-bit accumulators are exact for at most 4 terms");
    long long A = 0, B = 0;
#pragma unroll
    for (int t = 0; t < NT; t++) {
        A = fx_mad(vh[t], ch[t], A);
        B = fx_mad(vh[t], cl[t], B);
        B = fx_mad(vl[t], ch[t], B);
    }
    return A + (B >> 30);
}

// R * 2^k rounded to nearest double, any R (|R| < 2^63) and k: the conversion rounds R once, scalbn
// scales exactly unless the result leaves the normal range.
static __device__ __noinline__ double fx_to_double_any(long long R, int k) {
    return R == 0 ? 0.0 : scalbn(__ll2double_rn(R), k);
}

// R * 2^k for k in [kFxFastKMin, kFxFastKMax]: every non-zero |R| < 2^63 converts to an exponent
// field in [1023, 1086], which stays normal after adding k, so the power of two goes straight
// into the exponent field (kk = k << 20).
constexpr int kFxFastKMin = -1022, kFxFastKMax = 960;
__device__ __forceinline__ double fx_to_double_fast(long long R, int kk) {
    const double d = __ll2double_rn(R);
    const double s = __hiloint2double(__double2hiint(d) + kk, __double2loint(d));
    return R == 0 ? 0.0 : s;
}

// sum_{t<NT} c_t v_t for one output row in the general case (rare tuples: tiny, or with output
// exponents outside the fast range): limbs at exponent E, row limbs ch/cl, k0 = ec - 1082.
template <int NT>
__device__ __forceinline__ double fx_dot(const int32_t* vh, const int32_t* vl, const int32_t* ch,
                                         const int32_t* cl, uint32_t E, int k0) {
    return fx_to_double_any(fx_row_sum<NT>(vh, vl, ch, cl), int(E > 1u ? E : 1u) + k0);
}

}  // namespace qs
