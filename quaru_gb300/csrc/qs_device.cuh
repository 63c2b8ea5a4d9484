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

// Exact float -> double conversion with integer operations (floats below
// 2^-126 flush to zero).
__device__ __forceinline__ double df_f2d(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t mag = b & 0x7fffffffu;
    const uint32_t hi = ((mag >> 3) + (896u << 20)) | (b & 0x80000000u);
    return (mag >= 0x00800000u) ? __hiloint2double(int(hi), int(b << 29)) : 0.0;
}

// double -> float rounded to nearest even with integer operations, for values whose float lies in
// the normal range (|v| >= 2^-126 and finite; smaller values give zero, larger ones infinity).
__device__ __forceinline__ float d2f_int(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
    const int e = int((b >> 52) & 0x7ffu) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
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
