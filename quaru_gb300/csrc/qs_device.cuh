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
