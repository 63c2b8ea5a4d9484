// qs_rot.cuh — rotation arithmetic shared by the adjoint kernels and the batch kernel:
// R_A(theta) = cos(theta/2) I - i sin(theta/2) A on an amplitude pair, the per-pair term of
// Im<lambda|A|psi>, and their double-float forms (FP32 pipe) for complex128 state.
#pragma once

#include <cuda_runtime.h>

#include "qs_device.cuh"
#include "qs_reduce.cuh"

namespace qs {

// ---------------------------------------------------------------- rotations
// R_A(theta) = cos(theta/2) I - i sin(theta/2) A on the pair (a, b) = (bit 0, bit 1).
template <int AXIS, typename R>
__device__ __forceinline__ void rot_pair(R c, R s, R& ax, R& ay, R& bx, R& by) {
    if (AXIS == QS_GATE_RY) {  // [[c, -s], [s, c]]
        const R nax = c * ax - s * bx, nay = c * ay - s * by;
        const R nbx = s * ax + c * bx, nby = s * ay + c * by;
        ax = nax; ay = nay; bx = nbx; by = nby;
    } else if (AXIS == QS_GATE_RZ) {  // diag(c - i s, c + i s)
        const R nax = c * ax + s * ay, nay = c * ay - s * ax;
        const R nbx = c * bx - s * by, nby = c * by + s * bx;
        ax = nax; ay = nay; bx = nbx; by = nby;
    } else {  // RX: [[c, -i s], [-i s, c]]
        const R nax = c * ax + s * by, nay = c * ay - s * bx;
        const R nbx = c * bx + s * ay, nby = c * by - s * ax;
        ax = nax; ay = nay; bx = nbx; by = nby;
    }
}

// The term of Im<lambda|A|psi> from one pair (rows with the target bit 0: a, l0; 1: b, l1).
template <int AXIS>
__device__ __forceinline__ double im_term(double2 l0, double2 l1, double2 a, double2 b) {
    if (AXIS == QS_GATE_RX) return (l0.x * b.y - l0.y * b.x) + (l1.x * a.y - l1.y * a.x);
    if (AXIS == QS_GATE_RY) return (l1.x * a.x + l1.y * a.y) - (l0.x * b.x + l0.y * b.y);
    return (l0.x * a.y - l0.y * a.x) - (l1.x * b.y - l1.y * b.x);
}

// complex64: the pair's four products summed by an FMA chain (one float rounding per product), the
// pair sums then accumulated with TwoSum compensation, so the sum over a tile carries no FP32 drift.
template <int AXIS>
__device__ __forceinline__ void im_term_acc(DfAcc& acc, float2 l0, float2 l1, float2 a, float2 b) {
    float t;
    if (AXIS == QS_GATE_RX)
        t = __fmaf_rn(l0.x, b.y, __fmaf_rn(-l0.y, b.x, __fmaf_rn(l1.x, a.y, __fmul_rn(-l1.y, a.x))));
    else if (AXIS == QS_GATE_RY)
        t = __fmaf_rn(l1.x, a.x, __fmaf_rn(l1.y, a.y, __fmaf_rn(-l0.x, b.x, __fmul_rn(-l0.y, b.y))));
    else
        t = __fmaf_rn(l0.x, a.y, __fmaf_rn(-l0.y, a.x, __fmaf_rn(-l1.x, b.y, __fmul_rn(l1.y, b.x))));
    acc.add(t);
}

// ---- double-float forms. Amplitudes as float4 (re_hi, re_lo, im_hi, im_lo); each pair's
// Im<lambda|A|psi> is a double-float dot product (df_dot_pair), added to a compensated float-pair
// accumulator: no FP64 operation per pair.
template <int AXIS>
__device__ __forceinline__ void adj_im_df_acc(DfAcc& acc, float4 l0, float4 l1, float4 a, float4 b) {
    // terms u * x of Im<lambda|A|psi> (see im_term): u from lambda, x from psi
    float uh[4], ul[4], xh[4], xl[4];
    auto set = [&](int k, float vh, float vl, float wh, float wl, bool neg) {
        uh[k] = neg ? -vh : vh;
        ul[k] = neg ? -vl : vl;
        xh[k] = wh;
        xl[k] = wl;
    };
    if (AXIS == QS_GATE_RX) {  // l0.re*b.im - l0.im*b.re + l1.re*a.im - l1.im*a.re
        set(0, l0.x, l0.y, b.z, b.w, false); set(1, l0.z, l0.w, b.x, b.y, true);
        set(2, l1.x, l1.y, a.z, a.w, false); set(3, l1.z, l1.w, a.x, a.y, true);
    } else if (AXIS == QS_GATE_RY) {  // l1.re*a.re + l1.im*a.im - l0.re*b.re - l0.im*b.im
        set(0, l1.x, l1.y, a.x, a.y, false); set(1, l1.z, l1.w, a.z, a.w, false);
        set(2, l0.x, l0.y, b.x, b.y, true); set(3, l0.z, l0.w, b.z, b.w, true);
    } else {  // l0.re*a.im - l0.im*a.re - l1.re*b.im + l1.im*b.re
        set(0, l0.x, l0.y, a.z, a.w, false); set(1, l0.z, l0.w, a.x, a.y, true);
        set(2, l1.x, l1.y, b.z, b.w, true); set(3, l1.z, l1.w, b.x, b.y, false);
    }
    float h, l;
    df_dot_pair<4>(uh, ul, xh, xl, h, l);
    acc.add(h);
    acc.c = __fadd_rn(acc.c, l);
}

// c * p + q2 * r in double-float: the rot_pair formulas with (c, s) = (ch + cl, sh + sl).
__device__ __forceinline__ void df_lin2(float ch, float cl, float p_h, float p_l, float dh, float dl, float q_h,
                                        float q_l, float& oh, float& ol) {
    const float uh[2] = {ch, dh}, ul[2] = {cl, dl}, xh[2] = {p_h, q_h}, xl[2] = {p_l, q_l};
    df_dot_pair<2>(uh, ul, xh, xl, oh, ol);
}

template <int AXIS>
__device__ __forceinline__ void df_rot_pair(float ch, float cl, float sh, float sl, float4& a, float4& b) {
    float4 na, nb;
    if (AXIS == QS_GATE_RY) {  // [[c, -s], [s, c]]
        df_lin2(ch, cl, a.x, a.y, -sh, -sl, b.x, b.y, na.x, na.y);
        df_lin2(ch, cl, a.z, a.w, -sh, -sl, b.z, b.w, na.z, na.w);
        df_lin2(sh, sl, a.x, a.y, ch, cl, b.x, b.y, nb.x, nb.y);
        df_lin2(sh, sl, a.z, a.w, ch, cl, b.z, b.w, nb.z, nb.w);
    } else if (AXIS == QS_GATE_RZ) {  // diag(c - i s, c + i s)
        df_lin2(ch, cl, a.x, a.y, sh, sl, a.z, a.w, na.x, na.y);
        df_lin2(ch, cl, a.z, a.w, -sh, -sl, a.x, a.y, na.z, na.w);
        df_lin2(ch, cl, b.x, b.y, -sh, -sl, b.z, b.w, nb.x, nb.y);
        df_lin2(ch, cl, b.z, b.w, sh, sl, b.x, b.y, nb.z, nb.w);
    } else {  // RX: [[c, -i s], [-i s, c]]
        df_lin2(ch, cl, a.x, a.y, sh, sl, b.z, b.w, na.x, na.y);
        df_lin2(ch, cl, a.z, a.w, -sh, -sl, b.x, b.y, na.z, na.w);
        df_lin2(ch, cl, b.x, b.y, sh, sl, a.z, a.w, nb.x, nb.y);
        df_lin2(ch, cl, b.z, b.w, -sh, -sl, a.x, a.y, nb.z, nb.w);
    }
    a = na;
    b = nb;
}

}  // namespace qs
