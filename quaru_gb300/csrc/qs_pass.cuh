// qs_pass.cuh — register passes over a complex64 tile in shared memory.
//
// A pass holds 16 amplitudes per thread. Register j holds the amplitude at tuple base + off[j], off[j]
// depositing the bits of j on the pass's four register bits (tile bits >= 4); tile bits 0..3 are lane
// bits 0..3 of the warp, so a gate on one of them pairs a thread's register with the same register
// of lane ^ (1 << t) (a shuffle); the remaining tile bits select the thread's tuple. Every member
// arrives with a variant id computed on the host (qs_plan.cpp) that selects fully specialised code:
// one dispatch per member, no decoding of gate fields in the kernel.
#pragma once

#include <cuda_runtime.h>

#include "qs_device.cuh"
#include "qs_tile.h"

namespace qs {

__device__ __forceinline__ float2 pcmul(float ur, float ui, float2 x) {
    return make_float2(fmaf(ur, x.x, -ui * x.y), fmaf(ur, x.y, ui * x.x));
}

// Dense 2x2 on register bit J (rows a, a | 1 << J), optionally only where (a & fm) == fv.
template <int J, bool ALL>
__device__ __forceinline__ void pv_dense(const float* u, int fm, int fv, float2 (&x)[16]) {
    const float4 c0 = *reinterpret_cast<const float4*>(u), c1 = *reinterpret_cast<const float4*>(u + 4);
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if (a & (1 << J)) continue;
        if (!ALL && ((a & fm) != fv)) continue;
        const int b = a | (1 << J);
        const float2 xa = x[a], xb = x[b];
        float2 y0 = cfma(c0.z, c0.w, xb, czero<float2>());
        y0 = cfma(c0.x, c0.y, xa, y0);
        float2 y1 = cfma(c1.z, c1.w, xb, czero<float2>());
        y1 = cfma(c1.x, c1.y, xa, y1);
        x[a] = y0;
        x[b] = y1;
    }
}

template <int J, bool ALL>
__device__ __forceinline__ void pv_real(const float* u, int fm, int fv, float2 (&x)[16]) {
    const float4 c = *reinterpret_cast<const float4*>(u);
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if (a & (1 << J)) continue;
        if (!ALL && ((a & fm) != fv)) continue;
        const int b = a | (1 << J);
        const float2 xa = x[a], xb = x[b];
        x[a] = make_float2(fmaf(c.x, xa.x, c.y * xb.x), fmaf(c.x, xa.y, c.y * xb.y));
        x[b] = make_float2(fmaf(c.z, xa.x, c.w * xb.x), fmaf(c.z, xa.y, c.w * xb.y));
    }
}

// CODE: PC_SWAP (rows exchanged), PC_SWAPPH (exchanged, times the rows' factors), PC_DIAG2 (rows
// times their factors).
template <int J, int CODE, bool ALL>
__device__ __forceinline__ void pv_mono(const float* u, int fm, int fv, float2 (&x)[16]) {
    float4 p = make_float4(1.f, 0.f, 1.f, 0.f);
    if (CODE != PC_SWAP) p = *reinterpret_cast<const float4*>(u);
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if (a & (1 << J)) continue;
        if (!ALL && ((a & fm) != fv)) continue;
        const int b = a | (1 << J);
        const float2 xa = x[a], xb = x[b];
        if (CODE == PC_SWAP) {
            x[a] = xb;
            x[b] = xa;
        } else if (CODE == PC_SWAPPH) {
            x[a] = pcmul(p.x, p.y, xb);
            x[b] = pcmul(p.z, p.w, xa);
        } else {
            x[a] = pcmul(p.x, p.y, xa);
            x[b] = pcmul(p.z, p.w, xb);
        }
    }
}

// Swap on register bit J where register bit C is 1 (CNOT with both qubits in registers).
template <int J, int C>
__device__ __forceinline__ void pv_swapc(float2 (&x)[16]) {
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if ((a & (1 << J)) || !(a & (1 << C))) continue;
        const int b = a | (1 << J);
        const float2 t = x[a];
        x[a] = x[b];
        x[b] = t;
    }
}

// Dense gates on the register bits of mask M, in increasing bit order; their coefficients are the
// u of consecutive entries starting at m.
template <int M>
__device__ __forceinline__ void pv_multi(const TileOp* m, float2 (&x)[16]) {
    int e = 0;
    if (M & 1) pv_dense<0, true>(m[e++].pm.u, 0, 0, x);
    if (M & 2) pv_dense<1, true>(m[e++].pm.u, 0, 0, x);
    if (M & 4) pv_dense<2, true>(m[e++].pm.u, 0, 0, x);
    if (M & 8) pv_dense<3, true>(m[e++].pm.u, 0, 0, x);
}

// Gate on lane bit t: every thread computes its own row from its amplitude and its partner's; all
// lanes take part in the shuffles. NOCOND: no controls on tuple or lane bits (`on` is ignored).
template <int CODE, bool ALL, bool NOCOND>
__device__ __forceinline__ void pv_lane(const PassMember& g, uint32_t base, bool on, float2 (&x)[16]) {
    const int fm = g.fmv & 15, fv = (g.fmv >> 4) & 15;
    const int t = int((g.ctl >> 10) & 3u);
    const bool v = (base >> t) & 1u;  // this thread's row
    const int lm = 1 << t;
    float own_r, own_i, par_r = 0.f, par_i = 0.f;
    if (CODE == PC_DENSE) {  // own * x + par * partner
        own_r = v ? g.u[6] : g.u[0];
        own_i = v ? g.u[7] : g.u[1];
        par_r = v ? g.u[4] : g.u[2];
        par_i = v ? g.u[5] : g.u[3];
    } else if (CODE == PC_REAL) {
        own_r = v ? g.u[3] : g.u[0];
        par_r = v ? g.u[2] : g.u[1];
        own_i = 0.f;
    } else {  // the row's factor (swap: 1)
        own_r = (CODE == PC_SWAP) ? 1.f : (v ? g.u[2] : g.u[0]);
        own_i = (CODE == PC_SWAP) ? 0.f : (v ? g.u[3] : g.u[1]);
    }
#pragma unroll
    for (int j = 0; j < 16; j++) {
        if (!ALL && ((j & fm) != fv)) continue;  // uniform over the block: every lane skips together
        float2 y;
        if (CODE == PC_DIAG2) {
            y = pcmul(own_r, own_i, x[j]);
        } else {
            float2 p;
            p.x = __shfl_xor_sync(0xffffffffu, x[j].x, lm);
            p.y = __shfl_xor_sync(0xffffffffu, x[j].y, lm);
            if (CODE == PC_DENSE) {
                y = cfma(par_r, par_i, p, czero<float2>());
                y = cfma(own_r, own_i, x[j], y);
            } else if (CODE == PC_REAL) {
                y = make_float2(fmaf(own_r, x[j].x, par_r * p.x), fmaf(own_r, x[j].y, par_r * p.y));
            } else if (CODE == PC_SWAP) {
                y = p;
            } else {
                y = pcmul(own_r, own_i, p);
            }
        }
        if (NOCOND || on) x[j] = y;
    }
}

template <bool ALL>
__device__ __forceinline__ void pv_phase(const float* u, int fm, int fv, float2 (&x)[16]) {
    const float ur = u[0], ui = u[1];
#pragma unroll
    for (int j = 0; j < 16; j++) {
        if (!ALL && ((j & fm) != fv)) continue;
        x[j] = pcmul(ur, ui, x[j]);
    }
}

// Apply member m (its variant id in ctl) to the thread's registers.
__device__ __forceinline__ void pv_apply(const TileOp* m, uint32_t ctl, uint32_t base, float2 (&x)[16]) {
    const PassMember& g = m->pm;
    const uint32_t vid = ctl & 255u;
    const bool cond = ctl & (1u << 13);
    const bool on = !cond || (base & g.om) == g.ov;
    if ((vid < kPvLane || vid >= kPvPhase) && !on) return;  // register and phase gates: controls fail
    const int fm = g.fmv & 15, fv = (g.fmv >> 4) & 15;
    switch (vid) {
#define QS_PV_J(C, J, CALL_ALL, CALL_CTL) \
    case C * 8 + J * 2:                   \
        CALL_CTL;                         \
        break;                            \
    case C * 8 + J * 2 + 1:               \
        CALL_ALL;                         \
        break;
#define QS_PV_CODE(C, FN)                                                                                     \
    QS_PV_J(C, 0, (FN<0, true>(g.u, fm, fv, x)), (FN<0, false>(g.u, fm, fv, x)))                              \
    QS_PV_J(C, 1, (FN<1, true>(g.u, fm, fv, x)), (FN<1, false>(g.u, fm, fv, x)))                              \
    QS_PV_J(C, 2, (FN<2, true>(g.u, fm, fv, x)), (FN<2, false>(g.u, fm, fv, x)))                              \
    QS_PV_J(C, 3, (FN<3, true>(g.u, fm, fv, x)), (FN<3, false>(g.u, fm, fv, x)))
#define QS_PV_MONO(C)                                                                                          \
    QS_PV_J(C, 0, (pv_mono<0, C, true>(g.u, fm, fv, x)), (pv_mono<0, C, false>(g.u, fm, fv, x)))               \
    QS_PV_J(C, 1, (pv_mono<1, C, true>(g.u, fm, fv, x)), (pv_mono<1, C, false>(g.u, fm, fv, x)))               \
    QS_PV_J(C, 2, (pv_mono<2, C, true>(g.u, fm, fv, x)), (pv_mono<2, C, false>(g.u, fm, fv, x)))               \
    QS_PV_J(C, 3, (pv_mono<3, C, true>(g.u, fm, fv, x)), (pv_mono<3, C, false>(g.u, fm, fv, x)))
        QS_PV_CODE(0, pv_dense)
        QS_PV_CODE(1, pv_real)
        QS_PV_MONO(2)
        QS_PV_MONO(3)
        QS_PV_MONO(4)
#undef QS_PV_MONO
#undef QS_PV_CODE
#undef QS_PV_J
#define QS_PV_SC(J, C)                 \
    case kPvSwapC + J * 4 + C:         \
        pv_swapc<J, C>(x);             \
        break;
        QS_PV_SC(0, 1) QS_PV_SC(0, 2) QS_PV_SC(0, 3)
        QS_PV_SC(1, 0) QS_PV_SC(1, 2) QS_PV_SC(1, 3)
        QS_PV_SC(2, 0) QS_PV_SC(2, 1) QS_PV_SC(2, 3)
        QS_PV_SC(3, 0) QS_PV_SC(3, 1) QS_PV_SC(3, 2)
#undef QS_PV_SC
#define QS_PV_M(M)             \
    case kPvMulti + M:         \
        pv_multi<M>(m, x);     \
        break;
        QS_PV_M(3) QS_PV_M(5) QS_PV_M(6) QS_PV_M(7) QS_PV_M(9) QS_PV_M(10) QS_PV_M(11)
        QS_PV_M(12) QS_PV_M(13) QS_PV_M(14) QS_PV_M(15)
#undef QS_PV_M
#define QS_PV_L(C)                                        \
    case kPvLane + C * 4 + 0:                             \
        pv_lane<C, false, false>(g, base, on, x);         \
        break;                                            \
    case kPvLane + C * 4 + 1:                             \
        pv_lane<C, false, true>(g, base, on, x);          \
        break;                                            \
    case kPvLane + C * 4 + 2:                             \
        pv_lane<C, true, false>(g, base, on, x);          \
        break;                                            \
    case kPvLane + C * 4 + 3:                             \
        pv_lane<C, true, true>(g, base, on, x);           \
        break;
        QS_PV_L(0) QS_PV_L(1) QS_PV_L(2) QS_PV_L(3) QS_PV_L(4)
#undef QS_PV_L
        case kPvPhase:
            pv_phase<false>(g.u, fm, fv, x);
            break;
        case kPvPhase + 1:
            pv_phase<true>(g.u, fm, fv, x);
            break;
        default:
            break;
    }
}

// One register pass over the tile s. hdr is the OP_PASS header (its off[] and offsrc[] hold the 16
// register offsets), its member entries follow it; threads 0..255 take one tuple each per 4096
// amplitudes (2^(T-4) tuples, a multiple of 32).
__device__ __forceinline__ void pass_run_c64(float2* s, uint32_t tsize, uint64_t tile_base, const TileOp* hdr) {
    const int cnt = hdr->k;
    const uint32_t seg0 = hdr->seg[0], seg1 = hdr->seg[1], seg2 = hdr->seg[2], seg3 = hdr->seg[3],
                   seg4 = hdr->seg[4];
    // register offsets: read from shared memory (a broadcast) at the load and again at the store,
    // so they hold no registers while the members run
    auto off = [&](int j) -> uint32_t { return j < 8 ? hdr->off[j] : hdr->offsrc[j - 8]; };
    const uint32_t ntup = tsize >> kPassBits;
    for (uint32_t p = threadIdx.x; p < ntup; p += 256) {
        const uint32_t base = (p & seg0) | ((p << 1) & seg1) | ((p << 2) & seg2) | ((p << 3) & seg3) |
                              ((p << 4) & seg4);
        float2* sb = s + base;
        float2 x[16];
#pragma unroll
        for (int j = 0; j < 16; j++) x[j] = sb[off(j)];
        for (int mi = 1; mi <= cnt;) {
            const TileOp* m = hdr + mi;
            const uint32_t ctl = m->pm.ctl;
            if (!(ctl & (1u << 12)) || (tile_base & m->omask) == m->oval) pv_apply(m, ctl, base, x);
            mi += int((ctl >> 8) & 3u) + 1;
        }
#pragma unroll
        for (int j = 0; j < 16; j++) sb[off(j)] = x[j];
    }
}

}  // namespace qs
