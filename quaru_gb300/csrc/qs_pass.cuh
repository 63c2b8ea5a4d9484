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

// ---- tile-local index helpers (shared by the stage kernels)
__device__ __forceinline__ uint32_t expand_local(uint32_t t, const uint8_t* pos, int npos) {
    for (int i = 0; i < npos; i++) {
        const uint32_t p = pos[i];
        t = ((t >> p) << (p + 1)) | (t & ((1u << p) - 1u));
    }
    return t;
}

// Expanded tuple index of tuple t (local fixed bits' values ORed in).
__device__ __forceinline__ uint32_t tuple_index(uint32_t t, int npos, const uint32_t (&seg)[5], const uint8_t* pos,
                                                uint32_t fixval) {
    uint32_t e;
    if (npos <= 4) {
        e = t & seg[0];
        if (npos > 0) e |= (t << 1) & seg[1];
        if (npos > 1) e |= (t << 2) & seg[2];
        if (npos > 2) e |= (t << 3) & seg[3];
        if (npos > 3) e |= (t << 4) & seg[4];
    } else {
        e = expand_local(t, pos, npos);
    }
    return e | fixval;
}

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

// As pv_dense (no controls), on registers relabelled across bit J when `flip`: physical register
// a | 1 << J then holds logical row 0, so the gate runs with rows and columns exchanged.
template <int J>
__device__ __forceinline__ void pv_dense_flip(const float* u, bool flip, float2 (&x)[16]) {
    float4 c0 = *reinterpret_cast<const float4*>(u), c1 = *reinterpret_cast<const float4*>(u + 4);
    if (flip) {  // (u00, u01; u10, u11) -> (u11, u10; u01, u00)
        const float4 t0 = make_float4(c1.z, c1.w, c1.x, c1.y), t1 = make_float4(c0.z, c0.w, c0.x, c0.y);
        c0 = t0;
        c1 = t1;
    }
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if (a & (1 << J)) continue;
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

// Physical exchange of the registers across bit J (materialises a relabelling).
template <int J>
__device__ __forceinline__ void pv_xswap(float2 (&x)[16]) {
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if (a & (1 << J)) continue;
        const float2 t = x[a];
        x[a] = x[a | (1 << J)];
        x[a | (1 << J)] = t;
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

// Swap on register bit J where register bit C is V (CNOT with both qubits in registers; V = 0 when
// the registers are relabelled across bit C).
template <int J, int C, int V = 1>
__device__ __forceinline__ void pv_swapc(float2 (&x)[16]) {
#pragma unroll
    for (int a = 0; a < 16; a++) {
        if ((a & (1 << J)) || (((a >> C) & 1) != V)) continue;
        const int b = a | (1 << J);
        const float2 t = x[a];
        x[a] = x[b];
        x[b] = t;
    }
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

// Calls F<0..3>(...) by the two-bit field of v at `shift`, with bit tests (no jump table).
#define QS_PV_J4(v, shift, CALL) \
    if (((v) >> ((shift) + 1)) & 1u) {         \
        if (((v) >> (shift)) & 1u) {           \
            CALL(3);                            \
        } else {                                \
            CALL(2);                            \
        }                                       \
    } else {                                    \
        if (((v) >> (shift)) & 1u) {           \
            CALL(1);                            \
        } else {                                \
            CALL(0);                            \
        }                                       \
    }

// Apply member m (its variant id in ctl) to the thread's registers. The dispatch is a shallow tree
// of bit tests: a large switch costs about a hundred extra instructions per gate on sm_103a.
// COMMON: only the variants pass_common() admits are compiled (fewer live registers; the stage
// kernel with a copy warp runs at 96 registers per thread).
//
// COMMON also relabels registers: a swap without register controls toggles bit J of xm (logical
// register l lives in physical register l ^ xm) instead of moving data; register gates read xm
// (rows exchanged, control values adjusted), lane gates materialise it first (partners must agree),
// and the pass stores register p at the offset of p ^ xm.
template <bool COMMON>
__device__ __forceinline__ void pv_apply(const TileOp* m, uint32_t ctl, uint32_t base, float2 (&x)[16],
                                         uint32_t& xm) {
    const PassMember& g = m->pm;
    const uint32_t vid = ctl & 255u, cat = vid >> 4, low = vid & 15u;
    if (cat == PV_DENSES) {  // 1..4 dense gates without controls, one entry each
        int e = 0;
        if (COMMON) {
            if (low & 1u) pv_dense_flip<0>(m[e++].pm.u, xm & 1u, x);
            if (low & 2u) pv_dense_flip<1>(m[e++].pm.u, xm & 2u, x);
            if (low & 4u) pv_dense_flip<2>(m[e++].pm.u, xm & 4u, x);
            if (low & 8u) pv_dense_flip<3>(m[e++].pm.u, xm & 8u, x);
        } else {
            if (low & 1u) pv_dense<0, true>(m[e++].pm.u, 0, 0, x);
            if (low & 2u) pv_dense<1, true>(m[e++].pm.u, 0, 0, x);
            if (low & 4u) pv_dense<2, true>(m[e++].pm.u, 0, 0, x);
            if (low & 8u) pv_dense<3, true>(m[e++].pm.u, 0, 0, x);
        }
        return;
    }
    const bool on = !(ctl & (1u << 13)) || (base & g.om) == g.ov;
    const int fm = g.fmv & 15;
    const int fv = ((g.fmv >> 4) & 15) ^ int(xm & uint32_t(fm));  // controls read through the relabelling
    const bool all = low & 2u, nocond = low & 1u;
    if (cat == PV_LDENSE || cat == PV_LSWAP) {  // lane gates: every lane takes part in the shuffles
        if (COMMON && xm) {
            if (xm & 1u) pv_xswap<0>(x);
            if (xm & 2u) pv_xswap<1>(x);
            if (xm & 4u) pv_xswap<2>(x);
            if (xm & 8u) pv_xswap<3>(x);
            xm = 0;
        }
#define QS_PV_LANE(C)                                                          \
    {                                                                          \
        if (all) {                                                             \
            if (nocond) pv_lane<C, true, true>(g, base, on, x);               \
            else pv_lane<C, true, false>(g, base, on, x);                     \
        } else {                                                               \
            if (nocond) pv_lane<C, false, true>(g, base, on, x);              \
            else pv_lane<C, false, false>(g, base, on, x);                    \
        }                                                                      \
    }
        if (cat == PV_LDENSE) {
            if (COMMON)
                pv_lane<PC_DENSE, true, true>(g, base, on, x);
            else
                QS_PV_LANE(PC_DENSE)
        } else {
            QS_PV_LANE(PC_SWAP)
        }
        return;
    }
    if (!on) return;  // register and phase gates: this tuple fails the controls
    if (cat == PV_SWAP) {
        if (COMMON && all) {  // relabel instead of moving
            xm ^= 1u << (low >> 2);
            return;
        }
#define QS_PV_SW(J) \
    if (all) pv_mono<J, PC_SWAP, true>(g.u, fm, fv, x); else pv_mono<J, PC_SWAP, false>(g.u, fm, fv, x)
        QS_PV_J4(low, 2, QS_PV_SW)
#undef QS_PV_SW
        return;
    }
    if (cat == PV_SWAPC) {
        const uint32_t c = low & 3u;
        const bool v0 = COMMON && ((xm >> c) & 1u);  // the control bit is relabelled: it reads 1 where it holds 0
#define QS_PV_SC1(J, CC)                              \
    {                                                 \
        if (v0) pv_swapc<J, CC, 0>(x);                \
        else pv_swapc<J, CC, 1>(x);                   \
    }
#define QS_PV_SC(J)                                   \
    {                                                 \
        if (c == 0) QS_PV_SC1(J, (J == 0 ? 1 : 0))    \
        else if (c == 1) QS_PV_SC1(J, (J == 1 ? 0 : 1)) \
        else if (c == 2) QS_PV_SC1(J, (J == 2 ? 0 : 2)) \
        else QS_PV_SC1(J, (J == 3 ? 0 : 3))           \
    }
        QS_PV_J4(low, 2, QS_PV_SC)
#undef QS_PV_SC
#undef QS_PV_SC1
        return;
    }
    if (cat == PV_PHASE) {
        if (all) pv_phase<true>(g.u, fm, fv, x); else pv_phase<false>(g.u, fm, fv, x);
        return;
    }
    if (COMMON) return;
    // the rarer codes
    if (cat >= PV_LREAL) {
        if (cat == PV_LREAL) QS_PV_LANE(PC_REAL) else if (cat == PV_LSWAPPH) QS_PV_LANE(PC_SWAPPH) else QS_PV_LANE(PC_DIAG2)
        return;
    }
#undef QS_PV_LANE
    if (cat == PV_DENSE) {
#define QS_PV_D(J) if (all) pv_dense<J, true>(g.u, fm, fv, x); else pv_dense<J, false>(g.u, fm, fv, x)
        QS_PV_J4(low, 2, QS_PV_D)
#undef QS_PV_D
    } else if (cat == PV_REAL) {
#define QS_PV_R(J) if (all) pv_real<J, true>(g.u, fm, fv, x); else pv_real<J, false>(g.u, fm, fv, x)
        QS_PV_J4(low, 2, QS_PV_R)
#undef QS_PV_R
    } else if (cat == PV_SWAPPH) {
#define QS_PV_P(J) \
    if (all) pv_mono<J, PC_SWAPPH, true>(g.u, fm, fv, x); else pv_mono<J, PC_SWAPPH, false>(g.u, fm, fv, x)
        QS_PV_J4(low, 2, QS_PV_P)
#undef QS_PV_P
    } else {
#define QS_PV_G(J) \
    if (all) pv_mono<J, PC_DIAG2, true>(g.u, fm, fv, x); else pv_mono<J, PC_DIAG2, false>(g.u, fm, fv, x)
        QS_PV_J4(low, 2, QS_PV_G)
#undef QS_PV_G
    }
}
#undef QS_PV_J4

// One register pass over the tile s whose base amplitude index is *tile_base (read only for gates
// with controls outside the tile). hdr is the OP_PASS header (its off[] and offsrc[] hold the 16
// register offsets), its member entries follow it; threads 0..NT-1 take the 2^(T-4) tuples (a
// multiple of 32) in turn.
template <int NT = 256, bool COMMON = false>
__device__ __forceinline__ void pass_run_c64(float2* s, uint32_t tsize, const uint64_t* tile_base, const TileOp* hdr) {
    const int cnt = hdr->k;
    const uint32_t seg0 = hdr->seg[0], seg1 = hdr->seg[1], seg2 = hdr->seg[2], seg3 = hdr->seg[3],
                   seg4 = hdr->seg[4];
    // register offsets: read from shared memory (a broadcast) at the load and again at the store,
    // so they hold no registers while the members run
    auto off = [&](int j) -> uint32_t { return j < 8 ? hdr->off[j] : hdr->offsrc[j - 8]; };
    const uint32_t ntup = tsize >> kPassBits;
    for (uint32_t p = threadIdx.x; p < ntup; p += NT) {
        const uint32_t base = (p & seg0) | ((p << 1) & seg1) | ((p << 2) & seg2) | ((p << 3) & seg3) |
                              ((p << 4) & seg4);
        float2* sb = s + base;
        float2 x[16];
#pragma unroll
        for (int j = 0; j < 16; j++) x[j] = sb[off(j)];
        uint32_t xm = 0;  // register relabelling (COMMON only)
        for (int mi = 1; mi <= cnt;) {
            const TileOp* m = hdr + mi;
            const uint32_t ctl = m->pm.ctl;
            if (!(ctl & (1u << 12)) || (*tile_base & m->omask) == m->oval) pv_apply<COMMON>(m, ctl, base, x, xm);
            mi += int((ctl >> 8) & 3u) + 1;
        }
        // physical register j holds logical register j ^ xm: its offset is off(j) ^ off(xm)
        const uint32_t offx = off(0) ^ (((xm & 1u) ? hdr->off[1] : 0u) ^ ((xm & 2u) ? hdr->off[2] : 0u) ^
                                        ((xm & 4u) ? hdr->off[4] : 0u) ^ ((xm & 8u) ? hdr->offsrc[0] : 0u));
#pragma unroll
        for (int j = 0; j < 16; j++) sb[off(j) ^ offx] = x[j];
    }
}

}  // namespace qs
