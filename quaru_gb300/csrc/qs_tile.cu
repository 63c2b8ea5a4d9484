// qs_tile.cu — the cache-blocked stage kernel and its host driver.
//
// One CTA owns one tile (2^T amplitudes) at a time: it reads the tile from
// HBM with coalesced rows of 2^L amplitudes, applies every gate of the stage
// in shared memory, and writes the tile back. Gate arithmetic per
// representation:
//   REP 0  complex128, the reference's operation order (bit-identical to the
//          gate-by-gate run)
//   REP 1  complex128, FP64 fused multiply-add
//   REP 2  complex128 stored, double-float in shared memory (float4 per
//          amplitude: re_hi, re_lo, im_hi, im_lo), split once on load and
//          joined once on store
//   REP 3  complex64, FP32 fused multiply-add
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "qs_circuit.h"
#include "qs_device.cuh"
#include "qs_kernels.h"
#include "qs_tile.h"

namespace qs {

constexpr int kTileThreads = 256;

struct StageArgs {
    int T, L, H;
    int op_begin, op_end;
    IndexMap outer;        // expands a tile index into the base amplitude index
    uint8_t high[kTileMaxHigh];  // global qubit of local bit L + b
};

template <int REP>
struct TileElem;
template <>
struct TileElem<0> {
    using T = double2;
};
template <>
struct TileElem<1> {
    using T = double2;
};
template <>
struct TileElem<2> {
    using T = float4;
};
template <>
struct TileElem<3> {
    using T = float2;
};

__device__ __forceinline__ uint32_t expand_local(uint32_t t, const uint8_t* pos, int npos) {
    for (int i = 0; i < npos; i++) {
        const uint32_t p = pos[i];
        t = ((t >> p) << (p + 1)) | (t & ((1u << p) - 1u));
    }
    return t;
}

// ---- load / store conversions
template <int REP>
__device__ __forceinline__ typename TileElem<REP>::T tile_load(const void* st, uint64_t g);
template <>
__device__ __forceinline__ double2 tile_load<0>(const void* st, uint64_t g) {
    return static_cast<const double2*>(st)[g];
}
template <>
__device__ __forceinline__ double2 tile_load<1>(const void* st, uint64_t g) {
    return static_cast<const double2*>(st)[g];
}
template <>
__device__ __forceinline__ float4 tile_load<2>(const void* st, uint64_t g) {
    const double2 v = static_cast<const double2*>(st)[g];
    float4 r;
    df_split(v.x, r.x, r.y);
    df_split(v.y, r.z, r.w);
    return r;
}
template <>
__device__ __forceinline__ float2 tile_load<3>(const void* st, uint64_t g) {
    return static_cast<const float2*>(st)[g];
}

template <int REP>
__device__ __forceinline__ void tile_store(void* st, uint64_t g, typename TileElem<REP>::T v);
template <>
__device__ __forceinline__ void tile_store<0>(void* st, uint64_t g, double2 v) {
    static_cast<double2*>(st)[g] = v;
}
template <>
__device__ __forceinline__ void tile_store<1>(void* st, uint64_t g, double2 v) {
    static_cast<double2*>(st)[g] = v;
}
template <>
__device__ __forceinline__ void tile_store<2>(void* st, uint64_t g, float4 v) {
    static_cast<double2*>(st)[g] = make_double2(__dadd_rn(df_f2d(v.x), df_f2d(v.y)), __dadd_rn(df_f2d(v.z), df_f2d(v.w)));
}
template <>
__device__ __forceinline__ void tile_store<3>(void* st, uint64_t g, float2 v) {
    static_cast<float2*>(st)[g] = v;
}

// ---- value-exact phase moves (1, -1, i, -i) per representation
__device__ __forceinline__ double2 pf_move(double2 x, uint8_t c) { return apply_pf(x, c); }
__device__ __forceinline__ float2 pf_move(float2 x, uint8_t c) { return apply_pf(x, c); }
__device__ __forceinline__ float4 pf_move(float4 x, uint8_t c) {
    float4 r = x;
    if (c == 1) {
        r = make_float4(-x.x, -x.y, -x.z, -x.w);
    } else if (c == 2) {  // i * (re + i im) = -im + i re
        r = make_float4(-x.z, -x.w, x.x, x.y);
    } else if (c == 3) {  // -i * (re + i im) = im - i re
        r = make_float4(x.z, x.w, -x.x, -x.y);
    }
    return r;
}

// general complex phase p times x
__device__ __forceinline__ double2 phase_mul(const double* p, double2 x, int rep) {
    if (rep == 0) return cmul_exact(p[0], p[1], x);
    double2 r;
    r.x = fma(p[0], x.x, -p[1] * x.y);
    r.y = fma(p[0], x.y, p[1] * x.x);
    return r;
}
__device__ __forceinline__ float2 phase_mul(const double* p, float2 x, int) {
    const float pr = float(p[0]), pi = float(p[1]);
    return make_float2(fmaf(pr, x.x, -pi * x.y), fmaf(pr, x.y, pi * x.x));
}
__device__ __forceinline__ float4 phase_mul(const double* p, float4 x, int) {
    float ph[2], pl[2];
    df_split(p[0], ph[0], pl[0]);
    df_split(p[1], ph[1], pl[1]);
    float4 r;
    {   // re = pr*xr - pi*xi
        const float uh[2] = {ph[0], -ph[1]}, ul[2] = {pl[0], -pl[1]};
        const float xh[2] = {x.x, x.z}, xl[2] = {x.y, x.w};
        df_dot_pair<2>(uh, ul, xh, xl, r.x, r.y);
    }
    {   // im = pr*xi + pi*xr
        const float uh[2] = {ph[0], ph[1]}, ul[2] = {pl[0], pl[1]};
        const float xh[2] = {x.z, x.x}, xl[2] = {x.w, x.y};
        df_dot_pair<2>(uh, ul, xh, xl, r.z, r.w);
    }
    return r;
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

template <int REP>
struct DenseCoef;
template <>
struct DenseCoef<0> {
    double m[8];
};
template <>
struct DenseCoef<1> {
    double m[8];
};
template <>
struct DenseCoef<2> {
    float h[16], l[16];
};
template <>
struct DenseCoef<3> {
    float m[8];
};

__device__ __forceinline__ void load_coef(DenseCoef<0>& c, const TileOp& op) {
#pragma unroll
    for (int i = 0; i < 8; i++) c.m[i] = op.m[i];
}
__device__ __forceinline__ void load_coef(DenseCoef<1>& c, const TileOp& op) {
#pragma unroll
    for (int i = 0; i < 8; i++) c.m[i] = op.m[i];
}
__device__ __forceinline__ void load_coef(DenseCoef<2>& c, const TileOp& op) {
#pragma unroll
    for (int i = 0; i < 16; i++) {
        c.h[i] = op.dfh[i];
        c.l[i] = op.dfl[i];
    }
}
__device__ __forceinline__ void load_coef(DenseCoef<3>& c, const TileOp& op) {
#pragma unroll
    for (int i = 0; i < 8; i++) c.m[i] = op.mf[i];
}

__device__ __forceinline__ void dense_pair(const DenseCoef<0>& c, bool real, double2& a, double2& b) {
    double2 y0, y1;
    if (real) {
        y0 = cadd_exact(cmul_exact_real(c.m[0], a), cmul_exact_real(c.m[2], b));
        y1 = cadd_exact(cmul_exact_real(c.m[4], a), cmul_exact_real(c.m[6], b));
    } else {
        y0 = cadd_exact(cmul_exact(c.m[0], c.m[1], a), cmul_exact(c.m[2], c.m[3], b));
        y1 = cadd_exact(cmul_exact(c.m[4], c.m[5], a), cmul_exact(c.m[6], c.m[7], b));
    }
    a = y0;
    b = y1;
}
__device__ __forceinline__ void dense_pair(const DenseCoef<1>& c, bool, double2& a, double2& b) {
    double2 y0 = cfma(c.m[2], c.m[3], b, czero<double2>());
    y0 = cfma(c.m[0], c.m[1], a, y0);
    double2 y1 = cfma(c.m[6], c.m[7], b, czero<double2>());
    y1 = cfma(c.m[4], c.m[5], a, y1);
    a = y0;
    b = y1;
}
__device__ __forceinline__ void dense_pair(const DenseCoef<3>& c, bool, float2& a, float2& b) {
    float2 y0 = cfma(c.m[2], c.m[3], b, czero<float2>());
    y0 = cfma(c.m[0], c.m[1], a, y0);
    float2 y1 = cfma(c.m[6], c.m[7], b, czero<float2>());
    y1 = cfma(c.m[4], c.m[5], a, y1);
    a = y0;
    b = y1;
}
__device__ __forceinline__ void dense_pair(const DenseCoef<2>& c, bool real, float4& a, float4& b) {
    const float xh[4] = {a.x, a.z, b.x, b.z};  // x0.re, x0.im, x1.re, x1.im (hi)
    const float xl[4] = {a.y, a.w, b.y, b.w};
    float oh[4], ol[4];
#pragma unroll
    for (int o = 0; o < 4; o++) {
        if (real) {
            const float th[2] = {xh[o & 1], xh[2 + (o & 1)]}, tl[2] = {xl[o & 1], xl[2 + (o & 1)]};
            const float ch[2] = {c.h[4 * o], c.h[4 * o + 2]}, cl[2] = {c.l[4 * o], c.l[4 * o + 2]};
            df_dot_pair<2>(ch, cl, th, tl, oh[o], ol[o]);
        } else {
            float th[4], tl[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                th[t] = xh[(o & 1) ? (t ^ 1) : t];
                tl[t] = xl[(o & 1) ? (t ^ 1) : t];
            }
            df_dot_pair<4>(c.h + 4 * o, c.l + 4 * o, th, tl, oh[o], ol[o]);
        }
    }
    a = make_float4(oh[0], ol[0], oh[1], ol[1]);
    b = make_float4(oh[2], ol[2], oh[3], ol[3]);
}

// ---- register groups (complex64): each thread holds two 8-amplitude tuples of a 3-bit
// sub-cube in registers and applies the group's members to both; a member's fields are read
// once per pair of tuples and dispatched to code specialised for its target bit.
template <int REP>
__device__ __forceinline__ typename TileElem<REP>::T mono_row(const TileOp& m, int r, typename TileElem<REP>::T src) {
    const uint8_t c = m.pf[r];
    if (c == 255) return phase_mul(m.m + 2 * r, src, REP);
    return pf_move(src, c);
}

struct GMember {
    float u[8];     // dense coefficients, or the two rows' phases for monomials
    int fm, fv;     // fixed bits inside the group
    uint8_t pf0, pf1, s0, s1;
};

__device__ __forceinline__ float2 gm_row(uint8_t cls, const float* ph, float2 x) {
    if (cls == 255) return make_float2(fmaf(ph[0], x.x, -ph[1] * x.y), fmaf(ph[0], x.y, ph[1] * x.x));
    return apply_pf(x, cls);
}

template <int J, int CODE, bool ALL>
__device__ __forceinline__ void gm_apply(const GMember& g, float2 (&x)[8]) {
#pragma unroll
    for (int a = 0; a < 8; a++) {
        if (a & (1 << J)) continue;
        if (!ALL && ((a & g.fm) != g.fv)) continue;
        const int b = a | (1 << J);
        const float2 xa = x[a], xb = x[b];
        if (CODE == 0) {
            float2 y0 = cfma(g.u[2], g.u[3], xb, czero<float2>());
            y0 = cfma(g.u[0], g.u[1], xa, y0);
            float2 y1 = cfma(g.u[6], g.u[7], xb, czero<float2>());
            y1 = cfma(g.u[4], g.u[5], xa, y1);
            x[a] = y0;
            x[b] = y1;
        } else if (CODE == 1) {
            float2 y0, y1;
            y0.x = fmaf(g.u[0], xa.x, g.u[2] * xb.x);
            y0.y = fmaf(g.u[0], xa.y, g.u[2] * xb.y);
            y1.x = fmaf(g.u[4], xa.x, g.u[6] * xb.x);
            y1.y = fmaf(g.u[4], xa.y, g.u[6] * xb.y);
            x[a] = y0;
            x[b] = y1;
        } else {
            const float2 s0 = g.s0 ? xb : xa, s1 = g.s1 ? xb : xa;
            if (g.pf0 != PF_SKIP_DEV) x[a] = gm_row(g.pf0, g.u, s0);
            if (g.pf1 != PF_SKIP_DEV) x[b] = gm_row(g.pf1, g.u + 2, s1);
        }
    }
}

template <int CODE, bool ALL>
__device__ __forceinline__ void gm_dispatch_j(int j, const GMember& g, float2 (&x)[8]) {
    if (j == 0)
        gm_apply<0, CODE, ALL>(g, x);
    else if (j == 1)
        gm_apply<1, CODE, ALL>(g, x);
    else
        gm_apply<2, CODE, ALL>(g, x);
}

__device__ __forceinline__ void gm_dispatch(int code, int j, const GMember& g, float2 (&x)[8]) {
    const bool all = g.fm == 0;
    if (code == 3) {  // phase or sign on the fixed subspace (k = 0)
        if (g.pf0 == PF_SKIP_DEV) return;
#pragma unroll
        for (int r = 0; r < 8; r++)
            if ((r & g.fm) == g.fv) x[r] = gm_row(g.pf0, g.u, x[r]);
        return;
    }
    if (code == 0) {
        if (all) gm_dispatch_j<0, true>(j, g, x); else gm_dispatch_j<0, false>(j, g, x);
    } else if (code == 1) {
        if (all) gm_dispatch_j<1, true>(j, g, x); else gm_dispatch_j<1, false>(j, g, x);
    } else {
        if (all) gm_dispatch_j<2, true>(j, g, x); else gm_dispatch_j<2, false>(j, g, x);
    }
}

// One register group over the tile s (complex64). hdr is the OP_GROUP header, members follow it.
__device__ __forceinline__ void group_run_c64(float2* s, uint32_t tsize, uint64_t base, const TileOp* hdr) {
    const int cnt = hdr->k;
    uint32_t goff[8], seg[5];
#pragma unroll
    for (int j = 0; j < 8; j++) goff[j] = hdr->off[j];
#pragma unroll
    for (int j = 0; j < 5; j++) seg[j] = hdr->seg[j];
    const int npos = hdr->npos;
    const uint32_t ng = tsize >> 3;
    for (uint32_t p0 = threadIdx.x; p0 < ng; p0 += 2 * kTileThreads) {
        const bool two = p0 + kTileThreads < ng;
        const uint32_t b0 = tuple_index(p0, npos, seg, hdr->pos, 0u);
        const uint32_t b1 = two ? tuple_index(p0 + kTileThreads, npos, seg, hdr->pos, 0u) : b0;
        float2 x0[8], x1[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            x0[j] = s[b0 + goff[j]];
            x1[j] = s[b1 + goff[j]];
        }
        for (int mi = 1; mi <= cnt; mi++) {
            const TileOp& m = hdr[mi];
            if ((base & m.omask) != m.oval) continue;
            GMember g;
#pragma unroll
            for (int i = 0; i < 8; i++) g.u[i] = m.mf[i];
            g.fm = m.gfin_mask;
            g.fv = m.gfin_val;
            g.pf0 = m.pf[0];
            g.pf1 = m.pf[1];
            g.s0 = m.offsrc[0] != 0;
            g.s1 = m.offsrc[1] != 0;
            const int code = m.gcode, j = m.gj;
            const uint32_t om = m.gfout_mask, ov = m.gfout_val;
            if ((b0 & om) == ov) gm_dispatch(code, j, g, x0);
            if (two && (b1 & om) == ov) gm_dispatch(code, j, g, x1);
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            s[b0 + goff[j]] = x0[j];
            if (two) s[b1 + goff[j]] = x1[j];
        }
    }
}

// ---- fused 5-qubit blocks on the tensor cores (complex64 tiles, 3xTF32)
__device__ __forceinline__ uint32_t f2tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t deposit5(uint32_t r, const uint8_t* pos) {
    uint32_t o = 0;
#pragma unroll
    for (int b = 0; b < 5; b++) o |= ((r >> b) & 1u) << pos[b];
    return o;
}

// Y = U X for the 32-row block view of the tile: X^T (columns x 64 real) times
// B = M^T, M = [[Ur, -Ui], [Ui, Ur]]; D = A_lo B_hi + A_hi B_lo + A_hi B_hi in FP32.
// Warp w owns m-tiles w, w + 8, ... (16 columns each) and updates them in place.
__device__ __forceinline__ void block_apply(float* sf, uint32_t tsize, const TileOp& op,
                                            const float4* __restrict__ bfrag) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t nmt = (tsize >> 5) >> 4;
    uint8_t pos[5];
#pragma unroll
    for (int b = 0; b < 5; b++) pos[b] = op.pos[b];
    uint32_t rd[8], wr[8];
#pragma unroll
    for (int j = 0; j < 8; j++) rd[j] = deposit5(uint32_t(4 * j + t), pos);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        wr[2 * q] = deposit5(uint32_t(8 * q + 2 * t), pos);
        wr[2 * q + 1] = deposit5(uint32_t(8 * q + 2 * t + 1), pos);
    }
    const float4* bf = bfrag + op.bidx + lane;
    for (uint32_t mt = warp; mt < nmt; mt += kTileThreads / 32) {
        const uint32_t c0 = expand_local(16 * mt + g, pos, 5);
        const uint32_t c1 = expand_local(16 * mt + g + 8, pos, 5);
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll 1
        for (int comp = 0; comp < 2; comp++) {  // k-steps 0..3 read real parts, 4..7 imaginary parts
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int ks = 4 * comp + q;
                const float a0 = sf[2 * (c0 | rd[2 * q]) + comp], a1 = sf[2 * (c1 | rd[2 * q]) + comp];
                const float a2 = sf[2 * (c0 | rd[2 * q + 1]) + comp], a3 = sf[2 * (c1 | rd[2 * q + 1]) + comp];
                const uint32_t h0 = f2tf32(a0), h1 = f2tf32(a1), h2 = f2tf32(a2), h3 = f2tf32(a3);
                const uint32_t l0 = f2tf32(a0 - __uint_as_float(h0)), l1 = f2tf32(a1 - __uint_as_float(h1));
                const uint32_t l2 = f2tf32(a2 - __uint_as_float(h2)), l3 = f2tf32(a3 - __uint_as_float(h3));
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    const float4 b = __ldg(bf + (nt * 8 + ks) * 32);
                    const uint32_t bh0 = __float_as_uint(b.x), bh1 = __float_as_uint(b.y);
                    const uint32_t bl0 = __float_as_uint(b.z), bl1 = __float_as_uint(b.w);
                    mma_tf32(acc[nt], l0, l1, l2, l3, bh0, bh1);
                    mma_tf32(acc[nt], h0, h1, h2, h3, bl0, bl1);
                    mma_tf32(acc[nt], h0, h1, h2, h3, bh0, bh1);
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int comp = nt >> 2, q = nt & 3;
            sf[2 * (c0 | wr[2 * q]) + comp] = acc[nt][0];
            sf[2 * (c0 | wr[2 * q + 1]) + comp] = acc[nt][1];
            sf[2 * (c1 | wr[2 * q]) + comp] = acc[nt][2];
            sf[2 * (c1 | wr[2 * q + 1]) + comp] = acc[nt][3];
        }
        __syncwarp();
    }
}

// ---- TMA bulk copies and mbarriers
__device__ __forceinline__ uint32_t saddr(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase of `parity` to complete, at most ~2 s of SM clocks.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > 4000000000LL) return false;
    return true;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(saddr(src)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Element type of the state in global memory (the tile buffer holds it while a copy is in flight).
template <int REP>
struct GlobElem {
    using T = double2;
};
template <>
struct GlobElem<3> {
    using T = float2;
};

// One CTA walks its tiles with two shared-memory buffers: while it applies the stage to tile i,
// warp 0 has already issued the bulk row copies of tile i + 1 into the other buffer (completion
// on an mbarrier with expect-tx); finished tiles go back with bulk stores. Waits are bounded and
// set *err instead of hanging.
template <int REP, bool BLK>
__global__ void __launch_bounds__(kTileThreads, 2) k_tile(void* __restrict__ state, uint64_t ntiles,
                                                       const __grid_constant__ StageArgs sa,
                                                       const TileOp* __restrict__ ops,
                                                       const float4* __restrict__ bfrag, int* __restrict__ err) {
    using E = typename TileElem<REP>::T;
    using GE = typename GlobElem<REP>::T;
    static_assert(sizeof(E) == sizeof(GE), "tile element and state element must have the same size");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t tsize = 1u << sa.T;
    E* bufs = reinterpret_cast<E*>(smem_raw);
    const int nrows = 1 << sa.H;
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(smem_raw + 2 * (sizeof(E) << sa.T));
    uint64_t* mbar = rowoff + nrows;
    TileOp* sops = reinterpret_cast<TileOp*>(mbar + 2);
    __shared__ int s_abort;
    const int nops = sa.op_end - sa.op_begin;
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ops + sa.op_begin);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sops);
        const int words = nops * int(sizeof(TileOp) / 4);
        for (int w = threadIdx.x; w < words; w += kTileThreads) dst[w] = src[w];
    }
    for (int r = threadIdx.x; r < nrows; r += kTileThreads) {
        uint64_t o = 0;
        for (int b = 0; b < sa.H; b++)
            if (r >> b & 1) o |= 1ull << sa.high[b];
        rowoff[r] = o;
    }
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_mbar_init();
        s_abort = 0;
    }
    __syncthreads();
    const uint64_t first = blockIdx.x;
    const uint64_t nmy = (ntiles > first) ? (ntiles - 1 - first) / gridDim.x + 1 : 0;
    const uint32_t row_bytes = uint32_t(sizeof(GE)) << sa.L;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    GE* gstate = static_cast<GE*>(state);
    auto issue_load = [&](uint64_t i, int b) {  // warp 0 only
        const uint64_t tb = expand_index(first + i * gridDim.x, sa.outer);
        if (lane == 0) mbar_expect_tx(&mbar[b], row_bytes * uint32_t(nrows));
        __syncwarp();
        for (int r = lane; r < nrows; r += 32)
            bulk_load(bufs + size_t(b) * tsize + (size_t(r) << sa.L), gstate + tb + rowoff[r], row_bytes, &mbar[b]);
    };
    if (warp == 0 && nmy > 0) issue_load(0, 0);
    uint64_t it = 0;
    for (; it < nmy; it++) {
        const int bsel = int(it & 1);
        E* s = bufs + size_t(bsel) * tsize;
        const uint64_t base = expand_index(first + it * gridDim.x, sa.outer);
        if (warp == 0 && it + 1 < nmy) {
            bulk_wait_read_all();  // the other buffer's previous store has read shared memory
            __syncwarp();
            issue_load(it + 1, bsel ^ 1);
        }
        if (!mbar_wait_bounded(&mbar[bsel], uint32_t((it >> 1) & 1))) atomicOr(&s_abort, 1);
        __syncthreads();
        if (s_abort) break;
        if constexpr (REP == 2) {  // split the loaded doubles into double-float pairs, in place
            for (uint32_t i = threadIdx.x; i < tsize; i += kTileThreads) {
                const double2 v = reinterpret_cast<const double2*>(s)[i];
                float4 f;
                df_split(v.x, f.x, f.y);
                df_split(v.y, f.z, f.w);
                s[i] = f;
            }
            __syncthreads();
        }
        for (int o = 0; o < nops; o++) {
            const TileOp& op = sops[o];
            if ((base & op.omask) != op.oval) continue;
            const int npos = op.npos;
            const uint32_t ntup = tsize >> npos;
            const uint32_t fixv = op.lfixval;
            uint32_t seg[5];
#pragma unroll
            for (int j = 0; j < 5; j++) seg[j] = op.seg[j];
            const int kind = op.kind;
            if (BLK) {
                if constexpr (REP == 3 && BLK)
                    if (kind == OP_BLOCK) block_apply(reinterpret_cast<float*>(s), tsize, op, bfrag);
            } else if (REP == 3 && kind == OP_GROUP) {
                if constexpr (REP == 3 && !BLK) group_run_c64(reinterpret_cast<float2*>(s), tsize, base, &sops[o]);
                o += op.k;
            } else if (kind == OP_DENSE || kind == OP_DENSE_REAL) {
                const uint32_t tb = op.off[1];
                const bool real = kind == OP_DENSE_REAL;
                DenseCoef<REP> c;
                load_coef(c, op);
                for (uint32_t p = threadIdx.x; p < ntup; p += kTileThreads) {
                    const uint32_t i0 = tuple_index(p, npos, seg, op.pos, fixv);
                    E a = s[i0], b = s[i0 | tb];
                    dense_pair(c, real, a, b);
                    s[i0] = a;
                    s[i0 | tb] = b;
                }
            } else if (kind == OP_MONO || kind == OP_MONO_PF) {
                const int D = 1 << op.k;
                for (uint32_t p = threadIdx.x; p < ntup; p += kTileThreads) {
                    const uint32_t i0 = tuple_index(p, npos, seg, op.pos, fixv);
                    E y[8];
#pragma unroll
                    for (int r = 0; r < 8; r++)
                        if (r < D && op.pf[r] != PF_SKIP_DEV) y[r] = s[i0 + op.offsrc[r]];
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        if (r >= D || op.pf[r] == PF_SKIP_DEV) continue;
                        s[i0 + op.off[r]] = mono_row<REP>(op, r, y[r]);
                    }
                }
            }
            __syncthreads();
        }
        if constexpr (REP == 2) {  // join the double-float pairs back into doubles, in place
            for (uint32_t i = threadIdx.x; i < tsize; i += kTileThreads) {
                const float4 f = s[i];
                reinterpret_cast<double2*>(s)[i] =
                    make_double2(__dadd_rn(df_f2d(f.x), df_f2d(f.y)), __dadd_rn(df_f2d(f.z), df_f2d(f.w)));
            }
        }
        fence_async_shared();  // make this tile's shared-memory writes visible to the bulk stores
        __syncthreads();
        if (warp == 0) {
            for (int r = lane; r < nrows; r += 32)
                bulk_store(gstate + base + rowoff[r], s + (size_t(r) << sa.L), row_bytes);
            bulk_commit();
        }
    }
    if (warp == 0) bulk_wait_all();
    if (s_abort && threadIdx.x == 0) {
        atomicExch(err, 1);
        if (it + 1 < nmy) mbar_wait_bounded(&mbar[int((it + 1) & 1)], uint32_t(((it + 1) >> 1) & 1));
    }
}

static int tile_fail(cudaError_t e, const char* what, std::string* msg) {
    if (msg) *msg = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? QS_OUT_OF_MEMORY : QS_CUDA_ERROR;
}

template <int REP, bool BLK>
static cudaError_t launch_tile(void* state, int n, const TileStage& st, int op_begin, int op_end,
                               const TileOp* dops, const float4* dfrag, int* derr, cudaStream_t s, int sms) {
    using E = typename TileElem<REP>::T;
    StageArgs sa;
    std::memset(&sa, 0, sizeof(sa));
    sa.T = st.T;
    sa.L = st.L;
    sa.H = int(st.high.size());
    sa.op_begin = op_begin;
    sa.op_end = op_end;
    std::vector<int> qpos;
    for (int q = 0; q < st.L; q++) qpos.push_back(q);
    for (int q : st.high) qpos.push_back(q);
    std::sort(qpos.begin(), qpos.end());
    sa.outer.npos = int(qpos.size());
    for (size_t i = 0; i < qpos.size(); i++) sa.outer.pos[i] = uint8_t(qpos[i]);
    sa.outer.fixval = 0;
    for (int b = 0; b < sa.H; b++) sa.high[b] = uint8_t(st.high[b]);
    const size_t smem = 2 * (sizeof(E) << st.T) + (sizeof(uint64_t) << sa.H) + 2 * sizeof(uint64_t) +
                        sizeof(TileOp) * size_t(op_end - op_begin);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_tile<REP, BLK>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    const uint64_t ntiles = 1ull << (n - st.T);
    const int per_sm = std::max(1, std::min(8, int((220 * 1024) / smem)));
    const uint64_t grid = std::min<uint64_t>(ntiles, uint64_t(sms) * per_sm);
    k_tile<REP, BLK><<<int(grid), kTileThreads, smem, s>>>(state, ntiles, sa, dops, dfrag, derr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launches(1);
    return e;
}

static bool df64_range_ok(const OpDesc& op) {
    if (op.kind != OP_DENSE && op.kind != OP_DENSE_REAL) return true;
    for (double v : op.m) {
        const double a = v < 0 ? -v : v;
        if (a != 0.0 && (a > 0x1p100 || a < 0x1p-100)) return false;
    }
    return true;
}

int run_tiled(void* state, int n, int prec, int arith, const std::vector<OpDesc>& ops,
              const std::vector<TileStage>& stages, cudaStream_t s, int sms, std::string* msg,
              const std::vector<float>* block_frags) {
    int rep = (prec == QS_PREC_C64) ? 3 : (arith == QS_ARITH_EXACT ? 0 : (arith == QS_ARITH_FMA ? 1 : 2));
    if (rep == 2)
        for (const auto& op : ops)
            if (!df64_range_ok(op)) rep = 1;  // entries outside double-float range: FP64 FMA instead
    std::vector<TileOp> host;
    std::vector<int> first(stages.size(), 0);
    for (size_t i = 0; i < stages.size(); i++) {
        first[i] = int(host.size());
        if (!stages[i].tiled) continue;
        // Register groups pay off where shared-memory passes dominate (complex64); the
        // FP64 and double-float tiles are arithmetic-bound and keep one pass per gate.
        for (const TileOp& t : stage_program(ops, stages[i], rep == 3)) host.push_back(t);
    }
    // One allocation: the op table, then an error flag the tile kernels raise when a bounded wait gives up.
    TileOp* dops = nullptr;
    int* derr = nullptr;
    unsigned char* dblob = nullptr;
    const size_t ops_bytes = ((host.size() * sizeof(TileOp) + 255) / 256) * 256;
    {
        cudaError_t e = cudaMallocAsync((void**)&dblob, ops_bytes + 256, s);
        if (e != cudaSuccess) return tile_fail(e, "tile op table", msg);
        dops = reinterpret_cast<TileOp*>(dblob);
        derr = reinterpret_cast<int*>(dblob + ops_bytes);
        e = cudaMemsetAsync(derr, 0, sizeof(int), s);
        if (e == cudaSuccess && !host.empty())
            e = cudaMemcpyAsync(dops, host.data(), host.size() * sizeof(TileOp), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(dblob, s);
            return tile_fail(e, "tile op upload", msg);
        }
    }
    float4* dfrag = nullptr;
    if (block_frags && !block_frags->empty()) {
        cudaError_t e = cudaMallocAsync((void**)&dfrag, block_frags->size() * sizeof(float), s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dfrag, block_frags->data(), block_frags->size() * sizeof(float),
                                cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(dblob, s);
            return tile_fail(e, "block fragments", msg);
        }
    }
    int rc = QS_OK;
    for (size_t i = 0; i < stages.size() && rc == QS_OK; i++) {
        const TileStage& st = stages[i];
        if (!st.tiled) {
            rc = apply_op(state, n, prec, arith, ops[st.single], s, sms, msg);
            continue;
        }
        const int b = first[i], e2 = (i + 1 < stages.size()) ? first[i + 1] : int(host.size());
        cudaError_t e;
        switch (rep) {
            case 0: e = launch_tile<0, false>(state, n, st, b, e2, dops, dfrag, derr, s, sms); break;
            case 1: e = launch_tile<1, false>(state, n, st, b, e2, dops, dfrag, derr, s, sms); break;
            case 2: e = launch_tile<2, false>(state, n, st, b, e2, dops, dfrag, derr, s, sms); break;
            default:
                if (dfrag)
                    e = launch_tile<3, true>(state, n, st, b, e2, dops, dfrag, derr, s, sms);
                else
                    e = launch_tile<3, false>(state, n, st, b, e2, dops, dfrag, derr, s, sms);
                break;
        }
        if (e != cudaSuccess) rc = tile_fail(e, "tile kernel", msg);
    }
    if (rc == QS_OK) {  // a bounded wait inside a tile kernel that gave up is reported here
        int herr = 0;
        cudaError_t e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            rc = tile_fail(e, "tile status", msg);
        else if (herr) {
            if (msg) *msg = "a tile kernel's bounded wait for its bulk copies gave up";
            rc = QS_TIMEOUT;
        }
    }
    cudaFreeAsync(dblob, s);
    if (dfrag) cudaFreeAsync(dfrag, s);
    return rc;
}

}  // namespace qs
