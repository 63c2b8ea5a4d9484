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

// ---- register groups: the 8 amplitudes of a 3-bit sub-cube held in registers
template <int REP>
__device__ __forceinline__ typename TileElem<REP>::T mono_row(const TileOp& m, int r, typename TileElem<REP>::T src) {
    const uint8_t c = m.pf[r];
    if (c == 255) return phase_mul(m.m + 2 * r, src, REP);
    return pf_move(src, c);
}

// Pair (a, b) of a k = 1 gate on group-local bit j; a has bit j clear.
template <int REP>
__device__ __forceinline__ void group_pair(const TileOp& m, const DenseCoef<REP>& c, bool dense, bool real,
                                           typename TileElem<REP>::T& xa, typename TileElem<REP>::T& xb) {
    using E = typename TileElem<REP>::T;
    if (dense) {
        dense_pair(c, real, xa, xb);
    } else {
        const E s0 = m.offsrc[0] ? xb : xa;
        const E s1 = m.offsrc[1] ? xb : xa;
        if (m.pf[0] != PF_SKIP_DEV) xa = mono_row<REP>(m, 0, s0);
        if (m.pf[1] != PF_SKIP_DEV) xb = mono_row<REP>(m, 1, s1);
    }
}

#define QS_GPAIR(A, B)                                                          \
    if (((A) & fm) == fv) group_pair<REP>(m, c, dense, real, x[A], x[B]);

template <int REP>
__device__ __forceinline__ void group_apply(const TileOp& m, typename TileElem<REP>::T (&x)[8]) {
    const int fm = m.gfin_mask, fv = m.gfin_val;
    const int kind = m.kind;
    if (m.k == 0) {  // phase or sign on the fixed subspace
#pragma unroll
        for (int r = 0; r < 8; r++)
            if ((r & fm) == fv && m.pf[0] != PF_SKIP_DEV) x[r] = mono_row<REP>(m, 0, x[r]);
        return;
    }
    const bool dense = kind == OP_DENSE || kind == OP_DENSE_REAL;
    const bool real = kind == OP_DENSE_REAL;
    DenseCoef<REP> c;
    if (dense) load_coef(c, m);
    switch (m.gj) {
        case 0:
            QS_GPAIR(0, 1) QS_GPAIR(2, 3) QS_GPAIR(4, 5) QS_GPAIR(6, 7) break;
        case 1:
            QS_GPAIR(0, 2) QS_GPAIR(1, 3) QS_GPAIR(4, 6) QS_GPAIR(5, 7) break;
        default:
            QS_GPAIR(0, 4) QS_GPAIR(1, 5) QS_GPAIR(2, 6) QS_GPAIR(3, 7) break;
    }
}
#undef QS_GPAIR

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

template <int REP, bool BLK>
__global__ void __launch_bounds__(kTileThreads, (REP == 3 && !BLK) ? 3 : 2) k_tile(void* __restrict__ state, uint64_t ntiles,
                                                       const __grid_constant__ StageArgs sa,
                                                       const TileOp* __restrict__ ops,
                                                       const float4* __restrict__ bfrag) {
    using E = typename TileElem<REP>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    E* s = reinterpret_cast<E*>(smem_raw);
    const int nrows = 1 << sa.H;
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(smem_raw + (sizeof(E) << sa.T));
    TileOp* sops = reinterpret_cast<TileOp*>(rowoff + nrows);
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
    __syncthreads();
    const uint32_t tsize = 1u << sa.T;
    const uint32_t lmask = (1u << sa.L) - 1u;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = expand_index(tile, sa.outer);
        for (uint32_t i = threadIdx.x; i < tsize; i += kTileThreads)
            s[i] = tile_load<REP>(state, base + rowoff[i >> sa.L] + (i & lmask));
        __syncthreads();
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
              if constexpr (REP == 3 && !BLK) {
                const int cnt = op.k;
                uint32_t goff[8];
#pragma unroll
                for (int j = 0; j < 8; j++) goff[j] = op.off[j];
                for (uint32_t p = threadIdx.x; p < ntup; p += kTileThreads) {
                    const uint32_t b0 = tuple_index(p, npos, seg, op.pos, 0u);
                    E x[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) x[j] = s[b0 + goff[j]];
                    for (int mi = 1; mi <= cnt; mi++) {
                        const TileOp& m = sops[o + mi];
                        if ((base & m.omask) != m.oval) continue;
                        if ((b0 & m.gfout_mask) != m.gfout_val) continue;
                        group_apply<REP>(m, x);
                    }
#pragma unroll
                    for (int j = 0; j < 8; j++) s[b0 + goff[j]] = x[j];
                }
                o += cnt;
              }
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
        for (uint32_t i = threadIdx.x; i < tsize; i += kTileThreads)
            tile_store<REP>(state, base + rowoff[i >> sa.L] + (i & lmask), s[i]);
        __syncthreads();
    }
}

static int tile_fail(cudaError_t e, const char* what, std::string* msg) {
    if (msg) *msg = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? QS_OUT_OF_MEMORY : QS_CUDA_ERROR;
}

template <int REP, bool BLK>
static cudaError_t launch_tile(void* state, int n, const TileStage& st, int op_begin, int op_end,
                               const TileOp* dops, const float4* dfrag, cudaStream_t s, int sms) {
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
    const size_t smem = (sizeof(E) << st.T) + (sizeof(uint64_t) << sa.H) + sizeof(TileOp) * size_t(op_end - op_begin);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_tile<REP, BLK>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    const uint64_t ntiles = 1ull << (n - st.T);
    const int per_sm = std::max(1, std::min(8, int((220 * 1024) / smem)));
    const uint64_t grid = std::min<uint64_t>(ntiles, uint64_t(sms) * per_sm);
    k_tile<REP, BLK><<<int(grid), kTileThreads, smem, s>>>(state, ntiles, sa, dops, dfrag);
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
    TileOp* dops = nullptr;
    if (!host.empty()) {
        cudaError_t e = cudaMallocAsync((void**)&dops, host.size() * sizeof(TileOp), s);
        if (e != cudaSuccess) return tile_fail(e, "tile op table", msg);
        e = cudaMemcpyAsync(dops, host.data(), host.size() * sizeof(TileOp), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(dops, s);
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
            if (dops) cudaFreeAsync(dops, s);
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
            case 0: e = launch_tile<0, false>(state, n, st, b, e2, dops, dfrag, s, sms); break;
            case 1: e = launch_tile<1, false>(state, n, st, b, e2, dops, dfrag, s, sms); break;
            case 2: e = launch_tile<2, false>(state, n, st, b, e2, dops, dfrag, s, sms); break;
            default:
                if (dfrag)
                    e = launch_tile<3, true>(state, n, st, b, e2, dops, dfrag, s, sms);
                else
                    e = launch_tile<3, false>(state, n, st, b, e2, dops, dfrag, s, sms);
                break;
        }
        if (e != cudaSuccess) rc = tile_fail(e, "tile kernel", msg);
    }
    if (dops) cudaFreeAsync(dops, s);
    if (dfrag) cudaFreeAsync(dfrag, s);
    return rc;
}

}  // namespace qs
