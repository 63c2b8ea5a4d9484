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
#include "qs_stage.h"
#include "qs_pass.cuh"
#include "qs_tc05.cuh"
#include "qs_tma.cuh"

namespace qs {

constexpr int kTileThreads = 256;

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
__device__ __forceinline__ void dense_pair(const DenseCoef<1>& c, bool real, double2& a, double2& b) {
    if (real) {  // real matrix (H, RY): 2 FMAs per output component instead of 4
        const double2 y0 = cfma_real(c.m[0], a, cfma_real(c.m[2], b, czero<double2>()));
        const double2 y1 = cfma_real(c.m[4], a, cfma_real(c.m[6], b, czero<double2>()));
        a = y0;
        b = y1;
        return;
    }
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

template <int REP>
__device__ __forceinline__ typename TileElem<REP>::T mono_row(const TileOp& m, int r, typename TileElem<REP>::T src) {
    const uint8_t c = m.pf[r];
    if (c == 255) return phase_mul(m.m + 2 * r, src, REP);
    return pf_move(src, c);
}

// ---- fused 5-qubit blocks on the tensor cores (complex64 tiles, 3xTF32)
// x rounded to TF32 (10 explicit significand bits), to nearest with ties away from zero: add half
// a TF32 unit to the magnitude bits and clear the 13 dropped bits (two integer operations; a carry
// into the exponent field is the correct rounding up to the next binade).
__device__ __forceinline__ uint32_t f2tf32(float x) { return (__float_as_uint(x) + 0x1000u) & 0xffffe000u; }

__device__ __forceinline__ int warp_id() { return int(threadIdx.x >> 5); }

// Operand image of a tensor-core block in shared memory (qs_tc05.cuh layout): the block matrix B.
constexpr uint32_t kTcBBytes = 64u * 64u * 4u;   // one B image
constexpr uint32_t kTcLbo = 128u, kTcSbo = 2048u;
// Tensor-memory columns of one group: D (64 FP32 columns), then the A high and low parts.
constexpr uint32_t kTcAHi = 64u, kTcALo = 128u, kTcGroupCols = 256u;

// Complex64 tiles of the tensor-core stages are swizzled at 16-byte granularity (swz16, two
// amplitudes per unit): amplitude t sits at tile_swz(t).
__host__ __device__ __forceinline__ uint32_t tile_swz(uint32_t t) { return (swz16(t >> 1) << 1) | (t & 1u); }

// Float offsets of a block op inside the swizzled tile: column m (the 7 tile bits outside the
// block, 0..127) starts at tab[m]; block row j (0..31) XORs in tab[128 + b] (the swizzled weight of
// block qubit b) for every set bit b of j (the swizzle is linear and the column and row bits are
// disjoint). The real part sits at the offset, the imaginary part one float further. Built once
// per CTA for each block op of the stage.
constexpr int kTcIdxWords = 128 + 8;
__device__ __forceinline__ void block_index_table(const TileOp& op, uint32_t* tab, int nthreads) {
    uint8_t pos[5];
#pragma unroll
    for (int b = 0; b < 5; b++) pos[b] = op.pos[b];
    for (int i = threadIdx.x; i < kTcIdxWords; i += nthreads)
        tab[i] = i < 128 ? 2u * tile_swz(expand_local(uint32_t(i), pos, 5))
                         : (i < 133 ? 2u * tile_swz(1u << pos[i - 128]) : 0u);
}

// Y = U X for the 32-row block view of a 12-qubit complex64 tile on the tensor cores (3xTF32), by
// one group of kTcGroupThreads threads: D = A_lo B_hi + A_hi B_lo + A_hi B_hi accumulated in FP32
// in tensor memory. A (128 x 64) holds the tile's 128 columns (the 7 tile bits outside the block)
// by their 64 real block components (real parts of rows 0..31 in K columns 0..31, imaginary parts
// in 32..63), split once into TF32 high and low parts and stored straight into the group's
// tensor-memory columns; B (64 x 64, the block's [[Ur, -Ui], [Ui, Ur]]) is resident in shared
// memory. Warp w of the group owns tile column (lane) 32 (w % 4) + lane and block rows
// 16 (w / 4) .. + 15, both parts (64-bit shared accesses). One thread issues the 24 MMAs and
// commits them to `bar`; the group then reads D back into the tile. False when the bounded wait
// for the MMAs gave up (*abort is set and the tile is left unchanged).
constexpr int kTcGroupThreads = 256;
__device__ __forceinline__ bool block_apply_tc(float* sf, const uint32_t* tab, const float* sb, uint64_t* bar,
                                               uint32_t* parity, uint32_t tcol, int gt, int barrier_id,
                                               int* abort) {
    const int gw = gt >> 5, lane = gt & 31;
    const uint32_t quarter = uint32_t(gw & 3) << 21;  // lane base 32 (w % 4), in bits 16.. of the address
    const uint32_t kc = 16u * uint32_t(gw >> 2);     // this warp's rows, as K (and D) columns
    const uint32_t col = tab[32 * (gw & 3) + lane] ^ ((gw >> 2) ? tab[132] : 0u);
    uint32_t w[4];
#pragma unroll
    for (int b = 0; b < 4; b++) w[b] = tab[128 + b];
    {
        float hre[16], him[16], lre[16], lim[16];
        uint32_t r = col;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            if (i > 0) r ^= w[low_bit(i)];
            const float2 a = *reinterpret_cast<const float2*>(sf + r);
            const int j = gray_code(i);
            hre[j] = __uint_as_float(f2tf32(a.x));
            lre[j] = __uint_as_float(f2tf32(a.x - hre[j]));
            him[j] = __uint_as_float(f2tf32(a.y));
            lim[j] = __uint_as_float(f2tf32(a.y - him[j]));
        }
        const uint32_t ta = tcol + quarter + kc;
        tc_st16_nowait(ta + kTcAHi, hre);
        tc_st16_nowait(ta + kTcAHi + 32u, him);
        tc_st16_nowait(ta + kTcALo, lre);
        tc_st16_nowait(ta + kTcALo + 32u, lim);
        tc_wait_st();
    }
    tc_fence_before();
    named_sync(barrier_id, kTcGroupThreads);
    tc_fence_after();
    if (gt == 0) {
        constexpr uint32_t idesc = tc_idesc_tf32(128, 64);
        const uint32_t bh = saddr(sb), bl = bh + kTcBBytes;
#pragma unroll 1
        for (uint32_t ks = 0; ks < 8; ks++) {  // K = 8 per MMA
            const uint32_t o = ks * 2u * kTcLbo;
            tc_mma_tf32_ta(tcol, tcol + kTcALo + 8u * ks, tc_smem_desc(bh + o, kTcLbo, kTcSbo), idesc, ks);
            tc_mma_tf32_ta(tcol, tcol + kTcAHi + 8u * ks, tc_smem_desc(bl + o, kTcLbo, kTcSbo), idesc, 1);
            tc_mma_tf32_ta(tcol, tcol + kTcAHi + 8u * ks, tc_smem_desc(bh + o, kTcLbo, kTcSbo), idesc, 1);
        }
        tc_commit(bar);
    }
    // One warp polls the barrier; the group barrier releases the other warps without spinning.
    if (gt < 32 && !mbar_wait_bounded(bar, *parity) && gt == 0) *abort = 1;
    *parity ^= 1u;
    tc_fence_before();
    named_sync(barrier_id, kTcGroupThreads);
    tc_fence_after();
    const bool ok = *abort == 0;
    if (ok) {
        uint32_t vre[16], vim[16];
        tc_ld16_nowait(tcol + quarter + kc, vre);
        tc_ld16_nowait(tcol + quarter + kc + 32u, vim);
        tc_wait_ld();
        uint32_t r = col;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            if (i > 0) r ^= w[low_bit(i)];
            const int j = gray_code(i);
            *reinterpret_cast<float2*>(sf + r) = make_float2(__uint_as_float(vre[j]), __uint_as_float(vim[j]));
        }
    }
    tc_fence_before();
    named_sync(barrier_id, kTcGroupThreads);
    tc_fence_after();
    return ok;
}

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
template <int REP>
__global__ void __launch_bounds__(kTileThreads, 2) k_tile(void* __restrict__ state, uint64_t ntiles,
                                                       const __grid_constant__ StageArgs sa,
                                                       const TileOp* __restrict__ ops, int* __restrict__ err) {
    using E = typename TileElem<REP>::T;
    using GE = typename GlobElem<REP>::T;
    static_assert(sizeof(E) == sizeof(GE), "tile element and state element must have the same size");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t tsize = 1u << sa.T;
    E* bufs = reinterpret_cast<E*>(smem_raw);
    const int nrows = 1 << sa.RH, nbuf = sa.nbuf;
    const int nops = sa.op_end - sa.op_begin;
    // [tile buffers][nbuf mbarriers, padded to 32 bytes][ops (16-byte aligned)][row offsets]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + size_t(nbuf) * (sizeof(E) << sa.T));
    TileOp* sops = reinterpret_cast<TileOp*>(mbar + 4);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(sops + nops);
    __shared__ int s_abort;
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ops + sa.op_begin);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sops);
        const int words = nops * int(sizeof(TileOp) / 4);
        for (int w = threadIdx.x; w < words; w += kTileThreads) dst[w] = src[w];
    }
    for (int r = threadIdx.x; r < nrows; r += kTileThreads) {
        uint64_t o = 0;
        for (int b = 0; b < sa.RH; b++)
            if (r >> b & 1) o |= 1ull << sa.rhigh[b];
        rowoff[r] = o;
    }
    // Long rows (at most 8 per tile): warp 0 moves the tile with bulk copies. Short
    // rows: each bulk copy costs the copy engine ~90 cycles, so all threads move the tile in 16-byte
    // pieces (cp.async in, shared loads + global stores out), two tiles ahead in a ring of three.
    const bool bulk = nrows <= 8;
    if (threadIdx.x == 0) {
        for (int b = 0; b < nbuf; b++) mbar_init(&mbar[b], bulk ? 1 : kTileThreads);
        fence_mbar_init();
        s_abort = 0;
    }
    __syncthreads();
    const uint64_t first = blockIdx.x;
    const uint64_t nmy = (ntiles > first) ? (ntiles - 1 - first) / gridDim.x + 1 : 0;
    const uint32_t row_bytes = uint32_t(sizeof(GE)) << sa.RL;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    GE* gstate = static_cast<GE*>(state);
    constexpr uint32_t kPer = 16 / sizeof(GE);  // amplitudes per 16-byte piece
    const uint32_t rmask = (1u << sa.RL) - 1u, pieces = tsize / kPer;
    auto issue_load = [&](uint64_t i, int b) {  // bulk: warp 0 only; pieces: every thread
        const uint64_t tb = expand_index(first + i * gridDim.x, sa.outer);
        GE* dst = reinterpret_cast<GE*>(bufs + size_t(b) * tsize);
        if (bulk) {
            if (lane == 0) mbar_expect_tx(&mbar[b], row_bytes * uint32_t(nrows));
            __syncwarp();
            for (int r = lane; r < nrows; r += 32)
                bulk_load(dst + (size_t(r) << sa.RL), gstate + tb + rowoff[r], row_bytes, &mbar[b]);
        } else {
            for (uint32_t c = threadIdx.x; c < pieces; c += kTileThreads) {
                const uint32_t a = c * kPer;
                cp_async16(dst + a, gstate + tb + rowoff[a >> sa.RL] + (a & rmask));
            }
            cp_async_mbar_arrive(&mbar[b]);
        }
    };
    const int ahead = bulk ? 1 : nbuf - 1;  // tiles in flight beyond the one being computed
    if (bulk) {
        if (warp == 0 && nmy > 0) issue_load(0, 0);
    } else {
        for (int k = 0; k < ahead && uint64_t(k) < nmy; k++) issue_load(uint64_t(k), k);
    }
    uint64_t it = 0;
    int bsel = 0;          // buffer of tile it
    uint32_t phase = 0;    // bit b: parity of buffer b's next completion
    for (; it < nmy; it++) {
        E* s = bufs + size_t(bsel) * tsize;
        const uint64_t base = expand_index(first + it * gridDim.x, sa.outer);
        if (bulk) {
            if (warp == 0 && it + 1 < nmy) {
                // Tile it + 1 reuses the buffer of tile it + 1 - nbuf, whose stores were committed
                // nbuf - 1 groups ago: wait until those have read shared memory.
                if (nbuf == 3)
                    bulk_wait_read<1>();
                else
                    bulk_wait_read<0>();
                __syncwarp();
                issue_load(it + 1, bsel + 1 == nbuf ? 0 : bsel + 1);
            }
        } else if (it + ahead < nmy) {
            // tile it + ahead takes the buffer of tile it + ahead - nbuf = it - 1, written back at
            // the end of the previous iteration by the same threads that now load into it
            int nb = bsel + ahead;
            if (nb >= nbuf) nb -= nbuf;
            issue_load(it + ahead, nb);
        }
        if (!mbar_wait_bounded(&mbar[bsel], (phase >> bsel) & 1u)) atomicOr(&s_abort, 1);
        phase ^= 1u << bsel;
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
            if (REP == 3 && kind == OP_PASS) {
                if constexpr (REP == 3) pass_run_c64(reinterpret_cast<float2*>(s), tsize, &base, &sops[o]);
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
        if (bulk) {
            fence_async_shared();  // make this tile's shared-memory writes visible to the bulk stores
            __syncthreads();
            if (warp == 0) {
                for (int r = lane; r < nrows; r += 32)
                    bulk_store(gstate + base + rowoff[r], s + (size_t(r) << sa.RL), row_bytes);
                bulk_commit();
            }
        } else {
            __syncthreads();
            const GE* src = reinterpret_cast<const GE*>(s);
            for (uint32_t c = threadIdx.x; c < pieces; c += kTileThreads) {
                const uint32_t a = c * kPer;
                *reinterpret_cast<float4*>(gstate + base + rowoff[a >> sa.RL] + (a & rmask)) =
                    *reinterpret_cast<const float4*>(src + a);
            }
        }
        bsel = bsel + 1 == nbuf ? 0 : bsel + 1;
    }
    if (bulk) {
        if (warp == 0) bulk_wait_all();
        if (s_abort && threadIdx.x == 0) {
            atomicExch(err, 1);
            // the load of tile it + 1 may still be in flight: wait for it (bounded) before exiting
            const int nb = bsel + 1 == nbuf ? 0 : bsel + 1;
            if (it + 1 < nmy) mbar_wait_bounded(&mbar[nb], (phase >> nb) & 1u);
        }
    } else {
        cp_async_wait_all();  // copies of tiles the loop did not reach
        if (s_abort && threadIdx.x == 0) atomicExch(err, 1);
    }
}

static int tile_fail(cudaError_t e, const char* what, std::string* msg) {
    if (msg) *msg = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? QS_OUT_OF_MEMORY : QS_CUDA_ERROR;
}

template <int REP>
static cudaError_t launch_tile(void* state, int n, const TileStage& st, int op_begin, int op_end,
                               const TileOp* dops, int* derr, cudaStream_t s, int sms) {
    using E = typename TileElem<REP>::T;
    StageArgs sa = stage_args(st, op_begin, op_end);
    const size_t tile_bytes = sizeof(E) << st.T;
    const size_t fixed = 4 * sizeof(uint64_t) + sizeof(TileOp) * size_t(op_end - op_begin) +
                         (sizeof(uint64_t) << sa.RH);
    sa.nbuf = (3 * tile_bytes + fixed <= 110 * 1024) ? 3 : 2;  // three buffers where two blocks still fit an SM
    const size_t smem = size_t(sa.nbuf) * tile_bytes + fixed;
    const uint64_t ntiles = 1ull << (n - st.T);
    // One wave exactly: every CTA walks the same number of tiles, so a grid larger than what is
    // resident would leave a second, partly empty wave.
    int per_sm = 0;
    cudaError_t oe = resident_blocks(reinterpret_cast<const void*>(k_tile<REP>), kTileThreads, smem, &per_sm);
    if (oe != cudaSuccess) return oe;
    per_sm = std::max(1, per_sm);
    const uint64_t grid = std::min<uint64_t>(ntiles, uint64_t(sms) * per_sm);
    k_tile<REP><<<int(grid), kTileThreads, smem, s>>>(state, ntiles, sa, dops, derr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launches(1);
    return e;
}

// ---- tensor-core block stages (complex64, 12-qubit tiles, only OP_BLOCK ops) ------------------
// Two groups of kTcGroupThreads threads per CTA walk their own tiles (two tile buffers each, the
// next tile's 16-byte pieces in flight while the current one is computed) and their own
// tensor-memory columns; the stage's block operands are loaded once per CTA and shared. While one
// group waits for its MMAs, the other builds its operands or moves its tiles.
constexpr int kTcGroups = 2;
constexpr int kTcThreads = kTcGroups * kTcGroupThreads;

__global__ void __launch_bounds__(kTcThreads, 1) k_tile_tc(float2* __restrict__ state, uint64_t ntiles,
                                                          const __grid_constant__ StageArgs sa,
                                                          const TileOp* __restrict__ ops,
                                                          const float4* __restrict__ bfrag, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_tc[];
    unsigned char* smem_raw = smem_tc;
    const int nops = sa.op_end - sa.op_begin;
    const uint32_t tsize = 1u << sa.T;
    const int nrows = 1 << sa.RH;
    // [B images, 32 KiB per op][tiles: kTcGroups x 2][index tables][ops][row offsets][mbarriers][tmem]
    float* sB = reinterpret_cast<float*>(smem_raw);
    float2* tiles = reinterpret_cast<float2*>(smem_raw + size_t(nops) * 2 * kTcBBytes);
    uint32_t* tabs = reinterpret_cast<uint32_t*>(tiles + size_t(2 * kTcGroups) * tsize);
    TileOp* sops = reinterpret_cast<TileOp*>(tabs + size_t(nops) * kTcIdxWords);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(sops + nops);
    uint64_t* bars = rowoff + nrows;  // [0]: B copy; [1 + g]: group g's MMAs; [1 + kTcGroups + 2g + b]: tile loads
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1 + 3 * kTcGroups);
    __shared__ int s_abort[kTcGroups];
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ops + sa.op_begin);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sops);
        const int words = nops * int(sizeof(TileOp) / 4);
        for (int w = threadIdx.x; w < words; w += kTcThreads) dst[w] = src[w];
    }
    for (int r = threadIdx.x; r < nrows; r += kTcThreads) {
        uint64_t o = 0;
        for (int b = 0; b < sa.RH; b++)
            if (r >> b & 1) o |= 1ull << sa.rhigh[b];
        rowoff[r] = o;
    }
    if (threadIdx.x < 32) tc_alloc(tslot, kTcGroups * kTcGroupCols);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        for (int g = 0; g < kTcGroups; g++) {
            mbar_init(&bars[1 + g], 1);
            mbar_init(&bars[1 + kTcGroups + 2 * g], kTcGroupThreads);
            mbar_init(&bars[2 + kTcGroups + 2 * g], kTcGroupThreads);
            s_abort[g] = 0;
        }
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    for (int o = 0; o < nops; o++) block_index_table(sops[o], tabs + o * kTcIdxWords, kTcThreads);
    if (threadIdx.x == 0) {  // the stage's block operands, loaded once per CTA
        mbar_expect_tx(&bars[0], uint32_t(nops) * 2u * kTcBBytes);
        for (int o = 0; o < nops; o++)
            bulk_load(sB + size_t(o) * 2 * kTcBBytes / 4, bfrag + size_t(sops[o].bidx) * kBlockFragFloat4,
                      2 * kTcBBytes, &bars[0]);
    }
    const bool b_ok = mbar_wait_bounded(&bars[0], 0);
    __syncthreads();
    const int g = threadIdx.x / kTcGroupThreads, gt = threadIdx.x % kTcGroupThreads;
    const int barrier_id = 1 + g;
    if (!b_ok && gt == 0) s_abort[g] = 1;
    const uint64_t gid = uint64_t(blockIdx.x) * kTcGroups + uint64_t(g), ngroups = uint64_t(gridDim.x) * kTcGroups;
    const uint64_t nmy = ntiles > gid ? (ntiles - 1 - gid) / ngroups + 1 : 0;
    float2* gbuf = tiles + size_t(2 * g) * tsize;
    uint64_t* lbar = &bars[1 + kTcGroups + 2 * g];
    const uint32_t rmask = (1u << sa.RL) - 1u, pieces = tsize / 2;  // 16-byte pieces: two amplitudes
    // The pieces of this thread, 2 (gt + 256 k), share tile bits 4..8, so their swizzle is one XOR.
    const uint32_t swz = tile_swz(2u * uint32_t(gt)) ^ (2u * uint32_t(gt));
    auto issue_load = [&](uint64_t i, int b) {
        const uint64_t tb = expand_index(gid + i * ngroups, sa.outer);
        float2* dst = gbuf + size_t(b) * tsize;
        for (uint32_t c = uint32_t(gt); c < pieces; c += kTcGroupThreads) {
            const uint32_t a = 2 * c;
            cp_async16(dst + (a ^ swz), state + tb + rowoff[a >> sa.RL] + (a & rmask));
        }
        cp_async_mbar_arrive(&lbar[b]);
    };
    if (nmy > 0 && b_ok) issue_load(0, 0);
    uint32_t lphase = 0, mma_parity = 0;
    const uint32_t tcol = tmem + uint32_t(g) * kTcGroupCols;
    for (uint64_t it = 0; it < nmy && b_ok; it++) {
        const int bsel = int(it & 1);
        if (it + 1 < nmy) issue_load(it + 1, bsel ^ 1);  // that buffer's tile was written back last iteration
        if (gt < 32 && !mbar_wait_bounded(&lbar[bsel], (lphase >> bsel) & 1u) && gt == 0) s_abort[g] = 1;
        lphase ^= 1u << bsel;
        named_sync(barrier_id, kTcGroupThreads);  // releases the warps that did not poll
        if (s_abort[g]) break;
        float* sf = reinterpret_cast<float*>(gbuf + size_t(bsel) * tsize);
        for (int o = 0; o < nops && !s_abort[g]; o++) {
            block_apply_tc(sf, tabs + o * kTcIdxWords, sB + size_t(o) * 2 * kTcBBytes / 4, &bars[1 + g],
                           &mma_parity, tcol, gt, barrier_id, &s_abort[g]);
        }
        const uint64_t base = expand_index(gid + it * ngroups, sa.outer);
        const float2* src = gbuf + size_t(bsel) * tsize;
        for (uint32_t c = uint32_t(gt); c < pieces; c += kTcGroupThreads) {
            const uint32_t a = 2 * c;
            *reinterpret_cast<float4*>(state + base + rowoff[a >> sa.RL] + (a & rmask)) =
                *reinterpret_cast<const float4*>(src + (a ^ swz));
        }
        named_sync(barrier_id, kTcGroupThreads);  // the buffer is free for the load two tiles ahead
    }
    cp_async_wait_all();  // copies of tiles the loop did not reach
    if (gt == 0 && (s_abort[g] || !b_ok)) atomicExch(err, 1);
    tc_fence_before();
    __syncthreads();  // both groups are done with tensor memory
    tc_fence_after();
    if (threadIdx.x < 32) tc_dealloc(tmem, kTcGroups * kTcGroupCols);
}

static cudaError_t launch_tile_tc(void* state, int n, const TileStage& st, int op_begin, int op_end,
                                  const TileOp* dops, const float4* dfrag, int* derr, cudaStream_t s, int sms) {
    const StageArgs sa = stage_args(st, op_begin, op_end);
    const int nops = op_end - op_begin;
    const size_t tile_bytes = sizeof(float2) << st.T;
    const size_t smem = size_t(nops) * 2 * kTcBBytes + size_t(2 * kTcGroups) * tile_bytes +
                        size_t(nops) * 4 * kTcIdxWords + sizeof(TileOp) * size_t(nops) + (sizeof(uint64_t) << sa.RH) +
                        sizeof(uint64_t) * (1 + 3 * kTcGroups) + 16;
    const uint64_t ntiles = 1ull << (n - st.T);
    int per_sm = 0;
    cudaError_t oe = resident_blocks(reinterpret_cast<const void*>(k_tile_tc), kTcThreads, smem, &per_sm);
    if (oe != cudaSuccess) return oe;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint64_t groups = (ntiles + kTcGroups - 1) / kTcGroups;
    const uint64_t grid = std::min<uint64_t>(groups, uint64_t(sms));  // one CTA per SM: its tensor memory
    k_tile_tc<<<int(grid), kTcThreads, smem, s>>>(static_cast<float2*>(state), ntiles, sa, dops, dfrag, derr);
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
              const std::vector<float>* block_frags, int* derr_dev) {
    // tile arithmetic: exact order, FP64 FMA (also for QS_ARITH_FX64, whose one-gate sweeps are
    // fixed-point), double-float, complex64
    int rep = (prec == QS_PREC_C64) ? 3 : (arith == QS_ARITH_EXACT ? 0 : (arith == QS_ARITH_DF64 ? 2 : 1));
    if (rep == 2)
        for (const auto& op : ops)
            if (!df64_range_ok(op)) rep = 1;  // entries outside double-float range: FP64 FMA instead
    std::vector<TileOp> host;
    std::vector<int> first(stages.size(), 0);
    std::vector<char> passes(stages.size(), 0);
    for (size_t i = 0; i < stages.size(); i++) {
        first[i] = int(host.size());
        if (!stages[i].tiled) continue;
        // Register passes pay off where shared-memory traffic dominates (complex64); the
        // FP64 and double-float tiles are arithmetic-bound and keep one pass per gate.
        const std::vector<TileOp> prog = stage_program(ops, stages[i], rep == 3);
        passes[i] = rep == 3 && pass_only(prog);
        for (const TileOp& t : prog) host.push_back(t);
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
        derr = derr_dev ? derr_dev : reinterpret_cast<int*>(dblob + ops_bytes);
        if (!derr_dev) e = cudaMemsetAsync(derr, 0, sizeof(int), s);
        if (e == cudaSuccess && !host.empty()) {
            const size_t bytes = host.size() * sizeof(TileOp);
            void* stage = pinned_staging(0, bytes);
            if (stage) std::memcpy(stage, host.data(), bytes);
            e = cudaMemcpyAsync(dops, stage ? stage : host.data(), bytes, cudaMemcpyHostToDevice, s);
        }
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
        if (dfrag && prec == QS_PREC_C128) {
            e = launch_tile_oz(state, n, st, b, e2, dops, reinterpret_cast<const unsigned char*>(dfrag), derr, s, sms);
            if (e != cudaSuccess) rc = tile_fail(e, "tile kernel", msg);
            continue;
        }
        switch (rep) {
            case 0: e = launch_tile<0>(state, n, st, b, e2, dops, derr, s, sms); break;
            case 1: e = launch_tile<1>(state, n, st, b, e2, dops, derr, s, sms); break;
            case 2: e = launch_tile<2>(state, n, st, b, e2, dops, derr, s, sms); break;
            default:
                if (dfrag)
                    e = launch_tile_tc(state, n, st, b, e2, dops, dfrag, derr, s, sms);
                else if (passes[i])
                    e = launch_pass(state, n, st, b, e2, dops, derr, s, sms);
                else
                    e = launch_tile<3>(state, n, st, b, e2, dops, derr, s, sms);
                break;
        }
        if (e != cudaSuccess) rc = tile_fail(e, "tile kernel", msg);
    }
    if (rc == QS_OK && !derr_dev) {  // a bounded wait inside a tile kernel that gave up is reported here
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
