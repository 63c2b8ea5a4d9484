// qs_tile_oz.cu — FP64-accurate fused 5-qubit blocks on complex128 registers, on the tensor cores.
//
// A stage applies one fused 5-qubit block U (32 x 32 complex, multiplied on the host in FP64) to
// every 12-qubit tile of a complex128 state. In its real form the block is a 64 x 64 product
// Y = X B per tile, X = the tile's 128 columns (the 7 tile bits outside the block) by their 64 real
// block components. The product runs as exact integer arithmetic on the BF16 tensor cores
// (an Ozaki-style split):
//
//  * every tile column m is scaled by the power of two of its largest component and rounded to a
//    55-bit integer X (|X| <= 2^55); every output column n of B likewise, to |Y| <= 2^54 (host);
//  * both are cut into 7 balanced base-256 digits, X = sum_s a_s 256^(6-s), Y = sum_t b_t 256^(6-t),
//    |a_s|, |b_t| <= 128 (top digits: 128 and 64), stored as BF16 values a_s 2^-8s, b_t 2^-8t
//    (exact: at most 8 significant bits);
//  * tcgen05.mma kind::f16 sums the digit products in FP32 accumulators in tensor memory, one per
//    level L = s + t for L <= 4 and one for L = 5, 6 together; the products of level L >= 7 are
//    dropped. The level sums I_L = sum_k sum_{s+t=L} a_s b_t are integers below 2^23 for L <= 4, so
//    those accumulators hold I_L 2^-8L exactly; the last one rounds at 2^-24 of terms below 2^-40;
//  * R = 2^36 sum_L acc_L, assembled in 64-bit integers, is X.Y / 2^60 to within 8 units (the
//    dropped levels cost at most 6.1, the tail's rounding and FP32 accumulation the rest); it is
//    rounded once to double and scaled by the two powers of two.
//
// The error of an output is at most ulp/2 + 2^(EE-1078) sum_k |u_k| + 2^(F-55) sum_k |x_k| (the
// operand roundings: about 2^-54 max|x| sum|u| + 2^-55 max|u| sum|x|) + 8 units of R (each below
// 2^-46 max|x| max|u|); an FP64 FMA chain over the same 64 terms has a worst case of about
// 2^-47 sum_k |u_k x_k|. Columns with a non-finite amplitude take an FP64 path (the block's FP64
// real form).
//
// One CTA per SM (its 512 tensor-memory columns: six 64-column accumulators and four 32-column
// slots that A slices stream through) runs a warp-specialised pipeline over its tiles:
//  * 16 math warps: warp w owns tile column 32 (w % 4) + lane (its tensor-memory lane) and block
//    rows 8 (w / 4) .. + 7 (K elements 16 (w / 4) .. + 15). Per tile they encode the column, write
//    its 7 slices into the slots (each slot handed over by an mbarrier: "full" when the 16 warps
//    have stored it, "free" when the MMAs that read it have completed), drain the previous tile's
//    accumulators into 64-bit integers while the current tile's first slices wait, and finish the
//    previous tile (rounding, scaling, stores straight from registers to the state) while the
//    current tile's MMAs run;
//  * one MMA warp: one thread issues each slice's MMAs as soon as the slice is stored (and, for a
//    tile's first slice, the previous tile's accumulators are drained) and commits them to the
//    slot's "free" barrier and, after the last slice, to "accumulators full".
// A tile is loaded by 16-byte cp.async pieces into one of two buffers one tile ahead; the only
// barrier among the math warps per tile is the exchange of the column exponents, which also marks
// the moment every read of the older buffer is done. Every wait is bounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qs_device.cuh"
#include "qs_kernels.h"
#include "qs_pass.cuh"
#include "qs_stage.h"
#include "qs_tc05.cuh"
#include "qs_tile.h"
#include "qs_tma.cuh"

namespace qs {

namespace {

constexpr int kOzMathWarps = 16;
constexpr int kOzMath = 32 * kOzMathWarps;   // math threads; the two MMA warps follow them
constexpr int kOzIssuers = 2;                // MMA warps: levels 0..4, and the tail (levels 5..6)
constexpr int kOzThreads = kOzMath + 32 * kOzIssuers;
constexpr int kOzRows = 8;                   // block rows per math thread
constexpr int kOzAcc = 6;                    // accumulators: levels 0..4, then 5..6
constexpr int kOzSlots = 4;                  // A slots in tensor memory
constexpr uint32_t kOzASlot = 64u * kOzAcc;  // tensor-memory column of A slot 0 (slot j: + 32 j)
constexpr uint32_t kOzTmemCols = 512u;
constexpr int kOzIdxWords = 128 + 16;
// mbarriers: B operand, tile loads (2), slot full (4), slot free (4), accumulators full / drained,
// final MMA completion
constexpr int kBarB = 0, kBarLoad = 1, kBarFull = 3, kBarFree = 7, kBarAccFull = 11, kBarAccFree = 12,
              kBarDone = 13, kOzBars = 14;
constexpr long long kOzBias = 0x808080808080LL;  // X + bias: digits 1..6 are bytes - 128
constexpr float kMagic = 12582912.0f;            // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

// Xb = X + kOzBias for X = round(|v| 2^(1077 - EE)) with the sign of v, for EE = max(largest
// exponent field of the column, 1) >= v's exponent field: the significand with its implicit bit,
// shifted left by 2 and right by EE - e with rounding to nearest (ties away from zero); |X| < 2^55.
// The sign and the bias go in together: X + bias = (|X| ^ sg) + (bias - sg) for sg = 0 or -1.
__device__ __forceinline__ long long oz_encode_biased(double v, uint32_t EE) {
    const uint32_t hi = uint32_t(__double2hiint(v)), lo = uint32_t(__double2loint(v));
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const uint32_t d = min(EE - max(e, 1u), 63u);
    // 2m = significand << 3 (< 2^56); X = ((2m >> d) + 1) >> 1 rounds m / 2^d to nearest
    const uint64_t m2 = ((uint64_t((hi & 0xfffffu) | (min(e, 1u) << 20)) << 32) | lo) << 3;
    const uint64_t X = ((m2 >> d) + 1u) >> 1;
    const long long sg = (long long)(int32_t(hi) >> 31);  // 0 or -1
    return ((long long)X ^ sg) + (kOzBias - sg);
}

// Digit s of Xb = X + kOzBias as a float, scaled by 2^-8s (s = 0: the signed top part Xb >> 48;
// s >= 1: byte 6 - s minus 128, placed under the float 2^(23-8s) by a byte permute and recovered
// by one exact subtraction).
template <int S>
__device__ __forceinline__ uint32_t oz_digit_bits(long long Xb) {
    if constexpr (S == 0) {
        const int d = int(uint32_t(uint64_t(Xb) >> 32)) >> 16;
        return __float_as_uint(__int_as_float(kMagicBits + d) - kMagic);
    } else {
        constexpr int i = 6 - S;
        constexpr uint32_t magic = uint32_t(150 - 8 * S) << 23;  // 2^(23 - 8 S)
        const uint32_t word = i < 4 ? uint32_t(uint64_t(Xb)) : uint32_t(uint64_t(Xb) >> 32);
        const uint32_t bits = __byte_perm(word, magic, 0x7650u | uint32_t(i & 3));
        return __float_as_uint(__uint_as_float(bits) - __uint_as_float(magic | 0x80u));
    }
}

// Slice S of the thread's 16 K elements (row r: real part at 2r, imaginary at 2r + 1), packed as
// BF16 pairs (element 2c in the low half of column c).
template <int S>
__device__ __forceinline__ void oz_slice(const long long (&X)[2 * kOzRows], uint32_t (&pk)[kOzRows]) {
#pragma unroll
    for (int c = 0; c < kOzRows; c++)
        pk[c] = __byte_perm(oz_digit_bits<S>(X[2 * c]), oz_digit_bits<S>(X[2 * c + 1]), 0x7632u);
}

// a * b + c with a 64-bit addend and result (one wide multiply-add).
__device__ __forceinline__ long long mad_wide(int a, int b, long long c) {
    long long d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// R = 2^36 (acc_0 + ... + acc_5) as an integer: levels 0..3 through the magic-number conversion
// (|I_L| < 2^22: i_L = bits(acc_L 2^8L + 1.5 2^23) - bits(1.5 2^23)), level 4 by a rounding
// conversion (|I_4| < 2^23), the tail rounded at 2^-36;
// R = (i0 256 + i1) 2^28 + (i2 256 + i3) 2^12 + i4 2^4 + t, the magic constants folded into one
// subtraction per partial sum (arithmetic modulo 2^32; the sums fit in 31 bits).
__device__ __forceinline__ long long oz_combine(float a0, float a1, float a2, float a3, float a4, float a5) {
    const uint32_t b0 = __float_as_uint(a0 + kMagic);
    const uint32_t b1 = __float_as_uint(fmaf(a1, 256.0f, kMagic));
    const uint32_t b2 = __float_as_uint(fmaf(a2, 65536.0f, kMagic));
    const uint32_t b3 = __float_as_uint(fmaf(a3, 16777216.0f, kMagic));
    const int i4 = __float2int_rn(a4 * 4294967296.0f);
    const uint32_t bt = __float_as_uint(fmaf(a5, 68719476736.0f, kMagic));
    constexpr uint32_t kM257 = 257u * uint32_t(kMagicBits);
    const int j01 = int(b0 * 256u + b1 - kM257);  // i0 256 + i1, |j01| < 2^30 + 2^22
    const int j23 = int(b2 * 256u + b3 - kM257);  // i2 256 + i3
    const int low = int(uint32_t(i4) * 16u + bt - uint32_t(kMagicBits));  // i4 16 + t, |low| < 2^28
    return mad_wide(j01, 1 << 28, mad_wide(j23, 1 << 12, (long long)low));
}

__device__ __forceinline__ double oz_to_double(long long R, int k) {
    return (k >= kFxFastKMin && k <= kFxFastKMax) ? fx_to_double_fast(R, k << 20) : fx_to_double_any(R, k);
}

// R 2^k for kk = k << 20, k in [kFxFastKMin, kFxFastKMax] (the exponent field stays normal): a
// non-zero integer converts to |d| >= 1, so a zero high word means R = 0 (and the result +0).
__device__ __forceinline__ double oz_scale_fast(long long R, int kk) {
    const double d = __ll2double_rn(R);
    const int h = __double2hiint(d);
    return __hiloint2double(h != 0 ? h + kk : 0, __double2loint(d));
}

// Wait for the phase of `parity`, suspending between polls (the hint bounds each suspension; the
// thread resumes when the phase completes), at most `limit` SM clocks; false if the wait gave up.
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, long long limit = 4000000000LL) {
    const uint32_t a = saddr(bar);
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity), "r"(10000000u)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > limit) return false;
    }
}

// The MMAs of A slice S (tensor-memory columns from aslot) against every B slice t with S + t <= 6
// whose level accumulator belongs to MMA warp ISSUER: issuer 0 levels 0..4, issuer 1 the tail
// (levels 5..6). Each accumulator has one issuer, so its MMAs keep their order (the reset first,
// then the accumulations). Descriptor of B slice 0: bdesc0; slice t and K step ks start
// (8192 t + 256 ks) bytes further, an offset the descriptor's 14-bit start-address field absorbs
// without carry. A tile's first slice starts levels 0..5 afresh (level 5 at t = 5, before t = 6
// adds to it). K step outermost, so consecutive MMAs go to different accumulators. Unrolled per
// slice: every offset and accumulate flag is a constant.
template <int S, int ISSUER>
__device__ __forceinline__ void oz_issue_slice(uint32_t tmem, uint32_t aslot, uint64_t bdesc0) {
    constexpr uint32_t idesc = tc_idesc_bf16(128, 64);
#pragma unroll
    for (uint32_t ks = 0; ks < 4; ks++)  // K = 16 per MMA
#pragma unroll
        for (int t = 0; t + S < kOzSlices; t++)
            if ((S + t < kOzAcc - 1) == (ISSUER == 0))
                tc_mma_f16_ta(tmem + 64u * uint32_t(min(S + t, kOzAcc - 1)), aslot + 8u * ks,
                              bdesc0 + ((uint64_t(t) * kOzSliceBytes + 256u * ks) >> 4), idesc,
                              (S > 0 || ks > 0 || t == kOzSlices - 1) ? 1u : 0u);
}

// Wait for the phase of `parity` with short sleeps between polls (the math warps: their polls would
// otherwise take issue slots from the warps that share their scheduler), at most `limit` SM clocks;
// false if the wait gave up.
__device__ __forceinline__ bool mbar_wait_nap(uint64_t* bar, uint32_t parity, long long limit = 4000000000LL) {
    const long long t0 = clock64();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        __nanosleep(40);
        if (clock64() - t0 > limit) return false;
    }
}

// Amplitude offset (16-byte units, swizzled) of block row j of this thread's column.
__device__ __forceinline__ uint32_t oz_row(uint32_t col0, const uint32_t* tab, int j) {
    uint32_t r = col0;
#pragma unroll
    for (int b = 0; b < 5; b++)
        if (j >> b & 1) r ^= tab[128 + b];
    return r;
}

// Barrier among the 16 math warps (hardware barrier 1) that also ORs `flag` over them.
__device__ __forceinline__ bool math_sync_or(bool flag) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(uint32_t(flag)), "n"(kOzMath)
        : "memory");
    return r != 0;
}

// Columns with a non-finite amplitude: the thread's 16 outputs in FP64 from the column's 64 inputs
// (all four row groups, read from the tile buffer, which no load refills before the next tile's
// exponent exchange) and the block's FP64 real form, stored straight to the state (dst = the
// tile's base). Rolled loops, so the common path keeps its registers.
__device__ __noinline__ void oz_rare_column(const double2* tl, const uint32_t* tab, int m, int g, const double* bd,
                                            double2* dst, const uint64_t* rowoff, uint32_t rmask, int RL,
                                            uint32_t lrow0) {
#pragma unroll 1
    for (int i = 0; i < kOzRows; i++) {
        double y[2];
#pragma unroll 1
        for (int c = 0; c < 2; c++) {
            const int nidx = 2 * (kOzRows * g + i) + c;
            double acc = 0.0;
#pragma unroll 1
            for (int j = 0; j < 32; j++) {
                const double2 v = tl[oz_row(tab[m], tab, j)];
                acc = fma(bd[nidx * 64 + 2 * j], v.x, acc);
                acc = fma(bd[nidx * 64 + 2 * j + 1], v.y, acc);
            }
            y[c] = acc;
        }
        uint32_t l = lrow0;
#pragma unroll 1
        for (int b = 0; b < 3; b++)
            if (i >> b & 1) l ^= tab[136 + b];
        dst[rowoff[l >> RL] + (l & rmask)] = make_double2(y[0], y[1]);
    }
}

__global__ void __launch_bounds__(kOzThreads, 1)
    k_tile_oz(double2* __restrict__ state, uint64_t ntiles, const __grid_constant__ StageArgs sa,
              const TileOp* __restrict__ ops, const unsigned char* __restrict__ frag, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_oz[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t tsize = 1u << sa.T;
    const int nrows = 1 << sa.RH;
    // [B slices][output exponents][tiles x 2][index table][op][row offsets][exponents x 2][bars][tmem]
    unsigned char* sB = smem_oz;
    const int* sscale = reinterpret_cast<const int*>(smem_oz + kOzBBytes);
    double2* tiles = reinterpret_cast<double2*>(smem_oz + kOzBBytes + kOzScaleBytes);
    uint32_t* tab = reinterpret_cast<uint32_t*>(tiles + 2 * size_t(tsize));
    TileOp* sop = reinterpret_cast<TileOp*>(tab + kOzIdxWords);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(sop + 1);
    uint32_t* ex = reinterpret_cast<uint32_t*>(rowoff + nrows);
    uint64_t* bars = reinterpret_cast<uint64_t*>(ex + 2 * kOzMath);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kOzBars);
    __shared__ int s_abort;
    __shared__ int s_srange[2];  // smallest and largest output exponent
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ops + sa.op_begin);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sop);
        for (int w = tid; w < int(sizeof(TileOp) / 4); w += kOzThreads) dst[w] = src[w];
    }
    for (int r = tid; r < nrows; r += kOzThreads) {
        uint64_t o = 0;
        for (int b = 0; b < sa.RH; b++)
            if (r >> b & 1) o |= 1ull << sa.rhigh[b];
        rowoff[r] = o;
    }
    if (warp == kOzMathWarps) tc_alloc(tslot, kOzTmemCols);  // the first MMA warp
    if (tid == 0) {
        mbar_init(&bars[kBarB], 1);
        for (int b = 0; b < 2; b++) mbar_init(&bars[kBarLoad + b], kOzMath);
        for (int j = 0; j < kOzSlots; j++) {
            mbar_init(&bars[kBarFull + j], kOzMathWarps);
            mbar_init(&bars[kBarFree + j], kOzIssuers);  // one commit per MMA warp
        }
        mbar_init(&bars[kBarAccFull], kOzIssuers);
        mbar_init(&bars[kBarAccFree], kOzMathWarps);
        mbar_init(&bars[kBarDone], kOzIssuers);
        fence_mbar_init();
        s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    {
        // [0, 128): swizzled tile unit of column i's row 0; [128, 133): swizzled unit offset of block
        // qubit b; [136, 141): the same offsets unswizzled (tile-local amplitude bits)
        uint8_t pos[5];
#pragma unroll
        for (int b = 0; b < 5; b++) pos[b] = sop->pos[b];
        for (int i = tid; i < kOzIdxWords; i += kOzThreads)
            tab[i] = i < 128   ? swz16(expand_local(uint32_t(i), pos, 5))
                     : i < 133 ? swz16(1u << pos[i - 128])
                     : (i >= 136 && i < 141) ? (1u << pos[i - 136])
                                             : 0u;
    }
    const unsigned char* bfrag = frag + size_t(sop->bidx) * kOzFragBytes;
    if (tid == 0) {  // the block's slices and output exponents, once per CTA
        mbar_expect_tx(&bars[kBarB], kOzBBytes + kOzScaleBytes);
        for (int s = 0; s < kOzSlices; s++)
            bulk_load(sB + s * kOzSliceBytes, bfrag + s * kOzSliceBytes, kOzSliceBytes, &bars[kBarB]);
        bulk_load(sB + kOzBBytes, bfrag + kOzBBytes, kOzScaleBytes, &bars[kBarB]);
    }
    if (warp == 0 && !mbar_wait_bounded(&bars[kBarB], 0) && lane == 0) s_abort = 1;
    __syncthreads();
    if (tid == 0) {
        int lo = sscale[0], hi = sscale[0];
        for (int n = 1; n < 64; n++) {
            lo = min(lo, sscale[n]);
            hi = max(hi, sscale[n]);
        }
        s_srange[0] = lo;
        s_srange[1] = hi;
    }
    __syncthreads();
    const double* bd = reinterpret_cast<const double*>(bfrag + kOzBBytes + kOzScaleBytes);

    const uint64_t first = blockIdx.x, stride = gridDim.x;
    const uint64_t nmy = ntiles > first ? (ntiles - 1 - first) / stride + 1 : 0;
    const uint32_t rmask = (1u << sa.RL) - 1u;

    if (warp >= kOzMathWarps) {
        // ---- the MMA warps: slice s of a tile against every B slice t with s + t <= 6, issuer 0 into
        // levels 0..4 (60 MMAs per tile), issuer 1 into the tail (52), each on its own scheduler
        const int issuer = warp - kOzMathWarps;
        if (lane == 0) {
            bool ok = s_abort == 0;
            const uint64_t bdesc0 = tc_smem_desc(saddr(sB), 128u, 1024u);
            for (uint64_t it = 0; ok && it < nmy; it++) {
                for (int s = 0; s < kOzSlices; s++) {
                    const uint64_t u = uint64_t(kOzSlices) * it + uint64_t(s);
                    const uint32_t slot = uint32_t(u & 3u);
                    if (!mbar_wait_sleep(&bars[kBarFull + slot], uint32_t((u >> 2) & 1u))) {
                        ok = false;
                        break;
                    }
                    // a tile's first MMAs overwrite the accumulators: the previous tile's must be drained
                    if (s == 0 && it > 0 && !mbar_wait_sleep(&bars[kBarAccFree], uint32_t((it - 1) & 1u))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t aslot = tmem + kOzASlot + 32u * slot;
                    switch (s) {
                        case 0: issuer ? oz_issue_slice<0, 1>(tmem, aslot, bdesc0) : oz_issue_slice<0, 0>(tmem, aslot, bdesc0); break;
                        case 1: issuer ? oz_issue_slice<1, 1>(tmem, aslot, bdesc0) : oz_issue_slice<1, 0>(tmem, aslot, bdesc0); break;
                        case 2: issuer ? oz_issue_slice<2, 1>(tmem, aslot, bdesc0) : oz_issue_slice<2, 0>(tmem, aslot, bdesc0); break;
                        case 3: issuer ? oz_issue_slice<3, 1>(tmem, aslot, bdesc0) : oz_issue_slice<3, 0>(tmem, aslot, bdesc0); break;
                        case 4: issuer ? oz_issue_slice<4, 1>(tmem, aslot, bdesc0) : oz_issue_slice<4, 0>(tmem, aslot, bdesc0); break;
                        case 5: issuer ? oz_issue_slice<5, 1>(tmem, aslot, bdesc0) : oz_issue_slice<5, 0>(tmem, aslot, bdesc0); break;
                        default: issuer ? oz_issue_slice<6, 1>(tmem, aslot, bdesc0) : oz_issue_slice<6, 0>(tmem, aslot, bdesc0); break;
                    }
                    tc_commit(&bars[kBarFree + slot]);
                    if (s == kOzSlices - 1) tc_commit(&bars[kBarAccFull]);
                }
            }
            tc_commit(&bars[kBarDone]);  // arrives once every MMA issued above has completed
            if (!mbar_wait_sleep(&bars[kBarDone], 0)) ok = false;
            if (!ok) s_abort = 1;
        }
        __syncwarp();
    } else {
        // ---- the math warps
        bool bad = s_abort != 0;
        const int q = warp & 3, g = warp >> 2, m = 32 * q + lane;  // row group g: block rows 8 g .. 8 g + 7
        const uint32_t quarter = uint32_t(32 * q) << 16;
        const uint32_t col0 = tab[m] ^ ((g & 1) ? tab[131] : 0u) ^ ((g & 2) ? tab[132] : 0u);  // row 8 g
        const uint32_t lrow0 = swz16(col0);  // the swizzle is its own inverse
        uint32_t w[3], ub[3];
#pragma unroll
        for (int b = 0; b < 3; b++) {
            w[b] = tab[128 + b];
            ub[b] = tab[136 + b];
        }
        const uint32_t ta = tmem + quarter + kOzASlot + uint32_t(kOzRows * g);
        // The pieces of this thread, tid + 512 k, share unit bits 3..7, so their swizzle is one XOR.
        const uint32_t swz = swz16(uint32_t(tid)) ^ uint32_t(tid);
        // load tile i into buffer b; returns the tile's base amplitude index
        auto issue_load = [&](uint64_t i, int b) -> uint64_t {
            const uint64_t tb = expand_index(first + i * stride, sa.outer);
            double2* dst = tiles + size_t(b) * tsize;
            const double2* src = state + tb;
            for (uint32_t c = uint32_t(tid); c < tsize; c += kOzMath)
                cp_async16(dst + (c ^ swz), src + rowoff[c >> sa.RL] + (c & rmask));
            cp_async_mbar_arrive(&bars[kBarLoad + b]);
            return tb;
        };

        // slice s of tile `it` into slot (7 it + s) % 4, once the MMAs that read that slot last are done
        auto put = [&](uint64_t it, int s, const uint32_t(&pk)[kOzRows]) {
            const uint64_t u = uint64_t(kOzSlices) * it + uint64_t(s);
            const uint32_t slot = uint32_t(u & 3u);
            if (u >= uint64_t(kOzSlots) && !bad &&
                !mbar_wait_nap(&bars[kBarFree + slot], uint32_t(((u >> 2) - 1u) & 1u)))
                bad = true;
            __syncwarp();
            tc_fence_after();
            tc_st8u_nowait(ta + 32u * slot, pk);
            tc_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars[kBarFull + slot]);
        };
        // R = the previous tile's outputs as integers (row 8 g + i: R[2 i] real, R[2 i + 1] imaginary)
        long long R[2 * kOzRows];
        auto drain = [&](uint64_t itp) {
            if (!bad && !mbar_wait_nap(&bars[kBarAccFull], uint32_t(itp & 1u))) bad = true;
            __syncwarp();
            tc_fence_after();
#pragma unroll
            for (int i = 0; i < kOzRows; i++) {  // one row (two D columns) at a time
                uint32_t a[kOzAcc][2];
#pragma unroll
                for (int L = 0; L < kOzAcc; L++)
                    tc_ld2_nowait(tmem + quarter + 64u * L + uint32_t(2 * kOzRows * g) + 2u * i, a[L]);
                tc_wait_ld();
#pragma unroll
                for (int e = 0; e < 2; e++)
                    R[2 * i + e] = oz_combine(__uint_as_float(a[0][e]), __uint_as_float(a[1][e]),
                                              __uint_as_float(a[2][e]), __uint_as_float(a[3][e]),
                                              __uint_as_float(a[4][e]), __uint_as_float(a[5][e]));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars[kBarAccFree]);
        };
        // the previous tile's outputs: rounded once, scaled, stored in place
        auto finish = [&](uint64_t base, int kE, bool rare) {
            if (rare) return;  // the FP64 path has stored this column
            double2* dst = state + base;
            const int* ss = sscale + 2 * kOzRows * g;
            // a column exponent that keeps every output exponent in the fast conversion range
            const bool fast = kE + s_srange[0] >= kFxFastKMin && kE + s_srange[1] <= kFxFastKMax;
            uint32_t l = lrow0;
#pragma unroll
            for (int i = 0; i < kOzRows; i++) {
                if (i > 0) l ^= ub[low_bit(i)];
                const int r = gray_code(i);
                double2 y;
                if (fast) {
                    y.x = oz_scale_fast(R[2 * r], (kE + ss[2 * r]) << 20);
                    y.y = oz_scale_fast(R[2 * r + 1], (kE + ss[2 * r + 1]) << 20);
                } else {
                    y.x = oz_to_double(R[2 * r], kE + ss[2 * r]);
                    y.y = oz_to_double(R[2 * r + 1], kE + ss[2 * r + 1]);
                }
                dst[rowoff[l >> sa.RL] + (l & rmask)] = y;
            }
        };

        uint64_t base_next = (nmy > 0 && !bad) ? issue_load(0, 0) : 0;
        uint64_t base_prev = 0;
        int kE_prev = 1;
        bool rare_prev = false, left = false;
        for (uint64_t it = 0; it < nmy; it++) {
            const int b = int(it & 1u);
            if (!bad && !mbar_wait_nap(&bars[kBarLoad + b], uint32_t((it >> 1) & 1u))) bad = true;
            const double2* tl = tiles + size_t(b) * tsize;

            // the column's exponent over this thread's 8 amplitudes (read again to encode them below)
            uint32_t emax = 0;
            {
                uint32_t r = col0;
#pragma unroll
                for (int i = 0; i < kOzRows; i++) {
                    if (i > 0) r ^= w[low_bit(i)];
                    const double2 v = tl[r];
                    emax = max(emax, max(fx_efield(v.x), fx_efield(v.y)));
                }
            }
            uint32_t* exb = ex + uint32_t(it & 1u) * kOzMath;
            exb[g * 128 + m] = emax;
            // Every math thread has read its amplitudes of tile it - 1 (and its FP64 columns) before
            // this barrier, so that buffer takes the next load; a wait that gave up ends the loop here.
            if (math_sync_or(bad)) {
                left = true;
                break;
            }
            const uint64_t base = base_next;
            if (it + 1 < nmy) base_next = issue_load(it + 1, b ^ 1);
            emax = max(max(exb[m], exb[128 + m]), max(exb[256 + m], exb[384 + m]));
            const bool rare = emax == 0x7ffu;
            if (rare) oz_rare_column(tl, tab, m, g, bd, state + base, rowoff, rmask, sa.RL, lrow0);

            long long X[2 * kOzRows];
            {
                const uint32_t EE = max(emax, 1u);
                uint32_t r = col0;
#pragma unroll
                for (int i = 0; i < kOzRows; i++) {
                    if (i > 0) r ^= w[low_bit(i)];
                    const double2 v = tl[r];
                    const int j = gray_code(i);
                    X[2 * j] = rare ? kOzBias : oz_encode_biased(v.x, EE);
                    X[2 * j + 1] = rare ? kOzBias : oz_encode_biased(v.y, EE);
                }
            }
            uint32_t pk[kOzRows];
            oz_slice<0>(X, pk);
            put(it, 0, pk);
            oz_slice<1>(X, pk);
            put(it, 1, pk);
            oz_slice<2>(X, pk);
            put(it, 2, pk);
            oz_slice<3>(X, pk);
            put(it, 3, pk);
            if (it > 0) {
                drain(it - 1);  // frees the accumulators for this tile's MMAs
                finish(base_prev, kE_prev, rare_prev);  // overlaps this tile's first MMAs
            }
            oz_slice<4>(X, pk);
            put(it, 4, pk);
            oz_slice<5>(X, pk);
            put(it, 5, pk);
            oz_slice<6>(X, pk);
            put(it, 6, pk);
            base_prev = base;
            kE_prev = int(max(emax, 1u));
            rare_prev = rare;
        }
        if (!left && nmy > 0) {
            drain(nmy - 1);
            finish(base_prev, kE_prev, rare_prev);
        }
        cp_async_wait_all();  // copies of tiles the loop did not reach
        if (bad) s_abort = 1;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0 && s_abort) atomicExch(err, 1);
    if (warp == kOzMathWarps) tc_dealloc(tmem, kOzTmemCols);
}

}  // namespace

cudaError_t launch_tile_oz(void* state, int n, const TileStage& st, int op_begin, int op_end, const TileOp* dops,
                           const unsigned char* frag, int* derr, cudaStream_t s, int sms) {
    if (op_end - op_begin != 1 || st.T != 12) return cudaErrorInvalidValue;
    const StageArgs sa = stage_args(st, op_begin, op_end);
    const size_t tile_bytes = sizeof(double2) << st.T;
    const size_t smem = kOzBBytes + kOzScaleBytes + 2 * tile_bytes + 4 * size_t(kOzIdxWords) + sizeof(TileOp) +
                        (sizeof(uint64_t) << sa.RH) + 2 * kOzMath * 4 + kOzBars * sizeof(uint64_t) + 16;
    const uint64_t ntiles = 1ull << (n - st.T);
    int per_sm = 0;
    cudaError_t oe = resident_blocks(reinterpret_cast<const void*>(k_tile_oz), kOzThreads, smem, &per_sm);
    if (oe != cudaSuccess) return oe;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint64_t grid = std::min<uint64_t>(ntiles, uint64_t(sms));  // one CTA per SM: its tensor memory
    k_tile_oz<<<int(grid), kOzThreads, smem, s>>>(static_cast<double2*>(state), ntiles, sa, dops, frag, derr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launches(1);
    return e;
}

// Balanced base-256 digits of Y (|Y| <= 2^54), most significant first: Y = sum_t d[t] 256^(6-t).
static void oz_digits(long long Y, int (&d)[kOzSlices]) {
    const long long Yb = Y + kOzBias;
    for (int i = 0; i < 6; i++) d[6 - i] = int((Yb >> (8 * i)) & 255) - 128;
    d[0] = int(Yb >> 48);
}

static uint16_t bf16_exact(double v) {  // v has at most 8 significant bits
    const float f = float(v);
    uint32_t bits;
    std::memcpy(&bits, &f, 4);
    return uint16_t(bits >> 16);
}

void oz_fragments(const std::vector<double>& u, unsigned char* out) {
    // real form: input component k = 2j + c, output component n = 2i + c'
    auto B = [&](int n, int k) -> double {
        const int i = n >> 1, j = k >> 1;
        const double re = u[2 * (i * 32 + j)], im = u[2 * (i * 32 + j) + 1];
        const bool out_im = n & 1, in_im = k & 1;
        if (out_im == in_im) return re;
        return out_im ? im : -im;  // yi += Ui xr; yr -= Ui xi
    };
    std::memset(out, 0, kOzFragBytes);
    int32_t* scale = reinterpret_cast<int32_t*>(out + kOzBBytes);
    double* bd = reinterpret_cast<double*>(out + kOzBBytes + kOzScaleBytes);
    for (int n = 0; n < 64; n++) {
        double mx = 0.0;
        for (int k = 0; k < 64; k++) mx = std::max(mx, std::fabs(B(n, k)));
        int F = 0;
        if (mx > 0.0) std::frexp(mx, &F);
        scale[n] = F - 1071;
        for (int k = 0; k < 64; k++) {
            const double v = B(n, k);
            bd[n * 64 + k] = v;
            const long long Y = std::llrint(std::ldexp(v, 54 - F));
            int d[kOzSlices];
            oz_digits(Y, d);
            for (int t = 0; t < kOzSlices; t++) {
                const uint16_t h = bf16_exact(std::ldexp(double(d[t]), -8 * t));
                std::memcpy(out + t * kOzSliceBytes + tc_kmajor_off16(uint32_t(n), uint32_t(k), 8u), &h, 2);
            }
        }
    }
}

}  // namespace qs
