// qs_state.cu — state-wide kernels: initialisation, measurement, read-back.
//
// Measurement replaces the two scalar passes of Register::try_measure
// (src/register.rs:306-339): a deterministic FP64 reduction of |a|^2 split by
// the target bit (fixed grid, warp shuffles, fixed-order block and grid
// combination), the outcome decision on the host, then one collapse sweep.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "qs_device.cuh"
#include "qs_kernels.h"

namespace qs {

static inline cudaError_t counted(cudaError_t e, uint64_t launches = 1) {
    if (e == cudaSuccess) note_launches(launches);
    return e;
}

constexpr int kT = 256;

static int grid_cap(uint64_t work, int sms, int per_thread = 1) {
    uint64_t b = (work + uint64_t(kT) * per_thread - 1) / (uint64_t(kT) * per_thread);
    uint64_t cap = uint64_t(sms) * 32;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return int(b);
}

__device__ __forceinline__ double2 to_d2(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2(float2 v) { return make_double2(double(v.x), double(v.y)); }
// Reductions and the collapse read complex64 amplitudes through an integer-pipe conversion: the FP64
// pipe (~1/64 of the FP32 rate on GB300) is left to the sums and quotients themselves. Exact for
// every float (subnormals take a rare branch), so the values equal double(v).
__device__ __forceinline__ double2 to_d2_int(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2_int(float2 v) { return make_double2(df_f2d(v.x), df_f2d(v.y)); }
__device__ __forceinline__ void from_d2(double2* dst, double2 v) { *dst = v; }
__device__ __forceinline__ void from_d2(float2* dst, double2 v) { *dst = make_float2(float(v.x), float(v.y)); }

// ---------------------------------------------------------------- initialisation
template <typename T>
__global__ void __launch_bounds__(kT) k_init_basis(T* __restrict__ st, uint64_t N, uint64_t index) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < N; i += stride) {
        double2 v = make_double2(i == index ? 1.0 : 0.0, 0.0);
        from_d2(&st[i], v);
    }
}

struct ProductArgs {
    int n;
    double q[64][4];  // qubit j: (re0, im0, re1, im1)
};

// Register::try_from_qubits folds kron(q_j, acc) from qubit 0 upwards
// (src/register.rs:91-96); amplitude i is q_{n-1}[b] * (... * (q_0[b] * 1)),
// each product rounded as num-complex does.
template <typename T>
__global__ void __launch_bounds__(kT) k_init_product(T* __restrict__ st, uint64_t N,
                                                     const __grid_constant__ ProductArgs a) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < N; i += stride) {
        double2 acc = make_double2(1.0, 0.0);
        for (int j = 0; j < a.n; j++) {
            const int b = int((i >> j) & 1ull);
            acc = cmul_exact(a.q[j][2 * b], a.q[j][2 * b + 1], acc);
        }
        from_d2(&st[i], acc);
    }
}

cudaError_t launch_init_basis(void* state, int n, int prec, uint64_t index, cudaStream_t s, int sms) {
    const uint64_t N = 1ull << n;
    if (prec == QS_PREC_C64)
        k_init_basis<float2><<<grid_cap(N, sms), kT, 0, s>>>((float2*)state, N, index);
    else
        k_init_basis<double2><<<grid_cap(N, sms), kT, 0, s>>>((double2*)state, N, index);
    return counted(cudaGetLastError());
}

// One doubling level of the same fold: the partial product after qubits 0..j-1 depends only on the
// low j bits of the index, so st[0, half) holding those partials becomes
// st[b * half + k] = q_j[b] * st[k] for b = 0, 1: the very products the per-amplitude loop forms at
// step j, computed once per partial instead of once per amplitude.
__global__ void __launch_bounds__(kT) k_product_level(double2* __restrict__ st, uint64_t half, double q0r, double q0i,
                                                      double q1r, double q1i) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t k = uint64_t(blockIdx.x) * kT + threadIdx.x; k < half; k += stride) {
        const double2 v = st[k];
        st[k + half] = cmul_exact(q1r, q1i, v);
        st[k] = cmul_exact(q0r, q0i, v);
    }
}

cudaError_t launch_init_product(void* state, int n, int prec, const double* qubits, cudaStream_t s, int sms) {
    ProductArgs a;
    std::memset(&a, 0, sizeof(a));
    // complex128: the first 16 qubits per amplitude, the rest by doubling levels (2^(n+1) products
    // in all instead of n * 2^n). complex64 keeps the whole product in double and rounds it once.
    const int n0 = (prec == QS_PREC_C64) ? n : std::min(n, 16);
    a.n = n0;
    for (int j = 0; j < n0; j++)
        for (int c = 0; c < 4; c++) a.q[j][c] = qubits[4 * j + c];
    const uint64_t N0 = 1ull << n0;
    if (prec == QS_PREC_C64) {
        k_init_product<float2><<<grid_cap(N0, sms), kT, 0, s>>>((float2*)state, N0, a);
        return counted(cudaGetLastError());
    }
    k_init_product<double2><<<grid_cap(N0, sms), kT, 0, s>>>((double2*)state, N0, a);
    cudaError_t e = counted(cudaGetLastError());
    for (int j = n0; j < n && e == cudaSuccess; j++) {
        const uint64_t half = 1ull << j;
        const double* q = qubits + 4 * j;
        k_product_level<<<grid_cap(half, sms), kT, 0, s>>>((double2*)state, half, q[0], q[1], q[2], q[3]);
        e = counted(cudaGetLastError());
    }
    return e;
}

// ---------------------------------------------------------------- measurement
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of (a, b) in a fixed order; result valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double sa[kT / 32], sb[kT / 32];
    a = warp_sum(a);
    b = warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int i = 0; i < kT / 32; i++) {
            ta += sa[i];
            tb += sb[i];
        }
        a = ta;
        b = tb;
    }
}

// A measurement visits the pairs (i0, i0 | tb) of its target inside the register's live subspace:
// amplitudes whose collapsed qubits (earlier measurements, no gate on them since) differ from the
// recorded outcomes are exact zeros, so they add nothing to a probability sum and a collapse leaves
// them as they are. The pair index t expands to i0 with the target bit 0 and the collapsed bits at
// their values.
static IndexMap subspace_map(int target, uint64_t zmask, uint64_t zval) {
    IndexMap m;
    std::memset(&m, 0, sizeof(m));
    const uint64_t pos = (zmask & ~(1ull << target)) | (1ull << target);
    int k = 0;
    for (int b = 0; b < 64; b++)
        if (pos >> b & 1ull) m.pos[k++] = uint8_t(b);
    m.npos = k;
    m.fixval = zval & zmask & ~(1ull << target);
    return m;
}

static uint64_t subspace_pairs(int n, int target, uint64_t zmask) {
    return 1ull << (n - 1 - __builtin_popcountll(zmask & ~(1ull << target)));
}

template <typename T>
__global__ void __launch_bounds__(kT) k_prob_partials(const T* __restrict__ st, uint64_t npairs, uint64_t tb,
                                                      const __grid_constant__ IndexMap map,
                                                      double* __restrict__ partials) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    double p0 = 0.0, p1 = 0.0;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < npairs; t += stride) {
        const uint64_t i0 = expand_index(t, map);
        const double2 a = to_d2_int(st[i0]);
        const double2 b = to_d2_int(st[i0 | tb]);
        p0 = fma(a.x, a.x, p0);
        p0 = fma(a.y, a.y, p0);
        p1 = fma(b.x, b.x, p1);
        p1 = fma(b.y, b.y, p1);
    }
    block_sum2(p0, p1);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = p0;
        partials[2 * blockIdx.x + 1] = p1;
    }
}

__global__ void __launch_bounds__(kT) k_prob_final(const double* __restrict__ partials, int nblocks,
                                                   double* __restrict__ out) {
    double p0 = 0.0, p1 = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kT) {
        p0 += partials[2 * b];
        p1 += partials[2 * b + 1];
    }
    block_sum2(p0, p1);
    if (threadIdx.x == 0) {
        out[0] = p0;
        out[1] = p1;
    }
}

// The probability sums in the reference's order (src/register.rs:306-315): norm_sqr = re*re + im*im
// rounded per operation, added to prob_0 or prob_1 one amplitude after another in index order. One
// block stages chunks of amplitudes in shared memory; the bit-0 and bit-1 chains are independent
// sums and run on two threads. Amplitudes outside the live subspace are exact zeros, which leave a
// running sum unchanged, so only the subspace is read.
constexpr int kSeqChunk = 2048;
__global__ void __launch_bounds__(kT) k_prob_sequential(const double2* __restrict__ st, uint64_t count, int target,
                                                        const __grid_constant__ IndexMap map,
                                                        double* __restrict__ out) {
    __shared__ double pr[kSeqChunk];
    __shared__ uint8_t bit[kSeqChunk];
    double acc = 0.0;  // thread 0: prob_0, thread 32: prob_1
    for (uint64_t base = 0; base < count; base += kSeqChunk) {
        const int len = int(count - base < uint64_t(kSeqChunk) ? count - base : uint64_t(kSeqChunk));
        for (int j = threadIdx.x; j < len; j += kT) {
            const uint64_t i = expand_index(base + uint64_t(j), map);
            const double2 a = st[i];
            pr[j] = __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y));
            bit[j] = uint8_t((i >> target) & 1ull);
        }
        __syncthreads();
        if (threadIdx.x == 0 || threadIdx.x == 32) {
            const uint8_t want = threadIdx.x == 32 ? 1 : 0;
            for (int j = 0; j < len; j++)
                if (bit[j] == want) acc = __dadd_rn(acc, pr[j]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = acc;
    if (threadIdx.x == 32) out[1] = acc;
}

cudaError_t launch_measure_probs(const void* state, int n, int prec, int target, double* partials,
                                 int max_partials, double* out, cudaStream_t s, int sms, uint64_t zmask,
                                 uint64_t zval, bool sequential) {
    const IndexMap map = subspace_map(target, zmask, zval);
    const uint64_t npairs = subspace_pairs(n, target, zmask);
    const uint64_t tb = 1ull << target;
    if (sequential && prec == QS_PREC_C128) {
        // every amplitude of the subspace in index order: the free bits are all bits but the
        // collapsed ones (the target's bit is free here)
        IndexMap all;
        std::memset(&all, 0, sizeof(all));
        int k = 0;
        const uint64_t fixed = zmask & ~tb;
        for (int b = 0; b < 64; b++)
            if (fixed >> b & 1ull) all.pos[k++] = uint8_t(b);
        all.npos = k;
        all.fixval = zval & fixed;
        k_prob_sequential<<<1, kT, 0, s>>>((const double2*)state, 2 * npairs, target, all, out);
        return counted(cudaGetLastError());
    }
    int grid = grid_cap(npairs, sms, 4);
    if (grid > max_partials) grid = max_partials;
    if (prec == QS_PREC_C64)
        k_prob_partials<float2><<<grid, kT, 0, s>>>((const float2*)state, npairs, tb, map, partials);
    else
        k_prob_partials<double2><<<grid, kT, 0, s>>>((const double2*)state, npairs, tb, map, partials);
    k_prob_final<<<1, kT, 0, s>>>(partials, grid, out);
    return counted(cudaGetLastError(), 2);
}

// x / d for the kept half. With rinv = RN(1/d), q = RN(x * rinv) is within
// one ulp of x/d, and Markstein's correction (r = x - q*d exactly by FMA,
// q' = RN(q + r*rinv); P. Markstein, IBM J. Res. Dev. 34(1), 1990) rounds
// it to the correctly rounded quotient, the value Rust's `/` gives.
__device__ __forceinline__ double div_markstein(double x, double d, double rinv) {
    const double q = x * rinv;
    const double r = fma(-q, d, x);
    return fma(r, rinv, q);
}

// How the kept amplitudes are divided by d = sqrt(total): the correctly rounded quotient (Markstein's
// step; what Rust's `/` gives, for registers in the reference's arithmetic), a true division (when
// RN(1/d) is not usable), or one multiply by RN(1/d), within one ulp of the quotient (registers in
// the other arithmetic forms, held to 1e-14: GB300's FP64 pipe bounds a collapse, and this form
// takes 2 FP64 operations per amplitude instead of 6).
constexpr int kDivMarkstein = 0, kDivTrue = 1, kDivMul = 2;

// The kept amplitude divided by sqrt(total) (src/register.rs:337), in the state's type.
template <typename T, int DIV>
__device__ __forceinline__ T collapse_value(T v, double d, double rinv, double2* as_double) {
    if constexpr (sizeof(T) == 8 && DIV != kDivTrue) {
        // complex64: one FP64 multiply by RN(1/d) per component, rounded to float on the integer
        // pipe (the quotient is stored as a float, so the exactly rounded double quotient of the
        // complex128 path buys nothing here)
        const double2 x = to_d2_int(v);
        const T y{d2f_int(x.x * rinv), d2f_int(x.y * rinv)};
        *as_double = make_double2(df_f2d(y.x), df_f2d(y.y));
        return y;
    } else {
        const double2 x = to_d2_int(v);
        double2 y;
        if constexpr (DIV == kDivTrue) {
            y.x = x.x / d;
            y.y = x.y / d;
        } else if constexpr (DIV == kDivMul) {
            y.x = x.x * rinv;
            y.y = x.y * rinv;
        } else {
            y.x = div_markstein(x.x, d, rinv);
            y.y = div_markstein(x.y, d, rinv);
        }
        T r;
        from_d2(&r, y);
        *as_double = to_d2_int(r);
        return r;
    }
}

template <typename T, int DIV>
__global__ void __launch_bounds__(kT) k_collapse(T* __restrict__ st, uint64_t npairs, uint64_t tb,
                                                 const __grid_constant__ IndexMap map, int outcome, double d,
                                                 double rinv) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < npairs; t += stride) {
        const uint64_t i0 = expand_index(t, map);
        const uint64_t keep = outcome ? (i0 | tb) : i0, drop = outcome ? i0 : (i0 | tb);
        double2 unused;
        st[keep] = collapse_value<T, DIV>(st[keep], d, rinv, &unused);
        st[drop] = T{0, 0};
    }
}

// The collapse of one measurement fused with the probability sums of the next one (measure_circuit,
// src/register.rs:371-377): the kept amplitudes, once divided, are the only non-zero amplitudes the
// next target sees, so their squares are summed by that target's bit in the same pass.
template <typename T, int DIV>
__global__ void __launch_bounds__(kT) k_collapse_probs(T* __restrict__ st, uint64_t npairs, uint64_t tb,
                                                       const __grid_constant__ IndexMap map, int outcome, double d,
                                                       double rinv, uint64_t next_tb, double* __restrict__ partials) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    double p0 = 0.0, p1 = 0.0;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < npairs; t += stride) {
        const uint64_t i0 = expand_index(t, map);
        const uint64_t keep = outcome ? (i0 | tb) : i0, drop = outcome ? i0 : (i0 | tb);
        double2 y;
        st[keep] = collapse_value<T, DIV>(st[keep], d, rinv, &y);
        st[drop] = T{0, 0};
        const double q = fma(y.x, y.x, y.y * y.y);
        if (keep & next_tb)
            p1 += q;
        else
            p0 += q;
    }
    block_sum2(p0, p1);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = p0;
        partials[2 * blockIdx.x + 1] = p1;
    }
}

static int div_mode(double d, double rinv, bool exact_quotient) {
    // Markstein's step and the multiply need a finite reciprocal of a normal divisor.
    if (!(std::isfinite(rinv) && d > 1e-300 && std::isfinite(d))) return kDivTrue;
    return exact_quotient ? kDivMarkstein : kDivMul;
}

template <typename T, int DIV>
static void collapse_t(void* state, uint64_t npairs, uint64_t tb, const IndexMap& map, int outcome, double d,
                       double rinv, int grid, cudaStream_t s) {
    k_collapse<T, DIV><<<grid, kT, 0, s>>>((T*)state, npairs, tb, map, outcome, d, rinv);
}

template <typename T, int DIV>
static void collapse_probs_t(void* state, uint64_t npairs, uint64_t tb, const IndexMap& map, int outcome, double d,
                             double rinv, uint64_t ntb, double* partials, int grid, cudaStream_t s) {
    k_collapse_probs<T, DIV><<<grid, kT, 0, s>>>((T*)state, npairs, tb, map, outcome, d, rinv, ntb, partials);
}

cudaError_t launch_collapse(void* state, int n, int prec, int target, int outcome, double d, double rinv,
                            cudaStream_t s, int sms, uint64_t zmask, uint64_t zval, bool exact_quotient) {
    const IndexMap map = subspace_map(target, zmask, zval);
    const uint64_t npairs = subspace_pairs(n, target, zmask);
    const uint64_t tb = 1ull << target;
    const int grid = grid_cap(npairs, sms, 2);
    const int mode = div_mode(d, rinv, exact_quotient);
    if (prec == QS_PREC_C64) {  // complex64 multiplies by RN(1/d) unless it must divide
        if (mode == kDivTrue)
            collapse_t<float2, kDivTrue>(state, npairs, tb, map, outcome, d, rinv, grid, s);
        else
            collapse_t<float2, kDivMul>(state, npairs, tb, map, outcome, d, rinv, grid, s);
    } else if (mode == kDivTrue) {
        collapse_t<double2, kDivTrue>(state, npairs, tb, map, outcome, d, rinv, grid, s);
    } else if (mode == kDivMul) {
        collapse_t<double2, kDivMul>(state, npairs, tb, map, outcome, d, rinv, grid, s);
    } else {
        collapse_t<double2, kDivMarkstein>(state, npairs, tb, map, outcome, d, rinv, grid, s);
    }
    return counted(cudaGetLastError());
}

cudaError_t launch_collapse_probs(void* state, int n, int prec, int target, int outcome, double d, double rinv,
                                  int next_target, double* partials, int max_partials, double* out, cudaStream_t s,
                                  int sms, uint64_t zmask, uint64_t zval, bool exact_quotient) {
    const IndexMap map = subspace_map(target, zmask, zval);
    const uint64_t npairs = subspace_pairs(n, target, zmask);
    const uint64_t tb = 1ull << target, ntb = 1ull << next_target;
    int grid = grid_cap(npairs, sms, 2);
    if (grid > max_partials) grid = max_partials;
    const int mode = div_mode(d, rinv, exact_quotient);
    if (prec == QS_PREC_C64) {
        if (mode == kDivTrue)
            collapse_probs_t<float2, kDivTrue>(state, npairs, tb, map, outcome, d, rinv, ntb, partials, grid, s);
        else
            collapse_probs_t<float2, kDivMul>(state, npairs, tb, map, outcome, d, rinv, ntb, partials, grid, s);
    } else if (mode == kDivTrue) {
        collapse_probs_t<double2, kDivTrue>(state, npairs, tb, map, outcome, d, rinv, ntb, partials, grid, s);
    } else if (mode == kDivMul) {
        collapse_probs_t<double2, kDivMul>(state, npairs, tb, map, outcome, d, rinv, ntb, partials, grid, s);
    } else {
        collapse_probs_t<double2, kDivMarkstein>(state, npairs, tb, map, outcome, d, rinv, ntb, partials, grid, s);
    }
    k_prob_final<<<1, kT, 0, s>>>(partials, grid, out);
    return counted(cudaGetLastError(), 2);
}

// ---------------------------------------------------------------- measurement on a compact subspace
// A measurement sequence on a dense state (qs_measure_sequence): after the first collapse the live
// amplitudes are strided through the state (the measured qubits' bits fixed), so in-place passes
// move whole 32-byte sectors for every live 16-byte amplitude. Here each pass instead reads the
// kept half of a buffer whose index runs over the free bits only and writes it, divided, densely
// into the next buffer; the sums of the next target come from the same pass. Every pass visits the
// pairs t in the order and with the grid of k_collapse_probs (the free bits in ascending order, the
// target's bit inserted) and divides as it does, so the sums, outcomes and divided amplitudes are
// bit for bit those of the in-place passes.
template <typename T, int DIV, bool SUMS>
__global__ void __launch_bounds__(kT) k_collapse_compact(const T* __restrict__ src, T* __restrict__ dst,
                                                         uint64_t npairs, const __grid_constant__ IndexMap map,
                                                         uint64_t keepbit, double d, double rinv, uint64_t next_bit,
                                                         double* __restrict__ partials) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    double p0 = 0.0, p1 = 0.0;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < npairs; t += stride) {
        double2 y;
        dst[t] = collapse_value<T, DIV>(src[expand_index(t, map) | keepbit], d, rinv, &y);
        if constexpr (SUMS) {
            const double q = fma(y.x, y.x, y.y * y.y);
            if (t & next_bit)
                p1 += q;
            else
                p0 += q;
        }
    }
    if constexpr (SUMS) {
        block_sum2(p0, p1);
        if (threadIdx.x == 0) {
            partials[2 * blockIdx.x] = p0;
            partials[2 * blockIdx.x + 1] = p1;
        }
    }
}

template <typename T, int DIV>
static void collapse_compact_t(const void* src, void* dst, uint64_t npairs, const IndexMap& map, uint64_t keepbit,
                               double d, double rinv, int next_pos, double* partials, int grid, cudaStream_t s) {
    if (next_pos >= 0)
        k_collapse_compact<T, DIV, true><<<grid, kT, 0, s>>>((const T*)src, (T*)dst, npairs, map, keepbit, d, rinv,
                                                             1ull << next_pos, partials);
    else
        k_collapse_compact<T, DIV, false><<<grid, kT, 0, s>>>((const T*)src, (T*)dst, npairs, map, keepbit, d, rinv,
                                                              0ull, partials);
}

cudaError_t launch_collapse_compact(const void* src, void* dst, int nfree, int prec, int pos, int outcome, double d,
                                    double rinv, int next_pos, double* partials, int max_partials, double* out,
                                    cudaStream_t s, int sms, bool exact_quotient) {
    const IndexMap map = subspace_map(pos, 0, 0);
    const uint64_t npairs = 1ull << (nfree - 1);
    const uint64_t keepbit = outcome ? (1ull << pos) : 0ull;
    int grid = grid_cap(npairs, sms, 2);
    if (next_pos >= 0 && grid > max_partials) grid = max_partials;  // the in-place pass's grid
    const int mode = div_mode(d, rinv, exact_quotient);
    if (prec == QS_PREC_C64) {
        if (mode == kDivTrue)
            collapse_compact_t<float2, kDivTrue>(src, dst, npairs, map, keepbit, d, rinv, next_pos, partials, grid, s);
        else
            collapse_compact_t<float2, kDivMul>(src, dst, npairs, map, keepbit, d, rinv, next_pos, partials, grid, s);
    } else if (mode == kDivTrue) {
        collapse_compact_t<double2, kDivTrue>(src, dst, npairs, map, keepbit, d, rinv, next_pos, partials, grid, s);
    } else if (mode == kDivMul) {
        collapse_compact_t<double2, kDivMul>(src, dst, npairs, map, keepbit, d, rinv, next_pos, partials, grid, s);
    } else {
        collapse_compact_t<double2, kDivMarkstein>(src, dst, npairs, map, keepbit, d, rinv, next_pos, partials, grid,
                                                   s);
    }
    if (next_pos < 0) return counted(cudaGetLastError());
    k_prob_final<<<1, kT, 0, s>>>(partials, grid, out);
    return counted(cudaGetLastError(), 2);
}

template <typename T>
__global__ void __launch_bounds__(kT) k_scatter_live(T* __restrict__ st, const T* __restrict__ src, uint64_t count,
                                                     const __grid_constant__ IndexMap map) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < count; t += stride) st[expand_index(t, map)] = src[t];
}

cudaError_t launch_scatter_live(void* state, const void* src, int n, int prec, uint64_t zmask, uint64_t zval,
                                cudaStream_t s, int sms) {
    IndexMap map;
    std::memset(&map, 0, sizeof(map));
    int k = 0;
    for (int b = 0; b < 64; b++)
        if (zmask >> b & 1ull) map.pos[k++] = uint8_t(b);
    map.npos = k;
    map.fixval = zval & zmask;
    const uint64_t count = 1ull << (n - k);
    const int grid = grid_cap(count, sms, 2);
    if (prec == QS_PREC_C64)
        k_scatter_live<float2><<<grid, kT, 0, s>>>((float2*)state, (const float2*)src, count, map);
    else
        k_scatter_live<double2><<<grid, kT, 0, s>>>((double2*)state, (const double2*)src, count, map);
    return counted(cudaGetLastError());
}

// ---------------------------------------------------------------- read-back
// norm_sqr = re*re + im*im, rounded as num-complex computes it.
template <typename T>
__global__ void __launch_bounds__(kT) k_norm_sqr(const T* __restrict__ st, uint64_t first, uint64_t count,
                                                 double* __restrict__ dst) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < count; i += stride) {
        const double2 a = to_d2(st[first + i]);
        dst[i] = __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y));
    }
}

cudaError_t launch_norm_sqr(const void* state, int prec, uint64_t first, uint64_t count, double* dst,
                            cudaStream_t s, int sms) {
    if (prec == QS_PREC_C64)
        k_norm_sqr<float2><<<grid_cap(count, sms), kT, 0, s>>>((const float2*)state, first, count, dst);
    else
        k_norm_sqr<double2><<<grid_cap(count, sms), kT, 0, s>>>((const double2*)state, first, count, dst);
    return counted(cudaGetLastError());
}

__global__ void __launch_bounds__(kT) k_f2_to_d2(const float2* __restrict__ st, uint64_t first, uint64_t count,
                                                 double2* __restrict__ dst) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < count; i += stride)
        dst[i] = to_d2(st[first + i]);
}
__global__ void __launch_bounds__(kT) k_d2_to_f2(float2* __restrict__ st, uint64_t first, uint64_t count,
                                                 const double2* __restrict__ src) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < count; i += stride)
        from_d2(&st[first + i], src[i]);
}

cudaError_t launch_to_c128(const void* state, int prec, uint64_t first, uint64_t count, double* dst,
                           cudaStream_t s, int sms) {
    if (prec != QS_PREC_C64) return cudaErrorInvalidValue;
    k_f2_to_d2<<<grid_cap(count, sms), kT, 0, s>>>((const float2*)state, first, count, (double2*)dst);
    return counted(cudaGetLastError());
}
cudaError_t launch_from_c128(void* state, int prec, uint64_t first, uint64_t count, const double* src,
                             cudaStream_t s, int sms) {
    if (prec != QS_PREC_C64) return cudaErrorInvalidValue;
    k_d2_to_f2<<<grid_cap(count, sms), kT, 0, s>>>((float2*)state, first, count, (const double2*)src);
    return counted(cudaGetLastError());
}

// PartialEq (src/register.rs:409-413): all(|a_i - b_i| < tol) with norm() = hypot.
template <typename TA, typename TB>
__global__ void __launch_bounds__(kT) k_count_diff(const TA* __restrict__ a, const TB* __restrict__ b, uint64_t N,
                                                   double tol, unsigned long long* count) {
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    unsigned long long c = 0;
    for (uint64_t i = uint64_t(blockIdx.x) * kT + threadIdx.x; i < N; i += stride) {
        const double2 x = to_d2(a[i]), y = to_d2(b[i]);
        if (!(hypot(x.x - y.x, x.y - y.y) < tol)) c++;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

cudaError_t launch_count_diff(const void* a, const void* b, int n, int prec, double tol,
                              unsigned long long* count, cudaStream_t s, int sms) {
    const uint64_t N = 1ull << n;
    if (prec == QS_PREC_C64)
        k_count_diff<float2, float2><<<grid_cap(N, sms), kT, 0, s>>>((const float2*)a, (const float2*)b, N, tol,
                                                                     count);
    else
        k_count_diff<double2, double2><<<grid_cap(N, sms), kT, 0, s>>>((const double2*)a, (const double2*)b, N,
                                                                       tol, count);
    return counted(cudaGetLastError());
}

}  // namespace qs
