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
// normal floats; subnormal floats (< 2^-126) read as zero, far below every tolerance they feed.
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

template <typename T>
__global__ void __launch_bounds__(kT) k_prob_partials(const T* __restrict__ st, uint64_t npairs, int target,
                                                      double* __restrict__ partials) {
    const uint64_t lo_mask = (1ull << target) - 1ull, tb = 1ull << target;
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    double p0 = 0.0, p1 = 0.0;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < npairs; t += stride) {
        const uint64_t i0 = ((t & ~lo_mask) << 1) | (t & lo_mask);
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

cudaError_t launch_measure_probs(const void* state, int n, int prec, int target, double* partials,
                                 int max_partials, double* out, cudaStream_t s, int sms) {
    const uint64_t npairs = 1ull << (n - 1);
    int grid = grid_cap(npairs, sms, 4);
    if (grid > max_partials) grid = max_partials;
    if (prec == QS_PREC_C64)
        k_prob_partials<float2><<<grid, kT, 0, s>>>((const float2*)state, npairs, target, partials);
    else
        k_prob_partials<double2><<<grid, kT, 0, s>>>((const double2*)state, npairs, target, partials);
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

template <typename T, bool TRUEDIV>
__global__ void __launch_bounds__(kT) k_collapse(T* __restrict__ st, uint64_t npairs, int target, int outcome,
                                                 double d, double rinv) {
    const uint64_t lo_mask = (1ull << target) - 1ull, tb = 1ull << target;
    const uint64_t stride = uint64_t(gridDim.x) * kT;
    for (uint64_t t = uint64_t(blockIdx.x) * kT + threadIdx.x; t < npairs; t += stride) {
        const uint64_t i0 = ((t & ~lo_mask) << 1) | (t & lo_mask);
        const uint64_t keep = outcome ? (i0 | tb) : i0, drop = outcome ? i0 : (i0 | tb);
        if constexpr (sizeof(T) == 8 && !TRUEDIV) {
            // complex64: one FP64 multiply by RN(1/d) per component, rounded to float on the
            // integer pipe (the quotient is stored as a float, so the exactly rounded double
            // quotient of the complex128 path buys nothing here)
            const double2 x = to_d2_int(st[keep]);
            st[keep] = T{d2f_int(x.x * rinv), d2f_int(x.y * rinv)};
            st[drop] = T{0.0f, 0.0f};
            continue;
        }
        const double2 x = to_d2_int(st[keep]);
        double2 y;
        if (TRUEDIV) {
            y.x = x.x / d;
            y.y = x.y / d;
        } else {
            y.x = div_markstein(x.x, d, rinv);
            y.y = div_markstein(x.y, d, rinv);
        }
        from_d2(&st[keep], y);
        from_d2(&st[drop], make_double2(0.0, 0.0));
    }
}

cudaError_t launch_collapse(void* state, int n, int prec, int target, int outcome, double d, double rinv,
                            cudaStream_t s, int sms) {
    const uint64_t npairs = 1ull << (n - 1);
    const int grid = grid_cap(npairs, sms, 2);
    // Markstein's step needs a finite reciprocal of a normal divisor.
    const bool truediv = !(std::isfinite(rinv) && d > 1e-300 && std::isfinite(d));
    if (prec == QS_PREC_C64) {
        if (truediv)
            k_collapse<float2, true><<<grid, kT, 0, s>>>((float2*)state, npairs, target, outcome, d, rinv);
        else
            k_collapse<float2, false><<<grid, kT, 0, s>>>((float2*)state, npairs, target, outcome, d, rinv);
    } else {
        if (truediv)
            k_collapse<double2, true><<<grid, kT, 0, s>>>((double2*)state, npairs, target, outcome, d, rinv);
        else
            k_collapse<double2, false><<<grid, kT, 0, s>>>((double2*)state, npairs, target, outcome, d, rinv);
    }
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
