// qs_noalloc.cu — measurement probabilities for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs while a
// framework owns every byte of device memory through its own allocator, code
// on a latency-critical path where an allocation (and the implicit
// synchronisation it can bring) is not acceptable, or code that must stay
// within a fixed, pre-planned memory budget. They hold their state vector in
// a buffer they allocated themselves and need the probability sums of
// Register::try_measure (src/register.rs:303-315) for it.
//
// qs_measure_probabilities_noalloc() computes them with no allocation of any
// kind: the per-block partial sums go to the file-scope array below, which
// the CUDA module holds on every GPU that loads this library until the
// process exits. The reduction is the same as qs_measure_probabilities():
// the same grid, the same per-thread order, the same fixed-order block and
// final combination, so both give the same sums.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "qs_device.cuh"
#include "qs_kernels.h"

namespace qs {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxBlocks = 4096;  // scratch capacity: 2 doubles per block, 64 KiB in total
constexpr int kNaMaxDevices = 64;

// The scratch: written by every call, read by the same call's final kernel.
// Calls that overlap on the GPU (different streams, or host threads racing)
// share it and race; callers serialise them.
static __device__ __align__(256) double g_noalloc_partials[2 * kNaMaxBlocks];

// Device address of g_noalloc_partials, looked up once per device.
void* g_scratch_addr[kNaMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

__device__ __forceinline__ double na_to_d(double v) { return v; }
__device__ __forceinline__ double na_to_d(float v) { return double(v); }

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void na_block_sum2(double& a, double& b) {
    __shared__ double sa[kNaThreads / 32], sb[kNaThreads / 32];
    a = na_warp_sum(a);
    b = na_warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int i = 0; i < kNaThreads / 32; i++) {
            ta += sa[i];
            tb += sb[i];
        }
        a = ta;
        b = tb;
    }
}

template <typename T>
__global__ void __launch_bounds__(kNaThreads) k_na_prob_partials(const T* __restrict__ st, uint64_t npairs,
                                                                 int target, double* __restrict__ partials) {
    const uint64_t lo_mask = (1ull << target) - 1ull, tb = 1ull << target;
    const uint64_t stride = uint64_t(gridDim.x) * kNaThreads;
    double p0 = 0.0, p1 = 0.0;
    for (uint64_t t = uint64_t(blockIdx.x) * kNaThreads + threadIdx.x; t < npairs; t += stride) {
        const uint64_t i0 = ((t & ~lo_mask) << 1) | (t & lo_mask);
        const T a = st[i0];
        const T b = st[i0 | tb];
        const double ax = na_to_d(a.x), ay = na_to_d(a.y), bx = na_to_d(b.x), by = na_to_d(b.y);
        p0 = fma(ax, ax, p0);
        p0 = fma(ay, ay, p0);
        p1 = fma(bx, bx, p1);
        p1 = fma(by, by, p1);
    }
    na_block_sum2(p0, p1);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = p0;
        partials[2 * blockIdx.x + 1] = p1;
    }
}

__global__ void __launch_bounds__(kNaThreads) k_na_prob_final(const double* __restrict__ partials, int nblocks,
                                                              double* __restrict__ out) {
    double p0 = 0.0, p1 = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kNaThreads) {
        p0 += partials[2 * b];
        p1 += partials[2 * b + 1];
    }
    na_block_sum2(p0, p1);
    if (threadIdx.x == 0) {
        out[0] = p0;
        out[1] = p1;
    }
}

int na_err(int code, const std::string& msg) {
    set_last_error_message(msg);
    return code;
}

// Set-up, once per device, with that device current: the host-side name of
// g_noalloc_partials is only a stand-in, so look up its device address. The
// address is kept for the life of the process; cudaDeviceReset (or any other
// teardown of the device's primary context) unloads the module and makes it
// stale, so callers do not reset a device they keep using this entry point on.
int scratch_for_current_device(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_err(QS_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kNaMaxDevices) return na_err(QS_INVALID_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || !p)
            return na_err(QS_CUDA_ERROR, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return QS_OK;
}

}  // namespace
}  // namespace qs

extern "C" int qs_measure_probabilities_noalloc(const void* state, size_t n, int precision, size_t target,
                                                double* out, void* stream, size_t* err) {
    using namespace qs;
    if (!state || !out) return na_err(QS_INVALID_ARGUMENT, "state and out must be device pointers");
    if (precision != QS_PREC_C128 && precision != QS_PREC_C64) return na_err(QS_INVALID_ARGUMENT, "unknown precision");
    // The kernels load whole amplitudes (16 or 8 bytes) and store doubles: a misaligned pointer
    // would fault on the GPU and end the caller's context, so it is refused here instead.
    const uintptr_t amp_align = precision == QS_PREC_C128 ? 16 : 8;
    if (reinterpret_cast<uintptr_t>(state) % amp_align != 0 || reinterpret_cast<uintptr_t>(out) % 8 != 0)
        return na_err(QS_INVALID_ARGUMENT, "state must be aligned to its amplitude size and out to 8 bytes");
    if (n < 1 || n > 40) return na_err(QS_INVALID_ARGUMENT, "n must be in 1..40");
    if (target >= n) {
        if (err) err[0] = target;
        return na_err(QS_INVALID_TARGET, "InvalidTarget(" + std::to_string(target) + ")");
    }
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) return na_err(QS_CUDA_ERROR, "cudaGetDevice failed");
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // Same grid as qs_measure_probabilities: min(ceil(pairs / (256 * 4)), 32 per SM, 4096).
    const uint64_t npairs = 1ull << (n - 1);
    uint64_t blocks = (npairs + uint64_t(kNaThreads) * 4 - 1) / (uint64_t(kNaThreads) * 4);
    if (blocks > uint64_t(sms) * 32) blocks = uint64_t(sms) * 32;
    if (blocks > uint64_t(kNaMaxBlocks)) blocks = kNaMaxBlocks;
    if (blocks < 1) blocks = 1;
    if (blocks * 2 * sizeof(double) > sizeof(g_noalloc_partials))
        return na_err(QS_INVALID_ARGUMENT, "reduction needs more scratch than the 64 KiB static buffer holds");
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* partials = static_cast<double*>(scratch);
    if (precision == QS_PREC_C64)
        k_na_prob_partials<float2><<<int(blocks), kNaThreads, 0, s>>>(static_cast<const float2*>(state), npairs,
                                                                       int(target), partials);
    else
        k_na_prob_partials<double2><<<int(blocks), kNaThreads, 0, s>>>(static_cast<const double2*>(state), npairs,
                                                                        int(target), partials);
    k_na_prob_final<<<1, kNaThreads, 0, s>>>(partials, int(blocks), out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return na_err(QS_CUDA_ERROR, std::string("launch: ") + cudaGetErrorString(e));
    note_launches(2);
    return QS_OK;
}
