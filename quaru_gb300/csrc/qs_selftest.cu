// qs_selftest.cu — failure detection, exercised on the GPU without a fault.
//
// Every device-side wait of the engine is bounded: the tile and pass kernels wait on mbarriers
// (mbar_wait_bounded) and the batched persistent kernel on other blocks' completion counters
// (counter_wait_bounded). A wait that gives up makes its kernel raise an error flag and return,
// and the host reports QS_TIMEOUT with the context still usable. This self-test runs both wait
// helpers on conditions that nothing ever satisfies (an mbarrier no thread arrives on, a counter
// no block increments) with a short limit, so each gives up, and reports what the kernel saw.
#include <cuda_runtime.h>

#include <string>

#include "qs_internal.h"
#include "qs_kernels.h"
#include "qs_tma.cuh"

namespace qs {
namespace {

__global__ void k_wait_selftest(int* status, const unsigned int* counter, long long limit) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);  // one arrival completes phase 0; none comes
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        status[0] = mbar_wait_bounded(&bar, 0u, limit) ? 0 : 1;
        status[1] = counter_wait_bounded(counter, 1u, limit) ? 0 : 1;  // the counter stays 0
    }
}

}  // namespace
}  // namespace qs

extern "C" int qs_selftest_bounded_waits(int* mbar_timed_out, int* counter_timed_out) {
    if (!mbar_timed_out || !counter_timed_out) {
        qs::set_last_error_message("null argument");
        return QS_INVALID_ARGUMENT;
    }
    int* d = nullptr;  // [status 0, status 1, counter]
    cudaError_t e = cudaMalloc(&d, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d, 0, 4 * sizeof(int));
    if (e == cudaSuccess) {
        constexpr long long kLimit = 200000000LL;  // ~0.1 s at 2 GHz per wait
        qs::k_wait_selftest<<<1, 32>>>(d, reinterpret_cast<const unsigned int*>(d + 2), kLimit);
        e = cudaGetLastError();
        if (e == cudaSuccess) qs::note_launches(1);
    }
    int h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, 2 * sizeof(int), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) {
        qs::set_last_error_message(std::string("self-test: ") + cudaGetErrorString(e));
        return QS_CUDA_ERROR;
    }
    *mbar_timed_out = h[0];
    *counter_timed_out = h[1];
    return QS_OK;
}
