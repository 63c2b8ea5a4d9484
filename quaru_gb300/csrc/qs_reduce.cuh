// qs_reduce.cuh — fixed-order FP64 reductions (warp shuffles, then warps in order).
#pragma once

#include <cuda_runtime.h>

namespace qs {

__device__ __forceinline__ double rd_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum of (a, b) over a block of NT threads; valid in thread 0.
template <int NT>
__device__ __forceinline__ void rd_block_sum2(double& a, double& b) {
    __shared__ double sa[NT / 32], sb[NT / 32];
    a = rd_warp_sum(a);
    b = rd_warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int i = 0; i < NT / 32; i++) {
            ta += sa[i];
            tb += sb[i];
        }
        a = ta;
        b = tb;
    }
    __syncthreads();
}

// Compensated FP32 accumulator (Knuth TwoSum, Dekker TwoProduct by FMA):
// FP64-level accuracy for sums of float products on the FP32 pipe.
struct DfAcc {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float t = __fadd_rn(s, v);
        const float bb = __fsub_rn(t, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(v, bb));
        s = t;
        c = __fadd_rn(c, e);
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = __fmul_rn(a, b);
        c = __fadd_rn(c, __fmaf_rn(a, b, -p));
        add(p);
    }
    __device__ __forceinline__ void sub_prod(float a, float b) { add_prod(-a, b); }
    // Sum over the warp in lane 0 (fixed shuffle order), still as a float pair.
    __device__ __forceinline__ void warp_reduce() {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float os = __shfl_down_sync(0xffffffffu, s, o), oc = __shfl_down_sync(0xffffffffu, c, o);
            add(os);
            c = __fadd_rn(c, oc);
        }
    }
};

}  // namespace qs
