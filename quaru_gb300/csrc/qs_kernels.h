// qs_kernels.h — host-callable launchers of the engine's kernels.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "qs_internal.h"

#include <nvtx3/nvToolsExt.h>

namespace qs {

// An NVTX range around one public call, named after it (nothing is recorded unless a profiler is
// attached): sweeps, circuits, measurements, gradients and batch runs show up as ranges in a trace.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

constexpr uint8_t PF_SKIP_DEV = 4;  // PfClass::PF_SKIP as seen by device code

// Count kernel launches made by this library (read back through qs_launch_count).
void note_launches(uint64_t count);

// Resident blocks per SM of kernel `func` at `threads` threads and `smem` bytes of dynamic shared
// memory, raising the kernel's dynamic shared memory limit to `smem` first where needed. Both the
// limit and the occupancy are remembered per device, kernel and size, so a launcher pays for the
// two runtime queries once.
cudaError_t resident_blocks(const void* func, int threads, size_t smem, int* per_sm);

// Page-locked host staging buffer `slot` (0 or 1) of the calling thread, at least `bytes` long, or
// null if it cannot be had. Uploads from it do not wait for earlier work on the stream (uploads from
// pageable memory may). A slot is rewritten by the thread's next request for it: callers wait for
// the stream that reads it before returning, so the next request finds the copy done.
void* pinned_staging(int slot, size_t bytes);

// Set the message qs_last_error() returns on the calling thread.
void set_last_error_message(const std::string& msg);

// The autotune cache: one line "key a b" per tuned configuration, in QS_AUTOTUNE_CACHE or
// ~/.cache/quaru_gb300_autotune.txt; shared by the batch and circuit tuners (qs_autotune.cpp).
bool autotune_cache_lookup(const std::string& key, int* a, int* b);
void autotune_cache_store(const std::string& key, int a, int b);

// Device tables of a sub-operation wider than kMaxSmallK qubits.
struct BigOpBuffers {
    const uint64_t* off = nullptr;
    const uint64_t* off_src = nullptr;
    const uint8_t* pf = nullptr;
    const int8_t* lane = nullptr;
    const void* mat = nullptr;  // dense matrix or monomial phases, in the state's real type
};

// One sweep applying `op` (op.k <= kMaxSmallK) in place.
cudaError_t launch_op(const OpDesc& op, void* state, int n, int prec, int arith, cudaStream_t s, int sms);

// One sweep applying a wide `op`, reading the pre-gate state from `src`.
cudaError_t launch_op_big(const OpDesc& op, void* state, const void* src, int n, int prec, int arith,
                          const BigOpBuffers& b, cudaStream_t s, int sms);

// Host images of the tables launch_op_big reads.
void big_op_host_tables(const OpDesc& op, int prec, std::vector<uint64_t>* off, std::vector<uint64_t>* off_src,
                        std::vector<uint8_t>* pf, std::vector<int8_t>* lane, std::vector<unsigned char>* mat);

// ---- state-wide kernels (qs_state.cu) ----
cudaError_t launch_init_basis(void* state, int n, int prec, uint64_t index, cudaStream_t s, int sms);
cudaError_t launch_init_product(void* state, int n, int prec, const double* qubits, cudaStream_t s, int sms);
// FP64 probability sums of target bit 0 / 1 into out[0], out[1] (device), via per-block partials,
// over the live subspace (amplitudes whose zmask bits equal zval; the others must be zero).
// sequential (complex128 only): one block adds the squares in index order, as the reference does.
cudaError_t launch_measure_probs(const void* state, int n, int prec, int target, double* partials,
                                 int max_partials, double* out, cudaStream_t s, int sms, uint64_t zmask = 0,
                                 uint64_t zval = 0, bool sequential = false);
// Zero amplitudes whose target bit != outcome and divide the rest by d (rinv = 1/d), within the
// live subspace: complex128 with exact_quotient as the correctly rounded quotient (Rust's `/`),
// otherwise within one ulp of it (a multiply by rinv).
cudaError_t launch_collapse(void* state, int n, int prec, int target, int outcome, double d, double rinv,
                            cudaStream_t s, int sms, uint64_t zmask = 0, uint64_t zval = 0,
                            bool exact_quotient = true);
// The same collapse, with the probability sums of next_target over the kept amplitudes written to
// out[0], out[1] (device) in the same pass.
cudaError_t launch_collapse_probs(void* state, int n, int prec, int target, int outcome, double d, double rinv,
                                  int next_target, double* partials, int max_partials, double* out, cudaStream_t s,
                                  int sms, uint64_t zmask, uint64_t zval, bool exact_quotient = true);
// One pass of a measurement sequence on a compact buffer: `src` holds 2^nfree amplitudes indexed by
// the free bits in ascending order; the amplitudes whose bit `pos` equals `outcome` are divided by d
// (rinv = 1/d; correctly rounded with exact_quotient on complex128) and written densely to `dst`
// (2^(nfree-1) amplitudes, bit pos removed). With next_pos >= 0, the probability sums of bit
// next_pos of dst's index go to out[0], out[1] (device) in the same pass. Same pairs, order, grid and
// arithmetic as launch_collapse_probs.
cudaError_t launch_collapse_compact(const void* src, void* dst, int nfree, int prec, int pos, int outcome, double d,
                                    double rinv, int next_pos, double* partials, int max_partials, double* out,
                                    cudaStream_t s, int sms, bool exact_quotient);
// Write the 2^(n - popcount(zmask)) amplitudes of `src` (indexed by the free bits) to their places in
// the state: the bits of zmask set to those of zval.
cudaError_t launch_scatter_live(void* state, const void* src, int n, int prec, uint64_t zmask, uint64_t zval,
                                cudaStream_t s, int sms);
// norm_sqr of amplitudes [first, first + count) into dst (device).
cudaError_t launch_norm_sqr(const void* state, int prec, uint64_t first, uint64_t count, double* dst,
                            cudaStream_t s, int sms);
// Convert amplitudes [first, first+count) between the state's type and interleaved doubles.
cudaError_t launch_to_c128(const void* state, int prec, uint64_t first, uint64_t count, double* dst,
                           cudaStream_t s, int sms);
cudaError_t launch_from_c128(void* state, int prec, uint64_t first, uint64_t count, const double* src,
                             cudaStream_t s, int sms);
// Count amplitudes with |a_i - b_i| >= tol (hypot, as num-complex's norm) into *count (device).
cudaError_t launch_count_diff(const void* a, const void* b, int n, int prec, double tol,
                              unsigned long long* count, cudaStream_t s, int sms);

}  // namespace qs
