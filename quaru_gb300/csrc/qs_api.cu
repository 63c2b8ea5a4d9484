// qs_api.cu — the extern "C" boundary (include/quaru_gpu.h).
//
// Each function mirrors one item of Quaru's Register API (src/register.rs),
// with OperationError mapped to status codes and a thread-local message. A
// register owns one device buffer, one CUDA stream and small scratch areas.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "qs_adjoint.h"
#include "qs_circuit.h"
#include "qs_internal.h"
#include "qs_kernels.h"

struct qs_register {
    int n = 0;
    int prec = QS_PREC_C128;
    int arith = QS_ARITH_EXACT;
    int device = 0;
    int sms = 1;
    void* state = nullptr;
    cudaStream_t stream = nullptr;
    double* partials = nullptr;  // device: per-block reduction partials
    double* dres = nullptr;      // device: small results
    double* hres = nullptr;      // pinned host mirror of dres
    // Qubits collapsed by measurements with no gate on them since: every amplitude whose zmask bits
    // differ from zval is an exact zero, so later measurements visit only the live subspace.
    uint64_t zmask = 0;
    uint64_t zval = 0;
    // Scratch of the compact measurement sequences (half the state), allocated by the first one and
    // kept until the register is destroyed.
    void* mscratch = nullptr;
};

namespace qs {
static std::atomic<uint64_t> g_launches{0};
void note_launches(uint64_t count) { g_launches.fetch_add(count, std::memory_order_relaxed); }

namespace {
struct PinnedSlots {
    void* p[2] = {nullptr, nullptr};
    size_t cap[2] = {0, 0};
    ~PinnedSlots() {
        for (void* q : p)
            if (q) cudaFreeHost(q);
    }
};
thread_local PinnedSlots t_pinned;
}  // namespace

void* pinned_staging(int slot, size_t bytes) {
    if (slot < 0 || slot > 1) return nullptr;
    if (bytes <= t_pinned.cap[slot]) return t_pinned.p[slot];
    if (t_pinned.p[slot]) cudaFreeHost(t_pinned.p[slot]);
    t_pinned.p[slot] = nullptr;
    t_pinned.cap[slot] = 0;
    const size_t want = std::max<size_t>(bytes + bytes / 2, size_t(1) << 16);
    void* q = nullptr;
    if (cudaHostAlloc(&q, want, cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    t_pinned.p[slot] = q;
    t_pinned.cap[slot] = want;
    return q;
}

cudaError_t resident_blocks(const void* func, int threads, size_t smem, int* per_sm) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> limit;                     // dynamic smem limit set
    static std::map<std::tuple<int, const void*, int, size_t>, int> occupancy;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(dev, func, threads, smem);
    const auto hit = occupancy.find(key);
    if (hit != occupancy.end()) {
        *per_sm = hit->second;
        return cudaSuccess;
    }
    size_t& lim = limit[std::make_pair(dev, func)];
    if (smem > 48 * 1024 && smem > lim) {
        e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        lim = smem;
    }
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, func, threads, smem);
    if (e != cudaSuccess) return e;
    occupancy[key] = n;
    *per_sm = n;
    return cudaSuccess;
}
}  // namespace qs

namespace {

constexpr int kMaxPartials = 4096;
constexpr size_t kMaxQubits = 36;
thread_local std::string g_last_error;

int set_err(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_err(QS_OUT_OF_MEMORY, std::string(what) + ": out of device memory");
    }
    return set_err(QS_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

#define QS_CUDA(call, what)                             \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

size_t amp_bytes(int prec) { return prec == QS_PREC_C64 ? 8 : 16; }

void destroy(qs_register* r) {
    if (!r) return;
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->state) cudaFree(r->state);
    if (r->partials) cudaFree(r->partials);
    if (r->dres) cudaFree(r->dres);
    if (r->mscratch) cudaFree(r->mscratch);
    if (r->hres) cudaFreeHost(r->hres);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
}

// Allocate a register with uninitialised state.
int allocate(size_t n, int prec, qs_register** out) {
    if (!out) return set_err(QS_INVALID_ARGUMENT, "output pointer is null");
    *out = nullptr;
    if (prec != QS_PREC_C128 && prec != QS_PREC_C64) return set_err(QS_INVALID_ARGUMENT, "unknown precision");
    if (n > kMaxQubits) return set_err(QS_INVALID_ARGUMENT, "too many qubits for one GPU");
    auto* r = new qs_register();
    r->n = int(n);
    r->prec = prec;
    cudaError_t e = cudaGetDevice(&r->device);
    if (e != cudaSuccess) {
        delete r;
        return cuda_fail(e, "cudaGetDevice");
    }
    cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, r->device);
    if (r->sms < 1) r->sms = 1;
    const size_t bytes = (size_t(1) << n) * amp_bytes(prec);
    if ((e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&r->state, bytes)) != cudaSuccess ||
        (e = cudaMalloc(&r->partials, 2 * kMaxPartials * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&r->dres, 64 * sizeof(double))) != cudaSuccess ||
        (e = cudaMallocHost(&r->hres, 64 * sizeof(double))) != cudaSuccess) {
        destroy(r);
        return cuda_fail(e, "allocating register");
    }
    *out = r;
    return QS_OK;
}

}  // namespace

namespace qs {
void set_last_error_message(const std::string& msg) { g_last_error = msg; }
}  // namespace qs

namespace {

// A gate maps the live subspace of the qubits it does not act on into itself (zero amplitudes there
// stay exact zeros), so only its own targets leave the collapsed set. A matrix with a non-finite
// entry can turn zeros into NaNs: then nothing is assumed any more.
void touch_qubits(qs_register* reg, const double* matrix, const size_t* targets, size_t k) {
    for (size_t j = 0; j < k; j++) {
        const uint64_t b = 1ull << targets[j];
        reg->zmask &= ~b;
        reg->zval &= ~b;
    }
    const size_t entries = k < 32 ? (size_t(2) << (2 * k)) : 0;
    for (size_t i = 0; i < entries; i++)
        if (!std::isfinite(matrix[i])) {
            reg->zmask = reg->zval = 0;
            break;
        }
}

// Reference-order (sequential) probability sums for complex128 registers in the exact arithmetic
// up to this size; larger registers and the other forms use the parallel tree reduction.
constexpr int kSequentialMaxQubits = 20;

// Registers in the reference's arithmetic divide by sqrt(total) with the correctly rounded quotient
// (bit-identical collapses); the other forms multiply by its reciprocal (within one ulp).
bool exact_quotient(const qs_register* reg) { return reg->prec == QS_PREC_C128 && reg->arith == QS_ARITH_EXACT; }

bool sequential_sums(const qs_register* reg) {
    return reg->prec == QS_PREC_C128 && reg->arith == QS_ARITH_EXACT && reg->n <= kSequentialMaxQubits;
}

void record_outcome(qs_register* reg, size_t target, int res) {
    const uint64_t b = 1ull << target;
    reg->zmask |= b;
    reg->zval = (reg->zval & ~b) | (res ? b : 0ull);
}

}  // namespace

extern "C" {

const char* qs_last_error(void) { return g_last_error.c_str(); }
const char* qs_version(void) { return "quaru-gb300 0.1 (sm_103a)"; }

int qs_register_from_int(size_t n, size_t k, int precision, qs_register** out) {
    qs::TraceRange trace("qs_register_from_int");
    if (n < 64 && k >= (size_t(1) << n)) return set_err(QS_INVALID_ARGUMENT, "basis index out of range");
    int rc = allocate(n, precision, out);
    if (rc) return rc;
    cudaError_t e = qs::launch_init_basis((*out)->state, int(n), precision, k, (*out)->stream, (*out)->sms);
    if (e != cudaSuccess) {
        destroy(*out);
        *out = nullptr;
        return cuda_fail(e, "init_basis");
    }
    return QS_OK;
}

int qs_register_new(const uint8_t* bits, size_t n, int precision, qs_register** out) {
    qs::TraceRange trace("qs_register_new");
    if (n > 0 && !bits) return set_err(QS_INVALID_ARGUMENT, "bits is null");
    if (n > kMaxQubits) return set_err(QS_INVALID_ARGUMENT, "too many qubits for one GPU");
    // kron of |0>/|1> vectors (src/register.rs:47-50) is the basis state sum(bits[i] << i).
    size_t k = 0;
    for (size_t i = 0; i < n; i++)
        if (bits[i]) k |= size_t(1) << i;
    return qs_register_from_int(n, k, precision, out);
}

int qs_register_try_from_qubits(const double* qubits, size_t n, int precision, qs_register** out,
                                size_t* err) {
    qs::TraceRange trace("qs_register_try_from_qubits");
    if (!out) return set_err(QS_INVALID_ARGUMENT, "output pointer is null");
    *out = nullptr;
    if (n > 0 && !qubits) return set_err(QS_INVALID_ARGUMENT, "qubits is null");
    if (n > 64) return set_err(QS_INVALID_ARGUMENT, "too many qubits for one GPU");
    for (size_t q = 0; q < n; q++) {  // is_one (src/register.rs:107-115)
        double total = -1.0;
        for (int j = 0; j < 2; j++) {
            const double re = qubits[4 * q + 2 * j], im = qubits[4 * q + 2 * j + 1];
            total += re * re + im * im;
        }
        if (!(std::fabs(total) < 0.000001)) {
            if (err) err[0] = q;
            return set_err(QS_INVALID_QUBIT, "InvalidQubit(" + std::to_string(q) + ")");
        }
    }
    int rc = allocate(n, precision, out);
    if (rc) return rc;
    cudaError_t e = qs::launch_init_product((*out)->state, int(n), precision, qubits, (*out)->stream, (*out)->sms);
    if (e != cudaSuccess) {
        destroy(*out);
        *out = nullptr;
        return cuda_fail(e, "init_product");
    }
    return QS_OK;
}

int qs_register_clone(const qs_register* src, qs_register** out) {
    qs::TraceRange trace("qs_register_clone");
    if (!src) return set_err(QS_INVALID_ARGUMENT, "register is null");
    int rc = allocate(size_t(src->n), src->prec, out);
    if (rc) return rc;
    (*out)->arith = src->arith;
    (*out)->zmask = src->zmask;
    (*out)->zval = src->zval;
    cudaError_t e = cudaStreamSynchronize(src->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync((*out)->state, src->state, (size_t(1) << src->n) * amp_bytes(src->prec),
                            cudaMemcpyDeviceToDevice, (*out)->stream);
    if (e != cudaSuccess) {
        destroy(*out);
        *out = nullptr;
        return cuda_fail(e, "clone");
    }
    return QS_OK;
}

void qs_register_free(qs_register* reg) { destroy(reg); }

size_t qs_register_size(const qs_register* reg) { return reg ? size_t(reg->n) : 0; }

int qs_register_precision(const qs_register* reg) { return reg ? reg->prec : -1; }

int qs_register_set_arith(qs_register* reg, int arith) {
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (arith != QS_ARITH_EXACT && arith != QS_ARITH_FMA && arith != QS_ARITH_DF64 && arith != QS_ARITH_FX64)
        return set_err(QS_INVALID_ARGUMENT, "unknown arithmetic mode");
    reg->arith = arith;
    return QS_OK;
}

int qs_try_apply_fast(qs_register* reg, const double* matrix, size_t rows, size_t cols, const size_t* targets,
                      size_t k, size_t* err) {
    qs::TraceRange trace("qs_try_apply_fast");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    std::string msg;
    int rc = qs::validate_gate(size_t(reg->n), rows, cols, targets, k, err, &msg);
    if (rc) return set_err(rc, msg);
    if (!matrix) return set_err(QS_INVALID_ARGUMENT, "matrix is null");
    qs::OpDesc op;
    qs::classify_gate(matrix, k, targets, &op);
    touch_qubits(reg, matrix, targets, k);
    rc = qs::apply_op(reg->state, reg->n, reg->prec, reg->arith, op, reg->stream, reg->sms, &msg);
    return rc ? set_err(rc, msg) : QS_OK;
}

int qs_try_apply_all(qs_register* reg, const double* matrix, size_t rows, size_t cols, size_t k, size_t* err) {
    qs::TraceRange trace("qs_try_apply_all");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (k != 1) {  // src/register.rs:269-271
        if (err) err[0] = k;
        return set_err(QS_INVALID_ARITY, "InvalidArity(" + std::to_string(k) + ")");
    }
    for (int q = 0; q < reg->n; q++) {
        size_t t = size_t(q);
        int rc = qs_try_apply_fast(reg, matrix, rows, cols, &t, 1, err);
        if (rc) return rc;
    }
    return QS_OK;
}

int qs_apply_circuit(qs_register* reg, const qs_gate* gates, size_t m, const qs_circuit_options* opts,
                     size_t* err) {
    qs::TraceRange trace("qs_apply_circuit");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (m > 0 && !gates) return set_err(QS_INVALID_ARGUMENT, "gates is null");
    qs_circuit_options o;
    std::memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    std::vector<qs::OpDesc> ops(m);
    std::string msg;
    for (size_t g = 0; g < m; g++) {
        const size_t dim = gates[g].k < 64 ? (size_t(1) << gates[g].k) : 0;
        int rc = qs::validate_gate(size_t(reg->n), dim, dim, gates[g].targets, gates[g].k, err, &msg);
        if (!rc && !gates[g].matrix) rc = QS_INVALID_ARGUMENT, msg = "matrix is null";
        if (rc) {
            if (err) err[2] = g;
            return set_err(rc, "gate " + std::to_string(g) + ": " + msg);
        }
        qs::classify_gate(gates[g].matrix, gates[g].k, gates[g].targets, &ops[g]);
    }
    for (size_t g = 0; g < m; g++) touch_qubits(reg, gates[g].matrix, gates[g].targets, gates[g].k);
    if (o.fuse < 0 || o.fuse > 3) return set_err(QS_INVALID_ARGUMENT, "fuse must be 0..3");
    const bool tune = o.fuse == 3 || (o.fuse == 1 && o.tile_qubits == 0) || (o.fuse == 2 && o.max_width == 0);
    if (tune && qs::autotune_enabled()) {
        qs::TuneReport rep;
        int trc = qs::tune_circuit(reg->n, reg->prec, reg->arith, o.fuse, false, &rep, reg->sms, &msg);
        if (trc) return set_err(trc, msg);
        o.fuse = rep.best.fuse;
        o.max_width = rep.best.width;
        o.tile_qubits = rep.best.tile;
    } else if (o.fuse == 3) {
        o.fuse = 1;  // tuning switched off: stages at the automatic tile size
    }
    int rc = qs::run_circuit(reg->state, reg->n, reg->prec, reg->arith, ops, gates, o, reg->stream, reg->sms, &msg);
    return rc ? set_err(rc, msg) : QS_OK;
}

int qs_try_measure(qs_register* reg, size_t target, double draw, int* outcome, double* prob0, double* prob1,
                   size_t* err) {
    qs::TraceRange trace("qs_try_measure");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (target >= size_t(reg->n)) {  // src/register.rs:299-301
        if (err) err[0] = target;
        return set_err(QS_INVALID_TARGET, "InvalidTarget(" + std::to_string(target) + ")");
    }
    QS_CUDA(qs::launch_measure_probs(reg->state, reg->n, reg->prec, int(target), reg->partials, kMaxPartials,
                                     reg->dres, reg->stream, reg->sms, reg->zmask, reg->zval, sequential_sums(reg)),
            "measure_probs");
    QS_CUDA(cudaMemcpyAsync(reg->hres, reg->dres, 2 * sizeof(double), cudaMemcpyDeviceToHost, reg->stream),
            "measure readback");
    QS_CUDA(cudaStreamSynchronize(reg->stream), "measure sync");
    const double p0 = reg->hres[0], p1 = reg->hres[1];
    const int res = draw > p0 ? 1 : 0;  // src/register.rs:321
    const double total = res ? p1 : p0;  // :323
    const double d = std::sqrt(total);
    const double rinv = 1.0 / d;
    QS_CUDA(qs::launch_collapse(reg->state, reg->n, reg->prec, int(target), res, d, rinv, reg->stream, reg->sms,
                                reg->zmask, reg->zval, exact_quotient(reg)),
            "collapse");
    record_outcome(reg, target, res);
    if (outcome) *outcome = res;
    if (prob0) *prob0 = p0;
    if (prob1) *prob1 = p1;
    return QS_OK;
}

}  // extern "C"

namespace {

// A sequence of three or more distinct targets on a register of 14 qubits or more with no
// measurement recorded runs on a compact copy of the live subspace (launch_collapse_compact): the
// first collapse copies the kept half of the state, divided, into a half-size scratch buffer (the
// register's, allocated by its first such sequence and kept: allocating and mapping half a large
// state on every call costs milliseconds), later passes halve the live data between that buffer
// and the front of the state buffer, and at the end the state is zeroed (the value the in-place
// passes leave in every dropped amplitude) and the last live amplitudes are written back to their
// places. Results are bit-identical to the in-place passes; a pass moves its live data instead of
// whole DRAM sectors of a strided subspace. Returns 1 when the scratch buffer cannot be allocated,
// and the caller then runs the in-place passes.
constexpr int kCompactMinQubits = 14;

int measure_sequence_compact(qs_register* reg, const size_t* targets, size_t m, const double* draws, int* outcomes,
                             double* prob0s, double* prob1s) {
    const int n = reg->n;
    const size_t amp = amp_bytes(reg->prec);
    if (!reg->mscratch && cudaMalloc(&reg->mscratch, (size_t(1) << (n - 1)) * amp) != cudaSuccess) {
        cudaGetLastError();
        reg->mscratch = nullptr;
        return 1;
    }
    void* scratch = reg->mscratch;
    const bool exactq = exact_quotient(reg);
    QS_CUDA(qs::launch_measure_probs(reg->state, n, reg->prec, int(targets[0]), reg->partials, kMaxPartials,
                                     reg->dres, reg->stream, reg->sms),
            "measure_probs");
    std::vector<int> free_bits(n);  // the source buffer's index bits, as qubits, ascending
    for (int q = 0; q < n; q++) free_bits[q] = q;
    auto index_of = [&](size_t q) {
        return int(std::find(free_bits.begin(), free_bits.end(), int(q)) - free_bits.begin());
    };
    const void* src = reg->state;
    void* dst = nullptr;
    for (size_t k = 0; k < m; k++) {
        QS_CUDA(cudaMemcpyAsync(reg->hres, reg->dres, 2 * sizeof(double), cudaMemcpyDeviceToHost, reg->stream),
                "measure readback");
        QS_CUDA(cudaStreamSynchronize(reg->stream), "measure sync");
        const double p0 = reg->hres[0], p1 = reg->hres[1];
        const int res = draws[k] > p0 ? 1 : 0;  // src/register.rs:321
        const double total = res ? p1 : p0;
        const double d = std::sqrt(total);
        const double rinv = 1.0 / d;
        const int nfree = int(free_bits.size());
        const int pos = index_of(targets[k]);
        free_bits.erase(free_bits.begin() + pos);
        const int next_pos = k + 1 < m ? index_of(targets[k + 1]) : -1;
        dst = (k % 2 == 0) ? scratch : reg->state;  // the first pass reads the whole state
        QS_CUDA(qs::launch_collapse_compact(src, dst, nfree, reg->prec, pos, res, d, rinv, next_pos, reg->partials,
                                            kMaxPartials, reg->dres, reg->stream, reg->sms, exactq),
                "collapse_compact");
        record_outcome(reg, targets[k], res);
        src = dst;
        outcomes[k] = res;
        if (prob0s) prob0s[k] = p0;
        if (prob1s) prob1s[k] = p1;
    }
    const size_t live = size_t(1) << free_bits.size();
    if (dst == reg->state)
        QS_CUDA(cudaMemcpyAsync(scratch, reg->state, live * amp, cudaMemcpyDeviceToDevice, reg->stream),
                "compact copy");
    QS_CUDA(cudaMemsetAsync(reg->state, 0, (size_t(1) << n) * amp, reg->stream), "state zero");
    QS_CUDA(qs::launch_scatter_live(reg->state, scratch, n, reg->prec, reg->zmask, reg->zval, reg->stream, reg->sms),
            "scatter live");
    return QS_OK;
}

// QS_MEASURE_COMPACT=off keeps every measurement pass in place (for comparing the two forms).
bool compact_measurement_enabled() {
    const char* v = std::getenv("QS_MEASURE_COMPACT");
    return !(v && (std::strcmp(v, "off") == 0 || std::strcmp(v, "0") == 0));
}

bool distinct_targets(const size_t* targets, size_t m) {
    uint64_t seen = 0;
    for (size_t k = 0; k < m; k++) {
        if (seen >> targets[k] & 1ull) return false;
        seen |= 1ull << targets[k];
    }
    return true;
}

}  // namespace

extern "C" {

int qs_measure_sequence(qs_register* reg, const size_t* targets, size_t m, const double* draws, int* outcomes,
                        double* prob0s, double* prob1s, size_t* err) {
    qs::TraceRange trace("qs_measure_sequence");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (m && (!targets || !draws || !outcomes)) return set_err(QS_INVALID_ARGUMENT, "null argument");
    for (size_t k = 0; k < m; k++)
        if (targets[k] >= size_t(reg->n)) {  // src/register.rs:299-301, checked before any work
            if (err) {
                err[0] = targets[k];
                err[2] = k;
            }
            return set_err(QS_INVALID_TARGET, "InvalidTarget(" + std::to_string(targets[k]) + ")");
        }
    if (m == 0) return QS_OK;
    const bool seq = sequential_sums(reg);
    if (!seq && m >= 3 && reg->zmask == 0 && reg->n >= kCompactMinQubits && distinct_targets(targets, m) &&
        compact_measurement_enabled()) {
        const int rc = measure_sequence_compact(reg, targets, m, draws, outcomes, prob0s, prob1s);
        if (rc != 1) return rc;
    }
    QS_CUDA(qs::launch_measure_probs(reg->state, reg->n, reg->prec, int(targets[0]), reg->partials, kMaxPartials,
                                     reg->dres, reg->stream, reg->sms, reg->zmask, reg->zval, seq),
            "measure_probs");
    for (size_t k = 0; k < m; k++) {
        QS_CUDA(cudaMemcpyAsync(reg->hres, reg->dres, 2 * sizeof(double), cudaMemcpyDeviceToHost, reg->stream),
                "measure readback");
        QS_CUDA(cudaStreamSynchronize(reg->stream), "measure sync");
        const double p0 = reg->hres[0], p1 = reg->hres[1];
        const int res = draws[k] > p0 ? 1 : 0;
        const double total = res ? p1 : p0;
        const double d = std::sqrt(total);
        const double rinv = 1.0 / d;
        const int t = int(targets[k]);
        if (k + 1 < m && !seq) {
            QS_CUDA(qs::launch_collapse_probs(reg->state, reg->n, reg->prec, t, res, d, rinv, int(targets[k + 1]),
                                              reg->partials, kMaxPartials, reg->dres, reg->stream, reg->sms,
                                              reg->zmask, reg->zval, exact_quotient(reg)),
                    "collapse_probs");
            record_outcome(reg, targets[k], res);
        } else {
            QS_CUDA(qs::launch_collapse(reg->state, reg->n, reg->prec, t, res, d, rinv, reg->stream, reg->sms,
                                        reg->zmask, reg->zval, exact_quotient(reg)),
                    "collapse");
            record_outcome(reg, targets[k], res);
            if (k + 1 < m)
                QS_CUDA(qs::launch_measure_probs(reg->state, reg->n, reg->prec, int(targets[k + 1]), reg->partials,
                                                 kMaxPartials, reg->dres, reg->stream, reg->sms, reg->zmask,
                                                 reg->zval, seq),
                        "measure_probs");
        }
        outcomes[k] = res;
        if (prob0s) prob0s[k] = p0;
        if (prob1s) prob1s[k] = p1;
    }
    return QS_OK;
}

int qs_measure_probabilities(qs_register* reg, size_t target, double* prob0, double* prob1, size_t* err) {
    qs::TraceRange trace("qs_measure_probabilities");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (target >= size_t(reg->n)) {
        if (err) err[0] = target;
        return set_err(QS_INVALID_TARGET, "InvalidTarget(" + std::to_string(target) + ")");
    }
    QS_CUDA(qs::launch_measure_probs(reg->state, reg->n, reg->prec, int(target), reg->partials, kMaxPartials,
                                     reg->dres, reg->stream, reg->sms),
            "measure_probs");
    QS_CUDA(cudaMemcpyAsync(reg->hres, reg->dres, 2 * sizeof(double), cudaMemcpyDeviceToHost, reg->stream),
            "measure readback");
    QS_CUDA(cudaStreamSynchronize(reg->stream), "measure sync");
    if (prob0) *prob0 = reg->hres[0];
    if (prob1) *prob1 = reg->hres[1];
    return QS_OK;
}

int qs_inner_product(const qs_register* a, const qs_register* b, double* re, double* im) {
    qs::TraceRange trace("qs_inner_product");
    if (!a || !b) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if (a->n != b->n) return set_err(QS_INVALID_ARGUMENT, "registers differ in size");
    QS_CUDA(cudaStreamSynchronize(b->stream), "inner sync");
    qs_register* ra = const_cast<qs_register*>(a);
    if (qs::inner_product(a->state, a->prec, b->state, b->prec, a->n, ra->stream, ra->sms, ra->partials, ra->dres))
        return cuda_fail(cudaGetLastError(), "inner product");
    QS_CUDA(cudaMemcpyAsync(ra->hres, ra->dres, 2 * sizeof(double), cudaMemcpyDeviceToHost, ra->stream), "inner readback");
    QS_CUDA(cudaStreamSynchronize(ra->stream), "inner sync");
    if (re) *re = ra->hres[0];
    if (im) *im = ra->hres[1];
    return QS_OK;
}

static bool terms_fit(const qs_pauli_term* terms, size_t nterms, int n) {
    for (size_t t = 0; t < nterms; t++)
        if (n < 64 && ((terms[t].x_mask | terms[t].z_mask) >> n)) return false;
    return true;
}

int qs_expval_pauli(qs_register* reg, const qs_pauli_term* terms, size_t nterms, double* value) {
    qs::TraceRange trace("qs_expval_pauli");
    if (!reg || !value || (nterms && !terms)) return set_err(QS_INVALID_ARGUMENT, "null argument");
    if (!terms_fit(terms, nterms, reg->n)) return set_err(QS_INVALID_ARGUMENT, "Pauli term acts on a qubit >= n");
    std::string msg;
    int rc = qs::expval_pauli(reg->state, reg->prec, reg->n, terms, nterms, reg->stream, reg->sms, value, &msg);
    return rc ? set_err(rc, msg) : QS_OK;
}

int qs_adjoint_gradient(qs_register* reg, const qs_param_gate* gates, size_t m, const double* params, size_t nparams,
                        const qs_pauli_term* terms, size_t nterms, double* energy, double* grad, size_t* err) {
    qs::TraceRange trace("qs_adjoint_gradient");
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    if ((m && !gates) || (nparams && !params) || (nterms && !terms))
        return set_err(QS_INVALID_ARGUMENT, "null argument");
    if (reg->n < 1) return set_err(QS_INVALID_ARGUMENT, "register has no qubits");
    if (!terms_fit(terms, nterms, reg->n)) return set_err(QS_INVALID_ARGUMENT, "Pauli term acts on a qubit >= n");
    std::string msg;
    reg->zmask = reg->zval = 0;  // the state is restored on return, but not assumed collapsed any more
    int rc = qs::adjoint_gradient(reg->state, reg->n, reg->prec, reg->arith, gates, m, params, nparams, terms, nterms,
                                  reg->stream, reg->sms, energy, grad, err, &msg);
    return rc ? set_err(rc, msg) : QS_OK;
}

uint64_t qs_launch_count(void) { return qs::g_launches.load(std::memory_order_relaxed); }

int qs_circuit_autotune(size_t n, int precision, int arith, int fuse, int retune, qs_autotune_report* out) {
    qs::TraceRange trace("qs_circuit_autotune");
    if (!out) return set_err(QS_INVALID_ARGUMENT, "out is null");
    std::memset(out, 0, sizeof(*out));
    if (n < 1 || n > kMaxQubits) return set_err(QS_INVALID_ARGUMENT, "n out of range");
    if (precision != QS_PREC_C128 && precision != QS_PREC_C64) return set_err(QS_INVALID_ARGUMENT, "unknown precision");
    if (arith < QS_ARITH_EXACT || arith > QS_ARITH_FX64) return set_err(QS_INVALID_ARGUMENT, "unknown arithmetic mode");
    if (fuse < 1 || fuse > 3) return set_err(QS_INVALID_ARGUMENT, "fuse must be 1, 2 or 3");
    int dev = 0, sms = 1;
    QS_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    QS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    qs::TuneReport rep;
    std::string msg;
    int rc = qs::tune_circuit(int(n), precision, arith, fuse, retune != 0, &rep, sms, &msg);
    if (rc) return set_err(rc, msg);
    out->fuse = rep.best.fuse;
    out->max_width = rep.best.width;
    out->tile_qubits = rep.best.tile;
    out->from_cache = rep.from_cache ? 1 : 0;
    out->count = int(std::min<size_t>(rep.cand.size(), QS_AUTOTUNE_MAX_CANDIDATES));
    for (int i = 0; i < out->count; i++) {
        out->cand_fuse[i] = rep.cand[i].fuse;
        out->cand_width[i] = rep.cand[i].width;
        out->cand_tile[i] = rep.cand[i].tile;
        out->cand_ms[i] = rep.ms[i];
    }
    return QS_OK;
}

int qs_get_state(const qs_register* reg, double* dst) {
    qs::TraceRange trace("qs_get_state");
    if (!reg || !dst) return set_err(QS_INVALID_ARGUMENT, "null argument");
    const uint64_t N = 1ull << reg->n;
    if (reg->prec == QS_PREC_C128) {
        QS_CUDA(cudaMemcpyAsync(dst, reg->state, N * 16, cudaMemcpyDeviceToHost, reg->stream), "get_state");
        QS_CUDA(cudaStreamSynchronize(reg->stream), "get_state sync");
        return QS_OK;
    }
    const uint64_t chunk = std::min<uint64_t>(N, 1ull << 22);
    double* tmp = nullptr;
    QS_CUDA(cudaMallocAsync((void**)&tmp, chunk * 16, reg->stream), "get_state temp");
    for (uint64_t f = 0; f < N; f += chunk) {
        const uint64_t c = std::min<uint64_t>(chunk, N - f);
        QS_CUDA(qs::launch_to_c128(reg->state, reg->prec, f, c, tmp, reg->stream, reg->sms), "to_c128");
        QS_CUDA(cudaMemcpyAsync(dst + 2 * f, tmp, c * 16, cudaMemcpyDeviceToHost, reg->stream), "get_state copy");
    }
    QS_CUDA(cudaFreeAsync(tmp, reg->stream), "get_state free");
    QS_CUDA(cudaStreamSynchronize(reg->stream), "get_state sync");
    return QS_OK;
}

int qs_set_state(qs_register* reg, const double* src) {
    qs::TraceRange trace("qs_set_state");
    if (!reg || !src) return set_err(QS_INVALID_ARGUMENT, "null argument");
    reg->zmask = reg->zval = 0;
    const uint64_t N = 1ull << reg->n;
    if (reg->prec == QS_PREC_C128) {
        QS_CUDA(cudaMemcpyAsync(reg->state, src, N * 16, cudaMemcpyHostToDevice, reg->stream), "set_state");
        QS_CUDA(cudaStreamSynchronize(reg->stream), "set_state sync");
        return QS_OK;
    }
    const uint64_t chunk = std::min<uint64_t>(N, 1ull << 22);
    double* tmp = nullptr;
    QS_CUDA(cudaMallocAsync((void**)&tmp, chunk * 16, reg->stream), "set_state temp");
    for (uint64_t f = 0; f < N; f += chunk) {
        const uint64_t c = std::min<uint64_t>(chunk, N - f);
        QS_CUDA(cudaMemcpyAsync(tmp, src + 2 * f, c * 16, cudaMemcpyHostToDevice, reg->stream), "set_state copy");
        QS_CUDA(qs::launch_from_c128(reg->state, reg->prec, f, c, tmp, reg->stream, reg->sms), "from_c128");
    }
    QS_CUDA(cudaFreeAsync(tmp, reg->stream), "set_state free");
    QS_CUDA(cudaStreamSynchronize(reg->stream), "set_state sync");
    return QS_OK;
}

int qs_probabilities(const qs_register* reg, double* dst) {
    qs::TraceRange trace("qs_probabilities");
    if (!reg || !dst) return set_err(QS_INVALID_ARGUMENT, "null argument");
    const uint64_t N = 1ull << reg->n;
    const uint64_t chunk = std::min<uint64_t>(N, 1ull << 22);
    double* tmp = nullptr;
    QS_CUDA(cudaMallocAsync((void**)&tmp, chunk * 8, reg->stream), "probabilities temp");
    for (uint64_t f = 0; f < N; f += chunk) {
        const uint64_t c = std::min<uint64_t>(chunk, N - f);
        QS_CUDA(qs::launch_norm_sqr(reg->state, reg->prec, f, c, tmp, reg->stream, reg->sms), "norm_sqr");
        QS_CUDA(cudaMemcpyAsync(dst + f, tmp, c * 8, cudaMemcpyDeviceToHost, reg->stream), "probabilities copy");
    }
    QS_CUDA(cudaFreeAsync(tmp, reg->stream), "probabilities free");
    QS_CUDA(cudaStreamSynchronize(reg->stream), "probabilities sync");
    return QS_OK;
}

int qs_register_eq(const qs_register* a, const qs_register* b, double tol, int* equal) {
    if (!a || !b || !equal) return set_err(QS_INVALID_ARGUMENT, "null argument");
    if (a->n != b->n || a->prec != b->prec) {
        *equal = 0;
        return QS_OK;
    }
    QS_CUDA(cudaStreamSynchronize(b->stream), "eq sync");
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(a->dres + 8);
    QS_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), a->stream), "eq memset");
    QS_CUDA(qs::launch_count_diff(a->state, b->state, a->n, a->prec, tol, cnt, a->stream, a->sms), "count_diff");
    QS_CUDA(cudaMemcpyAsync(a->hres + 8, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, a->stream),
            "eq readback");
    QS_CUDA(cudaStreamSynchronize(a->stream), "eq sync");
    unsigned long long c;
    std::memcpy(&c, a->hres + 8, sizeof(c));
    *equal = (c == 0);
    return QS_OK;
}

int qs_synchronize(qs_register* reg) {
    if (!reg) return set_err(QS_INVALID_ARGUMENT, "register is null");
    QS_CUDA(cudaStreamSynchronize(reg->stream), "synchronize");
    return QS_OK;
}

void* qs_register_stream(qs_register* reg) { return reg ? (void*)reg->stream : nullptr; }

}  // extern "C"
