/*
 * quaru_gpu.h — C ABI of the GB300 state-vector engine (libquaru_gb300.so).
 *
 * Drop-in for the gate-application and measurement path of Quaru
 * (DATX11-22/quaru). Each entry point names the reference item it replaces
 * (path:line within the reference project). Plain pointers and sizes only:
 * complex data is interleaved (re, im) IEEE doubles — the memory layout of
 * ndarray's Array2<Complex<f64>> — and matrices are row-major 2^k x 2^k with
 * local index bit j <-> targets[j] (src/register.rs:163-176).
 *
 * Threading: one register is used by one host thread at a time (Rust's
 * `&mut self`); distinct registers may be used from distinct threads. Every
 * call is ordered on the register's own CUDA stream; calls that return data
 * to the host synchronise that stream. No exception crosses this boundary.
 *
 * Return value: QS_OK or a status below. `err` (nullable, 3 entries) carries
 * the payload of OperationError (src/register.rs:10-20): InvalidTarget(t) ->
 * err[0] = t; InvalidDimensions(r, c) -> err[0] = r, err[1] = c;
 * InvalidArity(k) -> err[0] = k; InvalidQubit(i) -> err[0] = i. Circuit calls
 * put the failing gate's index in err[2]. qs_last_error() gives a message.
 */
#ifndef QUARU_GPU_H
#define QUARU_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define QS_OK 0
#define QS_INVALID_TARGET 1     /* OperationError::InvalidTarget */
#define QS_INVALID_DIMENSIONS 2 /* OperationError::InvalidDimensions */
#define QS_INVALID_ARITY 3      /* OperationError::InvalidArity */
#define QS_INVALID_QUBIT 4      /* OperationError::InvalidQubit */
#define QS_INVALID_ARGUMENT 5   /* null pointer, n out of range, bad enum */
#define QS_CUDA_ERROR 6         /* a CUDA runtime call failed */
#define QS_OUT_OF_MEMORY 7      /* device allocation failed */
#define QS_TIMEOUT 8            /* a bounded device wait gave up */
#define QS_QASM_PARSE_ERROR 9   /* OpenQASMError::OpenQASMParseError */
#define QS_QASM_RUN_ERROR 10    /* OpenQASMError::OpenQASMRunError */

/* ---- state precision ---------------------------------------------------- */
#define QS_PREC_C128 0 /* complex128 state (the reference's c64 = Complex<f64>) */
#define QS_PREC_C64 1  /* complex64 state: the mixed-precision form */

/* ---- arithmetic of gate application on a complex128 register ------------ */
#define QS_ARITH_EXACT 0 /* the reference's operation order, no fused multiply-add:
                            bit-identical amplitudes (+0 and -0 compared as equal) */
#define QS_ARITH_FMA 1   /* FP64 fused multiply-add; within 1e-15 relative per gate */
#define QS_ARITH_DF64 2  /* double-float arithmetic on the FP32 pipe for dense gates;
                            ~2^-47 relative per gate; permutation/diagonal gates stay exact */
#define QS_ARITH_FX64 3  /* FP64-accurate fixed-point arithmetic on the integer pipes for dense
                            1-qubit gates: each output is an exact-to-2^-55 integer dot product
                            rounded once to double (error <= ulp/2 + 2^-55 max|u| max|x|, below
                            the FP64 FMA form's); fused dense blocks (qs_apply_circuit, fuse = 2,
                            12 qubits and more) run as FP64-accurate split-integer products on the
                            BF16 tensor cores; other gates and cache-blocked stages use FP64 FMA */

typedef struct qs_register qs_register;

/* ---- construction / lifetime -------------------------------------------- */

/* Register::new (src/register.rs:41-56): basis state from n booleans. */
int qs_register_new(const uint8_t* bits, size_t n, int precision, qs_register** out);

/* Register::from_int (src/register.rs:58-63): basis state |k> on n qubits. */
int qs_register_from_int(size_t n, size_t k, int precision, qs_register** out);

/* Register::try_from_qubits (src/register.rs:81-102): product state from n
 * single-qubit states (2 complex each, 4 doubles). InvalidQubit(i) when
 * |sum |q_i|^2 - 1| >= 1e-6 (src/register.rs:107-115). */
int qs_register_try_from_qubits(const double* qubits, size_t n, int precision,
                                qs_register** out, size_t* err);

/* #[derive(Clone)] on Register (src/register.rs:23): device-to-device copy. */
int qs_register_clone(const qs_register* src, qs_register** out);

/* Drop for Register. Null is ignored. */
void qs_register_free(qs_register* reg);

/* Register::size (src/register.rs:404-406). */
size_t qs_register_size(const qs_register* reg);

/* Precision the register was created with (QS_PREC_*). */
int qs_register_precision(const qs_register* reg);

/* Select the arithmetic of later gate applications (QS_ARITH_*); default
 * QS_ARITH_EXACT. Ignored by complex64 registers (FP32 FMA). */
int qs_register_set_arith(qs_register* reg, int arith);

/* ---- gate application --------------------------------------------------- */

/* Register::try_apply_fast (src/register.rs:140-191); Register::apply
 * (:134-137) is this call plus a panic on error. Validation order: shape
 * (InvalidDimensions), duplicate target (smallest duplicate), out-of-range
 * target (first in list order). The shape check rejects every shape that is
 * not 2^k x 2^k; the reference's own check (:141-145) fires only on (k, k)
 * and otherwise panics inside ndarray's dot, so every call the reference
 * rejects is rejected here with the same payload. */
int qs_try_apply_fast(qs_register* reg, const double* matrix, size_t rows, size_t cols,
                      const size_t* targets, size_t k, size_t* err);

/* Register::try_apply_all (src/register.rs:267-281): a 1-qubit operation on
 * every qubit, as n in-place sweeps instead of a dense 2^n x 2^n kron.
 * InvalidArity(k) when k != 1. */
int qs_try_apply_all(qs_register* reg, const double* matrix, size_t rows, size_t cols,
                     size_t k, size_t* err);

/* One gate of a circuit: arity k, k targets, 2^k x 2^k interleaved matrix. */
typedef struct qs_gate {
    size_t k;
    const size_t* targets;
    const double* matrix;
} qs_gate;

/* Options for qs_apply_circuit. */
typedef struct qs_circuit_options {
    int fuse;        /* 0: one sweep per gate; 1: cache-blocked stages (bit-identical to 0
                        under QS_ARITH_EXACT); 2: dense fused blocks (complex64 registers:
                        3xTF32 tensor-core blocks; complex128 registers in QS_ARITH_FX64:
                        FP64-accurate split-integer tensor-core blocks); 3: the autotuner picks
                        0, 1 (and its tile size) or 2 (and its width) */
    int max_width;   /* widest fused dense block, 2..5 (fuse == 2); 0 = autotuned (see
                        qs_circuit_autotune) */
    int tile_qubits; /* qubits per shared-memory tile for fuse == 1; 0 = autotuned */
    int reserved;
} qs_circuit_options;

/* The fusion autotuner (the counterpart of choosing QuantumCircuit reduction
 * passes by hand, src/operation.rs:114-269): the candidates of `fuse` (1: tile
 * sizes of stages; 2: block widths 2..5; 3: both, plus one sweep per gate) are
 * timed once per (n, precision, arith, fuse) on a scratch register running a
 * seeded stand-in workload of the benchmarks' family (six layers of random
 * dense 1-qubit gates on every qubit and CNOTs on a random matching) at
 * min(n, 26) qubits; the fastest is kept in memory and in the autotune cache
 * file (QS_AUTOTUNE_CACHE, default ~/.cache/quaru_gb300_autotune.txt). Later
 * qs_apply_circuit calls with fuse == 3, or fuse 1 / 2 with a zero tile size /
 * width, use that choice; QS_AUTOTUNE=off selects the fixed rules instead
 * (tile qubits min(11 or 12, max(8 or 9, n - 7)) for complex128 / complex64;
 * width 5 complex64, 3 double-float, 2 otherwise; fuse 3 -> 1). qs_circuit_autotune
 * returns the choice and, when it timed the candidates (first use, or
 * retune != 0), each candidate's time. It needs a device but no register. */
#define QS_AUTOTUNE_MAX_CANDIDATES 16
typedef struct qs_autotune_report {
    int fuse, max_width, tile_qubits;  /* the choice */
    int from_cache;                     /* 1: taken from the cache, no timings below */
    int count;                          /* candidates timed */
    int cand_fuse[QS_AUTOTUNE_MAX_CANDIDATES];
    int cand_width[QS_AUTOTUNE_MAX_CANDIDATES];
    int cand_tile[QS_AUTOTUNE_MAX_CANDIDATES];
    double cand_ms[QS_AUTOTUNE_MAX_CANDIDATES];
} qs_autotune_report;
int qs_circuit_autotune(size_t n, int precision, int arith, int fuse, int retune, qs_autotune_report* out);

/* The operations loop of Register::apply_circuit (src/register.rs:345-350):
 * applies gates[0..m) in order. Every gate is validated before any is
 * applied; on error nothing is applied, err[2] = index of the bad gate.
 * opts may be null (fuse = 0). */
int qs_apply_circuit(qs_register* reg, const qs_gate* gates, size_t m,
                     const qs_circuit_options* opts, size_t* err);

/* ---- measurement -------------------------------------------------------- */

/* Register::try_measure (src/register.rs:297-342) with the uniform draw in
 * [0, 1) supplied by the caller (the reference's thread_rng, :317-318, cannot
 * be seeded). outcome = draw > prob_0 (:321). prob0/prob1 are nullable and
 * receive the FP64 probability sums the decision used. Complex128 registers in
 * QS_ARITH_EXACT with n <= 20 add the squares in index order as the reference
 * does (:306-315), so sums, outcome and collapsed state are bit-identical to
 * it; larger registers and the other forms use a fixed-order parallel tree
 * (within 1e-14). The collapse divides by sqrt(prob) (:337): correctly rounded
 * on complex128 registers in QS_ARITH_EXACT, as Rust's `/`; the other forms
 * multiply by the rounded reciprocal (within one ulp of the quotient).
 * Qubits measured since their last gate stay collapsed: later measurements
 * read only the amplitudes that can still be non-zero. */
int qs_try_measure(qs_register* reg, size_t target, double draw, int* outcome,
                   double* prob0, double* prob1, size_t* err);

/* Register::measure_circuit (src/register.rs:371-377): try_measure of
 * targets[0..m) in order with draws[0..m), outcomes into outcomes[0..m),
 * probability sums into prob0s/prob1s (nullable). Every target is checked
 * before any work (InvalidTarget, err[2] = its index). Each collapse pass also
 * sums the next target's probabilities over the kept amplitudes, and each pass
 * reads only the live subspace, so measuring all n qubits costs about two
 * sweeps of the state instead of 2n. Three or more distinct targets on a
 * register of 14 qubits or more with no measurement recorded since its last
 * gate run on a compact copy of the live subspace (a scratch buffer of half
 * the state, allocated by the register's first such sequence and kept until
 * qs_register_free; without the memory the passes stay in place), with results bit
 * for bit those of the in-place passes; QS_MEASURE_COMPACT=off keeps them in
 * place. A call that fails with QS_CUDA_ERROR partway leaves the register's
 * state unspecified. */
int qs_measure_sequence(qs_register* reg, const size_t* targets, size_t m, const double* draws, int* outcomes,
                        double* prob0s, double* prob1s, size_t* err);

/* The probability sums of a measurement (src/register.rs:303-315) without the
 * draw and the collapse: p0 = sum |a_i|^2 over target bit 0, p1 over bit 1, a
 * fixed-order parallel FP64 tree over the whole state (within 1e-14 of the
 * reference's sequential sum). The state is left unchanged. */
int qs_measure_probabilities(qs_register* reg, size_t target, double* prob0, double* prob1, size_t* err);

/* For callers that cannot allocate device memory. No counterpart in the
 * reference: Quaru's Register always owns its state. Code that runs under a
 * framework's own allocator, inside a fixed pre-planned memory budget, or on
 * a path where cudaMalloc and its implicit synchronisation are not allowed
 * keeps its state vector in a buffer it allocated itself (2^n amplitudes,
 * interleaved complex128 or complex64 per `precision`) and gets the
 * probability sums of try_measure for it here. out is a device pointer to 2
 * doubles (prob_0, prob_1); work is queued on `stream` (a cudaStream_t, null =
 * default stream) and out is valid once that stream reaches it. The sums equal
 * those of qs_measure_probabilities for the same amplitudes.
 * Allocates nothing: per-block partial sums go to a 64 KiB file-scope
 * __device__ array that every GPU loading this library holds until exit, so
 * any n in 1..40 fits; a request needing more scratch than that is rejected
 * with QS_INVALID_ARGUMENT, and so is a state pointer not aligned to its
 * amplitude size (16 or 8 bytes) or an out pointer not aligned to 8 bytes.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process; make that
 * first call before any stream capture, and do not reset a device
 * (cudaDeviceReset) that later calls use, which would leave the kept address
 * stale. Every call shares the array: calls that overlap on the GPU (other
 * streams, other host threads) race and must be serialised. */
int qs_measure_probabilities_noalloc(const void* state, size_t n, int precision, size_t target,
                                     double* out, void* stream, size_t* err);

/* ---- observables and gradients (no counterpart in the reference) ---------- */

/* <a|b> = sum_i conj(a_i) b_i accumulated in FP64 on the GPU; a and b may
 * have different precisions (the fidelity of a complex64 run against a
 * complex128 run is |<a|b>|^2). */
int qs_inner_product(const qs_register* a, const qs_register* b, double* re, double* im);

/* One term coeff * P of a Pauli-sum observable. P acts with X on the qubits
 * in x_mask only, Z on z_mask only and Y on both (Y = iXZ per qubit). */
typedef struct qs_pauli_term {
    double coeff;
    uint64_t x_mask;
    uint64_t z_mask;
} qs_pauli_term;

/* <psi|H|psi> for H = sum_t coeff_t P_t, in FP64 on the GPU. */
int qs_expval_pauli(qs_register* reg, const qs_pauli_term* terms, size_t nterms, double* value);

/* Gates of a parameterised circuit. Rotations R_A(theta) = exp(-i theta A / 2)
 * for A = X, Y, Z act on targets[0] with theta = params[param]; QS_GATE_FIXED
 * is a matrix gate (k, targets, matrix as in qs_gate). */
#define QS_GATE_FIXED 0
#define QS_GATE_RX 1
#define QS_GATE_RY 2
#define QS_GATE_RZ 3
typedef struct qs_param_gate {
    int kind;
    int param;
    size_t k;
    const size_t* targets;
    const double* matrix;
} qs_param_gate;

/* Energy E = <psi|H|psi> of psi = U_m...U_1 |reg> and its gradient dE/dparams
 * by the adjoint method: one forward pass, then a reverse pass that un-applies
 * each gate from psi and from lambda = H psi and reads each rotation's
 * derivative off Im<lambda|A|psi> (FP64 accumulation; FP32-pipe compensated
 * sums on complex64 registers). No intermediate state is stored: memory is
 * three state vectors. The register's state is the initial state and is
 * unchanged on return. Gradients of rotations that share a parameter add up.
 * Errors: InvalidTarget / InvalidDimensions as try_apply_fast with err[2] =
 * gate index; QS_INVALID_ARGUMENT for a bad kind or parameter index. */
int qs_adjoint_gradient(qs_register* reg, const qs_param_gate* gates, size_t m, const double* params,
                        size_t nparams, const qs_pauli_term* terms, size_t nterms, double* energy,
                        double* grad, size_t* err);

/* ---- batched gradients (no counterpart in the reference) ------------------ */

/* One circuit of a batch: n qubits starting in |0..0>, gates (rotations, fixed
 * 1-qubit gates and CNOTs), its observable. */
typedef struct qs_batch_circuit {
    size_t n;
    const qs_param_gate* gates;
    size_t m;
    size_t nparams;
    const qs_pauli_term* terms;
    size_t nterms;
} qs_batch_circuit;

typedef struct qs_batch_options {
    int precision;       /* QS_PREC_C128 or QS_PREC_C64 */
    int chunk_log2;      /* amplitude pairs per work item = 2^chunk_log2; 0 = autotune */
    int ctas_per_sm;     /* persistent CTAs per SM; 0 = autotune */
    int arith;           /* QS_ARITH_DF64: complex128 stages of rotations and CNOTs in double-float
                            tiles; any other value: FP64 arithmetic */
} qs_batch_options;

typedef struct qs_batch qs_batch;

/* Prepare a batch: device states, gate and observable tables, the work-item
 * schedule, and a CUDA graph of the whole forward + adjoint pass (parameter
 * upload, state reset, one persistent kernel over all circuits, the
 * gradient reduction, result download). Validation errors carry err[2] =
 * circuit index. */
int qs_batch_create(const qs_batch_circuit* circuits, size_t count, const qs_batch_options* opts,
                    qs_batch** out, size_t* err);

/* Energies (count) and gradients (concatenated, nparams per circuit) for the
 * given parameters (concatenated likewise): one graph replay. QS_TIMEOUT if a
 * bounded dependency wait inside the persistent kernel gave up. */
int qs_batch_run(qs_batch* batch, const double* params, double* energies, double* grads);

/* The chunk size and CTAs per SM the batch runs with (after autotuning). */
int qs_batch_config(const qs_batch* batch, int* chunk_log2, int* ctas_per_sm);

void qs_batch_free(qs_batch* batch);

/* ---- OpenQASM 2.0 front end ---------------------------------------------- */

typedef struct qs_qasm_result qs_qasm_result;

/* openqasm::run_openqasm (src/openqasm.rs:52-142) on program text: one
 * register per qreg (all |0..0>), bits per creg; U, CX, measure, reset,
 * barrier, if(creg == n), gate definitions and the standard gates of
 * "qelib1.inc". Measurement draws come from a SplitMix64 generator seeded with
 * `seed` (the reference uses an unseeded thread_rng). Includes other than
 * qelib1.inc are read relative to base_dir (nullable). Errors:
 * QS_QASM_PARSE_ERROR (syntax, unknown names, bad arguments) and
 * QS_QASM_RUN_ERROR (CX across registers, a creg wider than 32 bits in an if),
 * message in qs_last_error(). */
int qs_qasm_run(const char* source, const char* base_dir, uint64_t seed, int precision, qs_qasm_result** out);

/* As qs_qasm_run on the contents of a file (includes relative to its directory). */
int qs_qasm_run_file(const char* path, uint64_t seed, int precision, qs_qasm_result** out);

/* OpenQASMResult's qregs / cregs maps (src/openqasm.rs:9-16), in declaration
 * order. Registers stay owned by the result. */
size_t qs_qasm_qreg_count(const qs_qasm_result* result);
const char* qs_qasm_qreg_name(const qs_qasm_result* result, size_t i);
qs_register* qs_qasm_qreg(qs_qasm_result* result, size_t i);
size_t qs_qasm_creg_count(const qs_qasm_result* result);
const char* qs_qasm_creg_name(const qs_qasm_result* result, size_t i);
size_t qs_qasm_creg_size(const qs_qasm_result* result, size_t i);
int qs_qasm_creg_bits(const qs_qasm_result* result, size_t i, uint8_t* bits);
void qs_qasm_free(qs_qasm_result* result);

/* ---- host views ---------------------------------------------------------- */

/* Read `pub state` (src/register.rs:35): 2^n complex, interleaved doubles. */
int qs_get_state(const qs_register* reg, double* dst);

/* Assign `pub state` (as examples/quantum_teleportation.rs:55-58 does). */
int qs_set_state(qs_register* reg, const double* src);

/* norm_sqr per amplitude, the numbers print_probabilities prints
 * (src/register.rs:379-384), computed on the GPU in FP64. */
int qs_probabilities(const qs_register* reg, double* dst);

/* PartialEq for Register (src/register.rs:409-413): equal when every
 * |a_i - b_i| < tol (the reference uses 1e-8). */
int qs_register_eq(const qs_register* a, const qs_register* b, double tol, int* equal);

/* Wait for all work queued on the register. */
int qs_synchronize(qs_register* reg);

/* The register's CUDA stream (cudaStream_t), for callers that time or order work. */
void* qs_register_stream(qs_register* reg);

/* Message for the last error on the calling host thread. */
const char* qs_last_error(void);

/* Number of kernels this library has launched in the process (all registers).
 * Diagnostic without a counterpart in the reference. */
uint64_t qs_launch_count(void);

/* Library version string. */
const char* qs_version(void);

/* Failure-detection self-test (no counterpart in the reference): runs the engine's two bounded
 * device waits, the mbarrier wait of the tile kernels and the completion-counter wait of the
 * batched kernel, on conditions nothing satisfies, with a ~0.1 s limit. Each wait gives up and
 * the out-parameters report 1 (timed out); the context stays usable, which the caller can check
 * with any later call. */
int qs_selftest_bounded_waits(int* mbar_timed_out, int* counter_timed_out);

#ifdef __cplusplus
}
#endif
#endif /* QUARU_GPU_H */
