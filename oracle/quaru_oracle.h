/*
 * quaru_oracle.h — CPU oracle for the Quaru register path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * algorithm (DATX11-22/quaru, src/register.rs), the oracle the GPU engine's
 * results are compared with. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it. The product library never links or calls it.
 *
 * Parity status: pinned by the reference's own known-answer tests
 * (tests/register_operation_tests.rs, examples/shors.rs:434-503,
 * examples/grovers.rs:274-312, examples/superdense_coding.rs:84-97,
 * examples/quantum_teleportation.rs:150-164), restated in
 * tests/test_oracle.py. The reference cannot be compiled in this container
 * (no Rust toolchain), so the summation order of ndarray 0.15.6's
 * `Array2::dot(&Array1)` is restated from that crate's published source
 * (numeric_util::unrolled_dot); it is not checked against a running build.
 */
#ifndef QUARU_ORACLE_H
#define QUARU_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (mirror OperationError, src/register.rs:10-20). */
#define ORC_OK 0
#define ORC_INVALID_TARGET 1
#define ORC_INVALID_DIMENSIONS 2
#define ORC_INVALID_ARITY 3
#define ORC_INVALID_QUBIT 4

/* All complex arrays are interleaved (re, im) doubles, the memory layout of
 * ndarray's Array2<Complex<f64>> in standard order. Matrices are row-major. */

/* Register::new (src/register.rs:41-56): kron fold of |0>/|1> vectors. */
void orc_register_new(const uint8_t* bits, size_t n, double* state);

/* Register::from_int (src/register.rs:58-63) via math::int_to_state (src/math.rs:44-49). */
void orc_register_from_int(size_t n, size_t k, double* state);

/* Register::try_from_qubits (src/register.rs:81-102) with the is_one check
 * (src/register.rs:107-115). qubits: n entries of 2 complex amplitudes.
 * Returns ORC_INVALID_QUBIT with err[0] = first bad qubit index. */
int orc_register_try_from_qubits(const double* qubits, size_t n, double* state, size_t* err);

/* Register::try_apply_fast (src/register.rs:140-191). Out-of-place update
 * through a full copy of the state, as the reference does. */
int orc_try_apply_fast(double* state, size_t n, const double* matrix, size_t rows, size_t cols,
                       const size_t* targets, size_t k, size_t* err);

/* Register::try_apply_all (src/register.rs:267-281): dense kron of the 1-qubit
 * matrix n times and one mat-vec. O(4^n): for n <= 10 in tests. */
int orc_try_apply_all(double* state, size_t n, const double* matrix, size_t rows, size_t cols,
                      size_t k, size_t* err);

/* Register::try_measure (src/register.rs:297-342) with the uniform draw
 * injected (the reference draws it from an unseeded thread_rng, :317-318).
 * prob0/prob1 (nullable) receive the two sequential sums. */
int orc_try_measure(double* state, size_t n, size_t target, double draw, int* outcome,
                    double* prob0, double* prob1, size_t* err);

/* norm_sqr of every amplitude (the values print_probabilities shows, src/register.rs:379-384). */
void orc_probabilities(const double* state, size_t n, double* probs);

/* Apply a list of gates in order (repeated try_apply_fast). Gate g has arity
 * ks[g], targets at targets[toff[g] ..], matrix at matrices[moff[g] ..] (in
 * doubles). Returns the first error; err[2] = failing gate index. */
int orc_apply_sequence(double* state, size_t n, size_t m, const size_t* ks, const size_t* toff,
                       const size_t* targets, const size_t* moff, const double* matrices,
                       size_t* err);

#ifdef __cplusplus
}
#endif
#endif
