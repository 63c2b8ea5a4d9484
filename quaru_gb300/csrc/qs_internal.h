// qs_internal.h — internal types shared by the host and device parts of the engine.
//
// A gate arrives as a dense 2^k x 2^k complex matrix plus targets, exactly like
// Quaru's Operation (src/operation.rs:49-52). The host classifies it once
// (qs_classify.cpp) into an OpDesc: the rows the gate leaves untouched are
// dropped, the local bits that every touched row shares become fixed bits
// (controls, including 0-controls), and the remaining sub-operation is either
// a monomial matrix (one non-zero per row and column: permutations, phases,
// X/Y/Z/S/CNOT/SWAP/Toffoli/CZ) or dense. Kernels then touch only the
// amplitudes a gate changes.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/quaru_gpu.h"

namespace qs {

enum OpKind : int {
    OP_NOOP = 0,        // identity: nothing to do
    OP_DENSE = 1,       // dense complex sub-matrix
    OP_DENSE_REAL = 2,  // dense sub-matrix whose imaginary parts are all zero
    OP_MONO = 3,        // one non-zero per row/column, general complex phases
    OP_MONO_PF = 4,     // one non-zero per row/column, every value in {1, -1, i, -i}
    OP_BLOCK = 11,      // fused dense 5-qubit block (tensor-core tiles)
};

// Phase classes of OP_MONO_PF rows (value-exact moves, no arithmetic).
enum PfClass : uint8_t { PF_ONE = 0, PF_NEG = 1, PF_I = 2, PF_NEG_I = 3, PF_SKIP = 4 };

constexpr int kMaxSmallK = 5;  // sub-operations up to 5 qubits run with the matrix in kernel params
constexpr int kMaxBigK = 14;   // larger dense/monomial sub-operations run out of place

// Classified gate in global qubit numbering.
struct OpDesc {
    int kind = OP_NOOP;
    int k = 0;                 // sub-operation arity
    int orig_k = 0;            // arity of the gate as given (sets the exact dot-product order)
    int tq[64] = {0};          // global qubit of sub-operation local bit j
    uint64_t fixmask = 0;      // global bits fixed by the gate's structure
    uint64_t fixval = 0;       // their values
    std::vector<double> m;     // dense: 2^k x 2^k complex, row-major, interleaved
    std::vector<int8_t> lane;  // exact order: lane of each sub-column (orig column & 7), -1 = sequential
    std::vector<uint32_t> perm;   // monomial: source sub-index of each row
    std::vector<double> phase;    // monomial: complex factor of each row
    std::vector<uint8_t> pf;      // monomial: PfClass per row (PF_SKIP for untouched rows)
    uint64_t touched_rows = 0;    // number of sub-rows the gate rewrites (for byte accounting)
    int block = -1;               // OP_BLOCK: index of the fused block
};

// Shape/target validation in the order of Register::try_apply_fast
// (src/register.rs:141-153). Returns QS_OK or a status with err filled.
int validate_gate(size_t n, size_t rows, size_t cols, const size_t* targets, size_t k, size_t* err,
                  std::string* msg);

// Build the OpDesc of a validated gate.
void classify_gate(const double* matrix, size_t k, const size_t* targets, OpDesc* out);

// Algorithmic HBM bytes one application of `op` moves on an n-qubit state with
// `amp_bytes` bytes per amplitude (one read + one write of every touched amplitude).
double op_bytes(const OpDesc& op, int n, int amp_bytes);

}  // namespace qs
