// qs_fuse.h — fusion of consecutive gates into dense blocks of up to W qubits.
#pragma once

#include <vector>

#include "qs_internal.h"

namespace qs {

struct FusedBlock {
    std::vector<int> qubits;    // sorted global qubits; local bit j of the matrix <-> qubits[j]
    std::vector<double> u;      // 2^k x 2^k complex, row-major, interleaved (FP64 product of the members)
    std::vector<int> members;   // gate indices, in application order
};

// Greedy fusion: each pass opens a block and absorbs every remaining gate that
// fits within W qubits and commutes with all gates deferred before it.
// Matrices are multiplied on the host in FP64. Gates wider than W become
// blocks of their own (their own matrix).
std::vector<FusedBlock> fuse_blocks(const qs_gate* gates, size_t m, int W);

// Widen a block to exactly `k` qubits by adding the lowest qubits of `allowed`
// that it does not use (identity on them).
void pad_block(FusedBlock* b, int k, int n);

}  // namespace qs
