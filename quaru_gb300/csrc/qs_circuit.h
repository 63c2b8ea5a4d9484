// qs_circuit.h — applying classified gates: single sweeps and fused stages.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "qs_internal.h"

namespace qs {

// Apply one classified gate (any width) in place on the register's stream.
int apply_op(void* state, int n, int prec, int arith, const OpDesc& op, cudaStream_t s, int sms, std::string* msg);

// Apply a classified gate list with the fusion strategy in `opts` (gates are
// the same list, unclassified, for dense-block fusion). derr_dev: see run_tiled.
int run_circuit(void* state, int n, int prec, int arith, const std::vector<OpDesc>& ops, const qs_gate* gates,
                const qs_circuit_options& opts, cudaStream_t s, int sms, std::string* msg, int* derr_dev = nullptr);

}  // namespace qs
