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

// ---- fusion autotuner (qs_autotune.cpp) ----
struct TuneChoice {
    int fuse;   // 0 one sweep per gate, 1 cache-blocked stages, 2 dense blocks
    int width;  // block width (fuse 2)
    int tile;   // tile qubits (fuse 1; 0 = the automatic size)
};
struct TuneReport {
    TuneChoice best{1, 0, 0};
    std::vector<TuneChoice> cand;  // measured candidates (empty when the choice came from the cache)
    std::vector<double> ms;        // stand-in workload time per candidate
    bool from_cache = false;
};
// False when QS_AUTOTUNE is "off" or "0": the fixed automatic rules apply.
bool autotune_enabled();
// Candidates of `mode` (1: tile sizes of stages, 2: block widths 2..5, 3: both plus single sweeps).
std::vector<TuneChoice> tune_candidates(int n, int prec, int mode);
// Time the candidates of `mode` on a scratch register (or take the cached choice unless retune).
int tune_circuit(int n, int prec, int arith, int mode, bool retune, TuneReport* rep, int sms, std::string* msg);

}  // namespace qs
