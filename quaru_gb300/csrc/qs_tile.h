// qs_tile.h — cache-blocked (tiled) circuit stages.
//
// A stage is a run of gates whose targets all fall inside one tile: the
// qubits 0..L-1 (contiguous in memory, so tile rows are coalesced) plus up to
// H = T - L higher qubits. Every tile of 2^T amplitudes is read from HBM
// once, all of the stage's gates are applied to it in shared memory, and it is
// written back once. Fixed bits (controls) may lie outside the tile: they
// become a per-tile condition.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "qs_internal.h"

namespace qs {

constexpr int kTileMaxHigh = 8;

// Gate as the tile kernel sees it (local bit numbering inside the tile).
struct TileOp {
    uint8_t kind;     // OpKind
    uint8_t k;        // sub-operation arity (<= 3)
    uint8_t tb[3];    // local bit of sub-operation target j
    uint8_t npos;     // number of sorted local positions below
    uint8_t pos[16];  // sorted local bits of targets and local fixed bits (for tuple expansion)
    uint32_t lfixval; // local fixed bits' values
    uint32_t seg[5];  // npos <= 4: expanded tuple index = OR_j ((t << j) & seg[j])
    uint64_t omask;   // fixed bits outside the tile (global positions)
    uint64_t oval;    // their required values
    uint32_t off[8];  // local offset of sub-row r
    uint32_t offsrc[8];  // local offset of its source row (monomial)
    uint8_t pf[8];    // monomial phase classes (PF_SKIP = untouched, 255 = general phase)
    double m[16];     // dense 1q matrix (interleaved) or monomial phases (8 rows x 2)
    float dfh[16];    // dense 1q double-float coefficients (see Dense1Args)
    float dfl[16];
    float mf[16];     // m rounded to float (complex64 registers)
};

struct TileStage {
    bool tiled = false;
    int single = -1;            // index of the op run on its own when !tiled
    int T = 0, L = 0;
    std::vector<int> high;      // sorted global qubits on local bits L..T-1
    std::vector<int> ops;       // op indices, in execution order
};

// Whether the tile kernel can run `op` (targets must still fit the tile).
bool tileable(const OpDesc& op);

// Greedy stage planner with reordering of commuting gates (gates that share no
// qubit). exact_order keeps arithmetic gates in their original relative order.
std::vector<TileStage> plan_tiles(const std::vector<OpDesc>& ops, int n, int T, int L, bool exact_order);

// Device image of one op inside `stage`.
TileOp make_tile_op(const OpDesc& op, const TileStage& stage);

// Run stages on the device; ops are the host descriptors.
int run_tiled(void* state, int n, int prec, int arith, const std::vector<OpDesc>& ops,
              const std::vector<TileStage>& stages, cudaStream_t s, int sms, std::string* msg);

}  // namespace qs
