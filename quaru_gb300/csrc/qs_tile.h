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
constexpr int kGroupBits = 3;          // register-group width: 8 amplitudes per thread
constexpr uint8_t OP_GROUP = 10;       // TileOp kind of a register-group header

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
    // Register-group member fields (valid when the op follows an OP_GROUP header):
    uint8_t gj;          // group-local target bit (0..2)
    uint8_t gfin_mask;   // fixed bits inside the group (group-local)
    uint8_t gfin_val;
    uint8_t gcode;       // 0 dense, 1 dense real, 2 monomial k = 1, 3 phase on a fixed subspace (k = 0)
    uint32_t gfout_mask; // fixed bits inside the tile but outside the group (tile-local)
    uint32_t gfout_val;
    uint32_t bidx;       // OP_BLOCK: offset of the block's B fragments (float4 units)
    uint32_t pad2_;
};

// Tensor-core fragments of one fused 5-qubit block: [n-tile 8][k-step 8][lane 32] float4
// (b0_hi, b1_hi, b0_lo, b1_lo) of B = M^T, M = [[Ur, -Ui], [Ui, Ur]] (64 x 64 real).
constexpr uint32_t kBlockFragFloat4 = 8 * 8 * 32;
void block_fragments(const std::vector<double>& u32x32, float* out /* 4 * kBlockFragFloat4 floats */);

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

// The device program of one stage: its ops, with runs of 1-qubit gates whose
// targets span at most kGroupBits tile bits gathered behind OP_GROUP headers.
// Gate order is unchanged.
std::vector<TileOp> stage_program(const std::vector<OpDesc>& ops, const TileStage& stage, bool groups);

// Run stages on the device; ops are the host descriptors.
int run_tiled(void* state, int n, int prec, int arith, const std::vector<OpDesc>& ops,
              const std::vector<TileStage>& stages, cudaStream_t s, int sms, std::string* msg,
              const std::vector<float>* block_frags = nullptr);

}  // namespace qs
