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
constexpr int kMaxStageOps = 64;       // gates per stage: the stage's op table lives in shared memory
constexpr int kPassBits = 4;           // register bits of a pass: 16 amplitudes per thread
constexpr int kLaneBits = 4;           // tile bits 0..3 live on the lanes of a warp during a pass
constexpr int kPassMinT = 9;           // passes need whole warps of tuples: 2^(T-4) >= 32
constexpr uint8_t OP_PASS = 10;        // TileOp kind of a register-pass header

// A gate inside a register pass (complex64 tiles). The pass holds 16 amplitudes per thread: the
// register bits R (4 tile bits >= 4, chosen per pass) index the thread's registers, tile bits 0..3
// are lane bits 0..3 of the warp, the remaining tile bits select the thread's tuple.
//
// Codes of a k = 1 gate: dense complex 2x2, dense real 2x2, swap (the rows exchanged: X, CNOT),
// swap with phases (Y), two-row phase (RZ); a k = 0 gate is a phase on one row (Z, S, phase, CZ).
enum PassCode : uint32_t { PC_DENSE = 0, PC_REAL = 1, PC_SWAP = 2, PC_SWAPPH = 3, PC_DIAG2 = 4 };
// Variant ids (PassMember::ctl bits 0-7): category in bits 4-7, its parameters in bits 0-3. The
// kernel dispatches on them with a shallow tree of bit tests and decodes nothing else.
//   0  dense gates with no controls on the register bits of mask M (1..4 gates, increasing bit
//      order, coefficients in consecutive entries)                                  low = M
//   1  swap on register bit J (X, CNOT with its control outside the registers)       low = J << 2 | all << 1
//   2  swap on register bit J where register bit C is 1 (CNOT inside the registers)  low = J << 2 | C
//   3  dense gate on a lane bit                                                      low = all << 1 | nocond
//   4  swap on a lane bit                                                            low = all << 1 | nocond
//   5  k = 0 phase                                                                   low = all << 1
//   6, 7, 8, 9  register gate with controls: dense, real, swap with phases, two-row phase
//                                                                                    low = J << 2 | all << 1
//   10, 11, 12  lane gate: real, swap with phases, two-row phase                     low = all << 1 | nocond
// all: no controls on the other register bits; nocond: no controls on tuple or lane bits.
enum PassCat : uint32_t {
    PV_DENSES = 0, PV_SWAP = 1, PV_SWAPC = 2, PV_LDENSE = 3, PV_LSWAP = 4, PV_PHASE = 5, PV_DENSE = 6,
    PV_REAL = 7, PV_SWAPPH = 8, PV_DIAG2 = 9, PV_LREAL = 10, PV_LSWAPPH = 11, PV_LDIAG2 = 12
};
struct alignas(16) PassMember {
    float u[8];     // dense: row-major 2x2 complex; real: m00, m01, m10, m11; swap with phases and
                    // two-row phase: factor of row 0 (u[0..1]) and row 1 (u[2..3]); k = 0: u[0..1]
    uint32_t ctl;   // variant id (bits 0-7) | entries it consumes - 1 (8-9) | lane bit (10-11) |
                    // controls outside the tile (12) | controls on tuple or lane bits (13)
    uint32_t fmv;   // register controls: mask (bits 0-3), values (4-7)
    uint32_t om;    // controls on tuple and lane bits (tile-local), compared with the tuple's base index
    uint32_t ov;
};

// Gate as the tile kernel sees it (local bit numbering inside the tile).
struct alignas(16) TileOp {
    PassMember pm;    // register-pass member fields (valid when the op follows an OP_PASS header)
    uint8_t kind;     // OpKind
    uint8_t k;        // sub-operation arity (<= 3); OP_PASS: number of members
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
    uint32_t bidx;       // OP_BLOCK: index of the block's operand images (each kernel knows their size)
};

// Tensor-core operand of one fused 5-qubit block: B = M, M = [[Ur, -Ui], [Ui, Ur]] (64 x 64 real,
// output n x input k), as two K-major core-matrix images (TF32 high parts, then low parts) of
// 4096 floats each; 32 KiB in all (kBlockFragFloat4 float4s).
constexpr uint32_t kBlockFragFloat4 = 8 * 8 * 32;
void block_fragments(const std::vector<double>& u32x32, float* out /* 4 * kBlockFragFloat4 floats */);

// Fused blocks per tensor-core stage: the stage's B images stay resident in shared memory.
constexpr int kMaxTcBlocks = 2;

// FP64-accurate operand of one fused 5-qubit block on complex128 registers (the split-integer
// product on the tensor cores, k_tile_oz): the block's real form B (64 x 64; input component
// k = 2j + c, output component n = 2i + c', c = 0 real, 1 imaginary), each output column scaled by
// its own power of two and rounded to a 55-bit integer, cut into 7 balanced base-256 digits: 7
// BF16 slices (digit s scaled by 2^-8s) in the K-major core-matrix layout (8 KiB each); then the 64
// output exponents (int32); then B itself in FP64, row n = output component (for amplitudes that
// are not finite). kOzFragBytes per block.
constexpr uint32_t kOzSliceBytes = 64u * 64u * 2u;
constexpr int kOzSlices = 7;
constexpr uint32_t kOzBBytes = kOzSlices * kOzSliceBytes;
constexpr uint32_t kOzScaleBytes = 256u;
constexpr uint32_t kOzFragBytes = kOzBBytes + kOzScaleBytes + 64u * 64u * 8u;
void oz_fragments(const std::vector<double>& u32x32, unsigned char* out /* kOzFragBytes */);

// Fused blocks per FP64-accurate tensor-core stage (the complex128 tiles take the room a second
// block's slices would need).
constexpr int kMaxOzBlocks = 1;

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
// qubit). exact_order keeps arithmetic gates in their original relative order; a stage holds at most
// max_ops (<= kMaxStageOps) gates. blocks_only (the tensor-core stages) admits OP_BLOCK ops only;
// every other op runs on its own.
std::vector<TileStage> plan_tiles(const std::vector<OpDesc>& ops, int n, int T, int L, bool exact_order,
                                  int max_ops = kMaxStageOps, bool blocks_only = false);

// Device image of one op inside `stage`.
TileOp make_tile_op(const OpDesc& op, const TileStage& stage);

// The device program of one stage: its ops in order, or (passes = true, complex64 tiles with
// T >= kPassMinT) runs of k <= 1 gates scheduled into register passes behind OP_PASS headers.
// Pass scheduling moves a gate only past gates that share no qubit with it.
std::vector<TileOp> stage_program(const std::vector<OpDesc>& ops, const TileStage& stage, bool passes);

// Whether a stage program (from stage_program) consists of register passes only, with the member
// variants the copy-warp pass kernel compiles (uncontrolled dense groups, swaps, uncontrolled lane
// dense gates, lane swaps, phases); other stages run in k_tile.
bool pass_only(const std::vector<TileOp>& prog);

// Launch the FP64-accurate complex128 block kernel for one stage (dops[op_begin] is its only op,
// an OP_BLOCK whose operand images start at frag + bidx * kOzFragBytes).
cudaError_t launch_tile_oz(void* state, int n, const TileStage& st, int op_begin, int op_end, const TileOp* dops,
                           const unsigned char* frag, int* derr, cudaStream_t s, int sms);

// Launch the warp-specialised complex64 pass kernel for one pass-only stage whose program is
// dops[op_begin, op_end).
cudaError_t launch_pass(void* state, int n, const TileStage& st, int op_begin, int op_end, const TileOp* dops,
                        int* derr, cudaStream_t s, int sms);

// Run stages on the device; ops are the host descriptors. With derr_dev null, waits for the stages and
// reports a tile kernel's bounded wait that gave up (QS_TIMEOUT); otherwise the kernels raise the
// caller's device flag *derr_dev (zeroed by the caller) and the call returns once the stages are
// queued, leaving the wait and the check to the caller.
int run_tiled(void* state, int n, int prec, int arith, const std::vector<OpDesc>& ops,
              const std::vector<TileStage>& stages, cudaStream_t s, int sms, std::string* msg,
              const std::vector<float>* block_frags = nullptr, int* derr_dev = nullptr);

}  // namespace qs
