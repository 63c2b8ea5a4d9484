// qs_stage.h — launch arguments of one tiled stage, shared by the tile kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "qs_device.cuh"
#include "qs_tile.h"

namespace qs {

struct StageArgs {
    int T, L, H;
    int op_begin, op_end;
    int RL, RH;            // copy rows: 2^RL contiguous amplitudes, 2^RH rows per tile
    int nbuf;              // tile buffers in the ring (2 or 3)
    IndexMap outer;        // expands a tile index into the base amplitude index
    uint8_t rhigh[kTileMaxHigh];  // global qubit of row bit b
};

// Stage arguments shared by the tile kernels: tile geometry, copy rows and the outer expansion.
inline StageArgs stage_args(const TileStage& st, int op_begin, int op_end) {
    StageArgs sa;
    std::memset(&sa, 0, sizeof(sa));
    sa.T = st.T;
    sa.L = st.L;
    sa.H = int(st.high.size());
    sa.op_begin = op_begin;
    sa.op_end = op_end;
    std::vector<int> qpos;
    for (int q = 0; q < st.L; q++) qpos.push_back(q);
    for (int q : st.high) qpos.push_back(q);
    std::sort(qpos.begin(), qpos.end());
    sa.outer.npos = int(qpos.size());
    for (size_t i = 0; i < qpos.size(); i++) sa.outer.pos[i] = uint8_t(qpos[i]);
    sa.outer.fixval = 0;
    // Copy rows: high qubits L, L + 1, ... continue the contiguous low run.
    int run = 0;
    while (run < sa.H && st.high[run] == st.L + run) run++;
    sa.RL = st.L + run;
    sa.RH = sa.H - run;
    for (int b = 0; b < sa.RH; b++) sa.rhigh[b] = uint8_t(st.high[run + b]);
    return sa;
}

// Tile buffers of the tensor-core stages are swizzled in shared memory at 16-byte granularity: the
// 16-byte unit u of a tile sits at swz16(u) = u ^ s(u >> 3), s a GF(2)-linear map of unit bits 3..7
// onto bits 0..2 (columns 7, 3, 5, 6, 1 for bits 3..7). A warp of the block kernels reads 32 tile
// columns that differ in the lowest tile bits outside the block; without the swizzle, blocks on the
// low tile bits send a quarter-warp's 16-byte accesses (or a half-warp's 8-byte accesses) to one
// bank group. Over all 792 placements of a 5-qubit block in a 12-qubit tile the swizzle brings the
// mean accesses per 16-byte slot from 2.75 to 1.16 for 16-byte elements and from 3.8 to 1.5 (per
// 8-byte slot) for 8-byte elements.
__host__ __device__ __forceinline__ uint32_t swz16(uint32_t u) {
    const uint32_t h = (u >> 3) & 31u;
    const uint32_t s = (uint32_t(__builtin_popcount(h & 0x17u)) & 1u) |
                       ((uint32_t(__builtin_popcount(h & 0x0Bu)) & 1u) << 1) |
                       ((uint32_t(__builtin_popcount(h & 0x0Du)) & 1u) << 2);
    return u ^ s;
}

// Block rows visited in Gray-code order: row gray_code(i) differs from the row before it in bit
// low_bit(i), so its offset is one XOR away (the swizzle is linear).
__host__ __device__ constexpr int gray_code(int i) { return i ^ (i >> 1); }
__host__ __device__ constexpr int low_bit(int i) { return (i & 1) ? 0 : (i & 2) ? 1 : (i & 4) ? 2 : 3; }

}  // namespace qs
