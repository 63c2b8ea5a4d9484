// qs_pass.cu — the warp-specialised stage kernel for complex64 stages made of register passes.
//
// A block is 8 (or 16) compute warps and 1 copy warp. The copy warp keeps a ring of tile buffers in
// shared memory filled with copies that complete on the buffer's `full` mbarrier (bulk TMA copies for
// long rows, per-lane 16-byte cp.async for short ones), and writes a finished tile back once the
// compute warps have arrived on its `done` mbarrier; a buffer is refilled only after it has been read. The compute warps never issue or wait on
// copies themselves: per tile they wait for `full`, run the stage's register passes (a named
// barrier among the 256 compute threads between passes), make their writes visible to the copy
// engine and arrive on `done`. Every wait is bounded; one that gives up raises the error flag and
// the block drains its copies before it exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "qs_device.cuh"
#include "qs_kernels.h"
#include "qs_pass.cuh"
#include "qs_tile.h"
#include "qs_tma.cuh"

namespace qs {

// NC compute threads (one tuple of 16 amplitudes each: 256 for 4096-amplitude tiles, 512 for 8192)
// plus the copy warp.

struct PassArgs {
    int T;
    int RL, RH;            // copy rows: 2^RL contiguous amplitudes, 2^RH rows per tile
    int nbuf;              // tile buffers in the ring (2 or 3)
    int op_begin, op_end;
    IndexMap outer;        // expands a tile index into the base amplitude index
    uint8_t rhigh[kTileMaxHigh];  // global qubit of row bit b
};

template <int NC>
__global__ void __maxnreg__(96) k_pass(float2* __restrict__ state, uint64_t ntiles,
                                                           const __grid_constant__ PassArgs pa,
                                                           const TileOp* __restrict__ ops, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t tsize = 1u << pa.T;
    const int nbuf = pa.nbuf, nops = pa.op_end - pa.op_begin, nrows = 1 << pa.RH;
    const bool bulk = nrows <= 8;
    // [tile buffers][full[4]][done[4]][tile base of each buffer[4]][ops (16-byte aligned)][row offsets]
    float2* bufs = reinterpret_cast<float2*>(smem_raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + size_t(nbuf) * (sizeof(float2) << pa.T));
    uint64_t* done = full + 4;
    uint64_t* tbase = done + 4;  // written by the copy warp before the load that completes full[b]
    TileOp* sops = reinterpret_cast<TileOp*>(tbase + 4);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(sops + nops);
    __shared__ volatile int s_abort;
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ops + pa.op_begin);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sops);
        const int words = nops * int(sizeof(TileOp) / 4);
        for (int w = threadIdx.x; w < words; w += NC + 32) dst[w] = src[w];
    }
    for (int r = threadIdx.x; r < nrows; r += NC + 32) {
        uint64_t o = 0;
        for (int b = 0; b < pa.RH; b++)
            if (r >> b & 1) o |= 1ull << pa.rhigh[b];
        rowoff[r] = o;
    }
    if (threadIdx.x == 0) {
        for (int b = 0; b < nbuf; b++) {
            mbar_init(&full[b], bulk ? 1 : 33);  // bulk: lane 0's expect-tx; pieces: 32 lanes + lane 0's release
            mbar_init(&done[b], NC);
        }
        fence_mbar_init();
        s_abort = 0;
    }
    __syncthreads();
    const uint64_t first = blockIdx.x;
    const uint64_t nmy = (ntiles > first) ? (ntiles - 1 - first) / gridDim.x + 1 : 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == NC / 32) {
        // ---------------------------------------------------------------- copy warp
        // Long rows (>= 4 KiB): a few bulk copies per tile. Short rows: every bulk copy costs the
        // copy engine ~90 cycles, so the lanes move the tile in 16-byte pieces instead (cp.async in,
        // shared loads + global stores out), a warp instruction covering 512 contiguous bytes.
        const uint32_t row_bytes = uint32_t(sizeof(float2)) << pa.RL;
        const uint32_t rmask = (1u << pa.RL) - 1u, chunks = tsize / 2;
        auto issue_load = [&](uint64_t i, int b) {
            const uint64_t tb = expand_index(first + i * gridDim.x, pa.outer);
            float2* dst = bufs + size_t(b) * tsize;
            if (bulk) {
                if (lane == 0) {
                    tbase[b] = tb;  // released to the compute warps by the mbarrier's phase completion
                    mbar_expect_tx(&full[b], row_bytes * uint32_t(nrows));
                }
                __syncwarp();
                for (int r = lane; r < nrows; r += 32)
                    bulk_load(dst + (size_t(r) << pa.RL), state + tb + rowoff[r], row_bytes, &full[b]);
            } else {
#pragma unroll 8
                for (uint32_t c = lane; c < chunks; c += 32) {
                    const uint32_t a = 2 * c;
                    cp_async16(dst + a, state + tb + rowoff[a >> pa.RL] + (a & rmask));
                }
                cp_async_mbar_arrive(&full[b]);  // one arrival per lane once its copies have landed
                if (lane == 0) {
                    tbase[b] = tb;
                    mbar_arrive(&full[b]);  // releases tbase[b]
                }
            }
        };
        uint64_t issued = 0;
        for (; issued < nmy && issued < uint64_t(nbuf); issued++) issue_load(issued, int(issued));
        uint64_t j = 0;
        int b = 0;
        uint32_t dphase = 0;  // bit b: parity of done[b]'s next completion
        bool ok = true;
        for (; j < nmy; j++) {
            int w = 1;
            if (lane == 0) w = mbar_wait_bounded(&done[b], (dphase >> b) & 1u) ? 1 : 0;
            w = __shfl_sync(0xffffffffu, w, 0);
            if (!w || s_abort) {
                ok = false;
                break;
            }
            dphase ^= 1u << b;
            const uint64_t base = expand_index(first + j * gridDim.x, pa.outer);
            float2* src = bufs + size_t(b) * tsize;
            if (bulk) {
                for (int r = lane; r < nrows; r += 32)
                    bulk_store(state + base + rowoff[r], src + (size_t(r) << pa.RL), row_bytes);
                bulk_commit();
            } else {
                // each lane stores exactly the pieces it loads, so its own later cp.async into this
                // buffer cannot overtake these shared-memory reads
#pragma unroll 8
                for (uint32_t c = lane; c < chunks; c += 32) {
                    const uint32_t a = 2 * c;
                    const float4 v = *reinterpret_cast<const float4*>(src + a);
                    *reinterpret_cast<float4*>(state + base + rowoff[a >> pa.RL] + (a & rmask)) = v;
                }
            }
            if (issued < nmy) {  // tile `issued` = j + nbuf takes this buffer once it has been read
                if (bulk) bulk_wait_read<0>();
                __syncwarp();
                issue_load(issued, b);
                issued++;
            }
            b = (b + 1 == nbuf) ? 0 : b + 1;
        }
        if (bulk) bulk_wait_all();
        if (!ok) {
            if (lane == 0) {
                s_abort = 1;
                atomicExch(err, 1);
                // loads the compute warps will not take: wait for them before the block exits
                for (uint64_t t = j; t < issued; t++)
                    mbar_wait_bounded(&full[int(t % uint64_t(nbuf))], uint32_t((t / uint64_t(nbuf)) & 1u));
            }
        }
        return;
    }

    // -------------------------------------------------------------------- compute warps
    uint32_t fphase = 0;  // bit b: parity of full[b]'s next completion
    int b = 0;
    for (uint64_t it = 0; it < nmy; it++) {
        if (!mbar_wait_bounded(&full[b], (fphase >> b) & 1u)) s_abort = 1;
        named_sync(1, NC);  // every compute thread sees the same s_abort
        if (s_abort) {
            if (threadIdx.x == 0) atomicExch(err, 1);
            break;
        }
        fphase ^= 1u << b;
        float2* s = bufs + size_t(b) * tsize;
        for (int o = 0; o < nops; o += int(sops[o].k) + 1) {
            if (o > 0) named_sync(1, NC);
            pass_run_c64<NC, true>(s, tsize, &tbase[b], &sops[o]);
        }
        fence_async_shared();  // this thread's writes, visible to the bulk stores
        mbar_arrive(&done[b]);
        b = (b + 1 == nbuf) ? 0 : b + 1;
    }
}

cudaError_t launch_pass(void* state, int n, const TileStage& st, int op_begin, int op_end, const TileOp* dops,
                        int* derr, cudaStream_t s, int sms) {
    PassArgs pa;
    std::memset(&pa, 0, sizeof(pa));
    pa.T = st.T;
    pa.op_begin = op_begin;
    pa.op_end = op_end;
    const int H = int(st.high.size());
    int run = 0;  // high qubits L, L + 1, ... continue the contiguous low run
    while (run < H && st.high[run] == st.L + run) run++;
    pa.RL = st.L + run;
    pa.RH = H - run;
    for (int b = 0; b < pa.RH; b++) pa.rhigh[b] = uint8_t(st.high[run + b]);
    std::vector<int> qpos;
    for (int q = 0; q < st.L; q++) qpos.push_back(q);
    for (int q : st.high) qpos.push_back(q);
    std::sort(qpos.begin(), qpos.end());
    pa.outer.npos = int(qpos.size());
    for (size_t i = 0; i < qpos.size(); i++) pa.outer.pos[i] = uint8_t(qpos[i]);
    pa.outer.fixval = 0;
    const size_t tile_bytes = sizeof(float2) << st.T;
    const size_t fixed =
        12 * sizeof(uint64_t) + sizeof(TileOp) * size_t(op_end - op_begin) + (sizeof(uint64_t) << pa.RH);
    // three buffers where two blocks still fit an SM (4096-amplitude tiles), or one block (8192)
    pa.nbuf = (3 * tile_bytes + fixed <= (st.T >= 13 ? 220 : 110) * 1024) ? 3 : 2;
    const size_t smem = size_t(pa.nbuf) * tile_bytes + fixed;
    const uint64_t ntiles = 1ull << (n - st.T);
    auto go = [&](auto kern, int nthreads) -> cudaError_t {
        int per_sm = 0;
        cudaError_t e = resident_blocks(reinterpret_cast<const void*>(kern), nthreads, smem, &per_sm);
        if (e != cudaSuccess) return e;
        const uint64_t grid = std::min<uint64_t>(ntiles, uint64_t(sms) * uint64_t(std::max(1, per_sm)));
        kern<<<int(grid), nthreads, smem, s>>>(static_cast<float2*>(state), ntiles, pa, dops, derr);
        return cudaSuccess;
    };
    cudaError_t e = (st.T >= 13) ? go(k_pass<512>, 512 + 32) : go(k_pass<256>, 256 + 32);
    if (e != cudaSuccess) return e;
    e = cudaGetLastError();
    if (e == cudaSuccess) note_launches(1);
    return e;
}

}  // namespace qs
