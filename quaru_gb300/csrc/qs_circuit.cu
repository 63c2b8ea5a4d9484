// qs_circuit.cu — gate dispatch and the circuit runner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "qs_circuit.h"
#include "qs_kernels.h"
#include "qs_fuse.h"
#include "qs_tile.h"

namespace qs {

static int fail(cudaError_t e, const char* what, std::string* msg) {
    if (msg) *msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return QS_OUT_OF_MEMORY;
    }
    return QS_CUDA_ERROR;
}

int apply_op(void* state, int n, int prec, int arith, const OpDesc& op, cudaStream_t s, int sms, std::string* msg) {
    if (op.kind == OP_NOOP) return QS_OK;
    if (op.k <= kMaxSmallK) {
        cudaError_t e = launch_op(op, state, n, prec, arith, s, sms);
        return e == cudaSuccess ? QS_OK : fail(e, "gate kernel", msg);
    }
    if (op.k > kMaxBigK) {
        if (msg) *msg = "dense or monomial sub-operation wider than " + std::to_string(kMaxBigK) + " qubits";
        return QS_INVALID_ARGUMENT;
    }
    // Wide gate: tables in device memory, read the pre-gate state from a copy.
    std::vector<uint64_t> off, off_src;
    std::vector<uint8_t> pf;
    std::vector<int8_t> lane;
    std::vector<unsigned char> mat;
    big_op_host_tables(op, prec, &off, &off_src, &pf, &lane, &mat);
    const size_t amp = prec == QS_PREC_C64 ? 8 : 16;
    const size_t sbytes = (size_t(1) << n) * amp;
    unsigned char* blob = nullptr;
    const size_t o_off = 0, o_src = o_off + off.size() * 8, o_pf = o_src + off_src.size() * 8,
                 o_lane = o_pf + ((pf.size() + 15) / 16) * 16, o_mat = o_lane + ((lane.size() + 15) / 16) * 16,
                 o_state = o_mat + ((mat.size() + 255) / 256) * 256, total = o_state + sbytes;
    cudaError_t e = cudaMallocAsync((void**)&blob, total, s);
    if (e != cudaSuccess) return fail(e, "wide gate buffers", msg);
    BigOpBuffers b;
    b.off = reinterpret_cast<const uint64_t*>(blob + o_off);
    b.off_src = reinterpret_cast<const uint64_t*>(blob + o_src);
    b.pf = blob + o_pf;
    b.lane = reinterpret_cast<const int8_t*>(blob + o_lane);
    b.mat = blob + o_mat;
    if (!off.empty()) e = cudaMemcpyAsync(blob + o_off, off.data(), off.size() * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !off_src.empty())
        e = cudaMemcpyAsync(blob + o_src, off_src.data(), off_src.size() * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !pf.empty()) e = cudaMemcpyAsync(blob + o_pf, pf.data(), pf.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !lane.empty())
        e = cudaMemcpyAsync(blob + o_lane, lane.data(), lane.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !mat.empty()) e = cudaMemcpyAsync(blob + o_mat, mat.data(), mat.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(blob + o_state, state, sbytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = launch_op_big(op, state, blob + o_state, n, prec, arith, b, s, sms);
    cudaFreeAsync(blob, s);
    return e == cudaSuccess ? QS_OK : fail(e, "wide gate", msg);
}

// fuse == 2: dense blocks of up to max_width qubits. On registers of at least 12 qubits, complex64
// or complex128 in fixed-point arithmetic, the blocks run on the tensor cores inside 12-qubit
// tiles; otherwise each block is one dense gate sweep.
static int run_blocks(void* state, int n, int prec, int arith, const qs_gate* gates, size_t m,
                      const qs_circuit_options& opts, cudaStream_t s, int sms, std::string* msg) {
    // Tensor-core blocks inside 12-qubit tiles: 3xTF32 on complex64 registers; on complex128
    // registers in fixed-point arithmetic, the FP64-accurate split-integer product (k_tile_oz).
    const bool oz = (prec == QS_PREC_C128) && arith == QS_ARITH_FX64 && n >= 12;
    const bool tensor = ((prec == QS_PREC_C64) && n >= 12) || oz;
    // automatic width: where each block's sweep stays cheap. Tensor-core blocks cost the same at any
    // width up to 5; complex128 double-float blocks run the double-float dense kernel up to 3
    // qubits (4- and 5-qubit blocks fall back to FP64, which GB300 runs at 1/64 of the FP32 rate);
    // FP64 blocks cost as many FP64 operations per amplitude as the gates they fuse, so 2 only halves
    // the sweeps.
    const int autow = tensor ? 5 : (prec == QS_PREC_C128 && arith == QS_ARITH_DF64) ? 3 : 2;
    const int W = std::max(2, std::min(5, opts.max_width > 0 ? opts.max_width : autow));
    std::vector<FusedBlock> blocks = fuse_blocks(gates, m, W);
    std::vector<OpDesc> ops;
    std::vector<float> frags;
    for (FusedBlock& b : blocks) {
        std::vector<size_t> tq(b.qubits.begin(), b.qubits.end());
        OpDesc op;
        if (tensor && int(b.qubits.size()) <= 5) {
            pad_block(&b, 5, n);
            op.kind = OP_BLOCK;
            op.k = 5;
            op.orig_k = 5;
            for (int j = 0; j < 5; j++) op.tq[j] = b.qubits[j];
            op.touched_rows = 32;
            const size_t per = oz ? kOzFragBytes / 4 : 4 * kBlockFragFloat4;  // floats per block
            op.block = int(frags.size() / per);
            frags.resize(frags.size() + per);
            if (oz)
                oz_fragments(b.u, reinterpret_cast<unsigned char*>(frags.data() + frags.size() - per));
            else
                block_fragments(b.u, frags.data() + frags.size() - per);
        } else {
            tq.assign(b.qubits.begin(), b.qubits.end());
            classify_gate(b.u.data(), tq.size(), tq.data(), &op);
        }
        ops.push_back(std::move(op));
    }
    if (!tensor) {
        for (const OpDesc& op : ops) {
            int rc = apply_op(state, n, prec, arith, op, s, sms, msg);
            if (rc) return rc;
        }
        return QS_OK;
    }
    const int T = std::min(12, n), L = std::min(5, T);
    std::vector<TileStage> stages = plan_tiles(ops, n, T, L, false, oz ? kMaxOzBlocks : kMaxTcBlocks, true);
    return run_tiled(state, n, prec, arith, ops, stages, s, sms, msg, &frags);
}

int run_circuit(void* state, int n, int prec, int arith, const std::vector<OpDesc>& ops, const qs_gate* gates,
                const qs_circuit_options& opts, cudaStream_t s, int sms, std::string* msg, int* derr_dev) {
    if (opts.fuse == 2 && gates) return run_blocks(state, n, prec, arith, gates, ops.size(), opts, s, sms, msg);
    if (opts.fuse >= 1) {
        // Tile qubits: 32 KiB of shared memory per tile by default; below 19 (complex64) or 18
        // (complex128) qubits smaller tiles, so that up to 128 blocks share the state (complex64
        // keeps the 9 tile qubits its register passes need).
        int T = opts.tile_qubits;
        if (T <= 0) {
            const int cap = prec == QS_PREC_C64 ? 12 : 11, floor = prec == QS_PREC_C64 ? 9 : 8;
            T = std::max(floor, std::min(cap, n - 7));
        }
        T = std::min(T, n);
        const int L = std::min(5, T);
        std::vector<TileStage> stages =
            plan_tiles(ops, n, T, L, prec == QS_PREC_C128 && arith == QS_ARITH_EXACT);
        return run_tiled(state, n, prec, arith, ops, stages, s, sms, msg, nullptr, derr_dev);
    }
    for (size_t g = 0; g < ops.size(); g++) {
        int rc = apply_op(state, n, prec, arith, ops[g], s, sms, msg);
        if (rc) return rc;
    }
    return QS_OK;
}

}  // namespace qs
