// qs_fuse.cpp — dense-block gate fusion (host, FP64).
//
// The reference's closest feature is QuantumCircuit's reduction passes
// (src/operation.rs:114-269), which multiply or kron neighbouring gates by
// heuristics (and cancel equal consecutive real gates, which is only correct
// for involutions). Here a block is the exact FP64 product of the gates it
// absorbs, in their application order; a gate is moved ahead only past gates
// with which it shares no qubit.
#include "qs_fuse.h"

#include <algorithm>
#include <cstring>

namespace qs {

static uint64_t gate_mask(const qs_gate& g) {
    uint64_t m = 0;
    for (size_t j = 0; j < g.k; j++) m |= 1ull << g.targets[j];
    return m;
}

// U <- G_expanded * U, where U is 2^k x 2^k over `qubits` and G acts on a subset.
static void left_multiply(std::vector<double>& U, const std::vector<int>& qubits, const qs_gate& g) {
    const int k = int(qubits.size());
    const uint64_t dim = 1ull << k;
    const int kg = int(g.k);
    const uint64_t gd = 1ull << kg;
    std::vector<int> lb(kg);  // local bit of gate target j inside the block
    uint64_t gmask = 0;
    for (int j = 0; j < kg; j++) {
        lb[j] = int(std::find(qubits.begin(), qubits.end(), int(g.targets[j])) - qubits.begin());
        gmask |= 1ull << lb[j];
    }
    std::vector<double> col(2 * gd), out(2 * gd);
    for (uint64_t c = 0; c < dim; c++) {            // every column of U is a state over the block
        for (uint64_t base = 0; base < dim; base++) {
            if (base & gmask) continue;
            for (uint64_t i = 0; i < gd; i++) {
                uint64_t r = base;
                for (int j = 0; j < kg; j++)
                    if (i >> j & 1) r |= 1ull << lb[j];
                col[2 * i] = U[2 * (r * dim + c)];
                col[2 * i + 1] = U[2 * (r * dim + c) + 1];
            }
            for (uint64_t i = 0; i < gd; i++) {
                double re = 0.0, im = 0.0;
                for (uint64_t j = 0; j < gd; j++) {
                    const double gr = g.matrix[2 * (i * gd + j)], gi = g.matrix[2 * (i * gd + j) + 1];
                    re += gr * col[2 * j] - gi * col[2 * j + 1];
                    im += gr * col[2 * j + 1] + gi * col[2 * j];
                }
                out[2 * i] = re;
                out[2 * i + 1] = im;
            }
            for (uint64_t i = 0; i < gd; i++) {
                uint64_t r = base;
                for (int j = 0; j < kg; j++)
                    if (i >> j & 1) r |= 1ull << lb[j];
                U[2 * (r * dim + c)] = out[2 * i];
                U[2 * (r * dim + c) + 1] = out[2 * i + 1];
            }
        }
    }
}

std::vector<FusedBlock> fuse_blocks(const qs_gate* gates, size_t m, int W) {
    std::vector<FusedBlock> blocks;
    std::vector<int> remaining(m);
    for (size_t i = 0; i < m; i++) remaining[i] = int(i);
    while (!remaining.empty()) {
        uint64_t bq = 0, blocked = 0;
        std::vector<int> members, rest;
        for (int idx : remaining) {
            const uint64_t qm = gate_mask(gates[idx]);
            if (qm & blocked) {
                blocked |= qm;
                rest.push_back(idx);
                continue;
            }
            if (__builtin_popcountll(bq | qm) <= W || members.empty()) {
                if (__builtin_popcountll(bq | qm) > W) {  // a gate wider than W: its own block
                    members.push_back(idx);
                    bq |= qm;
                    blocked = ~0ull;  // close the block
                    continue;
                }
                bq |= qm;
                members.push_back(idx);
            } else {
                blocked |= qm;
                rest.push_back(idx);
            }
        }
        FusedBlock b;
        for (int q = 0; q < 64; q++)
            if (bq >> q & 1ull) b.qubits.push_back(q);
        const uint64_t dim = 1ull << b.qubits.size();
        b.u.assign(2 * dim * dim, 0.0);
        for (uint64_t i = 0; i < dim; i++) b.u[2 * (i * dim + i)] = 1.0;
        for (int idx : members) left_multiply(b.u, b.qubits, gates[idx]);
        b.members = members;
        blocks.push_back(std::move(b));
        remaining.swap(rest);
    }
    return blocks;
}

void pad_block(FusedBlock* b, int k, int n) {
    while (int(b->qubits.size()) < k) {
        int q = 0;
        while (q < n && std::find(b->qubits.begin(), b->qubits.end(), q) != b->qubits.end()) q++;
        if (q >= n) return;
        // insert q keeping qubits sorted; the matrix gains an identity factor on q
        std::vector<int> nq = b->qubits;
        nq.push_back(q);
        std::sort(nq.begin(), nq.end());
        const int pos = int(std::find(nq.begin(), nq.end(), q) - nq.begin());
        const uint64_t od = 1ull << b->qubits.size(), nd = od << 1;
        std::vector<double> nu(2 * nd * nd, 0.0);
        auto expand = [&](uint64_t i, uint64_t bit) {  // insert `bit` at position pos of index i
            const uint64_t lo = i & ((1ull << pos) - 1ull);
            return ((i >> pos) << (pos + 1)) | (bit << pos) | lo;
        };
        for (uint64_t r = 0; r < od; r++)
            for (uint64_t c = 0; c < od; c++)
                for (uint64_t bit = 0; bit < 2; bit++) {
                    const uint64_t R = expand(r, bit), C = expand(c, bit);
                    nu[2 * (R * nd + C)] = b->u[2 * (r * od + c)];
                    nu[2 * (R * nd + C) + 1] = b->u[2 * (r * od + c) + 1];
                }
        b->qubits = nq;
        b->u.swap(nu);
    }
}

}  // namespace qs
