// qs_plan.cpp — the tile planner: packs gates into cache-blocked stages.
//
// No counterpart in the reference, whose QuantumCircuit reduction passes
// (src/operation.rs:114-269) multiply matrices instead; here gates keep their
// own arithmetic, so a planned circuit gives exactly the amplitudes of the
// gate-by-gate run. Gates are moved earlier only past gates with which they
// share no qubit (they commute). Commuting is exact in real arithmetic but
// not in floating point: two arithmetic gates on disjoint qubits round in a
// different order when swapped. With exact_order (QS_ARITH_EXACT) a gate that
// does arithmetic therefore never moves past another one; only pure moves
// (permutations with factors 1, -1, i, -i) pass or are passed, which is
// value-exact.
#include <algorithm>
#include <cstring>
#include <set>

#include "qs_tile.h"

namespace qs {

bool tileable(const OpDesc& op) {
    if (op.kind == OP_NOOP) return true;
    if (op.k + __builtin_popcountll(op.fixmask) > 16) return false;
    if (op.kind == OP_DENSE || op.kind == OP_DENSE_REAL) return op.k == 1;
    return op.k <= 3;  // monomial
}

static uint64_t qubit_mask(const OpDesc& op) {
    uint64_t m = op.fixmask;
    for (int j = 0; j < op.k; j++) m |= 1ull << op.tq[j];
    return m;
}

static bool pure_move(const OpDesc& op) { return op.kind == OP_MONO_PF || op.kind == OP_NOOP; }

std::vector<TileStage> plan_tiles(const std::vector<OpDesc>& ops, int n, int T, int L, bool exact_order) {
    std::vector<TileStage> stages;
    if (T > n) T = n;
    if (L > T) L = T;
    const int H = std::min(T - L, kTileMaxHigh);
    const uint64_t low_mask = (L >= 64) ? ~0ull : ((1ull << L) - 1ull);
    std::vector<int> remaining;
    for (size_t i = 0; i < ops.size(); i++)
        if (ops[i].kind != OP_NOOP) remaining.push_back(int(i));
    while (!remaining.empty()) {
        TileStage st;
        st.tiled = true;
        st.T = L + H;
        st.L = L;
        uint64_t high = 0, blocked = 0;
        bool arith_deferred = false;  // an arithmetic gate has been deferred in this pass
        std::vector<int> rest;
        for (int idx : remaining) {
            const OpDesc& op = ops[idx];
            const uint64_t qm = qubit_mask(op);
            if ((qm & blocked) || (exact_order && arith_deferred && !pure_move(op))) {
                blocked |= qm;
                if (!pure_move(op)) arith_deferred = true;
                rest.push_back(idx);
                continue;
            }
            uint64_t need = 0;
            for (int j = 0; j < op.k; j++) need |= 1ull << op.tq[j];
            need &= ~low_mask;
            if (tileable(op) && __builtin_popcountll(high | need) <= H) {
                high |= need;
                st.ops.push_back(idx);
            } else {
                blocked |= qm;
                if (!pure_move(op)) arith_deferred = true;
                rest.push_back(idx);
            }
        }
        if (st.ops.empty()) {
            // The first remaining gate cannot be tiled: it runs on its own.
            TileStage single;
            single.single = remaining[0];
            stages.push_back(single);
            remaining.erase(remaining.begin());
            continue;
        }
        // Fill unused high slots with the lowest free qubits above L so every tile has T qubits.
        for (int q = L; q < n && __builtin_popcountll(high) < H; q++) high |= 1ull << q;
        for (int q = 0; q < 64; q++)
            if (high >> q & 1ull) st.high.push_back(q);
        st.T = L + int(st.high.size());
        stages.push_back(st);
        remaining.swap(rest);
    }
    return stages;
}

TileOp make_tile_op(const OpDesc& op, const TileStage& st) {
    TileOp t;
    std::memset(&t, 0, sizeof(t));
    auto local = [&](int q) -> int {
        if (q < st.L) return q;
        for (size_t i = 0; i < st.high.size(); i++)
            if (st.high[i] == q) return st.L + int(i);
        return -1;
    };
    t.kind = uint8_t(op.kind);
    t.k = uint8_t(op.k);
    std::vector<int> pos;
    for (int j = 0; j < op.k; j++) {
        t.tb[j] = uint8_t(local(op.tq[j]));
        pos.push_back(t.tb[j]);
    }
    for (int b = 0; b < 64; b++) {
        if (!(op.fixmask >> b & 1ull)) continue;
        const int lb = local(b);
        const bool one = (op.fixval >> b) & 1ull;
        if (lb >= 0) {
            pos.push_back(lb);
            if (one) t.lfixval |= 1u << lb;
        } else {
            t.omask |= 1ull << b;
            if (one) t.oval |= 1ull << b;
        }
    }
    std::sort(pos.begin(), pos.end());
    t.npos = uint8_t(pos.size());
    for (size_t i = 0; i < pos.size() && i < 16; i++) t.pos[i] = uint8_t(pos[i]);
    if (pos.size() <= 4) {
        // Segment j of the expanded index holds the bits between the (j-1)-th and
        // j-th inserted zero; tuple bits land there shifted left by j.
        int lo = 0;
        for (size_t j = 0; j <= pos.size(); j++) {
            const int hi = (j < pos.size()) ? pos[j] : 32;
            uint32_t m = 0;
            for (int b = lo; b < hi && b < 32; b++) m |= 1u << b;
            t.seg[j] = m;
            lo = hi + 1;
        }
    }
    const int D = 1 << op.k;
    for (int r = 0; r < D; r++) {
        uint32_t o = 0;
        for (int b = 0; b < op.k; b++)
            if (r >> b & 1) o |= 1u << t.tb[b];
        t.off[r] = o;
    }
    if (op.kind == OP_MONO || op.kind == OP_MONO_PF) {
        for (int r = 0; r < D; r++) {
            t.offsrc[r] = t.off[op.perm[r]];
            t.pf[r] = op.pf[r];
            t.m[2 * r] = op.phase[2 * r];
            t.m[2 * r + 1] = op.phase[2 * r + 1];
        }
    } else if (op.kind == OP_DENSE || op.kind == OP_DENSE_REAL) {
        for (int i = 0; i < 8; i++) t.m[i] = op.m[i];
        // double-float coefficients, same layout as the single-gate kernel
        const int row[4] = {0, 0, 1, 1};
        for (int o = 0; o < 4; o++) {
            const bool im_out = o & 1;
            for (int u = 0; u < 4; u++) {
                const int col = u >> 1;
                const bool cross = u & 1;
                const int idx = 2 * (row[o] * 2 + col);
                const double v = !cross ? op.m[idx] : (im_out ? op.m[idx + 1] : -op.m[idx + 1]);
                const float h = float(v);
                t.dfh[4 * o + u] = h;
                t.dfl[4 * o + u] = float(v - double(h));
            }
        }
    }
    for (int i = 0; i < 16; i++) t.mf[i] = float(t.m[i]);
    return t;
}

}  // namespace qs
