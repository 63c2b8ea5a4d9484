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
    if (op.kind == OP_BLOCK) return op.k == 5;
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
    const int D = (op.kind == OP_BLOCK) ? 0 : (1 << op.k);
    for (int r = 0; r < D; r++) {
        uint32_t o = 0;
        for (int b = 0; b < op.k; b++)
            if (r >> b & 1) o |= 1u << t.tb[b];
        t.off[r] = o;
    }
    if (op.kind == OP_BLOCK) {
        t.bidx = uint32_t(op.block) * kBlockFragFloat4;
    } else if (op.kind == OP_MONO || op.kind == OP_MONO_PF) {
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

// cvt.rna.tf32.f32 on the host: round to nearest (ties away) at 10 fraction bits.
static float tf32_rna(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b = (b + 0x1000u) & ~0x1FFFu;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

void block_fragments(const std::vector<double>& u, float* out) {
    auto M = [&](int n, int k) -> double {  // [[Ur, -Ui], [Ui, Ur]]
        const int r = n & 31, c = k & 31;
        const double re = u[2 * (r * 32 + c)], im = u[2 * (r * 32 + c) + 1];
        if ((n < 32) == (k < 32)) return re;
        return (n < 32) ? -im : im;
    };
    for (int nt = 0; nt < 8; nt++)
        for (int ks = 0; ks < 8; ks++)
            for (int lane = 0; lane < 32; lane++) {
                const int g = lane >> 2, t = lane & 3;
                const double v0 = M(8 * nt + g, 8 * ks + t), v1 = M(8 * nt + g, 8 * ks + t + 4);
                const float h0 = tf32_rna(float(v0)), h1 = tf32_rna(float(v1));
                float* o = out + 4 * ((nt * 8 + ks) * 32 + lane);
                o[0] = h0;
                o[1] = h1;
                o[2] = tf32_rna(float(v0 - double(h0)));
                o[3] = tf32_rna(float(v1 - double(h1)));
            }
}

// Whether a tile op can join a register group (k <= 1 dense or monomial).
static bool groupable(const TileOp& t) {
    if (t.kind == OP_DENSE || t.kind == OP_DENSE_REAL) return t.k == 1;
    if (t.kind == OP_MONO || t.kind == OP_MONO_PF) return t.k <= 1;
    return false;
}

static TileOp group_header(uint32_t gbits, int T, int count) {
    TileOp h;
    std::memset(&h, 0, sizeof(h));
    h.kind = OP_GROUP;
    h.k = uint8_t(count);
    std::vector<int> pos;
    for (int b = 0; b < T; b++)
        if (gbits >> b & 1u) pos.push_back(b);
    h.npos = uint8_t(pos.size());
    for (size_t i = 0; i < pos.size(); i++) h.pos[i] = uint8_t(pos[i]);
    int lo = 0;
    for (size_t j = 0; j <= pos.size(); j++) {
        const int hi = (j < pos.size()) ? pos[j] : 32;
        uint32_t m = 0;
        for (int b = lo; b < hi && b < 32; b++) m |= 1u << b;
        h.seg[j] = m;
        lo = hi + 1;
    }
    for (int j = 0; j < (1 << kGroupBits); j++) {
        uint32_t o = 0;
        for (int b = 0; b < kGroupBits; b++)
            if (j >> b & 1) o |= 1u << pos[b];
        h.off[j] = o;
    }
    return h;
}

std::vector<TileOp> stage_program(const std::vector<OpDesc>& ops, const TileStage& st, bool groups) {
    std::vector<TileOp> prog, members;
    uint32_t gbits = 0;
    auto flush = [&]() {
        if (members.size() >= 2) {
            // pad the group to exactly kGroupBits tile bits
            for (int b = 0; b < st.T && __builtin_popcount(gbits) < kGroupBits; b++) gbits |= 1u << b;
            std::vector<int> pos;
            for (int b = 0; b < st.T; b++)
                if (gbits >> b & 1u) pos.push_back(b);
            auto gl = [&](int lb) -> int {
                for (size_t i = 0; i < pos.size(); i++)
                    if (pos[i] == lb) return int(i);
                return -1;
            };
            prog.push_back(group_header(gbits, st.T, int(members.size())));
            for (TileOp m : members) {
                m.gj = (m.k == 1) ? uint8_t(gl(m.tb[0])) : 0;
                m.gcode = (m.kind == OP_DENSE) ? 0 : (m.kind == OP_DENSE_REAL) ? 1 : (m.k == 1) ? 2 : 3;
                // local fixed bits: positions other than the target, with values in lfixval
                for (int i = 0; i < m.npos; i++) {
                    const int lb = m.pos[i];
                    if (m.k == 1 && lb == m.tb[0]) continue;
                    const bool one = (m.lfixval >> lb) & 1u;
                    const int j = gl(lb);
                    if (j >= 0) {
                        m.gfin_mask |= uint8_t(1u << j);
                        if (one) m.gfin_val |= uint8_t(1u << j);
                    } else {
                        m.gfout_mask |= 1u << lb;
                        if (one) m.gfout_val |= 1u << lb;
                    }
                }
                prog.push_back(m);
            }
        } else {
            for (const TileOp& m : members) prog.push_back(m);
        }
        members.clear();
        gbits = 0;
    };
    for (int idx : st.ops) {
        TileOp t = make_tile_op(ops[idx], st);
        if (groups && st.T >= kGroupBits && groupable(t)) {
            const uint32_t need = (t.k == 1) ? (1u << t.tb[0]) : 0u;
            if (__builtin_popcount(gbits | need) > kGroupBits) flush();
            gbits |= need;
            members.push_back(t);
        } else {
            flush();
            prog.push_back(t);
        }
    }
    flush();
    return prog;
}

}  // namespace qs
