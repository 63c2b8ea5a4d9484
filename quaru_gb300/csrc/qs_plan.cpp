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

std::vector<TileStage> plan_tiles(const std::vector<OpDesc>& ops, int n, int T, int L, bool exact_order,
                                  int max_ops, bool blocks_only) {
    std::vector<TileStage> stages;
    max_ops = std::max(1, std::min(max_ops, kMaxStageOps));
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
            const bool fits = blocks_only ? op.kind == OP_BLOCK : tileable(op);
            if (fits && __builtin_popcountll(high | need) <= H && st.ops.size() < size_t(max_ops)) {
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
    int pos[72], npos = 0;  // targets (k <= 5) and fixed bits (< 64)
    for (int j = 0; j < op.k; j++) {
        t.tb[j] = uint8_t(local(op.tq[j]));
        pos[npos++] = t.tb[j];
    }
    for (uint64_t fm = op.fixmask; fm; fm &= fm - 1) {
        const int b = __builtin_ctzll(fm);
        const int lb = local(b);
        const bool one = (op.fixval >> b) & 1ull;
        if (lb >= 0) {
            pos[npos++] = lb;
            if (one) t.lfixval |= 1u << lb;
        } else {
            t.omask |= 1ull << b;
            if (one) t.oval |= 1ull << b;
        }
    }
    std::sort(pos, pos + npos);
    t.npos = uint8_t(npos);
    for (int i = 0; i < npos && i < 16; i++) t.pos[i] = uint8_t(pos[i]);
    if (npos <= 4) {
        // Segment j of the expanded index holds the bits between the (j-1)-th and
        // j-th inserted zero; tuple bits land there shifted left by j.
        int lo = 0;
        for (int j = 0; j <= npos; j++) {
            const int hi = (j < npos) ? pos[j] : 32;
            const uint64_t below_hi = (hi >= 32) ? 0xffffffffull : ((1ull << hi) - 1ull);
            const uint64_t below_lo = (lo >= 32) ? 0xffffffffull : ((1ull << lo) - 1ull);
            t.seg[j] = uint32_t(below_hi & ~below_lo);
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
        t.bidx = uint32_t(op.block);
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
    // B[n][k] = M[n][k] (output n, input k), K-major in core matrices of 8 rows x 4 elements, 16 of
    // them along K per 8-row group: the shared-memory image the tensor-core descriptors read. The
    // high TF32 parts first, then the low parts.
    for (int n = 0; n < 64; n++)
        for (int k = 0; k < 64; k++) {
            const double v = M(n, k);
            const float h = tf32_rna(float(v));
            const int off = ((n >> 3) * 16 + (k >> 2)) * 32 + (n & 7) * 4 + (k & 3);
            out[off] = h;
            out[4096 + off] = tf32_rna(float(v - double(h)));
        }
}

// Whether a stage op can be a register-pass member (k <= 1 dense or monomial).
static bool passable(const OpDesc& op) {
    if (op.kind == OP_DENSE || op.kind == OP_DENSE_REAL) return op.k == 1;
    if (op.kind == OP_MONO || op.kind == OP_MONO_PF) return op.k <= 1;
    return false;
}

static TileOp pass_header(const int (&r)[kPassBits], int entries) {
    TileOp h;
    std::memset(&h, 0, sizeof(h));
    h.kind = OP_PASS;
    h.k = uint8_t(entries);
    h.npos = uint8_t(kPassBits);
    for (int i = 0; i < kPassBits; i++) h.pos[i] = uint8_t(r[i]);
    int lo = 0;
    for (int j = 0; j <= kPassBits; j++) {
        const int hi = (j < kPassBits) ? r[j] : 32;
        uint32_t m = 0;
        for (int b = lo; b < hi && b < 32; b++) m |= 1u << b;
        h.seg[j] = m;
        lo = hi + 1;
    }
    for (int j = 0; j < 16; j++) {  // register j's offset: the bits of j deposited on R
        uint32_t o = 0;
        for (int b = 0; b < kPassBits; b++)
            if (j >> b & 1) o |= 1u << r[b];
        (j < 8 ? h.off[j] : h.offsrc[j - 8]) = o;
    }
    return h;
}

// Fills the member fields of pass gate t (a tile op of kind dense / monomial, k <= 1) for register bits r.
static void pass_member(TileOp& t, const int (&r)[kPassBits]) {
    auto rix = [&](int lb) -> int {
        for (int i = 0; i < kPassBits; i++)
            if (r[i] == lb) return i;
        return -1;
    };
    PassMember& pm = t.pm;
    std::memset(&pm, 0, sizeof(pm));
    uint32_t fm = 0, fv = 0;
    for (int i = 0; i < t.npos; i++) {
        const int lb = t.pos[i];
        if (t.k == 1 && lb == t.tb[0]) continue;
        const bool one = (t.lfixval >> lb) & 1u;
        const int j = rix(lb);
        if (j >= 0) {
            fm |= 1u << j;
            if (one) fv |= 1u << j;
        } else {
            pm.om |= 1u << lb;
            if (one) pm.ov |= 1u << lb;
        }
    }
    pm.fmv = fm | (fv << 4);
    const uint32_t all = fm == 0 ? 1u : 0u, nocond = pm.om == 0 ? 1u : 0u;
    uint32_t vid, lane = 0;
    if (t.k == 0) {  // phase on the rows matching the controls
        vid = (PV_PHASE << 4) | (all << 1);
        pm.u[0] = float(t.m[0]);
        pm.u[1] = float(t.m[1]);
    } else {
        uint32_t code;
        if (t.kind == OP_DENSE) {
            code = PC_DENSE;
            for (int i = 0; i < 8; i++) pm.u[i] = float(t.m[i]);
        } else if (t.kind == OP_DENSE_REAL && !(all && nocond && !t.omask)) {
            code = PC_REAL;
            for (int i = 0; i < 4; i++) pm.u[i] = float(t.m[2 * i]);
        } else if (t.kind == OP_DENSE_REAL) {  // uncontrolled (H, RY): joins the dense groups
            code = PC_DENSE;
            for (int i = 0; i < 8; i++) pm.u[i] = float(t.m[i]);
        } else {
            // k = 1 monomial of a unitary: the rows exchanged (X, Y, CNOT) or kept (RZ), each with
            // a factor; the classifier drops untouched rows, so both rows are touched here.
            const bool swapped = t.offsrc[0] != 0;
            bool ones = true;
            for (int row = 0; row < 2; row++) {
                pm.u[2 * row] = float(t.m[2 * row]);
                pm.u[2 * row + 1] = float(t.m[2 * row + 1]);
                if (t.pf[row] != PF_ONE) ones = false;
            }
            code = swapped ? (ones ? PC_SWAP : PC_SWAPPH) : PC_DIAG2;
            if (code != PC_SWAP && all && nocond && !t.omask) {
                // uncontrolled phases (RZ, S, T, Y): the 2x2 matrix they are (dest row r takes factor_r
                // times source row perm[r]) joins the dense groups, which the copy-warp pass kernel runs
                const double f[4] = {t.m[0], t.m[1], t.m[2], t.m[3]};
                for (int i = 0; i < 16; i++) t.m[i] = 0.0;
                const int c0 = swapped ? 1 : 0;  // column of row 0's source
                t.m[2 * c0] = f[0];
                t.m[2 * c0 + 1] = f[1];
                t.m[4 + 2 * (1 - c0)] = f[2];
                t.m[4 + 2 * (1 - c0) + 1] = f[3];
                for (int i = 0; i < 8; i++) pm.u[i] = float(t.m[i]);
                code = PC_DENSE;
            }
        }
        const int lb = t.tb[0];
        if (lb < kLaneBits) {
            static const uint32_t lane_cat[5] = {PV_LDENSE, PV_LREAL, PV_LSWAP, PV_LSWAPPH, PV_LDIAG2};
            lane = uint32_t(lb);
            vid = (lane_cat[code] << 4) | (all << 1) | nocond;
        } else {
            const uint32_t J = uint32_t(rix(lb));
            const bool plain = all && nocond && !t.omask;
            if (code == PC_DENSE && plain)
                vid = (PV_DENSES << 4) | (1u << J);
            else if (code == PC_SWAP && fm && __builtin_popcount(fm) == 1 && fv == fm && nocond)
                vid = (PV_SWAPC << 4) | (J << 2) | uint32_t(__builtin_ctz(fm));  // CNOT inside the registers
            else {
                static const uint32_t reg_cat[5] = {PV_DENSE, PV_REAL, PV_SWAP, PV_SWAPPH, PV_DIAG2};
                vid = (reg_cat[code] << 4) | (J << 2) | (all << 1);
            }
        }
    }
    pm.ctl = vid | (lane << 10) | (t.omask ? (1u << 12) : 0u) | (pm.om ? (1u << 13) : 0u);
}

// Whether member entry e is a single dense gate on a register bit with no controls of any kind.
static bool plain_dense(const TileOp& e, int* J) {
    const uint32_t vid = e.pm.ctl & 255u;
    if ((vid >> 4) != PV_DENSES || __builtin_popcount(vid & 15u) != 1) return false;
    *J = __builtin_ctz(vid & 15u);
    return true;
}

// Emits a pass: header, then the members with runs of plain dense gates on distinct register bits
// merged into one multi-gate entry (bits in increasing order; such gates commute).
static void emit_pass(const int (&r)[kPassBits], const std::vector<TileOp>& tops, const std::vector<int>& members,
                      std::vector<TileOp>& prog) {
    const size_t head_at = prog.size();
    prog.push_back(pass_header(r, 0));
    for (size_t i = 0; i < members.size();) {
        int J;
        if (!plain_dense(tops[members[i]], &J)) {
            prog.push_back(tops[members[i++]]);
            continue;
        }
        uint32_t mask = 0;
        int byj[kPassBits] = {-1, -1, -1, -1};
        size_t k = i;
        while (k < members.size() && plain_dense(tops[members[k]], &J) && !(mask >> J & 1u)) {
            mask |= 1u << J;
            byj[J] = members[k];
            k++;
        }
        if (__builtin_popcount(mask) < 2) {
            prog.push_back(tops[members[i++]]);
            continue;
        }
        bool head = true;
        for (int j = 0; j < kPassBits; j++) {
            if (byj[j] < 0) continue;
            prog.push_back(tops[byj[j]]);
            if (head) prog.back().pm.ctl = (PV_DENSES << 4) | mask | (uint32_t(__builtin_popcount(mask) - 1) << 8);
            head = false;
        }
        i = k;
    }
    prog[head_at].k = uint8_t(prog.size() - head_at - 1);
}

static uint64_t op_qubits(const OpDesc& op) {
    uint64_t m = op.fixmask;
    for (int j = 0; j < op.k; j++) m |= 1ull << op.tq[j];
    return m;
}

// Schedules a run of pass gates (stage-local indices into `seg`) into passes: each pass picks the
// register bits that let the most gates run, a gate runs once every earlier gate sharing a qubit
// with it has run, and gates keep their relative order within a pass.
static void schedule_passes(const std::vector<OpDesc>& ops, const TileStage& st, const std::vector<int>& run,
                            std::vector<TileOp>& prog) {
    const int m = int(run.size());
    std::vector<TileOp> tops(m);
    std::vector<uint64_t> qm(m);
    std::vector<int> tgt(m);
    for (int i = 0; i < m; i++) {
        tops[i] = make_tile_op(ops[run[i]], st);
        qm[i] = op_qubits(ops[run[i]]);
        tgt[i] = (tops[i].k == 1) ? tops[i].tb[0] : -1;
    }
    std::vector<char> done(m, 0);
    int left = m;
    std::vector<int> upper;
    for (int b = kLaneBits; b < st.T; b++) upper.push_back(b);
    const int U = int(upper.size());
    // need[i]: the upper tile bit gate i's target must hold as a register bit (0: a lane bit or none)
    std::vector<uint32_t> need(m, 0u);
    for (int i = 0; i < m; i++)
        if (tgt[i] >= kLaneBits) need[i] = 1u << (tgt[i] - kLaneBits);
    // the gates a choice c of register bits (a mask over `upper`) lets run in this pass, over the
    // gates not yet scheduled (live, in order): branch-free, it runs for every choice of 4 bits
    std::vector<int> live;
    std::vector<uint32_t> lneed;
    std::vector<uint64_t> lqm;
    std::vector<uint64_t> cand;
    auto runnable = [&](uint32_t c) {
        uint64_t blocked = 0;
        int count = 0;
        const size_t nl = live.size();
        for (size_t i = 0; i < nl; i++) {
            const bool ok = !(lneed[i] & ~c) && !(lqm[i] & blocked);
            count += ok;
            blocked |= ok ? 0ull : lqm[i];
        }
        return count;
    };
    while (left > 0) {
        live.clear();
        lneed.clear();
        lqm.clear();
        for (int i = 0; i < m; i++)
            if (!done[i]) {
                live.push_back(i);
                lneed.push_back(need[i]);
                lqm.push_back(qm[i]);
            }
        // Exhaustive over the choices, in order of an upper bound (the gates whose targets a choice
        // holds, blocked or not); the first choice with the most runnable gates wins, as in a plain
        // scan over c, and no choice whose bound cannot beat (or tie at a smaller c) is evaluated.
        int cnt0 = 0, cnt[32] = {0};
        for (size_t i = 0; i < live.size(); i++) {
            if (lneed[i])
                cnt[__builtin_ctz(lneed[i])]++;
            else
                cnt0++;
        }
        cand.clear();
        for (uint32_t c = 0; c < (1u << U); c++) {
            if (__builtin_popcount(c) != kPassBits) continue;
            int ub = cnt0;
            for (uint32_t x = c; x; x &= x - 1) ub += cnt[__builtin_ctz(x)];
            cand.push_back((uint64_t(uint32_t(~ub)) << 32) | c);  // bound descending, then c ascending
        }
        std::sort(cand.begin(), cand.end());
        int best_count = -1;
        uint32_t best_c = 0;
        for (uint64_t key : cand) {
            const int ub = int(~uint32_t(key >> 32));
            const uint32_t c = uint32_t(key);
            if (ub < best_count || (ub == best_count && c > best_c)) {
                if (ub < best_count) break;
                continue;
            }
            const int count = runnable(c);
            if (count > best_count || (count == best_count && c < best_c)) {
                best_count = count;
                best_c = c;
            }
        }
        int best_r[kPassBits], ri = 0;
        for (int i = 0; i < U; i++)
            if (best_c >> i & 1u) best_r[ri++] = upper[i];
        std::vector<int> best_sel;
        {
            uint64_t blocked = 0;
            for (size_t i = 0; i < live.size(); i++) {
                if (!(lneed[i] & ~best_c) && !(lqm[i] & blocked))
                    best_sel.push_back(live[i]);
                else
                    blocked |= lqm[i];
            }
        }
        for (int i : best_sel) {
            pass_member(tops[i], best_r);
            done[i] = 1;
            left--;
        }
        emit_pass(best_r, tops, best_sel, prog);
    }
}

std::vector<TileOp> stage_program(const std::vector<OpDesc>& ops, const TileStage& st, bool passes) {
    std::vector<TileOp> prog;
    if (!passes || st.T < kPassMinT) {
        for (int idx : st.ops) prog.push_back(make_tile_op(ops[idx], st));
        return prog;
    }
    std::vector<int> run;
    for (int idx : st.ops) {
        const OpDesc& op = ops[idx];
        if (op.kind == OP_NOOP) continue;
        if (passable(op) && !(op.k == 0 && op.pf.size() && op.pf[0] == PF_SKIP)) {
            run.push_back(idx);
            continue;
        }
        if (!run.empty()) schedule_passes(ops, st, run, prog);
        run.clear();
        prog.push_back(make_tile_op(op, st));
    }
    if (!run.empty()) schedule_passes(ops, st, run, prog);
    return prog;
}

bool pass_only(const std::vector<TileOp>& prog) {
    if (prog.empty()) return false;
    for (size_t i = 0; i < prog.size(); i += size_t(prog[i].k) + 1) {
        if (prog[i].kind != OP_PASS) return false;
        for (size_t j = i + 1; j <= i + prog[i].k;) {  // the member variants the copy-warp kernel compiles
            const uint32_t ctl = prog[j].pm.ctl, cat = (ctl & 255u) >> 4, low = ctl & 15u;
            const bool common = cat == PV_DENSES || cat == PV_SWAP || cat == PV_SWAPC || cat == PV_LSWAP ||
                                cat == PV_PHASE || (cat == PV_LDENSE && low == 3u);
            if (!common) return false;
            j += ((ctl >> 8) & 3u) + 1;
        }
    }
    return true;
}

}  // namespace qs
