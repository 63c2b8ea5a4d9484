// CPU emulation of the tile kernel, linked against the engine's real host
// planner (qs_plan.cpp) and classifier (qs_classify.cpp). Used by
// tests/test_planner.py to check, without a GPU, that planned stages applied
// tile by tile give exactly the amplitudes of the gate-by-gate oracle.
//
// stdin (little-endian): n, T, L (int32); m (int32); per gate: k (int32),
// k targets (int32), 2^k x 2^k complex (2*4^k doubles); then 2^n complex
// amplitudes. argv: [mode ("pass" or anything else)] [largest gate count per stage].
// stdout: 2^n complex amplitudes, the number of stages, the number of register passes, the most
// gates any stage holds.
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../quaru_gb300/csrc/qs_internal.h"
#include "../../quaru_gb300/csrc/qs_tile.h"

namespace {

struct C {
    double re, im;
};

C cmul(double ur, double ui, C x) { return {ur * x.re - ui * x.im, ur * x.im + ui * x.re}; }
C cadd(C a, C b) { return {a.re + b.re, a.im + b.im}; }

C pf(C x, uint8_t c) {
    if (c == 1) return {-x.re, -x.im};
    if (c == 2) return {-x.im, x.re};
    if (c == 3) return {x.im, -x.re};
    return x;
}

uint32_t expand_local(uint32_t t, const uint8_t* pos, int npos) {
    for (int i = 0; i < npos; i++) {
        const uint32_t p = pos[i];
        t = ((t >> p) << (p + 1)) | (t & ((1u << p) - 1u));
    }
    return t;
}

uint64_t expand(uint64_t t, const std::vector<int>& pos) {
    for (int p : pos) t = ((t >> p) << (p + 1)) | (t & ((1ull << p) - 1ull));
    return t;
}

// One register pass (OP_PASS header at tops[oi]) over the tile s, decoding the kernel's variant ids
// (qs_tile.h) independently of the kernel: tuple p holds 16 registers at base(p) | off[j]; tile bits
// 0..3 are lane bits, so a gate on lane bit t pairs tuple p with tuple p ^ (1 << t). Arithmetic uses
// the entries' double coefficients (TileOp::m), in the layouts the variants read as floats.
void run_pass(std::vector<C>& s, uint32_t tsize, uint64_t tile_base, const std::vector<qs::TileOp>& tops,
              size_t oi) {
    const qs::TileOp& h = tops[oi];
    const uint32_t ntup = tsize >> 4;
    std::vector<uint32_t> base(ntup);
    std::vector<std::array<C, 16>> X(ntup);
    auto off = [&](int j) { return j < 8 ? h.off[j] : h.offsrc[j - 8]; };
    for (int j = 0; j < 16; j++) {  // the header's offsets must deposit j on the register bits
        uint32_t o = 0;
        for (int b = 0; b < 4; b++)
            if (j >> b & 1) o |= 1u << h.pos[b];
        if (off(j) != o) std::abort();
    }
    for (uint32_t p = 0; p < ntup; p++) {
        uint32_t b0 = p & h.seg[0];
        for (int j = 1; j <= 4; j++) b0 |= (p << j) & h.seg[j];
        base[p] = b0;
        for (int j = 0; j < 16; j++) X[p][j] = s[b0 | off(j)];
    }
    auto dense = [&](const double* m, C x0, C x1, int row) {
        return cadd(cmul(m[4 * row], m[4 * row + 1], x0), cmul(m[4 * row + 2], m[4 * row + 3], x1));
    };
    // register gate of `code` on bit J with coefficients m, where (a & fm) == fv
    auto reg_gate = [&](std::array<C, 16>& x, int code, int J, const double* m, int fm, int fv) {
        for (int a = 0; a < 16; a++) {
            if (a >> J & 1) continue;
            if ((a & fm) != fv) continue;
            const int b = a | (1 << J);
            const C x0 = x[a], x1 = x[b];
            if (code == qs::PC_DENSE) {
                x[a] = dense(m, x0, x1, 0);
                x[b] = dense(m, x0, x1, 1);
            } else if (code == qs::PC_REAL) {
                x[a] = cadd(cmul(m[0], 0, x0), cmul(m[2], 0, x1));
                x[b] = cadd(cmul(m[4], 0, x0), cmul(m[6], 0, x1));
            } else if (code == qs::PC_SWAP) {
                x[a] = x1;
                x[b] = x0;
            } else if (code == qs::PC_SWAPPH) {
                x[a] = cmul(m[0], m[1], x1);
                x[b] = cmul(m[2], m[3], x0);
            } else {
                x[a] = cmul(m[0], m[1], x0);
                x[b] = cmul(m[2], m[3], x1);
            }
        }
    };
    for (int mi = 1; mi <= h.k;) {
        const qs::TileOp& m = tops[oi + mi];
        const qs::PassMember& g = m.pm;
        const uint32_t vid = g.ctl & 255u, cat = vid >> 4, low = vid & 15u;
        const int first = mi;
        mi += int((g.ctl >> 8) & 3u) + 1;
        if ((g.ctl & (1u << 12)) && (tile_base & m.omask) != m.oval) continue;
        const bool cond = g.ctl & (1u << 13);
        int fm = g.fmv & 15, fv = (g.fmv >> 4) & 15;
        const bool lane = cat == qs::PV_LDENSE || cat == qs::PV_LSWAP || cat >= qs::PV_LREAL;
        if (lane) {
            const int code = cat == qs::PV_LDENSE ? qs::PC_DENSE : cat == qs::PV_LSWAP ? qs::PC_SWAP
                           : cat == qs::PV_LREAL ? qs::PC_REAL : cat == qs::PV_LSWAPPH ? qs::PC_SWAPPH : qs::PC_DIAG2;
            const int t = int((g.ctl >> 10) & 3u);
            if (low & 2u) fm = fv = 0;
            const bool nocond = low & 1u;
            auto Y = X;
            for (uint32_t p = 0; p < ntup; p++) {
                if (!nocond && (base[p] & g.om) != g.ov) continue;
                const uint32_t q = p ^ (1u << t);
                const int v = (base[p] >> t) & 1;
                for (int j = 0; j < 16; j++) {
                    if ((j & fm) != fv) continue;
                    std::array<C, 16> pair{};
                    pair[0] = v ? X[q][j] : X[p][j];
                    pair[1] = v ? X[p][j] : X[q][j];
                    reg_gate(pair, code, 0, m.m, 0, 0);
                    Y[p][j] = pair[v];
                }
            }
            X.swap(Y);
            continue;
        }
        for (uint32_t p = 0; p < ntup; p++) {
            auto& x = X[p];
            if (cat == qs::PV_DENSES) {  // no controls: every tuple
                int e = 0;
                for (int J = 0; J < 4; J++)
                    if (low >> J & 1u) reg_gate(x, qs::PC_DENSE, J, tops[oi + first + e++].m, 0, 0);
                continue;
            }
            if (cond && (base[p] & g.om) != g.ov) continue;
            const int J = int(low >> 2);
            const int lfm = (low & 2u) ? 0 : fm, lfv = (low & 2u) ? 0 : fv;
            switch (cat) {
                case qs::PV_SWAP: reg_gate(x, qs::PC_SWAP, J, m.m, lfm, lfv); break;
                case qs::PV_SWAPC: reg_gate(x, qs::PC_SWAP, J, m.m, 1 << (low & 3u), 1 << (low & 3u)); break;
                case qs::PV_PHASE:
                    for (int j = 0; j < 16; j++)
                        if ((j & lfm) == lfv) x[j] = cmul(m.m[0], m.m[1], x[j]);
                    break;
                case qs::PV_DENSE: reg_gate(x, qs::PC_DENSE, J, m.m, lfm, lfv); break;
                case qs::PV_REAL: reg_gate(x, qs::PC_REAL, J, m.m, lfm, lfv); break;
                case qs::PV_SWAPPH: reg_gate(x, qs::PC_SWAPPH, J, m.m, lfm, lfv); break;
                case qs::PV_DIAG2: reg_gate(x, qs::PC_DIAG2, J, m.m, lfm, lfv); break;
                default: std::abort();
            }
        }
    }
    for (uint32_t p = 0; p < ntup; p++)
        for (int j = 0; j < 16; j++) s[base[p] | off(j)] = X[p][j];
}

// Emulates k_tile for one stage (k_tile<0>'s arithmetic for the per-gate ops).
void run_stage(std::vector<C>& st, int n, const qs::TileStage& stage, const std::vector<qs::TileOp>& tops) {
    const int T = stage.T, L = stage.L, H = int(stage.high.size());
    std::vector<int> qpos;
    for (int q = 0; q < L; q++) qpos.push_back(q);
    for (int q : stage.high) qpos.push_back(q);
    std::sort(qpos.begin(), qpos.end());
    std::vector<uint64_t> rowoff(1u << H);
    for (uint32_t r = 0; r < (1u << H); r++) {
        uint64_t o = 0;
        for (int b = 0; b < H; b++)
            if (r >> b & 1) o |= 1ull << stage.high[b];
        rowoff[r] = o;
    }
    const uint32_t tsize = 1u << T, lmask = (1u << L) - 1u;
    std::vector<C> s(tsize);
    for (uint64_t tile = 0; tile < (1ull << (n - T)); tile++) {
        const uint64_t base = expand(tile, qpos);
        for (uint32_t i = 0; i < tsize; i++) s[i] = st[base + rowoff[i >> L] + (i & lmask)];
        for (size_t oi = 0; oi < tops.size(); oi++) {
            const qs::TileOp& op = tops[oi];
            if ((base & op.omask) != op.oval) continue;
            const uint32_t ntup = tsize >> op.npos;
            if (op.kind == qs::OP_PASS) {
                run_pass(s, tsize, base, tops, oi);
                oi += op.k;
                continue;
            }
            for (uint32_t p = 0; p < ntup; p++) {
                uint32_t i0;
                if (op.npos <= 4) {  // the kernel's segment-mask expansion
                    i0 = p & op.seg[0];
                    for (int j = 1; j <= op.npos; j++) i0 |= (p << j) & op.seg[j];
                } else {
                    i0 = expand_local(p, op.pos, op.npos);
                }
                i0 |= op.lfixval;
                if (op.kind == qs::OP_DENSE || op.kind == qs::OP_DENSE_REAL) {
                    const uint32_t tb = op.off[1];
                    C a = s[i0], b = s[i0 | tb];
                    C y0 = cadd(cmul(op.m[0], op.m[1], a), cmul(op.m[2], op.m[3], b));
                    C y1 = cadd(cmul(op.m[4], op.m[5], a), cmul(op.m[6], op.m[7], b));
                    s[i0] = y0;
                    s[i0 | tb] = y1;
                } else {
                    const int D = 1 << op.k;
                    C y[8];
                    for (int r = 0; r < D; r++)
                        if (op.pf[r] != 4) y[r] = s[i0 + op.offsrc[r]];
                    for (int r = 0; r < D; r++) {
                        if (op.pf[r] == 4) continue;
                        s[i0 + op.off[r]] = (op.pf[r] == 255) ? cmul(op.m[2 * r], op.m[2 * r + 1], y[r]) : pf(y[r], op.pf[r]);
                    }
                }
            }
        }
        for (uint32_t i = 0; i < tsize; i++) st[base + rowoff[i >> L] + (i & lmask)] = s[i];
    }
}

template <typename V>
bool rd(V* v, size_t count) {
    return fread(v, sizeof(V), count, stdin) == count;
}

}  // namespace

int main(int argc, char** argv) {
    // argv[1] == "pass": plan as for complex64 (commuting gates may reorder) with register passes;
    // otherwise the exact-order plan with one shared-memory pass per gate.
    const bool passes = argc > 1 && std::strcmp(argv[1], "pass") == 0;
    int32_t n, T, L, m;
    if (!rd(&n, 1) || !rd(&T, 1) || !rd(&L, 1) || !rd(&m, 1)) return 2;
    std::vector<qs::OpDesc> ops(m);
    std::vector<std::vector<double>> mats(m);
    std::vector<std::vector<size_t>> tg(m);
    for (int g = 0; g < m; g++) {
        int32_t k;
        if (!rd(&k, 1)) return 2;
        std::vector<int32_t> t(k);
        if (k && !rd(t.data(), k)) return 2;
        tg[g].assign(t.begin(), t.end());
        mats[g].resize(size_t(2) << (2 * k));
        if (!rd(mats[g].data(), mats[g].size())) return 2;
        qs::classify_gate(mats[g].data(), size_t(k), tg[g].data(), &ops[g]);
    }
    std::vector<C> st(size_t(1) << n);
    if (!rd(reinterpret_cast<double*>(st.data()), 2 * st.size())) return 2;
    const int max_ops = argc > 2 ? std::atoi(argv[2]) : qs::kMaxStageOps;
    const auto stages = qs::plan_tiles(ops, n, T, L, !passes, max_ops);
    int32_t widest = 0;
    for (const auto& stage : stages) widest = std::max<int32_t>(widest, int32_t(stage.ops.size()));
    int32_t npasses = 0;
    for (const auto& stage : stages) {
        if (!stage.tiled) {
            // single wide or dense gate: apply like the reference (sequential order suffices for
            // the gates the tests send down this path: dense k <= 2)
            const qs::OpDesc& op = ops[stage.single];
            const int g = stage.single;
            const int k = int(tg[g].size());
            const size_t dim = size_t(1) << k;
            std::vector<C> out = st;
            uint64_t tmask = 0;
            for (size_t t : tg[g]) tmask |= 1ull << t;
            for (uint64_t idx = 0; idx < st.size(); idx++) {
                if (idx & tmask) continue;
                for (size_t r = 0; r < dim; r++) {
                    C acc = {0.0, 0.0};
                    for (size_t c = 0; c < dim; c++) {
                        uint64_t p = idx;
                        for (int j = 0; j < k; j++)
                            if (c >> j & 1) p |= 1ull << tg[g][j];
                        const double* u = &mats[g][2 * (r * dim + c)];
                        acc = cadd(acc, cmul(u[0], u[1], st[p]));
                    }
                    uint64_t p = idx;
                    for (int j = 0; j < k; j++)
                        if (r >> j & 1) p |= 1ull << tg[g][j];
                    out[p] = acc;
                }
            }
            (void)op;
            st.swap(out);
            continue;
        }
        const std::vector<qs::TileOp> tops = qs::stage_program(ops, stage, passes);
        for (const auto& t : tops) npasses += t.kind == qs::OP_PASS;
        run_stage(st, n, stage, tops);
    }
    fwrite(st.data(), sizeof(C), st.size(), stdout);
    int32_t ns = int32_t(stages.size());
    fwrite(&ns, sizeof(ns), 1, stdout);
    fwrite(&npasses, sizeof(npasses), 1, stdout);
    fwrite(&widest, sizeof(widest), 1, stdout);
    return 0;
}
