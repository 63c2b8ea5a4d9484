// CPU emulation of the tile kernel, linked against the engine's real host
// planner (qs_plan.cpp) and classifier (qs_classify.cpp). Used by
// tests/test_planner.py to check, without a GPU, that planned stages applied
// tile by tile give exactly the amplitudes of the gate-by-gate oracle.
//
// stdin (little-endian): n, T, L (int32); m (int32); per gate: k (int32),
// k targets (int32), 2^k x 2^k complex (2*4^k doubles); then 2^n complex
// amplitudes. stdout: 2^n complex amplitudes, then the number of stages.
#include <algorithm>
#include <cstdint>
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

// One k <= 1 member op of a register group applied to the 8 registers x.
void group_apply(const qs::TileOp& m, C (&x)[8]) {
    const int fm = m.gfin_mask, fv = m.gfin_val;
    auto mono_row = [&](int r, C src) -> C {
        return (m.pf[r] == 255) ? cmul(m.m[2 * r], m.m[2 * r + 1], src) : pf(src, m.pf[r]);
    };
    if (m.k == 0) {
        for (int r = 0; r < 8; r++)
            if ((r & fm) == fv && m.pf[0] != 4) x[r] = mono_row(0, x[r]);
        return;
    }
    const int j = m.gj;
    for (int a = 0; a < 8; a++) {
        if (a >> j & 1) continue;
        if ((a & fm) != fv) continue;
        const int b = a | (1 << j);
        if (m.kind == qs::OP_DENSE || m.kind == qs::OP_DENSE_REAL) {
            C y0 = cadd(cmul(m.m[0], m.m[1], x[a]), cmul(m.m[2], m.m[3], x[b]));
            C y1 = cadd(cmul(m.m[4], m.m[5], x[a]), cmul(m.m[6], m.m[7], x[b]));
            x[a] = y0;
            x[b] = y1;
        } else {
            const C s0 = m.offsrc[0] ? x[b] : x[a];
            const C s1 = m.offsrc[1] ? x[b] : x[a];
            if (m.pf[0] != 4) x[a] = mono_row(0, s0);
            if (m.pf[1] != 4) x[b] = mono_row(1, s1);
        }
    }
}

// Emulates k_tile<0> (the exact representation) for one stage.
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
            if (op.kind == qs::OP_GROUP) {
                for (uint32_t p = 0; p < ntup; p++) {
                    uint32_t b0 = p & op.seg[0];
                    for (int j = 1; j <= op.npos; j++) b0 |= (p << j) & op.seg[j];
                    C x[8];
                    for (int j = 0; j < 8; j++) x[j] = s[b0 + op.off[j]];
                    for (int mi = 1; mi <= op.k; mi++) {
                        const qs::TileOp& m = tops[oi + mi];
                        if ((base & m.omask) != m.oval) continue;
                        if ((b0 & m.gfout_mask) != m.gfout_val) continue;
                        group_apply(m, x);
                    }
                    for (int j = 0; j < 8; j++) s[b0 + op.off[j]] = x[j];
                }
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

int main() {
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
    const auto stages = qs::plan_tiles(ops, n, T, L, true);
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
        const std::vector<qs::TileOp> tops = qs::stage_program(ops, stage, true);
        run_stage(st, n, stage, tops);
    }
    fwrite(st.data(), sizeof(C), st.size(), stdout);
    int32_t ns = int32_t(stages.size());
    fwrite(&ns, sizeof(ns), 1, stdout);
    return 0;
}
