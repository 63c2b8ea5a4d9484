// CPU check of the dense-block fusion (quaru_gb300/csrc/qs_fuse.cpp): the fused
// blocks, applied one after another as dense matrices, must reproduce the
// gate-by-gate result. stdin: n, W (int32); m (int32); per gate k, targets,
// matrix (as tile_emulator); then 2^n amplitudes. stdout: 2^n amplitudes, then
// the number of blocks (int32).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../quaru_gb300/csrc/qs_fuse.h"

template <typename V>
static bool rd(V* v, size_t c) {
    return fread(v, sizeof(V), c, stdin) == c;
}

int main() {
    int32_t n, W, m;
    if (!rd(&n, 1) || !rd(&W, 1) || !rd(&m, 1)) return 2;
    std::vector<std::vector<size_t>> tg(m);
    std::vector<std::vector<double>> mats(m);
    std::vector<qs_gate> gates(m);
    for (int g = 0; g < m; g++) {
        int32_t k;
        if (!rd(&k, 1)) return 2;
        std::vector<int32_t> t(k);
        if (k && !rd(t.data(), k)) return 2;
        tg[g].assign(t.begin(), t.end());
        mats[g].resize(size_t(2) << (2 * k));
        if (!rd(mats[g].data(), mats[g].size())) return 2;
        gates[g] = qs_gate{size_t(k), tg[g].data(), mats[g].data()};
    }
    const size_t N = size_t(1) << n;
    std::vector<double> st(2 * N);
    if (!rd(st.data(), st.size())) return 2;
    auto blocks = qs::fuse_blocks(gates.data(), gates.size(), W);
    for (auto& b : blocks) {
        const int k = int(b.qubits.size());
        const size_t dim = size_t(1) << k;
        uint64_t mask = 0;
        for (int q : b.qubits) mask |= 1ull << q;
        std::vector<double> x(2 * dim), y(2 * dim);
        for (uint64_t base = 0; base < N; base++) {
            if (base & mask) continue;
            auto idx = [&](size_t i) {
                uint64_t r = base;
                for (int j = 0; j < k; j++)
                    if (i >> j & 1) r |= 1ull << b.qubits[j];
                return r;
            };
            for (size_t i = 0; i < dim; i++) {
                x[2 * i] = st[2 * idx(i)];
                x[2 * i + 1] = st[2 * idx(i) + 1];
            }
            for (size_t r = 0; r < dim; r++) {
                double re = 0, im = 0;
                for (size_t c = 0; c < dim; c++) {
                    const double ur = b.u[2 * (r * dim + c)], ui = b.u[2 * (r * dim + c) + 1];
                    re += ur * x[2 * c] - ui * x[2 * c + 1];
                    im += ur * x[2 * c + 1] + ui * x[2 * c];
                }
                y[2 * r] = re;
                y[2 * r + 1] = im;
            }
            for (size_t i = 0; i < dim; i++) {
                st[2 * idx(i)] = y[2 * i];
                st[2 * idx(i) + 1] = y[2 * i + 1];
            }
        }
    }
    fwrite(st.data(), sizeof(double), st.size(), stdout);
    int32_t nb = int32_t(blocks.size());
    fwrite(&nb, 4, 1, stdout);
    return 0;
}
