// qs_classify.cpp — host-side validation and structural classification of gates.
//
// Validation follows Register::try_apply_fast (src/register.rs:141-153) and
// get_duplicate (src/register.rs:418-429). Classification is new: the
// reference pushes every gate through a dense mat-vec (src/register.rs:183).
//
// Why dropping structure keeps results identical to the reference: the
// reference computes y_r = sum_c U[r,c] * x_c with the sum in ndarray's
// unrolled_dot order. A term with U[r,c] == 0 (both parts +-0) is +-0, and
// adding +-0 to a value leaves that value unchanged, so (up to the sign of a
// zero) y_r equals the same ordered sum over the non-zero columns only. An
// untouched row (U[r,r] == 1, rest of row and column zero) gives y_r == x_r.
// A monomial row gives y_r == U[r,p] * x_p, one rounded complex product.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <sstream>

#include "qs_internal.h"

namespace qs {

int validate_gate(size_t n, size_t rows, size_t cols, const size_t* targets, size_t k, size_t* err,
                  std::string* msg) {
    // Shape: the reference rejects (k, k) (src/register.rs:141-145); any other
    // shape that is not 2^k x 2^k panics in ndarray's dot. Both become
    // InvalidDimensions(rows, cols) here.
    bool bad = (rows == k && cols == k) || k >= 64 || rows != (size_t(1) << k) ||
               cols != (size_t(1) << k);
    if (bad) {
        if (err) {
            err[0] = rows;
            err[1] = cols;
        }
        if (msg) {
            std::ostringstream s;
            s << "InvalidDimensions(" << rows << ", " << cols << ") for " << k << " targets";
            *msg = s.str();
        }
        return QS_INVALID_DIMENSIONS;
    }
    if (k > 0 && targets == nullptr) {
        if (msg) *msg = "targets is null";
        return QS_INVALID_ARGUMENT;
    }
    // Duplicates: the smallest value that occurs twice (sorted scan).
    std::vector<size_t> sorted(targets, targets + k);
    std::sort(sorted.begin(), sorted.end());
    for (size_t i = 1; i < k; i++) {
        if (sorted[i] == sorted[i - 1]) {
            if (err) err[0] = sorted[i];
            if (msg) *msg = "InvalidTarget(" + std::to_string(sorted[i]) + "): duplicate target";
            return QS_INVALID_TARGET;
        }
    }
    // Range: first target in list order that is >= n.
    for (size_t j = 0; j < k; j++) {
        if (targets[j] >= n) {
            if (err) err[0] = targets[j];
            if (msg)
                *msg = "InvalidTarget(" + std::to_string(targets[j]) + "): register has " +
                       std::to_string(n) + " qubits";
            return QS_INVALID_TARGET;
        }
    }
    return QS_OK;
}

static inline bool is_zero(const double* z) { return z[0] == 0.0 && z[1] == 0.0; }
static inline bool is_one(const double* z) { return z[0] == 1.0 && z[1] == 0.0; }

// Place the bits of s at the positions set in `mask` (ascending), like PDEP.
static inline uint64_t deposit(uint64_t s, uint64_t mask) {
    uint64_t r = 0;
    for (int b = 0; b < 64 && mask; b++) {
        if (mask & 1ull) {
            r |= (s & 1ull) << b;
            s >>= 1;
        }
        mask >>= 1;
    }
    return r;
}

// Zero-filled scratch array of n entries: on the stack up to 64 (gates of up to 6 qubits, the
// common case), on the heap beyond.
template <typename T>
struct Scratch {
    T local[64];
    std::vector<T> heap;
    T* p;
    explicit Scratch(size_t n) {
        if (n <= 64) {
            p = local;
        } else {
            heap.resize(n);
            p = heap.data();
        }
        std::fill(p, p + n, T());
    }
    T& operator[](size_t i) { return p[i]; }
};

void classify_gate(const double* U, size_t k, const size_t* targets, OpDesc* op) {
    const uint64_t dim = 1ull << k;
    auto at = [&](uint64_t r, uint64_t c) { return U + 2 * (r * dim + c); };
    *op = OpDesc();
    op->orig_k = int(k);

    // 1. Rows the gate leaves untouched.
    Scratch<uint8_t> ident(dim);
    for (uint64_t r = 0; r < dim; r++) {
        if (!is_one(at(r, r))) continue;
        bool ok = true;
        for (uint64_t c = 0; c < dim && ok; c++)
            if (c != r && (!is_zero(at(r, c)) || !is_zero(at(c, r)))) ok = false;
        ident[r] = ok;
    }
    uint64_t common1 = dim - 1, common0 = dim - 1, touched = 0;
    for (uint64_t r = 0; r < dim; r++) {
        if (ident[r]) continue;
        touched++;
        common1 &= r;
        common0 &= ~r;
    }
    if (touched == 0) {
        op->kind = OP_NOOP;
        return;
    }
    // 2. Local bits shared by every touched row become fixed bits.
    const uint64_t fixed_local = (common1 | common0) & (dim - 1);
    const uint64_t free_local = (dim - 1) & ~fixed_local;
    int kk = 0;
    for (size_t j = 0; j < k; j++) {
        if (free_local >> j & 1ull) {
            op->tq[kk++] = int(targets[j]);
        } else {
            op->fixmask |= 1ull << targets[j];
            if (common1 >> j & 1ull) op->fixval |= 1ull << targets[j];
        }
    }
    op->k = kk;
    const uint64_t sdim = 1ull << kk;
    Scratch<uint64_t> full(sdim);
    for (uint64_t s = 0; s < sdim; s++) full[s] = deposit(s, free_local) | (common1 & fixed_local);

    // 3. Monomial test on the sub-matrix.
    bool mono = true;
    Scratch<uint32_t> perm(sdim);
    Scratch<uint32_t> colcount(sdim);
    for (uint64_t s = 0; s < sdim && mono; s++) {
        int nz = 0;
        for (uint64_t c = 0; c < sdim; c++) {
            if (!is_zero(at(full[s], full[c]))) {
                nz++;
                perm[s] = uint32_t(c);
                colcount[c]++;
            }
        }
        if (nz != 1) mono = false;
    }
    if (mono)
        for (uint64_t c = 0; c < sdim; c++)
            if (colcount[c] != 1) mono = false;

    if (mono) {
        op->perm.assign(perm.p, perm.p + sdim);
        op->phase.resize(2 * sdim);
        op->pf.resize(sdim);
        bool pf_all = true;
        uint64_t rows_touched = 0;
        for (uint64_t s = 0; s < sdim; s++) {
            const double* v = at(full[s], full[perm[s]]);
            op->phase[2 * s] = v[0];
            op->phase[2 * s + 1] = v[1];
            uint8_t cls;
            if (perm[s] == s && is_one(v))
                cls = PF_SKIP;
            else if (v[0] == 1.0 && v[1] == 0.0)
                cls = PF_ONE;
            else if (v[0] == -1.0 && v[1] == 0.0)
                cls = PF_NEG;
            else if (v[0] == 0.0 && v[1] == 1.0)
                cls = PF_I;
            else if (v[0] == 0.0 && v[1] == -1.0)
                cls = PF_NEG_I;
            else {
                cls = 255;
                pf_all = false;
            }
            op->pf[s] = cls;
            if (cls != PF_SKIP) rows_touched++;
        }
        op->kind = pf_all ? OP_MONO_PF : OP_MONO;
        op->touched_rows = rows_touched;
        return;
    }

    // 4. Dense sub-matrix.
    op->m.resize(2 * sdim * sdim);
    bool real = true;
    for (uint64_t r = 0; r < sdim; r++)
        for (uint64_t c = 0; c < sdim; c++) {
            const double* v = at(full[r], full[c]);
            op->m[2 * (r * sdim + c)] = v[0];
            op->m[2 * (r * sdim + c) + 1] = v[1];
            if (v[1] != 0.0) real = false;
        }
    op->kind = real ? OP_DENSE_REAL : OP_DENSE;
    op->touched_rows = sdim;
    // Exact order: ndarray's unrolled_dot keeps 8 partial sums (column mod 8)
    // when the row length is >= 8, and sums sequentially otherwise.
    op->lane.resize(sdim);
    for (uint64_t c = 0; c < sdim; c++) op->lane[c] = (dim >= 8) ? int8_t(full[c] & 7) : int8_t(-1);
}

double op_bytes(const OpDesc& op, int n, int amp_bytes) {
    if (op.kind == OP_NOOP) return 0.0;
    int nfixed = __builtin_popcountll(op.fixmask);
    double tuples = std::ldexp(1.0, n - op.k - nfixed);
    return 2.0 * tuples * double(op.touched_rows) * amp_bytes;
}

}  // namespace qs
