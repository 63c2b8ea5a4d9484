/*
 * quaru_oracle.c — CPU oracle for the Quaru register path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the GPU engine's results, never part
 * of the product. Plain-C restatement of DATX11-22/quaru src/register.rs (cited per
 * function), compiled with -O2 -ffp-contract=off so every floating-point
 * operation rounds exactly where the Rust code rounds (Rust never contracts
 * a*b+c into a fused multiply-add).
 *
 * Third-party arithmetic restated here (the crates are not vendored in the
 * reference and cannot be built in this container):
 *  - num-complex 0.4 (via num 0.4.0): Complex<f64> multiply is
 *    (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re); add is component-wise;
 *    Complex / f64 divides re and im separately; norm_sqr = re*re + im*im.
 *  - ndarray 0.15.6: Array2::dot(&Array1) -> general_mat_vec_mul_impl with
 *    alpha = 1, beta = 0 computes, per output row, row.dot(x) * alpha; 1-D
 *    dot of contiguous slices is numeric_util::unrolled_dot: eight running
 *    partial sums p0..p7 over strides of 8, then
 *    sum = (((0 + (p0+p4)) + (p1+p5)) + (p2+p6)) + (p3+p7), then a
 *    sequential tail of at most 7 terms. linalg::kron(a, b) writes a_ij * b
 *    block by block.
 *  - rand 0.8.5 thread_rng().gen::<f64>() is replaced by an injected draw.
 */
#include "quaru_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double re, im;
} cplx;

/* num-complex Mul for Complex<f64>. */
static inline cplx c_mul(cplx a, cplx b) {
    cplx r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}

/* num-complex Add for Complex<f64>. */
static inline cplx c_add(cplx a, cplx b) {
    cplx r;
    r.re = a.re + b.re;
    r.im = a.im + b.im;
    return r;
}

static const cplx C_ZERO = {0.0, 0.0};
static const cplx C_ONE = {1.0, 0.0};

/* ndarray 0.15.6 numeric_util::unrolled_dot for contiguous slices. */
static cplx unrolled_dot(const cplx* xs, const cplx* ys, size_t len) {
    cplx sum = C_ZERO;
    cplx p[8];
    for (int j = 0; j < 8; j++) p[j] = C_ZERO;
    size_t i = 0;
    while (len - i >= 8) {
        for (int j = 0; j < 8; j++) p[j] = c_add(p[j], c_mul(xs[i + j], ys[i + j]));
        i += 8;
    }
    sum = c_add(sum, c_add(p[0], p[4]));
    sum = c_add(sum, c_add(p[1], p[5]));
    sum = c_add(sum, c_add(p[2], p[6]));
    sum = c_add(sum, c_add(p[3], p[7]));
    for (size_t t = 0; i + t < len; t++) {
        if (t >= 7) break;
        sum = c_add(sum, c_mul(xs[i + t], ys[i + t]));
    }
    return sum;
}

/* ndarray general_mat_vec_mul_impl (alpha = 1, beta = 0, no BLAS):
 * y[r] = row_r.dot(x) * alpha. */
static void mat_vec(const cplx* a, size_t rows, size_t cols, const cplx* x, cplx* y) {
    for (size_t r = 0; r < rows; r++) y[r] = c_mul(unrolled_dot(a + r * cols, x, cols), C_ONE);
}

void orc_register_new(const uint8_t* bits, size_t n, double* state) {
    /* src/register.rs:41-56: fold(base=[1], |acc, q| kron(q, acc)) over
     * to_qbit_vector(bit) (src/math.rs:13-18). kron(q, acc)[i*len+j] = q_i * acc_j. */
    size_t len = (size_t)1 << n;
    cplx* out = (cplx*)state;
    cplx* tmp = (cplx*)malloc(len * sizeof(cplx));
    out[0] = C_ONE;
    size_t cur = 1;
    for (size_t q = 0; q < n; q++) {
        cplx v[2];
        if (bits[q]) {
            v[0] = C_ZERO;
            v[1] = C_ONE;
        } else {
            v[0] = C_ONE;
            v[1] = C_ZERO;
        }
        for (size_t i = 0; i < 2; i++)
            for (size_t j = 0; j < cur; j++) tmp[i * cur + j] = c_mul(v[i], out[j]);
        memcpy(out, tmp, 2 * cur * sizeof(cplx));
        cur *= 2;
    }
    free(tmp);
}

void orc_register_from_int(size_t n, size_t k, double* state) {
    /* src/math.rs:44-49: zeros, then state[k] = 1. */
    size_t len = (size_t)1 << n;
    memset(state, 0, len * sizeof(cplx));
    ((cplx*)state)[k] = C_ONE;
}

int orc_register_try_from_qubits(const double* qubits, size_t n, double* state, size_t* err) {
    const cplx* qb = (const cplx*)qubits;
    /* src/register.rs:83-89 with is_one (:107-115): total = -1 + sum norm_sqr, |total| < 1e-6. */
    for (size_t q = 0; q < n; q++) {
        double total = -1.0;
        for (int j = 0; j < 2; j++) total += qb[2 * q + j].re * qb[2 * q + j].re + qb[2 * q + j].im * qb[2 * q + j].im;
        if (!(fabs(total) < 0.000001)) {
            if (err) err[0] = q;
            return ORC_INVALID_QUBIT;
        }
    }
    /* src/register.rs:91-96: fold(base=[1], |acc, q| kron(q, acc)). */
    size_t len = (size_t)1 << n;
    cplx* out = (cplx*)state;
    cplx* tmp = (cplx*)malloc(len * sizeof(cplx));
    out[0] = C_ONE;
    size_t cur = 1;
    for (size_t q = 0; q < n; q++) {
        for (size_t i = 0; i < 2; i++)
            for (size_t j = 0; j < cur; j++) tmp[i * cur + j] = c_mul(qb[2 * q + i], out[j]);
        memcpy(out, tmp, 2 * cur * sizeof(cplx));
        cur *= 2;
    }
    free(tmp);
    return ORC_OK;
}

/* get_duplicate (src/register.rs:418-429): smallest value occurring twice. */
static int get_duplicate(const size_t* t, size_t k, size_t* dup) {
    size_t* c = (size_t*)malloc((k ? k : 1) * sizeof(size_t));
    memcpy(c, t, k * sizeof(size_t));
    /* insertion sort: k is small */
    for (size_t i = 1; i < k; i++) {
        size_t v = c[i], j = i;
        while (j > 0 && c[j - 1] > v) {
            c[j] = c[j - 1];
            j--;
        }
        c[j] = v;
    }
    int found = 0;
    for (size_t i = 1; i < k; i++)
        if (c[i] == c[i - 1]) {
            *dup = c[i];
            found = 1;
            break;
        }
    free(c);
    return found;
}

int orc_try_apply_fast(double* state, size_t n, const double* matrix, size_t rows, size_t cols,
                       const size_t* targets, size_t k, size_t* err) {
    /* src/register.rs:141-145. The reference's check fires only when the
     * shape equals (k, k); a shape that is not 2^k x 2^k makes ndarray's dot
     * panic later (Operation::new, src/operation.rs:60-70, rejects it up
     * front). Both cases are reported here as InvalidDimensions. */
    if ((rows == k && cols == k) || k >= 64 || rows != ((size_t)1 << k) || cols != ((size_t)1 << k)) {
        if (err) {
            err[0] = rows;
            err[1] = cols;
        }
        return ORC_INVALID_DIMENSIONS;
    }
    size_t dup;
    if (get_duplicate(targets, k, &dup)) { /* :146-148 */
        if (err) err[0] = dup;
        return ORC_INVALID_TARGET;
    }
    for (size_t j = 0; j < k; j++) /* :149-153 */
        if (targets[j] >= n) {
            if (err) err[0] = targets[j];
            return ORC_INVALID_TARGET;
        }

    size_t len = (size_t)1 << n, dim = (size_t)1 << k;
    cplx* st = (cplx*)state;
    cplx* new_state = (cplx*)malloc(len * sizeof(cplx)); /* :155 clone */
    memcpy(new_state, st, len * sizeof(cplx));
    size_t* perm = (size_t*)malloc(dim * sizeof(size_t));
    cplx* arr = (cplx*)malloc(dim * sizeof(cplx));
    cplx* res = (cplx*)malloc(dim * sizeof(cplx));
    size_t tmask = 0;
    for (size_t j = 0; j < k; j++) tmask |= (size_t)1 << targets[j];
    for (size_t index = 0; index < len; index++) { /* :156-160 */
        if (index & tmask) continue;
        for (size_t i = 0; i < dim; i++) { /* :163-176 */
            size_t p = index;
            for (size_t j = 0; j < k; j++)
                if ((i >> j) & 1) p |= (size_t)1 << targets[j];
            perm[i] = p;
        }
        for (size_t i = 0; i < dim; i++) arr[i] = st[perm[i]];  /* :178-181 */
        mat_vec((const cplx*)matrix, dim, dim, arr, res);        /* :183 */
        for (size_t i = 0; i < dim; i++) new_state[perm[i]] = res[i]; /* :185-187 */
    }
    memcpy(st, new_state, len * sizeof(cplx)); /* :189 */
    free(new_state);
    free(perm);
    free(arr);
    free(res);
    return ORC_OK;
}

int orc_try_apply_all(double* state, size_t n, const double* matrix, size_t rows, size_t cols,
                      size_t k, size_t* err) {
    /* src/register.rs:267-281 */
    if (k != 1) {
        if (err) err[0] = k;
        return ORC_INVALID_ARITY;
    }
    if (rows != 2 || cols != 2) {
        if (err) {
            err[0] = rows;
            err[1] = cols;
        }
        return ORC_INVALID_DIMENSIONS;
    }
    size_t len = (size_t)1 << n;
    const cplx* u = (const cplx*)matrix;
    /* fold(base=[[1]], |acc, _| kron(acc, U)): kron(acc, U)[(i*2+a), (j*2+b)] = acc_ij * U_ab */
    cplx* m = (cplx*)malloc(len * len * sizeof(cplx));
    cplx* t = (cplx*)malloc(len * len * sizeof(cplx));
    m[0] = C_ONE;
    size_t cur = 1;
    for (size_t q = 0; q < n; q++) {
        size_t nxt = cur * 2;
        for (size_t i = 0; i < cur; i++)
            for (size_t j = 0; j < cur; j++)
                for (size_t a = 0; a < 2; a++)
                    for (size_t b = 0; b < 2; b++)
                        t[(i * 2 + a) * nxt + (j * 2 + b)] = c_mul(m[i * cur + j], u[a * 2 + b]);
        cplx* s = m;
        m = t;
        t = s;
        cur = nxt;
    }
    cplx* out = (cplx*)malloc(len * sizeof(cplx));
    mat_vec(m, len, len, (const cplx*)state, out); /* :279 */
    memcpy(state, out, len * sizeof(cplx));
    free(out);
    free(m);
    free(t);
    return ORC_OK;
}

int orc_try_measure(double* state, size_t n, size_t target, double draw, int* outcome,
                    double* prob0, double* prob1, size_t* err) {
    if (target >= n) { /* src/register.rs:299-301 */
        if (err) err[0] = target;
        return ORC_INVALID_TARGET;
    }
    size_t len = (size_t)1 << n;
    cplx* st = (cplx*)state;
    double p1 = 0.0, p0 = 0.0;
    for (size_t i = 0; i < len; i++) { /* :306-315 sequential sum in index order */
        double p = st[i].re * st[i].re + st[i].im * st[i].im;
        if ((i >> target) & 1)
            p1 += p;
        else
            p0 += p;
    }
    int res = draw > p0;               /* :321 */
    double total = res ? p1 : p0;      /* :323 */
    double s = sqrt(total);
    for (size_t i = 0; i < len; i++) { /* :324-339 */
        if ((int)((i >> target) & 1) != res) {
            st[i] = C_ZERO;
        } else {
            st[i].re = st[i].re / s;
            st[i].im = st[i].im / s;
        }
    }
    if (outcome) *outcome = res;
    if (prob0) *prob0 = p0;
    if (prob1) *prob1 = p1;
    return ORC_OK;
}

void orc_probabilities(const double* state, size_t n, double* probs) {
    const cplx* st = (const cplx*)state;
    size_t len = (size_t)1 << n;
    for (size_t i = 0; i < len; i++) probs[i] = st[i].re * st[i].re + st[i].im * st[i].im;
}

int orc_apply_sequence(double* state, size_t n, size_t m, const size_t* ks, const size_t* toff,
                       const size_t* targets, const size_t* moff, const double* matrices,
                       size_t* err) {
    for (size_t g = 0; g < m; g++) {
        size_t dim = (size_t)1 << ks[g];
        int rc = orc_try_apply_fast(state, n, matrices + moff[g], dim, dim, targets + toff[g], ks[g], err);
        if (rc != ORC_OK) {
            if (err) err[2] = g;
            return rc;
        }
    }
    return ORC_OK;
}
