// qs_adjoint.cu — inner products, Pauli-sum expectation values and adjoint gradients.
//
// No counterpart in the reference (Quaru has no observables or gradients).
// The adjoint method follows Jones & Gacon, "Efficient calculation of
// gradients in classical simulations of variational quantum algorithms"
// (arXiv:2009.02823): psi = U_m...U_1 psi_0, lambda = H psi; walking the
// gates backwards, a rotation R_A(theta) = exp(-i theta A/2) contributes
// dE/dtheta = Im<lambda|A|psi> (both taken after the gate) and is then
// un-applied from both vectors, so no intermediate state is stored.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "qs_adjoint.h"
#include "qs_circuit.h"
#include "qs_device.cuh"
#include "qs_kernels.h"
#include "qs_reduce.cuh"

namespace qs {

constexpr int kAT = 256;

__device__ __forceinline__ double2 ld2(const double2* p, uint64_t i) { return p[i]; }
__device__ __forceinline__ double2 ld2(const float2* p, uint64_t i) {
    const float2 v = p[i];
    return make_double2(double(v.x), double(v.y));
}
__device__ __forceinline__ void st2(double2* p, uint64_t i, double2 v) { p[i] = v; }
__device__ __forceinline__ void st2(float2* p, uint64_t i, double2 v) { p[i] = make_float2(float(v.x), float(v.y)); }

static int grid_for_pairs(uint64_t work, int sms) {
    uint64_t b = (work + kAT - 1) / kAT;
    return int(std::max<uint64_t>(1, std::min<uint64_t>(b, uint64_t(sms) * 16)));
}

// ---------------------------------------------------------------- <a|b>
template <typename TA, typename TB>
__global__ void __launch_bounds__(kAT) k_inner(const TA* __restrict__ a, const TB* __restrict__ b, uint64_t N,
                                               double* __restrict__ partials) {
    double re = 0.0, im = 0.0;
    for (uint64_t i = uint64_t(blockIdx.x) * kAT + threadIdx.x; i < N; i += uint64_t(gridDim.x) * kAT) {
        const double2 x = ld2(a, i), y = ld2(b, i);
        re = fma(x.x, y.x, fma(x.y, y.y, re));
        im = fma(x.x, y.y, fma(-x.y, y.x, im));
    }
    rd_block_sum2<kAT>(re, im);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = re;
        partials[2 * blockIdx.x + 1] = im;
    }
}

__global__ void __launch_bounds__(kAT) k_pair_final(const double* __restrict__ partials, int nblocks,
                                                    double* __restrict__ out) {
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += kAT) {
        a += partials[2 * i];
        b += partials[2 * i + 1];
    }
    rd_block_sum2<kAT>(a, b);
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = b;
    }
}

// ---------------------------------------------------------------- H psi
struct PauliDev {
    double c;
    uint64_t x, z;
};

// out_i = sum_t c_t * i^{|x&z|} * (-1)^{|z & (i^x)|} * psi_{i^x}
template <typename T>
__global__ void __launch_bounds__(kAT) k_pauli_sum(const T* __restrict__ psi, T* __restrict__ out, uint64_t N,
                                                   const PauliDev* __restrict__ terms, int nt) {
    for (uint64_t i = uint64_t(blockIdx.x) * kAT + threadIdx.x; i < N; i += uint64_t(gridDim.x) * kAT) {
        double re = 0.0, im = 0.0;
        for (int t = 0; t < nt; t++) {
            const PauliDev p = terms[t];
            const uint64_t j = i ^ p.x;
            const double2 v = ld2(psi, j);
            double c = p.c;
            if (__popcll(p.z & j) & 1) c = -c;
            switch (__popcll(p.x & p.z) & 3) {
                case 0: re = fma(c, v.x, re); im = fma(c, v.y, im); break;
                case 1: re = fma(-c, v.y, re); im = fma(c, v.x, im); break;  // i * v
                case 2: re = fma(-c, v.x, re); im = fma(-c, v.y, im); break;
                default: re = fma(c, v.y, re); im = fma(-c, v.x, im); break;  // -i * v
            }
        }
        st2(out, i, make_double2(re, im));
    }
}

// ---------------------------------------------------------------- rotations
// R_A(theta) = cos(theta/2) I - i sin(theta/2) A on the pair (a, b) = (bit 0, bit 1).
template <int AXIS, typename R>
__device__ __forceinline__ void rot_pair(R c, R s, R& ax, R& ay, R& bx, R& by) {
    if (AXIS == QS_GATE_RY) {  // [[c, -s], [s, c]]
        const R nax = c * ax - s * bx, nay = c * ay - s * by;
        const R nbx = s * ax + c * bx, nby = s * ay + c * by;
        ax = nax; ay = nay; bx = nbx; by = nby;
    } else if (AXIS == QS_GATE_RZ) {  // diag(c - i s, c + i s)
        const R nax = c * ax + s * ay, nay = c * ay - s * ax;
        const R nbx = c * bx - s * by, nby = c * by + s * bx;
        ax = nax; ay = nay; bx = nbx; by = nby;
    } else {  // RX: [[c, -i s], [-i s, c]]
        const R nax = c * ax + s * by, nay = c * ay - s * bx;
        const R nbx = c * bx + s * ay, nby = c * by - s * ax;
        ax = nax; ay = nay; bx = nbx; by = nby;
    }
}

template <typename T, int AXIS>
__global__ void __launch_bounds__(kAT) k_rot(T* __restrict__ psi, uint64_t npairs, int q,
                                             const double2* __restrict__ cs, int slot, int inverse) {
    using R = decltype(psi[0].x);
    const double2 t = cs[slot];
    const R c = R(t.x), s = R(inverse ? -t.y : t.y);
    const uint64_t lo = (1ull << q) - 1ull, tb = 1ull << q;
    for (uint64_t p = uint64_t(blockIdx.x) * kAT + threadIdx.x; p < npairs; p += uint64_t(gridDim.x) * kAT) {
        const uint64_t i0 = ((p & ~lo) << 1) | (p & lo);
        T a = psi[i0], b = psi[i0 | tb];
        rot_pair<AXIS>(c, s, a.x, a.y, b.x, b.y);
        psi[i0] = a;
        psi[i0 | tb] = b;
    }
}

// Im<lambda|A|psi> over the pairs of qubit q, then psi, lambda <- R_A(-theta) psi, lambda.
template <int AXIS>
__device__ __forceinline__ double im_term(double2 l0, double2 l1, double2 a, double2 b) {
    if (AXIS == QS_GATE_RX) return (l0.x * b.y - l0.y * b.x) + (l1.x * a.y - l1.y * a.x);
    if (AXIS == QS_GATE_RY) return (l1.x * a.x + l1.y * a.y) - (l0.x * b.x + l0.y * b.y);
    return (l0.x * a.y - l0.y * a.x) - (l1.x * b.y - l1.y * b.x);
}

template <int AXIS>
__device__ __forceinline__ void im_term_acc(DfAcc& acc, float2 l0, float2 l1, float2 a, float2 b) {
    if (AXIS == QS_GATE_RX) {
        acc.add_prod(l0.x, b.y); acc.sub_prod(l0.y, b.x); acc.add_prod(l1.x, a.y); acc.sub_prod(l1.y, a.x);
    } else if (AXIS == QS_GATE_RY) {
        acc.add_prod(l1.x, a.x); acc.add_prod(l1.y, a.y); acc.sub_prod(l0.x, b.x); acc.sub_prod(l0.y, b.y);
    } else {
        acc.add_prod(l0.x, a.y); acc.sub_prod(l0.y, a.x); acc.sub_prod(l1.x, b.y); acc.add_prod(l1.y, b.x);
    }
}

template <typename T, int AXIS>
__global__ void __launch_bounds__(kAT) k_adj_rot(T* __restrict__ psi, T* __restrict__ lam, uint64_t npairs, int q,
                                                 const double2* __restrict__ cs, int slot,
                                                 double* __restrict__ partials) {
    using R = decltype(psi[0].x);
    const double2 t = cs[slot];
    const R c = R(t.x), s = R(-t.y);
    const uint64_t lo = (1ull << q) - 1ull, tb = 1ull << q;
    double acc = 0.0;
    DfAcc facc;
    for (uint64_t p = uint64_t(blockIdx.x) * kAT + threadIdx.x; p < npairs; p += uint64_t(gridDim.x) * kAT) {
        const uint64_t i0 = ((p & ~lo) << 1) | (p & lo);
        T a = psi[i0], b = psi[i0 | tb], l0 = lam[i0], l1 = lam[i0 | tb];
        if constexpr (sizeof(R) == 8) {
            acc += im_term<AXIS>(l0, l1, a, b);
        } else {
            im_term_acc<AXIS>(facc, l0, l1, a, b);
        }
        rot_pair<AXIS>(c, s, a.x, a.y, b.x, b.y);
        rot_pair<AXIS>(c, s, l0.x, l0.y, l1.x, l1.y);
        psi[i0] = a;
        psi[i0 | tb] = b;
        lam[i0] = l0;
        lam[i0 | tb] = l1;
    }
    if constexpr (sizeof(R) == 4) acc = __dadd_rn(df_f2d(facc.s), df_f2d(facc.c));
    double dummy = 0.0;
    rd_block_sum2<kAT>(acc, dummy);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// Block g sums partials[g * nblocks .. (g+1) * nblocks) into out[g].
__global__ void __launch_bounds__(kAT) k_grad_final(const double* __restrict__ partials, int nblocks,
                                                    double* __restrict__ out) {
    const double* p = partials + size_t(blockIdx.x) * nblocks;
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += kAT) a += p[i];
    rd_block_sum2<kAT>(a, b);
    if (threadIdx.x == 0) out[blockIdx.x] = a;
}

// ---------------------------------------------------------------- host side
static int fail(cudaError_t e, const char* what, std::string* msg) {
    if (msg) *msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return QS_OUT_OF_MEMORY;
    }
    return QS_CUDA_ERROR;
}

#define AJ_CHECK(call, what)                            \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) { rc = fail(e_, what, msg); goto done; } \
    } while (0)

int inner_product(const void* a, int pa, const void* b, int pb, int n, cudaStream_t s, int sms, double* scratch,
                  double* out2) {
    const uint64_t N = 1ull << n;
    const int grid = std::min(grid_for_pairs(N, sms), 4096);
    if (pa == QS_PREC_C128 && pb == QS_PREC_C128)
        k_inner<double2, double2><<<grid, kAT, 0, s>>>((const double2*)a, (const double2*)b, N, scratch);
    else if (pa == QS_PREC_C128)
        k_inner<double2, float2><<<grid, kAT, 0, s>>>((const double2*)a, (const float2*)b, N, scratch);
    else if (pb == QS_PREC_C128)
        k_inner<float2, double2><<<grid, kAT, 0, s>>>((const float2*)a, (const double2*)b, N, scratch);
    else
        k_inner<float2, float2><<<grid, kAT, 0, s>>>((const float2*)a, (const float2*)b, N, scratch);
    k_pair_final<<<1, kAT, 0, s>>>(scratch, grid, out2);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launches(2);
    return e == cudaSuccess ? QS_OK : QS_CUDA_ERROR;
}

static std::vector<PauliDev> pauli_table(const qs_pauli_term* terms, size_t nt) {
    std::vector<PauliDev> v(nt);
    for (size_t t = 0; t < nt; t++) v[t] = {terms[t].coeff, terms[t].x_mask, terms[t].z_mask};
    return v;
}

template <typename T>
static void launch_pauli_sum(const void* psi, void* out, int n, const PauliDev* dterms, int nt, cudaStream_t s,
                             int sms) {
    const uint64_t N = 1ull << n;
    k_pauli_sum<T><<<grid_for_pairs(N, sms), kAT, 0, s>>>((const T*)psi, (T*)out, N, dterms, nt);
    note_launches(1);
}

int expval_pauli(const void* psi, int prec, int n, const qs_pauli_term* terms, size_t nt, cudaStream_t s, int sms,
                 double* value, std::string* msg) {
    const size_t amp = prec == QS_PREC_C64 ? 8 : 16;
    const uint64_t N = 1ull << n;
    int rc = QS_OK;
    unsigned char* blob = nullptr;
    const size_t o_terms = 0, o_part = ((nt * sizeof(PauliDev) + 255) / 256) * 256, o_res = o_part + 4096 * 16,
                 o_lam = o_res + 256, total = o_lam + N * amp;
    std::vector<PauliDev> ht = pauli_table(terms, nt);
    double res[2] = {0, 0};
    AJ_CHECK(cudaMallocAsync((void**)&blob, total, s), "expval buffers");
    if (nt) AJ_CHECK(cudaMemcpyAsync(blob + o_terms, ht.data(), nt * sizeof(PauliDev), cudaMemcpyHostToDevice, s),
                     "terms upload");
    if (prec == QS_PREC_C64)
        launch_pauli_sum<float2>(psi, blob + o_lam, n, (const PauliDev*)(blob + o_terms), int(nt), s, sms);
    else
        launch_pauli_sum<double2>(psi, blob + o_lam, n, (const PauliDev*)(blob + o_terms), int(nt), s, sms);
    AJ_CHECK(cudaGetLastError(), "pauli sum");
    if (inner_product(psi, prec, blob + o_lam, prec, n, s, sms, (double*)(blob + o_part), (double*)(blob + o_res)))
        AJ_CHECK(cudaGetLastError(), "inner product");
    AJ_CHECK(cudaMemcpyAsync(res, blob + o_res, 16, cudaMemcpyDeviceToHost, s), "expval readback");
    AJ_CHECK(cudaStreamSynchronize(s), "expval sync");
    *value = res[0];
done:
    if (blob) cudaFreeAsync(blob, s);
    return rc;
}

template <typename T>
static void launch_rot(int kind, void* psi, int n, int q, const double2* cs, int slot, int inverse, cudaStream_t s,
                       int sms) {
    const uint64_t np = 1ull << (n - 1);
    const int grid = grid_for_pairs(np, sms);
    if (kind == QS_GATE_RX)
        k_rot<T, QS_GATE_RX><<<grid, kAT, 0, s>>>((T*)psi, np, q, cs, slot, inverse);
    else if (kind == QS_GATE_RY)
        k_rot<T, QS_GATE_RY><<<grid, kAT, 0, s>>>((T*)psi, np, q, cs, slot, inverse);
    else
        k_rot<T, QS_GATE_RZ><<<grid, kAT, 0, s>>>((T*)psi, np, q, cs, slot, inverse);
    note_launches(1);
}

template <typename T>
static void launch_adj_rot(int kind, void* psi, void* lam, int n, int q, const double2* cs, int slot,
                           double* partials, int grid, cudaStream_t s) {
    const uint64_t np = 1ull << (n - 1);
    if (kind == QS_GATE_RX)
        k_adj_rot<T, QS_GATE_RX><<<grid, kAT, 0, s>>>((T*)psi, (T*)lam, np, q, cs, slot, partials);
    else if (kind == QS_GATE_RY)
        k_adj_rot<T, QS_GATE_RY><<<grid, kAT, 0, s>>>((T*)psi, (T*)lam, np, q, cs, slot, partials);
    else
        k_adj_rot<T, QS_GATE_RZ><<<grid, kAT, 0, s>>>((T*)psi, (T*)lam, np, q, cs, slot, partials);
    note_launches(1);
}

int adjoint_gradient(void* state, int n, int prec, int arith, const qs_param_gate* gates, size_t m,
                     const double* params, size_t np, const qs_pauli_term* terms, size_t nt, cudaStream_t s, int sms,
                     double* energy, double* grad, size_t* err, std::string* msg) {
    // ---- validation (nothing is launched before every gate checks out)
    std::vector<OpDesc> fwd(m), inv(m);
    std::vector<int> rot_slot(m, -1);
    int nrot = 0;
    for (size_t g = 0; g < m; g++) {
        const qs_param_gate& G = gates[g];
        if (G.kind == QS_GATE_FIXED) {
            const size_t dim = G.k < 64 ? (size_t(1) << G.k) : 0;
            int rc = validate_gate(size_t(n), dim, dim, G.targets, G.k, err, msg);
            if (!rc && !G.matrix) rc = QS_INVALID_ARGUMENT, *msg = "matrix is null";
            if (rc) {
                if (err) err[2] = g;
                return rc;
            }
            classify_gate(G.matrix, G.k, G.targets, &fwd[g]);
            std::vector<double> h(2 * dim * dim);
            for (size_t r = 0; r < dim; r++)
                for (size_t c = 0; c < dim; c++) {  // conjugate transpose
                    h[2 * (r * dim + c)] = G.matrix[2 * (c * dim + r)];
                    h[2 * (r * dim + c) + 1] = -G.matrix[2 * (c * dim + r) + 1];
                }
            classify_gate(h.data(), G.k, G.targets, &inv[g]);
        } else if (G.kind == QS_GATE_RX || G.kind == QS_GATE_RY || G.kind == QS_GATE_RZ) {
            if (G.k != 1 || !G.targets) {
                if (err) err[0] = G.k, err[2] = g;
                *msg = "rotation gates take exactly one target";
                return QS_INVALID_ARITY;
            }
            if (G.targets[0] >= size_t(n)) {
                if (err) err[0] = G.targets[0], err[2] = g;
                *msg = "InvalidTarget(" + std::to_string(G.targets[0]) + ")";
                return QS_INVALID_TARGET;
            }
            if (G.param < 0 || size_t(G.param) >= np) {
                if (err) err[2] = g;
                *msg = "rotation parameter index out of range";
                return QS_INVALID_ARGUMENT;
            }
            rot_slot[g] = nrot++;
        } else {
            if (err) err[2] = g;
            *msg = "unknown gate kind";
            return QS_INVALID_ARGUMENT;
        }
    }
    // ---- tables
    std::vector<double2> cs(std::max<size_t>(m, 1));
    for (size_t g = 0; g < m; g++)
        if (rot_slot[g] >= 0) {
            const double th = params[gates[g].param];
            cs[g] = make_double2(std::cos(0.5 * th), std::sin(0.5 * th));
        }
    std::vector<PauliDev> ht = pauli_table(terms, nt);
    const size_t amp = prec == QS_PREC_C64 ? 8 : 16;
    const uint64_t N = 1ull << n;
    const int pgrid = grid_for_pairs(N >> 1, sms);
    auto al = [](size_t x) { return ((x + 255) / 256) * 256; };
    const size_t o_cs = 0, o_terms = o_cs + al(cs.size() * 16), o_part = o_terms + al(nt * sizeof(PauliDev) + 1),
                 o_res = o_part + al(size_t(std::max(nrot, 1)) * pgrid * 8 + 4096 * 16),
                 o_lam = o_res + al((2 + size_t(nrot)) * 8), o_save = o_lam + al(N * amp), total = o_save + N * amp;
    unsigned char* blob = nullptr;
    std::vector<double> res(2 + nrot, 0.0);
    int rc = QS_OK;
    AJ_CHECK(cudaMallocAsync((void**)&blob, total, s), "adjoint buffers");
    {
        const double2* dcs = (const double2*)(blob + o_cs);
        void* lam = blob + o_lam;
        double* part = (double*)(blob + o_part);
        double* dres = (double*)(blob + o_res);
        AJ_CHECK(cudaMemcpyAsync(blob + o_cs, cs.data(), cs.size() * 16, cudaMemcpyHostToDevice, s), "cs upload");
        if (nt)
            AJ_CHECK(cudaMemcpyAsync(blob + o_terms, ht.data(), nt * sizeof(PauliDev), cudaMemcpyHostToDevice, s),
                     "terms upload");
        AJ_CHECK(cudaMemcpyAsync(blob + o_save, state, N * amp, cudaMemcpyDeviceToDevice, s), "save state");
        // forward
        for (size_t g = 0; g < m; g++) {
            if (rot_slot[g] >= 0) {
                if (prec == QS_PREC_C64)
                    launch_rot<float2>(gates[g].kind, state, n, int(gates[g].targets[0]), dcs, int(g), 0, s, sms);
                else
                    launch_rot<double2>(gates[g].kind, state, n, int(gates[g].targets[0]), dcs, int(g), 0, s, sms);
                AJ_CHECK(cudaGetLastError(), "rotation");
            } else if ((rc = apply_op(state, n, prec, arith, fwd[g], s, sms, msg)) != QS_OK) {
                goto done;
            }
        }
        // lambda = H psi, E = Re<psi|lambda>
        if (prec == QS_PREC_C64)
            launch_pauli_sum<float2>(state, lam, n, (const PauliDev*)(blob + o_terms), int(nt), s, sms);
        else
            launch_pauli_sum<double2>(state, lam, n, (const PauliDev*)(blob + o_terms), int(nt), s, sms);
        AJ_CHECK(cudaGetLastError(), "pauli sum");
        if (inner_product(state, prec, lam, prec, n, s, sms, part + size_t(std::max(nrot, 1)) * pgrid, dres))
            AJ_CHECK(cudaGetLastError(), "energy");
        // reverse
        for (size_t gg = m; gg-- > 0;) {
            if (rot_slot[gg] >= 0) {
                double* p = part + size_t(rot_slot[gg]) * pgrid;
                if (prec == QS_PREC_C64)
                    launch_adj_rot<float2>(gates[gg].kind, state, lam, n, int(gates[gg].targets[0]), dcs, int(gg), p,
                                           pgrid, s);
                else
                    launch_adj_rot<double2>(gates[gg].kind, state, lam, n, int(gates[gg].targets[0]), dcs, int(gg), p,
                                            pgrid, s);
                AJ_CHECK(cudaGetLastError(), "adjoint rotation");
            } else {
                if ((rc = apply_op(state, n, prec, arith, inv[gg], s, sms, msg)) != QS_OK) goto done;
                if ((rc = apply_op(lam, n, prec, arith, inv[gg], s, sms, msg)) != QS_OK) goto done;
            }
        }
        if (nrot) {
            k_grad_final<<<nrot, kAT, 0, s>>>(part, pgrid, dres + 2);
            note_launches(1);
            AJ_CHECK(cudaGetLastError(), "gradient reduction");
        }
        AJ_CHECK(cudaMemcpyAsync(res.data(), dres, res.size() * 8, cudaMemcpyDeviceToHost, s), "readback");
        AJ_CHECK(cudaMemcpyAsync(state, blob + o_save, N * amp, cudaMemcpyDeviceToDevice, s), "restore state");
        AJ_CHECK(cudaStreamSynchronize(s), "adjoint sync");
        if (energy) *energy = res[0];
        if (grad) {
            for (size_t p = 0; p < np; p++) grad[p] = 0.0;
            for (size_t g = 0; g < m; g++)
                if (rot_slot[g] >= 0) grad[gates[g].param] += res[2 + rot_slot[g]];
        }
    }
done:
    if (blob) cudaFreeAsync(blob, s);
    return rc;
}

}  // namespace qs
