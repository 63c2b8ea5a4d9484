// qs_batch.cu — forward + adjoint gradients for a batch of circuits in one persistent launch.
//
// No counterpart in the reference. Work item = (circuit c, step s, chunk j):
// steps 0..G-1 apply the circuit's gates, step G forms lambda = H psi and the
// energy partial sums, steps G+1..2G walk the gates backwards (adjoint
// rotations with per-chunk partial derivatives; fixed gates un-applied from
// psi and lambda). Items are ordered by step round across circuits, so an item
// only ever waits for items handed out before it; those are held by running
// CTAs, which makes the schedule deadlock-free without any co-residency
// assumption. Every wait is bounded: when it gives up it raises an error flag
// that makes every CTA return, and the host reports QS_TIMEOUT.
//
// The whole pass (parameter upload, state reset, persistent kernel, partial
// reduction, result download) is captured once in a CUDA graph; a run writes
// new parameters into pinned memory and replays it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "qs_device.cuh"
#include "qs_kernels.h"
#include "qs_reduce.cuh"

namespace qs {
namespace {

constexpr int kBT = 256;
constexpr int kFix1 = 16;  // fixed dense 1-qubit gate
constexpr int kCnot = 17;  // CNOT (q0 = target, q1 = control)
constexpr long long kWaitCycles = 20000000000LL;  // ~10 s at 2 GHz: dependency waits give up after this

struct BCirc {
    unsigned long long psi, lam;
    int n, ngates, gate_off, nterms, term_off, nsteps, counter_off, part_off, nch_log, nrot;
};

struct BGate {
    int kind, q0, q1, cs;
    int rslot, pad0, pad1, pad2;
    double m[8];  // kFix1: the 2x2 matrix; its adjoint is formed on the fly
};

struct BPauli {
    double c;
    unsigned long long x, z;
};

template <typename T>
struct St;
template <>
struct St<double2> {
    static __device__ __forceinline__ double2 ld(const double2* p, uint64_t i) { return __ldcg(p + i); }
    static __device__ __forceinline__ void st(double2* p, uint64_t i, double2 v) { __stcg(p + i, v); }
    static __device__ __forceinline__ double2 d(double2 v) { return v; }
    static __device__ __forceinline__ double2 from(double2 v) { return v; }
};
template <>
struct St<float2> {
    static __device__ __forceinline__ float2 ld(const float2* p, uint64_t i) { return __ldcg(p + i); }
    static __device__ __forceinline__ void st(float2* p, uint64_t i, float2 v) { __stcg(p + i, v); }
    static __device__ __forceinline__ double2 d(float2 v) { return make_double2(v.x, v.y); }
    static __device__ __forceinline__ float2 from(double2 v) { return make_float2(float(v.x), float(v.y)); }
};

// R_A(theta) on a pair, with (c, s) = (cos, sin) of theta/2 (s negated for the inverse).
template <typename R>
__device__ __forceinline__ void rot(int kind, R c, R s, R& ax, R& ay, R& bx, R& by) {
    if (kind == QS_GATE_RY) {
        const R nax = c * ax - s * bx, nay = c * ay - s * by, nbx = s * ax + c * bx, nby = s * ay + c * by;
        ax = nax; ay = nay; bx = nbx; by = nby;
    } else if (kind == QS_GATE_RZ) {
        const R nax = c * ax + s * ay, nay = c * ay - s * ax, nbx = c * bx - s * by, nby = c * by + s * bx;
        ax = nax; ay = nay; bx = nbx; by = nby;
    } else {
        const R nax = c * ax + s * by, nay = c * ay - s * bx, nbx = c * bx + s * ay, nby = c * by - s * ax;
        ax = nax; ay = nay; bx = nbx; by = nby;
    }
}

// y = M x for a 2x2 complex matrix (adjoint: M^H).
__device__ __forceinline__ void mat2(const double* m, bool adj, double2& a, double2& b) {
    double u[8];
#pragma unroll
    for (int i = 0; i < 8; i++) u[i] = m[i];
    if (adj) {  // (M^H)_{rc} = conj(M_{cr})
        const double t[8] = {u[0], -u[1], u[4], -u[5], u[2], -u[3], u[6], -u[7]};
#pragma unroll
        for (int i = 0; i < 8; i++) u[i] = t[i];
    }
    const double2 x = a, y = b;
    a = make_double2(u[0] * x.x - u[1] * x.y + u[2] * y.x - u[3] * y.y, u[0] * x.y + u[1] * x.x + u[2] * y.y + u[3] * y.x);
    b = make_double2(u[4] * x.x - u[5] * x.y + u[6] * y.x - u[7] * y.y, u[4] * x.y + u[5] * x.x + u[6] * y.y + u[7] * y.x);
}

__device__ __forceinline__ double im_lam_a_psi(int kind, double2 l0, double2 l1, double2 a, double2 b) {
    if (kind == QS_GATE_RX) return (l0.x * b.y - l0.y * b.x) + (l1.x * a.y - l1.y * a.x);
    if (kind == QS_GATE_RY) return (l1.x * a.x + l1.y * a.y) - (l0.x * b.x + l0.y * b.y);
    return (l0.x * a.y - l0.y * a.x) - (l1.x * b.y - l1.y * b.x);
}

template <typename T>
__global__ void __launch_bounds__(kBT) k_batch_reset(const BCirc* __restrict__ circs) {
    const BCirc C = circs[blockIdx.y];
    T* psi = reinterpret_cast<T*>(C.psi);
    const uint64_t N = 1ull << C.n;
    for (uint64_t i = uint64_t(blockIdx.x) * kBT + threadIdx.x; i < N; i += uint64_t(gridDim.x) * kBT)
        St<T>::st(psi, i, St<T>::from(make_double2(i == 0 ? 1.0 : 0.0, 0.0)));
}

template <typename T>
__global__ void __launch_bounds__(kBT) k_batch(const BCirc* __restrict__ circs, const BGate* __restrict__ gates,
                                               const BPauli* __restrict__ terms, const double2* __restrict__ cs,
                                               const uint32_t* __restrict__ seg_first, const int4* __restrict__ segs,
                                               int nsegs, uint32_t nitems, int chunk_log,
                                               unsigned int* __restrict__ counters, double* __restrict__ partials,
                                               unsigned int* __restrict__ ticket, int* __restrict__ err) {
    using R = decltype(T().x);
    __shared__ uint32_t s_item;
    __shared__ int s_seg, s_stop;
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(ticket, 1u);
            s_stop = (s_item >= nitems) || (*reinterpret_cast<volatile int*>(err) != 0);
            if (!s_stop) {  // segment holding this item: last seg_first <= item
                int lo = 0, hi = nsegs - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (seg_first[mid] <= s_item) lo = mid; else hi = mid - 1;
                }
                s_seg = lo;
            }
        }
        __syncthreads();
        if (s_stop) return;
        const int4 sg = segs[s_seg];
        const int c = sg.x, s = sg.y, nch = sg.z;
        const uint32_t j = s_item - seg_first[s_seg];
        const BCirc C = circs[c];
        if (s > 0 && threadIdx.x == 0) {  // every chunk of the previous step must be done
            volatile unsigned int* prev = counters + C.counter_off + s - 1;
            const long long t0 = clock64();
            while (*prev < unsigned(nch)) {
                __nanosleep(100);
                if (clock64() - t0 > kWaitCycles) {
                    atomicExch(err, 1);
                    s_stop = 1;
                    break;
                }
            }
            __threadfence();
        }
        __syncthreads();
        if (s_stop) return;
        T* psi = reinterpret_cast<T*>(C.psi);
        T* lam = reinterpret_cast<T*>(C.lam);
        const int G = C.ngates;
        const int cl = min(chunk_log, C.n - 1);
        const uint64_t pairs = 1ull << (C.n - 1);
        const uint64_t p0 = uint64_t(j) << cl;
        const uint64_t p1 = (p0 + (1ull << cl) < pairs) ? p0 + (1ull << cl) : pairs;
        if (s < G || s > G) {
            const bool fwd = s < G;
            const BGate g = gates[C.gate_off + (fwd ? s : 2 * G - s)];
            const uint64_t lo = (1ull << g.q0) - 1ull, tb = 1ull << g.q0;
            R cc = 0, ss = 0;
            if (g.kind <= QS_GATE_RZ) {
                const double2 t = cs[g.cs];
                cc = R(t.x);
                ss = R(fwd ? t.y : -t.y);
            }
            double acc = 0.0;
            for (uint64_t p = p0 + threadIdx.x; p < p1; p += kBT) {
                const uint64_t i0 = ((p & ~lo) << 1) | (p & lo), i1 = i0 | tb;
                if (g.kind == kCnot) {
                    if (!((i0 >> g.q1) & 1ull)) continue;
                    const T a = St<T>::ld(psi, i0), b = St<T>::ld(psi, i1);
                    St<T>::st(psi, i0, b);
                    St<T>::st(psi, i1, a);
                    if (!fwd) {
                        const T la = St<T>::ld(lam, i0), lb = St<T>::ld(lam, i1);
                        St<T>::st(lam, i0, lb);
                        St<T>::st(lam, i1, la);
                    }
                } else if (g.kind == kFix1) {
                    double2 a = St<T>::d(St<T>::ld(psi, i0)), b = St<T>::d(St<T>::ld(psi, i1));
                    mat2(g.m, !fwd, a, b);
                    St<T>::st(psi, i0, St<T>::from(a));
                    St<T>::st(psi, i1, St<T>::from(b));
                    if (!fwd) {
                        double2 la = St<T>::d(St<T>::ld(lam, i0)), lb = St<T>::d(St<T>::ld(lam, i1));
                        mat2(g.m, true, la, lb);
                        St<T>::st(lam, i0, St<T>::from(la));
                        St<T>::st(lam, i1, St<T>::from(lb));
                    }
                } else {
                    T a = St<T>::ld(psi, i0), b = St<T>::ld(psi, i1);
                    if (!fwd) {
                        T l0 = St<T>::ld(lam, i0), l1 = St<T>::ld(lam, i1);
                        acc += im_lam_a_psi(g.kind, St<T>::d(l0), St<T>::d(l1), St<T>::d(a), St<T>::d(b));
                        rot<R>(g.kind, cc, ss, l0.x, l0.y, l1.x, l1.y);
                        St<T>::st(lam, i0, l0);
                        St<T>::st(lam, i1, l1);
                    }
                    rot<R>(g.kind, cc, ss, a.x, a.y, b.x, b.y);
                    St<T>::st(psi, i0, a);
                    St<T>::st(psi, i1, b);
                }
            }
            if (!fwd && g.kind <= QS_GATE_RZ) {
                double dummy = 0.0;
                rd_block_sum2<kBT>(acc, dummy);
                if (threadIdx.x == 0) partials[C.part_off + (1 + g.rslot) * nch + j] = acc;
            }
        } else {  // lambda = H psi over amplitudes [2 p0, 2 p1), energy partial
            double e = 0.0;
            for (uint64_t i = 2 * p0 + threadIdx.x; i < 2 * p1; i += kBT) {
                double re = 0.0, im = 0.0;
                for (int t = 0; t < C.nterms; t++) {
                    const BPauli P = terms[C.term_off + t];
                    const uint64_t k = i ^ P.x;
                    const double2 v = St<T>::d(St<T>::ld(psi, k));
                    double cf = P.c;
                    if (__popcll(P.z & k) & 1) cf = -cf;
                    switch (__popcll(P.x & P.z) & 3) {
                        case 0: re = fma(cf, v.x, re); im = fma(cf, v.y, im); break;
                        case 1: re = fma(-cf, v.y, re); im = fma(cf, v.x, im); break;
                        case 2: re = fma(-cf, v.x, re); im = fma(-cf, v.y, im); break;
                        default: re = fma(cf, v.y, re); im = fma(-cf, v.x, im); break;
                    }
                }
                St<T>::st(lam, i, St<T>::from(make_double2(re, im)));
                const double2 p = St<T>::d(St<T>::ld(psi, i));
                e = fma(p.x, re, fma(p.y, im, e));
            }
            double dummy = 0.0;
            rd_block_sum2<kBT>(e, dummy);
            if (threadIdx.x == 0) partials[C.part_off + j] = e;
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd(counters + C.counter_off + s, 1u);
    }
}

// res[r] = sum of partials[rtab[r].x .. + rtab[r].y), in a fixed order.
__global__ void __launch_bounds__(kBT) k_batch_reduce(const double* __restrict__ partials, const int2* __restrict__ rtab,
                                                      int nres, double* __restrict__ res) {
    for (int r = blockIdx.x; r < nres; r += gridDim.x) {
        const int2 t = rtab[r];
        double a = 0.0, b = 0.0;
        for (int i = threadIdx.x; i < t.y; i += kBT) a += partials[t.x + i];
        rd_block_sum2<kBT>(a, b);
        if (threadIdx.x == 0) res[r] = a;
    }
}

}  // namespace
}  // namespace qs

struct qs_batch {
    int prec = QS_PREC_C128, count = 0, sms = 1, chunk_log = 12, ctas = 2;
    cudaStream_t stream = nullptr;
    unsigned char* arena = nullptr;
    size_t arena_bytes = 0;
    qs::BCirc* dcirc = nullptr;
    qs::BGate* dgates = nullptr;
    qs::BPauli* dterms = nullptr;
    double2* dcs = nullptr;
    uint32_t* dseg_first = nullptr;
    int4* dsegs = nullptr;
    unsigned int* dcounters = nullptr;
    double* dpart = nullptr;
    double* dres = nullptr;
    int2* drtab = nullptr;
    int* derr = nullptr;
    unsigned int* dticket = nullptr;
    double2* hcs = nullptr;   // pinned: (cos, sin) of theta/2 per rotation
    double* hres = nullptr;   // pinned: results
    int* herr = nullptr;      // pinned
    int nsegs = 0, nres = 0, ncs = 0, ncounters = 0;
    uint32_t nitems = 0;
    size_t total_params = 0;
    std::vector<size_t> param_off;
    std::vector<int> cs_param;       // parameter index (global) of each rotation
    std::vector<int> res_circ_base;  // first result of each circuit
    std::vector<std::vector<int>> rot_param;  // per circuit: parameter index (local) of rotation slot r
    std::vector<qs::BCirc> hcirc;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

using namespace qs;

thread_local std::string g_batch_err;

bool is_cnot(const qs_param_gate& g) {
    if (g.k != 2 || !g.matrix) return false;
    static const double c[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0};
    for (int r = 0; r < 4; r++)
        for (int cc = 0; cc < 4; cc++)
            if (g.matrix[2 * (r * 4 + cc)] != c[r * 4 + cc] || g.matrix[2 * (r * 4 + cc) + 1] != 0.0) return false;
    return true;
}

size_t al(size_t x) { return (x + 255) / 256 * 256; }

void release(qs_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->arena) cudaFree(b->arena);
    if (b->hcs) cudaFreeHost(b->hcs);
    if (b->hres) cudaFreeHost(b->hres);
    if (b->herr) cudaFreeHost(b->herr);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Work-item schedule for a chunk size: segments (circuit, step, chunks) ordered by step round.
void build_schedule(qs_batch* b, int chunk_log, std::vector<uint32_t>* first, std::vector<int4>* segs,
                    uint64_t* nitems) {
    first->clear();
    segs->clear();
    int maxsteps = 0;
    for (const auto& c : b->hcirc) maxsteps = std::max(maxsteps, c.nsteps);
    uint64_t item = 0;
    for (int s = 0; s < maxsteps; s++)
        for (int c = 0; c < b->count; c++) {
            const BCirc& C = b->hcirc[c];
            if (s >= C.nsteps) continue;
            const int cl = std::min(chunk_log, C.n - 1);
            const int nch = 1 << (C.n - 1 - cl);
            first->push_back(uint32_t(item));
            segs->push_back(make_int4(c, s, nch, 0));
            item += uint64_t(nch);
        }
    *nitems = item;
}

cudaError_t capture(qs_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec), b->exec = nullptr;
    if (b->graph) cudaGraphDestroy(b->graph), b->graph = nullptr;
    cudaStream_t s = b->stream;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    if (b->ncs) cudaMemcpyAsync(b->dcs, b->hcs, sizeof(double2) * b->ncs, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(b->dcounters, 0, sizeof(unsigned int) * b->ncounters, s);
    cudaMemsetAsync(b->dticket, 0, sizeof(unsigned int), s);
    cudaMemsetAsync(b->derr, 0, sizeof(int), s);
    const dim3 rg(uint32_t(b->sms * 2), uint32_t(b->count));
    if (b->prec == QS_PREC_C64) {
        k_batch_reset<float2><<<rg, kBT, 0, s>>>(b->dcirc);
        k_batch<float2><<<b->sms * b->ctas, kBT, 0, s>>>(b->dcirc, b->dgates, b->dterms, b->dcs, b->dseg_first,
                                                         b->dsegs, b->nsegs, b->nitems, b->chunk_log, b->dcounters,
                                                         b->dpart, b->dticket, b->derr);
    } else {
        k_batch_reset<double2><<<rg, kBT, 0, s>>>(b->dcirc);
        k_batch<double2><<<b->sms * b->ctas, kBT, 0, s>>>(b->dcirc, b->dgates, b->dterms, b->dcs, b->dseg_first,
                                                          b->dsegs, b->nsegs, b->nitems, b->chunk_log, b->dcounters,
                                                          b->dpart, b->dticket, b->derr);
    }
    k_batch_reduce<<<std::min(b->nres, b->sms * 8), kBT, 0, s>>>(b->dpart, b->drtab, b->nres, b->dres);
    cudaMemcpyAsync(b->hres, b->dres, sizeof(double) * b->nres, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(b->herr, b->derr, sizeof(int), cudaMemcpyDeviceToHost, s);
    e = cudaStreamEndCapture(s, &b->graph);
    if (e != cudaSuccess) return e;
    return cudaGraphInstantiate(&b->exec, b->graph, 0);
}

// Upload a schedule for chunk_log into the arena's schedule area (sized for the smallest chunk).
cudaError_t upload_schedule(qs_batch* b, int chunk_log) {
    std::vector<uint32_t> first;
    std::vector<int4> segs;
    uint64_t n = 0;
    build_schedule(b, chunk_log, &first, &segs, &n);
    b->nsegs = int(segs.size());
    b->nitems = uint32_t(n);
    b->chunk_log = chunk_log;
    cudaError_t e = cudaMemcpy(b->dseg_first, first.data(), first.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->dsegs, segs.data(), segs.size() * sizeof(int4), cudaMemcpyHostToDevice);
    return e;
}

std::string cache_path() {
    if (const char* p = std::getenv("QS_AUTOTUNE_CACHE")) return p;
    const char* home = std::getenv("HOME");
    return home ? std::string(home) + "/.cache/quaru_gb300_autotune.txt" : std::string();
}

bool cache_lookup(const std::string& key, int* cl, int* ct) {
    const std::string p = cache_path();
    if (p.empty()) return false;
    std::ifstream f(p);
    std::string k;
    int a, b;
    while (f >> k >> a >> b)
        if (k == key) {
            *cl = a;
            *ct = b;
            return true;
        }
    return false;
}

void cache_store(const std::string& key, int cl, int ct) {
    const std::string p = cache_path();
    if (p.empty()) return;
    std::ofstream f(p, std::ios::app);
    if (f) f << key << " " << cl << " " << ct << "\n";
}

}  // namespace

extern "C" int qs_batch_create(const qs_batch_circuit* circuits, size_t count, const qs_batch_options* opts,
                               qs_batch** out, size_t* err) {
    auto fail = [&](int code, const std::string& m) {
        set_last_error_message(m);
        return code;
    };
    if (!out || !circuits || count == 0) return fail(QS_INVALID_ARGUMENT, "need at least one circuit");
    *out = nullptr;
    qs_batch_options o{};
    o.precision = QS_PREC_C128;
    if (opts) o = *opts;
    if (o.precision != QS_PREC_C128 && o.precision != QS_PREC_C64) return fail(QS_INVALID_ARGUMENT, "unknown precision");
    auto* b = new qs_batch();
    b->prec = o.precision;
    b->count = int(count);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    // ---- validate and build host tables
    std::vector<BGate> gates;
    std::vector<BPauli> terms;
    std::vector<int2> rtab;
    size_t amp = b->prec == QS_PREC_C64 ? 8 : 16, state_bytes = 0;
    int counters = 0, minlog = 30;
    for (size_t c = 0; c < count; c++) {
        const qs_batch_circuit& q = circuits[c];
        if (q.n < 1 || q.n > 30 || (q.m && !q.gates) || (q.nterms && !q.terms)) {
            if (err) err[2] = c;
            release(b);
            return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + ": bad size or null table");
        }
        BCirc C{};
        C.n = int(q.n);
        C.ngates = int(q.m);
        C.gate_off = int(gates.size());
        C.nterms = int(q.nterms);
        C.term_off = int(terms.size());
        C.nsteps = 2 * int(q.m) + 1;
        C.counter_off = counters;
        counters += C.nsteps;
        b->param_off.push_back(b->total_params);
        b->total_params += q.nparams;
        std::vector<int> rp;
        for (size_t g = 0; g < q.m; g++) {
            const qs_param_gate& G = q.gates[g];
            BGate d{};
            const bool rotk = G.kind == QS_GATE_RX || G.kind == QS_GATE_RY || G.kind == QS_GATE_RZ;
            if (rotk) {
                if (G.k != 1 || !G.targets || G.targets[0] >= q.n || G.param < 0 || size_t(G.param) >= q.nparams) {
                    if (err) err[0] = G.targets ? G.targets[0] : 0, err[2] = c;
                    release(b);
                    return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + " gate " + std::to_string(g) +
                                                         ": bad rotation");
                }
                d.kind = G.kind;
                d.q0 = int(G.targets[0]);
                d.cs = int(b->cs_param.size());
                d.rslot = int(rp.size());
                b->cs_param.push_back(int(b->param_off[c]) + G.param);
                rp.push_back(G.param);
            } else if (G.kind == QS_GATE_FIXED && G.k == 1 && G.matrix && G.targets && G.targets[0] < q.n) {
                d.kind = kFix1;
                d.q0 = int(G.targets[0]);
                for (int i = 0; i < 8; i++) d.m[i] = G.matrix[i];
            } else if (G.kind == QS_GATE_FIXED && is_cnot(G) && G.targets && G.targets[0] < q.n &&
                       G.targets[1] < q.n && G.targets[0] != G.targets[1]) {
                d.kind = kCnot;
                d.q0 = int(G.targets[0]);
                d.q1 = int(G.targets[1]);
            } else {
                if (err) err[2] = c;
                release(b);
                return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + " gate " + std::to_string(g) +
                                                     ": the batch path takes rotations, 1-qubit gates and CNOTs");
            }
            gates.push_back(d);
        }
        for (size_t t = 0; t < q.nterms; t++) {
            if ((q.terms[t].x_mask | q.terms[t].z_mask) >> q.n) {
                if (err) err[2] = c;
                release(b);
                return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + ": Pauli term acts on a qubit >= n");
            }
            terms.push_back({q.terms[t].coeff, q.terms[t].x_mask, q.terms[t].z_mask});
        }
        C.nrot = int(rp.size());
        b->rot_param.push_back(rp);
        state_bytes += 2 * al((size_t(1) << q.n) * amp);
        minlog = std::min(minlog, C.n - 1);
        b->hcirc.push_back(C);
    }
    b->ncs = int(b->cs_param.size());
    b->ncounters = counters;
    // partial and result tables depend on the chunk size; size them for the smallest candidate (2^8 pairs)
    const int kMinChunk = 8;
    size_t part_max = 0;
    for (const BCirc& C : b->hcirc) {
        const int nch = 1 << (C.n - 1 - std::min(kMinChunk, C.n - 1));
        part_max += size_t(1 + C.nrot) * nch;
    }
    for (int c = 0; c < b->count; c++) {
        b->res_circ_base.push_back(int(rtab.size()));
        for (int r = 0; r <= b->hcirc[c].nrot; r++) rtab.push_back(make_int2(0, 0));
    }
    b->nres = int(rtab.size());
    // segments: at most count * maxsteps
    size_t max_segs = 0;
    for (const BCirc& C : b->hcirc) max_segs += size_t(C.nsteps);
    // ---- arena
    const size_t o_circ = 0, o_gates = o_circ + al(sizeof(BCirc) * count + 1),
                 o_terms = o_gates + al(sizeof(BGate) * gates.size() + 1),
                 o_cs = o_terms + al(sizeof(BPauli) * terms.size() + 1), o_first = o_cs + al(16 * (size_t(b->ncs) + 1)),
                 o_segs = o_first + al(4 * max_segs + 4), o_ctr = o_segs + al(sizeof(int4) * max_segs + 16),
                 o_part = o_ctr + al(4 * size_t(counters) + 4), o_res = o_part + al(8 * part_max + 8),
                 o_rtab = o_res + al(8 * size_t(b->nres) + 8), o_err = o_rtab + al(8 * size_t(b->nres) + 8),
                 o_tick = o_err + 256, o_states = o_tick + 256, total = o_states + state_bytes;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->arena, total);
    if (e == cudaSuccess) e = cudaMallocHost(&b->hcs, 16 * (size_t(b->ncs) + 1));
    if (e == cudaSuccess) e = cudaMallocHost(&b->hres, 8 * (size_t(b->nres) + 1));
    if (e == cudaSuccess) e = cudaMallocHost(&b->herr, sizeof(int));
    if (e != cudaSuccess) {
        release(b);
        return fail(e == cudaErrorMemoryAllocation ? QS_OUT_OF_MEMORY : QS_CUDA_ERROR,
                    std::string("batch allocation: ") + cudaGetErrorString(e));
    }
    unsigned char* A = b->arena;
    b->dcirc = reinterpret_cast<BCirc*>(A + o_circ);
    b->dgates = reinterpret_cast<BGate*>(A + o_gates);
    b->dterms = reinterpret_cast<BPauli*>(A + o_terms);
    b->dcs = reinterpret_cast<double2*>(A + o_cs);
    b->dseg_first = reinterpret_cast<uint32_t*>(A + o_first);
    b->dsegs = reinterpret_cast<int4*>(A + o_segs);
    b->dcounters = reinterpret_cast<unsigned int*>(A + o_ctr);
    b->dpart = reinterpret_cast<double*>(A + o_part);
    b->dres = reinterpret_cast<double*>(A + o_res);
    b->drtab = reinterpret_cast<int2*>(A + o_rtab);
    b->derr = reinterpret_cast<int*>(A + o_err);
    b->dticket = reinterpret_cast<unsigned int*>(A + o_tick);
    size_t off = o_states;
    for (auto& C : b->hcirc) {
        C.psi = reinterpret_cast<unsigned long long>(A + off);
        off += al((size_t(1) << C.n) * amp);
        C.lam = reinterpret_cast<unsigned long long>(A + off);
        off += al((size_t(1) << C.n) * amp);
    }
    // per chunk size: partial offsets and result table
    auto layout = [&](int cl) {
        int part = 0;
        std::vector<int2> rt;
        for (auto& C : b->hcirc) {
            const int nch = 1 << (C.n - 1 - std::min(cl, C.n - 1));
            C.part_off = part;
            C.nch_log = C.n - 1 - std::min(cl, C.n - 1);
            for (int r = 0; r <= C.nrot; r++) rt.push_back(make_int2(part + r * nch, nch));
            part += (1 + C.nrot) * nch;
        }
        cudaError_t e2 = cudaMemcpy(b->dcirc, b->hcirc.data(), sizeof(BCirc) * count, cudaMemcpyHostToDevice);
        if (e2 == cudaSuccess && !rt.empty())
            e2 = cudaMemcpy(b->drtab, rt.data(), sizeof(int2) * rt.size(), cudaMemcpyHostToDevice);
        if (e2 == cudaSuccess) e2 = upload_schedule(b, cl);
        return e2;
    };
    if (!gates.empty()) e = cudaMemcpy(b->dgates, gates.data(), sizeof(BGate) * gates.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !terms.empty())
        e = cudaMemcpy(b->dterms, terms.data(), sizeof(BPauli) * terms.size(), cudaMemcpyHostToDevice);
    for (int i = 0; i < b->ncs; i++) b->hcs[i] = make_double2(1.0, 0.0);
    // ---- chunk size and persistence: from options, the autotune cache, or by timing candidates
    std::ostringstream key;
    key << "batch:p" << b->prec << ":c" << count << ":items";
    {
        uint64_t sig = 0;
        for (const BCirc& C : b->hcirc) sig = sig * 1315423911ull + uint64_t(C.n) * 131 + uint64_t(C.ngates);
        key << sig;
    }
    int cl = o.chunk_log2, ct = o.ctas_per_sm;
    if (cl <= 0 || ct <= 0) {
        int ccl = 0, cct = 0;
        if (cache_lookup(key.str(), &ccl, &cct)) {
            if (cl <= 0) cl = ccl;
            if (ct <= 0) ct = cct;
        }
    }
    if (e == cudaSuccess && (cl <= 0 || ct <= 0)) {
        // autotune: time one run per candidate
        double best = 1e30;
        int bcl = 12, bct = 2;
        const std::vector<int> cls = cl > 0 ? std::vector<int>{cl} : std::vector<int>{9, 11, 13};
        const std::vector<int> cts = ct > 0 ? std::vector<int>{ct} : std::vector<int>{2, 4};
        for (int tcl : cls) {
            for (int tct : cts) {
                b->ctas = tct;
                if ((e = layout(std::max(kMinChunk, tcl))) != cudaSuccess || (e = capture(b)) != cudaSuccess) break;
                cudaGraphLaunch(b->exec, b->stream);
                cudaStreamSynchronize(b->stream);
                const auto t0 = std::chrono::steady_clock::now();
                cudaGraphLaunch(b->exec, b->stream);
                e = cudaStreamSynchronize(b->stream);
                const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                if (e != cudaSuccess || *b->herr) break;
                if (dt < best) best = dt, bcl = tcl, bct = tct;
            }
            if (e != cudaSuccess) break;
        }
        cl = bcl;
        ct = bct;
        if (e == cudaSuccess) cache_store(key.str(), cl, ct);
    }
    b->ctas = std::max(1, ct);
    if (e == cudaSuccess) e = layout(std::max(kMinChunk, cl));
    if (e == cudaSuccess) e = capture(b);
    if (e != cudaSuccess) {
        release(b);
        return fail(QS_CUDA_ERROR, std::string("batch setup: ") + cudaGetErrorString(e));
    }
    if (*b->herr) {
        release(b);
        return fail(QS_TIMEOUT, "batch setup: a dependency wait gave up");
    }
    *out = b;
    return QS_OK;
}

extern "C" int qs_batch_run(qs_batch* b, const double* params, double* energies, double* grads) {
    if (!b || (b->total_params && !params)) {
        set_last_error_message("null argument");
        return QS_INVALID_ARGUMENT;
    }
    for (int i = 0; i < b->ncs; i++) {
        const double th = params[b->cs_param[i]];
        b->hcs[i] = make_double2(std::cos(0.5 * th), std::sin(0.5 * th));
    }
    cudaError_t e = cudaGraphLaunch(b->exec, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        set_last_error_message(std::string("batch run: ") + cudaGetErrorString(e));
        return QS_CUDA_ERROR;
    }
    if (*b->herr) {
        set_last_error_message("batch run: a dependency wait in the persistent kernel gave up");
        return QS_TIMEOUT;
    }
    for (int c = 0; c < b->count; c++) {
        const int base = b->res_circ_base[c];
        if (energies) energies[c] = b->hres[base];
        if (grads) {
            const size_t po = b->param_off[c];
            const size_t np = (size_t(c + 1) < b->param_off.size() ? b->param_off[c + 1] : b->total_params) - po;
            for (size_t p = 0; p < np; p++) grads[po + p] = 0.0;
            for (size_t r = 0; r < b->rot_param[c].size(); r++) grads[po + b->rot_param[c][r]] += b->hres[base + 1 + r];
        }
    }
    return QS_OK;
}

extern "C" int qs_batch_config(const qs_batch* b, int* chunk_log2, int* ctas_per_sm) {
    if (!b) return QS_INVALID_ARGUMENT;
    if (chunk_log2) *chunk_log2 = b->chunk_log;
    if (ctas_per_sm) *ctas_per_sm = b->ctas;
    return QS_OK;
}

extern "C" void qs_batch_free(qs_batch* b) { release(b); }
