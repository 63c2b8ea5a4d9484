// qs_batch.cu — forward + adjoint gradients for a batch of circuits in one persistent launch.
//
// No counterpart in the reference. Each circuit's gates are planned into tiled stages (the planner
// of the fused forward path, qs_plan.cpp): forward stages, one step forming lambda = H psi with the
// energy partial sums, and reverse stages walking the gates backwards (rotations with their
// Im<lambda|A|psi> partials, fixed gates un-applied from psi and lambda). A work item is
// (circuit c, step s, chunk j): a range of tiles of one stage, each tile loaded once into shared
// memory, taken through all of the stage's gates and written back once (or, for the H psi step, a
// range of amplitude pairs). Items are ordered by step round across circuits, so an item only ever
// waits for items handed out before it; those are held by running CTAs, which makes the schedule
// deadlock-free without any co-residency assumption. Every wait is bounded: when it gives up it
// raises an error flag that makes every CTA return, and the host reports QS_TIMEOUT.
//
// The whole pass (parameter upload, state reset, persistent kernel, partial reduction, result
// download) is captured once in a CUDA graph; a run writes new parameters into pinned memory and
// replays it. Complex128 batches with QS_ARITH_DF64 hold the tiles of stages made of rotations and
// CNOTs as double-float values (FP32 pipe), with the inner products accumulated in FP64.
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
#include "qs_rot.cuh"
#include "qs_tile.h"
#include "qs_tma.cuh"

namespace qs {
namespace {

constexpr int kBT = 256;
constexpr int kFix1 = 16;  // fixed dense 1-qubit gate
constexpr int kCnot = 17;  // CNOT
constexpr int kBTileMax = 11;  // tile qubits
constexpr int kBMaxRot = kMaxStageOps;  // rotations per stage
constexpr long long kWaitCycles = 20000000000LL;  // ~10 s at 2 GHz: dependency waits give up after this

struct BCirc {
    unsigned long long psi, lam;
    int n, nterms, term_off, nsteps, counter_off, nrot;
    int epart_off, rpart_off;  // partials: energy (2^nche_log), then rotation r at rpart_off + r * 2^ncht_log
    int nche_log, ncht_log;    // chunks of the H psi step and of every tile stage
    int T, stage_off, nfwd;    // tile qubits, first stage, forward stages (step nfwd is H psi)
};

struct BStage {
    int op_off, nops, nrot, df;  // df: double-float tiles
    int L, H, pad0, pad1;
    uint8_t pos[16];   // the tile's qubits, sorted (its base index skips them)
    uint8_t high[8];   // qubit of local bit L + b
};

struct BOp {
    int kind;   // QS_GATE_RX / RY / RZ, kFix1, kCnot
    int tb;     // local target bit
    int cb;     // CNOT: local control bit, or -1
    int cglob;  // CNOT: control qubit outside the tile, or -1
    int cs;     // rotation: index of (cos, sin) of theta/2
    int rslot;  // rotation: circuit-level slot
    int lrot;   // rotation: stage-local slot
    int pad;
    double m[8];  // kFix1: the 2x2 matrix (forward); its adjoint is formed on the fly
};

struct BPauli {
    double c;
    unsigned long long x, z;
    float ch, cl;  // c as a float pair (complex64 circuits)
    uint32_t cls;  // |x & z| mod 4: the term's factor i^cls
    uint32_t pad_;
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
    // integer-pipe conversion (exact for normal floats; subnormals read as zero)
    static __device__ __forceinline__ double2 d(float2 v) { return make_double2(df_f2d(v.x), df_f2d(v.y)); }
    static __device__ __forceinline__ float2 from(double2 v) { return make_float2(float(v.x), float(v.y)); }
};

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

template <typename T>
__global__ void __launch_bounds__(kBT) k_batch_reset(const BCirc* __restrict__ circs) {
    const BCirc C = circs[blockIdx.y];
    T* psi = reinterpret_cast<T*>(C.psi);
    const uint64_t N = 1ull << C.n;
    for (uint64_t i = uint64_t(blockIdx.x) * kBT + threadIdx.x; i < N; i += uint64_t(gridDim.x) * kBT)
        St<T>::st(psi, i, St<T>::from(make_double2(i == 0 ? 1.0 : 0.0, 0.0)));
}

__device__ __forceinline__ uint32_t pair_index(uint32_t p, int tb) {
    return ((p >> tb) << (tb + 1)) | (p & ((1u << tb) - 1u));
}

// One gate of a stage on the tile(s) in shared memory. fwd: psi only; reverse: psi and lambda, with
// a rotation's inner-product term accumulated (before it is un-applied) into acc.
template <typename T, int AXIS, typename R = decltype(T().x)>
__device__ __forceinline__ auto tile_rot(T* sp, T* sl, uint32_t half, int tb, R c, R sn, bool fwd) {
    const R cc = c, ss = fwd ? sn : -sn;
    double acc = 0.0;
    DfAcc facc;  // complex64: compensated pair sums, reduced over the warp as a float pair
    for (uint32_t p = threadIdx.x; p < half; p += kBT) {
        const uint32_t i0 = pair_index(p, tb), i1 = i0 | (1u << tb);
        T a = sp[i0], b = sp[i1];
        if (!fwd) {
            T l0 = sl[i0], l1 = sl[i1];
            if constexpr (sizeof(R) == 8)
                acc += im_term<AXIS>(l0, l1, a, b);
            else
                im_term_acc<AXIS>(facc, l0, l1, a, b);
            rot_pair<AXIS>(cc, ss, l0.x, l0.y, l1.x, l1.y);
            sl[i0] = l0;
            sl[i1] = l1;
        }
        rot_pair<AXIS>(cc, ss, a.x, a.y, b.x, b.y);
        sp[i0] = a;
        sp[i1] = b;
    }
    if constexpr (sizeof(R) == 4)
        return facc;
    else
        return acc;
}

template <int AXIS>
__device__ __forceinline__ DfAcc tile_rot_df(float4* sp, float4* sl, uint32_t half, int tb, double c, double sn,
                                              bool fwd) {
    float ch, cl, sh, slo;
    df_split(c, ch, cl);
    df_split(fwd ? sn : -sn, sh, slo);
    DfAcc acc;
    for (uint32_t p = threadIdx.x; p < half; p += kBT) {
        const uint32_t i0 = pair_index(p, tb), i1 = i0 | (1u << tb);
        float4 a = sp[i0], b = sp[i1];
        if (!fwd) {
            float4 l0 = sl[i0], l1 = sl[i1];
            adj_im_df_acc<AXIS>(acc, l0, l1, a, b);
            df_rot_pair<AXIS>(ch, cl, sh, slo, l0, l1);
            sl[i0] = l0;
            sl[i1] = l1;
        }
        df_rot_pair<AXIS>(ch, cl, sh, slo, a, b);
        sp[i0] = a;
        sp[i1] = b;
    }
    return acc;
}

template <typename E>
__device__ __forceinline__ void tile_cnot(E* s, uint32_t half, int tb, int cb) {
    for (uint32_t p = threadIdx.x; p < half; p += kBT) {
        const uint32_t i0 = pair_index(p, tb);
        if (cb >= 0 && !((i0 >> cb) & 1u)) continue;
        const uint32_t i1 = i0 | (1u << tb);
        const E t = s[i0];
        s[i0] = s[i1];
        s[i1] = t;
    }
}

template <typename T>
__device__ __forceinline__ void tile_fix1(T* s, uint32_t half, int tb, const double* m, bool adj) {
    for (uint32_t p = threadIdx.x; p < half; p += kBT) {
        const uint32_t i0 = pair_index(p, tb), i1 = i0 | (1u << tb);
        double2 a = St<T>::d(s[i0]), b = St<T>::d(s[i1]);
        mat2(m, adj, a, b);
        s[i0] = St<T>::from(a);
        s[i1] = St<T>::from(b);
    }
}

template <typename T>
__global__ void __launch_bounds__(kBT) k_batch(const BCirc* __restrict__ circs, const BStage* __restrict__ stages,
                                               const BOp* __restrict__ ops, const BPauli* __restrict__ terms,
                                               const double2* __restrict__ cs, const uint32_t* __restrict__ seg_first,
                                               const int4* __restrict__ segs, int nsegs, uint32_t nitems,
                                               unsigned int* __restrict__ counters, double* __restrict__ partials,
                                               unsigned int* __restrict__ ticket, int* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sp = reinterpret_cast<T*>(smem_raw);
    T* sl = sp + (1u << kBTileMax);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(sl + (1u << kBTileMax));
    double* sacc = reinterpret_cast<double*>(rowoff + 64);  // [kBMaxRot][8 warps]
    __shared__ uint32_t s_item;
    __shared__ int s_seg, s_stop;
    __shared__ float2 s_csf[kBMaxRot];  // complex64: the stage's rotation (cos, sin) rounded to float
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
        const int c = sg.x, s = sg.y, prevnch = sg.w;
        const uint32_t j = s_item - seg_first[s_seg];
        const BCirc C = circs[c];
        if (s > 0 && threadIdx.x == 0) {  // every chunk of the previous step must be done
            if (!counter_wait_bounded(counters + C.counter_off + s - 1, unsigned(prevnch), kWaitCycles)) {
                atomicExch(err, 1);
                s_stop = 1;
            }
            __threadfence();
        }
        __syncthreads();
        if (s_stop) return;
        T* psi = reinterpret_cast<T*>(C.psi);
        T* lam = reinterpret_cast<T*>(C.lam);
        if (s == C.nfwd) {  // lambda = H psi over amplitudes [2 p0, 2 p1), energy partial
            const int cl = C.n - 1 - C.nche_log;
            const uint64_t p0 = uint64_t(j) << cl, p1 = p0 + (1ull << cl);
            double e = 0.0;
            DfAcc eacc;  // complex64: the energy terms as a compensated float pair
            for (uint64_t i = 2 * p0 + threadIdx.x; i < 2 * p1; i += kBT) {
                if constexpr (sizeof(T) == 8) {  // complex64: products and sums in compensated float pairs
                    DfAcc fre, fim;
                    for (int t = 0; t < C.nterms; t++) {
                        const BPauli& P = terms[C.term_off + t];
                        const uint64_t k = i ^ P.x;
                        const float2 v = St<T>::ld(psi, k);
                        const bool neg = __popcll(P.z & k) & 1;
                        const float ch = neg ? -P.ch : P.ch, cl = neg ? -P.cl : P.cl;
                        float xr, xi;  // i^cls * v
                        switch (P.cls) {
                            case 0: xr = v.x; xi = v.y; break;
                            case 1: xr = -v.y; xi = v.x; break;
                            case 2: xr = -v.x; xi = -v.y; break;
                            default: xr = v.y; xi = -v.x; break;
                        }
                        fre.add_prod(ch, xr);
                        fre.c = __fmaf_rn(cl, xr, fre.c);
                        fim.add_prod(ch, xi);
                        fim.c = __fmaf_rn(cl, xi, fim.c);
                    }
                    const float2 lv = make_float2(__fadd_rn(fre.s, fre.c), __fadd_rn(fim.s, fim.c));
                    St<T>::st(lam, i, lv);
                    const float2 pv = St<T>::ld(psi, i);  // energy term Re(conj(psi_i) lambda_i)
                    eacc.add_prod(pv.x, lv.x);
                    eacc.add_prod(pv.y, lv.y);
                    continue;
                }
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
                const double2 pv = St<T>::d(St<T>::ld(psi, i));
                e = fma(pv.x, re, fma(pv.y, im, e));
            }
            if constexpr (sizeof(T) == 8) e = __dadd_rn(df_f2d(eacc.s), df_f2d(eacc.c));
            double dummy = 0.0;
            rd_block_sum2<kBT>(e, dummy);
            if (threadIdx.x == 0) partials[C.epart_off + j] = e;
        } else {  // a tiled stage: tiles [j * tpi, (j + 1) * tpi)
            const bool fwd = s < C.nfwd;
            const BStage S = stages[C.stage_off + (fwd ? s : s - 1)];
            const uint32_t tsize = 1u << C.T, half = tsize >> 1;
            const uint64_t tpi = 1ull << (C.n - C.T - C.ncht_log);
            const uint32_t lmask = (1u << S.L) - 1u;
            for (int r = threadIdx.x; r < (1 << S.H); r += kBT) {
                uint64_t o = 0;
                for (int b = 0; b < S.H; b++)
                    if (r >> b & 1) o |= 1ull << S.high[b];
                rowoff[r] = o;
            }
            if (!fwd)
                for (int r = threadIdx.x; r < S.nrot * (kBT / 32); r += kBT) sacc[r] = 0.0;
            if constexpr (sizeof(T) == 8)  // one conversion per rotation per item, not per thread and tile
                for (int o = threadIdx.x; o < S.nops; o += kBT) {
                    const BOp op = ops[S.op_off + o];
                    if (op.kind != kCnot && op.kind != kFix1) {
                        const double2 t2 = cs[op.cs];
                        s_csf[o] = make_float2(float(t2.x), float(t2.y));
                    }
                }
            __syncthreads();
            float4* fp = reinterpret_cast<float4*>(sp);
            float4* fl = reinterpret_cast<float4*>(sl);
            const bool df = sizeof(T) == 16 && S.df;
            for (uint64_t t = uint64_t(j) * tpi; t < uint64_t(j + 1) * tpi; t++) {
                uint64_t base = t;  // insert the tile's qubits as zero bits
                for (int k = 0; k < C.T; k++) {
                    const int q = S.pos[k];
                    base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1ull));
                }
                for (uint32_t i = threadIdx.x; i < tsize; i += kBT) {
                    const uint64_t g = base + rowoff[i >> S.L] + (i & lmask);
                    const T v = St<T>::ld(psi, g);
                    T w = v;
                    if (!fwd) w = St<T>::ld(lam, g);
                    if (df) {
                        const double2 dv = St<T>::d(v), dw = St<T>::d(w);
                        float4 f;
                        df_split(dv.x, f.x, f.y);
                        df_split(dv.y, f.z, f.w);
                        fp[i] = f;
                        if (!fwd) {
                            df_split(dw.x, f.x, f.y);
                            df_split(dw.y, f.z, f.w);
                            fl[i] = f;
                        }
                    } else {
                        sp[i] = v;
                        if (!fwd) sl[i] = w;
                    }
                }
                __syncthreads();
                for (int o = 0; o < S.nops; o++) {
                    const BOp op = ops[S.op_off + o];
                    if (op.kind == kCnot) {
                        if (op.cglob < 0 || ((base >> op.cglob) & 1ull)) {  // outside control: the whole tile
                            if (df) {
                                tile_cnot(fp, half, op.tb, op.cb);
                                if (!fwd) tile_cnot(fl, half, op.tb, op.cb);
                            } else {
                                tile_cnot(sp, half, op.tb, op.cb);
                                if (!fwd) tile_cnot(sl, half, op.tb, op.cb);
                            }
                        }
                    } else if (op.kind == kFix1) {  // never in double-float stages
                        if constexpr (true) {
                            tile_fix1(sp, half, op.tb, op.m, !fwd);
                            if (!fwd) tile_fix1(sl, half, op.tb, op.m, true);
                        }
                    } else if constexpr (sizeof(T) == 8) {  // complex64
                        const float2 t2 = s_csf[o];
                        DfAcc f;
                        if (op.kind == QS_GATE_RX) f = tile_rot<T, QS_GATE_RX>(sp, sl, half, op.tb, t2.x, t2.y, fwd);
                        else if (op.kind == QS_GATE_RY) f = tile_rot<T, QS_GATE_RY>(sp, sl, half, op.tb, t2.x, t2.y, fwd);
                        else f = tile_rot<T, QS_GATE_RZ>(sp, sl, half, op.tb, t2.x, t2.y, fwd);
                        if (!fwd) {  // the warp's float pairs reduced on the FP32 pipe, one FP64 rejoin
                            f.warp_reduce();
                            if (lane == 0) sacc[op.lrot * (kBT / 32) + warp] += __dadd_rn(df_f2d(f.s), df_f2d(f.c));
                        }
                    } else {
                        const double2 t2 = cs[op.cs];
                        double v;
                        if (df) {
                            DfAcc f;
                            if (op.kind == QS_GATE_RX) f = tile_rot_df<QS_GATE_RX>(fp, fl, half, op.tb, t2.x, t2.y, fwd);
                            else if (op.kind == QS_GATE_RY) f = tile_rot_df<QS_GATE_RY>(fp, fl, half, op.tb, t2.x, t2.y, fwd);
                            else f = tile_rot_df<QS_GATE_RZ>(fp, fl, half, op.tb, t2.x, t2.y, fwd);
                            v = 0.0;
                            if (!fwd) {  // float pairs over the warp, one FP64 rejoin
                                f.warp_reduce();
                                v = __dadd_rn(df_f2d(f.s), df_f2d(f.c));
                            }
                        } else {
                            if (op.kind == QS_GATE_RX) v = tile_rot<T, QS_GATE_RX>(sp, sl, half, op.tb, t2.x, t2.y, fwd);
                            else if (op.kind == QS_GATE_RY) v = tile_rot<T, QS_GATE_RY>(sp, sl, half, op.tb, t2.x, t2.y, fwd);
                            else v = tile_rot<T, QS_GATE_RZ>(sp, sl, half, op.tb, t2.x, t2.y, fwd);
                        }
                        if (!fwd) {
                            if (!df) v = rd_warp_sum(v);
                            if (lane == 0) sacc[op.lrot * (kBT / 32) + warp] += v;
                        }
                    }
                    __syncthreads();
                }
                for (uint32_t i = threadIdx.x; i < tsize; i += kBT) {
                    const uint64_t g = base + rowoff[i >> S.L] + (i & lmask);
                    if (df) {
                        const float4 f = fp[i];
                        St<T>::st(psi, g, St<T>::from(make_double2(__dadd_rn(df_f2d(f.x), df_f2d(f.y)),
                                                                   __dadd_rn(df_f2d(f.z), df_f2d(f.w)))));
                        if (!fwd) {
                            const float4 h = fl[i];
                            St<T>::st(lam, g, St<T>::from(make_double2(__dadd_rn(df_f2d(h.x), df_f2d(h.y)),
                                                                       __dadd_rn(df_f2d(h.z), df_f2d(h.w)))));
                        }
                    } else {
                        St<T>::st(psi, g, sp[i]);
                        if (!fwd) St<T>::st(lam, g, sl[i]);
                    }
                }
                __syncthreads();
            }
            if (!fwd) {  // this item's partial of every rotation of the stage
                for (int o = threadIdx.x; o < S.nops; o += kBT) {
                    const BOp op = ops[S.op_off + o];
                    if (op.kind == kCnot || op.kind == kFix1) continue;
                    double v = 0.0;
                    for (int w = 0; w < kBT / 32; w++) v += sacc[op.lrot * (kBT / 32) + w];
                    partials[C.rpart_off + size_t(op.rslot << C.ncht_log) + j] = v;
                }
            }
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
    int prec = QS_PREC_C128, arith = QS_ARITH_FMA, count = 0, sms = 1, chunk_log = 12, ctas = 2;
    cudaStream_t stream = nullptr;
    unsigned char* arena = nullptr;
    qs::BCirc* dcirc = nullptr;
    qs::BStage* dstages = nullptr;
    qs::BOp* dops = nullptr;
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
    size_t total_params = 0, smem = 0;
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

// Chunks of step s of circuit C for the current chunk size (the H psi step counts pair chunks).
int step_chunks(const BCirc& C, int s) { return 1 << (s == C.nfwd ? C.nche_log : C.ncht_log); }

// Work-item schedule: segments (circuit, step, chunks, chunks of the previous step) by step round.
void build_schedule(qs_batch* b, std::vector<uint32_t>* first, std::vector<int4>* segs, uint64_t* nitems) {
    first->clear();
    segs->clear();
    int maxsteps = 0;
    for (const auto& c : b->hcirc) maxsteps = std::max(maxsteps, c.nsteps);
    uint64_t item = 0;
    for (int s = 0; s < maxsteps; s++)
        for (int c = 0; c < b->count; c++) {
            const BCirc& C = b->hcirc[c];
            if (s >= C.nsteps) continue;
            const int nch = step_chunks(C, s);
            first->push_back(uint32_t(item));
            segs->push_back(make_int4(c, s, nch, s > 0 ? step_chunks(C, s - 1) : 0));
            item += uint64_t(nch);
        }
    *nitems = item;
}

size_t batch_smem(int prec) {
    const size_t amp = prec == QS_PREC_C64 ? 8 : 16;
    return 2 * (amp << kBTileMax) + 64 * 8 + size_t(kBMaxRot) * (kBT / 32) * 8;
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
        k_batch<float2><<<b->sms * b->ctas, kBT, b->smem, s>>>(b->dcirc, b->dstages, b->dops, b->dterms, b->dcs,
                                                               b->dseg_first, b->dsegs, b->nsegs, b->nitems,
                                                               b->dcounters, b->dpart, b->dticket, b->derr);
    } else {
        k_batch_reset<double2><<<rg, kBT, 0, s>>>(b->dcirc);
        k_batch<double2><<<b->sms * b->ctas, kBT, b->smem, s>>>(b->dcirc, b->dstages, b->dops, b->dterms, b->dcs,
                                                                b->dseg_first, b->dsegs, b->nsegs, b->nitems,
                                                                b->dcounters, b->dpart, b->dticket, b->derr);
    }
    k_batch_reduce<<<std::min(b->nres, b->sms * 8), kBT, 0, s>>>(b->dpart, b->drtab, b->nres, b->dres);
    cudaMemcpyAsync(b->hres, b->dres, sizeof(double) * b->nres, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(b->herr, b->derr, sizeof(int), cudaMemcpyDeviceToHost, s);
    e = cudaStreamEndCapture(s, &b->graph);
    if (e != cudaSuccess) return e;
    return cudaGraphInstantiate(&b->exec, b->graph, 0);
}

// Planning form of one gate (targets forced into the tile, controls free): rotations and fixed
// 1-qubit gates as dense 1-qubit gates on their target, CNOT as classified (target + control).
OpDesc plan_desc(const qs_param_gate& G, bool cnot) {
    OpDesc d;
    if (cnot) {
        classify_gate(G.matrix, 2, G.targets, &d);
        return d;
    }
    d.kind = OP_DENSE;
    d.k = d.orig_k = 1;
    d.tq[0] = int(G.targets[0]);
    d.m.assign(8, 0.0);
    d.touched_rows = 2;
    return d;
}

// Stages of one circuit (forward gates, then the reverse sweep) into the stage and op tables.
void plan_circuit(const qs_batch_circuit& q, int T, bool df_ok, BCirc* C, const std::vector<int>& cs_of,
                  const std::vector<int>& rslot_of, std::vector<BStage>* stages, std::vector<BOp>* ops) {
    const int n = int(q.n), L = std::min(5, T);
    std::vector<char> cnot(q.m);
    std::vector<OpDesc> fw;
    for (size_t g = 0; g < q.m; g++) {
        cnot[g] = q.gates[g].kind == QS_GATE_FIXED && q.gates[g].k == 2;
        fw.push_back(plan_desc(q.gates[g], cnot[g]));
    }
    auto emit = [&](const std::vector<int>& order, bool fwd) {
        std::vector<OpDesc> list;
        for (int g : order) list.push_back(fw[g]);
        const std::vector<TileStage> st = plan_tiles(list, n, T, L, false);
        int count = 0;
        for (const TileStage& S : st) {
            BStage B{};
            B.op_off = int(ops->size());
            B.L = S.L;
            B.H = int(S.high.size());
            std::vector<int> qpos;
            for (int qb = 0; qb < S.L; qb++) qpos.push_back(qb);
            for (int qb : S.high) qpos.push_back(qb);
            std::sort(qpos.begin(), qpos.end());
            for (size_t i = 0; i < qpos.size(); i++) B.pos[i] = uint8_t(qpos[i]);
            for (int i = 0; i < B.H; i++) B.high[i] = uint8_t(S.high[i]);
            auto local = [&](int qb) -> int {
                if (qb < S.L) return qb;
                for (int i = 0; i < B.H; i++)
                    if (S.high[i] == qb) return S.L + i;
                return -1;
            };
            B.df = df_ok ? 1 : 0;
            for (int idx : S.ops) {
                const int g = order[idx];
                const qs_param_gate& G = q.gates[g];
                BOp o{};
                o.cb = o.cglob = -1;
                if (cnot[g]) {  // CNOT's matrix: targets[1] = 1 swaps the rows of targets[0]
                    o.kind = kCnot;
                    o.tb = local(int(G.targets[0]));
                    o.cb = local(int(G.targets[1]));
                    if (o.cb < 0) o.cglob = int(G.targets[1]);
                } else if (G.kind == QS_GATE_FIXED) {
                    o.kind = kFix1;
                    o.tb = local(int(G.targets[0]));
                    for (int i = 0; i < 8; i++) o.m[i] = G.matrix[i];
                    B.df = 0;  // double-float stages take rotations and CNOTs
                } else {
                    o.kind = G.kind;
                    o.tb = local(int(G.targets[0]));
                    o.cs = cs_of[g];
                    o.rslot = rslot_of[g];
                    o.lrot = B.nrot++;
                }
                ops->push_back(o);
                B.nops++;
            }
            stages->push_back(B);
            count++;
        }
        return count;
    };
    std::vector<int> order(q.m);
    for (size_t g = 0; g < q.m; g++) order[g] = int(g);
    C->stage_off = int(stages->size());
    C->nfwd = emit(order, true);
    std::reverse(order.begin(), order.end());
    const int nrev = emit(order, false);
    C->nsteps = C->nfwd + 1 + nrev;
}

}  // namespace

extern "C" int qs_batch_create(const qs_batch_circuit* circuits, size_t count, const qs_batch_options* opts,
                               qs_batch** out, size_t* err) {
    qs::TraceRange trace("qs_batch_create");
    auto fail = [&](int code, const std::string& m) {
        set_last_error_message(m);
        return code;
    };
    if (!out || !circuits || count == 0) return fail(QS_INVALID_ARGUMENT, "need at least one circuit");
    *out = nullptr;
    qs_batch_options o{};
    o.precision = QS_PREC_C128;
    o.arith = QS_ARITH_FMA;
    if (opts) o = *opts;
    if (o.precision != QS_PREC_C128 && o.precision != QS_PREC_C64) return fail(QS_INVALID_ARGUMENT, "unknown precision");
    auto* b = new qs_batch();
    b->prec = o.precision;
    b->arith = o.arith;
    b->count = int(count);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    // ---- validate and plan
    std::vector<BStage> stages;
    std::vector<BOp> ops;
    std::vector<BPauli> terms;
    const size_t amp = b->prec == QS_PREC_C64 ? 8 : 16;
    size_t state_bytes = 0;
    int counters = 0;
    for (size_t c = 0; c < count; c++) {
        const qs_batch_circuit& q = circuits[c];
        if (q.n < 1 || q.n > 30 || (q.m && !q.gates) || (q.nterms && !q.terms)) {
            if (err) err[2] = c;
            release(b);
            return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + ": bad size or null table");
        }
        BCirc C{};
        C.n = int(q.n);
        C.T = std::min(kBTileMax, C.n);
        C.nterms = int(q.nterms);
        C.term_off = int(terms.size());
        b->param_off.push_back(b->total_params);
        b->total_params += q.nparams;
        std::vector<int> rp, cs_of(q.m, -1), rslot_of(q.m, -1);
        for (size_t g = 0; g < q.m; g++) {
            const qs_param_gate& G = q.gates[g];
            const bool rotk = G.kind == QS_GATE_RX || G.kind == QS_GATE_RY || G.kind == QS_GATE_RZ;
            if (rotk) {
                if (G.k != 1 || !G.targets || G.targets[0] >= q.n || G.param < 0 || size_t(G.param) >= q.nparams) {
                    if (err) err[0] = G.targets ? G.targets[0] : 0, err[2] = c;
                    release(b);
                    return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + " gate " + std::to_string(g) +
                                                         ": bad rotation");
                }
                cs_of[g] = int(b->cs_param.size());
                rslot_of[g] = int(rp.size());
                b->cs_param.push_back(int(b->param_off[c]) + G.param);
                rp.push_back(G.param);
            } else if (G.kind == QS_GATE_FIXED && G.k == 1 && G.matrix && G.targets && G.targets[0] < q.n) {
            } else if (G.kind == QS_GATE_FIXED && is_cnot(G) && G.targets && G.targets[0] < q.n &&
                       G.targets[1] < q.n && G.targets[0] != G.targets[1]) {
            } else {
                if (err) err[2] = c;
                release(b);
                return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + " gate " + std::to_string(g) +
                                                     ": the batch path takes rotations, 1-qubit gates and CNOTs");
            }
        }
        for (size_t t = 0; t < q.nterms; t++) {
            if ((q.terms[t].x_mask | q.terms[t].z_mask) >> q.n) {
                if (err) err[2] = c;
                release(b);
                return fail(QS_INVALID_ARGUMENT, "circuit " + std::to_string(c) + ": Pauli term acts on a qubit >= n");
            }
            const double c = q.terms[t].coeff;
            const float ch = float(c);
            terms.push_back({c, q.terms[t].x_mask, q.terms[t].z_mask, ch, float(c - double(ch)),
                             uint32_t(__builtin_popcountll(q.terms[t].x_mask & q.terms[t].z_mask) & 3), 0u});
        }
        C.nrot = int(rp.size());
        plan_circuit(q, C.T, b->prec == QS_PREC_C128 && b->arith == QS_ARITH_DF64, &C, cs_of, rslot_of, &stages,
                     &ops);
        C.counter_off = counters;
        counters += C.nsteps;
        b->rot_param.push_back(rp);
        state_bytes += 2 * al((size_t(1) << q.n) * amp);
        b->hcirc.push_back(C);
    }
    b->ncs = int(b->cs_param.size());
    b->ncounters = counters;
    // partial tables depend on the chunk size; size them for the smallest candidate (2^8 pairs per item)
    const int kMinChunk = 8;
    size_t part_max = 0, max_segs = 0;
    for (const BCirc& C : b->hcirc) {
        part_max += (size_t(1) << (C.n - 1 - std::min(kMinChunk, C.n - 1))) + size_t(C.nrot) * (size_t(1) << (C.n - C.T));
        max_segs += size_t(C.nsteps);
    }
    std::vector<int2> rtab;
    for (int c = 0; c < b->count; c++) {
        b->res_circ_base.push_back(int(rtab.size()));
        for (int r = 0; r <= b->hcirc[c].nrot; r++) rtab.push_back(make_int2(0, 0));
    }
    b->nres = int(rtab.size());
    // ---- arena
    const size_t o_circ = 0, o_stages = o_circ + al(sizeof(BCirc) * count + 1),
                 o_ops = o_stages + al(sizeof(BStage) * stages.size() + 1),
                 o_terms = o_ops + al(sizeof(BOp) * ops.size() + 1),
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
    if (e == cudaSuccess) *b->herr = 0;  // page-locked memory comes uninitialised; read even when no run precedes
    b->smem = batch_smem(b->prec);
    if (e == cudaSuccess)
        e = b->prec == QS_PREC_C64
                ? cudaFuncSetAttribute(k_batch<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(b->smem))
                : cudaFuncSetAttribute(k_batch<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(b->smem));
    if (e != cudaSuccess) {
        release(b);
        return fail(e == cudaErrorMemoryAllocation ? QS_OUT_OF_MEMORY : QS_CUDA_ERROR,
                    std::string("batch allocation: ") + cudaGetErrorString(e));
    }
    unsigned char* A = b->arena;
    b->dcirc = reinterpret_cast<BCirc*>(A + o_circ);
    b->dstages = reinterpret_cast<BStage*>(A + o_stages);
    b->dops = reinterpret_cast<BOp*>(A + o_ops);
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
    // per chunk size (2^cl amplitude pairs per item): chunk counts, partial offsets, result table,
    // schedule
    auto layout = [&](int cl) {
        int part = 0;
        std::vector<int2> rt;
        for (auto& C : b->hcirc) {
            C.nche_log = C.n - 1 - std::min(cl, C.n - 1);
            C.ncht_log = (C.n - C.T) - std::min(C.n - C.T, std::max(0, cl + 1 - C.T));
            C.epart_off = part;
            part += 1 << C.nche_log;
            C.rpart_off = part;
            rt.push_back(make_int2(C.epart_off, 1 << C.nche_log));
            for (int r = 0; r < C.nrot; r++) rt.push_back(make_int2(C.rpart_off + (r << C.ncht_log), 1 << C.ncht_log));
            part += C.nrot << C.ncht_log;
        }
        std::vector<uint32_t> first;
        std::vector<int4> segs;
        uint64_t n = 0;
        build_schedule(b, &first, &segs, &n);
        b->nsegs = int(segs.size());
        b->nitems = uint32_t(n);
        b->chunk_log = cl;
        cudaError_t e2 = cudaMemcpy(b->dcirc, b->hcirc.data(), sizeof(BCirc) * count, cudaMemcpyHostToDevice);
        if (e2 == cudaSuccess && !rt.empty())
            e2 = cudaMemcpy(b->drtab, rt.data(), sizeof(int2) * rt.size(), cudaMemcpyHostToDevice);
        if (e2 == cudaSuccess) e2 = cudaMemcpy(b->dseg_first, first.data(), first.size() * 4, cudaMemcpyHostToDevice);
        if (e2 == cudaSuccess)
            e2 = cudaMemcpy(b->dsegs, segs.data(), segs.size() * sizeof(int4), cudaMemcpyHostToDevice);
        return e2;
    };
    if (!stages.empty())
        e = cudaMemcpy(b->dstages, stages.data(), sizeof(BStage) * stages.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !ops.empty())
        e = cudaMemcpy(b->dops, ops.data(), sizeof(BOp) * ops.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !terms.empty())
        e = cudaMemcpy(b->dterms, terms.data(), sizeof(BPauli) * terms.size(), cudaMemcpyHostToDevice);
    for (int i = 0; i < b->ncs; i++) b->hcs[i] = make_double2(1.0, 0.0);
    // ---- chunk size and persistence: from options, the autotune cache, or by timing candidates
    int max_per_sm = 1;
    if (e == cudaSuccess)
        e = b->prec == QS_PREC_C64
                ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_per_sm, k_batch<float2>, kBT, b->smem)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_per_sm, k_batch<double2>, kBT, b->smem);
    max_per_sm = std::max(1, max_per_sm);
    std::ostringstream key;
    key << "batch2:p" << b->prec << ":a" << (b->arith == QS_ARITH_DF64) << ":c" << count << ":items";
    {
        uint64_t sig = 0;
        for (size_t c = 0; c < count; c++) sig = sig * 1315423911ull + uint64_t(circuits[c].n) * 131 + circuits[c].m;
        key << sig;
    }
    int cl = o.chunk_log2, ct = o.ctas_per_sm;
    if (cl <= 0 || ct <= 0) {
        int ccl = 0, cct = 0;
        if (autotune_cache_lookup(key.str(), &ccl, &cct)) {
            if (cl <= 0) cl = ccl;
            if (ct <= 0) ct = cct;
        }
    }
    if (e == cudaSuccess && (cl <= 0 || ct <= 0)) {
        // autotune by coordinate descent: the chunk size (items of 1, 4 or 16 tiles of 2^11
        // amplitudes) at the most CTAs per SM, then the CTAs per SM at that chunk size. One timed run
        // per candidate, its graph uploaded first; one untimed run before the first (module loading).
        bool warmed = false;
        auto run = [&](int tcl, int tct, double* dt) -> cudaError_t {
            b->ctas = tct;
            cudaError_t r = layout(std::max(kMinChunk, tcl));
            if (r == cudaSuccess) r = capture(b);
            if (r == cudaSuccess) r = cudaGraphUpload(b->exec, b->stream);
            if (r == cudaSuccess && !warmed) {
                r = cudaGraphLaunch(b->exec, b->stream);
                if (r == cudaSuccess) note_launches(3);
                warmed = true;
            }
            if (r == cudaSuccess) r = cudaStreamSynchronize(b->stream);
            if (r != cudaSuccess) return r;
            const auto t0 = std::chrono::steady_clock::now();
            r = cudaGraphLaunch(b->exec, b->stream);
            if (r == cudaSuccess) r = cudaStreamSynchronize(b->stream);
            if (r == cudaSuccess) note_launches(3);
            *dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            return r;
        };
        double best = 1e30;
        int bcl = cl > 0 ? cl : 12, bct = ct > 0 ? ct : max_per_sm;
        const int first_ct = bct;
        const std::vector<int> cls = cl > 0 ? std::vector<int>{cl} : std::vector<int>{10, 12, 14};
        for (int tcl : cls) {
            double dt = 0;
            if ((e = run(tcl, first_ct, &dt)) != cudaSuccess || *b->herr) break;
            if (dt < best) best = dt, bcl = tcl;
        }
        if (e == cudaSuccess && !*b->herr && ct <= 0) {
            for (int tct = 1; tct <= max_per_sm; tct++) {
                if (tct == first_ct) continue;
                double dt = 0;
                if ((e = run(bcl, tct, &dt)) != cudaSuccess || *b->herr) break;
                if (dt < best) best = dt, bct = tct;
            }
        }
        cl = bcl;
        ct = bct;
        if (e == cudaSuccess && !*b->herr) autotune_cache_store(key.str(), cl, ct);
    }
    b->ctas = std::max(1, std::min(ct, max_per_sm));
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
    qs::TraceRange trace("qs_batch_run");
    if (!b || (b->total_params && !params)) {
        set_last_error_message("null argument");
        return QS_INVALID_ARGUMENT;
    }
    for (int i = 0; i < b->ncs; i++) {
        const double th = params[b->cs_param[i]];
        b->hcs[i] = make_double2(std::cos(0.5 * th), std::sin(0.5 * th));
    }
    cudaError_t e = cudaGraphLaunch(b->exec, b->stream);
    if (e == cudaSuccess) note_launches(3);  // the graph's reset, persistent and reduction kernels
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
