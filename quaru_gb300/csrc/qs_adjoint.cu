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
#include "qs_pass.cuh"
#include "qs_rot.cuh"
#include "qs_reduce.cuh"
#include "qs_tile.h"

namespace qs {

constexpr int kAT = 256;

__device__ __forceinline__ double2 ld2(const double2* p, uint64_t i) { return p[i]; }
__device__ __forceinline__ double2 ld2(const float2* p, uint64_t i) {  // integer-pipe conversion
    const float2 v = p[i];
    return make_double2(df_f2d(v.x), df_f2d(v.y));
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
    float ch, cl;  // c as a float pair, c = ch + cl + O(2^-48 |c|)
    uint32_t cls;  // |x & z| mod 4: the term's factor i^cls
    uint32_t pad_;
};

// out_i = sum_t c_t * i^{|x&z|} * (-1)^{|z & (i^x)|} * psi_{i^x}
template <typename T, bool DFC>
__global__ void __launch_bounds__(kAT) k_pauli_sum(const T* __restrict__ psi, T* __restrict__ out, uint64_t N,
                                                   const PauliDev* __restrict__ terms, int nt) {
    static_assert(!DFC || sizeof(T) == 8, "float-pair coefficients serve complex64 states");
    if constexpr (DFC) {
        // complex64: each term's product by TwoProduct on the FP32 pipe, summed with TwoSum (DfAcc), the
        // coefficient's low float folded into the compensation; one rounding to float at the end
        for (uint64_t i = uint64_t(blockIdx.x) * kAT + threadIdx.x; i < N; i += uint64_t(gridDim.x) * kAT) {
            DfAcc re, im;
            for (int t = 0; t < nt; t++) {
                const PauliDev& p = terms[t];
                const uint64_t j = i ^ p.x;
                const float2 v = reinterpret_cast<const float2*>(psi)[j];
                const bool neg = __popcll(p.z & j) & 1;
                const float ch = neg ? -p.ch : p.ch, cl = neg ? -p.cl : p.cl;
                float xr, xi;  // i^cls * v
                switch (p.cls) {
                    case 0: xr = v.x; xi = v.y; break;
                    case 1: xr = -v.y; xi = v.x; break;
                    case 2: xr = -v.x; xi = -v.y; break;
                    default: xr = v.y; xi = -v.x; break;
                }
                re.add_prod(ch, xr);
                re.c = __fmaf_rn(cl, xr, re.c);
                im.add_prod(ch, xi);
                im.c = __fmaf_rn(cl, xi, im.c);
            }
            reinterpret_cast<float2*>(out)[i] = make_float2(__fadd_rn(re.s, re.c), __fadd_rn(im.s, im.c));
        }
    } else {
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

// ---------------------------------------------------------------- tiled reverse sweep
// One stage of the reverse sweep over tiles of 2^T amplitudes: psi and lambda tiles side by side in
// shared memory, the stage's gates taken in reverse order. A rotation adds Im<lambda|A|psi> over the
// tile's pairs to its slot (FP64, per warp, in shared memory) and is un-applied from both tiles; a
// fixed gate (its inverse) is applied to both. Gates were reordered only past gates on disjoint
// qubits, with which they commute, so every inner product equals the one of the gate-by-gate sweep.
constexpr int kAdjT = 11;           // tile qubits of the reverse sweep (largest; see adj_tile_qubits)
constexpr int kAdjThreads = 256;
constexpr int kAdjMaxOps = 32;      // gates per stage: the op table is staged in shared memory
constexpr int kAdjMaxRot = kAdjMaxOps;  // rotations per launch

struct AdjOpDev {
    TileOp t;      // tile-local form (target bit, tuple expansion, controls, matrix of a fixed gate)
    int rot;       // stage-local rotation slot, or -1 for a fixed gate
    int axis;      // QS_GATE_RX / RY / RZ
    double c, s;   // cos(theta/2), -sin(theta/2): the inverse rotation
    float cf, sf;  // the same rounded to float (complex64 tiles)
};

static_assert(sizeof(AdjOpDev) % 16 == 0, "the op table is copied to shared memory in 16-byte words");

struct AdjStageArgs {
    int T, RL, RH;
    int nops, nrot;
    IndexMap outer;
    uint8_t rhigh[kTileMaxHigh];
    int slot[kAdjMaxRot];  // global rotation slot of each stage-local slot
};

template <typename T>
__device__ __forceinline__ void adj_fixed(T* s, const TileOp& op, uint32_t tsize) {
    using R = decltype(T().x);
    const uint32_t ntup = tsize >> op.npos;
    uint32_t seg[5];
#pragma unroll
    for (int j = 0; j < 5; j++) seg[j] = op.seg[j];
    if (op.kind == OP_DENSE || op.kind == OP_DENSE_REAL) {
        const uint32_t tb = op.off[1];
        // complex64 tiles read the host-rounded float copy (no FP64-pipe conversions per thread)
        const auto* mm = [&] {
            if constexpr (sizeof(R) == 4)
                return op.mf;
            else
                return op.m;
        }();
        const R m0 = mm[0], m1 = mm[1], m2 = mm[2], m3 = mm[3], m4 = mm[4], m5 = mm[5], m6 = mm[6], m7 = mm[7];
        for (uint32_t p = threadIdx.x; p < ntup; p += kAdjThreads) {
            const uint32_t i0 = tuple_index(p, op.npos, seg, op.pos, op.lfixval);
            const T a = s[i0], b = s[i0 | tb];
            T y0 = cfma(m2, m3, b, czero<T>());
            y0 = cfma(m0, m1, a, y0);
            T y1 = cfma(m6, m7, b, czero<T>());
            y1 = cfma(m4, m5, a, y1);
            s[i0] = y0;
            s[i0 | tb] = y1;
        }
        return;
    }
    const int D = 1 << op.k;  // monomial: permutation with factors
    for (uint32_t p = threadIdx.x; p < ntup; p += kAdjThreads) {
        const uint32_t i0 = tuple_index(p, op.npos, seg, op.pos, op.lfixval);
        T y[8];
#pragma unroll
        for (int r = 0; r < 8; r++)
            if (r < D && op.pf[r] != PF_SKIP_DEV) y[r] = s[i0 + op.offsrc[r]];
#pragma unroll
        for (int r = 0; r < 8; r++) {
            if (r >= D || op.pf[r] == PF_SKIP_DEV) continue;
            T v = y[r];
            if (op.pf[r] == 255) {
                R pr, pi;
                if constexpr (sizeof(R) == 4)
                    pr = op.mf[2 * r], pi = op.mf[2 * r + 1];
                else
                    pr = op.m[2 * r], pi = op.m[2 * r + 1];
                v = cfma(pr, pi, y[r], czero<T>());
            } else {
                v = apply_pf(y[r], op.pf[r]);
            }
            s[i0 + op.off[r]] = v;
        }
    }
}

// The rotation un-applied from both tiles; returns this thread's share of Im<lambda|A|psi> (complex128:
// an FP64 sum; complex64: a compensated float pair).
template <typename T, int AXIS>
__device__ __forceinline__ auto adj_rot_tile(T* sp, T* sl, const AdjOpDev& op, uint32_t tsize) {
    using R = decltype(T().x);
    const TileOp& t = op.t;
    uint32_t seg[5];
#pragma unroll
    for (int j = 0; j < 5; j++) seg[j] = t.seg[j];
    const uint32_t tb = 1u << t.tb[0];
    R c, sn;
    if constexpr (sizeof(R) == 4)
        c = op.cf, sn = op.sf;
    else
        c = op.c, sn = op.s;
    double acc = 0.0;
    DfAcc facc;
    for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += kAdjThreads) {
        const uint32_t i0 = tuple_index(p, t.npos, seg, t.pos, 0u), i1 = i0 | tb;
        T a = sp[i0], b = sp[i1], l0 = sl[i0], l1 = sl[i1];
        if constexpr (sizeof(R) == 8)
            acc += im_term<AXIS>(l0, l1, a, b);
        else
            im_term_acc<AXIS>(facc, l0, l1, a, b);
        rot_pair<AXIS>(c, sn, a.x, a.y, b.x, b.y);
        rot_pair<AXIS>(c, sn, l0.x, l0.y, l1.x, l1.y);
        sp[i0] = a;
        sp[i1] = b;
        sl[i0] = l0;
        sl[i1] = l1;
    }
    if constexpr (sizeof(R) == 4)
        return facc;
    else
        return acc;
}

template <int AXIS>
__device__ __forceinline__ DfAcc adj_rot_tile_df(float4* sp, float4* sl, const AdjOpDev& op, uint32_t tsize) {
    const TileOp& t = op.t;
    uint32_t seg[5];
#pragma unroll
    for (int j = 0; j < 5; j++) seg[j] = t.seg[j];
    const uint32_t tb = 1u << t.tb[0];
    float ch, cl, sh, sl_;
    df_split(op.c, ch, cl);
    df_split(op.s, sh, sl_);
    DfAcc acc;
    for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += kAdjThreads) {
        const uint32_t i0 = tuple_index(p, t.npos, seg, t.pos, 0u), i1 = i0 | tb;
        float4 a = sp[i0], b = sp[i1], l0 = sl[i0], l1 = sl[i1];
        adj_im_df_acc<AXIS>(acc, l0, l1, a, b);
        df_rot_pair<AXIS>(ch, cl, sh, sl_, a, b);
        df_rot_pair<AXIS>(ch, cl, sh, sl_, l0, l1);
        sp[i0] = a;
        sp[i1] = b;
        sl[i0] = l0;
        sl[i1] = l1;
    }
    return acc;
}

// pure moves (permutations with factors 1, -1, i, -i) on double-float amplitudes
__device__ __forceinline__ float4 df_pf(float4 x, uint8_t c) {
    if (c == 1) return make_float4(-x.x, -x.y, -x.z, -x.w);
    if (c == 2) return make_float4(-x.z, -x.w, x.x, x.y);
    if (c == 3) return make_float4(x.z, x.w, -x.x, -x.y);
    return x;
}

__device__ __forceinline__ void adj_move_df(float4* s, const TileOp& op, uint32_t tsize) {
    const uint32_t ntup = tsize >> op.npos;
    uint32_t seg[5];
#pragma unroll
    for (int j = 0; j < 5; j++) seg[j] = op.seg[j];
    const int D = 1 << op.k;
    for (uint32_t p = threadIdx.x; p < ntup; p += kAdjThreads) {
        const uint32_t i0 = tuple_index(p, op.npos, seg, op.pos, op.lfixval);
        float4 y[8];
#pragma unroll
        for (int r = 0; r < 8; r++)
            if (r < D && op.pf[r] != PF_SKIP_DEV) y[r] = s[i0 + op.offsrc[r]];
#pragma unroll
        for (int r = 0; r < 8; r++)
            if (r < D && op.pf[r] != PF_SKIP_DEV) s[i0 + op.off[r]] = df_pf(y[r], op.pf[r]);
    }
}

template <typename T, bool DF>
__global__ void __launch_bounds__(kAdjThreads) k_adj_stage(T* __restrict__ psi, T* __restrict__ lam, uint64_t ntiles,
                                                           const __grid_constant__ AdjStageArgs a,
                                                           const AdjOpDev* __restrict__ ops,
                                                           double* __restrict__ partials) {
    static_assert(!DF || sizeof(T) == 16, "double-float tiles hold complex128 registers");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t tsize = 1u << a.T;
    T* sp = reinterpret_cast<T*>(smem_raw);
    T* sl = sp + tsize;
    float4* fp = reinterpret_cast<float4*>(sp);  // the same buffers as double-float amplitudes
    float4* fl = reinterpret_cast<float4*>(sl);
    double* sacc = reinterpret_cast<double*>(sl + tsize);  // [nrot][8 warps]
    AdjOpDev* sops = reinterpret_cast<AdjOpDev*>(sacc + size_t(a.nrot) * (kAdjThreads / 32));
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(sops + a.nops);
    const int nrows = 1 << a.RH, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < a.nrot * (kAdjThreads / 32); i += kAdjThreads) sacc[i] = 0.0;
    {  // the launch's op table, read by every thread for every gate of every tile
        const uint4* src = reinterpret_cast<const uint4*>(ops);
        uint4* dst = reinterpret_cast<uint4*>(sops);
        const int words = a.nops * int(sizeof(AdjOpDev) / 16);
        for (int w = threadIdx.x; w < words; w += kAdjThreads) dst[w] = src[w];
    }
    for (int r = threadIdx.x; r < nrows; r += kAdjThreads) {
        uint64_t o = 0;
        for (int b = 0; b < a.RH; b++)
            if (r >> b & 1) o |= 1ull << a.rhigh[b];
        rowoff[r] = o;
    }
    __syncthreads();
    const uint32_t rmask = (1u << a.RL) - 1u;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = expand_index(tile, a.outer);
        for (uint32_t i = threadIdx.x; i < tsize; i += kAdjThreads) {
            const uint64_t g = base + rowoff[i >> a.RL] + (i & rmask);
            if constexpr (DF) {
                const double2 v = reinterpret_cast<const double2*>(psi)[g], w = reinterpret_cast<const double2*>(lam)[g];
                float4 f;
                df_split(v.x, f.x, f.y);
                df_split(v.y, f.z, f.w);
                fp[i] = f;
                df_split(w.x, f.x, f.y);
                df_split(w.y, f.z, f.w);
                fl[i] = f;
            } else {
                sp[i] = psi[g];
                sl[i] = lam[g];
            }
        }
        __syncthreads();
        for (int o = 0; o < a.nops; o++) {
            const AdjOpDev& op = sops[o];
            if ((base & op.t.omask) != op.t.oval) continue;  // the same for the whole block
            if (op.rot >= 0) {
                double v;
                if constexpr (DF) {  // the warp's float pairs reduced on the FP32 pipe, one FP64 rejoin
                    DfAcc f;
                    if (op.axis == QS_GATE_RX)
                        f = adj_rot_tile_df<QS_GATE_RX>(fp, fl, op, tsize);
                    else if (op.axis == QS_GATE_RY)
                        f = adj_rot_tile_df<QS_GATE_RY>(fp, fl, op, tsize);
                    else
                        f = adj_rot_tile_df<QS_GATE_RZ>(fp, fl, op, tsize);
                    f.warp_reduce();
                    v = __dadd_rn(df_f2d(f.s), df_f2d(f.c));
                } else if constexpr (sizeof(T) == 8) {
                    // complex64: the warp's compensated float pairs reduced on the FP32 pipe, one
                    // FP64 rejoin per warp
                    DfAcc f;
                    if (op.axis == QS_GATE_RX)
                        f = adj_rot_tile<T, QS_GATE_RX>(sp, sl, op, tsize);
                    else if (op.axis == QS_GATE_RY)
                        f = adj_rot_tile<T, QS_GATE_RY>(sp, sl, op, tsize);
                    else
                        f = adj_rot_tile<T, QS_GATE_RZ>(sp, sl, op, tsize);
                    f.warp_reduce();
                    v = __dadd_rn(df_f2d(f.s), df_f2d(f.c));
                } else {
                    if (op.axis == QS_GATE_RX)
                        v = adj_rot_tile<T, QS_GATE_RX>(sp, sl, op, tsize);
                    else if (op.axis == QS_GATE_RY)
                        v = adj_rot_tile<T, QS_GATE_RY>(sp, sl, op, tsize);
                    else
                        v = adj_rot_tile<T, QS_GATE_RZ>(sp, sl, op, tsize);
                    v = rd_warp_sum(v);
                }
                if (lane == 0) sacc[op.rot * (kAdjThreads / 32) + warp] += v;
            } else if constexpr (DF) {
                adj_move_df(fp, op.t, tsize);
                adj_move_df(fl, op.t, tsize);
            } else {
                adj_fixed(sp, op.t, tsize);
                adj_fixed(sl, op.t, tsize);
            }
            __syncthreads();
        }
        for (uint32_t i = threadIdx.x; i < tsize; i += kAdjThreads) {
            const uint64_t g = base + rowoff[i >> a.RL] + (i & rmask);
            if constexpr (DF) {
                const float4 f = fp[i], h = fl[i];
                reinterpret_cast<double2*>(psi)[g] =
                    make_double2(__dadd_rn(df_f2d(f.x), df_f2d(f.y)), __dadd_rn(df_f2d(f.z), df_f2d(f.w)));
                reinterpret_cast<double2*>(lam)[g] =
                    make_double2(__dadd_rn(df_f2d(h.x), df_f2d(h.y)), __dadd_rn(df_f2d(h.z), df_f2d(h.w)));
            } else {
                psi[g] = sp[i];
                lam[g] = sl[i];
            }
        }
        __syncthreads();
    }
    for (int r = threadIdx.x; r < a.nrot; r += kAdjThreads) {
        double v = 0.0;
        for (int w = 0; w < kAdjThreads / 32; w++) v += sacc[r * (kAdjThreads / 32) + w];
        partials[size_t(a.slot[r]) * gridDim.x + blockIdx.x] = v;
    }
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
    for (size_t t = 0; t < nt; t++) {
        const double c = terms[t].coeff;
        const float ch = float(c);
        v[t] = {c, terms[t].x_mask, terms[t].z_mask, ch, float(c - double(ch)),
                uint32_t(__builtin_popcountll(terms[t].x_mask & terms[t].z_mask) & 3), 0u};
    }
    return v;
}

// Whether every coefficient lies where its float pair carries it to FP64 accuracy.
static bool pauli_df_ok(const std::vector<PauliDev>& ht) {
    for (const PauliDev& p : ht) {
        const double a = std::fabs(p.c);
        if (a != 0.0 && !(a >= 0x1p-90 && a <= 0x1p90)) return false;
    }
    return true;
}

template <typename T>
static void launch_pauli_sum(const void* psi, void* out, int n, const PauliDev* dterms, int nt, bool df_ok,
                             cudaStream_t s, int sms) {
    const uint64_t N = 1ull << n;
    if (sizeof(T) == 8 && df_ok)
        k_pauli_sum<float2, true><<<grid_for_pairs(N, sms), kAT, 0, s>>>((const float2*)psi, (float2*)out, N, dterms, nt);
    else
        k_pauli_sum<T, false><<<grid_for_pairs(N, sms), kAT, 0, s>>>((const T*)psi, (T*)out, N, dterms, nt);
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
        launch_pauli_sum<float2>(psi, blob + o_lam, n, (const PauliDev*)(blob + o_terms), int(nt), pauli_df_ok(ht),
                                 s, sms);
    else
        launch_pauli_sum<double2>(psi, blob + o_lam, n, (const PauliDev*)(blob + o_terms), int(nt), false, s, sms);
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

// R_A(theta) as a row-major interleaved 2x2 matrix (the convention of rot_pair).
static std::vector<double> rotation_matrix(int axis, double c, double s) {
    if (axis == QS_GATE_RX) return {c, 0, 0, -s, 0, -s, c, 0};
    if (axis == QS_GATE_RY) return {c, 0, -s, 0, s, 0, c, 0};
    return {c, -s, 0, 0, 0, 0, c, s};
}

// Tile qubits for an n-qubit state: `cap` for large states, fewer below n = cap + 7 so that 128
// tiles (blocks) share the work of mid-size states, never fewer than 8 (16 tiles at 12 qubits),
// and the whole state in one tile up to 8 qubits (one block runs every gate without a launch each).
static int adj_tile_qubits(int n, int cap) { return std::min(n, std::max(8, std::min(cap, n - 7))); }

constexpr int kAdjTiledMin = 6;  // from this many qubits the gradient runs as tiled stages

// Grid of the tiled reverse sweep for n qubits in tiles of tq qubits (the same for every stage, so
// partials line up).
template <typename T>
static int adj_grid(int n, int tq, int sms) {
    const size_t smem = 2 * (sizeof(T) << kAdjT) + size_t(kAdjMaxRot) * (kAdjThreads / 32) * 8 +
                        size_t(kAdjMaxOps) * sizeof(AdjOpDev) + (8u << 6);
    int per_sm = 1;  // the smaller of the two variants' occupancies (each variant's limit raised to smem)
    resident_blocks(reinterpret_cast<const void*>(k_adj_stage<T, false>), kAdjThreads, smem, &per_sm);
    if (sizeof(T) == 16) {
        int df = 1;
        resident_blocks(reinterpret_cast<const void*>(k_adj_stage<T, sizeof(T) == 16>), kAdjThreads, smem, &df);
        per_sm = std::min(per_sm, df);
    }
    const uint64_t ntiles = 1ull << (n - tq);
    return int(std::min<uint64_t>(ntiles, uint64_t(sms) * uint64_t(std::max(1, per_sm))));
}

// The reverse sweep as tiled stages: gates m-1 .. 0, rotations with their inner products, fixed
// gates as their inverses (inv, whose entries are moved out). Partials of rotation slot r land in
// part[r * grid .. + grid).
template <typename T>
static int reverse_tiled(void* state, void* lam, int n, int prec, int arith, const qs_param_gate* gates, size_t m,
                         const double* params, const std::vector<int>& rot_slot, std::vector<OpDesc>& inv,
                         double* part, int grid, cudaStream_t s, int sms, std::string* msg) {
    std::vector<OpDesc> rops;
    std::vector<int> src;
    rops.reserve(m);
    src.reserve(m);
    for (size_t gg = m; gg-- > 0;) {
        if (rot_slot[gg] >= 0) {  // planning form: a dense 1-qubit gate on the rotation's target
            OpDesc d;
            d.kind = OP_DENSE;
            d.k = d.orig_k = 1;
            d.tq[0] = int(gates[gg].targets[0]);
            d.m.assign(8, 0.0);
            d.touched_rows = 2;
            rops.push_back(std::move(d));
        } else {
            rops.push_back(std::move(inv[gg]));  // consumed: the caller reads inv no further
        }
        src.push_back(int(gg));
    }
    const int tq = adj_tile_qubits(n, kAdjT);
    const std::vector<TileStage> stages = plan_tiles(rops, n, tq, 5, false, kAdjMaxOps);
    // device tables: every stage's ops (split so a launch holds at most kAdjMaxRot rotations)
    std::vector<AdjOpDev> host;
    struct Launch {
        int stage, first, count, nrot;
        int slot[kAdjMaxRot];
        bool moves_only;  // every fixed gate a pure move (double-float tiles can take the launch)
    };
    std::vector<Launch> launches;
    for (size_t si = 0; si < stages.size(); si++) {
        const TileStage& st = stages[si];
        if (!st.tiled) {
            launches.push_back(Launch{int(si), -1, 0, 0, {}, false});
            continue;
        }
        Launch cur{int(si), int(host.size()), 0, 0, {}, true};
        for (int idx : st.ops) {
            const int g = src[idx];
            if (rot_slot[g] >= 0 && cur.nrot == kAdjMaxRot) {
                launches.push_back(cur);
                cur = Launch{int(si), int(host.size()), 0, 0, {}, true};
            }
            AdjOpDev e;
            std::memset(&e, 0, sizeof(e));
            e.t = make_tile_op(rops[idx], st);
            e.rot = -1;
            if (rot_slot[g] < 0 && rops[idx].kind != OP_MONO_PF) cur.moves_only = false;
            if (rot_slot[g] >= 0) {
                const double th = params[gates[g].param];
                e.rot = cur.nrot;
                cur.slot[cur.nrot++] = rot_slot[g];
                e.axis = gates[g].kind;
                e.c = std::cos(0.5 * th);
                e.s = -std::sin(0.5 * th);
                e.cf = float(e.c);
                e.sf = float(e.s);
            }
            host.push_back(e);
            cur.count++;
        }
        launches.push_back(cur);
    }
    AdjOpDev* dops = nullptr;
    if (!host.empty()) {
        const size_t bytes = host.size() * sizeof(AdjOpDev);
        cudaError_t e = cudaMallocAsync((void**)&dops, bytes, s);
        if (e == cudaSuccess) {  // page-locked: the upload does not wait for the forward pass queued before it
            void* stage = pinned_staging(1, bytes);
            if (stage) std::memcpy(stage, host.data(), bytes);
            e = cudaMemcpyAsync(dops, stage ? stage : host.data(), bytes, cudaMemcpyHostToDevice, s);
        }
        if (e != cudaSuccess) return fail(e, "reverse-sweep tables", msg);
    }
    int rc = QS_OK;
    const uint64_t ntiles = 1ull << (n - tq);
    for (const Launch& L : launches) {
        const TileStage& st = stages[L.stage];
        if (L.first < 0) {  // a gate no tile holds: its inverse on psi and lambda, one sweep each
            const OpDesc& op = rops[st.single];
            if ((rc = apply_op(state, n, prec, arith, op, s, sms, msg)) != QS_OK) break;
            if ((rc = apply_op(lam, n, prec, arith, op, s, sms, msg)) != QS_OK) break;
            continue;
        }
        AdjStageArgs a;
        std::memset(&a, 0, sizeof(a));
        a.T = st.T;
        const int H = int(st.high.size());
        int run = 0;
        while (run < H && st.high[run] == st.L + run) run++;
        a.RL = st.L + run;
        a.RH = H - run;
        for (int b = 0; b < a.RH; b++) a.rhigh[b] = uint8_t(st.high[run + b]);
        std::vector<int> qpos;
        for (int q = 0; q < st.L; q++) qpos.push_back(q);
        for (int q : st.high) qpos.push_back(q);
        std::sort(qpos.begin(), qpos.end());
        a.outer.npos = int(qpos.size());
        for (size_t i = 0; i < qpos.size(); i++) a.outer.pos[i] = uint8_t(qpos[i]);
        a.nops = L.count;
        a.nrot = L.nrot;
        for (int r = 0; r < L.nrot; r++) a.slot[r] = L.slot[r];
        const size_t smem = 2 * (sizeof(T) << st.T) + size_t(a.nrot) * (kAdjThreads / 32) * 8 +
                            size_t(a.nops) * sizeof(AdjOpDev) + (8u << a.RH);
        if (sizeof(T) == 16 && L.moves_only && arith == QS_ARITH_DF64)
            k_adj_stage<T, sizeof(T) == 16><<<grid, kAdjThreads, smem, s>>>((T*)state, (T*)lam, ntiles, a,
                                                                           dops + L.first, part);
        else
            k_adj_stage<T, false><<<grid, kAdjThreads, smem, s>>>((T*)state, (T*)lam, ntiles, a, dops + L.first,
                                                                  part);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            rc = fail(e, "reverse-sweep stage", msg);
            break;
        }
        note_launches(1);
    }
    if (dops) cudaFreeAsync(dops, s);
    return rc;
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
    const bool tiled = n >= kAdjTiledMin;  // forward as fused stages, reverse sweep as tiled stages
    const int tq = adj_tile_qubits(n, kAdjT);
    const int pgrid = tiled ? (prec == QS_PREC_C64 ? adj_grid<float2>(n, tq, sms) : adj_grid<double2>(n, tq, sms))
                            : grid_for_pairs(N >> 1, sms);
    auto al = [](size_t x) { return ((x + 255) / 256) * 256; };
    const size_t o_cs = 0, o_terms = o_cs + al(cs.size() * 16), o_part = o_terms + al(nt * sizeof(PauliDev) + 1),
                 o_res = o_part + al(size_t(std::max(nrot, 1)) * pgrid * 8 + 4096 * 16),
                 o_err = o_res + al((2 + size_t(nrot)) * 8), o_lam = o_err + al(sizeof(int)),
                 o_save = o_lam + al(N * amp), total = o_save + N * amp;
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
        int* derr = reinterpret_cast<int*>(blob + o_err);  // raised by a forward tile kernel's bounded wait
        AJ_CHECK(cudaMemsetAsync(derr, 0, sizeof(int), s), "status flag");
        int herr = 0;
        // forward
        if (tiled) {
            std::vector<OpDesc> fops(m);
            std::vector<double> rmat(8 * m);  // the rotations' matrices, in gate order
            for (size_t g = 0; g < m; g++) {
                if (rot_slot[g] >= 0) {
                    const std::vector<double> R = rotation_matrix(gates[g].kind, cs[g].x, cs[g].y);
                    std::copy(R.begin(), R.end(), rmat.begin() + 8 * g);
                    classify_gate(R.data(), 1, gates[g].targets, &fops[g]);
                } else {
                    fops[g] = std::move(fwd[g]);  // the tiled path reads fwd no further
                }
            }
            if (prec == QS_PREC_C128 && arith == QS_ARITH_DF64 && n >= 18) {
                // double-float dense blocks (3 qubits, the automatic width): the fastest complex128
                // double-float form of a circuit of 1-qubit rotations and CNOTs at 11-qubit tiles (1.85x
                // the stages at 20 qubits; below 18 qubits the smaller stage tiles win); the blocks are
                // products of the gates' FP64 matrices
                std::vector<qs_gate> qg(m);
                for (size_t g = 0; g < m; g++)
                    qg[g] = rot_slot[g] >= 0 ? qs_gate{1, gates[g].targets, rmat.data() + 8 * g}
                                             : qs_gate{gates[g].k, gates[g].targets, gates[g].matrix};
                const qs_circuit_options fo{2, 0, 0, 0};
                if ((rc = run_circuit(state, n, prec, arith, fops, qg.data(), fo, s, sms, msg, derr)) != QS_OK)
                    goto done;
            } else {
                // tiles as in the reverse sweep: below 18 (complex128) or 19 (complex64) qubits smaller
                // than the default so that smaller states still spread over many blocks
                const qs_circuit_options fo{1, 5, adj_tile_qubits(n, prec == QS_PREC_C64 ? 12 : 11), 0};
                // queued without waiting: the reverse sweep is planned while the forward runs
                if ((rc = run_circuit(state, n, prec, arith, fops, nullptr, fo, s, sms, msg, derr)) != QS_OK)
                    goto done;
            }
        }
        for (size_t g = 0; g < m && !tiled; g++) {
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
            launch_pauli_sum<float2>(state, lam, n, (const PauliDev*)(blob + o_terms), int(nt), pauli_df_ok(ht), s,
                                     sms);
        else
            launch_pauli_sum<double2>(state, lam, n, (const PauliDev*)(blob + o_terms), int(nt), false, s, sms);
        AJ_CHECK(cudaGetLastError(), "pauli sum");
        if (inner_product(state, prec, lam, prec, n, s, sms, part + size_t(std::max(nrot, 1)) * pgrid, dres))
            AJ_CHECK(cudaGetLastError(), "energy");
        // reverse
        if (tiled) {
            rc = prec == QS_PREC_C64
                     ? reverse_tiled<float2>(state, lam, n, prec, arith, gates, m, params, rot_slot, inv, part, pgrid,
                                             s, sms, msg)
                     : reverse_tiled<double2>(state, lam, n, prec, arith, gates, m, params, rot_slot, inv, part,
                                              pgrid, s, sms, msg);
            if (rc != QS_OK) goto done;
        }
        for (size_t gg = m; gg-- > 0 && !tiled;) {
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
        AJ_CHECK(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s), "status readback");
        AJ_CHECK(cudaMemcpyAsync(state, blob + o_save, N * amp, cudaMemcpyDeviceToDevice, s), "restore state");
        AJ_CHECK(cudaStreamSynchronize(s), "adjoint sync");
        if (herr) {
            *msg = "a tile kernel's bounded wait for its bulk copies gave up";
            rc = QS_TIMEOUT;
            goto done;
        }
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
