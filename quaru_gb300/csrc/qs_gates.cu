// qs_gates.cu — gate-application kernels (one sweep per gate).
//
// Replaces the hot loop of Register::try_apply_fast (src/register.rs:155-189):
// the reference clones the state, filters all 2^n indices for "target bits
// zero" and, per base index, gathers 2^k amplitudes, runs a dense mat-vec and
// scatters the result. Here one thread owns one tuple of amplitudes, reads
// every amplitude it will rewrite before writing any (so the update can be in
// place), and only rows the gate changes are read or written.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qs_device.cuh"
#include "qs_kernels.h"

namespace qs {

static inline cudaError_t counted(cudaError_t e, uint64_t launches = 1) {
    if (e == cudaSuccess) note_launches(launches);
    return e;
}

constexpr int kThreads = 256;

// ---------------------------------------------------------------- 1-qubit dense
template <typename R>
struct Dense1Args {
    IndexMap map;
    uint64_t tbit;  // 1 << target
    R m[8];         // u00, u01, u10, u11 interleaved
    // QS_ARITH_DF64: per output (y0.re, y0.im, y1.re, y1.im) four coefficients
    // (sign folded in) as float pairs, applied to the inputs listed in kDfIn.
    float dfh[16];
    float dfl[16];
};

// DF64 term t of output o multiplies input component (x0.re, x0.im, x1.re,
// x1.im = 0..3) number t for real outputs and t ^ 1 for imaginary outputs.

// MODE 0: exact complex, 1: exact real, 2: FMA complex, 3: FMA real,
// 4: double-float complex, 5: double-float real (4-5: complex128 only).
template <typename R, int MODE, int ILP>
__global__ void __launch_bounds__(kThreads) k_dense1(typename Cplx<R>::T* __restrict__ st, uint64_t ntup,
                                                     const __grid_constant__ Dense1Args<R> a) {
    using T = typename Cplx<R>::T;
    const uint64_t stride = uint64_t(gridDim.x) * kThreads * ILP;
    for (uint64_t t0 = uint64_t(blockIdx.x) * kThreads * ILP + threadIdx.x; t0 < ntup; t0 += stride) {
        uint64_t i0[ILP];
        T x0[ILP], x1[ILP];
#pragma unroll
        for (int u = 0; u < ILP; u++) {
            const uint64_t t = t0 + uint64_t(u) * kThreads;
            i0[u] = (t < ntup) ? expand_index(t, a.map) : ~0ull;
            if (t < ntup) {
                x0[u] = st[i0[u]];
                x1[u] = st[i0[u] | a.tbit];
            }
        }
#pragma unroll
        for (int u = 0; u < ILP; u++) {
            if (i0[u] == ~0ull) continue;
            T y0, y1;
            if constexpr (MODE == 0) {
                y0 = cadd_exact(cmul_exact(a.m[0], a.m[1], x0[u]), cmul_exact(a.m[2], a.m[3], x1[u]));
                y1 = cadd_exact(cmul_exact(a.m[4], a.m[5], x0[u]), cmul_exact(a.m[6], a.m[7], x1[u]));
            } else if constexpr (MODE == 1) {
                y0 = cadd_exact(cmul_exact_real(a.m[0], x0[u]), cmul_exact_real(a.m[2], x1[u]));
                y1 = cadd_exact(cmul_exact_real(a.m[4], x0[u]), cmul_exact_real(a.m[6], x1[u]));
            } else if constexpr (MODE == 4 || MODE == 5) {
                float xh[4], xl[4];
                df_split(x0[u].x, xh[0], xl[0]);
                df_split(x0[u].y, xh[1], xl[1]);
                df_split(x1[u].x, xh[2], xl[2]);
                df_split(x1[u].y, xh[3], xl[3]);
                double out[4];
#pragma unroll
                for (int o = 0; o < 4; o++) {
                    if constexpr (MODE == 4) {
                        float th[4], tl[4];
#pragma unroll
                        for (int t = 0; t < 4; t++) {
                            th[t] = xh[(o & 1) ? (t ^ 1) : t];
                            tl[t] = xl[(o & 1) ? (t ^ 1) : t];
                        }
                        out[o] = df_dot<4>(a.dfh + 4 * o, a.dfl + 4 * o, th, tl);
                    } else {
                        // real matrix: y.re uses x.re terms 0 and 2, y.im uses x.im terms
                        const float th[2] = {xh[(o & 1)], xh[2 + (o & 1)]};
                        const float tl[2] = {xl[(o & 1)], xl[2 + (o & 1)]};
                        const float ch[2] = {a.dfh[4 * o], a.dfh[4 * o + 2]};  // u.re of columns 0 and 1
                        const float cl[2] = {a.dfl[4 * o], a.dfl[4 * o + 2]};
                        out[o] = df_dot<2>(ch, cl, th, tl);
                    }
                }
                y0.x = out[0];
                y0.y = out[1];
                y1.x = out[2];
                y1.y = out[3];
            } else if constexpr (MODE == 2) {
                y0 = cfma(a.m[2], a.m[3], x1[u], czero<T>());
                y0 = cfma(a.m[0], a.m[1], x0[u], y0);
                y1 = cfma(a.m[6], a.m[7], x1[u], czero<T>());
                y1 = cfma(a.m[4], a.m[5], x0[u], y1);
            } else {
                y0.x = a.m[0] * x0[u].x;
                y0.y = a.m[0] * x0[u].y;
                y0 = cfma_real(a.m[2], x1[u], y0);
                y1.x = a.m[4] * x0[u].x;
                y1.y = a.m[4] * x0[u].y;
                y1 = cfma_real(a.m[6], x1[u], y1);
            }
            st[i0[u]] = y0;
            st[i0[u] | a.tbit] = y1;
        }
    }
}

// ---------------------------------------------------------------- 1-qubit dense, fixed point
// QS_ARITH_FX64 (see fx_encode in qs_device.cuh): each output component of a pair is an integer dot
// product rounded once to double. Outputs o = (y0.re, y0.im, y1.re, y1.im), terms t over
// (x0.re, x0.im, x1.re, x1.im); a real matrix uses terms (o & 1) and 2 + (o & 1) only.
struct Dense1FxArgs {
    IndexMap map;       // tuple expansion (gates with fixed bits)
    uint64_t tbit;      // 1 << target
    int32_t fxh[16];    // row o, term t: 30-bit limbs of C = RN(c * 2^(60 - ec))
    int32_t fxl[16];
    int32_t fxk[4];     // ec - 1082 per output
    int32_t fxkk[4];    // (ec - 1082) << 20
    int32_t kmin, kmax; // range of fxk over the outputs
    double m[8];        // the matrix, for tuples with infinite or NaN components (FP64 FMA)
};

// Every tuple the fast path does not take: infinite or NaN components (FP64 FMA propagates them),
// components all below 2^-958, or output exponents near the ends of the double range.
template <bool REAL>
__device__ __noinline__ void fx_pair_slow(double2 x0, double2 x1, const Dense1FxArgs& a, double2* y0, double2* y1) {
    const double v[4] = {x0.x, x0.y, x1.x, x1.y};
    const uint32_t E = max(max(fx_efield(v[0]), fx_efield(v[1])), max(fx_efield(v[2]), fx_efield(v[3])));
    if (E == 0x7ffu) {
        *y0 = cfma(a.m[0], a.m[1], x0, cfma(a.m[2], a.m[3], x1, czero<double2>()));
        *y1 = cfma(a.m[4], a.m[5], x0, cfma(a.m[6], a.m[7], x1, czero<double2>()));
        return;
    }
    int32_t vh[4], vl[4];
    for (int t = 0; t < 4; t++) {
        if (E >= kFxMinE)
            fx_encode(v[t], E, vh[t], vl[t]);
        else
            fx_encode_small(v[t], E, vh[t], vl[t]);
    }
    double out[4];
    for (int o = 0; o < 4; o++) {
        if (REAL) {
            const int32_t th[2] = {vh[o & 1], vh[2 + (o & 1)]}, tl[2] = {vl[o & 1], vl[2 + (o & 1)]};
            const int32_t ch[2] = {a.fxh[4 * o + (o & 1)], a.fxh[4 * o + 2 + (o & 1)]};
            const int32_t cl[2] = {a.fxl[4 * o + (o & 1)], a.fxl[4 * o + 2 + (o & 1)]};
            out[o] = fx_dot<2>(th, tl, ch, cl, E, a.fxk[o]);
        } else {
            out[o] = fx_dot<4>(vh, vl, a.fxh + 4 * o, a.fxl + 4 * o, E, a.fxk[o]);
        }
    }
    *y0 = make_double2(out[0], out[1]);
    *y1 = make_double2(out[2], out[3]);
}

// PLAIN: the gate has no fixed bits, so a tuple index expands by one inserted bit.
template <bool REAL, bool PLAIN>
__global__ void __launch_bounds__(kThreads, 6) k_dense1_fx(double2* __restrict__ st, uint64_t ntup,
                                                        const __grid_constant__ Dense1FxArgs a) {
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    const uint64_t lo_mask = a.tbit - 1ull;
    for (uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x; t < ntup; t += stride) {
        const uint64_t i0 = PLAIN ? (((t & ~lo_mask) << 1) | (t & lo_mask)) : expand_index(t, a.map);
        const double2 x0 = st[i0], x1 = st[i0 | a.tbit];
        double2 y0, y1;
        const uint32_t E = max(max(fx_efield(x0.x), fx_efield(x0.y)), max(fx_efield(x1.x), fx_efield(x1.y)));
        if (E == 0u) {  // zeros and subnormals only; all four zero: every output is +0, as R = 0 gives
            const uint32_t his = uint32_t(__double2hiint(x0.x) | __double2hiint(x0.y) | __double2hiint(x1.x) |
                                          __double2hiint(x1.y)) & 0x7fffffffu;
            const uint32_t los = uint32_t(__double2loint(x0.x) | __double2loint(x0.y) | __double2loint(x1.x) |
                                          __double2loint(x1.y));
            if ((his | los) == 0u) {
                st[i0] = make_double2(0.0, 0.0);
                st[i0 | a.tbit] = make_double2(0.0, 0.0);
                continue;
            }
        }
        if (E >= kFxMinE && E < 0x7ffu && int(E) + a.kmin >= kFxFastKMin && int(E) + a.kmax <= kFxFastKMax) {
            int32_t vh[4], vl[4];
            fx_encode(x0.x, E, vh[0], vl[0]);
            fx_encode(x0.y, E, vh[1], vl[1]);
            fx_encode(x1.x, E, vh[2], vl[2]);
            fx_encode(x1.y, E, vh[3], vl[3]);
            const int ek = int(E << 20);
            double out[4];
#pragma unroll
            for (int o = 0; o < 4; o++) {
                long long R;
                if constexpr (REAL) {
                    const int32_t th[2] = {vh[o & 1], vh[2 + (o & 1)]}, tl[2] = {vl[o & 1], vl[2 + (o & 1)]};
                    const int32_t ch[2] = {a.fxh[4 * o + (o & 1)], a.fxh[4 * o + 2 + (o & 1)]};
                    const int32_t cl[2] = {a.fxl[4 * o + (o & 1)], a.fxl[4 * o + 2 + (o & 1)]};
                    R = fx_row_sum<2>(th, tl, ch, cl);
                } else {
                    R = fx_row_sum<4>(vh, vl, a.fxh + 4 * o, a.fxl + 4 * o);
                }
                out[o] = fx_to_double_fast(R, int(uint32_t(ek) + uint32_t(a.fxkk[o])));
            }
            y0 = make_double2(out[0], out[1]);
            y1 = make_double2(out[2], out[3]);
        } else {
            fx_pair_slow<REAL>(x0, x1, a, &y0, &y1);
        }
        st[i0] = y0;
        st[i0 | a.tbit] = y1;
    }
}

// ---------------------------------------------------------------- k-qubit dense (2..5)
template <typename R, int K>
struct DenseKArgs {
    IndexMap map;
    uint64_t off[1 << K];    // amplitude offset of sub-index j
    int8_t lane[1 << K];     // exact order: ndarray partial-sum lane, -1 = sequential
    R m[2 * (1 << K) * (1 << K)];
};

template <typename T>
__device__ __forceinline__ void lane_add(T (&p)[8], int lane, T v) {
    switch (lane) {
        case 1: p[1] = cadd_exact(p[1], v); break;
        case 2: p[2] = cadd_exact(p[2], v); break;
        case 3: p[3] = cadd_exact(p[3], v); break;
        case 4: p[4] = cadd_exact(p[4], v); break;
        case 5: p[5] = cadd_exact(p[5], v); break;
        case 6: p[6] = cadd_exact(p[6], v); break;
        case 7: p[7] = cadd_exact(p[7], v); break;
        default: p[0] = cadd_exact(p[0], v); break;
    }
}

// MODE 0: exact complex, 1: exact real, 2: FMA complex, 3: FMA real.
template <typename R, int K, int MODE>
__global__ void __launch_bounds__(kThreads) k_denseK(typename Cplx<R>::T* __restrict__ st, uint64_t ntup,
                                                     const __grid_constant__ DenseKArgs<R, K> a) {
    using T = typename Cplx<R>::T;
    constexpr int D = 1 << K;
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    for (uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x; t < ntup; t += stride) {
        const uint64_t base = expand_index(t, a.map);
        T x[D];
#pragma unroll
        for (int c = 0; c < D; c++) x[c] = st[base + a.off[c]];
#pragma unroll 1
        for (int r = 0; r < D; r++) {
            const R* row = a.m + 2 * r * D;
            T y;
            if constexpr (MODE <= 1) {
                // ndarray unrolled_dot: 8 partial sums, combined as
                // (((0 + (p0+p4)) + (p1+p5)) + (p2+p6)) + (p3+p7); sequential when len < 8.
                T p[8];
#pragma unroll
                for (int j = 0; j < 8; j++) p[j] = czero<T>();
#pragma unroll
                for (int c = 0; c < D; c++) {
                    T term = (MODE == 0) ? cmul_exact(row[2 * c], row[2 * c + 1], x[c])
                                         : cmul_exact_real(row[2 * c], x[c]);
                    lane_add(p, a.lane[c], term);
                }
                if (a.lane[0] < 0) {
                    y = p[0];
                } else {
                    y = cadd_exact(czero<T>(), cadd_exact(p[0], p[4]));
                    y = cadd_exact(y, cadd_exact(p[1], p[5]));
                    y = cadd_exact(y, cadd_exact(p[2], p[6]));
                    y = cadd_exact(y, cadd_exact(p[3], p[7]));
                }
            } else {
                y = czero<T>();
#pragma unroll
                for (int c = 0; c < D; c++) {
                    if constexpr (MODE == 2)
                        y = cfma(row[2 * c], row[2 * c + 1], x[c], y);
                    else
                        y = cfma_real(row[2 * c], x[c], y);
                }
            }
            st[base + a.off[r]] = y;
        }
    }
}

// ---------------------------------------------------------------- monomial (0..5)
template <typename R, int K>
struct MonoArgs {
    IndexMap map;
    uint64_t off[1 << K];      // destination offset of sub-row r
    uint64_t off_src[1 << K];  // offset of its source, off[perm[r]]
    uint8_t pf[1 << K];        // PfClass (PF_SKIP rows untouched); 255 = general phase
    R ph[2 * (1 << K)];        // general phases
};

template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_mono(typename Cplx<R>::T* __restrict__ st, uint64_t ntup,
                                                   const __grid_constant__ MonoArgs<R, K> a) {
    using T = typename Cplx<R>::T;
    constexpr int D = 1 << K;
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    for (uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x; t < ntup; t += stride) {
        const uint64_t base = expand_index(t, a.map);
        T y[D];
#pragma unroll
        for (int r = 0; r < D; r++)
            if (a.pf[r] != PF_SKIP_DEV) y[r] = st[base + a.off_src[r]];
#pragma unroll
        for (int r = 0; r < D; r++) {
            const uint8_t cls = a.pf[r];
            if (cls == PF_SKIP_DEV) continue;
            T v;
            if (cls == 255) {
                if constexpr (sizeof(R) == 8) {
                    v = cmul_exact(a.ph[2 * r], a.ph[2 * r + 1], y[r]);
                } else {
                    v.x = a.ph[2 * r] * y[r].x - a.ph[2 * r + 1] * y[r].y;
                    v.y = a.ph[2 * r] * y[r].y + a.ph[2 * r + 1] * y[r].x;
                }
            } else {
                v = apply_pf(y[r], cls);
            }
            st[base + a.off[r]] = v;
        }
    }
}

// ---------------------------------------------------------------- large sub-operations
// Out of place: src is a copy of the state taken before the gate.
template <typename R, bool EXACT>
__global__ void __launch_bounds__(kThreads) k_dense_big(typename Cplx<R>::T* __restrict__ st,
                                                        const typename Cplx<R>::T* __restrict__ src,
                                                        uint64_t ntup, int k, IndexMap map,
                                                        const uint64_t* __restrict__ off,
                                                        const int8_t* __restrict__ lane,
                                                        const R* __restrict__ m) {
    using T = typename Cplx<R>::T;
    const uint64_t D = 1ull << k;
    const uint64_t total = ntup * D;
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    for (uint64_t w = uint64_t(blockIdx.x) * kThreads + threadIdx.x; w < total; w += stride) {
        const uint64_t t = w >> k, r = w & (D - 1);
        const uint64_t base = expand_index(t, map);
        const R* row = m + 2 * r * D;
        T y;
        if constexpr (EXACT) {
            T p[8];
#pragma unroll
            for (int j = 0; j < 8; j++) p[j] = czero<T>();
            for (uint64_t c = 0; c < D; c++) {
                T term = cmul_exact(row[2 * c], row[2 * c + 1], src[base + off[c]]);
                lane_add(p, lane[c], term);
            }
            if (lane[0] < 0) {
                y = p[0];
            } else {
                y = cadd_exact(czero<T>(), cadd_exact(p[0], p[4]));
                y = cadd_exact(y, cadd_exact(p[1], p[5]));
                y = cadd_exact(y, cadd_exact(p[2], p[6]));
                y = cadd_exact(y, cadd_exact(p[3], p[7]));
            }
        } else {
            y = czero<T>();
            for (uint64_t c = 0; c < D; c++) y = cfma(row[2 * c], row[2 * c + 1], src[base + off[c]], y);
        }
        st[base + off[r]] = y;
    }
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_mono_big(typename Cplx<R>::T* __restrict__ st,
                                                       const typename Cplx<R>::T* __restrict__ src,
                                                       uint64_t ntup, int k, IndexMap map,
                                                       const uint64_t* __restrict__ off,
                                                       const uint64_t* __restrict__ off_src,
                                                       const uint8_t* __restrict__ pf, const R* __restrict__ ph) {
    using T = typename Cplx<R>::T;
    const uint64_t D = 1ull << k;
    const uint64_t total = ntup * D;
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    for (uint64_t w = uint64_t(blockIdx.x) * kThreads + threadIdx.x; w < total; w += stride) {
        const uint64_t t = w >> k, r = w & (D - 1);
        const uint8_t cls = pf[r];
        if (cls == PF_SKIP_DEV) continue;
        const uint64_t base = expand_index(t, map);
        T x = src[base + off_src[r]];
        T v;
        if (cls == 255) {
            if constexpr (sizeof(R) == 8) {
                v = cmul_exact(ph[2 * r], ph[2 * r + 1], x);
            } else {
                v.x = ph[2 * r] * x.x - ph[2 * r + 1] * x.y;
                v.y = ph[2 * r] * x.y + ph[2 * r + 1] * x.x;
            }
        } else {
            v = apply_pf(x, cls);
        }
        st[base + off[r]] = v;
    }
}

// ---------------------------------------------------------------- host launchers
static IndexMap make_map(const OpDesc& op) {
    IndexMap m;
    std::memset(&m, 0, sizeof(m));
    std::vector<int> pos;
    for (int j = 0; j < op.k; j++) pos.push_back(op.tq[j]);
    for (int b = 0; b < 64; b++)
        if (op.fixmask >> b & 1ull) pos.push_back(b);
    std::sort(pos.begin(), pos.end());
    m.npos = int(pos.size());
    for (size_t i = 0; i < pos.size(); i++) m.pos[i] = uint8_t(pos[i]);
    m.fixval = op.fixval;
    return m;
}

static uint64_t sub_offset(const OpDesc& op, uint64_t j) {
    uint64_t o = 0;
    for (int b = 0; b < op.k; b++)
        if (j >> b & 1ull) o |= 1ull << op.tq[b];
    return o;
}

static int grid_for(uint64_t work, int num_sms, int per_thread = 1) {
    uint64_t blocks = (work + uint64_t(kThreads) * per_thread - 1) / (uint64_t(kThreads) * per_thread);
    uint64_t cap = uint64_t(num_sms) * 64;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return int(blocks);
}

// Split the 2x2 matrix into the float-pair coefficients of the DF64 modes.
// Returns false when an entry is outside the range double-float handles.
template <typename R>
static bool fill_df64(Dense1Args<R>& a) {
    // coefficient of term t of output o: (row, column, part, sign); inputs follow kDfIn
    const int row[4] = {0, 0, 1, 1};
    for (int o = 0; o < 4; o++) {
        const bool im_out = o & 1;
        for (int t = 0; t < 4; t++) {
            const int col = t >> 1;           // terms 0,1 -> x0 ; 2,3 -> x1
            const bool cross = (t & 1) != 0;  // term uses the other component of x
            // re out: u.re * x.re (t even), -u.im * x.im (t odd)
            // im out: u.re * x.im (t even),  u.im * x.re (t odd)
            double v;
            const int idx = 2 * (row[o] * 2 + col);
            if (!cross)
                v = double(a.m[idx]);
            else
                v = im_out ? double(a.m[idx + 1]) : -double(a.m[idx + 1]);
            const double av = v < 0 ? -v : v;
            if (av != 0.0 && (av > 0x1p100 || av < 0x1p-100)) return false;
            const float h = float(v);
            a.dfh[4 * o + t] = h;
            a.dfl[4 * o + t] = float(v - double(h));
        }
    }
    return true;
}

// Fixed-point coefficients of one output row (QS_ARITH_FX64): C_t = RN(c_t * 2^(60 - ec)) split into
// 30-bit limbs, ec the frexp exponent of the row's largest |c_t|; k0 = ec - 1082. False for
// non-finite entries (the FP64 kernel runs instead).
static bool fx_row(const double* c, int nt, int32_t* h, int32_t* l, int32_t* k0) {
    double cmax = 0.0;
    for (int t = 0; t < nt; t++) {
        if (!std::isfinite(c[t])) return false;
        cmax = std::max(cmax, std::fabs(c[t]));
    }
    int ec = 0;
    if (cmax > 0.0) std::frexp(cmax, &ec);
    for (int t = 0; t < nt; t++) {
        const long long C = std::llrint(std::ldexp(c[t], 60 - ec));  // |C| < 2^60
        const long long lo = (long long)((unsigned long long)C << 34) >> 34;  // low 30 bits, balanced
        h[t] = int32_t((C - lo) >> 30);
        l[t] = int32_t(lo);
    }
    *k0 = ec - 1082;
    return true;
}

// The coefficients of k_dense1_fx: output o = (y0.re, y0.im, y1.re, y1.im), term t over
// (x0.re, x0.im, x1.re, x1.im). False for non-finite entries (the FP64 kernel runs instead).
static bool fill_fx(const OpDesc& op, Dense1FxArgs& a) {
    for (int i = 0; i < 8; i++) a.m[i] = op.m[i];
    a.kmin = 1 << 30;
    a.kmax = -(1 << 30);
    for (int o = 0; o < 4; o++) {
        const int row = o >> 1;
        const double ar = op.m[4 * row], ai = op.m[4 * row + 1];      // u[row][0]
        const double br = op.m[4 * row + 2], bi = op.m[4 * row + 3];  // u[row][1]
        double c[4];
        if ((o & 1) == 0) {  // re = ar x0r - ai x0i + br x1r - bi x1i
            c[0] = ar; c[1] = -ai; c[2] = br; c[3] = -bi;
        } else {             // im = ai x0r + ar x0i + bi x1r + br x1i
            c[0] = ai; c[1] = ar; c[2] = bi; c[3] = br;
        }
        if (!fx_row(c, 4, a.fxh + 4 * o, a.fxl + 4 * o, a.fxk + o)) return false;
        a.fxkk[o] = int32_t(uint32_t(a.fxk[o]) << 20);
        a.kmin = std::min(a.kmin, a.fxk[o]);
        a.kmax = std::max(a.kmax, a.fxk[o]);
    }
    return true;
}

template <typename R>
static cudaError_t launch_dense1(const OpDesc& op, void* state, int n, bool exact, cudaStream_t s, int sms,
                                 bool df64 = false, bool fx64 = false) {
    using T = typename Cplx<R>::T;
    Dense1Args<R> a;
    std::memset(&a, 0, sizeof(a));
    a.map = make_map(op);
    a.tbit = 1ull << op.tq[0];
    for (int i = 0; i < 8; i++) a.m[i] = R(op.m[i]);
    const uint64_t ntup = 1ull << (n - 1 - __builtin_popcountll(op.fixmask));
    const bool real = op.kind == OP_DENSE_REAL;
    constexpr int ILP = sizeof(R) == 8 ? 2 : 4;
    const int grid = grid_for(ntup, sms, ILP);
    T* st = static_cast<T*>(state);
    if constexpr (sizeof(R) == 8) {
        if (exact) {
            if (real)
                k_dense1<R, 1, ILP><<<grid, kThreads, 0, s>>>(st, ntup, a);
            else
                k_dense1<R, 0, ILP><<<grid, kThreads, 0, s>>>(st, ntup, a);
            return counted(cudaGetLastError());
        }
        if (fx64) {
            Dense1FxArgs f;
            std::memset(&f, 0, sizeof(f));
            if (fill_fx(op, f)) {
                f.map = a.map;
                f.tbit = a.tbit;
                // one pair per thread: the integer form needs few registers, so 64 warps fit per SM
                const int g1 = grid_for(ntup, sms, 1);
                double2* sd = reinterpret_cast<double2*>(state);
                const bool plain = op.fixmask == 0;
                if (real && plain)
                    k_dense1_fx<true, true><<<g1, kThreads, 0, s>>>(sd, ntup, f);
                else if (real)
                    k_dense1_fx<true, false><<<g1, kThreads, 0, s>>>(sd, ntup, f);
                else if (plain)
                    k_dense1_fx<false, true><<<g1, kThreads, 0, s>>>(sd, ntup, f);
                else
                    k_dense1_fx<false, false><<<g1, kThreads, 0, s>>>(sd, ntup, f);
                return counted(cudaGetLastError());
            }
        }
        if (df64 && fill_df64(a)) {
            if (real)
                k_dense1<R, 5, 1><<<grid_for(ntup, sms, 1), kThreads, 0, s>>>(st, ntup, a);
            else
                k_dense1<R, 4, 1><<<grid_for(ntup, sms, 1), kThreads, 0, s>>>(st, ntup, a);
            return counted(cudaGetLastError());
        }
    }
    if (real)
        k_dense1<R, 3, ILP><<<grid, kThreads, 0, s>>>(st, ntup, a);
    else
        k_dense1<R, 2, ILP><<<grid, kThreads, 0, s>>>(st, ntup, a);
    return counted(cudaGetLastError());
}

// Dense k-qubit gate (k = 2, 3) on complex128 state in double-float arithmetic (QS_ARITH_DF64):
// each output component is one double-float dot product over the 2^(k+1) real terms of its row,
// rounded once to FP64 (df_dot). The amplitudes are split into float pairs with integer operations.
template <int K>
struct DenseKDfArgs {
    IndexMap map;
    uint64_t off[1 << K];
    float reh[1 << K][2 << K], rel[1 << K][2 << K];  // row r, real part: terms over (x.re[0..D), x.im[0..D))
    float imh[1 << K][2 << K], iml[1 << K][2 << K];  // row r, imaginary part: terms over (x.im[0..D), x.re[0..D))
};

template <int K>
__global__ void __launch_bounds__(kThreads) k_denseK_df(double2* __restrict__ st, uint64_t ntup,
                                                        const __grid_constant__ DenseKDfArgs<K> a) {
    constexpr int D = 1 << K;
    const uint64_t stride = uint64_t(gridDim.x) * kThreads;
    for (uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x; t < ntup; t += stride) {
        const uint64_t base = expand_index(t, a.map);
        float xh[2 * D], xl[2 * D], ph[2 * D], pl[2 * D];  // (re, im) and (im, re) orders
#pragma unroll
        for (int c = 0; c < D; c++) {
            const double2 v = st[base + a.off[c]];
            df_split(v.x, xh[c], xl[c]);
            df_split(v.y, xh[D + c], xl[D + c]);
            ph[c] = xh[D + c];
            pl[c] = xl[D + c];
            ph[D + c] = xh[c];
            pl[D + c] = xl[c];
        }
#pragma unroll 1
        for (int r = 0; r < D; r++) {
            const double re = df_dot<2 * D>(a.reh[r], a.rel[r], xh, xl);
            const double im = df_dot<2 * D>(a.imh[r], a.iml[r], ph, pl);
            st[base + a.off[r]] = make_double2(re, im);
        }
    }
}

// The double-float coefficients of a dense k-qubit matrix; false when an entry is outside the
// range double-float handles (the FP64 kernel runs instead).
template <int K>
static bool fill_denseK_df(const OpDesc& op, DenseKDfArgs<K>& a) {
    constexpr int D = 1 << K;
    auto split = [](double v, float& h, float& l) {
        const double av = v < 0 ? -v : v;
        if (av != 0.0 && (av > 0x1p100 || av < 0x1p-100)) return false;
        h = float(v);
        l = float(v - double(h));
        return true;
    };
    for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) {
            const double mr = op.m[2 * (r * D + c)], mi = op.m[2 * (r * D + c) + 1];
            if (!split(mr, a.reh[r][c], a.rel[r][c]) || !split(-mi, a.reh[r][D + c], a.rel[r][D + c]) ||
                !split(mr, a.imh[r][c], a.iml[r][c]) || !split(mi, a.imh[r][D + c], a.iml[r][D + c]))
                return false;
        }
    return true;
}

template <typename R, int K>
static cudaError_t launch_denseK(const OpDesc& op, void* state, int n, bool exact, cudaStream_t s, int sms,
                                 bool df64 = false) {
    using T = typename Cplx<R>::T;
    constexpr int D = 1 << K;
    if constexpr (sizeof(R) == 8 && K <= 3) {
        if (df64) {
            DenseKDfArgs<K> d;
            std::memset(&d, 0, sizeof(d));
            if (fill_denseK_df<K>(op, d)) {
                d.map = make_map(op);
                for (int j = 0; j < D; j++) d.off[j] = sub_offset(op, j);
                const uint64_t ntup = 1ull << (n - K - __builtin_popcountll(op.fixmask));
                k_denseK_df<K><<<grid_for(ntup, sms), kThreads, 0, s>>>(static_cast<double2*>(state), ntup, d);
                return counted(cudaGetLastError());
            }
        }
    }
    DenseKArgs<R, K> a;
    std::memset(&a, 0, sizeof(a));
    a.map = make_map(op);
    for (int j = 0; j < D; j++) {
        a.off[j] = sub_offset(op, j);
        a.lane[j] = op.lane[j];
    }
    for (int i = 0; i < 2 * D * D; i++) a.m[i] = R(op.m[i]);
    const uint64_t ntup = 1ull << (n - K - __builtin_popcountll(op.fixmask));
    const int grid = grid_for(ntup, sms);
    const bool real = op.kind == OP_DENSE_REAL;
    T* st = static_cast<T*>(state);
    if constexpr (sizeof(R) == 8) {
        if (exact) {
            if (real)
                k_denseK<R, K, 1><<<grid, kThreads, 0, s>>>(st, ntup, a);
            else
                k_denseK<R, K, 0><<<grid, kThreads, 0, s>>>(st, ntup, a);
            return counted(cudaGetLastError());
        }
    }
    if (real)
        k_denseK<R, K, 3><<<grid, kThreads, 0, s>>>(st, ntup, a);
    else
        k_denseK<R, K, 2><<<grid, kThreads, 0, s>>>(st, ntup, a);
    return counted(cudaGetLastError());
}

template <typename R, int K>
static cudaError_t launch_mono(const OpDesc& op, void* state, int n, cudaStream_t s, int sms) {
    using T = typename Cplx<R>::T;
    constexpr int D = 1 << K;
    MonoArgs<R, K> a;
    std::memset(&a, 0, sizeof(a));
    a.map = make_map(op);
    for (int r = 0; r < D; r++) {
        a.off[r] = sub_offset(op, r);
        a.off_src[r] = sub_offset(op, op.perm[r]);
        a.pf[r] = op.pf[r];
        a.ph[2 * r] = R(op.phase[2 * r]);
        a.ph[2 * r + 1] = R(op.phase[2 * r + 1]);
    }
    const uint64_t ntup = 1ull << (n - K - __builtin_popcountll(op.fixmask));
    k_mono<R, K><<<grid_for(ntup, sms), kThreads, 0, s>>>(static_cast<T*>(state), ntup, a);
    return counted(cudaGetLastError());
}

template <typename R>
static cudaError_t launch_small(const OpDesc& op, void* state, int n, bool exact, cudaStream_t s, int sms,
                                bool df64 = false, bool fx64 = false) {
    if (op.kind == OP_MONO || op.kind == OP_MONO_PF) {
        switch (op.k) {
            case 0: return launch_mono<R, 0>(op, state, n, s, sms);
            case 1: return launch_mono<R, 1>(op, state, n, s, sms);
            case 2: return launch_mono<R, 2>(op, state, n, s, sms);
            case 3: return launch_mono<R, 3>(op, state, n, s, sms);
            case 4: return launch_mono<R, 4>(op, state, n, s, sms);
            case 5: return launch_mono<R, 5>(op, state, n, s, sms);
        }
    } else {
        switch (op.k) {
            case 0: {
                // A 1x1 dense sub-matrix can only be the zero scalar (a non-zero
                // one is monomial): every touched amplitude becomes 0.
                OpDesc z = op;
                z.kind = OP_MONO_PF;
                z.perm.assign(1, 0);
                z.pf.assign(1, PF_ONE);
                z.phase.assign(2, 0.0);
                z.pf[0] = 255;
                return launch_mono<R, 0>(z, state, n, s, sms);
            }
            case 1: return launch_dense1<R>(op, state, n, exact, s, sms, df64, fx64);
            case 2: return launch_denseK<R, 2>(op, state, n, exact, s, sms, df64);
            case 3: return launch_denseK<R, 3>(op, state, n, exact, s, sms, df64);
            case 4: return launch_denseK<R, 4>(op, state, n, exact, s, sms);
            case 5: return launch_denseK<R, 5>(op, state, n, exact, s, sms);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_op(const OpDesc& op, void* state, int n, int prec, int arith, cudaStream_t s, int sms) {
    if (op.kind == OP_NOOP) return cudaSuccess;
    if (op.k > kMaxSmallK) return cudaErrorInvalidValue;
    const bool exact = (arith == QS_ARITH_EXACT);
    if (prec == QS_PREC_C64) return launch_small<float>(op, state, n, false, s, sms);
    return launch_small<double>(op, state, n, exact, s, sms, arith == QS_ARITH_DF64, arith == QS_ARITH_FX64);
}

cudaError_t launch_op_big(const OpDesc& op, void* state, const void* src, int n, int prec, int arith,
                          const BigOpBuffers& b, cudaStream_t s, int sms) {
    IndexMap map = make_map(op);
    const uint64_t ntup = 1ull << (n - op.k - __builtin_popcountll(op.fixmask));
    const uint64_t work = ntup << op.k;
    const int grid = grid_for(work, sms);
    if (op.kind == OP_MONO || op.kind == OP_MONO_PF) {
        if (prec == QS_PREC_C64)
            k_mono_big<float><<<grid, kThreads, 0, s>>>((float2*)state, (const float2*)src, ntup, op.k, map, b.off,
                                                        b.off_src, b.pf, (const float*)b.mat);
        else
            k_mono_big<double><<<grid, kThreads, 0, s>>>((double2*)state, (const double2*)src, ntup, op.k, map,
                                                         b.off, b.off_src, b.pf, (const double*)b.mat);
    } else {
        if (prec == QS_PREC_C64)
            k_dense_big<float, false><<<grid, kThreads, 0, s>>>((float2*)state, (const float2*)src, ntup, op.k, map,
                                                                b.off, b.lane, (const float*)b.mat);
        else if (arith == QS_ARITH_EXACT)
            k_dense_big<double, true><<<grid, kThreads, 0, s>>>((double2*)state, (const double2*)src, ntup, op.k,
                                                                map, b.off, b.lane, (const double*)b.mat);
        else
            k_dense_big<double, false><<<grid, kThreads, 0, s>>>((double2*)state, (const double2*)src, ntup, op.k,
                                                                 map, b.off, b.lane, (const double*)b.mat);
    }
    return counted(cudaGetLastError());
}

void big_op_host_tables(const OpDesc& op, int prec, std::vector<uint64_t>* off, std::vector<uint64_t>* off_src,
                        std::vector<uint8_t>* pf, std::vector<int8_t>* lane, std::vector<unsigned char>* mat) {
    const uint64_t D = 1ull << op.k;
    off->resize(D);
    for (uint64_t j = 0; j < D; j++) (*off)[j] = sub_offset(op, j);
    const size_t rsz = (prec == QS_PREC_C64) ? sizeof(float) : sizeof(double);
    if (op.kind == OP_MONO || op.kind == OP_MONO_PF) {
        off_src->resize(D);
        for (uint64_t j = 0; j < D; j++) (*off_src)[j] = sub_offset(op, op.perm[j]);
        *pf = op.pf;
        mat->resize(2 * D * rsz);
        for (uint64_t i = 0; i < 2 * D; i++) {
            if (prec == QS_PREC_C64) {
                float v = float(op.phase[i]);
                std::memcpy(mat->data() + i * rsz, &v, rsz);
            } else {
                std::memcpy(mat->data() + i * rsz, &op.phase[i], rsz);
            }
        }
    } else {
        *lane = op.lane;
        mat->resize(2 * D * D * rsz);
        for (uint64_t i = 0; i < 2 * D * D; i++) {
            if (prec == QS_PREC_C64) {
                float v = float(op.m[i]);
                std::memcpy(mat->data() + i * rsz, &v, rsz);
            } else {
                std::memcpy(mat->data() + i * rsz, &op.m[i], rsz);
            }
        }
    }
}

}  // namespace qs
