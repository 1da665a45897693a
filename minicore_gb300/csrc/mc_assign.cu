// Hard assignment kernels: argmin over centers of cmp::msr_with_prior
// (include/minicore/clustering/solve.h:234-285, include/minicore/dist/applicator.h:1632-1915).
//
// k_assign_tiled   FP32 CUDA-core tiles of BM rows x BN centers, the column loop sequential
//                  per pair (bit-identical to the oracle's dense path).  Rows come from a
//                  dense matrix or from CSR rows densified in the tile loader (the exact
//                  O(d)-per-pair form used for JSD and for the pair-dependent prior).
// k_assign_sparse  CSR rows, one warp per row: for the measures whose sum over the zero
//                  columns of a row folds into per-center constants (SQRL2, L1, MKL,
//                  Hellinger), only the row's nonzeros are visited:
//                    MKL:  H_c - log(rhinc) A_c + sum_nz a_j (log rhinc - log b_j)
//                    HELL: A_c + B_x - 2 sqrt(rhinc) Q_c + 2 sum_nz sqrt(a_j)(sqrt(rhinc) - sqrt(b_j))
//                    SQRL2: |c|^2 + sum_nz x_j (x_j - 2 c_j)
//                    L1:   E_c + sum_nz (|c'_j - x'_j| - |c'_j - pv|),  c' = c + pv, x' = x + pv
// The pair scalars (pv, lhrsi, lhinc, rhrsi, rhinc) follow applicator.h:1642-1656.  When
// pv is the same for every pair ("constant prior", any prior > 0 in practice) the
// center-side and row-side transforms are precomputed; otherwise (prior 0) every pair
// recomputes them ("pair mode").
#include "mc_assign.cuh"
#include "mc_tune.cuh"

namespace mc {

// ------------------------------------------------------------------------------------
// center preparation
// ------------------------------------------------------------------------------------
// CT0/CT1: [d][kp] transposed center transforms; consts: per-center FP64 constants
//   consts[c*4+0]: MKL H_c = sum a log a | HELL A_c | SQRL2 |c|^2 | L1 E_c
//   consts[c*4+1]: MKL A_c = sum a      | HELL Q_c = sum sqrt(a)
template <int MSR, bool PAIR>
__global__ void k_prep_centers(const float *__restrict__ C, uint32_t k, uint32_t kp, uint64_t d,
                               const double *__restrict__ csum, float pv, float *CT0, float *CT1) {
    const uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (j >= d) return;
    for (uint32_t c = blockIdx.y; c < kp; c += gridDim.y) {
    float v0 = 0.f, v1 = 0.f;
    if (c < k) {
        const float x = C[uint64_t(c) * d + j];
        if (PAIR || MSR == SQRL2) {
            v0 = x;
        } else {
            float rsi, inc;
            side_scalars(pv, csum[c], d, rsi, inc);
            if (MSR == L1) v0 = x + pv;
            else if (MSR == HELLINGER) v0 = sqrtf(x * rsi + inc);
            else {
                const float a = x * rsi + inc;
                v0 = a;
                v1 = (MSR == MKL) ? logf(a) : a * logf(a);
            }
        }
    }
    CT0[j * kp + c] = v0;
    if (CT1) CT1[j * kp + c] = v1;
    }
}

// per-center FP64 constants for the sparse-dot kernels.  One warp per center: lane l adds the
// terms of columns l, l+32, ... (coalesced loads; the logs and square roots in parallel),
// then the 32 lane partials are added in lane order.
template <int MSR>
__global__ void __launch_bounds__(128) k_center_consts(const float *__restrict__ C, uint32_t k, uint64_t d,
                                                       const double *__restrict__ csum, float pv, double *consts) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t c = blockIdx.x * 4 + w;
    if (c >= k) return;  // whole warp; the block has no barrier
    float rsi = 0.f, inc = 0.f;
    if (MSR != SQRL2) side_scalars(pv, csum[c], d, rsi, inc);
    double s0 = 0.0, s1 = 0.0;
    const float *r = C + uint64_t(c) * d;
    for (uint64_t j = lane; j < d; j += 32) {
        const float x = r[j];
        if (MSR == SQRL2) {
            s0 = s0 + double(x) * double(x);
        } else if (MSR == L1) {
            s0 = s0 + double(fabsf((x + pv) - pv));
        } else {
            const float a = x * rsi + inc;
            if (MSR == MKL) {
                s0 = s0 + double(a) * double(logf(a));
                s1 = s1 + double(a);
            } else {  // HELLINGER
                s0 = s0 + double(a);
                s1 = s1 + double(sqrtf(a));
            }
        }
    }
    double t0 = 0.0, t1 = 0.0;
#pragma unroll
    for (int l = 0; l < 32; ++l) {
        t0 = t0 + __shfl_sync(0xffffffffu, s0, l);
        t1 = t1 + __shfl_sync(0xffffffffu, s1, l);
    }
    if (lane == 0) {
        consts[uint64_t(c) * 4 + 0] = t0;
        consts[uint64_t(c) * 4 + 1] = t1;
    }
}

// JSD sparse-dot table (see launch_jsd_ztable): one warp per (group, center); lane l adds the
// float terms of columns l, l+32, ... in FP64, the 32 lane partials are added in lane order.
__global__ void __launch_bounds__(256) k_jsd_ztable(const float *__restrict__ C, uint32_t k, uint64_t d,
                                                    const double *__restrict__ csum, float pv,
                                                    const float *__restrict__ gval, uint32_t ngrp, double *ztab) {
    const int lane = threadIdx.x & 31;
    const uint64_t wid = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    if (wid >= uint64_t(ngrp) * k) return;  // whole warp
    const uint32_t g = uint32_t(wid / k), c = uint32_t(wid % k);
    float rsi, inc;
    side_scalars(pv, csum[c], d, rsi, inc);
    const float b = gval[g];
    const float blb = b * logf(b);
    const float *r = C + uint64_t(c) * d;
    double s = 0.0;
    for (uint64_t j = lane; j < d; j += 32) {
        const float av = r[j] * rsi + inc;
        const float m = av + b;
        s = s + double((av * logf(av) + blb) - m * logf(m * 0.5f));
    }
    double t = 0.0;
#pragma unroll
    for (int l = 0; l < 32; ++l) t = t + __shfl_sync(0xffffffffu, s, l);
    if (lane == 0) ztab[wid] = t;
}

int launch_jsd_ztable(const float *C, uint32_t k, uint64_t d, const double *csum, float pv, const float *gval,
                      uint32_t ngrp, double *ztab, cudaStream_t st) {
    const uint64_t warps = uint64_t(ngrp) * k;
    if (warps == 0) return MC_OK;
    k_jsd_ztable<<<unsigned((warps + 7) / 8), 256, 0, st>>>(C, k, d, csum, pv, gval, ngrp, ztab), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// row-side scalars for the constant-prior path
__global__ void k_row_scalars(const double *__restrict__ rowsum, uint64_t n, uint64_t d, float pv, float *rsi,
                              float *rinc) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    float a, b;
    side_scalars(pv, rowsum[i], d, a, b);
    rsi[i] = a;
    rinc[i] = b;
}

// ------------------------------------------------------------------------------------
// argmin bookkeeping: lexicographic (value, index); NaN at center 0 wins (the reference's
// sequential scan then never moves off center 0), NaN elsewhere never wins.
// ------------------------------------------------------------------------------------
struct Best {
    float v;
    uint32_t j;
};

__device__ inline void best_init(Best &b) {
    b.v = __int_as_float(0x7f800000);
    b.j = 0xffffffffu;
}

__device__ inline void best_offer(Best &b, float v, uint32_t j) {
    if (v != v) {
        if (j != 0) return;
        v = __int_as_float(0xff800000);  // -inf marks "NaN at center 0"
    }
    if (v < b.v || (v == b.v && j < b.j)) {
        b.v = v;
        b.j = j;
    }
}

__device__ inline void best_merge_shfl(Best &b, int lanemask_xor) {
    const float ov = __shfl_xor_sync(0xffffffffu, b.v, lanemask_xor);
    const uint32_t oj = __shfl_xor_sync(0xffffffffu, b.j, lanemask_xor);
    if (ov < b.v || (ov == b.v && oj < b.j)) {
        b.v = ov;
        b.j = oj;
    }
}

// final value of a pair: compare key (float) and cost (double) per measure
template <int MSR>
__device__ inline float finish_key(float acc) {
    if (MSR == SQRL2) return acc;
    if (MSR == L1) return acc * 0.5f;
    if (MSR == HELLINGER) return sqrtf(acc);
    if (MSR == MKL) return post_divergence(acc);
    return post_divergence(acc * 0.5f);  // JSD
}

template <int MSR>
__device__ inline double key_to_cost(float key) {
    if (MSR == L1) return double(key) * 2.0;
    if (MSR == HELLINGER) return double(key) * kSqrt1_2;
    return double(key);
}

// ------------------------------------------------------------------------------------
// tiled kernel
// ------------------------------------------------------------------------------------
constexpr int kBK = 16;

template <int MSR>
struct Ops {
    static constexpr bool two_center = (MSR == MKL || MSR == JSD);
    static constexpr bool two_row = (MSR == JSD);
};

// element step.  c0/c1: center-side values, x0/x1: row-side values (constant-prior
// transforms), or raw values + pair scalars in pair mode.
template <int MSR, bool PAIR>
__device__ inline void elem(float &acc, float c0, float c1, float x0, float x1, const PairScalars &s) {
    if (!PAIR) {
        if (MSR == SQRL2 || MSR == HELLINGER) {
            const float df = c0 - x0;
            acc = fmaf(df, df, acc);
        } else if (MSR == L1) {
            acc = acc + fabsf(c0 - x0);
        } else if (MSR == MKL) {
            acc = fmaf(c0, c1 - x0, acc);
        } else {  // JSD: c0 = a, c1 = a log a, x0 = b, x1 = b log b
            const float m = c0 + x0;
            const float t = (c1 + x1) - m * logf(m * 0.5f);
            acc = acc + t;
        }
    } else {
        if (MSR == SQRL2) {
            const float df = c0 - x0;
            acc = fmaf(df, df, acc);
        } else if (MSR == L1) {
            const float a = c0 + s.pv, b = x0 + s.pv;
            acc = acc + fabsf(a - b);
        } else if (MSR == HELLINGER) {
            const float a = sqrtf(c0 * s.lhrsi + s.lhinc), b = sqrtf(x0 * s.rhrsi + s.rhinc);
            const float df = a - b;
            acc = fmaf(df, df, acc);
        } else if (MSR == MKL) {
            const float a = c0 * s.lhrsi + s.lhinc, b = x0 * s.rhrsi + s.rhinc;
            acc = fmaf(a, logf(a) - logf(b), acc);
        } else {
            const float a = c0 * s.lhrsi + s.lhinc, b = x0 * s.rhrsi + s.rhinc;
            const float m = a + b;
            const float t = (a * logf(a) + b * logf(b)) - m * logf(m * 0.5f);
            acc = acc + t;
        }
    }
}

// row-side transform of a raw value x for the constant-prior path
template <int MSR>
__device__ inline void row_xform(float x, float pv, float rsi, float rinc, float &x0, float &x1) {
    if (MSR == SQRL2) { x0 = x; x1 = 0.f; }
    else if (MSR == L1) { x0 = x + pv; x1 = 0.f; }
    else if (MSR == HELLINGER) { x0 = sqrtf(x * rsi + rinc); x1 = 0.f; }
    else {
        const float b = x * rsi + rinc;
        if (MSR == MKL) { x0 = logf(b); x1 = 0.f; }
        else { x0 = b; x1 = b * logf(b); }
    }
}

template <int MSR, bool PAIR, int TM, int TN, bool CSR>
__global__ void __launch_bounds__(256) k_assign_tiled(AssignArgs a) {
    constexpr int BM = 16 * TM, BN = 16 * TN;
    constexpr bool C2 = !PAIR && Ops<MSR>::two_center;
    constexpr bool R2 = !PAIR && Ops<MSR>::two_row;
    __shared__ float Xs0[BM][kBK + 1];
    __shared__ float Xs1[R2 ? BM : 1][kBK + 1];
    __shared__ __align__(16) float Cs0[kBK][BN];
    __shared__ __align__(16) float Cs1[C2 ? kBK : 1][C2 ? BN : 4];
    __shared__ uint64_t cursor[CSR ? BM : 1];

    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const uint64_t row0 = uint64_t(blockIdx.x) * BM;
    const uint64_t d = a.d;
    if (a.n_dev) {  // launched for the largest count: tiles past the device count leave at once
        const uint64_t nd = *a.n_dev;
        if (row0 >= nd) return;
        if (nd < a.n) a.n = nd;
    }

    float rpv = a.pv;
    Best best[TM];
#pragma unroll
    for (int i = 0; i < TM; ++i) best_init(best[i]);

    double rsum_reg[TM];
    if (PAIR) {
#pragma unroll
        for (int i = 0; i < TM; ++i) {
            const uint64_t r = row0 + ty * TM + i;
            rsum_reg[i] = r < a.n ? a.rowsum[r] : 0.0;
        }
    }

    for (uint32_t cbase = 0; cbase < a.k; cbase += BN) {
        float acc[TM][TN];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
        PairScalars ps[PAIR ? TM : 1][PAIR ? TN : 1];
        if (PAIR) {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    const uint32_t c = cbase + tx * TN + j;
                    const double cs = c < a.k ? a.csum[c] : 0.0;
                    ps[i][j] = pair_scalars(a.prior, a.prior_sum, rsum_reg[i], cs, d);
                }
        }
        if (CSR) {
            if (t < BM) {
                const uint64_t r = row0 + t;
                cursor[t] = r < a.n ? a.indptr[r] : 0;
            }
            __syncthreads();
        }
        for (uint64_t k0 = 0; k0 < d; k0 += kBK) {
            const int kmax = int(umin64(kBK, d - k0));
            // ---- row tile ----
            if (!CSR) {
                for (int e = t; e < BM * kBK; e += 256) {
                    const int r = e / kBK, kk = e % kBK;
                    const uint64_t row = row0 + r;
                    float x = 0.f;
                    if (row < a.n && kk < kmax) x = a.X[(a.rows ? uint64_t(a.rows[row]) : row) * d + k0 + kk];
                    if (PAIR) {
                        Xs0[r][kk] = x;
                    } else {
                        float x0, x1;
                        const float rsi = (MSR == SQRL2 || MSR == L1 || row >= a.n) ? 0.f : a.rsi[row];
                        const float rinc = (MSR == SQRL2 || MSR == L1 || row >= a.n) ? 0.f : a.rinc[row];
                        row_xform<MSR>(x, rpv, rsi, rinc, x0, x1);
                        Xs0[r][kk] = x0;
                        if (R2) Xs1[r][kk] = x1;
                    }
                }
            } else {
                // densify: fill with the transform of 0, then scatter this window's nonzeros
                for (int e = t; e < BM * kBK; e += 256) {
                    const int r = e / kBK, kk = e % kBK;
                    const uint64_t row = row0 + r;
                    if (PAIR) {
                        Xs0[r][kk] = 0.f;
                    } else {
                        float x0, x1;
                        const float rsi = (MSR == SQRL2 || MSR == L1 || row >= a.n) ? 0.f : a.rsi[row];
                        const float rinc = (MSR == SQRL2 || MSR == L1 || row >= a.n) ? 0.f : a.rinc[row];
                        row_xform<MSR>(0.f, rpv, rsi, rinc, x0, x1);
                        Xs0[r][kk] = x0;
                        if (R2) Xs1[r][kk] = x1;
                    }
                }
                __syncthreads();
                if (t < BM) {
                    const uint64_t row = row0 + t;
                    if (row < a.n) {
                        uint64_t p = cursor[t];
                        const uint64_t pe = a.indptr[row + 1];
                        const float rsi = (PAIR || MSR == SQRL2 || MSR == L1) ? 0.f : a.rsi[row];
                        const float rinc = (PAIR || MSR == SQRL2 || MSR == L1) ? 0.f : a.rinc[row];
                        while (p < pe) {
                            const uint64_t col = a.idx[p];
                            if (col >= k0 + kBK) break;
                            const float x = a.vals[p];
                            if (PAIR) {
                                Xs0[t][col - k0] = x;
                            } else {
                                float x0, x1;
                                row_xform<MSR>(x, rpv, rsi, rinc, x0, x1);
                                Xs0[t][col - k0] = x0;
                                if (R2) Xs1[t][col - k0] = x1;
                            }
                            ++p;
                        }
                        cursor[t] = p;
                    }
                }
            }
            // ---- center tile (CT is [d][kp]) ----
            for (int e = t; e < BN * kBK; e += 256) {
                const int kk = e / BN, c = e % BN;
                float v0 = 0.f, v1 = 0.f;
                if (kk < kmax) {
                    const uint64_t off = (k0 + kk) * a.kp + cbase + c;
                    v0 = a.CT0[off];
                    if (C2) v1 = a.CT1[off];
                }
                Cs0[kk][c] = v0;
                if (C2) Cs1[kk][c] = v1;
            }
            __syncthreads();
#pragma unroll 4
            for (int kk = 0; kk < kBK; ++kk) {
                if (kk < kmax) {
                    float xv0[TM], xv1[TM];
#pragma unroll
                    for (int i = 0; i < TM; ++i) {
                        xv0[i] = Xs0[ty * TM + i][kk];
                        xv1[i] = R2 ? Xs1[ty * TM + i][kk] : 0.f;
                    }
                    float cv0[TN], cv1[TN];
#pragma unroll
                    for (int j = 0; j < TN; ++j) {
                        cv0[j] = Cs0[kk][tx * TN + j];
                        cv1[j] = C2 ? Cs1[kk][tx * TN + j] : 0.f;
                    }
#pragma unroll
                    for (int i = 0; i < TM; ++i)
#pragma unroll
                        for (int j = 0; j < TN; ++j)
                            elem<MSR, PAIR>(acc[i][j], cv0[j], cv1[j], xv0[i], xv1[i], ps[PAIR ? i : 0][PAIR ? j : 0]);
                }
            }
            __syncthreads();
        }
        // ---- fold this center tile into the running argmin ----
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const uint32_t c = cbase + tx * TN + j;
            if (c < a.k) {
#pragma unroll
                for (int i = 0; i < TM; ++i) {
                    const float key = finish_key<MSR>(acc[i][j]);
                    best_offer(best[i], key, c);
                    if (a.dmode) {
                        const uint64_t row = row0 + ty * TM + i;
                        if (row < a.n) write_dist(a, a.rows ? uint64_t(a.rows[row]) : row, c, float(key_to_cost<MSR>(key)));
                    }
                }
            }
        }
    }
    // reduce across the 16 tx lanes that share rows (same half-warp)
#pragma unroll
    for (int i = 0; i < TM; ++i) {
#pragma unroll
        for (int m = 8; m >= 1; m >>= 1) best_merge_shfl(best[i], m);
    }
    if (tx == 0) {
#pragma unroll
        for (int i = 0; i < TM; ++i) {
            const uint64_t row = row0 + ty * TM + i;
            if (row < a.n) {
                const bool nan0 = best[i].v == __int_as_float(0xff800000);
                double cost = nan0 ? __longlong_as_double(0x7ff8000000000000ll) : key_to_cost<MSR>(best[i].v);
                if (CSR) cost = double(float(cost));
                const uint64_t orow = a.rows ? uint64_t(a.rows[row]) : row;
                a.asn[orow] = best[i].j;
                a.costs[orow] = cost;
            }
        }
    }
}

// ------------------------------------------------------------------------------------
// sparse-dot CSR kernel (constant prior; SQRL2, L1, MKL, HELLINGER)
// one warp per row; lane l owns centers l, l+32, ... of the current group of 32*KPL
// ------------------------------------------------------------------------------------
template <int KPL>
struct CenterVec;
template <>
struct CenterVec<1> {
    float v[1];
    __device__ __forceinline__ void load(const float *p) { v[0] = __ldg(p); }
    __device__ __forceinline__ void zero() { v[0] = 0.f; }
};
template <>
struct CenterVec<2> {
    float v[2];
    __device__ __forceinline__ void load(const float *p) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        v[0] = t.x;
        v[1] = t.y;
    }
    __device__ __forceinline__ void zero() { v[0] = v[1] = 0.f; }
};
template <>
struct CenterVec<4> {
    float v[4];
    __device__ __forceinline__ void load(const float *p) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
    }
    __device__ __forceinline__ void zero() { v[0] = v[1] = v[2] = v[3] = 0.f; }
};

// Lane l owns centers g0 + KPL*l .. + KPL-1 of the current group of 32*KPL (one vector load
// per nonzero; lanes past the padded centers idle).  Each
// chunk of 32 nonzeros is staged per warp in shared memory as (column, g) and read back by
// broadcast; SB nonzeros per batch (8, 4 or 16, picked by the autotuner) have their center
// loads issued before the first use.
// The per-(row, center) sum stays sequential over the nonzeros.
template <int MSR, int KPL, int SB>
__global__ void __launch_bounds__(256) k_assign_sparse(AssignArgs a) {
    __shared__ uint2 stage[8][32];  // per warp: (column, g bits) of the current 32 nonzeros
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    const uint64_t nwarps = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    const float pv = a.pv;
    for (uint64_t row = warp; row < a.n; row += nwarps) {
        const uint64_t pb = a.indptr[row], pe = a.indptr[row + 1];
        float rsi = 0.f, rinc = 0.f;
        if (MSR == MKL || MSR == HELLINGER || MSR == JSD) {
            rsi = a.rsi[row];
            rinc = a.rinc[row];
        }
        const float rl = (MSR == MKL) ? logf(rinc) : 0.f;
        const float srinc = (MSR == HELLINGER) ? sqrtf(rinc) : 0.f;
        Best best;
        best_init(best);
        // HELLINGER: sum of b over all columns; JSD: sum over the nonzeros of b log b - r log r
        double bx = 0.0;
        if (MSR == HELLINGER || MSR == JSD) {
            const float rlr = (MSR == JSD) ? rinc * logf(rinc) : 0.f;
            double s = 0.0;
            for (uint64_t p = pb + lane; p < pe; p += 32) {
                const float b = a.vals[p] * rsi + rinc;
                s += (MSR == JSD) ? double(b * logf(b) - rlr) : double(b);
            }
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
            bx = (MSR == JSD) ? s : s + double(a.d - (pe - pb)) * double(rinc);
        }
        const double *zrow = (MSR == JSD) ? a.ztab + uint64_t(a.grp[row]) * a.k : nullptr;
        for (uint32_t g0 = 0; g0 < a.k; g0 += 32 * KPL) {
            float acc[KPL];
#pragma unroll
            for (int q = 0; q < KPL; ++q) acc[q] = 0.f;
            const float *ctl = a.CT0 + g0 + KPL * lane;
            const bool lane_on = g0 + KPL * lane < a.kp;  // lanes past the padded centers idle
            for (uint64_t p0 = pb; p0 < pe; p0 += 32) {
                const uint64_t p = p0 + lane;
                // past the row's end: center column 0 with a g that adds exactly nothing
                // (MKL, Hellinger, SQRL2: g = 0 makes every term +-0 on a sum that is not
                // -0; L1: g = pv makes |c - g| - |c - pv| = +0; JSD: g = rinc makes the two
                // products of the term equal)
                uint32_t col = 0;
                float g = (MSR == L1) ? pv : (MSR == JSD) ? rinc : 0.f;
                if (p < pe) {
                    col = a.idx[p];
                    const float x = a.vals[p];
                    if (MSR == MKL) g = rl - logf(x * rsi + rinc);
                    else if (MSR == HELLINGER) g = srinc - sqrtf(x * rsi + rinc);
                    else if (MSR == L1) g = x + pv;
                    else if (MSR == JSD) g = x * rsi + rinc;
                    else g = x;
                }
                __syncwarp();
                stage[wib][lane] = make_uint2(col, __float_as_uint(g));
                __syncwarp();
                const int cnt = int(umin64(32, pe - p0));  // warp-uniform
                for (int q0 = 0; q0 < cnt; q0 += SB) {
                    CenterVec<KPL> cv[SB];
                    float gj[SB];
#pragma unroll
                    for (int u = 0; u < SB; ++u) {
                        const uint2 e = stage[wib][q0 + u];
                        if (lane_on) cv[u].load(ctl + uint64_t(e.x) * a.kp);
                        else cv[u].zero();
                        gj[u] = __uint_as_float(e.y);
                    }
#pragma unroll
                    for (int u = 0; u < SB; ++u) {
#pragma unroll
                        for (int r = 0; r < KPL; ++r) {
                            const float c = cv[u].v[r];
                            if (MSR == MKL || MSR == HELLINGER) {
                                acc[r] = fmaf(c, gj[u], acc[r]);
                            } else if (MSR == SQRL2) {
                                acc[r] = fmaf(gj[u], gj[u] - 2.f * c, acc[r]);
                            } else if (MSR == JSD) {
                                const float m0 = c + rinc, m1 = c + gj[u];
                                acc[r] = acc[r] + (m0 * logf(m0 * 0.5f) - m1 * logf(m1 * 0.5f));
                            } else {
                                acc[r] = acc[r] + (fabsf(c - gj[u]) - fabsf(c - pv));
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < KPL; ++r) {
                const uint32_t c = g0 + KPL * lane + r;
                if (c < a.k) {
                    float key;
                    double k0 = 0.0, k1 = 0.0;
                    if (MSR != JSD) k0 = a.consts[uint64_t(c) * 4 + 0], k1 = a.consts[uint64_t(c) * 4 + 1];
                    if (MSR == JSD) {
                        key = post_divergence(float((zrow[c] + bx + double(acc[r])) * 0.5));
                    } else if (MSR == MKL) {
                        key = post_divergence(float(k0 - double(rl) * k1 + double(acc[r])));
                    } else if (MSR == HELLINGER) {
                        double s = k0 + bx - 2.0 * double(srinc) * k1 + 2.0 * double(acc[r]);
                        if (s < 0.0) s = 0.0;
                        key = float(sqrt(s));
                    } else if (MSR == SQRL2) {
                        double s = k0 + double(acc[r]);
                        if (s < 0.0) s = 0.0;
                        key = float(s);
                    } else {
                        key = float(k0 + double(acc[r])) * 0.5f;
                    }
                    best_offer(best, key, c);
                    if (a.dmode) write_dist(a, row, c, float(key_to_cost<MSR>(key)));
                }
            }
        }
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) best_merge_shfl(best, m);
        if (lane == 0) {
            const bool nan0 = best.v == __int_as_float(0xff800000);
            const double cost = nan0 ? __longlong_as_double(0x7ff8000000000000ll) : key_to_cost<MSR>(best.v);
            a.asn[row] = best.j;
            a.costs[row] = double(float(cost));
        }
    }
}

// Two rows per warp for 64 padded centers: half-warp h of warp w takes row 2w + h, lane l of
// the half owns centers 4l .. 4l+3 (one float4 gather per nonzero), chunks of 16 nonzeros
// per half are staged in shared memory.  Both halves walk max(chunks) chunks, the shorter row
// padded with neutral entries (column 0, a g that adds exactly nothing), so the warp stays in
// lock step.  Per-(row, center) sums stay sequential over the nonzeros, as in k_assign_sparse.
template <int MSR, int SB>
__global__ void __launch_bounds__(256) k_assign_sparse_pair(AssignArgs a) {
    __shared__ uint2 stage[8][2][16];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, half = lane >> 4, hl = lane & 15;
    const unsigned hmask = half ? 0xffff0000u : 0x0000ffffu;
    const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    const uint64_t nwarps = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    const float pv = a.pv;
    for (uint64_t pair = warp; 2 * pair < a.n; pair += nwarps) {
        const uint64_t row = 2 * pair + half;
        const bool live = row < a.n;
        const uint64_t pb = live ? a.indptr[row] : 0, pe = live ? a.indptr[row + 1] : 0;
        float rsi = 0.f, rinc = 0.f;
        if (live && (MSR == MKL || MSR == HELLINGER || MSR == JSD)) {
            rsi = a.rsi[row];
            rinc = a.rinc[row];
        }
        const float rl = (MSR == MKL) ? logf(rinc) : 0.f;
        const float srinc = (MSR == HELLINGER) ? sqrtf(rinc) : 0.f;
        double bx = 0.0;
        if (MSR == HELLINGER || MSR == JSD) {
            const float rlr = (MSR == JSD) ? rinc * logf(rinc) : 0.f;
            double sb = 0.0;
            for (uint64_t p = pb + hl; p < pe; p += 16) {
                const float b = a.vals[p] * rsi + rinc;
                sb += (MSR == JSD) ? double(b * logf(b) - rlr) : double(b);
            }
#pragma unroll
            for (int m = 8; m >= 1; m >>= 1) sb += __shfl_xor_sync(0xffffffffu, sb, m);
            bx = (MSR == JSD) ? sb : sb + double(a.d - (pe - pb)) * double(rinc);
        }
        // chunks: the longer of the two rows decides
        const uint64_t mine = (pe - pb + 15) / 16;
        const uint64_t other = __shfl_xor_sync(0xffffffffu, mine, 16);
        const uint64_t nchunk = mine > other ? mine : other;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        const float *ctl = a.CT0 + 4 * hl;
        for (uint64_t ch = 0; ch < nchunk; ++ch) {
            const uint64_t p = pb + ch * 16 + hl;
            uint32_t col = 0;
            float g = (MSR == L1) ? pv : (MSR == JSD) ? rinc : 0.f;
            if (p < pe) {
                col = a.idx[p];
                const float x = a.vals[p];
                if (MSR == MKL) g = rl - logf(x * rsi + rinc);
                else if (MSR == HELLINGER) g = srinc - sqrtf(x * rsi + rinc);
                else if (MSR == L1) g = x + pv;
                else if (MSR == JSD) g = x * rsi + rinc;
                else g = x;
            }
            __syncwarp();
            stage[wib][half][hl] = make_uint2(col, __float_as_uint(g));
            __syncwarp();
#pragma unroll
            for (int q0 = 0; q0 < 16; q0 += SB) {
                float4 cv[SB];
                float gj[SB];
#pragma unroll
                for (int u = 0; u < SB; ++u) {
                    const uint2 e = stage[wib][half][q0 + u];
                    cv[u] = __ldg(reinterpret_cast<const float4 *>(ctl + uint64_t(e.x) * a.kp));
                    gj[u] = __uint_as_float(e.y);
                }
#pragma unroll
                for (int u = 0; u < SB; ++u) {
                    const float cc[4] = {cv[u].x, cv[u].y, cv[u].z, cv[u].w};
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        if (MSR == MKL || MSR == HELLINGER) {
                            acc[r] = fmaf(cc[r], gj[u], acc[r]);
                        } else if (MSR == SQRL2) {
                            acc[r] = fmaf(gj[u], gj[u] - 2.f * cc[r], acc[r]);
                        } else if (MSR == JSD) {
                            const float m0 = cc[r] + rinc, m1 = cc[r] + gj[u];
                            acc[r] = acc[r] + (m0 * logf(m0 * 0.5f) - m1 * logf(m1 * 0.5f));
                        } else {
                            acc[r] = acc[r] + (fabsf(cc[r] - gj[u]) - fabsf(cc[r] - pv));
                        }
                    }
                }
            }
        }
        Best best;
        best_init(best);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t c = 4 * hl + r;
            if (live && c < a.k) {
                float key;
                double k0 = 0.0, k1 = 0.0;
                if (MSR != JSD) k0 = a.consts[uint64_t(c) * 4 + 0], k1 = a.consts[uint64_t(c) * 4 + 1];
                if (MSR == JSD) {
                    key = post_divergence(float((a.ztab[uint64_t(a.grp[row]) * a.k + c] + bx + double(acc[r])) * 0.5));
                } else if (MSR == MKL) {
                    key = post_divergence(float(k0 - double(rl) * k1 + double(acc[r])));
                } else if (MSR == HELLINGER) {
                    double sv = k0 + bx - 2.0 * double(srinc) * k1 + 2.0 * double(acc[r]);
                    if (sv < 0.0) sv = 0.0;
                    key = float(sqrt(sv));
                } else if (MSR == SQRL2) {
                    double sv = k0 + double(acc[r]);
                    if (sv < 0.0) sv = 0.0;
                    key = float(sv);
                } else {
                    key = float(k0 + double(acc[r])) * 0.5f;
                }
                best_offer(best, key, c);
                if (a.dmode) write_dist(a, row, c, float(key_to_cost<MSR>(key)));
            }
        }
#pragma unroll
        for (int m = 8; m >= 1; m >>= 1) best_merge_shfl(best, m);
        (void)hmask;
        if (live && hl == 0) {
            const bool nan0 = best.v == __int_as_float(0xff800000);
            const double cost = nan0 ? __longlong_as_double(0x7ff8000000000000ll) : key_to_cost<MSR>(best.v);
            a.asn[row] = best.j;
            a.costs[row] = double(float(cost));
        }
    }
}

// Column-band form for 64 padded centers (MKL, Hellinger, SQRL2, L1).  The center transform
// CT0 ([d][64] floats, 5 MB at d = 20,000) does not fit in shared memory, and the gather
// kernels above read one 256-byte center column per nonzero from L1/L2, so they wait on
// cache misses.  Here a CTA streams CT0 through shared memory one band of kBandCols columns
// at a time (two buffers, cp.async 16-byte copies: the next band loads while this one is
// used), and each warp keeps kBandRows rows' accumulators in registers across all bands:
// warp-per-row, lane l owns centers 2l and 2l + 1 (one 8-byte shared load per nonzero).
// A row's nonzeros are visited once, in ascending column order: a window of the next 32
// (column, g) pairs sits one per lane, and the part of the window inside the current band
// is broadcast lane by lane.  Per (row, center) the sum is the same sequential fmaf chain
// over the row's nonzeros as in k_assign_sparse_pair, and Hellinger's row term is summed in
// that kernel's lane order, so the results are bit-identical to it (an autotuner variant).
constexpr int kBandCols = 384;                 // columns per band: 384 x 256 B = 96 KB
constexpr int kBandRows = 8;                   // rows per warp
constexpr int kBandThreads = 512;              // 16 warps: 128 rows per CTA chunk
constexpr size_t kBandSmem = 2ull * kBandCols * 64 * sizeof(float);

template <int MSR>
__global__ void __launch_bounds__(kBandThreads, 1) k_assign_sparse_band(AssignArgs a) {
    static_assert(MSR != JSD, "JSD's zero-entry table path is not banded");
    extern __shared__ __align__(16) float tband[];  // [2][kBandCols][64]
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    constexpr int R = kBandRows, WARPS = kBandThreads / 32, ROWS = WARPS * R;
    const uint64_t nbands = (a.d + kBandCols - 1) / kBandCols;
    const float pv = a.pv;
    // band b of CT0 into buffer buf: contiguous floats [b0 * 64, b1 * 64)
    auto stage = [&](uint64_t b, int buf) {
        const uint64_t b0 = b * kBandCols, b1 = umin64(b0 + kBandCols, a.d);
        const uint32_t items = uint32_t((b1 - b0) * 16);  // 16-byte items
        const float4 *src = reinterpret_cast<const float4 *>(a.CT0 + b0 * 64);
        float4 *dst = reinterpret_cast<float4 *>(tband + size_t(buf) * kBandCols * 64);
        for (uint32_t e = threadIdx.x; e < items; e += kBandThreads) {
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(uint32_t(__cvta_generic_to_shared(dst + e))),
                         "l"(src + e)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    for (uint64_t chunk = blockIdx.x; chunk * ROWS < a.n; chunk += gridDim.x) {
        uint64_t cur[R];   // next nonzero of row r not yet in its window
        uint32_t left[R];  // nonzeros of row r after cur
        uint32_t wst[R];   // window state: used prefix (bits 0-7), elements held (bits 8-15)
        uint32_t wcol[R];
        float wg[R];
        float acc[R][2];
        float rsi[R], rinc[R];
        double sb[R];
        // a window of the next 32 nonzeros of row r: lane l holds element cur + l
        auto load_window = [&](int r) {
            const uint64_t p = cur[r] + uint64_t(lane);
            const uint32_t cnt = left[r] < 32u ? left[r] : 32u;
            uint32_t col = 0;
            float g = 0.f;
            float hb = 0.f;  // Hellinger: this element's b
            if (uint32_t(lane) < cnt) {
                col = a.idx[p];
                const float x = a.vals[p];
                if (MSR == MKL) g = logf(rinc[r]) - logf(x * rsi[r] + rinc[r]);
                else if (MSR == HELLINGER) {
                    hb = x * rsi[r] + rinc[r];
                    g = sqrtf(rinc[r]) - sqrtf(hb);
                } else if (MSR == L1) g = x + pv;
                else g = x;
            }
            if (MSR == HELLINGER) {
                // k_assign_sparse_pair's lane order: half-warp lane h sums the elements at
                // offsets = h (mod 16) in ascending order; here lanes h and h + 16 hold the
                // window's two such elements, in that order
                const float hb2 = __shfl_down_sync(0xffffffffu, hb, 16);
                if (lane < 16) {
                    if (uint32_t(lane) < cnt) sb[r] += double(hb);
                    if (uint32_t(lane) + 16 < cnt) sb[r] += double(hb2);
                }
            }
            wcol[r] = col;
            wg[r] = g;
            wst[r] = cnt << 8;
            cur[r] += cnt;
            left[r] -= cnt;
        };
        for (int r = 0; r < R; ++r) {
            const uint64_t row = chunk * ROWS + uint64_t(wib) * R + r;
            const bool live = row < a.n;
            const uint64_t pb = live ? a.indptr[row] : 0, pe = live ? a.indptr[row + 1] : 0;
            cur[r] = pb;
            left[r] = uint32_t(pe - pb);
            rsi[r] = (live && (MSR == MKL || MSR == HELLINGER)) ? a.rsi[row] : 0.f;
            rinc[r] = (live && (MSR == MKL || MSR == HELLINGER)) ? a.rinc[row] : 0.f;
            acc[r][0] = acc[r][1] = 0.f;
            sb[r] = 0.0;
            load_window(r);
        }
        stage(0, 0);
        for (uint64_t b = 0; b < nbands; ++b) {
            const int buf = int(b & 1);
            if (b + 1 < nbands) {
                stage(b + 1, buf ^ 1);
                asm volatile("cp.async.wait_group 1;" ::: "memory");
            } else {
                asm volatile("cp.async.wait_group 0;" ::: "memory");
            }
            __syncthreads();
            const uint32_t b0 = uint32_t(b * kBandCols), bend = uint32_t(umin64(b0 + kBandCols, a.d));
            const float2 *tb = reinterpret_cast<const float2 *>(tband + size_t(buf) * kBandCols * 64) + lane;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                for (;;) {
                    // the window's elements before bend form a prefix (columns ascend)
                    const uint32_t held = wst[r] >> 8;
                    const unsigned in = __ballot_sync(0xffffffffu, uint32_t(lane) < held && wcol[r] < bend);
                    const uint32_t m = uint32_t(__popc(in));
                    // batches of 8: the 8 shared loads issue before the chain of fmaf uses
                    // them; slots past m load column b0 and are not added
                    for (uint32_t q0 = wst[r] & 0xffu; q0 < m; q0 += 8) {
                        float2 cv[8];
                        float gq[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const uint32_t q = q0 + uint32_t(u);
                            const uint32_t c = __shfl_sync(0xffffffffu, wcol[r], int(q & 31u));
                            gq[u] = __shfl_sync(0xffffffffu, wg[r], int(q & 31u));
                            cv[u] = tb[(q < m ? c - b0 : 0u) * 32];
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            if (q0 + uint32_t(u) < m) {
#pragma unroll
                                for (int h = 0; h < 2; ++h) {
                                    const float cc = h ? cv[u].y : cv[u].x;
                                    const float g = gq[u];
                                    if (MSR == MKL || MSR == HELLINGER) acc[r][h] = fmaf(cc, g, acc[r][h]);
                                    else if (MSR == SQRL2) acc[r][h] = fmaf(g, g - 2.f * cc, acc[r][h]);
                                    else acc[r][h] = acc[r][h] + (fabsf(cc - g) - fabsf(cc - pv));
                                }
                            }
                        }
                    }
                    if (m > (wst[r] & 0xffu)) wst[r] = (wst[r] & 0xff00u) | m;
                    if (m == held && left[r] > 0) {
                        load_window(r);  // all of this window used: the next 32 nonzeros
                        continue;
                    }
                    break;
                }
            }
            __syncthreads();  // every warp is done with buffer buf before it is refilled
        }
        // keys and argmin, as k_assign_sparse_pair
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint64_t row = chunk * ROWS + uint64_t(wib) * R + r;
            const bool live = row < a.n;
            const float rl = (MSR == MKL) ? logf(rinc[r]) : 0.f;
            const float srinc = (MSR == HELLINGER) ? sqrtf(rinc[r]) : 0.f;
            double bx = 0.0;
            if (MSR == HELLINGER) {
                double v = sb[r];
#pragma unroll
                for (int m = 8; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
                v = __shfl_sync(0xffffffffu, v, 0);  // lanes 0-15 hold the total; every lane needs it
                const uint64_t nz = live ? a.indptr[row + 1] - a.indptr[row] : 0;
                bx = v + double(a.d - nz) * double(rinc[r]);
            }
            Best best;
            best_init(best);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t c = 2 * lane + h;
                if (live && c < a.k) {
                    float key;
                    const double k0 = a.consts[uint64_t(c) * 4 + 0], k1 = a.consts[uint64_t(c) * 4 + 1];
                    if (MSR == MKL) {
                        key = post_divergence(float(k0 - double(rl) * k1 + double(acc[r][h])));
                    } else if (MSR == HELLINGER) {
                        double sv = k0 + bx - 2.0 * double(srinc) * k1 + 2.0 * double(acc[r][h]);
                        if (sv < 0.0) sv = 0.0;
                        key = float(sqrt(sv));
                    } else if (MSR == SQRL2) {
                        double sv = k0 + double(acc[r][h]);
                        if (sv < 0.0) sv = 0.0;
                        key = float(sv);
                    } else {
                        key = float(k0 + double(acc[r][h])) * 0.5f;
                    }
                    best_offer(best, key, c);
                    if (a.dmode) write_dist(a, row, c, float(key_to_cost<MSR>(key)));
                }
            }
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1) best_merge_shfl(best, m);
            if (live && lane == 0) {
                const bool nan0 = best.v == __int_as_float(0xff800000);
                const double cost = nan0 ? __longlong_as_double(0x7ff8000000000000ll) : key_to_cost<MSR>(best.v);
                a.asn[row] = best.j;
                a.costs[row] = double(float(cost));
            }
        }
    }
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
template <int MSR>
static int prep_centers_t(const AssignArgs &a, bool pair, float *C, cudaStream_t st) {
    dim3 g(unsigned((a.d + 255) / 256), a.kp < 65535 ? a.kp : 65535);
    if (pair) k_prep_centers<MSR, true><<<g, 256, 0, st>>>(C, a.k, a.kp, a.d, a.csum, a.pv, a.CT0, a.CT1), note_launch();
    else k_prep_centers<MSR, false><<<g, 256, 0, st>>>(C, a.k, a.kp, a.d, a.csum, a.pv, a.CT0, a.CT1), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

int launch_prep_centers(const AssignArgs &a, const float *C, bool pair, bool sparse_consts, cudaStream_t st) {
    float *Cm = const_cast<float *>(C);
    switch (a.msr) {
        case SQRL2: MC_TRY(prep_centers_t<SQRL2>(a, pair, Cm, st)); break;
        case L1: MC_TRY(prep_centers_t<L1>(a, pair, Cm, st)); break;
        case HELLINGER: MC_TRY(prep_centers_t<HELLINGER>(a, pair, Cm, st)); break;
        case MKL: MC_TRY(prep_centers_t<MKL>(a, pair, Cm, st)); break;
        case JSD: MC_TRY(prep_centers_t<JSD>(a, pair, Cm, st)); break;
        default: return fail(MC_EUNSUPPORTED, "measure not supported");
    }
    if (sparse_consts) {
        const unsigned g = (a.k + 3) / 4;
        switch (a.msr) {
            case SQRL2: k_center_consts<SQRL2><<<g, 128, 0, st>>>(C, a.k, a.d, a.csum, a.pv, a.consts), note_launch(); break;
            case L1: k_center_consts<L1><<<g, 128, 0, st>>>(C, a.k, a.d, a.csum, a.pv, a.consts), note_launch(); break;
            case HELLINGER: k_center_consts<HELLINGER><<<g, 128, 0, st>>>(C, a.k, a.d, a.csum, a.pv, a.consts), note_launch(); break;
            case MKL: k_center_consts<MKL><<<g, 128, 0, st>>>(C, a.k, a.d, a.csum, a.pv, a.consts), note_launch(); break;
            default: break;
        }
        MC_CUDA_TRY(cudaGetLastError());
    }
    return MC_OK;
}

int launch_row_scalars(const double *rowsum, uint64_t n, uint64_t d, float pv, float *rsi, float *rinc,
                       cudaStream_t st) {
    if (n == 0) return MC_OK;
    k_row_scalars<<<unsigned((n + 255) / 256), 256, 0, st>>>(rowsum, n, d, pv, rsi, rinc), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// L1 over CSR rows with the pair-dependent prior (prior 0): the sequential float sum of
// |(c + pv) - (x + pv)| over the columns in ascending order, skipping only columns where
// both are zero (they add |pv - pv| = 0, so the sum equals the tiled kernel's walk over
// every column bit for bit, and the reference's sparse merge walk).  One warp per row,
// centers in groups of 32 (lane = center), two ways to walk a group:
//   per lane:  each lane merges the row's columns with its own center's nonzero list
//              ((column, value bits), ended by column 0xffffffff) -- divergent, about
//              |row| + max_c |center c| steps;
//   lockstep:  the row's columns merged with U_g, the ascending columns where any center of
//              the group is nonzero, and V_g[i][lane] the values there -- warp-uniform,
//              broadcast row and U_g loads, coalesced V_g rows; |row| + |U_g| steps.
// The group's walk is chosen per row from those step counts.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_l1_center_lists(const float *__restrict__ C, uint64_t d, uint2 *lists,
                                                         uint32_t *cnz) {
    __shared__ uint32_t wtot[8];
    __shared__ uint64_t base;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t c = blockIdx.x;
    const float *cr = C + uint64_t(c) * d;
    uint2 *out = lists + uint64_t(c) * (d + 1);
    if (t == 0) base = 0;
    __syncthreads();
    for (uint64_t j0 = 0; j0 < d; j0 += 256) {
        const uint64_t j = j0 + t;
        const float v = j < d ? cr[j] : 0.f;
        const bool nz = v != 0.f;  // -0 is a zero; NaN is kept
        const unsigned bal = __ballot_sync(0xffffffffu, nz);
        if (lane == 0) wtot[warp] = __popc(bal);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int q = 0; q < 8; ++q) {
            before += q < warp ? wtot[q] : 0u;
            total += wtot[q];
        }
        if (nz) out[base + before + __popc(bal & ((1u << lane) - 1u))] = make_uint2(uint32_t(j), __float_as_uint(v));
        __syncthreads();
        if (t == 0) base += total;
        __syncthreads();
    }
    if (t == 0) {
        out[base] = make_uint2(0xffffffffu, 0u);
        cnz[c] = uint32_t(base);
    }
}

__global__ void __launch_bounds__(256) k_l1_center_groups(const float *__restrict__ C, uint32_t k, uint64_t d,
                                                          uint32_t *U, float *V, uint32_t *usize) {
    __shared__ uint32_t wtot[8];
    __shared__ uint64_t base;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t g = blockIdx.x, c0 = g * 32;
    uint32_t *Ug = U + uint64_t(g) * (d + 1);
    float *Vg = V + uint64_t(g) * d * 32;
    if (t == 0) base = 0;
    __syncthreads();
    for (uint64_t j0 = 0; j0 < d; j0 += 256) {
        const uint64_t j = j0 + t;
        bool nz = false;
        if (j < d)
            for (uint32_t c = c0; c < c0 + 32 && c < k; ++c) nz |= C[uint64_t(c) * d + j] != 0.f;
        const unsigned bal = __ballot_sync(0xffffffffu, nz);
        if (lane == 0) wtot[warp] = __popc(bal);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int q = 0; q < 8; ++q) {
            before += q < warp ? wtot[q] : 0u;
            total += wtot[q];
        }
        if (nz) {
            const uint64_t pos = base + before + __popc(bal & ((1u << lane) - 1u));
            Ug[pos] = uint32_t(j);
            for (uint32_t l = 0; l < 32; ++l) {
                const uint32_t c = c0 + l;
                Vg[pos * 32 + l] = c < k ? C[uint64_t(c) * d + j] : 0.f;
            }
        }
        __syncthreads();
        if (t == 0) base += total;
        __syncthreads();
    }
    if (t == 0) {
        Ug[base] = 0xffffffffu;
        usize[g] = uint32_t(base);
    }
}

__global__ void __launch_bounds__(256) k_assign_l1_union(AssignArgs a, const uint2 *__restrict__ lists,
                                                         const uint32_t *__restrict__ cnz,
                                                         const uint32_t *__restrict__ U,
                                                         const float *__restrict__ V,
                                                         const uint32_t *__restrict__ usize) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    const uint32_t ng = (a.k + 31) / 32;
    for (uint64_t r = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; r < a.n; r += nw) {
        const uint64_t rb = a.indptr[r], re = a.indptr[r + 1];
        const uint32_t nr = uint32_t(re - rb);
        const uint32_t *ri = a.idx + rb;
        const float *rx = a.vals + rb;
        const double rs = a.rowsum[r];
        Best best;
        best_init(best);
        for (uint32_t g = 0; g < ng; ++g) {
            const uint32_t c = g * 32 + lane;
            const float pv = pair_scalars(a.prior, a.prior_sum, rs, c < a.k ? a.csum[c] : 0.0, a.d).pv;
            uint32_t cmax = c < a.k ? cnz[c] : 0u;
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
            float acc = 0.f;
            uint32_t p = 0, rc = nr ? ri[0] : 0xffffffffu;
            float rv = nr ? rx[0] : 0.f;
            if (uint64_t(nr + usize[g]) * 4 <= uint64_t(nr + cmax) * 5) {
                const uint32_t *Ug = U + uint64_t(g) * (a.d + 1);
                const float *Vg = V + uint64_t(g) * a.d * 32 + lane;
                uint32_t q = 0, uc = Ug[0];
                float uv = uc != 0xffffffffu ? Vg[0] : 0.f;
                while ((rc & uc) != 0xffffffffu) {  // warp-uniform
                    const bool tr = rc <= uc, tu = uc <= rc;
                    const float av = (tu ? uv : 0.f) + pv;
                    const float bv = (tr ? rv : 0.f) + pv;
                    acc = acc + fabsf(av - bv);
                    if (tr) {
                        ++p;
                        rc = p < nr ? ri[p] : 0xffffffffu;
                        rv = p < nr ? rx[p] : 0.f;
                    }
                    if (tu) {
                        uc = Ug[++q];
                        uv = uc != 0xffffffffu ? Vg[uint64_t(q) * 32] : 0.f;
                    }
                }
            } else if (c < a.k) {
                const uint2 *cl = lists + uint64_t(c) * (a.d + 1);
                uint2 ce = cl[0];
                while ((rc & ce.x) != 0xffffffffu) {  // per lane
                    const bool tr = rc <= ce.x, tc = ce.x <= rc;
                    const float av = (tc ? __uint_as_float(ce.y) : 0.f) + pv;
                    const float bv = (tr ? rv : 0.f) + pv;
                    acc = acc + fabsf(av - bv);
                    if (tr) {
                        ++p;
                        rc = p < nr ? ri[p] : 0xffffffffu;
                        rv = p < nr ? rx[p] : 0.f;
                    }
                    if (tc) ce = *++cl;
                }
            }
            if (c < a.k) {
                const float key = finish_key<L1>(acc);
                best_offer(best, key, c);
                if (a.dmode) write_dist(a, r, c, float(key_to_cost<L1>(key)));
            }
        }
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) best_merge_shfl(best, m);
        if (lane == 0) {
            const bool nan0 = best.v == __int_as_float(0xff800000);
            const double cost = nan0 ? __longlong_as_double(0x7ff8000000000000ll) : key_to_cost<L1>(best.v);
            a.asn[r] = best.j;
            a.costs[r] = double(float(cost));
        }
    }
}

// The same union walk, always in lock step and from registers: per 32-center group the
// warp walks the merge of the row's columns with the group's column union U_g (all lanes
// take the same step, lane = center), and nothing on the step's path waits for memory.  The
// row's next 32 (column, value) pairs and U_g's next 32 columns sit one per lane and are
// read by shuffle; the matching 32 x 32 slice of V_g (the group's center values at U_g's
// columns) is staged in shared memory, one conflict-free load per step.  Each window is
// refilled with coalesced loads when the walk has used it up.  Per (row, center) the sum is
// the same sequential float chain over the union, ascending, as in k_assign_l1_union, so
// the two kernels are bit-identical (autotuner variants).
__global__ void __launch_bounds__(256) k_assign_l1_lockstep(AssignArgs a, const uint32_t *__restrict__ U,
                                                            const float *__restrict__ V,
                                                            const uint32_t *__restrict__ usize) {
    __shared__ float vs[8][32][33];  // per warp: V_g rows q0 .. q0+31 (padded: no bank conflicts)
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t nw = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    const uint32_t ng = (a.k + 31) / 32;
    constexpr uint32_t END = 0xffffffffu;
    for (uint64_t r = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; r < a.n; r += nw) {
        const uint64_t rb = a.indptr[r], re = a.indptr[r + 1];
        const uint32_t nr = uint32_t(re - rb);
        const uint32_t *ri = a.idx + rb;
        const float *rx = a.vals + rb;
        const double rs = a.rowsum[r];
        Best best;
        best_init(best);
        for (uint32_t g = 0; g < ng; ++g) {
            const uint32_t c = g * 32 + lane;
            const float pv = pair_scalars(a.prior, a.prior_sum, rs, c < a.k ? a.csum[c] : 0.0, a.d).pv;
            const uint32_t nu = usize[g];
            const uint32_t *Ug = U + uint64_t(g) * (a.d + 1);
            const float *Vg = V + uint64_t(g) * a.d * 32;
            // windows: row elements p0 + lane, union columns q0 + lane, V_g rows q0 .. q0 + 31
            uint32_t p = 0, q = 0;
            uint32_t wrc = uint32_t(lane) < nr ? ri[lane] : END;
            float wrv = uint32_t(lane) < nr ? rx[lane] : 0.f;
            uint32_t wuc = uint32_t(lane) < nu ? Ug[lane] : END;
            __syncwarp();
            for (int i = 0; i < 32; ++i) vs[wib][i][lane] = uint32_t(i) < nu ? Vg[uint64_t(i) * 32 + lane] : 0.f;
            __syncwarp();
            uint32_t rc = __shfl_sync(0xffffffffu, wrc, 0), uc = __shfl_sync(0xffffffffu, wuc, 0);
            float rv = __shfl_sync(0xffffffffu, wrv, 0);
            float uv = vs[wib][0][lane];
            float acc = 0.f;
            while ((rc & uc) != END) {  // warp-uniform
                const bool tr = rc <= uc, tu = uc <= rc;
                const float av = (tu ? uv : 0.f) + pv;
                const float bv = (tr ? rv : 0.f) + pv;
                acc = acc + fabsf(av - bv);
                if (tr) {
                    ++p;
                    if ((p & 31u) == 0) {
                        const uint32_t e = p + uint32_t(lane);
                        wrc = e < nr ? ri[e] : END;
                        wrv = e < nr ? rx[e] : 0.f;
                    }
                    rc = __shfl_sync(0xffffffffu, wrc, int(p & 31u));
                    rv = __shfl_sync(0xffffffffu, wrv, int(p & 31u));
                }
                if (tu) {
                    ++q;
                    if ((q & 31u) == 0) {
                        const uint32_t e = q + uint32_t(lane);
                        wuc = e < nu ? Ug[e] : END;
                        __syncwarp();
                        for (int i = 0; i < 32; ++i)
                            vs[wib][i][lane] = q + uint32_t(i) < nu ? Vg[uint64_t(q + uint32_t(i)) * 32 + lane] : 0.f;
                        __syncwarp();
                    }
                    uc = __shfl_sync(0xffffffffu, wuc, int(q & 31u));
                    uv = uc != END ? vs[wib][q & 31u][lane] : 0.f;
                }
            }
            if (c < a.k) {
                const float key = finish_key<L1>(acc);
                best_offer(best, key, c);
                if (a.dmode) write_dist(a, r, c, float(key_to_cost<L1>(key)));
            }
        }
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) best_merge_shfl(best, m);
        if (lane == 0) {
            const bool nan0 = best.v == __int_as_float(0xff800000);
            const double cost = nan0 ? __longlong_as_double(0x7ff8000000000000ll) : key_to_cost<L1>(best.v);
            a.asn[r] = best.j;
            a.costs[r] = double(float(cost));
        }
    }
}

uint64_t l1_union_work_entries(uint32_t k, uint64_t d) {
    const uint64_t ng = (k + 31) / 32;
    return uint64_t(k) * (d + 1) * 2 + ng * (d + 1) * 33 + k + ng + 8;
}

int launch_assign_l1_union(const AssignArgs &a, const float *C, float *work, int sms, cudaStream_t st, bool tune) {
    if (a.k == 0) return MC_OK;
    const uint32_t ng = (a.k + 31) / 32;
    // work: lists (8-byte aligned first), U, V, cnz, usize
    uint2 *lists = reinterpret_cast<uint2 *>(work);
    uint32_t *U = reinterpret_cast<uint32_t *>(work + uint64_t(a.k) * (a.d + 1) * 2);
    float *V = reinterpret_cast<float *>(U + uint64_t(ng) * (a.d + 1));
    uint32_t *cnz = reinterpret_cast<uint32_t *>(V + uint64_t(ng) * a.d * 32);
    uint32_t *usize = cnz + a.k;
    k_l1_center_lists<<<a.k, 256, 0, st>>>(C, a.d, lists, cnz), note_launch();
    k_l1_center_groups<<<ng, 256, 0, st>>>(C, a.k, a.d, U, V, usize), note_launch();
    if (a.n) {
        // the register-window lockstep walk, or the per-row choice of lockstep / per-lane
        // merge from global memory: bit-identical, so the autotuner picks
        const unsigned blocks = unsigned(umin64((a.n + 7) / 8, uint64_t(sms) * 16));
        const uint64_t avg = (a.nnz + a.n - 1) / a.n;
        const std::string key = "csr_l1_union|g" + std::to_string(ng) + "|d" + tune_bucket(a.d) + "|nnz" +
                                tune_bucket(avg);
        return tune_launch(key, 2, 0, st, tune, [&](int v) -> int {
            if (v == 0) k_assign_l1_lockstep<<<blocks, 256, 0, st>>>(a, U, V, usize), note_launch();
            else k_assign_l1_union<<<blocks, 256, 0, st>>>(a, lists, cnz, U, V, usize), note_launch();
            MC_CUDA_TRY(cudaGetLastError());
            return MC_OK;
        });
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

template <int MSR, bool CSR>
static int tiled_t(const AssignArgs &a, bool pair, bool big, cudaStream_t st, bool tune) {
    if (pair) {
        constexpr int BM = 32;
        k_assign_tiled<MSR, true, 2, 2, CSR><<<unsigned((a.n + BM - 1) / BM), 256, 0, st>>>(a), note_launch();
    } else if (big) {
        // SQRL2 with kp % 128 == 0: 8x8 register tiles (128 rows per CTA) or 4x4 (64 rows);
        // same per-pair arithmetic, so the autotuner may pick either
        const std::string key = std::string("dense_sqrl2|") + (CSR ? "csr" : "dense") + "|k" +
                                std::to_string(a.kp) + "|d" + tune_bucket(a.d) + "|n" + tune_bucket(a.n);
        return tune_launch(key, 2, 0, st, tune, [&](int v) -> int {
            if (v == 0)
                k_assign_tiled<MSR, false, 8, 8, CSR><<<unsigned((a.n + 127) / 128), 256, 0, st>>>(a), note_launch();
            else
                k_assign_tiled<MSR, false, 4, 4, CSR><<<unsigned((a.n + 63) / 64), 256, 0, st>>>(a), note_launch();
            MC_CUDA_TRY(cudaGetLastError());
            return MC_OK;
        });
    } else {
        constexpr int BM = 64;
        k_assign_tiled<MSR, false, 4, 4, CSR><<<unsigned((a.n + BM - 1) / BM), 256, 0, st>>>(a), note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

uint32_t tiled_center_pad(uint32_t k, bool pair, int msr) {
    const uint32_t bn = pair ? 32 : ((msr == SQRL2 && k >= 128) ? 128 : 64);
    return (k + bn - 1) / bn * bn;
}

int launch_assign_tiled(const AssignArgs &a, bool csr, bool pair, cudaStream_t st, bool tune) {
    if (a.n == 0) return MC_OK;
    // 8x8 register tiles for SQRL2 with many centers, 4x4 otherwise
    const bool big = (a.msr == SQRL2 && a.kp % 128 == 0);
    switch (a.msr) {
        case SQRL2:
            return csr ? tiled_t<SQRL2, true>(a, pair, big, st, tune) : tiled_t<SQRL2, false>(a, pair, big, st, tune);
        case L1: return csr ? tiled_t<L1, true>(a, pair, false, st, tune) : tiled_t<L1, false>(a, pair, false, st, tune);
        case HELLINGER:
            return csr ? tiled_t<HELLINGER, true>(a, pair, false, st, tune)
                       : tiled_t<HELLINGER, false>(a, pair, false, st, tune);
        case MKL: return csr ? tiled_t<MKL, true>(a, pair, false, st, tune) : tiled_t<MKL, false>(a, pair, false, st, tune);
        case JSD: return csr ? tiled_t<JSD, true>(a, pair, false, st, tune) : tiled_t<JSD, false>(a, pair, false, st, tune);
        default: return fail(MC_EUNSUPPORTED, "measure not supported");
    }
}

template <int MSR, int KPL>
static int sparse_kpl(const AssignArgs &a, cudaStream_t st, int sms, bool tune) {
    const unsigned blocks = unsigned(umin64((a.n + 7) / 8, uint64_t(sms) * 16));
    const unsigned pblocks = unsigned(umin64((a.n + 15) / 16, uint64_t(sms) * 16));
    const uint64_t avg = a.n ? (a.nnz + a.n - 1) / a.n : 0;
    // 64 padded centers also admit the two-rows-per-warp kernel and (except JSD) the
    // column-band kernel
    const int nvar = (KPL == 2 && a.kp == 64) ? (MSR == JSD ? 5 : 6) : 3;
    const unsigned bblocks = unsigned(umin64((a.n + 127) / 128, uint64_t(sms)));
    const std::string key = "csr_sparse|msr" + std::to_string(MSR) + "|kpl" + std::to_string(KPL) + "|g" +
                            std::to_string((a.k + 32 * KPL - 1) / (32 * KPL)) + "|nnz" + tune_bucket(avg) + "|v" +
                            std::to_string(nvar);
    return tune_launch(key, nvar, 0, st, tune, [&](int v) -> int {
        if (v == 0) k_assign_sparse<MSR, KPL, 8><<<blocks, 256, 0, st>>>(a), note_launch();
        else if (v == 1) k_assign_sparse<MSR, KPL, 4><<<blocks, 256, 0, st>>>(a), note_launch();
        else if (v == 2) k_assign_sparse<MSR, KPL, 16><<<blocks, 256, 0, st>>>(a), note_launch();
        else if (v == 3) k_assign_sparse_pair<MSR, 8><<<pblocks, 256, 0, st>>>(a), note_launch();
        else if (v == 4) k_assign_sparse_pair<MSR, 4><<<pblocks, 256, 0, st>>>(a), note_launch();
        else if constexpr (MSR != JSD) {
            MC_CUDA_TRY(cudaFuncSetAttribute(k_assign_sparse_band<MSR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(kBandSmem)));
            k_assign_sparse_band<MSR><<<bblocks, kBandThreads, kBandSmem, st>>>(a), note_launch();
        }
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    });
}

template <int MSR>
static int sparse_t(const AssignArgs &a, cudaStream_t st, int sms, bool tune) {
    if (a.kp <= 32) return sparse_kpl<MSR, 1>(a, st, sms, tune);
    if (a.kp <= 64) return sparse_kpl<MSR, 2>(a, st, sms, tune);
    return sparse_kpl<MSR, 4>(a, st, sms, tune);
}

// the warp-per-row kernel reads 32 * KPL consecutive centers of a column per group; whole
// groups keep every column's gather 128-byte aligned (measured faster than padding to 4)
uint32_t sparse_center_pad(uint32_t k) {
    if (k <= 32) return 32;
    if (k <= 64) return 64;
    return (k + 127) / 128 * 128;
}

int launch_assign_sparse(const AssignArgs &a, cudaStream_t st, int sms, bool tune) {
    if (a.n == 0) return MC_OK;
    switch (a.msr) {
        case SQRL2: return sparse_t<SQRL2>(a, st, sms, tune);
        case L1: return sparse_t<L1>(a, st, sms, tune);
        case HELLINGER: return sparse_t<HELLINGER>(a, st, sms, tune);
        case MKL: return sparse_t<MKL>(a, st, sms, tune);
        case JSD: return sparse_t<JSD>(a, st, sms, tune);
        default: return fail(MC_EUNSUPPORTED, "sparse-dot path does not cover this measure");
    }
}

}  // namespace mc
