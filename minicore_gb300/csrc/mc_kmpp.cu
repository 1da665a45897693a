// D^2 / k-means++ seeding (include/minicore/optim/kmeans.h:49-215, n_local_trials == 1).
//
// Round c: draw newc from (w *) dist with uniform u[c] (FP64 inverse CDF, mc_reduce.cu),
// set asn[newc] = c, then update every row i != newc with dist[i] > 0:
// dist[i] = min(dist[i], msr(row i, row newc)) (COMPUTE_X, kmeans.h:189-201), and finally
// dist[newc] = 0.  Nothing returns to the host between rounds, so the k rounds are queued
// back to back on one stream.
#include "mc_kmpp.cuh"
#include "mc_tc.cuh"
#include "mc_tune.cuh"

#include <cmath>
#include <mutex>
#include <unordered_map>

namespace mc {

template <int MSR>
__device__ inline float kp_finish_key(float acc) {
    if (MSR == SQRL2) return acc;
    if (MSR == L1) return acc * 0.5f;
    if (MSR == HELLINGER) return sqrtf(acc);
    if (MSR == MKL) return post_divergence(acc);
    return post_divergence(acc * 0.5f);
}

template <int MSR>
__device__ inline double kp_cost(float acc) {
    const float key = kp_finish_key<MSR>(acc);
    if (MSR == L1) return double(key) * 2.0;
    if (MSR == HELLINGER) return double(key) * kSqrt1_2;
    return double(key);
}

template <int MSR>
__device__ inline void kp_elem(float &acc, float c, float x, const PairScalars &s) {
    if (MSR == SQRL2) {
        const float df = c - x;
        acc = fmaf(df, df, acc);
    } else if (MSR == L1) {
        const float a = c + s.pv, b = x + s.pv;
        acc = acc + fabsf(a - b);
    } else if (MSR == HELLINGER) {
        const float a = sqrtf(c * s.lhrsi + s.lhinc), b = sqrtf(x * s.rhrsi + s.rhinc);
        const float df = a - b;
        acc = fmaf(df, df, acc);
    } else if (MSR == MKL) {
        const float a = c * s.lhrsi + s.lhinc, b = x * s.rhrsi + s.rhinc;
        acc = fmaf(a, logf(a) - logf(b), acc);
    } else {
        const float a = c * s.lhrsi + s.lhinc, b = x * s.rhrsi + s.rhinc;
        const float m = a + b;
        const float t = (a * logf(a) + b * logf(b)) - m * logf(m * 0.5f);
        acc = acc + t;
    }
}

// Dense SQRL2 pruning.  Row i's distance to its nearest center a = asn[i] so far is
// D = dist[i], the FP32 sequential fmaf sum of d squared differences, so the exact squared
// distance e_a lies in [D / (1 + g), D / (1 - g)] with g = (d + 2) 2^-24 / (1 - (d + 2) 2^-24).
// By the triangle inequality the exact squared distance to the new center is at least
// (delta - sqrt(e_a))^2 when delta = ||new center - center a|| exceeds sqrt(e_a), and the FP32
// value the update would compute is at least (1 - g) times that.  When that lower bound is
// at or above D, the update's test (new < D) is false, so the row can skip the distance:
// the result is the same as computing it.  All bound arithmetic is FP64 with margins for its
// own rounding; non-finite distances are always evaluated.
__device__ __forceinline__ bool kp_prune(const KmppArgs &a, uint64_t i, double cur) {
    if (!(cur < 1e300)) return false;
    const double g = a.prune_g;
    const double ea = sqrt(cur / (1.0 - g)) * (1.0 + 0x1p-50);
    const double dl = a.cgap[a.asn[i]];
    if (!(dl > ea)) return false;
    const double t = dl - ea;
    return t * t * (1.0 - g) * (1.0 - 0x1p-48) >= cur;
}

// per round: a lower bound of ||X[new center] - X[center a]|| for every earlier center
// a < round (one warp each; FP64 sum of squared differences of the float rows, shrunk by its
// rounding bound)
__global__ void __launch_bounds__(256) k_kmpp_center_gap(const KmppArgs a, uint32_t round, double *gap) {
    const int lane = threadIdx.x & 31;
    const uint32_t ca = uint32_t((blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5);
    if (ca >= round) return;
    const uint64_t c = *a.newc, o = a.center_ids[ca];
    const float *x = a.X + c * a.d, *y = a.X + o * a.d;
    double s = 0.0;
    for (uint64_t j = lane; j < a.d; j += 32) {
        const double df = double(x[j]) - double(y[j]);
        s = fma(df, df, s);
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    if (lane == 0) gap[ca] = sqrt(s * (1.0 - double(a.d + 16) * 0x1p-50)) * (1.0 - 0x1p-50);
}

// first center from u[0]
__global__ void k_kmpp_first(const double *u, uint64_t n, uint64_t *newc, uint32_t *center_ids) {
    uint64_t fc = uint64_t(u[0] * double(n));
    if (fc >= n) fc = n - 1;
    *newc = fc;
    center_ids[0] = uint32_t(fc);
}

// after a draw: record the center, densify its row into cbuf
__global__ void k_kmpp_take(const KmppArgs a, uint32_t ci) {
    const uint64_t c = *a.newc;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        a.center_ids[ci] = uint32_t(c);
        a.asn[c] = ci;
    }
    if (!a.csr) {
        for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < a.d; j += gridDim.x * uint64_t(blockDim.x))
            a.cbuf[j] = a.X[c * a.d + j];
    } else {
        for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < a.d; j += gridDim.x * uint64_t(blockDim.x))
            a.cbuf[j] = 0.f;
    }
}

__global__ void k_kmpp_scatter(const KmppArgs a) {
    const uint64_t c = *a.newc;
    for (uint64_t p = a.indptr[c] + blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < a.indptr[c + 1];
         p += gridDim.x * uint64_t(blockDim.x))
        a.cbuf[a.idx[p]] = a.vals[p];
}

__global__ void k_kmpp_zero(const KmppArgs a) { a.dist[*a.newc] = 0.0; }

// dense rows: one thread per row; the row and the new center are read with float4 loads
// in 32-column chunks (16 loads in flight per thread), the reduction stays sequential over
// the columns (the oracle's order).  Rounds after the first also record the center
// (center_ids, asn) and zero its distance, so no separate launches are needed.
template <int MSR, bool VEC4>
__global__ void __launch_bounds__(256) k_kmpp_dense(const KmppArgs a, int first) {
    const uint64_t c = *a.newc;
    if (!first && blockIdx.x == 0 && threadIdx.x == 0) {
        a.center_ids[a.round] = uint32_t(c);
        a.asn[c] = a.round;
    }
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    double cur = 0.0;
    if (!first) {
        if (i == c) {
            a.dist[i] = 0.0;
            return;
        }
        cur = a.dist[i];
        if (cur <= 0.0) return;
        if (MSR == SQRL2 && a.cgap && kp_prune(a, i, cur)) return;
    }
    PairScalars s = {};
    if (MSR != SQRL2) s = pair_scalars(a.prior, a.prior_sum, a.rowsum[i], a.rowsum[c], a.d);
    const float *xr = a.X + i * a.d, *cr = a.X + c * a.d;
    float acc = 0.f;
    if (VEC4) {
        const float4 *x4 = reinterpret_cast<const float4 *>(xr), *c4 = reinterpret_cast<const float4 *>(cr);
        const uint64_t d4 = a.d / 4;
        uint64_t q = 0;
        for (; q + 8 <= d4; q += 8) {
            float4 xv[8], cv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                xv[u] = __ldg(x4 + q + u);
                cv[u] = __ldg(c4 + q + u);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                kp_elem<MSR>(acc, cv[u].x, xv[u].x, s);
                kp_elem<MSR>(acc, cv[u].y, xv[u].y, s);
                kp_elem<MSR>(acc, cv[u].z, xv[u].z, s);
                kp_elem<MSR>(acc, cv[u].w, xv[u].w, s);
            }
        }
        for (; q < d4; ++q) {
            const float4 xv = __ldg(x4 + q), cv = __ldg(c4 + q);
            kp_elem<MSR>(acc, cv.x, xv.x, s);
            kp_elem<MSR>(acc, cv.y, xv.y, s);
            kp_elem<MSR>(acc, cv.z, xv.z, s);
            kp_elem<MSR>(acc, cv.w, xv.w, s);
        }
    } else {
        for (uint64_t j = 0; j < a.d; ++j) kp_elem<MSR>(acc, __ldg(cr + j), __ldg(xr + j), s);
    }
    const double v = kp_cost<MSR>(acc);
    if (first) {
        a.dist[i] = (i == c) ? 0.0 : v;
    } else if (v < cur) {
        a.dist[i] = v;
        a.asn[i] = a.round;
    }
}

// CSR rows (any measure, any prior): sum over all columns of f(a_j, b0) (b0: transform of a
// zero entry) plus, over the row's nonzeros, f(a_j, b_j) - f(a_j, b0).  A warp takes 32 rows
// at a time: lane l evaluates row g0 + l's skip test, prior scalars and FP64 cost (a warp-wide
// FP64 instruction costs the SM's FP64 pipe the same whatever its active lanes, so these run
// once per 32 rows), and the warp walks each row's columns together (lanes strided, a butterfly
// for the float sum), as one warp per row did: the arithmetic and its order are unchanged.
template <int MSR>
__global__ void __launch_bounds__(256) k_kmpp_csr(const KmppArgs a, int first, uint32_t round) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    const uint64_t nwarps = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    const uint64_t c = *a.newc;
    const double csum = a.rowsum[c];
    for (uint64_t g0 = warp * 32; g0 < a.n; g0 += nwarps * 32) {
        const uint64_t my = g0 + uint64_t(lane);
        const bool go = my < a.n && (first || (my != c && !(a.dist[my] <= 0.0)));
        PairScalars sm = {0.f, 0.f, 0.f, 0.f, 0.f};
        uint64_t pbm = 0, pem = 0;
        if (go) {
            sm = pair_scalars(a.prior, a.prior_sum, a.rowsum[my], csum, a.d);
            pbm = a.indptr[my];
            pem = a.indptr[my + 1];
        }
        float accm = 0.f;
        unsigned todo = __ballot_sync(0xffffffffu, go);
        while (todo) {
            const int r = __ffs(todo) - 1;
            todo &= todo - 1;
            PairScalars s;
            s.pv = __shfl_sync(0xffffffffu, sm.pv, r);
            s.lhrsi = __shfl_sync(0xffffffffu, sm.lhrsi, r);
            s.rhrsi = __shfl_sync(0xffffffffu, sm.rhrsi, r);
            s.lhinc = __shfl_sync(0xffffffffu, sm.lhinc, r);
            s.rhinc = __shfl_sync(0xffffffffu, sm.rhinc, r);
            const uint64_t pb = __shfl_sync(0xffffffffu, pbm, r), pe = __shfl_sync(0xffffffffu, pem, r);
            float acc = 0.f;
            for (uint64_t j = lane; j < a.d; j += 32) kp_elem<MSR>(acc, a.cbuf[j], 0.f, s);
            for (uint64_t p = pb + lane; p < pe; p += 32) {
                const float cj = a.cbuf[a.idx[p]];
                float t1 = 0.f, t0 = 0.f;
                kp_elem<MSR>(t1, cj, a.vals[p], s);
                kp_elem<MSR>(t0, cj, 0.f, s);
                acc = acc + (t1 - t0);
            }
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1) acc = acc + __shfl_xor_sync(0xffffffffu, acc, m);
            if (lane == r) accm = acc;
        }
        if (!go) continue;
        double v = kp_cost<MSR>(accm);
        if (MSR == SQRL2 && v < 0.0) v = 0.0;
        if (first) {
            a.dist[my] = (my == c) ? 0.0 : v;
        } else if (v < a.dist[my]) {
            a.dist[my] = v;
            a.asn[my] = round;
        }
    }
}

// Block sums of the per-thread FP64 partials (s0, s1) of a 1024-thread CTA: a pairwise tree
// over the 32 lanes of each warp (shfl_xor), then over the 32 warp totals; warps that held no
// column add nothing (their totals are 0).  Every thread gets the sums.  A dependent FP64 add
// costs about 75 ns here and a warp-wide FP64 instruction occupies the SM's FP64 pipe for the
// whole warp whatever its active lanes, so the trees replace sequential walks in every warp.
__device__ __forceinline__ void kp_block_sum2(double s0, double s1, uint64_t d, double *w0, double *w1, double &u0,
                                              double &u1) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (uint64_t(wid) * 32 < d) {
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) {
            s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, m);
            s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, m);
        }
    } else {
        s0 = 0.0;
        s1 = 0.0;
    }
    if (lane == 0) {
        w0[wid] = s0;
        w1[wid] = s1;
    }
    __syncthreads();
    if (wid == 0) {
        double t0 = w0[lane], t1 = w1[lane];
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) {
            t0 = t0 + __shfl_xor_sync(0xffffffffu, t0, m);
            t1 = t1 + __shfl_xor_sync(0xffffffffu, t1, m);
        }
        if (lane == 0) {
            w0[32] = t0;
            w1[32] = t1;
        }
    }
    __syncthreads();
    u0 = w0[32];
    u1 = w1[32];
}

// CSR rows against the new center in O(nnz) per row (SQRL2, L1, MKL, Hellinger; rows whose
// pair keeps the prior pv = prior): per-center FP64 constants over all columns plus a float
// sum over the row's nonzeros, the arithmetic of the sparse-dot assignment kernel:
//   SQRL2  key = max(K0 + sum x (x - 2c), 0)                  K0 = sum c^2
//   L1     key = (K0 + sum |c' - (x+pv)| - |c' - pv|) / 2     K0 = sum |c' - pv|, c' = c + pv
//   MKL    key = K0 - log(rinc) K1 + sum a (log rinc - log b) K0 = sum a log a, K1 = sum a
//   Hell.  key = sqrt(K0 - 2 s K1 + d s^2 + sum ((t - sqrt b)^2 - (t - s)^2))
//          t = sqrt a (float), s = sqrt(rinc), K0 = sum t^2, K1 = sum t; the zero columns'
//          part sum (t - s)^2 is formed whole and the nonzero terms in FP64, so a row equal
//          to the center gets a distance near 0 (a sum of a + b - 2 sqrt(ab) cancels to the
//          float rounding of its terms, which the square root lifts to ~1e-4)
//   JSD    key = (Z[g] + sum (b log b - r log r) + sum (m0 log(m0/2) - m1 log(m1/2))) / 2
//          m0 = a + r, m1 = a + b, r = rinc of the row's group g, Z[g] = sum over all
//          columns of f(a, r) (k_kmpp_jsd_zcol)
// with a = c * lhrsi + lhinc (center side), b = x * rhrsi + rhinc (row side).  Rows whose pair
// moves the prior to the smallest-pv floor take the column loop of k_kmpp_csr.
// k_kmpp_center_prep (one CTA) writes ct (c, c', a or sqrt a per column) and K0, K1: thread t
// adds columns t, t+1024, ... in FP64; the 32 lanes of a warp, then the 32 warps, are added by
// pairwise trees (kp_block_sum2).
template <int MSR>
__global__ void __launch_bounds__(1024) k_kmpp_center_prep(const KmppArgs a) {
    __shared__ double w0[33], w1[33];
    const uint64_t c = *a.newc;
    const float pv = float(a.prior);
    float rsi = 0.f, inc = 0.f;
    if (MSR != SQRL2) side_scalars(pv, a.rowsum[c], a.d, rsi, inc);
    double s0 = 0.0, s1 = 0.0;
    for (uint64_t j = threadIdx.x; j < a.d; j += 1024) {
        const float x = a.cbuf[j];
        float t;
        if (MSR == SQRL2) {
            t = x;
            s0 = s0 + double(x) * double(x);
        } else if (MSR == L1) {
            t = x + pv;
            s0 = s0 + double(fabsf(t - pv));
        } else {
            const float av = x * rsi + inc;
            if (MSR == JSD) {
                t = av;
            } else if (MSR == MKL) {
                t = av;
                s0 = s0 + double(av) * double(logf(av));
                s1 = s1 + double(av);
            } else {
                t = sqrtf(av);
                s0 = s0 + double(t) * double(t);
                s1 = s1 + double(t);
            }
        }
        a.ct[j] = t;
    }
    double u0, u1;
    kp_block_sum2(s0, s1, a.d, w0, w1, u0, u1);
    if (threadIdx.x == 0 && MSR != JSD) {
        a.cconst[0] = u0;
        a.cconst[1] = u1;
    }
}

// JSD: Z[g] = sum over all columns of f(a_j, r_g), one warp per group (lane l adds columns l,
// l+32, ... in FP64; the lane partials are added in lane order)
__global__ void __launch_bounds__(256) k_kmpp_jsd_zcol(const KmppArgs a) {
    const int lane = threadIdx.x & 31;
    const uint64_t g = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    if (g >= a.ngrp) return;  // whole warp
    const float b = a.gval[g];
    const float blb = b * logf(b);
    double s = 0.0;
    for (uint64_t j = lane; j < a.d; j += 32) {
        const float av = a.ct[j];
        const float m = av + b;
        s = s + double((av * logf(av) + blb) - m * logf(m * 0.5f));
    }
    double t = 0.0;
#pragma unroll
    for (int l = 0; l < 32; ++l) t = t + __shfl_sync(0xffffffffu, s, l);
    if (lane == 0) a.cconst[g] = t;
}

// the rows of one round: ct = transformed center, raw = densified center.  A warp takes 32
// rows at a time: lane l evaluates row g0 + l's skip test, prior scalars and FP64 key (one
// FP64 warp instruction per 32 rows), and the warp walks each row's nonzeros together (lanes
// strided over the nonzeros, a butterfly for the float sum), as one warp per row did: the
// arithmetic and its order are unchanged.
template <int MSR>
__device__ __forceinline__ void kp_nnz_rows(const KmppArgs &a, int first, uint32_t round, uint64_t c,
                                            const float *ct, const float *raw, double K0, double K1) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    const uint64_t nwarps = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    const double csum = a.rowsum[c];
    const float fp = float(a.prior);
    for (uint64_t g0 = warp * 32; g0 < a.n; g0 += nwarps * 32) {
        const uint64_t my = g0 + uint64_t(lane);
        const bool go = my < a.n && (first || (my != c && !(a.dist[my] <= 0.0)));
        PairScalars sm = {0.f, 0.f, 0.f, 0.f, 0.f};
        uint64_t pbm = 0, pem = 0;
        float rincm = 0.f, rlm = 0.f, rlrm = 0.f, srincm = 0.f;
        bool fastm = true;
        if (go) {
            sm = pair_scalars(a.prior, a.prior_sum, a.rowsum[my], csum, a.d);
            pbm = a.indptr[my];
            pem = a.indptr[my + 1];
            fastm = MSR == SQRL2 || sm.pv == fp;
            rincm = (MSR == JSD) ? a.gval[a.grp[my]] : sm.rhinc;
            rlrm = (MSR == JSD) ? rincm * logf(rincm) : 0.f;
            rlm = (MSR == MKL) ? logf(rincm) : 0.f;
            srincm = (MSR == HELLINGER) ? sqrtf(rincm) : 0.f;
        }
        float accm = 0.f;     // lane l: row g0 + l's float sum
        double bsumm = 0.0;   // lane l: row g0 + l's FP64 sum (Hellinger, JSD)
        unsigned todo = __ballot_sync(0xffffffffu, go);
        while (todo) {
            const int r = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint64_t pb = __shfl_sync(0xffffffffu, pbm, r), pe = __shfl_sync(0xffffffffu, pem, r);
            const bool fast = __shfl_sync(0xffffffffu, fastm ? 1 : 0, r) != 0;
            if (fast) {
                const float rsi = __shfl_sync(0xffffffffu, sm.rhrsi, r);
                const float rinc = __shfl_sync(0xffffffffu, rincm, r);
                const float rlr = __shfl_sync(0xffffffffu, rlrm, r);
                const float rl = __shfl_sync(0xffffffffu, rlm, r);
                const float srinc = __shfl_sync(0xffffffffu, srincm, r);
                float acc = 0.f;
                double bsum = 0.0;
#pragma unroll 4
                for (uint64_t p = pb + lane; p < pe; p += 32) {
                    const float x = a.vals[p];
                    const float cj = ct[a.idx[p]];
                    if (MSR == SQRL2) {
                        acc = fmaf(x, x - 2.f * cj, acc);
                    } else if (MSR == L1) {
                        acc = acc + (fabsf(cj - (x + fp)) - fabsf(cj - fp));
                    } else if (MSR == MKL) {
                        acc = fmaf(cj, rl - logf(x * rsi + rinc), acc);
                    } else if (MSR == JSD) {
                        const float b = x * rsi + rinc;
                        const float m0 = cj + rinc, m1 = cj + b;
                        acc = acc + (m0 * logf(m0 * 0.5f) - m1 * logf(m1 * 0.5f));
                        bsum = bsum + double(b * logf(b) - rlr);
                    } else {
                        // (sqrt a - sqrt b)^2 - (sqrt a - sqrt r)^2 in FP64 from the float roots
                        const float b = x * rsi + rinc;
                        const double dd = double(cj) - double(sqrtf(b)), de = double(cj) - double(srinc);
                        bsum = bsum + (dd * dd - de * de);
                    }
                }
#pragma unroll
                for (int m = 16; m >= 1; m >>= 1) {
                    acc = acc + __shfl_xor_sync(0xffffffffu, acc, m);
                    if (MSR == HELLINGER || MSR == JSD) bsum = bsum + __shfl_xor_sync(0xffffffffu, bsum, m);
                }
                if (lane == r) {
                    accm = acc;
                    bsumm = bsum;
                }
            } else {
                PairScalars s;
                s.pv = __shfl_sync(0xffffffffu, sm.pv, r);
                s.lhrsi = __shfl_sync(0xffffffffu, sm.lhrsi, r);
                s.rhrsi = __shfl_sync(0xffffffffu, sm.rhrsi, r);
                s.lhinc = __shfl_sync(0xffffffffu, sm.lhinc, r);
                s.rhinc = __shfl_sync(0xffffffffu, sm.rhinc, r);
                float acc = 0.f;
                for (uint64_t j = lane; j < a.d; j += 32) kp_elem<MSR>(acc, raw[j], 0.f, s);
                for (uint64_t p = pb + lane; p < pe; p += 32) {
                    const float cj = raw[a.idx[p]];
                    float t1 = 0.f, t0 = 0.f;
                    kp_elem<MSR>(t1, cj, a.vals[p], s);
                    kp_elem<MSR>(t0, cj, 0.f, s);
                    acc = acc + (t1 - t0);
                }
#pragma unroll
                for (int m = 16; m >= 1; m >>= 1) acc = acc + __shfl_xor_sync(0xffffffffu, acc, m);
                if (lane == r) accm = acc;
            }
        }
        if (!go) continue;
        double v;
        if (fastm) {
            float key;
            if (MSR == SQRL2) {
                double t = K0 + double(accm);
                key = float(t < 0.0 ? 0.0 : t);
                v = double(key);
            } else if (MSR == L1) {
                key = float(K0 + double(accm)) * 0.5f;
                v = double(key) * 2.0;
            } else if (MSR == MKL) {
                key = post_divergence(float(K0 - double(rlm) * K1 + double(accm)));
                v = double(key);
            } else if (MSR == JSD) {
                key = post_divergence(float((a.cconst[a.grp[my]] + bsumm + double(accm)) * 0.5));
                v = double(key);
            } else {
                const double sr = double(srincm);
                double t = (K0 - 2.0 * sr * K1 + double(a.d) * sr * sr) + bsumm;
                key = float(sqrt(t < 0.0 ? 0.0 : t));
                v = double(key) * kSqrt1_2;
            }
        } else {
            v = kp_cost<MSR>(accm);
            if (MSR == SQRL2 && v < 0.0) v = 0.0;
        }
        if (first) {
            a.dist[my] = (my == c) ? 0.0 : v;
        } else if (v < a.dist[my]) {
            a.dist[my] = v;
            a.asn[my] = round;
        }
    }
}

template <int MSR>
__global__ void __launch_bounds__(256) k_kmpp_csr_nnz(const KmppArgs a, int first, uint32_t round) {
    const uint64_t c = *a.newc;
    const double K0 = (MSR == JSD) ? 0.0 : a.cconst[0], K1 = (MSR == JSD) ? 0.0 : a.cconst[1];
    kp_nnz_rows<MSR>(a, first, round, c, a.ct, a.cbuf, K0, K1);
}

// Small d (2 d floats of shared memory): one launch per round.  Every CTA densifies the new
// center's CSR row into shared memory, forms ct and K0, K1 with the code and summation order
// of k_kmpp_center_prep (1024 threads), then runs its share of the rows; CTA 0 also records
// the center and zeroes its distance (k_kmpp_take / k_kmpp_zero).  Same results as the
// three-launch sequence.
template <int MSR>
__global__ void __launch_bounds__(1024) k_kmpp_csr_fused(const KmppArgs a, int first, uint32_t round) {
    extern __shared__ float sm_kp[];
    float *raw = sm_kp, *ct = sm_kp + a.d;
    __shared__ double w0[33], w1[33];
    const uint64_t c = *a.newc;
    const int tid = threadIdx.x;
    for (uint64_t j = tid; j < a.d; j += 1024) raw[j] = 0.f;
    __syncthreads();
    for (uint64_t p = a.indptr[c] + tid; p < a.indptr[c + 1]; p += 1024) raw[a.idx[p]] = a.vals[p];
    if (blockIdx.x == 0 && tid == 0) {
        a.center_ids[round] = uint32_t(c);
        a.asn[c] = round;
        if (!first) a.dist[c] = 0.0;
    }
    __syncthreads();
    const float pv = float(a.prior);
    float rsi = 0.f, inc = 0.f;
    if (MSR != SQRL2) side_scalars(pv, a.rowsum[c], a.d, rsi, inc);
    double s0 = 0.0, s1 = 0.0;
    for (uint64_t j = tid; j < a.d; j += 1024) {
        const float x = raw[j];
        float t;
        if (MSR == SQRL2) {
            t = x;
            s0 = s0 + double(x) * double(x);
        } else if (MSR == L1) {
            t = x + pv;
            s0 = s0 + double(fabsf(t - pv));
        } else {
            const float av = x * rsi + inc;
            if (MSR == MKL) {
                t = av;
                s0 = s0 + double(av) * double(logf(av));
                s1 = s1 + double(av);
            } else {
                t = sqrtf(av);
                s0 = s0 + double(t) * double(t);
                s1 = s1 + double(t);
            }
        }
        ct[j] = t;
    }
    double u0, u1;
    kp_block_sum2(s0, s1, a.d, w0, w1, u0, u1);
    kp_nnz_rows<MSR>(a, first, round, c, ct, raw, u0, u1);
}

__device__ __forceinline__ void kp_cp_async16(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(uint32_t(__cvta_generic_to_shared(dst))),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}

// dense rows with d % 4 == 0 and 16-byte aligned rows: a CTA of 128 threads (one row each)
// stages 32-column chunks of its 128 rows and of the new center in shared memory with
// cp.async (coalesced, double-buffered); each thread then reduces its row sequentially over
// the columns.  Same per-row arithmetic and bookkeeping as k_kmpp_dense.
template <int MSR>
__global__ void __launch_bounds__(128) k_kmpp_dense_staged(const KmppArgs a, int first) {
    __shared__ __align__(16) float xs[2][128][36];
    __shared__ __align__(16) float cs[2][32];
    const uint64_t c = *a.newc;
    if (!first && blockIdx.x == 0 && threadIdx.x == 0) {
        a.center_ids[a.round] = uint32_t(c);
        a.asn[c] = a.round;
    }
    const int t = threadIdx.x;
    const uint64_t row0 = uint64_t(blockIdx.x) * 128;
    const uint64_t i = row0 + t;
    bool active = i < a.n;
    double cur = 0.0;
    if (active && !first) {
        if (i == c) {
            a.dist[i] = 0.0;
            active = false;
        } else {
            cur = a.dist[i];
            if (cur <= 0.0) active = false;
            else if (MSR == SQRL2 && a.cgap && kp_prune(a, i, cur)) active = false;
        }
    }
    // rows that need no distance are not staged; a CTA with none left stops here
    __shared__ unsigned char act_s[128];
    act_s[t] = active ? 1 : 0;
    if (!__syncthreads_or(active ? 1 : 0)) return;
    PairScalars s = {};
    if (active && MSR != SQRL2) s = pair_scalars(a.prior, a.prior_sum, a.rowsum[i], a.rowsum[c], a.d);
    const uint64_t d = a.d;
    const uint64_t nchunk = (d + 31) / 32;
    auto stage = [&](uint64_t ci, int buf) {
        const uint64_t k0 = ci * 32;
        const int kmax = int(umin64(32, d - k0));
        for (int e = t; e < 128 * 8; e += 128) {
            const int r = e >> 3, q4 = e & 7;
            const bool ok = act_s[r] && 4 * q4 < kmax;
            kp_cp_async16(&xs[buf][r][4 * q4], ok ? a.X + (row0 + r) * d + k0 + 4 * q4 : a.X, ok ? 16 : 0);
        }
        if (t < 8) {
            const bool ok = 4 * t < kmax;
            kp_cp_async16(&cs[buf][4 * t], ok ? a.X + c * d + k0 + 4 * t : a.X, ok ? 16 : 0);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    float acc = 0.f;
    stage(0, 0);
    for (uint64_t ci = 0; ci < nchunk; ++ci) {
        const int buf = int(ci & 1);
        if (ci + 1 < nchunk) {
            stage(ci + 1, buf ^ 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const int kmax = int(umin64(32, d - ci * 32));
        if (active) {
            if (kmax == 32) {
#pragma unroll
                for (int kk = 0; kk < 32; ++kk) kp_elem<MSR>(acc, cs[buf][kk], xs[buf][t][kk], s);
            } else {
                for (int kk = 0; kk < kmax; ++kk) kp_elem<MSR>(acc, cs[buf][kk], xs[buf][t][kk], s);
            }
        }
        __syncthreads();  // buffer buf is restaged two chunks later
    }
    if (!active) return;
    const double v = kp_cost<MSR>(acc);
    if (first) {
        a.dist[i] = (i == c) ? 0.0 : v;
    } else if (v < cur) {
        a.dist[i] = v;
        a.asn[i] = a.round;
    }
}

// The same with persistent CTAs: each of sms x 4 CTAs walks its row tiles (stride gridDim)
// as one stream of (tile, 32-column chunk) items, staging the next item while it evaluates
// the current one, across tile boundaries too (the next tile's skip flags are read first).
// With one tile per CTA, every CTA waits for its first chunk from DRAM before any work; here
// the copies of the next tile overlap the last chunk of the current one.  Same per-row
// arithmetic and bookkeeping as k_kmpp_dense_staged.
template <int MSR>
__global__ void __launch_bounds__(128) k_kmpp_dense_persist(const KmppArgs a, int first) {
    __shared__ __align__(16) float xs[2][128][36];
    __shared__ __align__(16) float cs[2][32];
    __shared__ unsigned char act_s[2][128];
    const uint64_t c = *a.newc;
    if (!first && blockIdx.x == 0 && threadIdx.x == 0) {
        a.center_ids[a.round] = uint32_t(c);
        a.asn[c] = a.round;
    }
    const int t = threadIdx.x;
    const uint64_t d = a.d, nchunk = (d + 31) / 32, ntiles = (a.n + 127) / 128;
    auto row_state = [&](uint64_t m, bool &act, double &cur, PairScalars &ps) {
        const uint64_t i = m * 128 + uint64_t(t);
        act = i < a.n;
        cur = 0.0;
        ps = PairScalars{0.f, 0.f, 0.f, 0.f, 0.f};
        if (act && !first) {
            if (i == c) {
                a.dist[i] = 0.0;
                act = false;
            } else {
                cur = a.dist[i];
                if (cur <= 0.0) act = false;
                else if (MSR == SQRL2 && a.cgap && kp_prune(a, i, cur)) act = false;
            }
        }
        if (act && MSR != SQRL2) ps = pair_scalars(a.prior, a.prior_sum, a.rowsum[i], a.rowsum[c], a.d);
    };
    auto stage = [&](uint64_t m, uint64_t ci, int buf, int ab) {
        const uint64_t k0 = ci * 32, row0 = m * 128;
        const int kmax = int(umin64(32, d - k0));
        for (int e = t; e < 128 * 8; e += 128) {
            const int r = e >> 3, q4 = e & 7;
            const bool ok = act_s[ab][r] && 4 * q4 < kmax;
            kp_cp_async16(&xs[buf][r][4 * q4], ok ? a.X + (row0 + r) * d + k0 + 4 * q4 : a.X, ok ? 16 : 0);
        }
        if (t < 8) {
            const bool ok = 4 * t < kmax;
            kp_cp_async16(&cs[buf][4 * t], ok ? a.X + c * d + k0 + 4 * t : a.X, ok ? 16 : 0);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    uint64_t m = blockIdx.x;
    if (m >= ntiles) return;
    bool active;
    double cur;
    PairScalars ps;
    row_state(m, active, cur, ps);
    int ab = 0, buf = 0;
    act_s[ab][t] = active ? 1 : 0;
    __syncthreads();
    stage(m, 0, buf, ab);
    float acc = 0.f;
    for (;;) {
        for (uint64_t ci = 0; ci < nchunk; ++ci) {
            const bool last = ci + 1 == nchunk;
            const uint64_t mn = m + gridDim.x;
            const bool have_next = !last || mn < ntiles;
            bool act2 = false;
            double cur2 = 0.0;
            PairScalars ps2 = PairScalars{0.f, 0.f, 0.f, 0.f, 0.f};
            if (!last) {
                stage(m, ci + 1, buf ^ 1, ab);
            } else if (have_next) {
                row_state(mn, act2, cur2, ps2);
                act_s[ab ^ 1][t] = act2 ? 1 : 0;
                __syncthreads();
                stage(mn, 0, buf ^ 1, ab ^ 1);
            }
            if (have_next) asm volatile("cp.async.wait_group 1;" ::: "memory");
            else asm volatile("cp.async.wait_group 0;" ::: "memory");
            __syncthreads();
            const int kmax = int(umin64(32, d - ci * 32));
            if (active) {
                if (kmax == 32) {
#pragma unroll
                    for (int kk = 0; kk < 32; ++kk) kp_elem<MSR>(acc, cs[buf][kk], xs[buf][t][kk], ps);
                } else {
                    for (int kk = 0; kk < kmax; ++kk) kp_elem<MSR>(acc, cs[buf][kk], xs[buf][t][kk], ps);
                }
            }
            __syncthreads();  // buffer buf is restaged in the next iteration
            buf ^= 1;
            if (last) {
                if (active) {
                    const uint64_t i = m * 128 + uint64_t(t);
                    const double v = kp_cost<MSR>(acc);
                    if (first) {
                        a.dist[i] = (i == c) ? 0.0 : v;
                    } else if (v < cur) {
                        a.dist[i] = v;
                        a.asn[i] = a.round;
                    }
                }
                if (!have_next) return;
                m = mn;
                active = act2;
                cur = cur2;
                ps = ps2;
                ab ^= 1;
                acc = 0.f;
            }
        }
    }
}

// CSR update in one launch per round: the center row and its transform fit in 32 KB
static bool kmpp_csr_fused_ok(const KmppArgs &a) { return a.csr && a.msr != JSD && a.ct && a.d <= 4096; }

template <int MSR>
static int update_t(const KmppArgs &a, int first, uint32_t round, int sms, cudaStream_t st) {
    if (!a.csr) {
        KmppArgs b = a;
        b.round = round;
        const bool vec4 = a.d % 4 == 0 && (reinterpret_cast<uintptr_t>(a.X) & 15) == 0;
        if (vec4) {
            // rows staged through shared memory, or read directly with float4 loads (the same
            // per-row arithmetic): the autotuner keeps the faster for this measure and width
            const std::string key = "kmpp_dense|msr" + std::to_string(MSR) + "|d" + tune_bucket(a.d) + "|n" +
                                    tune_bucket(a.n);
            return tune_launch(key, 3, 0, st, true, [&](int v) -> int {
                if (v == 0)
                    k_kmpp_dense_staged<MSR><<<unsigned((a.n + 127) / 128), 128, 0, st>>>(b, first), note_launch();
                else if (v == 1)
                    k_kmpp_dense<MSR, true><<<unsigned((a.n + 255) / 256), 256, 0, st>>>(b, first), note_launch();
                else
                    k_kmpp_dense_persist<MSR><<<unsigned(umin64((a.n + 127) / 128, uint64_t(sms) * 4)), 128, 0, st>>>(
                        b, first), note_launch();
                MC_CUDA_TRY(cudaGetLastError());
                return MC_OK;
            });
        }
        k_kmpp_dense<MSR, false><<<unsigned((a.n + 255) / 256), 256, 0, st>>>(b, first), note_launch();
    } else {
        const unsigned blocks = unsigned(umin64((a.n + 7) / 8, uint64_t(sms) * 16));
        if (MSR != JSD && a.ct && kmpp_csr_fused_ok(a)) {
            const unsigned fb = unsigned(umin64((a.n + 31) / 32, uint64_t(sms) * 2));
            k_kmpp_csr_fused<MSR><<<fb, 1024, 2 * a.d * sizeof(float), st>>>(a, first, round), note_launch();
        } else if (a.ct) {
            k_kmpp_center_prep<MSR><<<1, 1024, 0, st>>>(a), note_launch();
            if (MSR == JSD) k_kmpp_jsd_zcol<<<unsigned((a.ngrp + 7) / 8), 256, 0, st>>>(a), note_launch();
            k_kmpp_csr_nnz<MSR><<<blocks, 256, 0, st>>>(a, first, round), note_launch();
        } else {
            k_kmpp_csr<MSR><<<blocks, 256, 0, st>>>(a, first, round), note_launch();
        }
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

static int update(const KmppArgs &a, int first, uint32_t round, int sms, cudaStream_t st) {
    switch (a.msr) {
        case SQRL2: return update_t<SQRL2>(a, first, round, sms, st);
        case L1: return update_t<L1>(a, first, round, sms, st);
        case HELLINGER: return update_t<HELLINGER>(a, first, round, sms, st);
        case MKL: return update_t<MKL>(a, first, round, sms, st);
        case JSD: return update_t<JSD>(a, first, round, sms, st);
        default: return fail(MC_EUNSUPPORTED, "measure not supported");
    }
}

// ------------------------------------------------------------------------------------
// Persistent seeding for small dense matrices: one thread-block cluster runs every round.
// The rounds above cost four to five dependent launches each (about 40 us per round at
// serving sizes, where the distance pass itself takes one or two); here the cluster's CTAs
// update their own 32-row blocks of the distances, leave each block's pairwise FP64 sum in
// `blk`, and meet at a cluster barrier; CTA 0 then builds every chunk's tree of 256 block
// sums and the tree over the chunk totals, descends them with u[r] S to one row (the
// arithmetic and descent of k_det_chunks / k_det_draw), and the CTAs meet again.  The
// barriers are the hardware's cluster barriers (the cluster's CTAs are co-scheduled), taken
// by every thread of every CTA the same number of times.  Distances, assignments, center ids
// and draws are bit-identical to the launch-per-round path.
// ------------------------------------------------------------------------------------
constexpr int kKcThreads = 512;
constexpr uint64_t kKcMaxRows = 32 * uint64_t(kDetChunk);  // 32 chunks: CTA 0's trees fit shared memory

__device__ __forceinline__ uint32_t kc_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t kc_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster; writes before it are visible to reads after it
__device__ __forceinline__ void kc_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// one row's update in round `round` (k_kmpp_dense's arithmetic); returns its distance after it
template <int MSR, bool VEC4>
__device__ __forceinline__ double kc_row(const KmppArgs &a, uint64_t i, uint64_t c, bool first, uint32_t round) {
    double cur = 0.0;
    if (!first) {
        if (i == c) {
            a.dist[i] = 0.0;
            return 0.0;
        }
        cur = a.dist[i];
        if (cur <= 0.0) return cur;
    }
    PairScalars s = {};
    if (MSR != SQRL2) s = pair_scalars(a.prior, a.prior_sum, a.rowsum[i], a.rowsum[c], a.d);
    const float *xr = a.X + i * a.d, *cr = a.X + c * a.d;
    float acc = 0.f;
    if (VEC4) {
        const float4 *x4 = reinterpret_cast<const float4 *>(xr), *c4 = reinterpret_cast<const float4 *>(cr);
        const uint64_t d4 = a.d / 4;
        uint64_t q = 0;
        for (; q + 8 <= d4; q += 8) {
            float4 xv[8], cv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                xv[u] = __ldg(x4 + q + u);
                cv[u] = __ldg(c4 + q + u);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                kp_elem<MSR>(acc, cv[u].x, xv[u].x, s);
                kp_elem<MSR>(acc, cv[u].y, xv[u].y, s);
                kp_elem<MSR>(acc, cv[u].z, xv[u].z, s);
                kp_elem<MSR>(acc, cv[u].w, xv[u].w, s);
            }
        }
        for (; q < d4; ++q) {
            const float4 xv = __ldg(x4 + q), cv = __ldg(c4 + q);
            kp_elem<MSR>(acc, cv.x, xv.x, s);
            kp_elem<MSR>(acc, cv.y, xv.y, s);
            kp_elem<MSR>(acc, cv.z, xv.z, s);
            kp_elem<MSR>(acc, cv.w, xv.w, s);
        }
    } else {
        for (uint64_t j = 0; j < a.d; ++j) kp_elem<MSR>(acc, __ldg(cr + j), __ldg(xr + j), s);
    }
    const double v = kp_cost<MSR>(acc);
    if (first) {
        const double nv = (i == c) ? 0.0 : v;
        a.dist[i] = nv;
        return nv;
    }
    if (v < cur) {
        a.dist[i] = v;
        a.asn[i] = round;
        return v;
    }
    return cur;
}

// pairwise sum of 32 consecutive values (det_block32's tree)
__device__ __forceinline__ double kc_block32(const double *v0) {
    double v[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) v[e] = v0[e];
#pragma unroll
    for (int sft = 1; sft < 32; sft <<= 1)
#pragma unroll
        for (int e = 0; e < 32; e += 2 * sft) v[e] = v[e] + v[e + sft];
    return v[0];
}

template <int MSR, bool VEC4>
__global__ void __launch_bounds__(kKcThreads, 1) k_kmpp_cluster(const KmppArgs a, const double *u, double *blk) {
    extern __shared__ double H[];  // CTA 0: [chunks][512] heaps of the block sums (leaves at 256..511)
    __shared__ double sval[kKcThreads + 32];
    __shared__ double T[2 * 32], E[64];
    __shared__ uint64_t sm_g, sm_b;
    __shared__ double sm_r;
    __shared__ int sm_pos;
    const int t = threadIdx.x;
    const uint32_t rank = kc_rank(), CS = kc_size();
    const uint64_t n = a.n, nblk = (n + 31) / 32;
    const uint64_t G = det_chunks(n), P = det_leaves(n);
    const uint64_t b_lo = nblk * rank / CS, b_hi = nblk * (rank + 1) / CS;  // this CTA's 32-row blocks
    const bool weighted = a.w != nullptr;
    uint64_t c = uint64_t(u[0] * double(n));
    if (c >= n) c = n - 1;
    for (uint32_t round = 0; round < a.k; ++round) {
        const bool first = round == 0;
        if (!first) c = __ldcg(a.newc);
        if (rank == 0 && t == 0) {
            a.center_ids[round] = uint32_t(c);
            if (!first) a.asn[c] = round;
        }
        // ---- distances of this CTA's rows, 512 at a time, and their 32-row block sums ----
        for (uint64_t r0 = b_lo * 32; r0 < b_hi * 32; r0 += kKcThreads) {
            const uint64_t i = r0 + uint64_t(t);
            double v = 0.0;
            if (i < b_hi * 32 && i < n) {
                v = kc_row<MSR, VEC4>(a, i, c, first, round);
                if (weighted) v = v * a.w[i];
            }
            sval[t] = v;
            __syncthreads();
            if (t < kKcThreads / 32) {
                const uint64_t b = r0 / 32 + uint64_t(t);
                if (b < b_hi) blk[b] = kc_block32(sval + 32 * t);
            }
            __syncthreads();
        }
        if (round + 1 == a.k) break;
        kc_sync();
        // ---- CTA 0: the draw of the next round ----
        if (rank == 0) {
            for (uint64_t e = t; e < G * 256; e += kKcThreads) {
                const uint64_t g = e >> 8, l = e & 255, b = g * 256 + l;
                H[g * 512 + 256 + l] = b < nblk ? __ldcg(blk + b) : 0.0;
            }
            __syncthreads();
            for (uint64_t lv = 128; lv >= 1; lv >>= 1) {
                for (uint64_t e = t; e < G * lv; e += kKcThreads) {
                    const uint64_t g = e / lv, j = lv + e % lv;
                    H[g * 512 + j] = H[g * 512 + 2 * j] + H[g * 512 + 2 * j + 1];
                }
                __syncthreads();
            }
            for (uint64_t g = t; g < P; g += kKcThreads) T[P + g] = g < G ? H[g * 512 + 1] : 0.0;
            __syncthreads();
            for (uint64_t lv = P >> 1; lv >= 1; lv >>= 1) {
                for (uint64_t j = lv + t; j < 2 * lv; j += kKcThreads) T[j] = T[2 * j] + T[2 * j + 1];
                __syncthreads();
            }
            if (t == 0) {
                const double S = T[1];
                sm_pos = S > 0.0;
                if (S > 0.0) {
                    double r = u[round + 1] * S;
                    const uint64_t g = det_heap_descend(T, P, r);
                    const uint64_t b = det_heap_descend(H + g * 512, 256, r);
                    sm_g = g;
                    sm_b = b;
                    sm_r = r;
                }
            }
            __syncthreads();
            if (!sm_pos) {
                // total not positive: the first maximum of the distances (k_det_draw's fallback)
                if (t == 0) {
                    uint64_t am = 0;
                    double best = __ldcg(a.dist);
                    for (uint64_t i = 1; i < n; ++i) {
                        const double v = __ldcg(a.dist + i);
                        if (v > best) {
                            best = v;
                            am = i;
                        }
                    }
                    *a.newc = am;
                }
            } else if (t < 32) {
                const uint64_t base = sm_g * kDetChunk + sm_b * 32, i = base + uint64_t(t);
                double v = 0.0;
                if (i < n) {
                    v = __ldcg(a.dist + i);
                    if (weighted) v = v * a.w[i];
                }
                E[32 + t] = v;
                __syncwarp();
                for (int lv = 16; lv >= 1; lv >>= 1) {
                    if (t < lv) E[lv + t] = E[2 * (lv + t)] + E[2 * (lv + t) + 1];
                    __syncwarp();
                }
                if (t == 0) {
                    double r = sm_r;
                    uint64_t res = base + det_heap_descend(E, 32, r);
                    if (res >= n) res = 0;
                    *a.newc = res;
                }
            }
        }
        kc_sync();
    }
}

// cluster size for this device (16 where a 16-CTA cluster of this kernel fits one GPC, else
// 8), 0 when none can be launched
static int kmpp_cluster_size(const void *kern, size_t smem) {
    static std::mutex mu;
    static std::unordered_map<const void *, int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::lock_guard<std::mutex> lk(mu);
    const void *key = reinterpret_cast<const char *>(kern) + dev;
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int best = 0;
    for (int cs : {16, 8}) {
        if (cs > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(unsigned(cs));
        cfg.blockDim = dim3(kKcThreads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = unsigned(cs);
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, kern, &cfg) == cudaSuccess && nc >= 1) {
            best = cs;
            break;
        }
        cudaGetLastError();
    }
    cache[key] = best;
    return best;
}

template <int MSR, bool VEC4>
static int kmpp_cluster_t(const KmppArgs &a, const double *u_dev, double *blk, cudaStream_t st) {
    auto kern = k_kmpp_cluster<MSR, VEC4>;
    const size_t smem = size_t(det_chunks(a.n)) * 512 * sizeof(double);
    MC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int cs = kmpp_cluster_size(reinterpret_cast<const void *>(kern), smem);
    if (cs == 0) return fail(MC_ECUDA, "k-means++: no thread-block cluster fits this device");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(cs));
    cfg.blockDim = dim3(kKcThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = unsigned(cs);
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    MC_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, a, u_dev, blk));
    note_launch();
    return MC_OK;
}

template <int MSR>
static int kmpp_cluster_m(const KmppArgs &a, const double *u_dev, double *blk, cudaStream_t st) {
    const bool vec4 = a.d % 4 == 0 && (reinterpret_cast<uintptr_t>(a.X) & 15) == 0;
    return vec4 ? kmpp_cluster_t<MSR, true>(a, u_dev, blk, st) : kmpp_cluster_t<MSR, false>(a, u_dev, blk, st);
}

static int run_kmeanspp_cluster(const KmppArgs &a, const double *u_dev, cudaStream_t st) {
    DBuf<double> blk;
    MC_TRY(blk.alloc((a.n + 31) / 32, st));
    MC_CUDA_TRY(cudaMemsetAsync(a.asn, 0, a.n * sizeof(uint32_t), st));
    switch (a.msr) {
        case SQRL2: MC_TRY(kmpp_cluster_m<SQRL2>(a, u_dev, blk.p, st)); break;
        case L1: MC_TRY(kmpp_cluster_m<L1>(a, u_dev, blk.p, st)); break;
        case HELLINGER: MC_TRY(kmpp_cluster_m<HELLINGER>(a, u_dev, blk.p, st)); break;
        case MKL: MC_TRY(kmpp_cluster_m<MKL>(a, u_dev, blk.p, st)); break;
        case JSD: MC_TRY(kmpp_cluster_m<JSD>(a, u_dev, blk.p, st)); break;
        default: return fail(MC_EUNSUPPORTED, "measure not supported");
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// Dense SQRL2 rounds screened through a BF16 copy of the rows.  A round can change row i only
// when the new center's FP32 distance v (the sequential fmaf sum the update computes) is
// below dist[i].  With xb = bf16(x) (round to nearest, 8-bit significand: |xb_j - x_j| <=
// 2^-8 |x_j|, so ||xb - x|| <= 2^-8 ||x||, plus 2^-130 for subnormal entries) and A the FP32 sum of
// (xb_j - c_j)^2 in any order, the exact squared distance S = ||x - c||^2 satisfies
//   |Sb - S| <= 2 ||xb - x|| sqrt(S) + ||xb - x||^2,  sqrt(S) <= sqrt(Sb) + ||xb - x||,
//   S >= Sb - 2^-7 ||x|| sqrt(Sb) - 3 2^-16 ||x||^2 (minus the subnormal slack's terms),
// where Sb = ||xb - c||^2 lies in [A / (1 + g), A / (1 - g)], and v >= S (1 - g), with
// g = (d + 2) 2^-24 / (1 - (d + 2) 2^-24) (the bound of an FP32 sum of d squared
// differences).  k_kmpp_screen evaluates that lower bound of v in FP32 with every rounding
// directed down (the subtracted terms up) and lists the rows where it does not exceed
// dist[i]; k_kmpp_exact_list then runs the update's own arithmetic on those rows only.
// Every other row keeps its distance and assignment, as the update would leave them, so the
// results are bit-identical to the unscreened rounds, and a round reads the 2-byte copy plus
// the listed rows' FP32 values instead of every FP32 value.
// ------------------------------------------------------------------------------------
struct ScreenArgs {
    const uint4 *Xb;       // [n][d / 8] BF16 rows
    const float *rn2;      // [n] FP32 squared row norms (sequential fmaf)
    float norm_up;         // (1 + (d + 4) 2^-24) rounded up: covers the error of sqrt(rn2)
    float one_m_g, one_p_2g;  // 1 - g rounded down, 1 + 2 g rounded up
    uint32_t *list;        // rows for the exact update
    unsigned *count;
};

// One row per thread, 128 rows per CTA: the rows' BF16 values staged in shared memory by
// cp.async (coalesced: 16 bytes per thread and copy), each thread then sums its own row.
template <int G>  // 16-byte groups per row: d / 8
__global__ void __launch_bounds__(128) k_kmpp_screen(const KmppArgs a, const ScreenArgs sa) {
    constexpr int P = G + 1;  // row pitch in 16-byte groups (4 banks apart)
    __shared__ __align__(16) uint4 xs[128 * P];
    __shared__ __align__(16) float cs[8 * G];
    const uint64_t c = *a.newc;
    const int t = threadIdx.x, lane = t & 31;
    if (blockIdx.x == 0 && t == 0) {
        a.center_ids[a.round] = uint32_t(c);
        a.asn[c] = a.round;
    }
    const uint64_t row0 = uint64_t(blockIdx.x) * 128;
    for (int e = t; e < 128 * G; e += 128) {
        const int r = e / G, q = e % G;
        const bool ok = row0 + uint64_t(r) < a.n;
        kp_cp_async16(&xs[r * P + q], ok ? sa.Xb + (row0 + uint64_t(r)) * G + q : sa.Xb, ok ? 16 : 0);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    for (int j = t; j < 8 * G; j += 128) cs[j] = a.X[c * a.d + uint64_t(j)];
    const uint64_t i = row0 + uint64_t(t);
    // the current distance's bits (no FP64 instruction here) and the squared norm
    const unsigned long long cb = i < a.n ? reinterpret_cast<const unsigned long long *>(a.dist)[i] : 0ull;
    const float r2 = i < a.n ? sa.rn2[i] : 0.f;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    bool need = false;
    // the update skips rows at distance 0 or below (and NaN never compares below): in bits,
    // zero, the sign bit, or above +inf
    if (i < a.n) {
        if (i == c) {
            a.dist[i] = 0.0;
        } else if (cb != 0ull && !(cb >> 63) && cb <= 0x7ff0000000000000ull) {
            float A = 0.f;
#pragma unroll
            for (int q = 0; q < G; ++q) {
                const uint4 w = xs[t * P + q];
                const uint32_t u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const float lo = __uint_as_float(u[h] << 16), hi = __uint_as_float(u[h] & 0xffff0000u);
                    const float d0 = lo - cs[8 * q + 2 * h], d1 = hi - cs[8 * q + 2 * h + 1];
                    A = fmaf(d0, d0, A);
                    A = fmaf(d1, d1, A);
                }
            }
            const float xn = __fmul_ru(__fsqrt_ru(r2), sa.norm_up);
            const float t1 = __fmul_rd(A, sa.one_m_g);
            const float t2 = __fmul_ru(__fmul_ru(xn, 0x1p-7f), __fsqrt_ru(__fmul_ru(A, sa.one_p_2g)));
            const float t3 = __fmul_ru(__fmul_ru(xn, xn), 4.57763671875e-05f);  // 3 2^-16
            // subnormal x_j round to BF16 with an absolute error up to 2^-134, so ||xb - x|| <=
            // 2^-8 ||x|| + 2^-130 (d <= 128): the cross terms of that slack
            const float t4 = __fadd_ru(__fadd_ru(__fmul_ru(__fsqrt_ru(__fmul_ru(A, sa.one_p_2g)), 0x1p-129f),
                                                 __fmul_ru(xn, 0x1p-135f)),
                                       0x1p-140f);
            const float slo = __fsub_rd(__fsub_rd(__fsub_rd(t1, t2), t3), t4);
            const float vlo = slo > 0.f ? __fmul_rd(slo, sa.one_m_g) : 0.f;
            // vlo as a double's bits (exact for a normal float; a subnormal or zero bound
            // counts as 0, which only lowers it), compared with the positive distance as
            // integers
            const uint32_t fb = __float_as_uint(vlo), fe = (fb >> 23) & 0xffu;
            const unsigned long long vb =
                fe == 0u ? 0ull : ((unsigned long long)(fe + 896u) << 52) | ((unsigned long long)(fb & 0x7fffffu) << 29);
            // a non-finite bound proves nothing: the exact update decides
            need = !(vb > cb) || !(A <= 3.402823466e+38f) || !(xn <= 3.402823466e+38f) || !(vlo <= 3.402823466e+38f);
        }
    }
    const unsigned nb = __ballot_sync(0xffffffffu, need);
    if (nb) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(sa.count, unsigned(__popc(nb)));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (need) sa.list[base + __popc(nb & ((1u << lane) - 1u))] = uint32_t(i);
    }
}

// The update's arithmetic (k_kmpp_dense) on the listed rows: the sequential fmaf sum over the
// columns, replaced only when below the current distance.
__global__ void __launch_bounds__(256) k_kmpp_exact_list(const KmppArgs a, const uint32_t *__restrict__ list,
                                                         const unsigned *__restrict__ count) {
    extern __shared__ __align__(16) float csm[];  // the new center's row
    const uint64_t c = *a.newc;
    for (uint64_t j = threadIdx.x; j < a.d; j += blockDim.x) csm[j] = a.X[c * a.d + j];
    __syncthreads();
    const unsigned cnt = *count;
    const PairScalars ps = {};
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < cnt; e += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t i = list[e];
        const float4 *xr = reinterpret_cast<const float4 *>(a.X + i * a.d);
        float acc = 0.f;
        // 32 columns at a time: their eight loads in flight together (d is a multiple of 16)
        for (uint64_t j0 = 0; j0 < a.d / 4; j0 += 8) {
            float4 x[8];
            const uint64_t m = a.d / 4 - j0 < 8 ? a.d / 4 - j0 : 8;
#pragma unroll
            for (int u = 0; u < 8; ++u) x[u] = uint64_t(u) < m ? xr[j0 + u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (uint64_t(u) < m) {
                    const float *cc = csm + 4 * (j0 + u);
                    kp_elem<SQRL2>(acc, cc[0], x[u].x, ps);
                    kp_elem<SQRL2>(acc, cc[1], x[u].y, ps);
                    kp_elem<SQRL2>(acc, cc[2], x[u].z, ps);
                    kp_elem<SQRL2>(acc, cc[3], x[u].w, ps);
                }
            }
        }
        const double v = kp_cost<SQRL2>(acc);
        if (v < a.dist[i]) {
            a.dist[i] = v;
            a.asn[i] = a.round;
        }
    }
}

// the screened rounds apply: dense SQRL2, d = 8 G with G in {2, 4, 8, 16} (a CTA's staged
// rows within 48 KB of static shared memory), 16-byte aligned rows
static bool kmpp_screen_ok(const KmppArgs &a) {
    const uint64_t g = a.d / 8;
    return !a.csr && a.msr == SQRL2 && a.d % 8 == 0 && (g == 2 || g == 4 || g == 8 || g == 16) &&
           (reinterpret_cast<uintptr_t>(a.X) & 15) == 0;
}

static int screened_round(const KmppArgs &a, uint32_t round, const ScreenArgs &sa, int sms, cudaStream_t st) {
    KmppArgs b = a;
    b.round = round;
    MC_CUDA_TRY(cudaMemsetAsync(sa.count, 0, sizeof(unsigned), st));
    const unsigned grid = unsigned((a.n + 127) / 128);
    switch (a.d / 8) {
        case 2: k_kmpp_screen<2><<<grid, 128, 0, st>>>(b, sa), note_launch(); break;
        case 4: k_kmpp_screen<4><<<grid, 128, 0, st>>>(b, sa), note_launch(); break;
        case 8: k_kmpp_screen<8><<<grid, 128, 0, st>>>(b, sa), note_launch(); break;
        default: k_kmpp_screen<16><<<grid, 128, 0, st>>>(b, sa), note_launch(); break;
    }
    // few rows are listed after the first rounds: a small grid (each CTA stages the center)
    k_kmpp_exact_list<<<unsigned(umin64((a.n + 255) / 256, uint64_t(sms) * 2)), 256, a.d * sizeof(float), st>>>(
        b, sa.list, sa.count), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

static int run_kmeanspp_launches(const KmppArgs &a0, const double *u_dev, double *chunk_tmp, int sms,
                                 cudaStream_t st, bool prune_ok, bool screen_ok = false);

int run_kmeanspp(const KmppArgs &a0, const double *u_dev, double *chunk_tmp, int sms, cudaStream_t st) {
    // dense rows up to 32 chunks and 2^23 values (a cluster of 8-16 SMs reads them in well
    // under the four to five launches of a round): the persistent cluster or a launch
    // sequence per round, whichever the autotuner measured faster for this shape (identical
    // results)
    if (!a0.csr && a0.n <= kKcMaxRows && a0.n * a0.d <= (uint64_t(1) << 23) && a0.k > 1) {
        // (time per round hardly depends on k: no k in the key, so a server tunes few buckets)
        const std::string key = "kmpp_run|msr" + std::to_string(a0.msr) + "|w" + std::to_string(a0.w ? 1 : 0) +
                                "|d" + tune_bucket(a0.d) + "|n" + tune_bucket(a0.n);
        return tune_launch(key, 2, 0, st, true, [&](int v) -> int {
            return v == 1 ? run_kmeanspp_cluster(a0, u_dev, st)
                          : run_kmeanspp_launches(a0, u_dev, chunk_tmp, sms, st, false);
        });
    }
    // dense SQRL2 over a large matrix: with or without the triangle-inequality pruning below
    // (it skips rows only where the result is provably unchanged, but costs dependent loads
    // before each row's distance: on the 2M x 64 Gaussian mixture it measured 19.2 ms per
    // 100-center run against 14.4 ms without), whichever the autotuner measures faster
    if (!a0.csr && a0.msr == SQRL2 && a0.k > 1 && a0.n * a0.d >= (uint64_t(1) << 20)) {
        const std::string key = "kmpp_prune|w" + std::to_string(a0.w ? 1 : 0) + "|d" + tune_bucket(a0.d) + "|n" +
                                tune_bucket(a0.n);
        // variant 2: rounds screened through a BF16 copy of the rows (also identical results)
        return tune_launch(key, kmpp_screen_ok(a0) ? 3 : 2, 0, st, true, [&](int v) -> int {
            return run_kmeanspp_launches(a0, u_dev, chunk_tmp, sms, st, v == 1, v == 2);
        });
    }
    return run_kmeanspp_launches(a0, u_dev, chunk_tmp, sms, st, false);
}

static int run_kmeanspp_launches(const KmppArgs &a0, const double *u_dev, double *chunk_tmp, int sms,
                                 cudaStream_t st, bool prune_ok, bool screen_ok) {
    KmppArgs a = a0;
    a.cgap = nullptr;
    const unsigned tb = 256, tg = unsigned(umin64((a.d + tb - 1) / tb, 1024));
    MC_CUDA_TRY(cudaMemsetAsync(a.asn, 0, a.n * sizeof(uint32_t), st));
    k_kmpp_first<<<1, 1, 0, st>>>(u_dev, a.n, a.newc, a.center_ids), note_launch();
    const bool fused = kmpp_csr_fused_ok(a);  // the update kernel takes the center itself
    if (a.csr && !fused) {
        k_kmpp_take<<<tg, tb, 0, st>>>(a, 0), note_launch();
        k_kmpp_scatter<<<64, 256, 0, st>>>(a), note_launch();
    }
    MC_TRY(update(a, 1, 0, sms, st));
    // rounds after the first may prune by the triangle inequality (one more small launch per
    // round; the results are unchanged)
    const bool prune = prune_ok && !a.csr && a.msr == SQRL2 && a.k > 1;
    DBuf<double> gap;
    if (prune) {
        MC_TRY(gap.alloc(a.k, st));
        const double g = double(a.d + 2) * 0x1p-24;
        a.prune_g = g / (1.0 - g);
    }
    const bool screen = screen_ok && !prune && kmpp_screen_ok(a) && a.k > 1;
    DBuf<uint4> xb;
    DBuf<float> rn2;
    DBuf<uint32_t> slist;
    DBuf<unsigned> scount;
    ScreenArgs sa{};
    if (screen) {
        MC_TRY(xb.alloc(a.n * a.d / 8, st));
        MC_TRY(rn2.alloc(a.n, st));
        MC_TRY(slist.alloc(a.n, st));
        MC_TRY(scount.alloc(1, st));
        MC_TRY(launch_to_bf16_flat8(a.X, a.n * a.d / 8, xb.p, sms, st));
        MC_TRY(launch_row_sums_dense(a.X, a.n, a.d, nullptr, rn2.p, st));
        const double g = double(a.d + 2) * 0x1p-24 / (1.0 - double(a.d + 2) * 0x1p-24);
        sa.Xb = xb.p;
        sa.rn2 = rn2.p;
        sa.norm_up = std::nextafter(float(1.0 + double(a.d + 4) * 0x1p-24), 2.0f);
        sa.one_m_g = std::nextafter(float(1.0 - g), 0.0f);
        sa.one_p_2g = std::nextafter(float(1.0 + 2.0 * g), 2.0f);
        sa.list = slist.p;
        sa.count = scount.p;
    }
    DetInput in{a.w ? DET_F64_W : DET_F64, a.dist, nullptr, a.w, a.n};
    for (uint32_t ci = 1; ci < a.k; ++ci) {
        MC_TRY(launch_det_draw(in, chunk_tmp, u_dev + ci, 0.0, 1, a.dist, a.newc, st));
        if (screen) {
            MC_TRY(screened_round(a, ci, sa, sms, st));
            continue;
        }
        if (prune) {
            k_kmpp_center_gap<<<unsigned((ci + 7) / 8), 256, 0, st>>>(a, ci, gap.p), note_launch();
            a.cgap = gap.p;
        }
        if (a.csr && !fused) {
            // CSR centers are densified into cbuf; the dense update reads the center row itself
            k_kmpp_take<<<tg, tb, 0, st>>>(a, ci), note_launch();
            k_kmpp_scatter<<<64, 256, 0, st>>>(a), note_launch();
        }
        MC_TRY(update(a, 0, ci, sms, st));
        if (a.csr && !fused) k_kmpp_zero<<<1, 1, 0, st>>>(a), note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// Greedy k-means++ (n_local_trials = L > 1, kmeans.h:79-177): the first center is the best
// (lowest objective) of L uniform picks; every later round draws L candidates from the
// distances without replacement (a drawn row's weight is zeroed for the next draw), adds
// each to the distances and keeps the one with the lowest objective.  As in the reference,
// candidate 0 updates the current distances in place while candidates 1.. start from the
// distances and assignments of the first center alone (`odists`, `oasn`, set once before the
// rounds, kmeans.h:106-107, 140-144).  Uniforms U(seed, r), one counter; draws and sums in
// the canonical FP64 order.
// ------------------------------------------------------------------------------------
__global__ void k_kmpp_exclude(double *dist, const uint64_t *cand, double *saved) {
    const uint64_t c = *cand;
    *saved = dist[c];
    dist[c] = 0.0;
}
__global__ void k_kmpp_restore(double *dist, const uint64_t *cand, const double *saved, uint32_t L) {
    for (int s = int(L) - 1; s >= 0; --s) dist[cand[s]] = saved[s];
}
// the candidate's own row: distance 0 (the plain update of the reference visits it too)
__global__ void k_kmpp_self(double *dist, uint32_t *asn, const uint64_t *cand, uint32_t round) {
    const uint64_t c = *cand;
    if (dist[c] > 0.0) {
        dist[c] = 0.0;
        asn[c] = round;
    }
}
__global__ void k_kmpp_set_center(double *dist, uint32_t *asn, uint32_t *center_ids, const uint64_t *cand,
                                  uint32_t round) {
    const uint64_t c = *cand;
    center_ids[round] = uint32_t(c);
    asn[c] = round;
    dist[c] = 0.0;
}
__global__ void k_kmpp_pick(const double *u, uint64_t n, uint64_t *out) {
    uint64_t fc = uint64_t(*u * double(n));
    if (fc >= n) fc = n - 1;
    *out = fc;
}

// the distances of b (dist, asn) with candidate *b.newc added in round `round` (first: the
// distances to the first center)
static int kmpp_add_candidate(const KmppArgs &b, int first, uint32_t round, int sms, cudaStream_t st) {
    const unsigned tb = 256, tg = unsigned(umin64((b.d + tb - 1) / tb, 1024));
    const bool fused = kmpp_csr_fused_ok(b);
    if (b.csr && !fused) {
        k_kmpp_take<<<tg, tb, 0, st>>>(b, round), note_launch();
        k_kmpp_scatter<<<64, 256, 0, st>>>(b), note_launch();
    }
    MC_TRY(update(b, first, round, sms, st));
    if (!first) k_kmpp_self<<<1, 1, 0, st>>>(b.dist, b.asn, b.newc, round), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

static int kmpp_cost(const KmppArgs &b, double *chunk_tmp, double *scal, cudaStream_t st, double *out) {
    DetInput in{b.w ? DET_F64_W : DET_F64, b.dist, nullptr, b.w, b.n};
    MC_TRY(launch_det_sum(in, chunk_tmp, scal, st));
    MC_CUDA_TRY(cudaMemcpyAsync(out, scal, sizeof(double), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    return MC_OK;
}

int run_kmeanspp_greedy(const KmppArgs &a0, uint32_t L, uint64_t seed, double *chunk_tmp, int sms, cudaStream_t st) {
    KmppArgs a = a0;
    const uint64_t n = a.n;
    uint64_t counter = 0;
    DBuf<double> ubuf, T, O, S, sav, scal;
    DBuf<uint32_t> OA, SA;
    DBuf<uint64_t> cand;
    MC_TRY(ubuf.alloc(1, st));
    MC_TRY(T.alloc(n, st));
    MC_TRY(O.alloc(n, st));
    MC_TRY(S.alloc(n, st));
    MC_TRY(sav.alloc(L, st));
    MC_TRY(scal.alloc(1, st));
    MC_TRY(OA.alloc(n, st));
    MC_TRY(SA.alloc(n, st));
    MC_TRY(cand.alloc(L, st));
    auto put_u = [&](double u) -> int {
        MC_CUDA_TRY(cudaMemcpyAsync(ubuf.p, &u, sizeof(double), cudaMemcpyHostToDevice, st));
        MC_CUDA_TRY(cudaStreamSynchronize(st));  // u lives on this frame
        return MC_OK;
    };
    // first center: the best of L uniform picks
    MC_CUDA_TRY(cudaMemsetAsync(a.asn, 0, n * sizeof(uint32_t), st));
    MC_TRY(put_u(uniform_at(seed, counter++)));
    k_kmpp_pick<<<1, 1, 0, st>>>(ubuf.p, n, a.newc), note_launch();
    MC_TRY(kmpp_add_candidate(a, 1, 0, sms, st));
    double fcost = 0.0;
    MC_TRY(kmpp_cost(a, chunk_tmp, scal.p, st, &fcost));
    uint64_t fc = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(&fc, a.newc, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    for (uint32_t t = 1; t < L; ++t) {
        KmppArgs b = a;
        b.dist = T.p;
        b.newc = cand.p;
        MC_TRY(put_u(uniform_at(seed, counter++)));
        k_kmpp_pick<<<1, 1, 0, st>>>(ubuf.p, n, cand.p), note_launch();
        MC_TRY(kmpp_add_candidate(b, 1, 0, sms, st));
        double oc = 0.0;
        MC_TRY(kmpp_cost(b, chunk_tmp, scal.p, st, &oc));
        if (oc < fcost) {
            fcost = oc;
            MC_CUDA_TRY(cudaMemcpyAsync(&fc, cand.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            MC_CUDA_TRY(cudaMemcpyAsync(a.dist, T.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            MC_CUDA_TRY(cudaStreamSynchronize(st));
        }
    }
    uint32_t fc32 = uint32_t(fc);
    MC_CUDA_TRY(cudaMemcpyAsync(a.center_ids, &fc32, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    MC_CUDA_TRY(cudaMemsetAsync(a.asn, 0, n * sizeof(uint32_t), st));
    MC_CUDA_TRY(cudaMemcpyAsync(O.p, a.dist, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    MC_CUDA_TRY(cudaMemsetAsync(OA.p, 0, n * sizeof(uint32_t), st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    DetInput in{a.w ? DET_F64_W : DET_F64, a.dist, nullptr, a.w, n};
    for (uint32_t ci = 1; ci < a.k; ++ci) {
        for (uint32_t s = 0; s < L; ++s) {
            MC_TRY(launch_det_draw(in, chunk_tmp, nullptr, uniform_at(seed, counter++), 0, nullptr, cand.p + s, st));
            k_kmpp_exclude<<<1, 1, 0, st>>>(a.dist, cand.p + s, sav.p + s), note_launch();
        }
        k_kmpp_restore<<<1, 1, 0, st>>>(a.dist, cand.p, sav.p, L), note_launch();
        double dsum = -1.0;
        uint32_t best = 0;
        for (uint32_t s = 0; s < L; ++s) {
            KmppArgs b = a;
            b.newc = cand.p + s;
            if (s > 0) {
                MC_CUDA_TRY(cudaMemcpyAsync(S.p, O.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
                MC_CUDA_TRY(cudaMemcpyAsync(SA.p, OA.p, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
                b.dist = S.p;
                b.asn = SA.p;
            }
            MC_TRY(kmpp_add_candidate(b, 0, ci, sms, st));
            double nsum = 0.0;
            MC_TRY(kmpp_cost(b, chunk_tmp, scal.p, st, &nsum));
            if (s == 0) {
                dsum = nsum;
            } else if (nsum < dsum) {
                dsum = nsum;
                best = s;
                MC_CUDA_TRY(cudaMemcpyAsync(a.dist, S.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
                MC_CUDA_TRY(cudaMemcpyAsync(a.asn, SA.p, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
            }
        }
        k_kmpp_set_center<<<1, 1, 0, st>>>(a.dist, a.asn, a.center_ids, cand.p + best, ci), note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// out[i] = distance of row i to the row *cand (0 for that row): the first-round update of
// the seeding kernels.  CSR centers pass through a.cbuf; a.center_ids[0] and a.asn[*cand]
// may be written (callers pass scratch for the former).
int kmpp_distances_to(const KmppArgs &a0, const uint64_t *cand, double *out, int sms, cudaStream_t st) {
    KmppArgs b = a0;
    b.dist = out;
    b.newc = const_cast<uint64_t *>(cand);
    return kmpp_add_candidate(b, 1, 0, sms, st);
}

// centers[c] = row ids[c] (dense copy, or a zero-filled row with the CSR entries scattered)
__global__ void k_gather_rows_dense(const float *__restrict__ X, uint64_t d, const uint32_t *__restrict__ ids,
                                    uint32_t k, float *__restrict__ C) {
    const uint64_t total = uint64_t(k) * d;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += gridDim.x * uint64_t(blockDim.x))
        C[e] = X[uint64_t(ids[e / d]) * d + e % d];
}

__global__ void k_gather_rows_csr(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                                  const uint64_t *__restrict__ indptr, uint64_t d, const uint32_t *__restrict__ ids,
                                  uint32_t k, float *__restrict__ C) {
    for (uint32_t c = blockIdx.x; c < k; c += gridDim.x) {
        float *row = C + uint64_t(c) * d;
        for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) row[j] = 0.f;
        __syncthreads();
        const uint32_t r = ids[c];
        for (uint64_t p = indptr[r] + threadIdx.x; p < indptr[r + 1]; p += blockDim.x) row[idx[p]] = vals[p];
        __syncthreads();
    }
}

int launch_gather_rows(bool csr, const float *X, const float *vals, const uint32_t *idx, const uint64_t *indptr,
                       uint64_t d, const uint32_t *ids, uint32_t k, float *C, cudaStream_t st) {
    if (k == 0) return MC_OK;
    if (csr) {
        k_gather_rows_csr<<<unsigned(umin64(k, 4096)), 256, 0, st>>>(vals, idx, indptr, d, ids, k, C), note_launch();
    } else {
        const uint64_t total = uint64_t(k) * d;
        k_gather_rows_dense<<<unsigned(umin64((total + 255) / 256, 4096)), 256, 0, st>>>(X, d, ids, k, C),
            note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

}  // namespace mc
