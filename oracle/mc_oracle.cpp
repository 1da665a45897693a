// ORACLE — test infrastructure only.
//
// A plain C++17 (+OpenMP) restatement of the CPU algorithm of dnbaker/minicore for the
// clustering hot path: cmp::msr_with_prior, coresets::kmeanspp, assign_points_hard,
// set_centroids_full_mean / set_center, perform_hard_clustering, and the CoresetSampler
// sensitivity + sampling code.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load this library, and only as the checker.  The product path
// (minicore_gb300) never calls it.
//
// Parity anchors (reference files, paths within the minicore project):
//   include/minicore/dist/applicator.h:1632-1915   msr_with_prior (prior setup, dense + sparse)
//   include/minicore/util/merge.h:26-65             for_each_by_case (sharednz)
//   include/minicore/optim/kmeans.h:49-215          kmeanspp
//   include/minicore/clustering/solve.h:98-285      perform_hard_clustering / assign_points_hard
//   include/minicore/clustering/centroid.h:81-178,649-779  set_center / set_centroids_full_mean
//   include/minicore/coreset/coreset.h:340-699      make_probs_* / sample
//
// Where the reference delegates to libraries that are absent from the reference tree
// (libkl reducers, libsimdsampling reservoir sampling, alias_sampler, wy RNG), this file
// fixes one explicit definition and the CUDA path implements the same definition:
//   * element reductions: sequential over columns, float arithmetic, fmaf where noted;
//   * every random draw consumes a caller-supplied uniform in [0,1) (splitmix64 stream);
//   * D^2 draws are an FP64 inverse CDF in a fixed blocked summation order (det_*);
//   * centroid sums use a fixed chunked order (compensated FP32 within a chunk of rows,
//     FP64 across chunks; FP64 fma when weighted);
//   * the alias table is Vose's method in FP64 over the float probabilities.
// Compile with -ffp-contract=off so that no multiply-add is fused behind our back.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <set>
#include <numeric>
#include <vector>

namespace {

enum Msr { L1 = 0, L2 = 1, SQRL2 = 2, JSM = 3, JSD = 4, MKL = 5, HELLINGER = 6 };

constexpr double kSqrt1_2 = 0.70710678118654752440;

// ---------------------------------------------------------------------------------------
// splitmix64 uniform stream: U(seed, i) in [0, 1)
// ---------------------------------------------------------------------------------------
inline double uniform_at(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return double(z >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------------------
// Canonical deterministic FP64 sums and draws (mirrors the CUDA det kernels exactly).
// Chunks of 8192 consecutive elements (zeros past n).  Inside a chunk, a pairwise tree over
// consecutive elements: level 1 adds elements (2i, 2i+1), level 2 adds the level-1 sums
// (2i, 2i+1), ... 13 levels to the chunk total.  The chunk totals, padded with zeros to a
// power of two P, form the leaves of the same pairwise tree, whose root is the sum.
// A draw with uniform u descends the tree from the root with r = u * S: at a node with
// children sums (L, R), go left when r < L or R is not positive, else r -= L and go right;
// at the chunk it continues down the chunk's tree to one element.
// ---------------------------------------------------------------------------------------
constexpr uint64_t kChunk = 8192, kThreads = 256, kPer = 32;

// heap layout: node j has children 2j, 2j+1; leaves at [P, 2P)
inline void build_heap(std::vector<double> &T, uint64_t P) {
    for (uint64_t j = P - 1; j >= 1; --j) T[j] = T[2 * j] + T[2 * j + 1];
}

template <class Get>
void chunk_heap(const Get &get, uint64_t n, uint64_t g, std::vector<double> &H) {
    H.assign(2 * kChunk, 0.0);
    const uint64_t base = g * kChunk;
    for (uint64_t e = 0; e < kChunk; ++e) H[kChunk + e] = base + e < n ? get(base + e) : 0.0;
    build_heap(H, kChunk);
}

template <class Get>
double chunk_total(const Get &get, uint64_t n, uint64_t g) {
    std::vector<double> H;
    chunk_heap(get, n, g, H);
    return H[1];
}

inline uint64_t pow2_at_least(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

template <class Get>
double det_sum(const Get &get, uint64_t n, std::vector<double> *top = nullptr) {
    const uint64_t G = (n + kChunk - 1) / kChunk;
    if (G == 0) return 0.0;
    const uint64_t P = pow2_at_least(G);
    std::vector<double> T(2 * P, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < int64_t(G); ++g) T[P + uint64_t(g)] = chunk_total(get, n, uint64_t(g));
    build_heap(T, P);
    const double S = P > 1 ? T[1] : T[P];
    if (top) *top = std::move(T);
    return S;
}

// descend a heap of P leaves from the root; returns the leaf and leaves the remainder in r
inline uint64_t heap_descend(const std::vector<double> &T, uint64_t P, double &r) {
    uint64_t j = 1;
    while (j < P) {
        const double L = T[2 * j], R = T[2 * j + 1];
        if (r < L || !(R > 0.0)) {
            j = 2 * j;
        } else {
            r = r - L;
            j = 2 * j + 1;
        }
    }
    return j - P;
}

// Inverse-CDF draw over non-negative weights v[0..n) with uniform u.  Returns n when the
// total weight is not positive.
template <class Get>
uint64_t det_draw(const Get &get, uint64_t n, double u) {
    std::vector<double> T;
    const double S = det_sum(get, n, &T);
    if (!(S > 0.0)) return n;
    const uint64_t G = (n + kChunk - 1) / kChunk;
    const uint64_t P = pow2_at_least(G);
    double r = u * S;
    const uint64_t g = P > 1 ? heap_descend(T, P, r) : 0;
    std::vector<double> H;
    chunk_heap(get, n, g, H);
    const uint64_t e = heap_descend(H, kChunk, r);
    return g * kChunk + e;
}

// ---------------------------------------------------------------------------------------
// msr_with_prior restatement (applicator.h:1632-1915).  FT = float.
// Role names: `row` is the reference's 2nd argument (`ctr`, the data row on every hot call
// site) and `cen` is its 3rd argument (`mr`, the center).  "lh" = center, "rh" = row.
// ---------------------------------------------------------------------------------------
struct PairScalars {
    float pv, lhsum, rhsum, lhrsi, rhrsi, lhinc, rhinc;
};

inline PairScalars pair_scalars(double prior, double prior_sum_arg, double rowsum, double ctrsum,
                                uint64_t nd) {
    PairScalars s;
    float lhsum = float(ctrsum + prior_sum_arg);
    float rhsum = float(rowsum + prior_sum_arg);
    const float smallest_pv = 7.0069e-42f * (lhsum + rhsum);
    const float pv = std::max(float(prior), smallest_pv);
    const float psum = pv * float(nd);
    lhsum = float(ctrsum + double(psum));
    rhsum = float(rowsum + double(psum));
    const float lhrsi = 1.f / lhsum, rhrsi = 1.f / rhsum;
    float lhinc = (pv != 0.f && lhsum != 0.f) ? pv * lhrsi : 0.f;
    float rhinc = (pv != 0.f && rhsum != 0.f) ? pv * rhrsi : 0.f;
    if (std::isnan(lhinc)) lhinc = 0.f;
    if (std::isnan(rhinc)) rhinc = 0.f;
    s.pv = pv; s.lhsum = lhsum; s.rhsum = rhsum; s.lhrsi = lhrsi; s.rhrsi = rhrsi;
    s.lhinc = lhinc; s.rhinc = rhinc;
    return s;
}

inline double post_divergence(double ret) {  // applicator.h:1754-1760
    ret = std::max(ret, 0.);
    if (ret == double(std::numeric_limits<float>::infinity())) ret = double(std::numeric_limits<float>::max());
    else if (ret == -double(std::numeric_limits<float>::infinity())) ret = 0.;
    return ret;
}

// element terms shared by the dense and sparse paths (libkl reducer definitions)
struct Reducer {
    int msr;
    PairScalars s;
    float acc = 0.f;
    inline void add(float c, float x) {
        switch (msr) {
            case SQRL2: { float d = c - x; acc = std::fma(d, d, acc); break; }
            case L1: { float a = c + s.pv, b = x + s.pv; acc = acc + std::fabs(a - b); break; }
            case HELLINGER: {
                float a = std::sqrt(c * s.lhrsi + s.lhinc), b = std::sqrt(x * s.rhrsi + s.rhinc);
                float d = a - b; acc = std::fma(d, d, acc); break;
            }
            case MKL: {
                float a = c * s.lhrsi + s.lhinc, b = x * s.rhrsi + s.rhinc;
                acc = std::fma(a, std::log(a) - std::log(b), acc); break;
            }
            case JSD: {
                float a = c * s.lhrsi + s.lhinc, b = x * s.rhrsi + s.rhinc;
                float m = a + b;
                float t = (a * std::log(a) + b * std::log(b)) - m * std::log(m * 0.5f);
                acc = acc + t; break;
            }
            default: break;
        }
    }
};

double msr_dense(int msr, const float *row, const float *cen, uint64_t d, double prior,
                 double prior_sum, double rowsum, double ctrsum) {
    Reducer r{msr, pair_scalars(prior, prior_sum, rowsum, ctrsum, d)};
    for (uint64_t j = 0; j < d; ++j) r.add(cen[j], row[j]);
    switch (msr) {
        case SQRL2: return double(r.acc);
        case L1: return double(r.acc * 0.5f) * 2.;
        case HELLINGER: return double(std::sqrt(r.acc)) * kSqrt1_2;
        case MKL: return post_divergence(double(r.acc));
        case JSD: return post_divergence(double(r.acc * 0.5f));
        default: return -1.;
    }
}

// sparse/sparse path: merge the union of the two index sets; sharednz = d - |union|
double msr_sparse(int msr, const float *rv, const uint32_t *ri, uint64_t rnz, const float *cv,
                  const uint32_t *ci, uint64_t cnz, uint64_t d, double prior, double prior_sum,
                  double rowsum, double ctrsum) {
    const PairScalars s = pair_scalars(prior, prior_sum, rowsum, ctrsum, d);
    Reducer r{msr, s};
    uint64_t a = 0, b = 0, nunion = 0;
    // MKL/JSD merge the scaled vectors (wr = mr * lhrsi, wc = ctr * rhrsi) and the reducer
    // adds the increments; the metric measures merge raw values.  The reducer applies the
    // scaling itself, so both orderings reduce to the same element terms.
    while (a < cnz || b < rnz) {
        float c, x;
        if (a < cnz && b < rnz && ci[a] == ri[b]) { c = cv[a++]; x = rv[b++]; }
        else if (b >= rnz || (a < cnz && ci[a] < ri[b])) { c = cv[a++]; x = 0.f; }
        else { c = 0.f; x = rv[b++]; }
        ++nunion;
        r.add(c, x);
    }
    const uint64_t sharednz = d - nunion;
    switch (msr) {
        case SQRL2: {
            double ret = r.acc;
            if (ret < 0.) ret = 0.;
            else if (std::isnan(ret)) ret = -1.;
            return ret;
        }
        case L1: return double(r.acc * 0.5f) * 2.;
        case HELLINGER: {
            double ret = double(r.acc) +
                         std::pow(std::sqrt(double(s.lhinc)) - std::sqrt(double(s.rhinc)), 2.) * double(sharednz);
            return std::sqrt(ret) * kSqrt1_2;
        }
        case MKL: {
            const float rhl = s.rhinc != 0.f ? std::log(s.rhinc) : 0.f;
            const float lhl = s.lhinc != 0.f ? std::log(s.lhinc) : 0.f;
            const float zc = float(sharednz) * s.lhinc * (lhl - rhl);
            return post_divergence(double(r.acc + zc));
        }
        case JSD: {
            const float rhl = s.rhinc != 0.f ? std::log(s.rhinc) : 0.f;
            const float lhl = s.lhinc != 0.f ? std::log(s.lhinc) : 0.f;
            const float rhincl = s.rhinc != 0.f ? rhl * s.rhinc : 0.f;
            const float lhincl = s.lhinc != 0.f ? lhl * s.lhinc : 0.f;
            const float shl = std::log((s.lhinc + s.rhinc) * 0.5f);
            const float shincl = (s.rhinc + s.lhinc > 0.f) ? (s.lhinc + s.rhinc) * shl : 0.f;
            const float zc = ((lhincl + rhincl - shincl) * float(sharednz)) * 0.5f;
            return post_divergence(double(r.acc * 0.5f + zc));
        }
        default: return -1.;
    }
}

// ---------------------------------------------------------------------------------------
// Matrix views
// ---------------------------------------------------------------------------------------
struct Mat {
    int kind;  // 0 dense row-major f32, 1 CSR f32/u32/u64
    uint64_t n, d;
    const float *vals;
    const uint32_t *idx;
    const uint64_t *indptr;
};

struct SparseVec { std::vector<uint32_t> i; std::vector<float> v; };

inline double row_sum(const Mat &m, uint64_t r) {  // Blaze rowwise sum into double
    double s = 0.;
    if (m.kind == 0) { for (uint64_t j = 0; j < m.d; ++j) s += m.vals[r * m.d + j]; }
    else for (uint64_t p = m.indptr[r]; p < m.indptr[r + 1]; ++p) s += m.vals[p];
    return s;
}

// center sums (canonical order of the device's k_center_sums): 32 strided FP64 partials
// (partial l holds columns l, l+32, ... in order), then the partials in order 0..31
inline double vec_sum(const float *v, uint64_t d) {
    double part[32] = {0.};
    for (uint64_t j = 0; j < d; ++j) part[j % 32] += v[j];
    double s = 0.;
    for (int l = 0; l < 32; ++l) s += part[l];
    return s;
}

SparseVec to_sparse(const float *dense, uint64_t d) {
    SparseVec s;
    for (uint64_t j = 0; j < d; ++j) if (dense[j] != 0.f) { s.i.push_back(uint32_t(j)); s.v.push_back(dense[j]); }
    return s;
}

// distance between data row r and a center (dense center for dense data, sparse for CSR)
struct CenterSet {
    uint64_t k, d;
    std::vector<float> dense;     // k*d
    std::vector<SparseVec> sp;    // CSR data only
    std::vector<double> sums;
    void set_from_dense(const float *C, uint64_t k_, uint64_t d_, bool sparse) {
        k = k_; d = d_;
        dense.assign(C, C + k * d);
        sums.resize(k);
        sp.clear();
        for (uint64_t c = 0; c < k; ++c) {
            sums[c] = vec_sum(&dense[c * d], d);
            if (sparse) sp.push_back(to_sparse(&dense[c * d], d));
        }
    }
    void set_row(uint64_t c, const std::vector<float> &v, bool sparse) {
        std::copy(v.begin(), v.end(), dense.begin() + c * d);
        sums[c] = vec_sum(v.data(), d);
        if (sparse) sp[c] = to_sparse(v.data(), d);
    }
};

inline double dist_row_center(const Mat &m, uint64_t r, const CenterSet &C, uint64_t c, int msr,
                              double prior, double psum, double rsum) {
    if (m.kind == 0)
        return msr_dense(msr, m.vals + r * m.d, &C.dense[c * m.d], m.d, prior, psum, rsum, C.sums[c]);
    const uint64_t b = m.indptr[r], e = m.indptr[r + 1];
    const SparseVec &s = C.sp[c];
    return msr_sparse(msr, m.vals + b, m.idx + b, e - b, s.v.data(), s.i.data(), s.i.size(), m.d, prior, psum,
                      rsum, C.sums[c]);
}

inline double dist_row_row(const Mat &m, uint64_t r, uint64_t cr, int msr, double prior, double psum,
                           double rsum, double csum) {
    if (m.kind == 0)
        return msr_dense(msr, m.vals + r * m.d, m.vals + cr * m.d, m.d, prior, psum, rsum, csum);
    const uint64_t b = m.indptr[r], e = m.indptr[r + 1], cb = m.indptr[cr], ce = m.indptr[cr + 1];
    return msr_sparse(msr, m.vals + b, m.idx + b, e - b, m.vals + cb, m.idx + cb, ce - cb, m.d, prior, psum, rsum,
                      csum);
}

std::vector<float> dense_row(const Mat &m, uint64_t r) {
    std::vector<float> v(m.d, 0.f);
    if (m.kind == 0) std::copy(m.vals + r * m.d, m.vals + (r + 1) * m.d, v.begin());
    else for (uint64_t p = m.indptr[r]; p < m.indptr[r + 1]; ++p) v[m.idx[p]] = m.vals[p];
    return v;
}

// assign_points_hard (solve.h:234-285): strict < keeps the lowest index on ties
// Costs are kept in double (the dense bindings store double costs, pycluster_dense.cpp:24);
// the CSR bindings store float costs (pycluster.h:160), so CSR values are rounded to float.
void assign_all(const Mat &m, const CenterSet &C, int msr, double prior, double psum, const std::vector<double> &rs,
                uint32_t *asn, double *costs) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < int64_t(m.n); ++i) {
        double best = dist_row_center(m, uint64_t(i), C, 0, msr, prior, psum, rs[i]);
        uint32_t bi = 0;
        for (uint64_t j = 1; j < C.k; ++j) {
            double v = dist_row_center(m, uint64_t(i), C, j, msr, prior, psum, rs[i]);
            if (v < best) { best = v; bi = uint32_t(j); }
        }
        asn[i] = bi;
        costs[i] = m.kind == 1 ? double(float(best)) : best;
    }
}

// ---------------------------------------------------------------------------------------
// Centroid accumulation in the canonical chunked order.
// Unweighted: per chunk of `ch` rows (rows of a cluster in ascending order), per column a
// compensated float sum (Knuth TwoSum, separate error accumulator); chunk value =
// double(s) + double(e); chunk values summed in FP64 in chunk order.  Weighted: per chunk
// FP64 fma(w, x, acc) and FP64 weight sum; then across chunks in FP64.
// ---------------------------------------------------------------------------------------
inline void two_sum_add(float &s, float &e, float x) {
    const float t = s + x;
    const float bp = t - s;
    const float err = (s - (t - bp)) + (x - bp);
    s = t;
    e = e + err;
}

uint64_t centroid_chunk_rows(const Mat &m) { return m.kind == 0 ? 256 : 4096; }

void mean_of_rows(const Mat &m, const std::vector<uint64_t> &rows, const double *w, float *out) {
    const uint64_t d = m.d, ch = centroid_chunk_rows(m);
    std::vector<double> S(d, 0.0), part(d);
    std::vector<float> ps(d), pe(d);
    double W = 0.0;
    bool first = true;
    for (uint64_t q0 = 0; q0 < rows.size(); q0 += ch) {
        const uint64_t q1 = std::min<uint64_t>(rows.size(), q0 + ch);
        if (w) {
            std::fill(part.begin(), part.end(), 0.0);
            double wq = 0.0;
            for (uint64_t q = q0; q < q1; ++q) {
                const uint64_t r = rows[q];
                const double wr = w[r];
                wq = wq + wr;
                if (m.kind == 0) { for (uint64_t j = 0; j < d; ++j) part[j] = std::fma(wr, double(m.vals[r * d + j]), part[j]); }
                else for (uint64_t p = m.indptr[r]; p < m.indptr[r + 1]; ++p) part[m.idx[p]] = std::fma(wr, double(m.vals[p]), part[m.idx[p]]);
            }
            W = first ? wq : W + wq;
        } else {
            std::fill(ps.begin(), ps.end(), 0.f);
            std::fill(pe.begin(), pe.end(), 0.f);
            for (uint64_t q = q0; q < q1; ++q) {
                const uint64_t r = rows[q];
                if (m.kind == 0) { for (uint64_t j = 0; j < d; ++j) two_sum_add(ps[j], pe[j], m.vals[r * d + j]); }
                else for (uint64_t p = m.indptr[r]; p < m.indptr[r + 1]; ++p) two_sum_add(ps[m.idx[p]], pe[m.idx[p]], m.vals[p]);
            }
            for (uint64_t j = 0; j < d; ++j) part[j] = double(ps[j]) + double(pe[j]);
        }
        if (first) { S = part; first = false; }
        else for (uint64_t j = 0; j < d; ++j) S[j] = S[j] + part[j];
    }
    const double denom = w ? W : double(rows.size());
    for (uint64_t j = 0; j < d; ++j) out[j] = float(S[j] / denom);
}

// total cost (solve.h:120-123) in FP64 canonical order, returned as FT=float
float compute_cost(const double *costs, const double *w, uint64_t n) {
    double s = w ? det_sum([&](uint64_t i) { return costs[i] * w[i]; }, n)
                 : det_sum([&](uint64_t i) { return costs[i]; }, n);
    return float(s);
}

// set_centroids_full_mean (centroid.h:649-779).  Returns 1 if any center was restarted,
// 0 otherwise, -1 on a NaN center.
int set_centroids_full_mean(const Mat &m, int msr, double prior, std::vector<uint32_t> &asn, std::vector<double> &costs,
                            CenterSet &C, const double *w, const std::vector<double> &rs, uint64_t seed,
                            uint64_t &restart_counter) {
    const uint64_t n = m.n, k = C.k;
    const bool sparse = m.kind == 1;
    std::vector<std::vector<uint64_t>> assigned(k);
    for (uint64_t i = 0; i < n; ++i) assigned[asn[i]].push_back(i);
    std::vector<uint32_t> empty;
    for (uint32_t i = 0; i < k; ++i) if (assigned[i].empty()) empty.push_back(i);
    int restarted = 0;
    if (!empty.empty()) {
        restarted = 1;
        // the reference passes prior[0] * prior.size() as the prior sum here (centroid.h:700)
        const double psum_restart = double(float(prior)) * 1.0;
        for (auto &a : assigned) a.clear();
        std::vector<uint64_t> rsel;
        for (uint32_t id : empty) {
            const double u = uniform_at(seed, restart_counter++);
            uint64_t r = det_draw([&](uint64_t i) { return costs[i]; }, n, u);
            if (r >= n) r = 0;
            rsel.push_back(r);
            C.set_row(id, dense_row(m, r), sparse);
        }
        std::vector<uint32_t> best(n);
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < int64_t(n); ++i) {
            double c0 = dist_row_center(m, uint64_t(i), C, 0, msr, prior, psum_restart, rs[i]);
            uint32_t bi = 0;
            for (uint64_t j = 0; j < k; ++j) {
                double c = dist_row_center(m, uint64_t(i), C, j, msr, prior, psum_restart, rs[i]);
                if (c < c0) { c0 = c; bi = uint32_t(j); }
            }
            costs[i] = m.kind == 1 ? double(float(c0)) : c0;
            best[i] = bi;
        }
        for (uint64_t i = 0; i < n; ++i) { asn[i] = best[i]; assigned[best[i]].push_back(i); }
        for (size_t e = 0; e < empty.size(); ++e) {
            const uint64_t pid = rsel[e];
            const uint32_t cid = empty[e];
            if (asn[pid] != cid) {  // the row also stays in its previous list (centroid.h:743-751)
                asn[pid] = cid;
                costs[pid] = 0.;
                assigned[cid].push_back(pid);
            }
        }
    }
    for (auto &a : assigned) std::sort(a.begin(), a.end());
    std::vector<float> out(m.d);
    for (uint32_t i = 0; i < k; ++i) {
        const auto &rows = assigned[i];
        if (rows.empty()) continue;
        if (rows.size() == 1) { C.set_row(i, dense_row(m, rows[0]), sparse); continue; }
        mean_of_rows(m, rows, w, out.data());
        for (float v : out) if (std::isnan(v)) return -1;
        C.set_row(i, out, sparse);
    }
    return restarted;
}

}  // namespace

// =======================================================================================
// C interface (test infrastructure)
// =======================================================================================
extern "C" {

struct orc_matrix {
    int32_t kind;
    int32_t pad;
    uint64_t n, d;
    const float *vals;
    const uint32_t *idx;
    const uint64_t *indptr;
};

static Mat to_mat(const orc_matrix *m) { return Mat{m->kind, m->n, m->d, m->vals, m->idx, m->indptr}; }

double orc_uniform(uint64_t seed, uint64_t i) { return uniform_at(seed, i); }
void orc_uniforms(uint64_t seed, uint64_t offset, uint64_t m, double *out) {
    for (uint64_t i = 0; i < m; ++i) out[i] = uniform_at(seed, offset + i);
}

double orc_det_sum(const double *v, uint64_t n) { return det_sum([&](uint64_t i) { return v[i]; }, n); }
uint64_t orc_det_draw(const double *v, uint64_t n, double u) { return det_draw([&](uint64_t i) { return v[i]; }, n, u); }

double orc_msr_dense(int msr, const float *row, const float *cen, uint64_t d, double prior, double prior_sum,
                     double rowsum, double ctrsum) {
    return msr_dense(msr, row, cen, d, prior, prior_sum, rowsum, ctrsum);
}
double orc_msr_sparse(int msr, const float *rv, const uint32_t *ri, uint64_t rnz, const float *cv,
                      const uint32_t *ci, uint64_t cnz, uint64_t d, double prior, double prior_sum, double rowsum,
                      double ctrsum) {
    return msr_sparse(msr, rv, ri, rnz, cv, ci, cnz, d, prior, prior_sum, rowsum, ctrsum);
}

// one hard assignment pass; centers dense k x d (sparse copies are made for CSR data)
int orc_assign(const orc_matrix *mm, const float *centers, uint32_t k, int msr, double prior, uint32_t *asn,
               double *costs) {
    const Mat m = to_mat(mm);
    CenterSet C;
    C.set_from_dense(centers, k, m.d, m.kind == 1);
    std::vector<double> rs(m.n);
    for (uint64_t i = 0; i < m.n; ++i) rs[i] = row_sum(m, i);
    const double psum = double(float(prior * double(m.d)));
    assign_all(m, C, msr, prior, psum, rs, asn, costs);
    return 0;
}

// coresets::kmeanspp (kmeans.h:49-215) with n_local_trials == 1 and no ls++.
// uniforms[0] picks the first center (floor(u * n)); uniforms[c] drives round c.
// greedy k-means++ (n_local_trials = L > 1, kmeans.h:79-177) with uniforms U(seed, r) from one
// counter: the first center is the best of L uniform picks (strictly lower objective wins);
// each round draws L candidates from (w *) dist without replacement (a drawn row's weight is
// zeroed for the next draw; index n -> 0), candidate 0 updates dist / asn in place (every row,
// its own included), candidates 1.. update copies of the first center's distances and
// assignments (odists, oasn) and replace dist / asn when their objective is strictly lower.
int orc_kmeanspp_greedy(const orc_matrix *mm, uint32_t k, int msr, double prior, const double *w, uint32_t L,
                        uint64_t seed, uint32_t *centers, uint32_t *asn_out, double *costs) {
    const Mat m = to_mat(mm);
    const uint64_t n = m.n;
    if (n == 0 || k == 0 || L < 2) return 1;
    if (k > n) k = uint32_t(n);
    std::vector<double> rs(n);
    for (uint64_t i = 0; i < n; ++i) rs[i] = row_sum(m, i);
    const double psum = prior * double(m.d);
    uint64_t counter = 0;
    auto U = [&]() { return uniform_at(seed, counter++); };
    auto pick = [&](double u) { uint64_t c = uint64_t(u * double(n)); return c >= n ? n - 1 : c; };
    auto cost_of = [&](const std::vector<double> &v) {
        return w ? det_sum([&](uint64_t i) { return w[i] * v[i]; }, n) : det_sum([&](uint64_t i) { return v[i]; }, n);
    };
    auto first_dists = [&](uint64_t c, std::vector<double> &v) {
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < int64_t(n); ++i)
            v[i] = (uint64_t(i) == c) ? 0. : dist_row_row(m, uint64_t(i), c, msr, prior, psum, rs[i], rs[c]);
    };
    std::vector<double> dist(n), tmp(n);
    uint64_t fc = pick(U());
    first_dists(fc, dist);
    double fcost = cost_of(dist);
    for (uint32_t t = 1; t < L; ++t) {
        const uint64_t ofc = pick(U());
        first_dists(ofc, tmp);
        const double oc = cost_of(tmp);
        if (oc < fcost) { std::swap(dist, tmp); fcost = oc; fc = ofc; }
    }
    std::vector<uint32_t> asn(n, 0u);
    centers[0] = uint32_t(fc);
    const std::vector<double> odists = dist;
    const std::vector<uint32_t> oasn = asn;
    std::vector<uint64_t> cand(L);
    std::vector<double> sv(n);
    std::vector<uint32_t> sa(n);
    for (uint32_t ci = 1; ci < k; ++ci) {
        std::vector<double> saved(L);
        for (uint32_t s = 0; s < L; ++s) {
            uint64_t c = w ? det_draw([&](uint64_t i) { return w[i] * dist[i]; }, n, U())
                           : det_draw([&](uint64_t i) { return dist[i]; }, n, U());
            if (c >= n) c = 0;
            cand[s] = c;
            saved[s] = dist[c];
            dist[c] = 0.;
        }
        for (int s = int(L) - 1; s >= 0; --s) dist[cand[s]] = saved[s];
        double dsum = -1.;
        uint32_t best = 0;
        for (uint32_t s = 0; s < L; ++s) {
            const uint64_t c = cand[s];
            std::vector<double> &V = s == 0 ? dist : sv;
            std::vector<uint32_t> &A = s == 0 ? asn : sa;
            if (s > 0) { sv = odists; sa = oasn; }
#pragma omp parallel for schedule(dynamic, 64)
            for (int64_t i = 0; i < int64_t(n); ++i) {
                const double dv = uint64_t(i) == c ? 0. : dist_row_row(m, uint64_t(i), c, msr, prior, psum, rs[i], rs[c]);
                if (dv < V[i]) { V[i] = dv; A[i] = ci; }
            }
            const double nsum = cost_of(V);
            if (s == 0) dsum = nsum;
            else if (nsum < dsum) { dsum = nsum; best = s; dist = sv; asn = sa; }
        }
        const uint64_t newc = cand[best];
        centers[ci] = uint32_t(newc);
        asn[newc] = ci;
        dist[newc] = 0.;
    }
    std::copy(asn.begin(), asn.end(), asn_out);
    std::copy(dist.begin(), dist.end(), costs);
    return 0;
}

// localsearch++ rounds (localsearchpp_rounds, optim/lsearchpp.h:21-123) on seeded centers.
// M[i][j] = msr(lh = row i, rh = center row j) (the kmeans++ oracle takes its first index as
// the center); dist = row minima of M.  Round r: u = U(seed ^ 0x4C53505053454544, r); sel drawn
// from dist (with weights: from the previous round's new costs times the weights, zeros
// before the first round; index n -> 0); nc[i] = msr(lh = row sel, rh = row i) (0 for sel);
// rows with nc > dist charge top2 - top1 of their M row (the reference's top-2 scan) to the
// top1 center unless tied, others add dist - nc to the gain; the first center with the least
// charge is replaced by sel when charge - gain < 0.  Charges per center and the gain are
// det_sum's of the masked per-row values.  Afterwards asn = first argmin of each M row.
int orc_lspp(const orc_matrix *mm, uint32_t k, int msr, double prior, const double *w, uint64_t rounds,
             uint64_t seed, uint32_t *centers, uint32_t *asn, double *costs) {
    const Mat m = to_mat(mm);
    const uint64_t n = m.n;
    if (k < 2 || n == 0) return 1;
    std::vector<double> rs(n);
    for (uint64_t i = 0; i < n; ++i) rs[i] = row_sum(m, i);
    const double psum = prior * double(m.d);
    std::vector<float> M(n * k);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < int64_t(n); ++i)
        for (uint32_t j = 0; j < k; ++j)
            M[uint64_t(i) * k + j] = float(dist_row_row(m, centers[j], uint64_t(i), msr, prior, psum, rs[centers[j]],
                                                        rs[uint64_t(i)]));
    std::vector<double> dist(n), nc(n, 0.), charge(n), gterm(n);
    std::vector<uint32_t> key(n);
    auto rowmin = [&]() {
        for (uint64_t i = 0; i < n; ++i) {
            float b = M[i * k];
            uint32_t bj = 0;
            for (uint32_t j = 1; j < k; ++j) if (M[i * k + j] < b) { b = M[i * k + j]; bj = j; }
            dist[i] = double(b);
            asn[i] = bj;
        }
    };
    rowmin();
    for (uint64_t r = 0; r < rounds; ++r) {
        const double u = uniform_at(seed ^ 0x4C53505053454544ull, r);
        uint64_t sel = w ? det_draw([&](uint64_t i) { return nc[i] * w[i]; }, n, u)
                         : det_draw([&](uint64_t i) { return dist[i]; }, n, u);
        if (sel >= n) sel = 0;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < int64_t(n); ++i)
            nc[i] = uint64_t(i) == sel ? 0. : dist_row_row(m, uint64_t(i), sel, msr, prior, psum, rs[uint64_t(i)], rs[sel]);
        for (uint64_t i = 0; i < n; ++i) {
            key[i] = 0xffffffffu; charge[i] = 0.; gterm[i] = 0.;
            if (nc[i] > dist[i]) {
                const float *row = &M[i * k];
                double v1 = row[0], v2 = row[1];
                uint32_t j1 = 0, j2 = 1;
                if (v2 < v1) { std::swap(v1, v2); std::swap(j1, j2); }
                for (uint32_t j = 2; j < k; ++j) {
                    const double v = row[j];
                    if (v < v2) {
                        if (v < v1) { v2 = v1; j2 = j1; v1 = v; j1 = j; }
                        else { v2 = v; j2 = j; }
                    }
                }
                if (v1 != v2) { key[i] = j1; charge[i] = v2 - v1; }
            } else {
                gterm[i] = dist[i] - nc[i];
            }
        }
        const double gain = det_sum([&](uint64_t i) { return gterm[i]; }, n);
        uint32_t am = 0;
        double best = 0.;
        for (uint32_t c = 0; c < k; ++c) {
            const double cc = det_sum([&](uint64_t i) { return key[i] == c ? charge[i] : 0.; }, n);
            if (c == 0 || cc < best) { best = cc; am = c; }
        }
        if (best - gain < 0.) {
            centers[am] = uint32_t(sel);
            for (uint64_t i = 0; i < n; ++i) M[i * k + am] = float(nc[i]);
            rowmin();
        }
    }
    rowmin();
    std::copy(dist.begin(), dist.end(), costs);
    return 0;
}

int orc_kmeanspp(const orc_matrix *mm, uint32_t k, int msr, double prior, const double *w, const double *uniforms,
                 uint32_t *centers, uint32_t *asn, double *costs) {
    const Mat m = to_mat(mm);
    const uint64_t n = m.n;
    if (n == 0 || k == 0) return 1;
    if (k > n) k = uint32_t(n);
    std::vector<double> rs(n);
    for (uint64_t i = 0; i < n; ++i) rs[i] = row_sum(m, i);
    const double psum = prior * double(m.d);
    std::vector<double> dist(n);
    uint64_t fc = uint64_t(uniforms[0] * double(n));
    if (fc >= n) fc = n - 1;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < int64_t(n); ++i)
        dist[i] = (uint64_t(i) == fc) ? 0. : dist_row_row(m, uint64_t(i), fc, msr, prior, psum, rs[i], rs[fc]);
    std::fill(asn, asn + n, 0u);
    centers[0] = uint32_t(fc);
    for (uint32_t ci = 1; ci < k; ++ci) {
        const double u = uniforms[ci];
        uint64_t newc = w ? det_draw([&](uint64_t i) { return w[i] * dist[i]; }, n, u)
                          : det_draw([&](uint64_t i) { return dist[i]; }, n, u);
        if (newc >= n || dist[newc] == 0.) {  // argmax fallback (kmeans.h:179-186): first maximum
            uint64_t am = 0;
            for (uint64_t i = 1; i < n; ++i) if (dist[i] > dist[am]) am = i;
            newc = am;
        }
        asn[newc] = ci;
        centers[ci] = uint32_t(newc);
        const double cs = rs[newc];
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < int64_t(n); ++i) {
            if (uint64_t(i) == newc) continue;
            if (dist[i] <= 0.) continue;
            const double dv = dist_row_row(m, uint64_t(i), newc, msr, prior, psum, rs[i], cs);
            if (dv < dist[i]) { asn[i] = ci; dist[i] = dv; }
        }
        dist[newc] = 0.;
    }
    std::copy(dist.begin(), dist.end(), costs);
    return 0;
}

// perform_hard_clustering (solve.h:98-175) from explicit dense centers.
// Returns 0 on success, 2 if a NaN center appeared, 3 for weighted L1 over CSR rows.
// L1 centers: set_centroids_l1 (clustering/centroid.h:435-504), dense rows (CSR rows: the
// sparse rule of l1_sparse_median below, a one-row cluster takes its row).  Empty clusters
// are reseeded one at a time (D^2 draw over the current costs, U(seed, r) with the restart
// counter), each followed by a pass that moves every row whose plain L1 distance to the new
// center (sequential float sum of |c - x|) is below its cost; repeated while clusters are
// empty.  Then every cluster takes the coordinate-wise median of its rows
// (optim/kmedian.h: l1_unweighted_median: sorted column, odd -> middle, even -> 0.5f * (the
// two middles)); with weights, weighted_median (kmedian.h:249-290) keeps wsum at 0, so it
// returns, per column, the value of the row with the largest weight (the smallest such value
// on ties).  Returns 0: the reference reports no restart from this policy.
inline float l1_plain(const float *c, const float *x, uint64_t d) {
    float a = 0.f;
    for (uint64_t j = 0; j < d; ++j) a = a + std::fabs(c[j] - x[j]);
    return a;
}

// l1_median over CSR rows, unweighted (util/csc.h:829-893), for the rows `rows` (nrows of
// them): per column the sorted nonzeros v (nel of them), h = nrows / 2, and
//   nel > h, all positive:  t = h - (nrows - nel); odd -> v[t], even -> 0.5f (v[t] + v[t+1])
//   nel > h, all negative:  t = nrows - h;          odd -> v[t], even -> 0.5f (v[t] + v[t+1])
//   nel > h, otherwise:     f = v and nrows - nel zeros, sorted; odd -> f[h], even ->
//                           0.5f (f[h] + f[h+1])
//   nrows odd, nel == h:    0.5f * v.front() if positive, 0.5f * v.back() if negative
//   else 0.
// A position past the end of its vector (where the reference reads out of bounds: nrows =
// 2, or all negative with nel = h + 1) takes the last element.
void l1_sparse_median(const Mat &m, const std::vector<uint64_t> &rows, std::vector<float> &out) {
    const uint64_t nrows = rows.size(), h = nrows / 2;
    std::map<uint32_t, std::vector<float>> feats;
    for (uint64_t r : rows)
        for (uint64_t p = m.indptr[r]; p < m.indptr[r + 1]; ++p) feats[m.idx[p]].push_back(m.vals[p]);
    out.assign(m.d, 0.f);
    auto at = [](const std::vector<float> &a, uint64_t q) { return a[std::min<uint64_t>(q, a.size() - 1)]; };
    for (auto &kv : feats) {
        std::vector<float> &v = kv.second;
        std::sort(v.begin(), v.end());
        const uint64_t nel = v.size();
        float r = 0.f;
        if (nel > h) {
            if (v.front() > 0.f || v.back() < 0.f) {
                const uint64_t t = v.front() > 0.f ? h - (nrows - nel) : nrows - h;
                r = (nrows & 1) ? at(v, t) : 0.5f * (at(v, t) + at(v, t + 1));
            } else {
                std::vector<float> f = v;
                f.resize(nrows, 0.f);
                std::sort(f.begin(), f.end());
                r = (nrows & 1) ? f[h] : 0.5f * (at(f, h) + at(f, h + 1));
            }
        } else if ((nrows & 1) && nel == h) {
            if (v.front() > 0.f) r = 0.5f * v.front();
            else if (v.back() < 0.f) r = 0.5f * v.back();
        }
        out[kv.first] = r;
    }
}

// set_centroids_l1 over dense or CSR rows; CSR rows with weights raise in the reference
// (util/csc.h:835): returns -3 then
int set_centroids_l1(const Mat &m, std::vector<uint32_t> &asn, std::vector<double> &costs, CenterSet &C,
                           const double *w, uint64_t seed, uint64_t &restart_counter) {
    const uint64_t n = m.n, k = C.k, d = m.d;
    std::vector<std::vector<uint64_t>> assigned(k);
    auto rebuild = [&](std::vector<uint32_t> &empty) {
        for (auto &a : assigned) a.clear();
        for (uint64_t i = 0; i < n; ++i) assigned[asn[i]].push_back(i);
        empty.clear();
        for (uint32_t c = 0; c < k; ++c) if (assigned[c].empty()) empty.push_back(c);
    };
    std::vector<uint32_t> empty;
    rebuild(empty);
    while (!empty.empty()) {
        for (uint32_t id : empty) {
            const double u = uniform_at(seed, restart_counter++);
            uint64_t r = det_draw([&](uint64_t i) { return costs[i]; }, n, u);
            if (r >= n) r = 0;
            const bool sparse = m.kind == 1;
            C.set_row(id, dense_row(m, r), sparse);
            const float *cr = &C.dense[uint64_t(id) * d];
            for (uint64_t i = 0; i < n; ++i) {
                const double c = sparse ? l1_plain(cr, dense_row(m, i).data(), d) : l1_plain(cr, m.vals + i * d, d);
                if (c < costs[i]) { asn[i] = id; costs[i] = c; }
            }
        }
        rebuild(empty);
    }
    std::vector<float> col, out(d);
    if (m.kind == 1) {
        if (w) return -3;
        for (uint32_t c = 0; c < k; ++c) {
            if (assigned[c].size() == 1) C.set_row(c, dense_row(m, assigned[c][0]), true);
            else {
                l1_sparse_median(m, assigned[c], out);
                C.set_row(c, out, true);
            }
        }
        return 0;
    }
    for (uint32_t c = 0; c < k; ++c) {
        const auto &rows = assigned[c];  // ascending
        const uint64_t mc = rows.size();
        if (w) {
            double maxw = -std::numeric_limits<double>::max();
            for (uint64_t r : rows) maxw = std::max(maxw, w[r]);
            for (uint64_t j = 0; j < d; ++j) {
                float best = std::numeric_limits<float>::infinity();
                for (uint64_t r : rows)
                    if (w[r] == maxw) best = std::min(best, m.vals[r * d + j]);
                out[j] = best;
            }
        } else {
            col.resize(mc);
            for (uint64_t j = 0; j < d; ++j) {
                for (uint64_t q = 0; q < mc; ++q) col[q] = m.vals[rows[q] * d + j];
                std::sort(col.begin(), col.end());
                const uint64_t h = mc / 2;
                out[j] = (mc & 1) ? col[h] : 0.5f * (col[h - 1] + col[h]);
            }
        }
        C.set_row(c, out, false);
    }
    return 0;
}

// the L1 center rule alone (no empty cluster allowed): centers_out[k][d]
int orc_l1_centers(const orc_matrix *mm, const uint32_t *asn_in, uint32_t k, const double *w, float *centers_out) {
    const Mat m = to_mat(mm);
    std::vector<uint32_t> asn(asn_in, asn_in + m.n);
    std::vector<double> costs(m.n, 0.0);
    CenterSet C;
    std::vector<float> zero(uint64_t(k) * m.d, 0.f);
    C.set_from_dense(zero.data(), k, m.d, m.kind == 1);
    uint64_t rc = 0;
    for (uint64_t i = 0; i < m.n; ++i) if (asn[i] >= k) return 2;
    std::vector<uint64_t> cnt(k, 0);
    for (uint64_t i = 0; i < m.n; ++i) ++cnt[asn[i]];
    for (uint32_t c = 0; c < k; ++c) if (!cnt[c]) return 3;
    if (set_centroids_l1(m, asn, costs, C, w, 0, rc) == -3) return 4;
    std::copy(C.dense.begin(), C.dense.end(), centers_out);
    return 0;
}

int orc_hcluster(const orc_matrix *mm, const float *centers_in, uint32_t k, int msr, double prior, const double *w,
                 double eps, uint64_t maxiter, uint64_t seed, float *centers_out, uint32_t *asn_out, double *costs_out,
                 double *initcost_out, double *finalcost_out, uint64_t *numiter_out) {
    const Mat m = to_mat(mm);
    const uint64_t n = m.n;
    const bool sparse = m.kind == 1;
    std::vector<double> rs(n);
    for (uint64_t i = 0; i < n; ++i) rs[i] = row_sum(m, i);
    const double psum = double(float(prior * double(m.d)));
    CenterSet centers, cpy;
    centers.set_from_dense(centers_in, k, m.d, sparse);
    std::vector<uint32_t> asn(n);
    std::vector<double> costs(n);
    uint64_t restart_counter = 0;
    assign_all(m, centers, msr, prior, psum, rs, asn.data(), costs.data());
    const float initcost = compute_cost(costs.data(), w, n);
    float cost = initcost;
    uint64_t iternum = 0;
    int rc = 0;
    if (cost == 0.f) {
        *initcost_out = 0.; *finalcost_out = 0.; *numiter_out = 0;
    } else {
        cpy = centers;
        for (;;) {
            // L1 takes coordinate-wise medians (centroid.h:203, 487-504; util/csc.h:829-893)
            int res = msr == L1 ? set_centroids_l1(m, asn, costs, cpy, w, seed, restart_counter)
                                : set_centroids_full_mean(m, msr, prior, asn, costs, cpy, w, rs, seed, restart_counter);
            if (res == -3) { rc = 3; break; }
            if (res < 0) { rc = 2; break; }
            assign_all(m, cpy, msr, prior, psum, rs, asn.data(), costs.data());
            const float newcost = compute_cost(costs.data(), w, n);
            if (newcost > cost && !res) {
                assign_all(m, centers, msr, prior, psum, rs, asn.data(), costs.data());
                break;
            }
            centers = cpy;
            ++iternum;
            const float oldcost = cost;
            cost = newcost;
            if (double(oldcost - newcost) < eps * std::max(double(newcost), double(oldcost)) || iternum > maxiter) break;
        }
        *initcost_out = initcost; *finalcost_out = cost; *numiter_out = iternum;
    }
    std::copy(centers.dense.begin(), centers.dense.end(), centers_out);
    std::copy(asn.begin(), asn.end(), asn_out);
    std::copy(costs.begin(), costs.end(), costs_out);
    return rc;
}

// perform_hard_minibatch_clustering (clustering/solve.h:386-582).  Every freq iterations
// (and at the last): exhaustive assignment, restart of centers with <= reseed_after rows
// (D^2 draw U(seed, r) over the costs, all restarts from the same costs; then every row
// takes the best restarted center if strictly cheaper), FP64 objective; between
// checkins: a sample of rows (minibatch_sample below), each assigned exactly, and each
// hit center replaced by the mean of its sampled rows (ascending, repeats included;
// singletons copy the row).  Distances use the prior itself as the prior sum
// (solve.h:405).  The centers of the best objective are returned.
static std::vector<uint32_t> minibatch_sample(uint64_t seed, uint64_t &counter, uint64_t n, uint64_t mbsize,
                                              bool with_rep) {
    const uint64_t s = seed ^ 0x6A09E667F3BCC908ull;
    std::vector<uint32_t> out;
    auto draw = [&]() {
        uint64_t r = uint64_t(uniform_at(s, counter++) * double(n));
        return uint32_t(r >= n ? n - 1 : r);
    };
    if (with_rep) {
        out.resize(mbsize);
        for (auto &v : out) v = draw();
    } else {
        const uint64_t target = std::min(mbsize, n);
        std::set<uint32_t> seen;
        while (out.size() < target) {
            const uint32_t r = draw();
            if (seen.insert(r).second) out.push_back(r);
        }
    }
    std::sort(out.begin(), out.end());
    return out;
}

int orc_minibatch(const orc_matrix *mm, const float *centers_in, uint32_t k, int msr, double prior, const double *w,
                  uint64_t mbsize, uint64_t maxiter, uint64_t freq, uint64_t reseed_after, int with_rep,
                  uint64_t seed, float *centers_out, uint32_t *asn_out, double *costs_out, double *initcost_out,
                  double *finalcost_out, uint64_t *numiter_out) {
    const Mat m = to_mat(mm);
    const uint64_t n = m.n, d = m.d;
    const bool sparse = m.kind == 1;
    if (freq == 0) freq = 1;
    std::vector<double> rs(n);
    for (uint64_t i = 0; i < n; ++i) rs[i] = row_sum(m, i);
    const double psum = double(float(prior));
    CenterSet C;
    C.set_from_dense(centers_in, k, d, sparse);
    std::vector<float> save = C.dense;
    std::vector<uint32_t> asn(n);
    std::vector<double> costs(n);
    uint64_t rc = 0, sc = 0, iternum = 0;
    double initcost = 0.0, bestcost = 0.0, cost = 0.0;
    for (;;) {
        if (iternum % freq == 0 || iternum == maxiter - 1) {
            assign_all(m, C, msr, prior, psum, rs, asn.data(), costs.data());
            std::vector<uint64_t> cnt(k, 0);
            for (uint64_t i = 0; i < n; ++i) ++cnt[asn[i]];
            std::vector<uint32_t> found;
            for (uint32_t c = 0; c < k; ++c) if (cnt[c] <= reseed_after) found.push_back(c);
            if (!found.empty()) {
                for (uint32_t c : found) {
                    const double u = uniform_at(seed, rc++);
                    uint64_t r = w ? det_draw([&](uint64_t i) { return costs[i] * w[i]; }, n, u)
                                   : det_draw([&](uint64_t i) { return costs[i]; }, n, u);
                    if (r >= n) r = 0;
                    C.set_row(c, dense_row(m, r), sparse);
                }
#pragma omp parallel for schedule(dynamic, 64)
                for (int64_t i = 0; i < int64_t(n); ++i) {
                    double best = dist_row_center(m, uint64_t(i), C, found[0], msr, prior, psum, rs[i]);
                    uint32_t bc = found[0];
                    for (size_t f = 1; f < found.size(); ++f) {
                        const double v = dist_row_center(m, uint64_t(i), C, found[f], msr, prior, psum, rs[i]);
                        if (v < best) { best = v; bc = found[f]; }
                    }
                    if (sparse) best = double(float(best));
                    if (best < costs[i]) { costs[i] = best; asn[i] = bc; }
                }
            }
            cost = w ? det_sum([&](uint64_t i) { return costs[i] * w[i]; }, n)
                     : det_sum([&](uint64_t i) { return costs[i]; }, n);
            if (iternum == 0) initcost = bestcost = cost;
            if (cost < bestcost) { bestcost = cost; save = C.dense; }
        }
        if (++iternum == maxiter) break;
        const std::vector<uint32_t> smp = minibatch_sample(seed, sc, n, mbsize, with_rep != 0);
        std::vector<std::vector<uint64_t>> groups(k);
        for (uint32_t r : smp) {
            double best = dist_row_center(m, r, C, 0, msr, prior, psum, rs[r]);
            uint32_t bc = 0;
            for (uint32_t c = 1; c < k; ++c) {
                const double v = dist_row_center(m, r, C, c, msr, prior, psum, rs[r]);
                if (v < best) { best = v; bc = c; }
            }
            groups[bc].push_back(r);
        }
        std::vector<float> out(d);
        for (uint32_t c = 0; msr == L1 && c < k; ++c) {
            // l1_median of the group (solve.h:559-561): CSR rows by the sparse rule (weights
            // raise); dense rows by the sorted median, or with weights by weighted_median over
            // rows(data, asp, nasn) reading the FULL weight vector at the group position q
            // (kmedian.h:329-344): largest w[q], smallest value among its ties
            const auto &g = groups[c];
            if (g.empty()) continue;
            if (sparse) {
                if (w) return 3;
                l1_sparse_median(m, g, out);
            } else if (w) {
                double mx = -std::numeric_limits<double>::max();
                for (uint64_t q = 0; q < g.size() && q < n; ++q) mx = std::max(mx, w[q]);
                for (uint64_t j = 0; j < d; ++j) {
                    float b = std::numeric_limits<float>::infinity();
                    for (uint64_t q = 0; q < g.size() && q < n; ++q)
                        if (w[q] == mx) b = std::min(b, m.vals[g[q] * d + j]);
                    out[j] = b;
                }
            } else {
                std::vector<float> col(g.size());
                for (uint64_t j = 0; j < d; ++j) {
                    for (uint64_t q = 0; q < g.size(); ++q) col[q] = m.vals[g[q] * d + j];
                    std::sort(col.begin(), col.end());
                    const uint64_t hh = g.size() / 2;
                    out[j] = (g.size() & 1) ? col[hh] : 0.5f * (col[hh - 1] + col[hh]);
                }
            }
            C.set_row(c, out, sparse);
        }
        for (uint32_t c = 0; msr != L1 && c < k; ++c) {
            const auto &g = groups[c];
            if (g.empty()) continue;
            if (g.size() == 1) { C.set_row(c, dense_row(m, g[0]), sparse); continue; }
            mean_of_rows(m, g, w, out.data());
            for (float v : out) if (std::isnan(v)) return 2;
            C.set_row(c, out, sparse);
        }
    }
    std::copy(save.begin(), save.end(), centers_out);
    std::copy(asn.begin(), asn.end(), asn_out);
    std::copy(costs.begin(), costs.end(), costs_out);
    *initcost_out = initcost;
    *finalcost_out = bestcost;
    *numiter_out = iternum;
    return 0;
}

// perform_soft_clustering (clustering/solve.h:287-374) over dense rows with the soft
// weighted means of set_centroids_full_mean (centroid.h:795-866): asn = row softmax of
// -temp * costs (max-shifted, sequential float sums; a NaN first entry becomes equal shares
// over the minimal costs, centroid.h:782-793), objective sum_i w_i dot(costs_i, asn_i) in the
// canonical FP64 order, center_c = (sum_i coef x_i) * (1 / sum_i coef) with coef = asn *
// float(w), compensated float sums over chunks of 256 rows and FP64 across chunks.
int orc_scluster(const orc_matrix *mm, const float *centers_in, uint32_t k, int msr, double prior, const double *w,
                 double temp, uint64_t maxiter, double eps, float *centers_out, float *costs_out, float *asn_out,
                 double *initcost_out, double *finalcost_out, uint64_t *numiter_out) {
    const Mat m = to_mat(mm);
    const uint64_t n = m.n, d = m.d;
    const bool sparse = m.kind == 1;
    // a weighted L1 median over CSR rows raises in the reference (util/csc.h:835)
    if (sparse && msr == L1) return -2;
    // CSR rows: the soft means read a dense copy (a zero adds exactly nothing to the
    // compensated sums, so this is the per-nonzero accumulation of the device path)
    std::vector<float> dense_all;
    if (sparse) {
        dense_all.assign(n * d, 0.f);
        for (uint64_t i = 0; i < n; ++i)
            for (uint64_t p = m.indptr[i]; p < m.indptr[i + 1]; ++p) dense_all[i * d + m.idx[p]] = m.vals[p];
    }
    const float *xv = sparse ? dense_all.data() : m.vals;
    std::vector<double> rs(n);
    for (uint64_t i = 0; i < n; ++i) rs[i] = row_sum(m, i);
    const double psum = double(float(prior * double(d)));
    CenterSet acc, cpy;
    acc.set_from_dense(centers_in, k, d, sparse);
    cpy = acc;
    std::vector<float> costs(n * k), asn(n * k);
    auto fill_costs = [&]() {
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < int64_t(n); ++i)
            for (uint32_t c = 0; c < k; ++c)
                costs[uint64_t(i) * k + c] = float(dist_row_center(m, uint64_t(i), cpy, c, msr, prior, psum, rs[i]));
    };
    fill_costs();
    double cost = std::numeric_limits<double>::max(), initcost = -1.0;
    uint64_t iternum = 0;
    const float ft = float(temp);
    std::vector<double> rowval(n);
    for (;;) {
        const double oldcost = cost;
        for (uint64_t i = 0; i < n; ++i) {
            const float *cr = &costs[i * k];
            float *ar = &asn[i * k];
            float mx = -ft * cr[0];
            for (uint32_t c = 1; c < k; ++c) mx = std::max(mx, -ft * cr[c]);
            float s = 0.f;
            for (uint32_t c = 0; c < k; ++c) { ar[c] = std::exp(-ft * cr[c] - mx); s = s + ar[c]; }
            for (uint32_t c = 0; c < k; ++c) ar[c] = ar[c] / s;
            if (std::isnan(ar[0])) {
                float best = cr[0];
                for (uint32_t c = 1; c < k; ++c) if (cr[c] < best) best = cr[c];
                uint32_t ties = 0;
                for (uint32_t c = 0; c < k; ++c) ties += cr[c] == best;
                const float per = 1.f / float(ties ? ties : 1u);
                for (uint32_t c = 0; c < k; ++c) ar[c] = cr[c] == best ? per : 0.f;
            }
            float dot = 0.f;
            for (uint32_t c = 0; c < k; ++c) dot = dot + cr[c] * ar[c];
            rowval[i] = double(dot);
        }
        cost = w ? det_sum([&](uint64_t i) { return rowval[i] * w[i]; }, n)
                 : det_sum([&](uint64_t i) { return rowval[i]; }, n);
        std::vector<float> nc(uint64_t(k) * d);
        // L1 (dense): weighted_median with the soft assignments as weights returns, per
        // column, the smallest value among the rows of largest weight (centroid.h:815-838)
        for (uint32_t c = 0; msr == L1 && c < k; ++c) {
            double mx = -std::numeric_limits<double>::max();
            for (uint64_t r = 0; r < n; ++r) mx = std::max(mx, (w ? w[r] : 1.0) * double(asn[r * k + c]));
            for (uint64_t j = 0; j < d; ++j) {
                float b = std::numeric_limits<float>::infinity();
                for (uint64_t r = 0; r < n; ++r)
                    if ((w ? w[r] : 1.0) * double(asn[r * k + c]) == mx) b = std::min(b, xv[r * d + j]);
                nc[uint64_t(c) * d + j] = b;
            }
        }
        for (uint32_t c = 0; msr != L1 && c < k; ++c) {
            for (uint64_t j = 0; j < d; ++j) {
                double num = 0.0, den = 0.0;
                for (uint64_t r0 = 0; r0 < n; r0 += 256) {
                    const uint64_t r1 = std::min<uint64_t>(n, r0 + 256);
                    float s = 0.f, e = 0.f, sw = 0.f, ew = 0.f;
                    for (uint64_t r = r0; r < r1; ++r) {
                        const float coef = w ? asn[r * k + c] * float(w[r]) : asn[r * k + c];
                        two_sum_add(s, e, coef * xv[r * d + j]);
                        two_sum_add(sw, ew, coef);
                    }
                    num = num + (double(s) + double(e));
                    den = den + (double(sw) + double(ew));
                }
                nc[uint64_t(c) * d + j] = float(num * (1.0 / den));
            }
        }
        cpy.set_from_dense(nc.data(), k, d, sparse);
        fill_costs();
        if (initcost < 0) initcost = cost;
        if (oldcost >= cost) acc = cpy;
        if (oldcost - cost <= eps * std::max(oldcost, cost) || ++iternum == maxiter) break;
    }
    std::copy(acc.dense.begin(), acc.dense.end(), centers_out);
    std::copy(costs.begin(), costs.end(), costs_out);
    std::copy(asn.begin(), asn.end(), asn_out);
    *initcost_out = initcost;
    *finalcost_out = cost;
    *numiter_out = iternum;
    return 0;
}

// CoresetSampler (coreset.h:340-578).  The sampler keeps point weights as float
// (CoresetSampler<float,uint32_t>::weights_, coreset.h:234,290), so `w` is float here.
// Per-cluster sums (weight, cost, count) are FP64 over the cluster's points in ascending
// index order, in chunks of 256 points (sequential within a chunk, chunk partials summed
// in order).  Per-point sensitivity arithmetic is FP64; probabilities are stored as float.
// methods: 0 BFL, 1 FL, 2 LFKF, 3 VX, 4 LBK.  costs_f64 != 0 -> costs is double*.
// ---------------------------------------------------------------------------------------
static std::vector<double> cluster_sums(uint64_t n, uint64_t nc, const uint32_t *asn,
                                        const std::function<double(uint64_t)> &val) {
    std::vector<std::vector<uint64_t>> lists(nc);
    for (uint64_t i = 0; i < n; ++i) lists[asn[i]].push_back(i);
    std::vector<double> out(nc, 0.0);
    for (uint64_t c = 0; c < nc; ++c) {
        const auto &L = lists[c];
        double S = 0.0;
        bool first = true;
        for (uint64_t q0 = 0; q0 < L.size(); q0 += 256) {
            double p = 0.0;
            for (uint64_t q = q0; q < std::min<uint64_t>(L.size(), q0 + 256); ++q) p = p + val(L[q]);
            S = first ? p : S + p;
            first = false;
        }
        out[c] = S;
    }
    return out;
}

int orc_sensitivity(uint64_t n, uint64_t ncenters, uint64_t k, const void *costs, int costs_f64, const uint32_t *asn,
                    const float *w, int method, double alpha_est, float *probs) {
    auto cost = [&](uint64_t i) -> double {
        return costs_f64 ? ((const double *)costs)[i] : double(((const float *)costs)[i]);
    };
    auto wt = [&](uint64_t i) -> double { return w ? double(w[i]) : 1.0; };
    for (uint64_t i = 0; i < n; ++i) if (asn[i] >= ncenters) return 1;
    const std::vector<double> cnt = cluster_sums(n, ncenters, asn, [&](uint64_t) { return 1.0; });
    const std::vector<double> wsum = cluster_sums(n, ncenters, asn, wt);
    std::vector<double> s(n);
    switch (method) {
        case 0: {  // BFL (coreset.h:534-578)
            const double total_cost = det_sum([&](uint64_t i) { return wt(i) * cost(i); }, n);
            for (uint64_t i = 0; i < n; ++i) {
                const double fraccost = wt(i) * cost(i) / total_cost;
                const double fracw = wt(i) / (wsum[asn[i]] * cnt[asn[i]]);
                s[i] = 0.5 * (fraccost + fracw);
            }
            break;
        }
        case 1: {  // FL (coreset.h:456-486): not normalised
            const double total_cost = det_sum([&](uint64_t i) { return wt(i) * cost(i); }, n);
            const double inv = 1.0 / total_cost;
            for (uint64_t i = 0; i < n; ++i) {
                if (w) probs[i] = float(wt(i) * cost(i) * inv);
                else probs[i] = float(std::ceil(double(n) * inv * cost(i)) + 1.0);
            }
            return 0;
        }
        case 2: {  // LFKF (coreset.h:340-381): squared costs, per-point (the reference sizes
                   // its per-point buffer by ncenters; the per-point intent is used here)
            const std::vector<double> csum = cluster_sums(n, ncenters, asn, [&](uint64_t i) { return wt(i) * cost(i) * cost(i); });
            const double tc2 = det_sum([&](uint64_t i) { return wt(i) * cost(i) * cost(i); }, n);
            for (uint64_t i = 0; i < n; ++i) {
                const uint32_t a = asn[i];
                s[i] = alpha_est * wt(i) * (cost(i) * cost(i) + csum[a] / wsum[a]) + 2.0 * tc2 / wsum[a];
            }
            break;
        }
        case 3: {  // VX (coreset.h:423-455)
            const double total_cost = det_sum([&](uint64_t i) { return wt(i) * cost(i); }, n);
            for (uint64_t i = 0; i < n; ++i) s[i] = wt(i) * cost(i) / total_cost + 1.0 / cnt[asn[i]];
            break;
        }
        case 4: {  // LBK (coreset.h:487-533)
            const std::vector<double> csum = cluster_sums(n, ncenters, asn, [&](uint64_t i) { return wt(i) * cost(i); });
            const double total_cost = det_sum([&](uint64_t i) { return wt(i) * cost(i); }, n);
            const double alpha = 16.0 * std::log(double(k)) + 32.0, alpha2 = 2.0 * alpha;
            double W = 0.0;
            for (uint64_t c = 0; c < ncenters; ++c) W = W + wsum[c];
            const double avg = total_cost / W;
            const double tcinv = alpha / avg;
            std::vector<double> adj(ncenters);
            for (uint64_t c = 0; c < ncenters; ++c) adj[c] = alpha2 * csum[c] / (wsum[c] * avg) + 4.0 * W / wsum[c];
            for (uint64_t i = 0; i < n; ++i) s[i] = tcinv * cost(i) + adj[asn[i]];
            break;
        }
        default: return 1;
    }
    const double tot = det_sum([&](uint64_t i) { return s[i]; }, n);
    const double inv = 1.0 / tot;
    for (uint64_t i = 0; i < n; ++i) probs[i] = float(s[i] * inv);
    return 0;
}

// Canonical FP64 scan (mirrors the CUDA scan kernels): chunks of 8192 elements, 256
// threads each owning a contiguous run of 32 elements scanned sequentially; run totals
// scanned sequentially within the chunk; chunk totals scanned sequentially.  Exclusive
// prefix of element e = (chunk offset + run offset) + local exclusive prefix.
static void canon_exclusive_scan(const std::vector<double> &v, std::vector<double> &P) {
    const uint64_t m = v.size();
    P.assign(m + 1, 0.0);
    const uint64_t G = (m + kChunk - 1) / kChunk;
    double chunk_off = 0.0;
    for (uint64_t g = 0; g < G; ++g) {
        double run_off = 0.0;
        for (uint64_t t = 0; t < kThreads; ++t) {
            const uint64_t b = g * kChunk + t * kPer;
            double loc = 0.0;
            for (uint64_t e = b; e < std::min<uint64_t>(m, b + kPer); ++e) {
                P[e] = (chunk_off + run_off) + loc;
                loc = loc + v[e];
            }
            run_off = run_off + loc;
        }
        chunk_off = chunk_off + run_off;
    }
    P[m] = chunk_off;
}

// Alias table ("sweep" construction in closed form, FP64).  q_i = p_i * n / sum(p) with
// the sum in the canonical det order.  Light items (q < 1, index order) have deficits
// 1 - q, heavy items (q >= 1, index order) have excesses q - 1; D and E are their
// canonical exclusive prefix sums.  Sweeping the lights in order against the heavies in
// order, light i is served by the first heavy j with E[j+1] >= D[i]; heavy j runs out
// while serving the first light i with D[i+1] > E[j+1] and then keeps probability
// 1 - (D[i+1] - E[j+1]) with heavy j+1 as its alias.  The result is the table the
// sequential sweep builds in exact arithmetic; every entry is computed independently.
int orc_alias_build(uint64_t n, const float *probs, double *prob_tab, uint32_t *alias_tab) {
    if (n == 0) return 1;
    const double S = det_sum([&](uint64_t i) { return double(probs[i]); }, n);
    if (!(S > 0.0)) return 1;
    const double scale = double(n) / S;
    std::vector<uint32_t> L, H;
    std::vector<double> dl, eh;
    auto q = [&](uint64_t i) { return double(probs[i]) * scale; };
    for (uint64_t i = 0; i < n; ++i) {
        if (q(i) < 1.0) { L.push_back(uint32_t(i)); dl.push_back(1.0 - q(i)); }
        else { H.push_back(uint32_t(i)); eh.push_back(q(i) - 1.0); }
    }
    if (H.empty()) {
        for (uint64_t i = 0; i < n; ++i) { prob_tab[i] = 1.0; alias_tab[i] = uint32_t(i); }
        return 0;
    }
    std::vector<double> D, E;
    canon_exclusive_scan(dl, D);
    canon_exclusive_scan(eh, E);
    const uint64_t nl = L.size(), nh = H.size();
    for (uint64_t i = 0; i < nl; ++i) {
        // first j with E[j+1] >= D[i]
        uint64_t lo = 0, hi = nh;  // search j in [0, nh)
        while (lo < hi) { uint64_t mid = (lo + hi) / 2; if (E[mid + 1] >= D[i]) hi = mid; else lo = mid + 1; }
        const uint64_t j = lo < nh ? lo : nh - 1;
        prob_tab[L[i]] = q(L[i]);
        alias_tab[L[i]] = H[j];
    }
    for (uint64_t j = 0; j < nh; ++j) {
        uint64_t i = nl;
        if (j + 1 < nh) {
            // first i with D[i+1] > E[j+1]
            uint64_t lo = 0, hi = nl;
            while (lo < hi) { uint64_t mid = (lo + hi) / 2; if (D[mid + 1] > E[j + 1]) hi = mid; else lo = mid + 1; }
            i = lo;
        }
        if (i < nl) { prob_tab[H[j]] = 1.0 - (D[i + 1] - E[j + 1]); alias_tab[H[j]] = H[j + 1]; }
        else { prob_tab[H[j]] = 1.0; alias_tab[H[j]] = H[j]; }
    }
    return 0;
}

uint64_t orc_alias_draw(uint64_t np, const double *prob_tab, const uint32_t *alias_tab, uint64_t seed, uint64_t s) {
    const double u1 = uniform_at(seed, 2 * s), u2 = uniform_at(seed, 2 * s + 1);
    uint64_t i = uint64_t(u1 * double(np));
    if (i >= np) i = np - 1;
    return (u2 < prob_tab[i]) ? i : alias_tab[i];
}

// CoresetSampler::sample (coreset.h:625-699).  Draw s uses U(seed, 2s) for the bucket and
// U(seed, 2s+1) for the coin.  With unique, draws continue until sampled_directly distinct
// indices were seen; the entries are sorted by index and weighted by their count, in the
// reference's float arithmetic (coreset.h:669).  FL samples m - b points directly and
// leaves the remaining b entries zero (no bicriteria points are set through the binding).
// Writes m entries.
void orc_coreset_sample(uint64_t np, const float *probs, const double *prob_tab, const uint32_t *alias_tab,
                        const float *w, int method, uint64_t b, uint64_t m, uint64_t seed, int unique,
                        float *weights_out, uint64_t *idx_out) {
    const uint64_t sampled_directly = (method == 1) ? (m > b ? m - b : 0) : m;
    auto wt = [&](uint64_t i) -> float { return w ? w[i] : 1.f; };
    for (uint64_t i = 0; i < m; ++i) { weights_out[i] = 0.f; idx_out[i] = 0; }
    if (!unique) {
        for (uint64_t s = 0; s < sampled_directly; ++s) {
            const uint64_t ind = orc_alias_draw(np, prob_tab, alias_tab, seed, s);
            idx_out[s] = ind;
            weights_out[s] = float(double(wt(ind)) / (double(m) * double(probs[ind])));
        }
        return;
    }
    std::map<uint64_t, uint32_t> ctr;
    for (uint64_t s = 0; ctr.size() < sampled_directly; ++s) ++ctr[orc_alias_draw(np, prob_tab, alias_tab, seed, s)];
    uint64_t o = 0;
    for (const auto &kv : ctr) {
        idx_out[o] = kv.first;
        weights_out[o] = float(kv.second) * (wt(kv.first) / (float(m) * probs[kv.first]));
        ++o;
    }
}

}  // extern "C"
