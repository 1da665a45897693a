// Sorting / centroid / statistics launchers (mc_reduce.cu).
#pragma once
#include "mc_internal.cuh"

namespace mc {

constexpr uint64_t kSortTile = 2048;

struct SortWork {
    DBuf<uint32_t> tile_counts;   // [k][ntiles] counts, then per-tile cursors
    DBuf<uint64_t> bucket_count;  // [k]
    DBuf<uint64_t> bucket_start;  // [k+1]
    DBuf<uint32_t> perm;          // rows grouped by bucket, ascending within a bucket
    DBuf<uint64_t> chunk_count;   // [k]
    DBuf<uint64_t> chunk_start;   // [k+1]
    DBuf<double> partial;         // [chunks][d]
    DBuf<double> partial_w;       // [chunks]
};

struct CentroidArgs {
    bool csr = false;
    uint64_t n = 0, d = 0;
    uint32_t k = 0;
    const float *X = nullptr;                 // dense
    const float *vals = nullptr;              // CSR
    const uint32_t *idx = nullptr;
    const uint64_t *indptr = nullptr;
    uint64_t nnz = 0;                         // CSR nonzeros (picks the row-pipelined kernel)
    const uint32_t *keys = nullptr;           // cluster of each row
    const uint32_t *keys2 = nullptr;          // optional second membership (0xffffffff none)
    uint64_t extra_members = 0;               // number of valid keys2 entries
    const double *w = nullptr;                // optional row weights
    float *centers = nullptr;                 // [k][d], updated in place
    int *nan_flag = nullptr;
};

int launch_sort_by_key(const uint32_t *keys, const uint32_t *keys2, uint64_t n, uint32_t k, SortWork &w,
                       cudaStream_t st);
// presorted: w already holds the counting sort of a.keys (no second membership)
int launch_centroids(const CentroidArgs &a, SortWork &w, cudaStream_t st, bool presorted = false);

// L1 centers over dense rows (set_centroids_l1, clustering/centroid.h:435-504), from the
// current counting sort of the rows by cluster: per cluster the coordinate-wise median
// (unweighted: odd -> middle, even -> 0.5f * (the two middles)); with weights, per column
// the value of the row with the largest weight (smallest such value on ties), which is what
// the reference's weighted_median returns.  Clusters without rows keep their center.
// nw_local > 0: the r-th row of a cluster (ascending) weighs weights[r], as the minibatch
// update's weighted_median(rows(data, asp, nasn), ret, *weights) reads them (kmedian.h:335);
// positions past nw_local take no part.
int launch_l1_medians(const float *X, uint64_t d, uint32_t k, const SortWork &w, const double *weights,
                      float *centers, cudaStream_t st, uint64_t nw_local = 0);
// the L1 restart's pass after reseeding center `id` at `center`: rows whose plain L1
// distance (sequential float sum of |c - x|) is below their cost move to it
int launch_l1_reseed_update(const float *X, uint64_t n, uint64_t d, const float *center, uint32_t id,
                            uint32_t *asn, double *costs, cudaStream_t st);
// L1 centers over CSR rows, unweighted (set_centroids_l1 -> util/csc.h:829-893): each
// (cluster, column) bucket of a cluster of m rows with nel nonzeros takes the reference's
// sparse median rule.  Up to 2^28 buckets: per-bucket counts, an atomic scatter of the value
// keys into their buckets and a radix select per bucket that needs an order statistic.  More
// buckets (or MC_L1CSR_SORT=1): every nonzero as ((cluster << 32) | column, value key),
// sorted by an LSD radix sort (digits of at most 11 bits: the value, then the column, then
// the cluster), then one thread per run.  Clusters with one row take that row; clusters
// without rows keep their center.
struct L1CsrWork {
    DBuf<uint64_t> key, key2;
    DBuf<uint32_t> val, val2, digit;
    SortWork sort;
    DBuf<uint64_t> cnt, off, cur, runs, scan;
};
int launch_l1_medians_csr(const float *vals, const uint32_t *idx, const uint64_t *indptr, uint64_t n, uint64_t d,
                          uint64_t nnz, uint32_t k, const uint32_t *asn, const SortWork &rows, L1CsrWork &w,
                          float *centers, cudaStream_t st);
// launch_l1_reseed_update over CSR rows, the new center being CSR row *rsel (device): the
// sequential float sum of |c_j - x_j| over the union of the two rows' columns, which equals
// the sum over every column
int launch_l1_reseed_update_csr(const float *vals, const uint32_t *idx, const uint64_t *indptr, uint64_t n,
                                const uint64_t *rsel, uint32_t id, uint32_t *asn, double *costs, cudaStream_t st);
// scratch: optional work space (kept by the caller, so that a captured graph allocates nothing)
int launch_exclusive_scan_u64(const uint64_t *in, uint64_t *out, uint64_t m, cudaStream_t st,
                              DBuf<uint64_t> *scratch = nullptr);
int launch_center_sums(const float *C, uint32_t k, uint64_t d, double *csum, float *cnorm, cudaStream_t st);

}  // namespace mc
