// k-means++ launcher (mc_kmpp.cu).
#pragma once
#include "mc_internal.cuh"

namespace mc {

struct KmppArgs {
    int msr = SQRL2;
    bool csr = false;
    uint64_t n = 0, d = 0;
    uint32_t k = 0;
    uint32_t round = 0;
    const float *X = nullptr;
    const float *vals = nullptr;
    const uint32_t *idx = nullptr;
    const uint64_t *indptr = nullptr;
    const double *rowsum = nullptr;
    const double *w = nullptr;
    double prior = 0.0, prior_sum = 0.0;
    float *cbuf = nullptr;        // densified current center row [d]
    double *dist = nullptr;       // [n]
    uint32_t *asn = nullptr;      // [n]
    uint32_t *center_ids = nullptr;  // [k]
    uint64_t *newc = nullptr;     // device scalar
    float *ct = nullptr;          // CSR O(nnz) path: transformed center row [d]
    double *cconst = nullptr;     // CSR O(nnz) path: center constants [2] (JSD: [ngrp])
    const uint32_t *grp = nullptr;  // CSR JSD: per-row group of equal rinc
    const float *gval = nullptr;    // CSR JSD: rinc of each group
    uint32_t ngrp = 0;
    // dense SQRL2 pruning (rounds after the first): lower bounds of the distance from the new
    // center to each earlier center, and the relative error bound of an FP32 row distance
    const double *cgap = nullptr;
    double prune_g = 0.0;
};

int run_kmeanspp(const KmppArgs &a, const double *u_dev, double *chunk_tmp, int sms, cudaStream_t st);
// distances of every row to row *cand (see mc_kmpp.cu)
int kmpp_distances_to(const KmppArgs &a, const uint64_t *cand, double *out, int sms, cudaStream_t st);
// n_local_trials = L > 1: greedy seeding with uniforms U(seed, r) (see mc_kmpp.cu)
int run_kmeanspp_greedy(const KmppArgs &a, uint32_t L, uint64_t seed, double *chunk_tmp, int sms, cudaStream_t st);

// CSR seeding takes the O(nnz)-per-row update (per-center FP64 constants, a.ct / a.cconst)
// for wide rows, and for large sparse matrices: each round then pays a few microseconds of
// dependent FP64 sums for the constants (about 75 ns per dependent add on this GPU), which
// the float column loop of k_kmpp_csr, O(d) per row (two logf per column for MKL), undercuts
// only while the whole column loop is small (n d < 2^25: tens of microseconds of logf per
// round, about the constants' latency) or the rows are not sparse (more than one nonzero in
// eight columns)
inline bool kmpp_csr_nnz_path(uint64_t n, uint64_t d, uint64_t nnz) {
    if (d > 2048) return true;
    return n * d >= (uint64_t(1) << 25) && nnz * 8 <= n * d;
}

// C[c] = row ids[c], c < k (CSR rows densified into d columns)
int launch_gather_rows(bool csr, const float *X, const float *vals, const uint32_t *idx, const uint64_t *indptr,
                       uint64_t d, const uint32_t *ids, uint32_t k, float *C, cudaStream_t st);

}  // namespace mc
