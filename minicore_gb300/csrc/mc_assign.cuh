// Assignment kernel arguments and launchers (mc_assign.cu).
#pragma once
#include "mc_internal.cuh"

namespace mc {

struct AssignArgs {
    int msr = SQRL2;
    uint64_t n = 0, d = 0;
    uint32_t k = 0, kp = 0;           // centers, padded center count of CT0/CT1
    const float *X = nullptr;         // dense rows
    const uint32_t *rows = nullptr;   // dense only: optional row list (row r of the pass = X row rows[r])
    const unsigned long long *n_dev = nullptr;  // tiled kernel: row count read on the device (<= n)
    const float *vals = nullptr;      // CSR rows
    const uint32_t *idx = nullptr;
    const uint64_t *indptr = nullptr;
    uint64_t nnz = 0;                 // CSR nonzeros (autotuner shape bucket)
    const double *rowsum = nullptr;   // per row (pair mode, sparse HELL)
    const float *rsi = nullptr;       // per-row 1/rhsum (constant prior)
    const float *rinc = nullptr;      // per-row pv/rhsum (constant prior)
    const double *csum = nullptr;     // per-center sums
    float *CT0 = nullptr;             // [d][kp] center transform
    float *CT1 = nullptr;             // [d][kp] second center transform (MKL, JSD)
    double *consts = nullptr;         // [k][4] per-center FP64 constants (sparse-dot path)
    const uint32_t *grp = nullptr;    // JSD sparse-dot: per-row group of rows with equal rinc
    const double *ztab = nullptr;     // JSD sparse-dot: [group][k] zero-entry sums (k_jsd_ztable)
    float pv = 0.f;                   // constant-prior pv
    double prior = 0.0, prior_sum = 0.0;
    uint32_t *asn = nullptr;
    double *costs = nullptr;
    // optional distance output (cmp / pcmp): every pair's distance as float
    //   dmode 1: dmat[row * ldm + c]   2: dmat[c * ldm + row]
    //   dmode 3: condensed upper triangle, pairs c < row at c*ldm - c(c+1)/2 + row - c - 1
    float *dmat = nullptr;
    uint64_t ldm = 0;
    int dmode = 0;
};

__device__ __forceinline__ void write_dist(const AssignArgs &a, uint64_t row, uint32_t c, float v) {
    if (a.dmode == 1) {
        a.dmat[row * a.ldm + c] = v;
    } else if (a.dmode == 2) {
        a.dmat[uint64_t(c) * a.ldm + row] = v;
    } else if (a.dmode == 3 && uint64_t(c) < row) {
        const uint64_t cc = c;
        a.dmat[cc * a.ldm - cc * (cc + 1) / 2 + row - cc - 1] = v;
    }
}

int launch_prep_centers(const AssignArgs &a, const float *C, bool pair, bool sparse_consts, cudaStream_t st);
int launch_row_scalars(const double *rowsum, uint64_t n, uint64_t d, float pv, float *rsi, float *rinc,
                       cudaStream_t st);
// tune: the autotuner may time kernel variants on the first call for a shape (callers that
// must not synchronise or allocate pass false)
int launch_assign_tiled(const AssignArgs &a, bool csr, bool pair, cudaStream_t st, bool tune = true);
int launch_assign_sparse(const AssignArgs &a, cudaStream_t st, int sms, bool tune = true);
// L1 over CSR rows in pair mode (prior 0): a walk over the union of nonzero columns,
// bit-identical to the tiled kernel; work: l1_union_work_entries(k, d) floats
int launch_assign_l1_union(const AssignArgs &a, const float *C, float *work, int sms, cudaStream_t st,
                           bool tune = true);
uint64_t l1_union_work_entries(uint32_t k, uint64_t d);
// the largest work space (in entries) for which the union kernel is used
constexpr uint64_t kL1UnionMaxEntries = 1ull << 29;
// JSD sparse-dot table: ztab[g * k + c] = sum over all columns j of f(a_cj, gval[g]) with
// f(a, b) = a log a + b log b - (a + b) log((a + b) / 2) and a_cj the center transform
int launch_jsd_ztable(const float *C, uint32_t k, uint64_t d, const double *csum, float pv, const float *gval,
                      uint32_t ngrp, double *ztab, cudaStream_t st);
uint32_t tiled_center_pad(uint32_t k, bool pair, int msr);
uint32_t sparse_center_pad(uint32_t k);

}  // namespace mc
