// Coreset sampler launchers (mc_coreset.cu).
#pragma once
#include "mc_internal.cuh"
#include "mc_reduce.cuh"

namespace mc {

struct ScanWork {
    DBuf<double> run_off, chunk_tot, chunk_off;
};

struct SensInput {
    int method = MC_BFL;
    uint64_t n = 0;
    uint32_t nc = 0;
    uint64_t k = 0;
    double alpha_est = 0.0;
    const double *cost = nullptr;   // device, n
    const double *wt = nullptr;     // device, n (float weights widened) or null
    const uint32_t *asn = nullptr;  // device, n
    float *probs = nullptr;         // device, n
};

struct SensWork {
    DBuf<double> vals, s, cnt, wsum, csum, scal, det_tmp;
    DBuf<int> flag;
    SortWork sort;
};

struct AliasWork {
    DBuf<double> tmp, S, dl, eh, D, E;
    DBuf<uint64_t> flag, pos;
    DBuf<uint32_t> L, H;
    ScanWork scan;
};

struct SampleArgs {
    uint64_t np = 0, m = 0, direct = 0, seed = 0;
    int unique = 0;
    const float *probs = nullptr;
    const double *prob_tab = nullptr;
    const uint32_t *alias_tab = nullptr;
    const float *wf = nullptr;
    float *w_out = nullptr;
    uint64_t *idx_out = nullptr;
};

struct SampleWork {
    DBuf<uint64_t> draws, flag, pos, nzflag, nzpos, stop;
    DBuf<unsigned long long> first;
    DBuf<uint32_t> cnt;
};

int canon_exclusive_scan(const double *v, uint64_t m, double *P, ScanWork &w, cudaStream_t st);
int compute_sensitivities(const SensInput &in, SensWork &w, cudaStream_t st, int sms);
int build_alias(const float *probs, uint64_t n, double *prob_tab, uint32_t *alias_tab, AliasWork &w, cudaStream_t st,
                int sms);
int run_sample(const SampleArgs &a, SampleWork &w, cudaStream_t st, int sms);
int launch_to_double(const float *x, uint64_t n, double *y, cudaStream_t st);

}  // namespace mc
