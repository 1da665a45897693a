// CoresetSampler on the device (include/minicore/coreset/coreset.h:340-699).
//
//  * per-cluster sums (weight, cost, count) in FP64 over each cluster's points in ascending
//    index order, chunks of 256 points (stable counting sort from mc_reduce.cu);
//  * per-point sensitivities for BFL, FL, LFKF, VX, LBK in FP64, probabilities stored as
//    float (CoresetSampler<float,...>::probs_);
//  * alias table in closed form from canonical FP64 prefix sums (every entry independent);
//  * draws: bucket from U(seed, 2t), coin from U(seed, 2t+1); unique mode keeps drawing
//    until the requested number of distinct indices was seen (coreset.h:636-672).
#include "mc_coreset.cuh"
#include "mc_reduce.cuh"

namespace mc {

// ------------------------------------------------------------------------------------
// canonical FP64 exclusive scan: chunk 8192 = 256 runs of 32 contiguous elements
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_scan_runs(const double *__restrict__ v, uint64_t m, double *run_off,
                                                   double *chunk_tot) {
    __shared__ double runs[256];
    const uint64_t g = blockIdx.x;
    const int t = threadIdx.x;
    const uint64_t b = g * kDetChunk + uint64_t(t) * kDetPer;
    double loc = 0.0;
    for (uint64_t e = b; e < umin64(m, b + kDetPer); ++e) loc = loc + v[e];
    runs[t] = loc;
    __syncthreads();
    if (t == 0) {
        double off = 0.0;
        for (int r = 0; r < 256; ++r) {
            run_off[g * 256 + r] = off;
            off = off + runs[r];
        }
        chunk_tot[g] = off;
    }
}

__global__ void k_scan_chunks(const double *chunk_tot, uint64_t G, double *chunk_off) {
    double off = 0.0;
    for (uint64_t g = 0; g < G; ++g) {
        chunk_off[g] = off;
        off = off + chunk_tot[g];
    }
    chunk_off[G] = off;
}

__global__ void __launch_bounds__(256) k_scan_write(const double *__restrict__ v, uint64_t m,
                                                    const double *__restrict__ run_off,
                                                    const double *__restrict__ chunk_off, double *P) {
    const uint64_t g = blockIdx.x;
    const int t = threadIdx.x;
    const uint64_t b = g * kDetChunk + uint64_t(t) * kDetPer;
    const double base = chunk_off[g] + run_off[g * 256 + t];
    double loc = 0.0;
    for (uint64_t e = b; e < umin64(m, b + kDetPer); ++e) {
        P[e] = base + loc;
        loc = loc + v[e];
    }
    if (g == 0 && t == 0) P[m] = chunk_off[gridDim.x];
}

int canon_exclusive_scan(const double *v, uint64_t m, double *P, ScanWork &w, cudaStream_t st) {
    const uint64_t G = det_chunks(m);
    if (G == 0) {
        MC_CUDA_TRY(cudaMemsetAsync(P, 0, sizeof(double), st));
        return MC_OK;
    }
    MC_TRY(w.run_off.alloc(G * 256, st));
    MC_TRY(w.chunk_tot.alloc(G, st));
    MC_TRY(w.chunk_off.alloc(G + 1, st));
    k_scan_runs<<<unsigned(G), 256, 0, st>>>(v, m, w.run_off.p, w.chunk_tot.p), note_launch();
    k_scan_chunks<<<1, 1, 0, st>>>(w.chunk_tot.p, G, w.chunk_off.p), note_launch();
    k_scan_write<<<unsigned(G), 256, 0, st>>>(v, m, w.run_off.p, w.chunk_off.p, P), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------
__global__ void k_to_double_f32(const float *x, uint64_t n, double *y) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        y[i] = double(x[i]);
}

int launch_to_double(const float *x, uint64_t n, double *y, cudaStream_t st) {
    if (n == 0) return MC_OK;
    k_to_double_f32<<<unsigned(umin64((n + 255) / 256, 65535)), 256, 0, st>>>(x, n, y), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

__global__ void k_check_asn(const uint32_t *asn, uint64_t n, uint64_t nc, int *bad) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        if (asn[i] >= nc) atomicExch(bad, 1);
}

// per-point values: kind 0 -> 1, 1 -> wt, 2 -> wt*cost, 3 -> wt*cost*cost
__global__ void k_point_vals(const double *cost, const double *wt, uint64_t n, int kind, double *out) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        const double w = wt ? wt[i] : 1.0;
        double v;
        if (kind == 0) v = 1.0;
        else if (kind == 1) v = w;
        else if (kind == 2) v = w * cost[i];
        else v = (w * cost[i]) * cost[i];
        out[i] = v;
    }
}

// cluster sums: one thread per chunk of 256 points (sequential), then per cluster over chunks
__global__ void k_cluster_partials(const double *__restrict__ vals, const uint32_t *__restrict__ perm,
                                   const uint64_t *__restrict__ bucket_start, const uint64_t *__restrict__ bucket_count,
                                   const uint64_t *__restrict__ chunk_start, uint32_t k, double *partial) {
    const uint64_t q = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (q >= chunk_start[k]) return;
    uint32_t lo = 0, hi = k;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (chunk_start[mid] <= q) lo = mid; else hi = mid;
    }
    const uint32_t c = lo;
    const uint64_t r0 = (q - chunk_start[c]) * 256, r1 = umin64(bucket_count[c], r0 + 256);
    const uint32_t *rows = perm + bucket_start[c];
    double p = 0.0;
    for (uint64_t r = r0; r < r1; ++r) p = p + vals[rows[r]];
    partial[q] = p;
}

__global__ void k_cluster_final(const double *partial, const uint64_t *chunk_start, uint32_t k, double *out) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    const uint64_t q0 = chunk_start[c], q1 = chunk_start[c + 1];
    double s = 0.0;
    if (q1 > q0) {
        s = partial[q0];
        for (uint64_t q = q0 + 1; q < q1; ++q) s = s + partial[q];
    }
    out[c] = s;
}

__global__ void k_chunks256(const uint64_t *bucket_count, uint32_t k, uint64_t *chunk_count) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < k) chunk_count[c] = (bucket_count[c] + 255) / 256;
}

// sensitivities
struct SensArgs {
    int method;
    uint64_t n;
    uint32_t nc;
    const double *cost, *wt;
    const uint32_t *asn;
    const double *cnt, *wsum, *csum;
    const double *total;   // device scalar: total (w * cost) or (w * cost^2) for LFKF
    double alpha, alpha_est;
    const double *W;       // LBK: sum of weight sums (device scalar)
    double *s;
    float *probs;          // FL writes probs directly
};

__global__ void k_lbk_W(const double *wsum, uint32_t nc, double *W) {
    double s = 0.0;
    for (uint32_t c = 0; c < nc; ++c) s = s + wsum[c];
    *W = s;
}

__global__ void k_sens(SensArgs a) {
    const double total = *a.total;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < a.n; i += gridDim.x * uint64_t(blockDim.x)) {
        const double w = a.wt ? a.wt[i] : 1.0;
        const double c = a.cost[i];
        const uint32_t g = a.asn[i];
        switch (a.method) {
            case MC_BFL: {
                const double fraccost = w * c / total;
                const double fracw = w / (a.wsum[g] * a.cnt[g]);
                a.s[i] = 0.5 * (fraccost + fracw);
                break;
            }
            case MC_FL: {
                const double inv = 1.0 / total;
                if (a.wt) a.probs[i] = float(w * c * inv);
                else a.probs[i] = float(ceil(double(a.n) * inv * c) + 1.0);
                break;
            }
            case MC_LFKF:
                a.s[i] = a.alpha_est * w * (c * c + a.csum[g] / a.wsum[g]) + 2.0 * total / a.wsum[g];
                break;
            case MC_VX:
                a.s[i] = w * c / total + 1.0 / a.cnt[g];
                break;
            default: {  // LBK
                const double W = *a.W;
                const double avg = total / W;
                const double tcinv = a.alpha / avg;
                const double adj = (2.0 * a.alpha) * a.csum[g] / (a.wsum[g] * avg) + 4.0 * W / a.wsum[g];
                a.s[i] = tcinv * c + adj;
            }
        }
    }
}

__global__ void k_normalize(const double *s, uint64_t n, const double *tot, float *probs) {
    const double inv = 1.0 / *tot;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        probs[i] = float(s[i] * inv);
}

static unsigned grid_for(uint64_t n, int sms) { return unsigned(umin64((n + 255) / 256, uint64_t(sms) * 32)) + 1; }

int compute_sensitivities(const SensInput &in, SensWork &w, cudaStream_t st, int sms) {
    const uint64_t n = in.n;
    const uint32_t nc = in.nc;
    MC_TRY(w.vals.alloc(n, st));
    MC_TRY(w.s.alloc(n, st));
    MC_TRY(w.cnt.alloc(nc, st));
    MC_TRY(w.wsum.alloc(nc, st));
    MC_TRY(w.csum.alloc(nc, st));
    MC_TRY(w.scal.alloc(4, st));
    MC_TRY(w.det_tmp.alloc(det_tmp_size(n), st));
    MC_TRY(w.flag.alloc(1, st));
    MC_CUDA_TRY(cudaMemsetAsync(w.flag.p, 0, sizeof(int), st));
    k_check_asn<<<grid_for(n, sms), 256, 0, st>>>(in.asn, n, nc, w.flag.p), note_launch();
    int bad = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(&bad, w.flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    if (bad) return fail(MC_EINVAL, "assignment out of range [0, ncenters)");
    // stable grouping of points by cluster
    MC_TRY(launch_sort_by_key(in.asn, nullptr, n, nc, w.sort, st));
    MC_TRY(w.sort.chunk_count.alloc(nc, st));
    MC_TRY(w.sort.chunk_start.alloc(uint64_t(nc) + 1, st));
    k_chunks256<<<(nc + 255) / 256, 256, 0, st>>>(w.sort.bucket_count.p, nc, w.sort.chunk_count.p), note_launch();
    MC_TRY(launch_exclusive_scan_u64(w.sort.chunk_count.p, w.sort.chunk_start.p, nc, st));
    const uint64_t maxq = (n + 255) / 256 + nc;
    MC_TRY(w.sort.partial.alloc(maxq, st));
    auto cluster_sum = [&](int kind, double *out) -> int {
        k_point_vals<<<grid_for(n, sms), 256, 0, st>>>(in.cost, in.wt, n, kind, w.vals.p), note_launch();
        k_cluster_partials<<<unsigned((maxq + 255) / 256), 256, 0, st>>>(w.vals.p, w.sort.perm.p, w.sort.bucket_start.p,
                                                                        w.sort.bucket_count.p, w.sort.chunk_start.p, nc,
                                                                        w.sort.partial.p), note_launch();
        k_cluster_final<<<(nc + 255) / 256, 256, 0, st>>>(w.sort.partial.p, w.sort.chunk_start.p, nc, out), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    };
    MC_TRY(cluster_sum(0, w.cnt.p));
    MC_TRY(cluster_sum(1, w.wsum.p));
    const int tkind = in.method == MC_LFKF ? 3 : 2;
    if (in.method == MC_LBK || in.method == MC_LFKF) MC_TRY(cluster_sum(tkind, w.csum.p));
    // total (w*cost, or w*cost^2 for LFKF) in the canonical det order
    k_point_vals<<<grid_for(n, sms), 256, 0, st>>>(in.cost, in.wt, n, tkind, w.vals.p), note_launch();
    DetInput di{DET_F64, w.vals.p, nullptr, nullptr, n};
    MC_TRY(launch_det_sum(di, w.det_tmp.p, w.scal.p + 0, st));
    if (in.method == MC_LBK) k_lbk_W<<<1, 1, 0, st>>>(w.wsum.p, nc, w.scal.p + 1), note_launch();
    SensArgs sa;
    sa.method = in.method;
    sa.n = n;
    sa.nc = nc;
    sa.cost = in.cost;
    sa.wt = in.wt;
    sa.asn = in.asn;
    sa.cnt = w.cnt.p;
    sa.wsum = w.wsum.p;
    sa.csum = w.csum.p;
    sa.total = w.scal.p + 0;
    sa.alpha = 16.0 * log(double(in.k)) + 32.0;
    sa.alpha_est = in.alpha_est;
    sa.W = w.scal.p + 1;
    sa.s = w.s.p;
    sa.probs = in.probs;
    k_sens<<<grid_for(n, sms), 256, 0, st>>>(sa), note_launch();
    if (in.method != MC_FL) {
        DetInput ds{DET_F64, w.s.p, nullptr, nullptr, n};
        MC_TRY(launch_det_sum(ds, w.det_tmp.p, w.scal.p + 2, st));
        k_normalize<<<grid_for(n, sms), 256, 0, st>>>(w.s.p, n, w.scal.p + 2, in.probs), note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// alias table
// ------------------------------------------------------------------------------------
__global__ void k_alias_flags(const float *probs, uint64_t n, const double *S, uint64_t *light_flag) {
    const double scale = double(n) / *S;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        light_flag[i] = (double(probs[i]) * scale < 1.0) ? 1 : 0;
}

__global__ void k_alias_lists(const float *probs, uint64_t n, const double *S, const uint64_t *light_pos,
                              uint32_t *L, uint32_t *H, double *dl, double *eh) {
    const double scale = double(n) / *S;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        const double q = double(probs[i]) * scale;
        const uint64_t lp = light_pos[i];
        if (q < 1.0) {
            L[lp] = uint32_t(i);
            dl[lp] = 1.0 - q;
        } else {
            const uint64_t hp = i - lp;
            H[hp] = uint32_t(i);
            eh[hp] = q - 1.0;
        }
    }
}

__global__ void k_alias_light(const float *probs, uint64_t n, const double *S, const uint32_t *L, uint64_t nl,
                              const uint32_t *H, uint64_t nh, const double *D, const double *E, double *prob_tab,
                              uint32_t *alias_tab) {
    const double scale = double(n) / *S;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < nl; i += gridDim.x * uint64_t(blockDim.x)) {
        const double Di = D[i];
        uint64_t lo = 0, hi = nh;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (E[mid + 1] >= Di) hi = mid; else lo = mid + 1;
        }
        const uint64_t j = lo < nh ? lo : nh - 1;
        const uint32_t li = L[i];
        prob_tab[li] = double(probs[li]) * scale;
        alias_tab[li] = H[j];
    }
}

__global__ void k_alias_heavy(const uint32_t *H, uint64_t nh, uint64_t nl, const double *D, const double *E,
                              double *prob_tab, uint32_t *alias_tab) {
    for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < nh; j += gridDim.x * uint64_t(blockDim.x)) {
        uint64_t i = nl;
        if (j + 1 < nh) {
            const double Ej = E[j + 1];
            uint64_t lo = 0, hi = nl;
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (D[mid + 1] > Ej) hi = mid; else lo = mid + 1;
            }
            i = lo;
        }
        const uint32_t hj = H[j];
        if (i < nl) {
            prob_tab[hj] = 1.0 - (D[i + 1] - E[j + 1]);
            alias_tab[hj] = H[j + 1];
        } else {
            prob_tab[hj] = 1.0;
            alias_tab[hj] = hj;
        }
    }
}

__global__ void k_alias_identity(uint64_t n, double *prob_tab, uint32_t *alias_tab) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        prob_tab[i] = 1.0;
        alias_tab[i] = uint32_t(i);
    }
}

int build_alias(const float *probs, uint64_t n, double *prob_tab, uint32_t *alias_tab, AliasWork &w, cudaStream_t st,
                int sms) {
    MC_TRY(w.tmp.alloc(det_tmp_size(n), st));
    MC_TRY(w.S.alloc(1, st));
    MC_TRY(w.flag.alloc(n, st));
    MC_TRY(w.pos.alloc(n + 1, st));
    MC_TRY(w.L.alloc(n, st));
    MC_TRY(w.H.alloc(n, st));
    MC_TRY(w.dl.alloc(n, st));
    MC_TRY(w.eh.alloc(n, st));
    MC_TRY(w.D.alloc(n + 1, st));
    MC_TRY(w.E.alloc(n + 1, st));
    DetInput di{DET_F32, nullptr, probs, nullptr, n};
    MC_TRY(launch_det_sum(di, w.tmp.p, w.S.p, st));
    double S = 0.0;
    MC_CUDA_TRY(cudaMemcpyAsync(&S, w.S.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    if (!(S > 0.0)) return fail(MC_EINVAL, "sampling probabilities sum to a non-positive value");
    k_alias_flags<<<grid_for(n, sms), 256, 0, st>>>(probs, n, w.S.p, w.flag.p), note_launch();
    MC_TRY(launch_exclusive_scan_u64(w.flag.p, w.pos.p, n, st));
    uint64_t nl = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(&nl, w.pos.p + n, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    const uint64_t nh = n - nl;
    if (nh == 0) {
        k_alias_identity<<<grid_for(n, sms), 256, 0, st>>>(n, prob_tab, alias_tab), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    }
    k_alias_lists<<<grid_for(n, sms), 256, 0, st>>>(probs, n, w.S.p, w.pos.p, w.L.p, w.H.p, w.dl.p, w.eh.p), note_launch();
    MC_TRY(canon_exclusive_scan(w.dl.p, nl, w.D.p, w.scan, st));
    MC_TRY(canon_exclusive_scan(w.eh.p, nh, w.E.p, w.scan, st));
    if (nl) k_alias_light<<<grid_for(nl, sms), 256, 0, st>>>(probs, n, w.S.p, w.L.p, nl, w.H.p, nh, w.D.p, w.E.p,
                                                             prob_tab, alias_tab), note_launch();
    k_alias_heavy<<<grid_for(nh, sms), 256, 0, st>>>(w.H.p, nh, nl, w.D.p, w.E.p, prob_tab, alias_tab), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// sampling
// ------------------------------------------------------------------------------------
__device__ inline uint64_t alias_draw(uint64_t np, const double *prob_tab, const uint32_t *alias_tab, uint64_t seed,
                                      uint64_t s) {
    const double u1 = uniform_at(seed, 2 * s), u2 = uniform_at(seed, 2 * s + 1);
    uint64_t i = uint64_t(u1 * double(np));
    if (i >= np) i = np - 1;
    return (u2 < prob_tab[i]) ? i : alias_tab[i];
}

__global__ void k_sample_plain(SampleArgs a) {
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < a.m; s += gridDim.x * uint64_t(blockDim.x)) {
        if (s < a.direct) {
            const uint64_t ind = alias_draw(a.np, a.prob_tab, a.alias_tab, a.seed, s);
            const double w = a.wf ? double(a.wf[ind]) : 1.0;
            a.idx_out[s] = ind;
            a.w_out[s] = float(w / (double(a.m) * double(a.probs[ind])));
        } else {
            a.idx_out[s] = 0;
            a.w_out[s] = 0.f;
        }
    }
}

__global__ void k_sample_draws(SampleArgs a, uint64_t B, uint64_t *draws, unsigned long long *first) {
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < B; s += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t ind = alias_draw(a.np, a.prob_tab, a.alias_tab, a.seed, s);
        draws[s] = ind;
        atomicMin(&first[ind], (unsigned long long)s);
    }
}

__global__ void k_first_flags(const uint64_t *draws, uint64_t B, const unsigned long long *first, uint64_t *flag) {
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < B; s += gridDim.x * uint64_t(blockDim.x))
        flag[s] = (first[draws[s]] == s) ? 1 : 0;
}

// the draw at which the target-th distinct index appears
__global__ void k_find_stop(const uint64_t *flag, const uint64_t *pos, uint64_t B, uint64_t target, uint64_t *stop) {
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < B; s += gridDim.x * uint64_t(blockDim.x))
        if (flag[s] && pos[s] == target - 1) *stop = s;
}

__global__ void k_count_draws(const uint64_t *draws, const uint64_t *stop, uint32_t *cnt) {
    const uint64_t last = *stop;
    for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s <= last; s += gridDim.x * uint64_t(blockDim.x))
        atomicAdd(&cnt[draws[s]], 1u);
}

__global__ void k_nonzero_flags(const uint32_t *cnt, uint64_t np, uint64_t *flag) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < np; i += gridDim.x * uint64_t(blockDim.x))
        flag[i] = cnt[i] ? 1 : 0;
}

__global__ void k_unique_write(SampleArgs a, const uint32_t *cnt, const uint64_t *pos) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < a.np; i += gridDim.x * uint64_t(blockDim.x)) {
        const uint32_t c = cnt[i];
        if (!c) continue;
        const uint64_t o = pos[i];
        if (o >= a.m) continue;
        const float w = a.wf ? a.wf[i] : 1.f;
        a.idx_out[o] = i;
        a.w_out[o] = float(c) * (w / (float(a.m) * a.probs[i]));
    }
}

int run_sample(const SampleArgs &a, SampleWork &w, cudaStream_t st, int sms) {
    if (!a.unique) {
        k_sample_plain<<<grid_for(a.m, sms), 256, 0, st>>>(a), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    }
    MC_CUDA_TRY(cudaMemsetAsync(a.idx_out, 0, a.m * sizeof(uint64_t), st));
    MC_CUDA_TRY(cudaMemsetAsync(a.w_out, 0, a.m * sizeof(float), st));
    if (a.direct == 0) return MC_OK;
    uint64_t B = a.direct * 2 + 1024;
    const uint64_t Bmax = a.direct * 4096 + 64 * a.np + (1ull << 20);
    MC_TRY(w.first.alloc(a.np, st));
    MC_TRY(w.cnt.alloc(a.np, st));
    MC_TRY(w.nzflag.alloc(a.np, st));
    MC_TRY(w.nzpos.alloc(a.np + 1, st));
    MC_TRY(w.stop.alloc(1, st));
    for (;;) {
        MC_TRY(w.draws.alloc(B, st));
        MC_TRY(w.flag.alloc(B, st));
        MC_TRY(w.pos.alloc(B + 1, st));
        MC_CUDA_TRY(cudaMemsetAsync(w.first.p, 0xff, a.np * sizeof(unsigned long long), st));
        k_sample_draws<<<grid_for(B, sms), 256, 0, st>>>(a, B, w.draws.p, w.first.p), note_launch();
        k_first_flags<<<grid_for(B, sms), 256, 0, st>>>(w.draws.p, B, w.first.p, w.flag.p), note_launch();
        MC_TRY(launch_exclusive_scan_u64(w.flag.p, w.pos.p, B, st));
        uint64_t distinct = 0;
        MC_CUDA_TRY(cudaMemcpyAsync(&distinct, w.pos.p + B, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        MC_CUDA_TRY(cudaStreamSynchronize(st));
        if (distinct >= a.direct) break;
        if (B >= Bmax)
            return fail(MC_EINVAL, "unique sampling: fewer points with positive probability than requested");
        B = B * 4 < Bmax ? B * 4 : Bmax;
    }
    MC_CUDA_TRY(cudaMemsetAsync(w.stop.p, 0, sizeof(uint64_t), st));
    k_find_stop<<<grid_for(B, sms), 256, 0, st>>>(w.flag.p, w.pos.p, B, a.direct, w.stop.p), note_launch();
    MC_CUDA_TRY(cudaMemsetAsync(w.cnt.p, 0, a.np * sizeof(uint32_t), st));
    k_count_draws<<<grid_for(B, sms), 256, 0, st>>>(w.draws.p, w.stop.p, w.cnt.p), note_launch();
    k_nonzero_flags<<<grid_for(a.np, sms), 256, 0, st>>>(w.cnt.p, a.np, w.nzflag.p), note_launch();
    MC_TRY(launch_exclusive_scan_u64(w.nzflag.p, w.nzpos.p, a.np, st));
    k_unique_write<<<grid_for(a.np, sms), 256, 0, st>>>(a, w.cnt.p, w.nzpos.p), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

}  // namespace mc
