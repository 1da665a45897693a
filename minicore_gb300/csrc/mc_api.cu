// C ABI of minicore_gb300 (include/minicore_gb300.h): context, device-resident jobs, the
// perform_hard_clustering loop (include/minicore/clustering/solve.h:98-175), kmeans++
// (include/minicore/optim/kmeans.h:49-215) and the coreset sampler
// (include/minicore/coreset/coreset.h:228-701).
#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <unordered_map>
#include <vector>

#include "mc_assign.cuh"
#include "mc_coreset.cuh"
#include "mc_internal.cuh"
#include "mc_kmpp.cuh"
#include "mc_reduce.cuh"
#include "mc_tc.cuh"

namespace mc {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};
static thread_local uint64_t t_launches = 0;  // this thread's share (graph captures count theirs)

void note_launch() {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ++t_launches;
}
static thread_local uint64_t t_allocs = 0;
void note_device_alloc() { ++t_allocs; }
uint64_t device_allocs() { return t_allocs; }

static std::atomic<bool> g_prof_on{false};
static std::mutex g_prof_mu;
struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
};
static std::vector<ProfRec> g_prof;

bool profiling_enabled() { return g_prof_on.load(std::memory_order_relaxed); }
void profile_record(const char *name, cudaEvent_t a, cudaEvent_t b) {
    std::lock_guard<std::mutex> lock(g_prof_mu);
    g_prof.push_back({name, a, b});
}

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

// Memory the current device's kernels may read and write directly: managed memory, or
// device memory of the current device.  Device memory of another GPU is not: a kernel
// launched here would fault on it without peer access and silently cross the link with it,
// so callers copy it like host memory (cudaMemcpyDefault moves it between GPUs).
bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (attr.type == cudaMemoryTypeManaged) return true;
    if (attr.type != cudaMemoryTypeDevice) return false;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.device == dev;
}

bool is_foreign_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice && attr.device != dev;
}

// copy `bytes` from src (host or device) into a device buffer unless src already lives on
// the device, in which case it is borrowed
template <class T>
static int stage(const T *src, size_t count, DBuf<T> &own, const T *&out, cudaStream_t st) {
    if (!src) {
        out = nullptr;
        return MC_OK;
    }
    if (is_device_ptr(src)) {
        out = src;
        return MC_OK;
    }
    MC_TRY(own.alloc(count, st));
    MC_CUDA_TRY(cudaMemcpyAsync(own.p, src, count * sizeof(T), cudaMemcpyDefault, st));
    out = own.p;
    return MC_OK;
}

template <class T>
static int copy_out(T *dst, const T *src, size_t count, cudaStream_t st) {
    if (!dst || count == 0) return MC_OK;
    MC_CUDA_TRY(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDefault, st));
    return MC_OK;
}

// CSR structure check (every kernel relies on it): indptr[0] == 0, nondecreasing,
// indptr[n] == nnz, column indices < d and strictly increasing within each row.
__global__ void k_validate_csr(const uint64_t *indptr, const uint32_t *idx, uint64_t n, uint64_t d, uint64_t nnz,
                               int *bad) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i == 0 && (indptr[0] != 0 || indptr[n] != nnz)) atomicExch(bad, 1);
    if (i >= n) return;
    const uint64_t b = indptr[i], e = indptr[i + 1];
    if (e < b || e > nnz) {
        atomicExch(bad, 2);
        return;
    }
    for (uint64_t p = b; p < e; ++p) {
        if (idx[p] >= d || (p > b && idx[p] <= idx[p - 1])) {
            atomicExch(bad, 3);
            return;
        }
    }
}

static int validate_csr(const uint64_t *indptr, const uint32_t *idx, uint64_t n, uint64_t d, uint64_t nnz,
                        cudaStream_t st) {
    DBuf<int> flag;
    MC_TRY(flag.alloc(1, st));
    MC_CUDA_TRY(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
    k_validate_csr<<<unsigned((n + 255) / 256), 256, 0, st>>>(indptr, idx, n, d, nnz, flag.p), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    int bad = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(&bad, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    if (bad == 1) return fail(MC_EINVAL, "CSR indptr must start at 0 and end at nnz");
    if (bad == 2) return fail(MC_EINVAL, "CSR indptr must be nondecreasing");
    if (bad == 3) return fail(MC_EINVAL, "CSR column indices must be < ncols and strictly increasing in each row");
    return MC_OK;
}

struct DevMatrix {
    int kind = MC_DENSE_F32;
    uint64_t n = 0, d = 0, nnz = 0;
    const float *X = nullptr, *vals = nullptr;
    const uint32_t *idx = nullptr;
    const uint64_t *indptr = nullptr;
    DBuf<float> X_own, vals_own;
    DBuf<uint32_t> idx_own;
    DBuf<uint64_t> indptr_own;

    int load(const mc_matrix *m, cudaStream_t st) {
        if (!m) return fail(MC_EINVAL, "matrix is null");
        kind = m->kind;
        n = m->nrows;
        d = m->ncols;
        if (n == 0 || d == 0) return fail(MC_EINVAL, "matrix has no rows or no columns");
        if (n >= (1ull << 32)) return fail(MC_EINVAL, "more than 2^32-1 rows");
        if (kind == MC_DENSE_F32) {
            if (!m->values) return fail(MC_EINVAL, "dense matrix without values");
            return stage(m->values, n * d, X_own, X, st);
        }
        if (kind != MC_CSR_F32) return fail(MC_EINVAL, "unknown matrix kind");
        if (!m->indptr) return fail(MC_EINVAL, "CSR matrix without indptr");
        nnz = m->nnz;
        if (nnz && (!m->values || !m->indices)) return fail(MC_EINVAL, "CSR matrix without values/indices");
        if (d >= (1ull << 32)) return fail(MC_EINVAL, "more than 2^32-1 columns");
        MC_TRY(stage(m->indptr, n + 1, indptr_own, indptr, st));
        MC_TRY(stage(m->values, nnz, vals_own, vals, st));
        MC_TRY(stage(m->indices, nnz, idx_own, idx, st));
        return validate_csr(indptr, idx, n, d, nnz, st);
    }
};

}  // namespace mc

using namespace mc;

struct mc_context {
    int device = 0;
    int sms = 152;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
};

struct mc_job {
    mc_context *ctx = nullptr;
    cudaStream_t st = nullptr;
    DevMatrix M;
    int msr = SQRL2;
    double prior = 0.0;
    int precision = MC_FP32;
    uint64_t seed = 0, restart_counter = 0;
    uint32_t k = 0, kp = 0;
    bool pair = false;
    bool sparse_path = false;
    float pv = 0.f;
    double psum = 0.0;
    DBuf<double> rowsum, w, costs, csum, consts, det_tmp, scal;
    DBuf<float> rownorm, rsi, rinc, C, Cw, CT0, CT1, cnorm;
    DBuf<float> costs32;  // mc_job_read_f32: the costs rounded to float on the device
    DBuf<uint32_t> asn, asn2;
    DBuf<int> flag;
    DBuf<uint64_t> idxbuf;
    // CSR JSD sparse-dot path: rows grouped by their zero-entry value rinc
    DBuf<uint32_t> grp;
    DBuf<float> gval;
    DBuf<double> ztab;
    uint32_t ngrp = 0;
    SortWork sort;
    L1CsrWork l1csr;  // L1 medians over CSR rows
    DBuf<float> clist;  // L1 pair-mode CSR assignment: per 32-center group, columns and values
    TcState tc;
    uint64_t last_recheck = 0;
    // Lloyd loop as one CUDA graph (mc_job_run); captured per run, and again after a host
    // iteration (which may have grown buffers the graph points at)
    cudaGraphExec_t loop_exec = nullptr;
    uint64_t loop_pre_launches = 0, loop_body_launches = 0;
    DBuf<unsigned char> loop_state;
    ~mc_job() {
        if (loop_exec) cudaGraphExecDestroy(loop_exec);
    }
};

struct mc_sampler {
    mc_context *ctx = nullptr;
    uint64_t np = 0, nc = 0, k = 0;
    int method = MC_BFL;
    DBuf<float> probs, wf;
    DBuf<double> prob_tab, cost_d, wt_d;
    DBuf<uint32_t> alias, asn;
    AliasWork aw;
    SensWork sw;
    SampleWork smp;
};

namespace {

int sync(cudaStream_t st) {
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    return MC_OK;
}

// CSR JSD with a constant prior: the zero entries of row i all take the value
// rinc_i = pv / (rowsum_i + pv d), so sum over all columns of f(a_cj, rinc_i) depends on the row
// only through rinc_i.  Rows with equal rinc (count data: equal row sums) form a group; one
// FP64 sum per (group, center) then leaves O(nnz) work per (row, center).  The grouping is
// kept only while the table (groups x d per center) costs at most half the nonzeros.
int build_rinc_groups(const double *rowsum, uint64_t n, uint64_t d, uint64_t nnz, float pv, cudaStream_t st,
                      DBuf<uint32_t> &grp, DBuf<float> &gval, uint32_t &ngrp) {
    ngrp = 0;
    if (n == 0 || !(pv > 0.f)) return MC_OK;
    DBuf<float> rsi, rinc;
    MC_TRY(rsi.alloc(n, st));
    MC_TRY(rinc.alloc(n, st));
    MC_TRY(launch_row_scalars(rowsum, n, d, pv, rsi.p, rinc.p, st));
    std::vector<float> h(n);
    MC_CUDA_TRY(cudaMemcpyAsync(h.data(), rinc.p, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    MC_TRY(sync(st));
    const uint64_t limit = std::max<uint64_t>(1, nnz / 2 / std::max<uint64_t>(d, 1));
    std::unordered_map<uint32_t, uint32_t> id;
    std::vector<uint32_t> g(n);
    std::vector<float> vals;
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t bits;
        std::memcpy(&bits, &h[i], 4);
        auto it = id.find(bits);
        if (it == id.end()) {
            if (vals.size() >= limit) return MC_OK;  // too many distinct values: no grouping
            it = id.emplace(bits, uint32_t(vals.size())).first;
            vals.push_back(h[i]);
        }
        g[i] = it->second;
    }
    MC_TRY(grp.alloc(n, st));
    MC_TRY(gval.alloc(vals.size(), st));
    MC_CUDA_TRY(cudaMemcpyAsync(grp.p, g.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    MC_CUDA_TRY(cudaMemcpyAsync(gval.p, vals.data(), vals.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    MC_TRY(sync(st));  // the host vectors go out of scope
    ngrp = uint32_t(vals.size());
    return MC_OK;
}

// optional distance output of an assignment pass (see AssignArgs::dmode)
struct DistOut {
    float *dmat = nullptr;
    uint64_t ldm = 0;
    int dmode = 0;
};

// the assignment pass with the centers in `C` (center sums / transforms refreshed here)
// graph_mode: no host round trip inside (for stream capture); the tensor-core path then
// leaves its bounded-wait status in j->tc.err for the caller
int job_assign_with(mc_job *j, const float *C, double prior_sum, bool force_exact, const DistOut *dout = nullptr,
                    bool graph_mode = false) {
    const uint64_t n = j->M.n, d = j->M.d;
    MC_TRY(launch_center_sums(C, j->k, d, j->csum.p, j->cnorm.p, j->st));
    const bool csr = j->M.kind == MC_CSR_F32;
    const bool tc = !csr && !force_exact && !dout && j->msr == SQRL2 && j->precision != MC_FP32;
    if (tc) {
        MC_TRY(tc_assign(j->tc, j->M.X, n, d, C, j->cnorm.p, j->k, j->precision, j->rownorm.p, j->asn.p,
                         j->costs.p, j->ctx->sms, j->st, &j->last_recheck, graph_mode));
        return MC_OK;
    }
    j->last_recheck = 0;
    AssignArgs a;
    a.msr = j->msr;
    a.n = n;
    a.d = d;
    a.k = j->k;
    a.X = j->M.X;
    a.vals = j->M.vals;
    a.idx = j->M.idx;
    a.indptr = j->M.indptr;
    a.nnz = j->M.nnz;
    a.rowsum = j->rowsum.p;
    a.rsi = j->rsi.p;
    a.rinc = j->rinc.p;
    a.csum = j->csum.p;
    a.pv = j->pv;
    a.prior = j->prior;
    a.prior_sum = prior_sum;
    a.asn = j->asn.p;
    a.costs = j->costs.p;
    if (dout) {
        a.dmat = dout->dmat;
        a.ldm = dout->ldm;
        a.dmode = dout->dmode;
    }
    if (csr && j->pair && j->msr == L1 && l1_union_work_entries(j->k, d) <= kL1UnionMaxEntries) {
        Phase ph("assign_csr_l1_union", j->st);
        MC_TRY(j->clist.alloc(l1_union_work_entries(j->k, d), j->st));
        return launch_assign_l1_union(a, C, j->clist.p, j->ctx->sms, j->st);
    }
    const bool sparse = csr && j->sparse_path;
    a.kp = sparse ? sparse_center_pad(j->k) : tiled_center_pad(j->k, j->pair, j->msr);
    MC_TRY(j->CT0.alloc(uint64_t(a.kp) * d, j->st));
    const bool ct1 = !sparse && !j->pair && (j->msr == MKL || j->msr == JSD);
    if (ct1) MC_TRY(j->CT1.alloc(uint64_t(a.kp) * d, j->st));
    a.CT0 = j->CT0.p;
    a.CT1 = ct1 ? j->CT1.p : nullptr;
    if (sparse) {
        MC_TRY(j->consts.alloc(uint64_t(j->k) * 4, j->st));
        a.consts = j->consts.p;
    }
    MC_TRY(launch_prep_centers(a, C, j->pair, sparse, j->st));
    if (sparse && j->msr == JSD) {
        MC_TRY(j->ztab.alloc(uint64_t(j->ngrp) * j->k, j->st));
        MC_TRY(launch_jsd_ztable(C, j->k, d, j->csum.p, j->pv, j->gval.p, j->ngrp, j->ztab.p, j->st));
        a.grp = j->grp.p;
        a.ztab = j->ztab.p;
    }
    if (sparse) {
        Phase ph("assign_csr_sparse", j->st);
        return launch_assign_sparse(a, j->st, j->ctx->sms);
    }
    Phase ph(csr ? "assign_csr_tiled" : "assign_dense_fp32", j->st);
    return launch_assign_tiled(a, csr, j->pair, j->st);
}

int job_cost(mc_job *j, float *out) {
    Phase ph("objective", j->st);
    DetInput in{j->w.p ? DET_F64_W : DET_F64, j->costs.p, nullptr, j->w.p, j->M.n};
    MC_TRY(launch_det_sum(in, j->det_tmp.p, j->scal.p, j->st));
    double s = 0.0;
    MC_CUDA_TRY(cudaMemcpyAsync(&s, j->scal.p, sizeof(double), cudaMemcpyDeviceToHost, j->st));
    MC_TRY(sync(j->st));
    *out = float(s);
    return MC_OK;
}

__global__ void k_copy_row_dense(const float *X, uint64_t d, const uint64_t *r, float *dst) {
    for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < d; j += gridDim.x * uint64_t(blockDim.x))
        dst[j] = X[*r * d + j];
}
__global__ void k_copy_row_csr_zero(uint64_t d, float *dst) {
    for (uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; j < d; j += gridDim.x * uint64_t(blockDim.x))
        dst[j] = 0.f;
}
__global__ void k_copy_row_csr(const float *vals, const uint32_t *idx, const uint64_t *indptr, const uint64_t *r,
                               float *dst) {
    for (uint64_t p = indptr[*r] + blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; p < indptr[*r + 1];
         p += gridDim.x * uint64_t(blockDim.x))
        dst[idx[p]] = vals[p];
}

// set_centroids_full_mean (centroid.h:649-779); returns 1 if a center was restarted
// weighted means of the buckets into Cw (presorted: the counting sort of asn is current);
// j->flag records a NaN center
int job_launch_centroids(mc_job *j, const uint32_t *keys2, uint64_t extra, bool presorted) {
    cudaStream_t st = j->st;
    Phase ph("centroid_update", st);
    CentroidArgs ca;
    ca.csr = j->M.kind == MC_CSR_F32;
    ca.n = j->M.n;
    ca.d = j->M.d;
    ca.k = j->k;
    ca.X = j->M.X;
    ca.vals = j->M.vals;
    ca.idx = j->M.idx;
    ca.indptr = j->M.indptr;
    ca.nnz = j->M.nnz;
    ca.keys = j->asn.p;
    ca.keys2 = keys2;
    ca.extra_members = extra;
    ca.w = j->w.p;
    ca.centers = j->Cw.p;
    ca.nan_flag = j->flag.p;
    MC_CUDA_TRY(cudaMemsetAsync(j->flag.p, 0, sizeof(int), st));
    return launch_centroids(ca, j->sort, st, presorted);
}

// L1: coordinate-wise medians (set_centroids_l1, clustering/centroid.h:203, 435-504) instead
// of means, over dense or CSR rows
bool l1_medians(const mc_job *j) { return j->msr == L1; }

// the medians of the current (sorted) assignment into Cw
int job_l1_medians(mc_job *j) {
    Phase ph("centroid_update", j->st);
    MC_CUDA_TRY(cudaMemsetAsync(j->flag.p, 0, sizeof(int), j->st));
    if (j->M.kind == MC_DENSE_F32)
        return launch_l1_medians(j->M.X, j->M.d, j->k, j->sort, j->w.p, j->Cw.p, j->st);
    // the reference's CSR median takes no weights (util/csc.h:835)
    if (j->w.p) return fail(MC_EUNSUPPORTED, "Not implemented: weighted L1 median for CSparseMatrix");
    return launch_l1_medians_csr(j->M.vals, j->M.idx, j->M.indptr, j->M.n, j->M.d, j->M.nnz, j->k, j->asn.p,
                                 j->sort, j->l1csr, j->Cw.p, j->st);
}

// set_centroids_l1: empty clusters are reseeded one at a time (D^2 draw over the current
// costs, then rows closer to the new center in plain L1 move to it), until none is empty;
// then the medians.  The reference reports no restart from this policy.
int job_set_centroids_l1(mc_job *j) {
    const uint64_t n = j->M.n, d = j->M.d;
    const uint32_t k = j->k;
    cudaStream_t st = j->st;
    std::vector<uint64_t> cnt(k);
    for (;;) {
        MC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), j->sort.bucket_count.p, k * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                    st));
        MC_TRY(sync(st));
        std::vector<uint32_t> empty;
        for (uint32_t c = 0; c < k; ++c)
            if (cnt[c] == 0) empty.push_back(c);
        if (empty.empty()) break;
        for (uint32_t id : empty) {
            const double u = uniform_at(j->seed, j->restart_counter++);
            DetInput in{DET_F64, j->costs.p, nullptr, nullptr, n};
            MC_TRY(launch_det_draw(in, j->det_tmp.p, nullptr, u, 0, nullptr, j->idxbuf.p + k, st));
            float *dst = j->Cw.p + uint64_t(id) * d;
            const unsigned gb = unsigned(umin64((d + 255) / 256, 1024));
            if (j->M.kind == MC_DENSE_F32) {
                k_copy_row_dense<<<gb, 256, 0, st>>>(j->M.X, d, j->idxbuf.p + k, dst), note_launch();
                MC_CUDA_TRY(cudaGetLastError());
                MC_TRY(launch_l1_reseed_update(j->M.X, n, d, dst, id, j->asn.p, j->costs.p, st));
            } else {
                k_copy_row_csr_zero<<<gb, 256, 0, st>>>(d, dst), note_launch();
                k_copy_row_csr<<<1, 256, 0, st>>>(j->M.vals, j->M.idx, j->M.indptr, j->idxbuf.p + k, dst),
                    note_launch();
                MC_CUDA_TRY(cudaGetLastError());
                MC_TRY(launch_l1_reseed_update_csr(j->M.vals, j->M.idx, j->M.indptr, n, j->idxbuf.p + k, id,
                                                   j->asn.p, j->costs.p, st));
            }
        }
        MC_TRY(launch_sort_by_key(j->asn.p, nullptr, n, k, j->sort, st));
    }
    return job_l1_medians(j);
}

int job_set_centroids(mc_job *j, int *restarted) {
    const uint64_t n = j->M.n, d = j->M.d;
    const uint32_t k = j->k;
    cudaStream_t st = j->st;
    *restarted = 0;
    MC_TRY(j->idxbuf.alloc(uint64_t(k) + 2, st));
    // the counting sort of the rows by cluster gives the bucket sizes; it is reused for the
    // centroid sums when no cluster is empty
    {
        Phase ph("centroid_update", st);
        MC_TRY(launch_sort_by_key(j->asn.p, nullptr, n, k, j->sort, st));
    }
    if (l1_medians(j)) return job_set_centroids_l1(j);
    std::vector<uint64_t> cnt(k);
    MC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), j->sort.bucket_count.p, k * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MC_TRY(sync(st));
    std::vector<uint32_t> empty;
    for (uint32_t c = 0; c < k; ++c)
        if (cnt[c] == 0) empty.push_back(c);
    const uint32_t *keys2 = nullptr;
    uint64_t extra = 0;
    if (!empty.empty()) {
        *restarted = 1;
        // D^2 draws over the current costs, one per empty center, all from the same costs
        std::vector<uint64_t> rsel;
        for (uint32_t id : empty) {
            const double u = uniform_at(j->seed, j->restart_counter++);
            DetInput in{DET_F64, j->costs.p, nullptr, nullptr, n};
            MC_TRY(launch_det_draw(in, j->det_tmp.p, nullptr, u, 0, nullptr, j->idxbuf.p + k, st));
            uint64_t r = 0;
            MC_CUDA_TRY(cudaMemcpyAsync(&r, j->idxbuf.p + k, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
            rsel.push_back(r);
            float *dst = j->Cw.p + uint64_t(id) * d;
            if (j->M.kind == MC_DENSE_F32) {
                k_copy_row_dense<<<unsigned(umin64((d + 255) / 256, 1024)), 256, 0, st>>>(j->M.X, d, j->idxbuf.p + k,
                                                                                          dst), note_launch();
            } else {
                k_copy_row_csr_zero<<<unsigned(umin64((d + 255) / 256, 1024)), 256, 0, st>>>(d, dst), note_launch();
                k_copy_row_csr<<<64, 256, 0, st>>>(j->M.vals, j->M.idx, j->M.indptr, j->idxbuf.p + k, dst), note_launch();
            }
            MC_CUDA_TRY(cudaGetLastError());
        }
        // full reassignment (the reference passes prior[0] as the prior sum here); the
        // tensor-core path returns the exact FP32 assignment, so it serves here too
        MC_TRY(job_assign_with(j, j->Cw.p, double(float(j->prior)), false));
        MC_TRY(j->asn2.alloc(n, st));
        MC_CUDA_TRY(cudaMemsetAsync(j->asn2.p, 0xff, n * sizeof(uint32_t), st));
        std::vector<uint32_t> cur(rsel.size());
        for (size_t e = 0; e < rsel.size(); ++e)
            MC_CUDA_TRY(cudaMemcpyAsync(&cur[e], j->asn.p + rsel[e], sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
        const double zero = 0.0;
        for (size_t e = 0; e < rsel.size(); ++e) {
            const uint64_t pid = rsel[e];
            const uint32_t cid = empty[e];
            uint32_t now = cur[e];
            for (size_t e2 = 0; e2 < e; ++e2)
                if (rsel[e2] == pid) now = empty[e2];
            if (now != cid) {
                // the row stays in its previous bucket too (centroid.h:743-751)
                MC_CUDA_TRY(cudaMemcpyAsync(j->asn2.p + pid, &now, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
                MC_CUDA_TRY(cudaMemcpyAsync(j->asn.p + pid, &cid, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
                MC_CUDA_TRY(cudaMemcpyAsync(j->costs.p + pid, &zero, sizeof(double), cudaMemcpyHostToDevice, st));
                MC_TRY(sync(st));
                ++extra;
            }
        }
        if (extra) keys2 = j->asn2.p;
    }
    MC_TRY(job_launch_centroids(j, keys2, extra, /*presorted=*/!*restarted));
    int nanf = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(&nanf, j->flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MC_TRY(sync(st));
    if (nanf) return fail(MC_ENAN, "Unexpected nan in ctr");
    return MC_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------------------------------
// Lloyd loop as one CUDA graph: [sort asn, check] -> while { centroids, assignment, objective,
// stop rule, commit, sort asn, check }.  The stop rule of the host loop runs on the device
// (k_loop_decide); the loop leaves the graph for the host only to finish (converged,
// maxiter, cost rose -> revert, NaN center, bounded wait expired) or when a cluster is empty
// (the D^2 restart of set_centroids_full_mean runs on the host, then the graph resumes).
// Each kernel and its order are those of the host loop, so the results are identical.
// ------------------------------------------------------------------------------------
enum : int { LOOP_RUN = 0, LOOP_DONE = 1, LOOP_REVERT = 2, LOOP_EMPTY = 3, LOOP_NAN = 4, LOOP_TIMEOUT = 5 };

struct LoopState {
    float cost;                  // objective of the committed centers C
    int reason;                  // LOOP_*
    unsigned long long iternum;  // committed updates
    unsigned long long maxiter;
    double eps;
    int commit;                  // the last decision copies Cw to C
    int pad;
};

// graph != 0: the kernel runs inside the loop graph and also sets its while-condition h
__global__ void k_loop_check_empty(const uint64_t *__restrict__ bucket_count, uint32_t k, LoopState *ls,
                                   cudaGraphConditionalHandle h, int graph) {
    __shared__ int any;
    if (ls->reason != LOOP_RUN) return;  // same value for the whole block
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < k; c += blockDim.x)
        if (bucket_count[c] == 0) any = 1;
    __syncthreads();
    if (threadIdx.x == 0 && any) {
        ls->reason = LOOP_EMPTY;
        if (graph) cudaGraphSetConditional(h, 0);
    }
}

// the stop rule of the host loop (perform_hard_clustering, clustering/solve.h:98-175)
__global__ void k_loop_decide(const double *__restrict__ cost_sum, const int *__restrict__ nan_flag,
                              const int *__restrict__ tc_err, LoopState *ls, cudaGraphConditionalHandle h,
                              int graph) {
    ls->commit = 0;
    if (*nan_flag) {
        ls->reason = LOOP_NAN;
        if (graph) cudaGraphSetConditional(h, 0);
        return;
    }
    if (tc_err && *tc_err) {
        ls->reason = LOOP_TIMEOUT;
        if (graph) cudaGraphSetConditional(h, 0);
        return;
    }
    const float newcost = float(*cost_sum);
    if (newcost > ls->cost) {
        ls->reason = LOOP_REVERT;
        if (graph) cudaGraphSetConditional(h, 0);
        return;
    }
    ls->commit = 1;
    ls->iternum += 1;
    const float oldcost = ls->cost;
    ls->cost = newcost;
    const double mx = double(newcost) < double(oldcost) ? double(oldcost) : double(newcost);
    if (double(oldcost - newcost) < ls->eps * mx || ls->iternum > ls->maxiter) {
        ls->reason = LOOP_DONE;
        if (graph) cudaGraphSetConditional(h, 0);
    } else {
        if (graph) cudaGraphSetConditional(h, 1);
    }
}

__global__ void k_loop_commit(const LoopState *__restrict__ ls, float *C, const float *__restrict__ Cw, uint64_t m) {
    if (!ls->commit) return;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < m; e += gridDim.x * uint64_t(blockDim.x))
        C[e] = Cw[e];
}

struct CaptureGuard {  // ends an unfinished capture on the error path
    cudaStream_t st;
    bool on = false;
    ~CaptureGuard() {
        if (on) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
        }
    }
};

// the loop's launch sequences (identical in the graph and in the fused host loop)
int job_loop_pre(mc_job *j, LoopState *ls, cudaGraphConditionalHandle h, int graph) {
    MC_TRY(launch_sort_by_key(j->asn.p, nullptr, j->M.n, j->k, j->sort, j->st));
    k_loop_check_empty<<<1, 256, 0, j->st>>>(j->sort.bucket_count.p, j->k, ls, h, graph), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// the centers of the current (sorted) assignment into Cw, no cluster empty
int job_update_centers(mc_job *j) {
    if (l1_medians(j)) return job_l1_medians(j);
    return job_launch_centroids(j, nullptr, 0, /*presorted=*/true);
}

int job_loop_body(mc_job *j, LoopState *ls, cudaGraphConditionalHandle h, int graph) {
    cudaStream_t st = j->st;
    const uint64_t n = j->M.n, d = j->M.d;
    const uint32_t k = j->k;
    const bool tc = j->M.kind == MC_DENSE_F32 && j->msr == SQRL2 && j->precision != MC_FP32;
    MC_TRY(job_update_centers(j));
    MC_TRY(job_assign_with(j, j->Cw.p, j->psum, false, nullptr, /*graph_mode=*/true));
    {
        DetInput in{j->w.p ? DET_F64_W : DET_F64, j->costs.p, nullptr, j->w.p, n};
        MC_TRY(launch_det_sum(in, j->det_tmp.p, j->scal.p, st));
    }
    k_loop_decide<<<1, 1, 0, st>>>(j->scal.p, j->flag.p, tc ? j->tc.err.p : nullptr, ls, h, graph), note_launch();
    const uint64_t m = uint64_t(k) * d;
    k_loop_commit<<<unsigned(umin64((m + 255) / 256, 1024)), 256, 0, st>>>(ls, j->C.p, j->Cw.p, m), note_launch();
    MC_TRY(launch_sort_by_key(j->asn.p, nullptr, n, k, j->sort, st));
    k_loop_check_empty<<<1, 256, 0, st>>>(j->sort.bucket_count.p, k, ls, h, graph), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

int job_build_loop_graph(mc_job *j) {
    if (j->loop_exec) {
        cudaGraphExecDestroy(j->loop_exec);
        j->loop_exec = nullptr;
    }
    cudaStream_t st = j->st;
    const uint64_t n = j->M.n, d = j->M.d;
    const uint32_t k = j->k;
    MC_TRY(j->loop_state.alloc(sizeof(LoopState), st));
    LoopState *ls = reinterpret_cast<LoopState *>(j->loop_state.p);
    const bool tc = j->M.kind == MC_DENSE_F32 && j->msr == SQRL2 && j->precision != MC_FP32;
    // every buffer the body touches exists before the capture: the sort and centroid work
    // space and the tensor-core path's FP32 rescan transform.  The centroid launch writes Cw,
    // which then takes the committed centers back (a restart on the host starts from Cw = C).
    MC_TRY(launch_sort_by_key(j->asn.p, nullptr, n, k, j->sort, st));
    MC_TRY(job_update_centers(j));
    MC_CUDA_TRY(cudaMemcpyAsync(j->Cw.p, j->C.p, uint64_t(k) * d * sizeof(float), cudaMemcpyDeviceToDevice, st));
    if (tc) MC_TRY(j->tc.CT0.alloc(uint64_t(tiled_center_pad(k, false, SQRL2)) * d, st));
    CaptureGuard guard{st};
    const uint64_t a0 = device_allocs();
    const uint64_t l0 = t_launches;
    MC_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    guard.on = true;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    MC_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle h;
    MC_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    MC_TRY(job_loop_pre(j, ls, h, 1));
    MC_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    MC_CUDA_TRY(cudaGraphAddNode(&wnode, g, deps, nullptr, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    MC_CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t top = nullptr;
    guard.on = false;
    MC_CUDA_TRY(cudaStreamEndCapture(st, &top));
    std::unique_ptr<CUgraph_st, cudaError_t (*)(cudaGraph_t)> top_owner(top, cudaGraphDestroy);
    const uint64_t l1 = t_launches;
    // the loop body, captured into the conditional node's graph
    MC_CUDA_TRY(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    guard.on = true;
    MC_TRY(job_loop_body(j, ls, h, 1));
    cudaGraph_t body_out = nullptr;
    guard.on = false;
    MC_CUDA_TRY(cudaStreamEndCapture(st, &body_out));
    const uint64_t l2 = t_launches;
    g_launches.fetch_sub(l2 - l0);  // counted when the graph runs
    if (device_allocs() != a0) return MC_EUNSUPPORTED;  // a buffer grew inside: stay on the host loop
    cudaGraphExec_t ex = nullptr;
    MC_CUDA_TRY(cudaGraphInstantiate(&ex, top, 0));
    j->loop_exec = ex;
    j->loop_pre_launches = l1 - l0;
    j->loop_body_launches = l2 - l1;
    return MC_OK;
}

// how mc_job_run runs the Lloyd loop (mc_loop_mode): MC_LOOP_HOST one host round trip per
// decision, MC_LOOP_FUSED one per iteration, MC_LOOP_GRAPH one per run; -1 = automatic
std::atomic<int> g_loop_mode{-2};  // -2: from MC_LOOP_MODE
thread_local int t_loop_graph = -1;  // 0: this thread never uses the graph

void drop_loop_graph(mc_job *j) {
    if (j->loop_exec) cudaGraphExecDestroy(j->loop_exec);
    j->loop_exec = nullptr;
}

int loop_mode_for(const mc_job *j, uint64_t maxiter) {
    int mode = g_loop_mode.load();
    if (mode == -2) {
        const char *e = std::getenv("MC_LOOP_MODE");
        mode = (e && e[0] >= '0' && e[0] <= '2' && !e[1]) ? e[0] - '0' : -1;
    }
    if (mode < 0) {
        // the graph pays one capture + instantiation per run; it wins when the run has many
        // iterations of little device work each
        const bool small = j->M.n * j->M.d <= (uint64_t(1) << 24);
        mode = (small && maxiter >= 16) ? MC_LOOP_GRAPH : MC_LOOP_FUSED;
    }
    if (mode == MC_LOOP_GRAPH && (t_loop_graph == 0 || profiling_enabled())) mode = MC_LOOP_FUSED;
    return mode;
}

// runs the loop graph from the host state (cost, iternum) until it hands back; the state
// comes back in `h`
// *ran = false: the loop could not be captured (the caller runs the host loop instead)
int job_run_loop_graph(mc_job *j, LoopState &h, bool *ran) {
    *ran = false;
    if (!j->loop_exec) {
        if (job_build_loop_graph(j) != MC_OK) {
            if (j->loop_exec) cudaGraphExecDestroy(j->loop_exec);
            j->loop_exec = nullptr;
            cudaGetLastError();
            return MC_OK;
        }
    }
    *ran = true;
    const unsigned long long it0 = h.iternum;
    MC_CUDA_TRY(cudaMemcpyAsync(j->loop_state.p, &h, sizeof(LoopState), cudaMemcpyHostToDevice, j->st));
    MC_CUDA_TRY(cudaGraphLaunch(j->loop_exec, j->st));
    MC_CUDA_TRY(cudaMemcpyAsync(&h, j->loop_state.p, sizeof(LoopState), cudaMemcpyDeviceToHost, j->st));
    MC_TRY(sync(j->st));
    const uint64_t bodies = (h.iternum - it0) + (h.reason == LOOP_REVERT || h.reason == LOOP_NAN ||
                                                  h.reason == LOOP_TIMEOUT ? 1 : 0);
    g_launches.fetch_add(j->loop_pre_launches + bodies * j->loop_body_launches);
    return MC_OK;
}

// The same launch sequence without a graph: one host round trip per iteration (the state
// after the body), instead of one per decision of the host loop.  Runs from the host state
// until the loop hands back.
int job_run_loop_fused(mc_job *j, LoopState &h) {
    cudaStream_t st = j->st;
    MC_TRY(j->loop_state.alloc(sizeof(LoopState), st));
    LoopState *ls = reinterpret_cast<LoopState *>(j->loop_state.p);
    cudaGraphConditionalHandle none = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(ls, &h, sizeof(LoopState), cudaMemcpyHostToDevice, st));
    MC_TRY(job_loop_pre(j, ls, none, 0));
    MC_CUDA_TRY(cudaMemcpyAsync(&h, ls, sizeof(LoopState), cudaMemcpyDeviceToHost, st));
    MC_TRY(sync(st));
    while (h.reason == LOOP_RUN) {
        MC_TRY(job_loop_body(j, ls, none, 0));
        MC_CUDA_TRY(cudaMemcpyAsync(&h, ls, sizeof(LoopState), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
    }
    return MC_OK;
}

}  // namespace

namespace {

__global__ void k_gather_dense_rows(const float *__restrict__ X, uint64_t d, const uint32_t *__restrict__ rows,
                                    uint64_t m, float *out) {
    const uint64_t total = m * d;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += gridDim.x * uint64_t(blockDim.x))
        out[e] = X[uint64_t(rows[e / d]) * d + e % d];
}

__global__ void k_gather_row_lens(const uint64_t *__restrict__ indptr, const uint32_t *__restrict__ rows, uint64_t m,
                                  uint64_t *lens) {
    const uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (t < m) lens[t] = indptr[rows[t] + 1] - indptr[rows[t]];
}

__global__ void k_gather_csr_rows(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                                  const uint64_t *__restrict__ indptr, const uint32_t *__restrict__ rows, uint64_t m,
                                  const uint64_t *__restrict__ subptr, float *ovals, uint32_t *oidx) {
    const uint64_t warp = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint64_t t = warp; t < m; t += (gridDim.x * uint64_t(blockDim.x)) >> 5) {
        const uint64_t b = indptr[rows[t]], e = indptr[rows[t] + 1], o = subptr[t];
        for (uint64_t p = b + lane; p < e; p += 32) {
            ovals[o + p - b] = vals[p];
            oidx[o + p - b] = idx[p];
        }
    }
}

__global__ void k_gather_f64(const double *__restrict__ v, const uint32_t *__restrict__ rows, uint64_t m, double *out) {
    const uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (t < m) out[t] = v[rows[t]];
}

// rows whose best restarted center beats their current cost take it (strict <; the
// restarted centers were searched in ascending order)
__global__ void k_merge_restarts(uint64_t n, const uint32_t *__restrict__ sub_asn, const double *__restrict__ sub_cost,
                                 const uint32_t *__restrict__ found, uint32_t *asn, double *costs) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i < n && sub_cost[i] < costs[i]) {
        asn[i] = found[sub_asn[i]];
        costs[i] = sub_cost[i];
    }
}

__global__ void k_gather_center_rows(const float *__restrict__ C, uint64_t d, const uint32_t *__restrict__ ids,
                                     uint64_t m, float *out) {
    const uint64_t total = m * d;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += gridDim.x * uint64_t(blockDim.x))
        out[e] = C[uint64_t(ids[e / d]) * d + e % d];
}

// Sample of the minibatch (the definition the oracle shares): U(seed ^ 0x6A09E667F3BCC908,
// counter++) -> floor(u * n); with replacement mbsize draws, otherwise draws until mbsize
// distinct rows (at most n); returned ascending (repeats adjacent).
std::vector<uint32_t> minibatch_sample(uint64_t seed, uint64_t &counter, uint64_t n, uint64_t mbsize, bool with_rep) {
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
        std::vector<uint8_t> seen;
        std::map<uint32_t, bool> seen_sparse;
        const bool dense_mark = n <= (uint64_t(64) << 20);
        if (dense_mark) seen.assign(n, 0);
        while (out.size() < target) {
            const uint32_t r = draw();
            if (dense_mark) {
                if (seen[r]) continue;
                seen[r] = 1;
            } else {
                if (seen_sparse.count(r)) continue;
                seen_sparse[r] = true;
            }
            out.push_back(r);
        }
    }
    std::sort(out.begin(), out.end());
    return out;
}

// the job's rows restricted to `rows` (device list of m ids) as a compact device matrix
struct SubRows {
    DBuf<float> X, vals;
    DBuf<uint32_t> idx;
    DBuf<uint64_t> lens, indptr;
    DBuf<double> w;
};

int gather_job_rows(mc_job *j, const uint32_t *rows, uint64_t m, SubRows &s, mc_matrix *out) {
    cudaStream_t st = j->st;
    const uint64_t d = j->M.d;
    if (j->w.p) {
        MC_TRY(s.w.alloc(m, st));
        k_gather_f64<<<unsigned((m + 255) / 256), 256, 0, st>>>(j->w.p, rows, m, s.w.p), note_launch();
    }
    if (j->M.kind == MC_DENSE_F32) {
        MC_TRY(s.X.alloc(m * d, st));
        k_gather_dense_rows<<<unsigned(umin64((m * d + 255) / 256, 65535)), 256, 0, st>>>(j->M.X, d, rows, m, s.X.p),
            note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        *out = mc_matrix{MC_DENSE_F32, 0, m, d, s.X.p, nullptr, nullptr, 0};
        return MC_OK;
    }
    MC_TRY(s.lens.alloc(m, st));
    MC_TRY(s.indptr.alloc(m + 1, st));
    k_gather_row_lens<<<unsigned((m + 255) / 256), 256, 0, st>>>(j->M.indptr, rows, m, s.lens.p), note_launch();
    MC_TRY(launch_exclusive_scan_u64(s.lens.p, s.indptr.p, m, st));
    uint64_t nnz = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(&nnz, s.indptr.p + m, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MC_TRY(sync(st));
    MC_TRY(s.vals.alloc(nnz ? nnz : 1, st));
    MC_TRY(s.idx.alloc(nnz ? nnz : 1, st));
    k_gather_csr_rows<<<unsigned(umin64((m + 7) / 8, 4096)), 256, 0, st>>>(j->M.vals, j->M.idx, j->M.indptr, rows, m,
                                                                         s.indptr.p, s.vals.p, s.idx.p), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    *out = mc_matrix{MC_CSR_F32, 0, m, d, s.vals.p, s.idx.p, s.indptr.p, nnz};
    return MC_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------
// soft clustering kernels (perform_soft_clustering, clustering/solve.h:287-374;
// set_centroids_full_mean soft form, clustering/centroid.h:795-866)
// ------------------------------------------------------------------------------------
// per row: asn = softmax(-temp * costs) (max-shifted, sequential sums in float); a NaN in
// the first entry is replaced by equal shares over the row's minimal costs (correct_softmax,
// centroid.h:782-793); rowval = dot(costs, asn) (sequential float) as double
__global__ void k_soft_rows(const float *__restrict__ costs, uint64_t n, uint32_t k, float temp, float *asn,
                            double *rowval) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const float *cr = costs + i * k;
    float *ar = asn + i * k;
    float m = -temp * cr[0];
    for (uint32_t c = 1; c < k; ++c) m = fmaxf(m, -temp * cr[c]);
    float s = 0.f;
    for (uint32_t c = 0; c < k; ++c) {
        const float e = expf(-temp * cr[c] - m);
        ar[c] = e;
        s = s + e;
    }
    for (uint32_t c = 0; c < k; ++c) ar[c] = ar[c] / s;
    if (ar[0] != ar[0]) {
        float best = cr[0];
        for (uint32_t c = 1; c < k; ++c) if (cr[c] < best) best = cr[c];
        uint32_t ties = 0;
        for (uint32_t c = 0; c < k; ++c) ties += (cr[c] == best) ? 1u : 0u;
        const float per = 1.f / float(ties ? ties : 1u);
        for (uint32_t c = 0; c < k; ++c) ar[c] = (cr[c] == best) ? per : 0.f;
    }
    float dot = 0.f;
    for (uint32_t c = 0; c < k; ++c) dot = dot + cr[c] * ar[c];
    rowval[i] = double(dot);
}

// soft weighted means in two steps with the order of a sequential walk: per chunk of 256
// rows and center c, thread j keeps a compensated float sum of coef * x[r][j] (coef = asn *
// float(w)) and of coef; then per (c, j) the chunk values are added in FP64 in chunk order,
// and center = num * (1 / den)
constexpr uint64_t kSoftChunk = 256;

__global__ void k_soft_center_chunks(const float *__restrict__ X, uint64_t n, uint64_t d,
                                     const float *__restrict__ asn, uint32_t k, const double *__restrict__ w,
                                     double *num /* [chunk][k][d] */, double *den /* [chunk][k] */) {
    const uint64_t q = blockIdx.x;
    const uint32_t c = blockIdx.y;
    const uint64_t r0 = q * kSoftChunk, r1 = umin64(n, r0 + kSoftChunk);
    for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) {
        float s = 0.f, e = 0.f, sw = 0.f, ew = 0.f;
        for (uint64_t r = r0; r < r1; ++r) {
            const float coef = w ? asn[r * k + c] * float(w[r]) : asn[r * k + c];
            const float t = coef * X[r * d + j];
            float tt = __fadd_rn(s, t), bp = __fsub_rn(tt, s);
            e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(tt, bp)), __fsub_rn(t, bp)));
            s = tt;
            tt = __fadd_rn(sw, coef);
            bp = __fsub_rn(tt, sw);
            ew = __fadd_rn(ew, __fadd_rn(__fsub_rn(sw, __fsub_rn(tt, bp)), __fsub_rn(coef, bp)));
            sw = tt;
        }
        num[(q * k + c) * d + j] = double(s) + double(e);
        if (j == 0) den[q * k + c] = double(sw) + double(ew);
    }
}

// adds the partials of chunks [0, nq) of one batch to the running FP64 sums, in chunk order
// CSR rows: the same chunk partials, accumulated over each row's nonzeros (a zero term adds
// exactly nothing to the compensated sums).  The running (s, e) of every column live in
// sb / eb ([chunk][k][d], zeroed by the caller); rows are taken in order, one after the
// other, and the columns of one row are distinct, so each column's sum keeps the row order.
__global__ void __launch_bounds__(256) k_soft_center_chunks_csr(const float *__restrict__ vals,
                                                                const uint32_t *__restrict__ idx,
                                                                const uint64_t *__restrict__ indptr, uint64_t n,
                                                                uint64_t d, const float *__restrict__ asn, uint32_t k,
                                                                const double *__restrict__ w, float *sb, float *eb,
                                                                double *num, double *den) {
    const uint64_t q = blockIdx.x;
    const uint32_t c = blockIdx.y;
    const uint64_t r0 = q * kSoftChunk, r1 = umin64(n, r0 + kSoftChunk);
    float *s = sb + (q * k + c) * d, *e = eb + (q * k + c) * d;
    float sw = 0.f, ew = 0.f;
    for (uint64_t r = r0; r < r1; ++r) {
        const float coef = w ? asn[r * k + c] * float(w[r]) : asn[r * k + c];
        for (uint64_t p = indptr[r] + threadIdx.x; p < indptr[r + 1]; p += blockDim.x) {
            const uint32_t j = idx[p];
            const float t = coef * vals[p];
            float tt = __fadd_rn(s[j], t), bp = __fsub_rn(tt, s[j]);
            e[j] = __fadd_rn(e[j], __fadd_rn(__fsub_rn(s[j], __fsub_rn(tt, bp)), __fsub_rn(t, bp)));
            s[j] = tt;
        }
        if (threadIdx.x == 0) {
            const float tt = __fadd_rn(sw, coef), bp = __fsub_rn(tt, sw);
            ew = __fadd_rn(ew, __fadd_rn(__fsub_rn(sw, __fsub_rn(tt, bp)), __fsub_rn(coef, bp)));
            sw = tt;
        }
        __syncthreads();
    }
    for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) num[(q * k + c) * d + j] = double(s[j]) + double(e[j]);
    if (threadIdx.x == 0) den[q * k + c] = double(sw) + double(ew);
}

// soft L1 centers over dense rows (set_centroids_soft, clustering/centroid.h:815-838, with
// optim/kmedian.h: weighted_median): per center c the weights are the soft assignments of
// column c (times the row weights); weighted_median never accumulates its weight total, so
// it returns per column the value of the row with the largest weight (the smallest such value
// on ties).  One CTA per (center, 32 columns): the largest weight, then the minima.
__global__ void __launch_bounds__(256) k_soft_l1_centers(const float *__restrict__ X, uint64_t n, uint64_t d,
                                                         const float *__restrict__ asn, uint32_t k,
                                                         const double *__restrict__ w, float *centers) {
    __shared__ double wmax[8];
    __shared__ float best[8][32];
    const uint32_t c = blockIdx.x;
    const uint64_t c0 = uint64_t(blockIdx.y) * 32;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    double mx = -1.7976931348623157e308;
    for (uint64_t r = t; r < n; r += 256) {
        const double wt = w ? w[r] * double(asn[r * k + c]) : double(asn[r * k + c]);
        mx = fmax(mx, wt);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) wmax[warp] = mx;
    __syncthreads();
    mx = wmax[0];
    for (int q = 1; q < 8; ++q) mx = fmax(mx, wmax[q]);
    const uint64_t col = c0 + lane;
    float bv = __int_as_float(0x7f800000);
    for (uint64_t r = warp; r < n; r += 8) {
        const double wt = w ? w[r] * double(asn[r * k + c]) : double(asn[r * k + c]);
        if (wt == mx && col < d) bv = fminf(bv, X[r * d + col]);
    }
    best[warp][lane] = bv;
    __syncthreads();
    if (t < 32 && col < d) {
        float v = best[0][lane];
        for (int q = 1; q < 8; ++q) v = fminf(v, best[q][lane]);
        centers[uint64_t(c) * d + col] = v;
    }
}

__global__ void k_soft_center_accumulate(const double *__restrict__ num, const double *__restrict__ den, uint64_t nq,
                                         uint32_t k, uint64_t d, double *acc_num, double *acc_den) {
    const uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    const uint32_t c = blockIdx.y;
    if (j >= d) return;
    double a = acc_num[uint64_t(c) * d + j], b = acc_den[c];
    for (uint64_t q = 0; q < nq; ++q) {
        a = a + num[(q * k + c) * d + j];
        b = b + den[q * k + c];
    }
    acc_num[uint64_t(c) * d + j] = a;
    if (j == 0) acc_den[c] = b;
}

__global__ void k_soft_center_finalize(const double *__restrict__ acc_num, const double *__restrict__ acc_den,
                                       uint32_t k, uint64_t d, float *centers) {
    const uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    const uint32_t c = blockIdx.y;
    if (j >= d) return;
    centers[uint64_t(c) * d + j] = float(acc_num[uint64_t(c) * d + j] * (1.0 / acc_den[c]));
}

extern "C" {

const char *mc_version(void) { return "minicore_gb300 0.1 (sm_103a)"; }
uint64_t mc_kernel_launches(void) { return g_launches.load(); }
int mc_test_tc_stall_once(void) {
    tc_stall_next();
    return MC_OK;
}

}  // extern "C"

namespace mc {
void set_thread_loop_graph(int on) { t_loop_graph = on; }
}  // namespace mc

extern "C" {

int mc_loop_mode(int mode) {
    if (mode < -1 || mode > 2) return fail(MC_EINVAL, "loop mode is -1 (automatic), 0, 1 or 2");
    g_loop_mode.store(mode);
    return MC_OK;
}

int mc_profile_enable(int on) {
    g_prof_on.store(on != 0);
    return MC_OK;
}

int mc_profile_reset(void) {
    std::lock_guard<std::mutex> lock(g_prof_mu);
    for (auto &r : g_prof) {
        cudaEventSynchronize(r.b);
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    g_prof.clear();
    return MC_OK;
}

int mc_profile_report(char *json, uint64_t cap) {
    std::lock_guard<std::mutex> lock(g_prof_mu);
    std::map<std::string, std::pair<uint64_t, double>> agg;
    for (auto &r : g_prof) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            auto &e = agg[r.name];
            e.first += 1;
            e.second += ms;
        }
    }
    std::string out = "{";
    bool first = true;
    for (auto &kv : agg) {
        out += (first ? "\"" : ", \"") + kv.first + "\": {\"count\": " + std::to_string(kv.second.first) +
               ", \"ms\": " + std::to_string(kv.second.second) + "}";
        first = false;
    }
    out += "}";
    if (!json || cap == 0) return fail(MC_EINVAL, "no output buffer");
    if (out.size() + 1 > cap) return fail(MC_EINVAL, "profile report needs " + std::to_string(out.size() + 1) + " bytes");
    std::memcpy(json, out.c_str(), out.size() + 1);
    return MC_OK;
}
const char *mc_last_error(void) { return g_last_error.c_str(); }

int mc_uniforms(uint64_t seed, uint64_t offset, uint64_t m, double *out) {
    if (!out && m) return fail(MC_EINVAL, "out is null");
    for (uint64_t i = 0; i < m; ++i) out[i] = uniform_at(seed, offset + i);
    return MC_OK;
}

int mc_context_create(int device, mc_context **out) {
    if (!out) return fail(MC_EINVAL, "out is null");
    int ndev = 0;
    MC_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(MC_EINVAL, "no such CUDA device");
    MC_CUDA_TRY(cudaSetDevice(device));
    auto *c = new mc_context();
    c->device = device;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) c->sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(MC_ECUDA, "stream creation failed");
    }
    c->stream = c->own;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = c;
    return MC_OK;
}

int mc_context_destroy(mc_context *ctx) {
    if (!ctx) return MC_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
    return MC_OK;
}

int mc_context_set_stream(mc_context *ctx, void *s) {
    if (!ctx) return fail(MC_EINVAL, "ctx is null");
    ctx->stream = s ? (cudaStream_t)s : ctx->own;
    return MC_OK;
}

int mc_context_synchronize(mc_context *ctx) {
    if (!ctx) return fail(MC_EINVAL, "ctx is null");
    MC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// jobs
// ------------------------------------------------------------------------------------
// centers == nullptr: seed them by D^2 sampling with U(seed, i), i < k, on the job's own
// device copy of the rows (kmeans.h:49-215), then copy the chosen rows into the centers,
// which is what minicore.cluster() does between kmeanspp and hcluster
// (python/minicore/__init__.py:235-261), without a host round trip.
static int job_create_impl(mc_context *ctx, const mc_matrix *X, const float *centers, uint32_t k, int msr,
                           double prior, const double *weights, int precision, uint64_t seed, uint32_t *center_ids,
                           mc_job **out) {
    if (!ctx || !out) return fail(MC_EINVAL, "null context or output");
    if (!measure_supported(msr)) return fail(MC_EUNSUPPORTED, "measure not implemented on this path");
    if (precision != MC_FP32 && precision != MC_TF32 && precision != MC_BF16)
        return fail(MC_EINVAL, "unknown precision");
    if (k == 0) return fail(MC_EINVAL, "no centers");
    MC_CUDA_TRY(cudaSetDevice(ctx->device));
    std::unique_ptr<mc_job> j(new mc_job());
    j->ctx = ctx;
    j->st = ctx->stream;
    cudaStream_t st = j->st;
    MC_TRY(j->M.load(X, st));
    if (precision != MC_FP32 && (msr != SQRL2 || j->M.kind != MC_DENSE_F32))
        return fail(MC_EUNSUPPORTED, "BF16/TF32 tensor-core assignment covers dense SQRL2 only");
    const uint64_t n = j->M.n, d = j->M.d;
    j->msr = msr;
    j->prior = prior;
    j->precision = precision;
    j->seed = seed;
    j->k = k;
    j->psum = double(float(prior * double(d)));
    MC_TRY(j->rowsum.alloc(n, st));
    MC_TRY(j->costs.alloc(n, st));
    MC_TRY(j->asn.alloc(n, st));
    MC_TRY(j->C.alloc(uint64_t(k) * d, st));
    MC_TRY(j->Cw.alloc(uint64_t(k) * d, st));
    MC_TRY(j->csum.alloc(k, st));
    MC_TRY(j->cnorm.alloc(k, st));
    MC_TRY(j->det_tmp.alloc(det_tmp_size(n), st));
    MC_TRY(j->scal.alloc(4, st));
    MC_TRY(j->flag.alloc(1, st));
    if (centers)
        MC_CUDA_TRY(cudaMemcpyAsync(j->C.p, centers, uint64_t(k) * d * sizeof(float), cudaMemcpyDefault, st));
    if (weights) {
        MC_TRY(j->w.alloc(n, st));
        MC_CUDA_TRY(cudaMemcpyAsync(j->w.p, weights, n * sizeof(double), cudaMemcpyDefault, st));
    }
    if (j->M.kind == MC_DENSE_F32) {
        MC_TRY(j->rownorm.alloc(n, st));
        // SQRL2 reads no row sums (the prior does not enter it)
        MC_TRY(launch_row_sums_dense(j->M.X, n, d, msr == SQRL2 ? nullptr : j->rowsum.p, j->rownorm.p, st));
    } else {
        MC_TRY(launch_row_sums_csr(j->M.vals, j->M.indptr, n, j->rowsum.p, st));
    }
    if (j->M.kind == MC_CSR_F32 && msr == JSD)
        MC_TRY(build_rinc_groups(j->rowsum.p, n, d, j->M.nnz, float(prior), st, j->grp, j->gval, j->ngrp));
    if (!centers) {
        if (k > n) return fail(MC_EINVAL, "k-means++ seeding needs k <= number of rows");
        std::vector<double> uh(k);
        for (uint32_t i = 0; i < k; ++i) uh[i] = uniform_at(seed, i);
        DBuf<double> u, dist, tmp;
        DBuf<float> cbuf, ct;
        DBuf<double> cconst;
        DBuf<uint32_t> ids;
        DBuf<uint64_t> newc;
        MC_TRY(u.alloc(k, st));
        MC_TRY(dist.alloc(n, st));
        MC_TRY(tmp.alloc(det_tmp_size(n), st));
        MC_TRY(cbuf.alloc(d, st));
        MC_TRY(ids.alloc(k, st));
        MC_TRY(newc.alloc(1, st));
        MC_CUDA_TRY(cudaMemcpyAsync(u.p, uh.data(), k * sizeof(double), cudaMemcpyHostToDevice, st));
        KmppArgs a;
        a.msr = msr;
        a.csr = j->M.kind == MC_CSR_F32;
        a.n = n;
        a.d = d;
        a.k = k;
        a.X = j->M.X;
        a.vals = j->M.vals;
        a.idx = j->M.idx;
        a.indptr = j->M.indptr;
        a.rowsum = j->rowsum.p;
        a.w = j->w.p;
        a.prior = prior;
        a.prior_sum = prior * double(d);
        a.cbuf = cbuf.p;
        if (a.csr && kmpp_csr_nnz_path(n, d, j->M.nnz) && (msr != JSD || j->ngrp)) {
            MC_TRY(ct.alloc(d, st));
            MC_TRY(cconst.alloc(msr == JSD ? j->ngrp : 2, st));
            a.ct = ct.p;
            a.cconst = cconst.p;
            a.grp = j->grp.p;
            a.gval = j->gval.p;
            a.ngrp = j->ngrp;
        }
        a.dist = dist.p;
        a.asn = j->asn.p;
        a.center_ids = ids.p;
        a.newc = newc.p;
        MC_TRY(run_kmeanspp(a, u.p, tmp.p, ctx->sms, st));
        MC_TRY(launch_gather_rows(j->M.kind == MC_CSR_F32, j->M.X, j->M.vals, j->M.idx, j->M.indptr, d, ids.p, k,
                                  j->C.p, st));
        if (center_ids) MC_TRY(copy_out(center_ids, ids.p, k, st));
        MC_TRY(sync(st));
    }
    // constant-prior check: pv == prior for every pair when prior >= smallest_pv at the
    // largest row and center sums (centers are means or rows, so bounded by the rows)
    if (msr != SQRL2) {
        MC_TRY(launch_center_sums(j->C.p, k, d, j->csum.p, j->cnorm.p, st));
        std::vector<double> rs(n), cs(k);
        MC_CUDA_TRY(cudaMemcpyAsync(rs.data(), j->rowsum.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        MC_CUDA_TRY(cudaMemcpyAsync(cs.data(), j->csum.p, k * sizeof(double), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
        double mr = rs.empty() ? 0.0 : *std::max_element(rs.begin(), rs.end());
        const double mc_ = cs.empty() ? 0.0 : *std::max_element(cs.begin(), cs.end());
        mr = std::max(mr, mc_);
        const float fp = float(prior);
        const float s0 = float(mr + j->psum);
        const float smallest = 7.0069e-42f * (s0 + s0);
        j->pair = !(fp > 0.f) || (fp < smallest);
        j->pv = fp;
        if (!j->pair) {
            MC_TRY(j->rsi.alloc(n, st));
            MC_TRY(j->rinc.alloc(n, st));
            MC_TRY(launch_row_scalars(j->rowsum.p, n, d, j->pv, j->rsi.p, j->rinc.p, st));
        }
    }
    j->sparse_path = j->M.kind == MC_CSR_F32 && !j->pair && (msr != JSD || j->ngrp > 0);
    *out = j.release();
    return MC_OK;
}

int mc_job_create(mc_context *ctx, const mc_matrix *X, const float *centers, uint32_t k, int msr, double prior,
                  const double *weights, int precision, uint64_t seed, mc_job **out) {
    if (!centers) return fail(MC_EINVAL, "no centers");
    return job_create_impl(ctx, X, centers, k, msr, prior, weights, precision, seed, nullptr, out);
}

int mc_job_create_kmeanspp(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior,
                           const double *weights, int precision, uint64_t seed, uint32_t *center_ids, mc_job **out) {
    return job_create_impl(ctx, X, nullptr, k, msr, prior, weights, precision, seed, center_ids, out);
}

int mc_job_destroy(mc_job *job) {
    if (!job) return MC_OK;
    cudaStreamSynchronize(job->st);
    delete job;
    return MC_OK;
}

int mc_job_assign(mc_job *j) {
    if (!j) return fail(MC_EINVAL, "job is null");
    return job_assign_with(j, j->C.p, j->psum, false);
}

int mc_job_cost(mc_job *j, double *cost) {
    if (!j || !cost) return fail(MC_EINVAL, "null argument");
    float c = 0.f;
    MC_TRY(job_cost(j, &c));
    *cost = c;
    return MC_OK;
}

int mc_job_lloyd_step(mc_job *j, int *restarted) {
    if (!j) return fail(MC_EINVAL, "job is null");
    int res = 0;
    MC_CUDA_TRY(cudaMemcpyAsync(j->Cw.p, j->C.p, uint64_t(j->k) * j->M.d * sizeof(float), cudaMemcpyDeviceToDevice,
                                j->st));
    MC_TRY(job_set_centroids(j, &res));
    MC_TRY(job_assign_with(j, j->Cw.p, j->psum, false));
    std::swap(j->C.p, j->Cw.p);
    std::swap(j->C.n, j->Cw.n);
    if (restarted) *restarted = res;
    return MC_OK;
}

int mc_job_run(mc_job *j, double eps, uint64_t maxiter, double *initcost_out, double *finalcost_out,
               uint64_t *numiter_out) {
    if (!j) return fail(MC_EINVAL, "job is null");
    MC_TRY(job_assign_with(j, j->C.p, j->psum, false));
    float initcost = 0.f;
    MC_TRY(job_cost(j, &initcost));
    float cost = initcost;
    uint64_t iternum = 0;
    if (cost == 0.f) {
        if (initcost_out) *initcost_out = 0.0;
        if (finalcost_out) *finalcost_out = 0.0;
        if (numiter_out) *numiter_out = 0;
        return MC_OK;
    }
    const size_t cbytes = uint64_t(j->k) * j->M.d * sizeof(float);
    MC_CUDA_TRY(cudaMemcpyAsync(j->Cw.p, j->C.p, cbytes, cudaMemcpyDeviceToDevice, j->st));
    const int mode = loop_mode_for(j, maxiter);
    bool graph = mode == MC_LOOP_GRAPH, fused = mode != MC_LOOP_HOST;
    drop_loop_graph(j);
    for (;;) {
        LoopState h = {};
        h.cost = cost;
        h.reason = LOOP_RUN;
        h.iternum = iternum;
        h.maxiter = maxiter;
        h.eps = eps;
        if (graph) MC_TRY(job_run_loop_graph(j, h, &graph));  // graph = false: not capturable
        if (!graph && fused) MC_TRY(job_run_loop_fused(j, h));
        if (fused) {
            cost = h.cost;
            iternum = h.iternum;
            if (h.reason == LOOP_DONE) break;
            if (h.reason == LOOP_REVERT) {
                MC_TRY(job_assign_with(j, j->C.p, j->psum, false));
                break;
            }
            if (h.reason == LOOP_NAN) return fail(MC_ENAN, "Unexpected nan in ctr");
            if (h.reason == LOOP_TIMEOUT)
                return fail(MC_ETIMEOUT, "tensor-core assignment: bounded wait expired");
            if (h.reason != LOOP_EMPTY) return fail(MC_ECUDA, "Lloyd loop graph returned without a decision");
            // an empty cluster: one update with the D^2 restart on the host, then the graph again
            drop_loop_graph(j);
        }
        int res = 0;
        MC_TRY(job_set_centroids(j, &res));
        MC_TRY(job_assign_with(j, j->Cw.p, j->psum, false));
        float newcost = 0.f;
        MC_TRY(job_cost(j, &newcost));
        if (newcost > cost && !res) {
            MC_TRY(job_assign_with(j, j->C.p, j->psum, false));
            break;
        }
        MC_CUDA_TRY(cudaMemcpyAsync(j->C.p, j->Cw.p, cbytes, cudaMemcpyDeviceToDevice, j->st));
        ++iternum;
        const float oldcost = cost;
        cost = newcost;
        if (double(oldcost - newcost) < eps * std::max(double(newcost), double(oldcost)) || iternum > maxiter) break;
    }
    MC_TRY(sync(j->st));
    if (initcost_out) *initcost_out = initcost;
    if (finalcost_out) *finalcost_out = cost;
    if (numiter_out) *numiter_out = iternum;
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// minibatch hard clustering (perform_hard_minibatch_clustering, clustering/solve.h:386-582)
// ------------------------------------------------------------------------------------

int mc_job_minibatch(mc_job *j, uint64_t mbsize, uint64_t maxiter, uint64_t calc_cost_freq, uint64_t reseed_after,
                     int with_replacement, double *initcost_out, double *finalcost_out, uint64_t *numiter_out) {
    if (!j) return fail(MC_EINVAL, "job is null");
    if (mbsize == 0) return fail(MC_EINVAL, "mbsize must be positive");
    if (maxiter == 0) return fail(MC_EINVAL, "maxiter must be positive");
    if (calc_cost_freq == 0) calc_cost_freq = 1;
    cudaStream_t st = j->st;
    const uint64_t n = j->M.n, d = j->M.d;
    const uint32_t k = j->k;
    const size_t cbytes = uint64_t(k) * d * sizeof(float);
    // every distance in this routine takes the prior itself as the prior sum, as the
    // reference's minibatch code does (solve.h:405: prior.size() * prior[0])
    const double psum_mb = double(float(j->prior));
    DBuf<float> save;
    MC_TRY(save.alloc(uint64_t(k) * d, st));
    MC_CUDA_TRY(cudaMemcpyAsync(save.p, j->C.p, cbytes, cudaMemcpyDeviceToDevice, st));
    MC_TRY(j->idxbuf.alloc(uint64_t(k) + 2, st));
    DBuf<uint32_t> rows_dev, found_dev;
    DBuf<float> Cs;
    double initcost = 0.0, bestcost = 0.0, cost = 0.0;
    uint64_t iternum = 0, sample_counter = 0;
    for (;;) {
        if (iternum % calc_cost_freq == 0 || iternum == maxiter - 1) {
            // exhaustive assignment; restart the centers holding few rows
            MC_TRY(job_assign_with(j, j->C.p, psum_mb, false));
            MC_TRY(launch_sort_by_key(j->asn.p, nullptr, n, k, j->sort, st));
            std::vector<uint64_t> cnt(k);
            MC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), j->sort.bucket_count.p, k * sizeof(uint64_t),
                                        cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
            std::vector<uint32_t> found;
            for (uint32_t c = 0; c < k; ++c)
                if (cnt[c] <= reseed_after) found.push_back(c);
            if (!found.empty()) {
                for (uint32_t c : found) {
                    const double u = uniform_at(j->seed, j->restart_counter++);
                    DetInput in{j->w.p ? DET_F64_W : DET_F64, j->costs.p, nullptr, j->w.p, n};
                    MC_TRY(launch_det_draw(in, j->det_tmp.p, nullptr, u, 0, nullptr, j->idxbuf.p + k, st));
                    float *dst = j->C.p + uint64_t(c) * d;
                    if (j->M.kind == MC_DENSE_F32) {
                        k_copy_row_dense<<<unsigned(umin64((d + 255) / 256, 1024)), 256, 0, st>>>(
                            j->M.X, d, j->idxbuf.p + k, dst), note_launch();
                    } else {
                        k_copy_row_csr_zero<<<unsigned(umin64((d + 255) / 256, 1024)), 256, 0, st>>>(d, dst), note_launch();
                        k_copy_row_csr<<<64, 256, 0, st>>>(j->M.vals, j->M.idx, j->M.indptr, j->idxbuf.p + k, dst),
                            note_launch();
                    }
                    MC_CUDA_TRY(cudaGetLastError());
                }
                // every row against the restarted centers only; better ones take over
                const uint64_t nf = found.size();
                MC_TRY(found_dev.alloc(nf, st));
                MC_CUDA_TRY(cudaMemcpyAsync(found_dev.p, found.data(), nf * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
                MC_TRY(Cs.alloc(nf * d, st));
                k_gather_center_rows<<<unsigned(umin64((nf * d + 255) / 256, 65535)), 256, 0, st>>>(j->C.p, d,
                                                                                                  found_dev.p, nf, Cs.p),
                    note_launch();
                mc_matrix all{j->M.kind, 0, n, d, j->M.kind == MC_DENSE_F32 ? j->M.X : j->M.vals, j->M.idx,
                              j->M.indptr, j->M.nnz};
                mc_job *rj = nullptr;
                MC_TRY(job_create_impl(j->ctx, &all, Cs.p, uint32_t(nf), j->msr, j->prior, nullptr, MC_FP32, j->seed,
                                       nullptr, &rj));
                std::unique_ptr<mc_job, int (*)(mc_job *)> rguard(rj, mc_job_destroy);
                MC_TRY(job_assign_with(rj, rj->C.p, psum_mb, true));
                k_merge_restarts<<<unsigned((n + 255) / 256), 256, 0, st>>>(n, rj->asn.p, rj->costs.p, found_dev.p,
                                                                            j->asn.p, j->costs.p), note_launch();
                MC_CUDA_TRY(cudaGetLastError());
            }
            DetInput in{j->w.p ? DET_F64_W : DET_F64, j->costs.p, nullptr, j->w.p, n};
            MC_TRY(launch_det_sum(in, j->det_tmp.p, j->scal.p, st));
            MC_CUDA_TRY(cudaMemcpyAsync(&cost, j->scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
            if (iternum == 0) initcost = bestcost = cost;
            if (cost < bestcost) {
                bestcost = cost;
                MC_CUDA_TRY(cudaMemcpyAsync(save.p, j->C.p, cbytes, cudaMemcpyDeviceToDevice, st));
            }
        }
        if (++iternum == maxiter) break;
        // sample, assign the sampled rows exactly, replace every hit center by its group's mean
        const std::vector<uint32_t> smp = minibatch_sample(j->seed, sample_counter, n, mbsize, with_replacement != 0);
        const uint64_t m = smp.size();
        MC_TRY(rows_dev.alloc(m, st));
        MC_CUDA_TRY(cudaMemcpyAsync(rows_dev.p, smp.data(), m * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        SubRows sr;
        mc_matrix subm;
        MC_TRY(gather_job_rows(j, rows_dev.p, m, sr, &subm));
        mc_job *sj = nullptr;
        MC_TRY(job_create_impl(j->ctx, &subm, j->C.p, k, j->msr, j->prior, sr.w.p, MC_FP32, j->seed, nullptr, &sj));
        std::unique_ptr<mc_job, int (*)(mc_job *)> sguard(sj, mc_job_destroy);
        MC_TRY(job_assign_with(sj, sj->C.p, psum_mb, true));
        if (j->msr == L1) {
            // l1_median over each group's sampled rows (solve.h:559-561; kmedian.h:329-344,
            // util/csc.h:829-893); groups without rows keep their center
            MC_TRY(launch_sort_by_key(sj->asn.p, nullptr, m, k, sj->sort, st));
            if (sj->M.kind == MC_DENSE_F32) {
                MC_TRY(launch_l1_medians(sj->M.X, d, k, sj->sort, j->w.p, j->C.p, st, n));
            } else {
                if (j->w.p) return fail(MC_EUNSUPPORTED, "Not implemented: weighted L1 median for CSparseMatrix");
                MC_TRY(launch_l1_medians_csr(sj->M.vals, sj->M.idx, sj->M.indptr, m, d, sj->M.nnz, k, sj->asn.p,
                                             sj->sort, sj->l1csr, j->C.p, st));
            }
            MC_TRY(sync(st));
            continue;
        }
        CentroidArgs ca;
        ca.csr = sj->M.kind == MC_CSR_F32;
        ca.n = m;
        ca.d = d;
        ca.k = k;
        ca.X = sj->M.X;
        ca.vals = sj->M.vals;
        ca.idx = sj->M.idx;
        ca.indptr = sj->M.indptr;
        ca.nnz = sj->M.nnz;
        ca.keys = sj->asn.p;
        ca.w = sj->w.p;
        ca.centers = j->C.p;  // groups with no sampled row keep their center
        ca.nan_flag = j->flag.p;
        MC_CUDA_TRY(cudaMemsetAsync(j->flag.p, 0, sizeof(int), st));
        MC_TRY(launch_centroids(ca, sj->sort, st));
        int nanf = 0;
        MC_CUDA_TRY(cudaMemcpyAsync(&nanf, j->flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
        if (nanf) return fail(MC_ENAN, "Unexpected nan in ctr");
    }
    MC_CUDA_TRY(cudaMemcpyAsync(j->C.p, save.p, cbytes, cudaMemcpyDeviceToDevice, st));
    MC_TRY(sync(st));
    if (initcost_out) *initcost_out = initcost;
    if (finalcost_out) *finalcost_out = bestcost;
    if (numiter_out) *numiter_out = iternum;
    return MC_OK;
}

int mc_hcluster_minibatch(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr,
                          double prior, const double *weights, uint64_t mbsize, uint64_t maxiter, uint64_t ncheckins,
                          uint64_t reseed_count, int with_replacement, uint64_t seed, int precision,
                          float *centers_out, uint32_t *asn, double *costs, double *initcost, double *finalcost,
                          uint64_t *numiter) {
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, X, centers_in, k, msr, prior, weights, precision, seed, &j));
    std::unique_ptr<mc_job, int (*)(mc_job *)> guard(j, mc_job_destroy);
    if (ncheckins == 0) ncheckins = 10;
    const uint64_t freq = (maxiter + ncheckins - 1) / ncheckins;  // pycluster.h:36-37
    MC_TRY(mc_job_minibatch(j, mbsize, maxiter, freq, reseed_count, with_replacement, initcost, finalcost, numiter));
    return mc_job_read(j, centers_out, asn, costs);
}

}  // extern "C"

namespace {

__global__ void k_f64_to_f32(const double *__restrict__ a, uint64_t n, float *b) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        b[i] = float(a[i]);
}

// after an assignment against the restarted centers only (asn holds their positions in
// `found`): a row moves to the best restarted center when that is strictly cheaper than
// its previous cost, else it keeps (save_asn, save_cost)
__global__ void k_merge_restarted(uint64_t n, const uint32_t *__restrict__ found, const uint32_t *__restrict__ save_asn,
                                  const double *__restrict__ save_cost, uint32_t *asn, double *costs) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        if (costs[i] < save_cost[i]) {
            asn[i] = found[asn[i]];
        } else {
            asn[i] = save_asn[i];
            costs[i] = save_cost[i];
        }
    }
}

// minibatch-by-coreset EM (hmb_coreset_clustering, clustering/solve.h:593-789), the
// reference's cs=True path (python/pycluster.h:36-39): rounds of an exhaustive assignment,
// restarts of the centers holding <= reseed_after rows (D^2 draws U(seed, r) over the costs,
// weighted by the row weights; each row then moves to a restarted center that is strictly
// cheaper), the objective (best centers kept), then calc_cost_freq times: a coreset of
// min(mbsize, n) distinct rows (LBK sensitivities, VX for L1, alpha = msr2alpha; sample seed
// floor(U(seed, r) 2^53)) and perform_hard_clustering on it (eps 1e-3, 1 update, 3 in the
// first two rounds; weights = coreset weights times row weights; restart seed = coreset
// size).  The uniform counter r is shared by the restarts and the sample seeds, in order.
int job_coreset_minibatch(mc_job *j, uint64_t mbsize, uint64_t maxiter, uint64_t calc_cost_freq,
                          uint64_t reseed_after, float *best_centers, double *initcost_out, double *finalcost_out,
                          uint64_t *numiter_out) {
    cudaStream_t st = j->st;
    const uint64_t n = j->M.n, d = j->M.d;
    const uint32_t k = j->k;
    const size_t cbytes = uint64_t(k) * d * sizeof(float);
    if (calc_cost_freq == 0) calc_cost_freq = 1;
    const uint64_t rounds = (calc_cost_freq - 1 + maxiter) / calc_cost_freq;
    const uint64_t m = std::min<uint64_t>(std::max<uint64_t>(mbsize, 1), n);
    const double alpha = j->msr == L1 ? 1.0 : j->msr == SQRL2 ? 2.0 : 4.0;  // msr2alpha, distance.h:310-318
    const int method = j->msr == L1 ? MC_VX : MC_LBK;
    uint64_t counter = 0;
    DBuf<float> wf;
    if (j->w.p) {
        MC_TRY(wf.alloc(n, st));
        k_f64_to_f32<<<unsigned(umin64((n + 255) / 256, 4096)), 256, 0, st>>>(j->w.p, n, wf.p), note_launch();
    }
    MC_CUDA_TRY(cudaMemcpyAsync(best_centers, j->C.p, cbytes, cudaMemcpyDefault, st));
    DBuf<uint32_t> save_asn, found_dev, rows_dev;
    DBuf<double> save_cost;
    DBuf<float> Cs;
    MC_TRY(j->idxbuf.alloc(uint64_t(k) + 2, st));
    double initcost = 0.0, bestcost = 0.0, cost = 0.0;
    uint64_t iternum = 0;
    std::vector<float> cw_f(m);
    std::vector<uint64_t> cidx(m);
    std::vector<uint32_t> rows32(m);
    std::vector<double> cw(m), wrow(j->w.p ? n : 0);
    if (j->w.p) {
        MC_CUDA_TRY(cudaMemcpyAsync(wrow.data(), j->w.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
    }
    for (;;) {
        MC_TRY(job_assign_with(j, j->C.p, j->psum, false));
        MC_TRY(launch_sort_by_key(j->asn.p, nullptr, n, k, j->sort, st));
        std::vector<uint64_t> cnt(k);
        MC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), j->sort.bucket_count.p, k * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
        std::vector<uint32_t> found;
        for (uint32_t c = 0; c < k; ++c)
            if (cnt[c] <= reseed_after) found.push_back(c);
        if (!found.empty()) {
            for (uint32_t fidx : found) {
                const double u = uniform_at(j->seed, counter++);
                DetInput in{j->w.p ? DET_F64_W : DET_F64, j->costs.p, nullptr, j->w.p, n};
                MC_TRY(launch_det_draw(in, j->det_tmp.p, nullptr, u, 0, nullptr, j->idxbuf.p + k, st));
                float *dst = j->C.p + uint64_t(fidx) * d;
                if (j->M.kind == MC_DENSE_F32) {
                    k_copy_row_dense<<<unsigned(umin64((d + 255) / 256, 1024)), 256, 0, st>>>(j->M.X, d, j->idxbuf.p + k,
                                                                                              dst), note_launch();
                } else {
                    k_copy_row_csr_zero<<<unsigned(umin64((d + 255) / 256, 1024)), 256, 0, st>>>(d, dst), note_launch();
                    k_copy_row_csr<<<64, 256, 0, st>>>(j->M.vals, j->M.idx, j->M.indptr, j->idxbuf.p + k, dst),
                        note_launch();
                }
                MC_CUDA_TRY(cudaGetLastError());
            }
            // the rows against the restarted centers only, then the strict-improvement merge
            const uint32_t nf = uint32_t(found.size());
            MC_TRY(save_asn.alloc(n, st));
            MC_TRY(save_cost.alloc(n, st));
            MC_TRY(found_dev.alloc(nf, st));
            MC_TRY(Cs.alloc(uint64_t(nf) * d, st));
            MC_CUDA_TRY(cudaMemcpyAsync(save_asn.p, j->asn.p, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
            MC_CUDA_TRY(cudaMemcpyAsync(save_cost.p, j->costs.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            MC_CUDA_TRY(cudaMemcpyAsync(found_dev.p, found.data(), nf * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            for (uint32_t q = 0; q < nf; ++q)
                MC_CUDA_TRY(cudaMemcpyAsync(Cs.p + uint64_t(q) * d, j->C.p + uint64_t(found[q]) * d, d * sizeof(float),
                                            cudaMemcpyDeviceToDevice, st));
            const uint32_t k_all = j->k;
            j->k = nf;
            const int rc = job_assign_with(j, Cs.p, j->psum, false);
            j->k = k_all;
            MC_TRY(rc);
            k_merge_restarted<<<unsigned(umin64((n + 255) / 256, 4096)), 256, 0, st>>>(n, found_dev.p, save_asn.p,
                                                                                     save_cost.p, j->asn.p, j->costs.p),
                note_launch();
            MC_CUDA_TRY(cudaGetLastError());
            MC_TRY(sync(st));  // host vectors above go out of scope
        }
        {
            DetInput in{j->w.p ? DET_F64_W : DET_F64, j->costs.p, nullptr, j->w.p, n};
            MC_TRY(launch_det_sum(in, j->det_tmp.p, j->scal.p, st));
            MC_CUDA_TRY(cudaMemcpyAsync(&cost, j->scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
        }
        if (iternum == 0) {
            initcost = bestcost = cost;
        } else if (cost < bestcost) {
            bestcost = cost;
            MC_CUDA_TRY(cudaMemcpyAsync(best_centers, j->C.p, cbytes, cudaMemcpyDefault, st));
        }
        if (++iternum > rounds) break;
        mc_sampler *smp = nullptr;
        MC_TRY(mc_sampler_create(j->ctx, n, k, k, j->costs.p, 1, j->asn.p, j->w.p ? wf.p : nullptr, method, alpha, &smp));
        std::unique_ptr<mc_sampler, int (*)(mc_sampler *)> sguard(smp, mc_sampler_destroy);
        for (uint64_t jj = 0; jj < calc_cost_freq; ++jj) {
            const uint64_t sseed = uint64_t(uniform_at(j->seed, counter++) * 9007199254740992.0);
            MC_TRY(mc_sampler_sample(smp, m, sseed, 1, cw_f.data(), cidx.data()));
            for (uint64_t q = 0; q < m; ++q) {
                rows32[q] = uint32_t(cidx[q]);
                cw[q] = j->w.p ? double(cw_f[q]) * wrow[cidx[q]] : double(cw_f[q]);
            }
            MC_TRY(rows_dev.alloc(m, st));
            MC_CUDA_TRY(cudaMemcpyAsync(rows_dev.p, rows32.data(), m * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            SubRows sub;
            mc_matrix subm;
            MC_TRY(gather_job_rows(j, rows_dev.p, m, sub, &subm));
            DBuf<uint32_t> sasn;
            DBuf<double> scost, sw;
            MC_TRY(sasn.alloc(m, st));
            MC_TRY(scost.alloc(m, st));
            MC_TRY(sw.alloc(m, st));
            MC_CUDA_TRY(cudaMemcpyAsync(sw.p, cw.data(), m * sizeof(double), cudaMemcpyHostToDevice, st));
            double ic = 0, fc = 0;
            uint64_t it = 0;
            const uint64_t subiter = 1 + (iternum < 2 ? 2 : 0);
            MC_TRY(mc_hcluster(j->ctx, &subm, j->C.p, k, j->msr, j->prior, sw.p, 1e-3, subiter, m, j->precision,
                               j->C.p, sasn.p, scost.p, &ic, &fc, &it));
            MC_TRY(sync(st));
        }
    }
    if (initcost_out) *initcost_out = initcost;
    if (finalcost_out) *finalcost_out = bestcost;
    if (numiter_out) *numiter_out = iternum;
    return sync(st);
}

}  // namespace

extern "C" {

int mc_hcluster_coreset(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr,
                        double prior, const double *weights, uint64_t mbsize, uint64_t maxiter, uint64_t ncheckins,
                        uint64_t reseed_count, uint64_t seed, int precision, float *centers_out, uint32_t *asn,
                        double *costs, double *initcost, double *finalcost, uint64_t *numiter) {
    if (!centers_out) return fail(MC_EINVAL, "centers_out is null");
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, X, centers_in, k, msr, prior, weights, precision, seed, &j));
    std::unique_ptr<mc_job, int (*)(mc_job *)> guard(j, mc_job_destroy);
    if (ncheckins == 0) ncheckins = 10;
    const uint64_t freq = (maxiter + ncheckins - 1) / ncheckins;  // pycluster.h:34-38
    DBuf<float> best;
    MC_TRY(best.alloc(uint64_t(k) * j->M.d, j->st));
    MC_TRY(job_coreset_minibatch(j, mbsize, maxiter, freq, reseed_count, best.p, initcost, finalcost, numiter));
    // the best centers; assignments and costs of the last exhaustive pass
    MC_TRY(mc_job_read(j, nullptr, asn, costs));
    MC_CUDA_TRY(cudaMemcpyAsync(centers_out, best.p, uint64_t(k) * j->M.d * sizeof(float), cudaMemcpyDefault, j->st));
    return sync(j->st);
}

int mc_scluster(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr, double prior,
                const double *weights, double temp, uint64_t maxiter, double eps, float *centers_out,
                float *costs_out, float *asn_out, double *initcost_out, double *finalcost_out, uint64_t *numiter_out) {
    if (!ctx || !X || !centers_in) return fail(MC_EINVAL, "null argument");
    // the reference's weighted L1 median over CSR rows raises (util/csc.h:835)
    if (msr == L1 && X->kind != MC_DENSE_F32)
        return fail(MC_EUNSUPPORTED, "Not implemented: weighted L1 median for CSparseMatrix");
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, X, centers_in, k, msr, prior, weights, MC_FP32, 1, &j));
    std::unique_ptr<mc_job, int (*)(mc_job *)> guard(j, mc_job_destroy);
    cudaStream_t st = j->st;
    const uint64_t n = j->M.n, d = j->M.d;
    const size_t cbytes = uint64_t(k) * d * sizeof(float);
    DBuf<float> costs, asn;
    // chunk partials in batches of at most 256 MB, added in chunk order
    const uint64_t nq_all = (n + kSoftChunk - 1) / kSoftChunk;
    const bool csr = j->M.kind == MC_CSR_F32;
    const uint64_t per_chunk = (csr ? 16ull : 8ull) * k * d + 8ull * k;
    const uint64_t batch = std::max<uint64_t>(1, std::min<uint64_t>(nq_all, (256ull << 20) / per_chunk));
    DBuf<double> rowval, snum, sden, acc_num, acc_den;
    DBuf<float> sbuf, ebuf;
    if (csr) {
        MC_TRY(sbuf.alloc(batch * k * d, st));
        MC_TRY(ebuf.alloc(batch * k * d, st));
    }
    MC_TRY(snum.alloc(batch * k * d, st));
    MC_TRY(sden.alloc(batch * k, st));
    MC_TRY(acc_num.alloc(uint64_t(k) * d, st));
    MC_TRY(acc_den.alloc(k, st));
    MC_TRY(costs.alloc(n * k, st));
    MC_TRY(asn.alloc(n * k, st));
    MC_TRY(rowval.alloc(n, st));
    DistOut o;
    o.dmat = costs.p;
    o.ldm = k;
    o.dmode = 1;
    // centers_cpy evolves in Cw; accepted centers in C
    MC_CUDA_TRY(cudaMemcpyAsync(j->Cw.p, j->C.p, cbytes, cudaMemcpyDeviceToDevice, st));
    MC_TRY(job_assign_with(j, j->Cw.p, j->psum, true, &o));
    double cost = std::numeric_limits<double>::max(), initcost = -1.0;
    uint64_t iternum = 0;
    for (;;) {
        const double oldcost = cost;
        k_soft_rows<<<unsigned((n + 255) / 256), 256, 0, st>>>(costs.p, n, k, float(temp), asn.p, rowval.p),
            note_launch();
        DetInput in{j->w.p ? DET_F64_W : DET_F64, rowval.p, nullptr, j->w.p, n};
        MC_TRY(launch_det_sum(in, j->det_tmp.p, j->scal.p, st));
        MC_CUDA_TRY(cudaMemsetAsync(acc_num.p, 0, uint64_t(k) * d * sizeof(double), st));
        MC_CUDA_TRY(cudaMemsetAsync(acc_den.p, 0, uint64_t(k) * sizeof(double), st));
        if (msr == L1)
            k_soft_l1_centers<<<dim3(k, unsigned((d + 31) / 32)), 256, 0, st>>>(j->M.X, n, d, asn.p, k, j->w.p, j->Cw.p),
                note_launch();
        for (uint64_t q0 = 0; msr != L1 && q0 < nq_all; q0 += batch) {
            const uint64_t nq = umin64(batch, nq_all - q0), r0 = q0 * kSoftChunk;
            if (csr) {
                MC_CUDA_TRY(cudaMemsetAsync(sbuf.p, 0, nq * k * d * sizeof(float), st));
                MC_CUDA_TRY(cudaMemsetAsync(ebuf.p, 0, nq * k * d * sizeof(float), st));
                k_soft_center_chunks_csr<<<dim3(unsigned(nq), k), 256, 0, st>>>(
                    j->M.vals, j->M.idx, j->M.indptr + r0, umin64(n - r0, nq * kSoftChunk), d, asn.p + r0 * k, k,
                    j->w.p ? j->w.p + r0 : nullptr, sbuf.p, ebuf.p, snum.p, sden.p), note_launch();
            } else {
                k_soft_center_chunks<<<dim3(unsigned(nq), k), unsigned(umin64(d, 128)), 0, st>>>(
                    j->M.X + r0 * d, umin64(n - r0, nq * kSoftChunk), d, asn.p + r0 * k, k,
                    j->w.p ? j->w.p + r0 : nullptr, snum.p, sden.p), note_launch();
            }
            k_soft_center_accumulate<<<dim3(unsigned((d + 127) / 128), k), 128, 0, st>>>(snum.p, sden.p, nq, k, d,
                                                                                         acc_num.p, acc_den.p),
                note_launch();
        }
        if (msr != L1)
            k_soft_center_finalize<<<dim3(unsigned((d + 127) / 128), k), 128, 0, st>>>(acc_num.p, acc_den.p, k, d,
                                                                                       j->Cw.p), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        MC_TRY(job_assign_with(j, j->Cw.p, j->psum, true, &o));
        MC_CUDA_TRY(cudaMemcpyAsync(&cost, j->scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        MC_TRY(sync(st));
        if (initcost < 0) initcost = cost;
        if (oldcost >= cost) MC_CUDA_TRY(cudaMemcpyAsync(j->C.p, j->Cw.p, cbytes, cudaMemcpyDeviceToDevice, st));
        if (oldcost - cost <= eps * std::max(oldcost, cost) || ++iternum == maxiter) break;
    }
    MC_TRY(copy_out(centers_out, j->C.p, uint64_t(k) * d, st));
    MC_TRY(copy_out(costs_out, costs.p, n * k, st));
    MC_TRY(copy_out(asn_out, asn.p, n * k, st));
    MC_TRY(sync(st));
    if (initcost_out) *initcost_out = initcost;
    if (finalcost_out) *finalcost_out = cost;
    if (numiter_out) *numiter_out = iternum;
    return MC_OK;
}

int mc_job_read(mc_job *j, float *centers, uint32_t *asn, double *costs) {
    if (!j) return fail(MC_EINVAL, "job is null");
    MC_TRY(copy_out(centers, j->C.p, uint64_t(j->k) * j->M.d, j->st));
    MC_TRY(copy_out(asn, j->asn.p, j->M.n, j->st));
    MC_TRY(copy_out(costs, j->costs.p, j->M.n, j->st));
    MC_TRY(sync(j->st));
    return MC_OK;
}

}  // extern "C"

namespace {
__global__ void k_costs_to_f32(const double *__restrict__ c, uint64_t n, float *out) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        out[i] = float(c[i]);  // round to nearest, as a float32 cast of the FP64 costs
}
}  // namespace

extern "C" {

int mc_job_read_f32(mc_job *j, float *centers, uint32_t *asn, float *costs) {
    if (!j) return fail(MC_EINVAL, "job is null");
    MC_TRY(copy_out(centers, j->C.p, uint64_t(j->k) * j->M.d, j->st));
    MC_TRY(copy_out(asn, j->asn.p, j->M.n, j->st));
    if (costs && j->M.n) {
        MC_TRY(j->costs32.alloc(j->M.n, j->st));
        k_costs_to_f32<<<unsigned(umin64((j->M.n + 255) / 256, uint64_t(j->ctx->sms) * 8)), 256, 0, j->st>>>(
            j->costs.p, j->M.n, j->costs32.p), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        MC_TRY(copy_out(costs, j->costs32.p, j->M.n, j->st));
    }
    MC_TRY(sync(j->st));
    return MC_OK;
}

int mc_job_recheck_count(mc_job *j, uint64_t *count) {
    if (!j || !count) return fail(MC_EINVAL, "null argument");
    *count = j->last_recheck;
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// one-shot entry points
// ------------------------------------------------------------------------------------
int mc_assign(mc_context *ctx, const mc_matrix *X, const float *centers, uint32_t k, int msr, double prior,
              int precision, uint32_t *asn, double *costs) {
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, X, centers, k, msr, prior, nullptr, precision, 0, &j));
    std::unique_ptr<mc_job> guard(j);
    MC_TRY(mc_job_assign(j));
    return mc_job_read(j, nullptr, asn, costs);
}

// ------------------------------------------------------------------------------------
// pairwise distance matrices (python/pycmp.cpp:15-300, python/pyarrcmp.cpp:52-144)
// ------------------------------------------------------------------------------------
__global__ void k_densify_csr(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                              const uint64_t *__restrict__ indptr, uint64_t n, uint64_t d, float *out) {
    for (uint64_t r = blockIdx.x; r < n; r += gridDim.x) {
        float *dst = out + r * d;
        for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) dst[j] = 0.f;
        __syncthreads();
        for (uint64_t p = indptr[r] + threadIdx.x; p < indptr[r + 1]; p += blockDim.x) dst[idx[p]] = vals[p];
        __syncthreads();
    }
}

// the rows of X as a dense device matrix: borrowed when X is dense on the device, else a copy
static int dense_rows(const mc_matrix *X, cudaStream_t st, int sms, DevMatrix &M, DBuf<float> &own,
                      const float **out) {
    MC_TRY(M.load(X, st));
    if (M.kind == MC_DENSE_F32) {
        *out = M.X;
        return MC_OK;
    }
    MC_TRY(own.alloc(M.n * M.d, st));
    k_densify_csr<<<unsigned(umin64(M.n, uint64_t(sms) * 8)), 256, 0, st>>>(M.vals, M.idx, M.indptr, M.n, M.d, own.p),
        note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    *out = own.p;
    return MC_OK;
}

// one exact FP32 assignment pass of `rows` against `centers` writing every pair's distance
static int distance_pass(mc_context *ctx, const mc_matrix *rows, const float *centers, uint64_t k, int msr,
                         double prior, float *out, uint64_t out_count, uint64_t ldm, int dmode) {
    if (k == 0 || k >= (1ull << 32)) return fail(MC_EINVAL, "center count out of range");
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, rows, centers, uint32_t(k), msr, prior, nullptr, MC_FP32, 1, &j));
    std::unique_ptr<mc_job, int (*)(mc_job *)> guard(j, mc_job_destroy);
    DBuf<float> dbuf;
    float *D = out;
    if (!is_device_ptr(out)) {
        MC_TRY(dbuf.alloc(out_count, j->st));
        D = dbuf.p;
    }
    DistOut o;
    o.dmat = D;
    o.ldm = ldm;
    o.dmode = dmode;
    MC_TRY(job_assign_with(j, j->C.p, j->psum, true, &o));
    if (D != out) MC_CUDA_TRY(cudaMemcpyAsync(out, D, out_count * sizeof(float), cudaMemcpyDefault, j->st));
    return sync(j->st);
}

int mc_cmp(mc_context *ctx, const mc_matrix *X, const float *Y, uint64_t m, int msr, double prior, int reverse,
           float *out) {
    if (!ctx || !X || !Y || !out) return fail(MC_EINVAL, "null argument");
    if (m == 0) return fail(MC_EINVAL, "no rows in the second operand");
    if (!measure_supported(msr)) return fail(MC_EUNSUPPORTED, "measure not implemented on this path");
    MC_CUDA_TRY(cudaSetDevice(ctx->device));
    const uint64_t n = X->nrows, d = X->ncols;
    if (!reverse) {
        // out[i][j] = msr(lh = Y[j], rh = X[i]): the rows of X against Y as centers
        return distance_pass(ctx, X, Y, m, msr, prior, out, n * m, m, 1);
    }
    // out[i][j] = msr(lh = X[i], rh = Y[j]): the rows of Y against X (densified) as centers
    DevMatrix M;
    DBuf<float> own;
    const float *Xd = nullptr;
    MC_TRY(dense_rows(X, ctx->stream, ctx->sms, M, own, &Xd));
    mc_matrix Ym{MC_DENSE_F32, 0, m, d, Y, nullptr, nullptr, 0};
    return distance_pass(ctx, &Ym, Xd, n, msr, prior, out, n * m, m, 2);
}

int mc_pcmp(mc_context *ctx, const mc_matrix *X, int msr, double prior, float *out) {
    if (!ctx || !X || !out) return fail(MC_EINVAL, "null argument");
    if (!measure_supported(msr)) return fail(MC_EUNSUPPORTED, "measure not implemented on this path");
    MC_CUDA_TRY(cudaSetDevice(ctx->device));
    const uint64_t n = X->nrows;
    if (n < 2) return MC_OK;
    // condensed entry (i < j) = msr(lh = row i, rh = row j): rows of X against X as centers
    DevMatrix M;
    DBuf<float> own;
    const float *Xd = nullptr;
    MC_TRY(dense_rows(X, ctx->stream, ctx->sms, M, own, &Xd));
    return distance_pass(ctx, X, Xd, n, msr, prior, out, n * (n - 1) / 2, n, 3);
}

int mc_hcluster(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr, double prior,
                const double *weights, double eps, uint64_t maxiter, uint64_t seed, int precision,
                float *centers_out, uint32_t *asn, double *costs, double *initcost, double *finalcost,
                uint64_t *numiter) {
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, X, centers_in, k, msr, prior, weights, precision, seed, &j));
    std::unique_ptr<mc_job> guard(j);
    MC_TRY(mc_job_run(j, eps, maxiter, initcost, finalcost, numiter));
    return mc_job_read(j, centers_out, asn, costs);
}

int mc_hcluster_f32(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr,
                    double prior, const double *weights, double eps, uint64_t maxiter, uint64_t seed, int precision,
                    float *centers_out, uint32_t *asn, float *costs, double *initcost, double *finalcost,
                    uint64_t *numiter) {
    mc_job *j = nullptr;
    MC_TRY(mc_job_create(ctx, X, centers_in, k, msr, prior, weights, precision, seed, &j));
    std::unique_ptr<mc_job> guard(j);
    MC_TRY(mc_job_run(j, eps, maxiter, initcost, finalcost, numiter));
    return mc_job_read_f32(j, centers_out, asn, costs);
}

}  // extern "C"

namespace {

// ------------------------------------------------------------------------------------
// localsearch++ rounds after the seeding (localsearchpp_rounds, optim/lsearchpp.h:21-123).
// M[i][j] is the reference's oracle(i, center j) = msr(lh = row i, rh = center row j) (its
// kmeans++ oracle takes the first index as the center), distances the row minima of M.
// Each round draws a row sel (from the distances; with weights, from the previous round's
// new costs times the weights, as the reference does, zeros before the first round), takes
// new[i] = msr(lh = row sel, rh = row i); a row with new[i] > dist[i] charges
// top2 - top1 of its M row to its top1 center (none on a tie), any other row adds
// dist[i] - new[i] to the gain; the center with the smallest charge (first on ties) is
// swapped for sel when charge - gain < 0.  Per-center charges and the gain are canonical
// FP64 sums; the reference adds them with atomics.  Uniforms U(seed ^ 0x4C53505053454544, r).
// ------------------------------------------------------------------------------------
constexpr uint64_t kLsppStream = 0x4C53505053454544ull;

__global__ void k_lspp_rowmin(const float *__restrict__ M, uint64_t n, uint32_t k, double *dist, uint32_t *asn) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        const float *r = M + i * k;
        float b = r[0];
        uint32_t bj = 0;
        for (uint32_t j = 1; j < k; ++j)
            if (r[j] < b) { b = r[j]; bj = j; }
        dist[i] = double(b);
        if (asn) asn[i] = bj;
    }
}

__global__ void k_lspp_rows(const float *__restrict__ M, uint64_t n, uint32_t k, const double *__restrict__ dist,
                            const double *__restrict__ nc, uint32_t *key, double *charge, double *gterm) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        key[i] = 0xffffffffu;
        charge[i] = 0.0;
        gterm[i] = 0.0;
        if (nc[i] > dist[i]) {
            const float *r = M + i * k;
            double v1 = r[0], v2 = r[1];
            uint32_t j1 = 0, j2 = 1;
            if (v2 < v1) { const double tv = v1; v1 = v2; v2 = tv; const uint32_t tj = j1; j1 = j2; j2 = tj; }
            for (uint32_t j = 2; j < k; ++j) {
                const double v = r[j];
                if (v < v2) {
                    if (v < v1) { v2 = v1; j2 = j1; v1 = v; j1 = j; }
                    else { v2 = v; j2 = j; }
                }
            }
            (void)j2;
            if (v1 != v2) {
                key[i] = j1;
                charge[i] = v2 - v1;
            }
        } else {
            gterm[i] = dist[i] - nc[i];
        }
    }
}

__global__ void k_lspp_set_col(float *M, uint64_t n, uint32_t k, uint32_t col, const double *__restrict__ nc) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        M[i * k + col] = float(nc[i]);
}

int run_lspp(mc_context *ctx, const mc_matrix *X, const KmppArgs &a, uint32_t k, int msr, double prior,
             uint64_t rounds, uint64_t seed, uint32_t *ids, uint32_t *asn, double *dist, double *det_tmp,
             cudaStream_t st) {
    const uint64_t n = a.n, d = a.d;
    if (k < 2) return fail(MC_EINVAL, "localsearch++ needs k >= 2");
    DBuf<float> C, M;
    DBuf<double> nc, charge, gterm, scal;
    DBuf<uint32_t> key, ids_scratch;
    DBuf<uint64_t> sel_dev;
    MC_TRY(C.alloc(uint64_t(k) * d, st));
    MC_TRY(M.alloc(n * k, st));
    MC_TRY(nc.alloc(n, st));
    MC_TRY(charge.alloc(n, st));
    MC_TRY(gterm.alloc(n, st));
    MC_TRY(scal.alloc(1, st));
    MC_TRY(key.alloc(n, st));
    MC_TRY(ids_scratch.alloc(1, st));
    MC_TRY(sel_dev.alloc(1, st));
    MC_TRY(launch_gather_rows(a.csr, a.X, a.vals, a.idx, a.indptr, d, ids, k, C.p, st));
    MC_TRY(sync(st));
    MC_TRY(mc_cmp(ctx, X, C.p, k, msr, prior, 1, M.p));
    const unsigned g = unsigned(umin64((n + 255) / 256, 4096));
    k_lspp_rowmin<<<g, 256, 0, st>>>(M.p, n, k, dist, nullptr), note_launch();
    MC_CUDA_TRY(cudaMemsetAsync(nc.p, 0, n * sizeof(double), st));
    std::vector<uint32_t> hids(k);
    MC_CUDA_TRY(cudaMemcpyAsync(hids.data(), ids, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    MC_TRY(sync(st));
    KmppArgs b = a;
    b.center_ids = ids_scratch.p;
    for (uint64_t r = 0; r < rounds; ++r) {
        const double u = uniform_at(seed ^ kLsppStream, r);
        DetInput din{a.w ? DET_F64_W : DET_F64, a.w ? nc.p : dist, nullptr, a.w, n};
        MC_TRY(launch_det_draw(din, det_tmp, nullptr, u, 0, nullptr, sel_dev.p, st));
        MC_TRY(kmpp_distances_to(b, sel_dev.p, nc.p, ctx->sms, st));
        k_lspp_rows<<<g, 256, 0, st>>>(M.p, n, k, dist, nc.p, key.p, charge.p, gterm.p), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        std::vector<double> cc(k);
        double gain = 0.0;
        {
            DetInput gi{DET_F64, gterm.p, nullptr, nullptr, n};
            MC_TRY(launch_det_sum(gi, det_tmp, scal.p, st));
            MC_CUDA_TRY(cudaMemcpyAsync(&gain, scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
        }
        for (uint32_t c = 0; c < k; ++c) {
            DetInput ci{DET_F64_KEY, charge.p, nullptr, nullptr, n, key.p, c};
            MC_TRY(launch_det_sum(ci, det_tmp, scal.p, st));
            MC_CUDA_TRY(cudaMemcpyAsync(&cc[c], scal.p, sizeof(double), cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
        }
        uint32_t am = 0;
        for (uint32_t c = 1; c < k; ++c)
            if (cc[c] < cc[am]) am = c;
        if (cc[am] - gain < 0.0) {
            uint64_t sel = 0;
            MC_CUDA_TRY(cudaMemcpyAsync(&sel, sel_dev.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            MC_TRY(sync(st));
            hids[am] = uint32_t(sel);
            k_lspp_set_col<<<g, 256, 0, st>>>(M.p, n, k, am, nc.p), note_launch();
            k_lspp_rowmin<<<g, 256, 0, st>>>(M.p, n, k, dist, nullptr), note_launch();
        }
    }
    MC_CUDA_TRY(cudaMemcpyAsync(ids, hids.data(), k * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    k_lspp_rowmin<<<g, 256, 0, st>>>(M.p, n, k, dist, asn), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return sync(st);
}

}  // namespace

static int kmeanspp_impl(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior, const double *weights,
                         const double *uniforms, uint32_t local_trials, uint64_t seed, uint32_t *center_ids,
                         uint32_t *asn, double *costs, uint64_t lspp_rounds = 0) {
    if (!ctx) return fail(MC_EINVAL, "ctx is null");
    if (!measure_supported(msr)) return fail(MC_EUNSUPPORTED, "measure not implemented on this path");
    if (!uniforms && local_trials <= 1) return fail(MC_EINVAL, "uniforms is null");
    MC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    DevMatrix M;
    MC_TRY(M.load(X, st));
    const uint64_t n = M.n, d = M.d;
    if (k == 0) return fail(MC_EINVAL, "k must be positive");
    if (k > n) k = uint32_t(n);
    DBuf<double> rowsum, dist, u, w, tmp;
    DBuf<float> cbuf, rn, ct, gval;
    DBuf<double> cconst;
    DBuf<uint32_t> grp;
    DBuf<uint32_t> asnb, ids;
    DBuf<uint64_t> newc;
    MC_TRY(rowsum.alloc(n, st));
    MC_TRY(dist.alloc(n, st));
    MC_TRY(u.alloc(k, st));
    MC_TRY(tmp.alloc(det_tmp_size(n), st));
    MC_TRY(cbuf.alloc(d, st));
    MC_TRY(asnb.alloc(n, st));
    MC_TRY(ids.alloc(k, st));
    MC_TRY(newc.alloc(1, st));
    if (local_trials <= 1) MC_CUDA_TRY(cudaMemcpyAsync(u.p, uniforms, k * sizeof(double), cudaMemcpyDefault, st));
    if (weights) {
        MC_TRY(w.alloc(n, st));
        MC_CUDA_TRY(cudaMemcpyAsync(w.p, weights, n * sizeof(double), cudaMemcpyDefault, st));
    }
    if (M.kind != MC_DENSE_F32) MC_TRY(launch_row_sums_csr(M.vals, M.indptr, n, rowsum.p, st));
    else if (msr != SQRL2) MC_TRY(launch_row_sums_dense(M.X, n, d, rowsum.p, nullptr, st));  // SQRL2 reads none
    KmppArgs a;
    a.msr = msr;
    a.csr = M.kind == MC_CSR_F32;
    a.n = n;
    a.d = d;
    a.k = k;
    a.X = M.X;
    a.vals = M.vals;
    a.idx = M.idx;
    a.indptr = M.indptr;
    a.rowsum = rowsum.p;
    a.w = w.p;
    a.prior = prior;
    a.prior_sum = prior * double(d);
    a.cbuf = cbuf.p;
    uint32_t ngrp = 0;
    if (a.csr && msr == JSD) MC_TRY(build_rinc_groups(rowsum.p, n, d, M.nnz, float(prior), st, grp, gval, ngrp));
    if (a.csr && kmpp_csr_nnz_path(n, d, M.nnz) && (msr != JSD || ngrp)) {
        MC_TRY(ct.alloc(d, st));
        MC_TRY(cconst.alloc(msr == JSD ? ngrp : 2, st));
        a.ct = ct.p;
        a.cconst = cconst.p;
        a.grp = grp.p;
        a.gval = gval.p;
        a.ngrp = ngrp;
    }
    a.dist = dist.p;
    a.asn = asnb.p;
    a.center_ids = ids.p;
    a.newc = newc.p;
    if (local_trials > 1) MC_TRY(run_kmeanspp_greedy(a, local_trials, seed, tmp.p, ctx->sms, st));
    else MC_TRY(run_kmeanspp(a, u.p, tmp.p, ctx->sms, st));
    if (lspp_rounds) MC_TRY(run_lspp(ctx, X, a, k, msr, prior, lspp_rounds, seed, ids.p, asnb.p, dist.p, tmp.p, st));
    MC_TRY(copy_out(center_ids, ids.p, k, st));
    MC_TRY(copy_out(asn, asnb.p, n, st));
    MC_TRY(copy_out(costs, dist.p, n, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" {

int mc_kmeanspp(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior, const double *weights,
                const double *uniforms, uint32_t *center_ids, uint32_t *asn, double *costs) {
    return kmeanspp_impl(ctx, X, k, msr, prior, weights, uniforms, 1, 0, center_ids, asn, costs);
}

int mc_kmeanspp_ex(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior, const double *weights,
                   uint32_t n_local_trials, uint64_t lspp_rounds, uint64_t seed, uint32_t *center_ids, uint32_t *asn,
                   double *costs) {
    if (n_local_trials == 0) return fail(MC_EINVAL, "n_local_trials must be positive");
    if (n_local_trials == 1) {
        std::vector<double> u(k);
        for (uint32_t i = 0; i < k; ++i) u[i] = uniform_at(seed, i);
        return kmeanspp_impl(ctx, X, k, msr, prior, weights, u.data(), 1, seed, center_ids, asn, costs, lspp_rounds);
    }
    return kmeanspp_impl(ctx, X, k, msr, prior, weights, nullptr, n_local_trials, seed, center_ids, asn, costs,
                         lspp_rounds);
}

int mc_kmeanspp_greedy(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior, const double *weights,
                       uint32_t n_local_trials, uint64_t seed, uint32_t *center_ids, uint32_t *asn, double *costs) {
    if (n_local_trials == 0) return fail(MC_EINVAL, "n_local_trials must be positive");
    if (n_local_trials == 1) {
        std::vector<double> u(k);
        for (uint32_t i = 0; i < k; ++i) u[i] = uniform_at(seed, i);
        return kmeanspp_impl(ctx, X, k, msr, prior, weights, u.data(), 1, 0, center_ids, asn, costs);
    }
    return kmeanspp_impl(ctx, X, k, msr, prior, weights, nullptr, n_local_trials, seed, center_ids, asn, costs);
}

// ------------------------------------------------------------------------------------
// coreset sampler
// ------------------------------------------------------------------------------------
__global__ void k_widen_costs(const float *c, uint64_t n, double *out) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x))
        out[i] = double(c[i]);
}

int mc_sampler_create(mc_context *ctx, uint64_t np, uint64_t ncenters, uint64_t k, const void *costs, int costs_f64,
                      const uint32_t *asn, const float *weights, int method, double alpha_est, mc_sampler **out) {
    if (!ctx || !out) return fail(MC_EINVAL, "null context or output");
    if (np == 0 || ncenters == 0 || !costs || !asn) return fail(MC_EINVAL, "empty input");
    if (method < MC_BFL || method > MC_LBK) return fail(MC_EINVAL, "Invalid SensitivityMethod");
    if (np >= (1ull << 32)) return fail(MC_EINVAL, "more than 2^32-1 points");
    MC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    std::unique_ptr<mc_sampler> s(new mc_sampler());
    s->ctx = ctx;
    s->np = np;
    s->nc = ncenters;
    s->k = k ? k : ncenters;
    s->method = method;
    MC_TRY(s->cost_d.alloc(np, st));
    if (costs_f64) {
        MC_CUDA_TRY(cudaMemcpyAsync(s->cost_d.p, costs, np * sizeof(double), cudaMemcpyDefault, st));
    } else {
        DBuf<float> cf;
        const float *cp = nullptr;
        MC_TRY(stage((const float *)costs, np, cf, cp, st));
        k_widen_costs<<<unsigned(umin64((np + 255) / 256, 65535)), 256, 0, st>>>(cp, np, s->cost_d.p), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        MC_TRY(sync(st));
    }
    MC_TRY(s->asn.alloc(np, st));
    MC_CUDA_TRY(cudaMemcpyAsync(s->asn.p, asn, np * sizeof(uint32_t), cudaMemcpyDefault, st));
    if (weights) {
        MC_TRY(s->wf.alloc(np, st));
        MC_TRY(s->wt_d.alloc(np, st));
        MC_CUDA_TRY(cudaMemcpyAsync(s->wf.p, weights, np * sizeof(float), cudaMemcpyDefault, st));
        MC_TRY(launch_to_double(s->wf.p, np, s->wt_d.p, st));
    }
    MC_TRY(s->probs.alloc(np, st));
    SensInput in;
    in.method = method;
    in.n = np;
    in.nc = uint32_t(ncenters);
    in.k = s->k;
    in.alpha_est = alpha_est;
    in.cost = s->cost_d.p;
    in.wt = weights ? s->wt_d.p : nullptr;
    in.asn = s->asn.p;
    in.probs = s->probs.p;
    MC_TRY(compute_sensitivities(in, s->sw, st, ctx->sms));
    MC_TRY(s->prob_tab.alloc(np, st));
    MC_TRY(s->alias.alloc(np, st));
    MC_TRY(build_alias(s->probs.p, np, s->prob_tab.p, s->alias.p, s->aw, st, ctx->sms));
    MC_TRY(sync(st));
    *out = s.release();
    return MC_OK;
}

// A sampler over given probabilities (the state CoresetSampler::read restores,
// coreset.h:306-338): the alias table is rebuilt from them; sampling is the plain (non-FL)
// form.  weights: optional float32 per point.
int mc_sampler_from_probs(mc_context *ctx, uint64_t np, const float *probs, const float *weights, mc_sampler **out) {
    if (!ctx || !out || !probs) return fail(MC_EINVAL, "null argument");
    if (np == 0) return fail(MC_EINVAL, "empty input");
    if (np >= (1ull << 32)) return fail(MC_EINVAL, "more than 2^32-1 points");
    MC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    std::unique_ptr<mc_sampler> s(new mc_sampler());
    s->ctx = ctx;
    s->np = np;
    s->method = MC_BFL;
    MC_TRY(s->probs.alloc(np, st));
    MC_CUDA_TRY(cudaMemcpyAsync(s->probs.p, probs, np * sizeof(float), cudaMemcpyDefault, st));
    if (weights) {
        MC_TRY(s->wf.alloc(np, st));
        MC_TRY(s->wt_d.alloc(np, st));
        MC_CUDA_TRY(cudaMemcpyAsync(s->wf.p, weights, np * sizeof(float), cudaMemcpyDefault, st));
        MC_TRY(launch_to_double(s->wf.p, np, s->wt_d.p, st));
    }
    MC_TRY(s->prob_tab.alloc(np, st));
    MC_TRY(s->alias.alloc(np, st));
    MC_TRY(build_alias(s->probs.p, np, s->prob_tab.p, s->alias.p, s->aw, st, ctx->sms));
    MC_TRY(sync(st));
    *out = s.release();
    return MC_OK;
}

int mc_sampler_info(mc_sampler *s, uint64_t *np, int *method, int *has_weights) {
    if (!s) return fail(MC_EINVAL, "sampler is null");
    if (np) *np = s->np;
    if (method) *method = s->method;
    if (has_weights) *has_weights = s->wf.p ? 1 : 0;
    return MC_OK;
}

int mc_sampler_weights(mc_sampler *s, float *weights) {
    if (!s || !weights) return fail(MC_EINVAL, "null argument");
    if (!s->wf.p) return fail(MC_EINVAL, "the sampler has no weights");
    MC_TRY(copy_out(weights, s->wf.p, s->np, s->ctx->stream));
    return sync(s->ctx->stream);
}

int mc_sampler_destroy(mc_sampler *s) {
    if (!s) return MC_OK;
    cudaStreamSynchronize(s->ctx->stream);
    delete s;
    return MC_OK;
}

int mc_sampler_probs(mc_sampler *s, float *probs) {
    if (!s || !probs) return fail(MC_EINVAL, "null argument");
    MC_TRY(copy_out(probs, s->probs.p, s->np, s->ctx->stream));
    return sync(s->ctx->stream);
}

int mc_sampler_alias(mc_sampler *s, double *prob_table, uint32_t *alias_table) {
    if (!s) return fail(MC_EINVAL, "null argument");
    MC_TRY(copy_out(prob_table, s->prob_tab.p, s->np, s->ctx->stream));
    MC_TRY(copy_out(alias_table, s->alias.p, s->np, s->ctx->stream));
    return sync(s->ctx->stream);
}

int mc_sampler_sample(mc_sampler *s, uint64_t m, uint64_t seed, int unique, float *weights, uint64_t *indices) {
    if (!s || !weights || !indices) return fail(MC_EINVAL, "null argument");
    if (m == 0) return MC_OK;
    cudaStream_t st = s->ctx->stream;
    DBuf<float> wo;
    DBuf<uint64_t> io;
    MC_TRY(wo.alloc(m, st));
    MC_TRY(io.alloc(m, st));
    SampleArgs a;
    a.np = s->np;
    a.m = m;
    a.direct = (s->method == MC_FL) ? (m > s->nc ? m - s->nc : 0) : m;
    a.seed = seed;
    a.unique = unique;
    a.probs = s->probs.p;
    a.prob_tab = s->prob_tab.p;
    a.alias_tab = s->alias.p;
    a.wf = s->wf.p;
    a.w_out = wo.p;
    a.idx_out = io.p;
    MC_TRY(run_sample(a, s->smp, st, s->ctx->sms));
    MC_TRY(copy_out(weights, wo.p, m, st));
    MC_TRY(copy_out(indices, io.p, m, st));
    return sync(st);
}

}  // extern "C"
