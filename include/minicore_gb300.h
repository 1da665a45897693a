/*
 * minicore_gb300 — C ABI of the GB300-native clustering hot path.
 *
 * Every entry point here replaces one call the reference makes on its hot path
 * (dnbaker/minicore, paths within that project):
 *
 *   mc_kmeanspp          coresets::kmeanspp            include/minicore/optim/kmeans.h:49-215
 *                        driven by py_kmeanspp_noso(_dense) python/smw.h:179-412
 *   mc_assign            assign_points_hard            include/minicore/clustering/solve.h:234-285
 *                        (per-pair cmp::msr_with_prior include/minicore/dist/applicator.h:1632-1915)
 *   mc_job_lloyd_step    set_centroids_full_mean       include/minicore/clustering/centroid.h:649-779
 *                        + set_center                  centroid.h:81-112 (CSR), 137-178 (dense)
 *   mc_hcluster          perform_hard_clustering       include/minicore/clustering/solve.h:98-175
 *                        driven by cpp_pycluster_from_centers python/pycluster.h:10-63
 *                        (mc_hcluster_f32: the costs as that binding returns them, float32)
 *   mc_sampler_*         CoresetSampler::make_sampler  include/minicore/coreset/coreset.h:386-422
 *                        make_probs_{bfl,fl,vx,lbk}, make_gmm_sampler coreset.h:340-578,
 *                        sample                        coreset.h:625-699
 *   mc_job_* / mc_server_*  resident-state jobs and the continuous-batching server (no
 *                        reference counterpart: the reference runs one call at a time).
 *
 * Conventions
 *  - Every pointer argument may point to host memory or to device memory of the
 *    context's GPU; the library detects which (cudaPointerGetAttributes) and copies as
 *    needed.  Outputs are written in place.
 *  - Calls return an mc_status; mc_last_error() returns a thread-local message for the
 *    last failing call on the calling thread.
 *  - Measures use the reference's numbering (include/minicore/dist/distance.h:24-64).
 *  - Randomness: every draw consumes a uniform in [0,1).  Where an entry point takes a
 *    seed, draw i uses U(seed, i) of the splitmix64 stream that mc_uniforms() produces.
 */
#ifndef MINICORE_GB300_H_
#define MINICORE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mc_status {
    MC_OK = 0,
    MC_EINVAL = 1,       /* invalid argument (reference: std::invalid_argument)        */
    MC_ENOMEM = 2,       /* device allocation failed / admission refused                */
    MC_ETIMEOUT = 3,     /* a bounded device wait gave up                                */
    MC_ECUDA = 4,        /* CUDA runtime error                                           */
    MC_ENAN = 5,         /* NaN center (reference: runtime_error "Unexpected nan in ctr") */
    MC_EUNSUPPORTED = 6, /* measure / option outside the implemented hot path            */
    MC_EBUSY = 7         /* result not ready yet (mc_server_poll)                        */
} mc_status;

typedef enum mc_measure {
    MC_L1 = 0,
    MC_SQRL2 = 2,
    MC_JSD = 4,
    MC_MKL = 5,
    MC_HELLINGER = 6
} mc_measure;

typedef enum mc_precision {
    MC_FP32 = 0, /* exact FP32 CUDA-core distances                                   */
    MC_TF32 = 1, /* SQRL2 dense: tcgen05 TF32 GEMM + FP32 re-check of near ties      */
    MC_BF16 = 2  /* SQRL2 dense: tcgen05 BF16 GEMM + FP32 re-check of near ties      */
} mc_precision;

typedef enum mc_sensitivity {
    MC_BFL = 0, MC_FL = 1, MC_LFKF = 2, MC_VX = 3, MC_LBK = 4
} mc_sensitivity;

typedef enum mc_matrix_kind { MC_DENSE_F32 = 0, MC_CSR_F32 = 1 } mc_matrix_kind;

/* Dense row-major float32 matrix, or CSR with float32 values, uint32 column indices
 * (ascending within each row) and uint64 row offsets: the zero-copy view the reference's
 * PyCSparseMatrix keeps (python/pycsparse.h:33-70). */
typedef struct mc_matrix {
    int32_t kind;              /* mc_matrix_kind                                */
    int32_t reserved;
    uint64_t nrows, ncols;
    const float *values;       /* dense: nrows*ncols; CSR: nnz                  */
    const uint32_t *indices;   /* CSR only                                      */
    const uint64_t *indptr;    /* CSR only, nrows+1 entries                     */
    uint64_t nnz;              /* CSR only                                      */
} mc_matrix;

typedef struct mc_context mc_context;
typedef struct mc_sampler mc_sampler;
typedef struct mc_job mc_job;
typedef struct mc_server mc_server;

const char *mc_version(void);
const char *mc_last_error(void);
/* Number of CUDA kernels this library has launched in this process (diagnostics). */
uint64_t mc_kernel_launches(void);
/* Test hook for the device-side failure path (no reference counterpart; the reference polls
 * for interrupts on the host, clustering/solve.h:26-30): the next tensor-core assignment
 * pass in this process makes its MMA issuer wait on a barrier that nothing completes.  The
 * wait's bound (about one second) runs out, the kernel drains its copies in flight, frees
 * its tensor memory and returns, and the call reports MC_ETIMEOUT; the context stays
 * usable.  One shot: later passes run normally. */
int mc_test_tc_stall_once(void);
/* Measured logf throughput of `device` (logf results per second, full occupancy, 8
 * independent chains per thread): the compute roof against which the CSR JSD sparse dot
 * (two logf per nonzero and center) is reported.  Diagnostics; no reference counterpart. */
int mc_diag_logf_rate(int device, double *logs_per_s);
/* Phase profiler (diagnostics, off by default): CUDA events around the library's phases
 * (tensor-core passes, exact finalize, FP32/CSR assignment, centroid update, objective).
 * mc_profile_report writes {"phase": {"count": c, "ms": total}, ...} as JSON. */
int mc_profile_enable(int on);
int mc_profile_reset(void);
int mc_profile_report(char *json, uint64_t capacity);

int mc_context_create(int device, mc_context **out);
int mc_context_destroy(mc_context *ctx);
/* Launch on this stream (a cudaStream_t) instead of the context's own stream. */
int mc_context_set_stream(mc_context *ctx, void *cuda_stream);
int mc_context_synchronize(mc_context *ctx);

/* U(seed, offset + i), i < m, into host memory. */
int mc_uniforms(uint64_t seed, uint64_t offset, uint64_t m, double *out);

/* D^2 / k-means++ seeding (kmeans.h:49-215, n_local_trials == 1, no ls++).
 * uniforms: k values; uniforms[0] picks the first center (floor(u*n)), uniforms[c] drives
 * round c.  weights: optional (double, n).  Outputs: center_ids[k], asn[n] (center
 * ordinal), costs[n] (distance to the nearest chosen center). */
int mc_kmeanspp(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior,
                const double *weights, const double *uniforms,
                uint32_t *center_ids, uint32_t *asn, double *costs);
/* Greedy k-means++ (n_local_trials > 1, kmeans.h:79-177; python/pydense.cpp:34-77): the
 * first center is the best of n_local_trials uniform picks; each later round draws
 * n_local_trials candidates from the distances without replacement and keeps the one with
 * the lowest objective.  Candidate 0 extends the current distances; later candidates extend
 * the distances of the first center alone, as the reference does (kmeans.h:140-144).
 * Uniforms U(seed, r), one counter r.  n_local_trials = 1 is mc_kmeanspp with U(seed, i). */
int mc_kmeanspp_greedy(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior,
                       const double *weights, uint32_t n_local_trials, uint64_t seed,
                       uint32_t *center_ids, uint32_t *asn, double *costs);
/* mc_kmeanspp_greedy followed by lspp_rounds of localsearch++ (localsearchpp_rounds,
 * optim/lsearchpp.h:21-123; kmeanspp's lspp argument, kmeans.h:209-212): swaps a center for
 * a D^2-drawn row when that lowers the objective.  Charges and gains are canonical FP64
 * sums; draws use U(seed ^ 0x4C53505053454544, r).  On return costs are the row minima of
 * the reference's lspp matrix (msr(lh = row, rh = center)) and asn their first argmin.
 * lspp_rounds > 0 needs k >= 2. */
int mc_kmeanspp_ex(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior,
                   const double *weights, uint32_t n_local_trials, uint64_t lspp_rounds, uint64_t seed,
                   uint32_t *center_ids, uint32_t *asn, double *costs);

/* One hard assignment pass (solve.h:234-285): asn[i] = argmin_j msr(row i, center j),
 * lowest index on ties; costs[i] = that distance.  centers: dense k x ncols float32. */
int mc_assign(mc_context *ctx, const mc_matrix *X, const float *centers, uint32_t k, int msr,
              double prior, int precision, uint32_t *asn, double *costs);

/* Lloyd / Bregman EM from explicit centers (solve.h:98-175): eps, maxiter and the
 * revert-on-increase rule as in the reference; empty clusters restart by D^2 draws
 * U(seed, r).  weights: optional (double, n).  L1 takes coordinate-wise medians
 * (set_centroids_l1, centroid.h:435-504): dense rows by the sorted median (weighted: the
 * largest-weight row's value, as weighted_median returns), CSR rows by the sparse rule of
 * util/csc.h:829-893; weighted L1 over CSR rows returns MC_EUNSUPPORTED as the reference
 * raises. */
int mc_hcluster(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr,
                double prior, const double *weights, double eps, uint64_t maxiter, uint64_t seed,
                int precision, float *centers_out, uint32_t *asn, double *costs,
                double *initcost, double *finalcost, uint64_t *numiter);
/* mc_hcluster with the costs rounded to float32 on the device, as the reference's Python
 * binding returns them (python/pycluster.h:59, vec2fnp<..., float>): half the bytes to copy
 * back and no host-side conversion. */
int mc_hcluster_f32(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr,
                    double prior, const double *weights, double eps, uint64_t maxiter, uint64_t seed,
                    int precision, float *centers_out, uint32_t *asn, float *costs,
                    double *initcost, double *finalcost, uint64_t *numiter);

/* Pairwise distances (python/pycmp.cpp:15-300, python/pyarrcmp.cpp:52-144), exact FP32,
 * written as float32.  Y: dense m x ncols float32.  reverse == 0: out[i][j] =
 * msr(lh = Y[j], rh = X[i]) (the assignment's roles: Y as centers), reverse != 0:
 * out[i][j] = msr(lh = X[i], rh = Y[j]).  out: nrows x m. */
int mc_cmp(mc_context *ctx, const mc_matrix *X, const float *Y, uint64_t m, int msr, double prior,
           int reverse, float *out);
/* Condensed pairwise distances among the rows of X (pcmp): for i < j, entry
 * i*n - i*(i+1)/2 + j - i - 1 = msr(lh = row i, rh = row j); out holds n*(n-1)/2 floats. */
int mc_pcmp(mc_context *ctx, const mc_matrix *X, int msr, double prior, float *out);

/* Coreset sampler (coreset.h:386-422).  costs: float32 or float64 (costs_f64 != 0);
 * weights: optional float32 (the reference stores them as float). k: the k of LBK's
 * alpha (pass ncenters for the reference default). */
int mc_sampler_create(mc_context *ctx, uint64_t np, uint64_t ncenters, uint64_t k,
                      const void *costs, int costs_f64, const uint32_t *asn, const float *weights,
                      int method, double alpha_est, mc_sampler **out);
/* A sampler over stored probabilities (what CoresetSampler::read restores,
 * coreset.h:306-338): the alias table is rebuilt, sampling is the plain form.  weights:
 * optional float32 per point. */
int mc_sampler_from_probs(mc_context *ctx, uint64_t np, const float *probs, const float *weights,
                          mc_sampler **out);
int mc_sampler_info(mc_sampler *s, uint64_t *np, int *method, int *has_weights);
int mc_sampler_weights(mc_sampler *s, float *weights);   /* MC_EINVAL without weights */
int mc_sampler_destroy(mc_sampler *s);
int mc_sampler_probs(mc_sampler *s, float *probs);
int mc_sampler_alias(mc_sampler *s, double *prob_table, uint32_t *alias_table);
/* m draws (coreset.h:625-699); draw t uses U(seed, 2t) and U(seed, 2t+1).  Writes m
 * weights and indices (unused FL slots stay zero, as in the reference). */
int mc_sampler_sample(mc_sampler *s, uint64_t m, uint64_t seed, int unique, float *weights,
                      uint64_t *indices);

/* Resident jobs: the matrix, centers, assignments and costs stay on the device. */
int mc_job_create(mc_context *ctx, const mc_matrix *X, const float *centers, uint32_t k, int msr,
                  double prior, const double *weights, int precision, uint64_t seed, mc_job **out);
int mc_job_destroy(mc_job *job);
int mc_job_assign(mc_job *job);                       /* assignment pass with current centers */
int mc_job_lloyd_step(mc_job *job, int *restarted);   /* centroid update + assignment */
int mc_job_cost(mc_job *job, double *cost);           /* FP64 objective of current asn/costs */
int mc_job_run(mc_job *job, double eps, uint64_t maxiter, double *initcost, double *finalcost,
               uint64_t *numiter);                    /* the perform_hard_clustering loop */
int mc_job_read(mc_job *job, float *centers, uint32_t *asn, double *costs);
int mc_job_read_f32(mc_job *job, float *centers, uint32_t *asn, float *costs);  /* costs as float32 */
/* Minibatch hard clustering on a job (perform_hard_minibatch_clustering,
 * clustering/solve.h:386-582): every calc_cost_freq iterations (and at the last) an
 * exhaustive assignment, restarts of the centers holding <= reseed_after rows (D^2 draws
 * U(seed, r) over the costs), and the objective; between them, a sample of mbsize rows
 * (U(seed ^ 0x6A09E667F3BCC908, t), with or without replacement) is assigned and every hit
 * center is replaced by its group's mean (L1: its group's median; with weights over dense
 * rows, weighted_median reading the full weight vector at the group position, as
 * solve.h:559-561 does).  Distances use the prior as the prior sum, as
 * the reference's minibatch code does.  The centers of the best objective are kept; asn and
 * costs are those of the last exhaustive assignment. */
int mc_job_minibatch(mc_job *job, uint64_t mbsize, uint64_t maxiter, uint64_t calc_cost_freq,
                     uint64_t reseed_after, int with_replacement, double *initcost, double *finalcost,
                     uint64_t *numiter);
/* hcluster with mbsize > 0 (python/pycluster.h:31-40): checkin frequency
 * ceil(maxiter / ncheckins), ncheckins 0 -> 10. */
int mc_hcluster_minibatch(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k,
                          int msr, double prior, const double *weights, uint64_t mbsize,
                          uint64_t maxiter, uint64_t ncheckins, uint64_t reseed_count,
                          int with_replacement, uint64_t seed, int precision, float *centers_out,
                          uint32_t *asn, double *costs, double *initcost, double *finalcost,
                          uint64_t *numiter);
/* hcluster with mbsize > 0 and cs=True: minibatch-by-coreset EM (hmb_coreset_clustering,
 * clustering/solve.h:593-789; python/pycluster.h:36-38).  Rounds of an exhaustive
 * assignment, restarts of centers holding <= reseed_count rows (D^2 draws U(seed, r); rows
 * move to a restarted center when strictly cheaper), the FP64 objective (best centers kept),
 * then ceil(maxiter / ncheckins) times: a coreset of min(mbsize, n) distinct rows (LBK
 * sensitivities, VX for L1; alpha 1 for L1, 2 for SQRL2, 4 otherwise; sample seed
 * floor(U(seed, r) * 2^53)) clustered by perform_hard_clustering (eps 1e-3, 1 update, 3 in
 * the first two rounds; weights = coreset weights x row weights; restart seed = coreset
 * size).  One uniform counter r serves the restarts and the sample seeds in order.
 * centers_out: the best centers; asn, costs: the last exhaustive assignment. */
int mc_hcluster_coreset(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k,
                        int msr, double prior, const double *weights, uint64_t mbsize,
                        uint64_t maxiter, uint64_t ncheckins, uint64_t reseed_count, uint64_t seed,
                        int precision, float *centers_out, uint32_t *asn, double *costs,
                        double *initcost, double *finalcost, uint64_t *numiter);
/* Soft clustering (perform_soft_clustering, clustering/solve.h:287-374, with the soft
 * weighted means of centroid.h:795-866) over dense rows: per iteration asn = row softmax of
 * -temp * costs (NaN rows: equal shares over the minimal costs), objective sum_i w_i
 * dot(costs_i, asn_i) (FP64), centers = soft weighted means, costs = msr(rows, centers).
 * Stops when the objective improves by <= eps * max(old, new) or after maxiter iterations;
 * centers are taken only on improvement.  costs_out / asn_out: nrows x k float32 (the last
 * ones computed).  L1 over dense rows: per center the value, per column, of the row with
 * the largest soft weight (weighted_median with the soft assignments, centroid.h:815-838);
 * L1 over CSR rows returns MC_EUNSUPPORTED (the reference raises). */
int mc_scluster(mc_context *ctx, const mc_matrix *X, const float *centers_in, uint32_t k, int msr,
                double prior, const double *weights, double temp, uint64_t maxiter, double eps,
                float *centers_out, float *costs_out, float *asn_out, double *initcost,
                double *finalcost, uint64_t *numiter);
/* rows whose BF16/TF32 margin fell below the bound in the last pass (0 for FP32) */
int mc_job_recheck_count(mc_job *job, uint64_t *count);
/* A job whose k centers are seeded on the device by D^2 sampling with uniforms U(seed, i),
 * i < k (what minicore.cluster does between kmeanspp and hcluster,
 * python/minicore/__init__.py:235-261, without the host round trip).  center_ids: optional
 * k seed row ids.  Requires k <= nrows. */
int mc_job_create_kmeanspp(mc_context *ctx, const mc_matrix *X, uint32_t k, int msr, double prior,
                           const double *weights, int precision, uint64_t seed, uint32_t *center_ids,
                           mc_job **out);

/* Continuous-batching server (no reference counterpart).  S slots, each a host thread with
 * its own stream; queued jobs are admitted first-fit against a device-memory budget
 * (mem_budget_bytes, 0 = 90% of free memory) and the device's free memory; a job that would
 * run alone is always admitted.  Every pointer in a job description (rows, centers,
 * weights, outputs) must stay valid until the job's result has been returned. */
typedef struct mc_job_desc {
    mc_matrix X;               /* rows: host or device memory                                */
    const float *centers;      /* k x ncols initial centers, or NULL for k-means++ seeding   */
    uint32_t k;
    int msr;
    double prior;
    const double *weights;     /* optional, n                                                */
    int precision;             /* MC_FP32 / MC_TF32 / MC_BF16                                */
    double eps;
    uint64_t maxiter;
    uint64_t seed;             /* seeding uniforms and empty-cluster restarts                */
    float *centers_out;        /* optional outputs, host or device: k x ncols                */
    uint32_t *asn_out;         /* n                                                          */
    double *costs_out;         /* n                                                          */
    uint32_t *center_ids_out;  /* k seed row ids (only when centers == NULL)                 */
} mc_job_desc;

typedef struct mc_job_result {
    int status;                /* mc_status of the job                                       */
    uint64_t numiter;
    double initcost, finalcost;
    double queue_ms, run_ms, total_ms;  /* submit->admit, admit->done, submit->done          */
    char error[256];           /* mc_last_error() text when status != MC_OK                  */
    /* run_ms in parts: rows uploaded and validated, centers given or seeded (k-means++ on
     * the device); the Lloyd loop; outputs copied back */
    double setup_ms, loop_ms, read_ms;
} mc_job_result;

int mc_server_create(int device, uint32_t slots, uint64_t mem_budget_bytes, mc_server **out);
int mc_server_submit(mc_server *s, const mc_job_desc *job, uint64_t *ticket);
/* MC_EBUSY while the job runs; MC_OK with the result, after which the ticket is released. */
int mc_server_poll(mc_server *s, uint64_t ticket, mc_job_result *result);
/* Blocks up to timeout_ms (MC_ETIMEOUT after); releases the ticket on MC_OK. */
int mc_server_wait(mc_server *s, uint64_t ticket, uint64_t timeout_ms, mc_job_result *result);
/* JSON: completed, failed, queued, running, max_running, slots, budget_bytes and p50/p99 of
 * the total, queue and run latencies (ms) of the jobs completed since the last reset. */
int mc_server_stats(mc_server *s, char *json, uint64_t capacity);
int mc_server_reset_stats(mc_server *s);
/* Runs every queued job to completion, then stops the slots. */
int mc_server_destroy(mc_server *s);

/* Kernel-variant autotuner (no reference counterpart).  Some kernels come in variants that
 * compute bit-identical results (same per-element arithmetic and summation order) at
 * different speeds: the CSR sparse-dot batch size, the SQRL2 FP32 register tile and the
 * kmeans++ distance-update load path.  The first call for a shape bucket times each variant
 * and keeps the fastest.  Decisions persist in a cache file (MC_AUTOTUNE_CACHE, default
 * $XDG_CACHE_HOME or $HOME/.cache + /minicore_gb300/autotune.tsv); MC_AUTOTUNE=0 or
 * mc_autotune_enable(0) keeps the defaults. */
int mc_autotune_enable(int on);

/* How mc_job_run (and mc_hcluster, the server's jobs) runs the Lloyd loop (no reference
 * counterpart; the reference's loop is solve.h:98-175).  Every mode gives the same results.
 *   MC_LOOP_HOST   the host decides after each step (one round trip per decision)
 *   MC_LOOP_FUSED  the stop rule (objective test, revert, empty-cluster check) runs on the
 *                  device after each iteration: one round trip per iteration
 *   MC_LOOP_GRAPH  one CUDA graph: a while-conditional node whose body is the centroid update,
 *                  the assignment pass, the objective and the stop rule; one round trip per
 *                  run, plus one capture and instantiation
 * Every mode hands back to the host for the D^2 restart of an empty cluster.  -1 (default)
 * picks the graph for runs of >= 16 iterations over n*d <= 2^24 values, else the fused loop;
 * the server's workers never use the graph.  MC_LOOP_MODE=0|1|2 sets the mode from the
 * environment; an active mc_profile_enable keeps the graph off. */
enum { MC_LOOP_HOST = 0, MC_LOOP_FUSED = 1, MC_LOOP_GRAPH = 2 };
int mc_loop_mode(int mode);
int mc_autotune_reset(void);                    /* forget every decision (not the file)      */
int mc_autotune_load(const char *path);         /* add decisions from a cache file           */
int mc_autotune_save(const char *path);         /* write every decision to a cache file      */
/* JSON: {"enabled": b, "entries": {key: {"variant": v, "ms": [per-variant best ms]}}} */
int mc_autotune_report(char *json, uint64_t capacity);

/* Capacity of mc_assign_sqrl2_noalloc's fixed scratch array, in floats (4 MiB). */
#define MC_NOALLOC_SCRATCH_FLOATS (1u << 20)

/* Dense SQRL2 FP32 assignment that allocates no device memory (no counterpart in the
 * reference; it exists for callers that cannot allocate on the call path, e.g. hosts that
 * reserve their whole GPU memory budget up front or that only hand the library buffers
 * they own).  Same results as mc_assign(..., MC_SQRL2, prior, MC_FP32, ...).
 * X (n x d row-major float32), centers (k x d float32), asn (n) and costs (n) must be
 * device pointers; the work is queued on cuda_stream (a cudaStream_t, may be NULL) and the
 * call returns without waiting.  Its scratch (the centers transposed) lives in one fixed
 * device array of MC_NOALLOC_SCRATCH_FLOATS floats per GPU: kp * d must fit, kp being k
 * rounded up to a multiple of 64 (k < 128) or 128 (k >= 128), else MC_EINVAL.  The first
 * call on a device looks up that array's address (which may load the module holding it: a
 * one-time 4 MiB), so make it before any stream capture; inside a capture it is refused.
 * Pointers and stream must belong to the current device (another GPU's memory: MC_EINVAL).
 * All calls on a device share the array: calls that overlap on the GPU race. */
int mc_assign_sqrl2_noalloc(const float *X, uint64_t n, uint64_t d, const float *centers, uint32_t k,
                            uint32_t *asn, double *costs, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* MINICORE_GB300_H_ */
