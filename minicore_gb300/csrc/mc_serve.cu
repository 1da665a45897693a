// Continuous-batching server for clustering jobs.  The reference has no counterpart: its
// entry points (python/minicore/__init__.py:235-261 cluster, clustering/solve.h:98-175
// perform_hard_clustering) run one call at a time on the caller's OpenMP threads.
//
// A server owns S slots.  Each slot is a host worker thread with its own mc_context (its
// own non-blocking CUDA stream), so the jobs that the slots hold run concurrently and their
// kernels overlap on the GPU.  Submitted jobs wait in a FIFO queue; a slot that frees up
// admits the first queued job whose estimated device footprint fits both in the budget not
// yet reserved by running jobs and in what the device can still hand out (cudaMemGetInfo
// plus the unused part of the stream-ordered pool).  A smaller job may therefore pass a
// larger one that does not fit yet; a job that runs alone is always admitted.
//
// Each job keeps its rows, centers, assignments and costs on the device from upload to
// completion (an mc_job): upload if the rows are in host memory, k-means++ seeding on the
// device when no centers are given (mc_job_create_kmeanspp), the perform_hard_clustering
// loop (mc_job_run), then one copy of the requested outputs.  The results do not depend on
// which other jobs run beside it: every kernel's reduction order is fixed by the job alone.
//
// Latency per job: queue = admission - submission, run = completion - admission,
// total = completion - submission (host steady clock).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mc_internal.cuh"

using namespace mc;

namespace {

using Clock = std::chrono::steady_clock;

// Device bytes a job will hold at its peak, from the allocations mc_job_create and the
// assignment / centroid passes make (rounded up; the admission check, not an allocator).
uint64_t job_footprint(const mc_job_desc &j) {
    const mc_matrix &m = j.X;
    const uint64_t n = m.nrows, d = m.ncols, k = j.k;
    uint64_t b = 0;
    if (m.kind == MC_DENSE_F32) {
        if (!is_device_ptr(m.values)) b += n * d * 4;                   // device copy of the rows
        if (j.precision != MC_FP32) b += n * ((d + 63) / 64 * 64) * 4;  // tensor-core operand copy
    } else if (!is_device_ptr(m.values)) {
        b += m.nnz * 8 + (n + 1) * 8;
    }
    b += n * 112;                                  // per-row state, sort and candidates
    b += k * ((d + 127) / 128 * 128) * 4 * 6;      // centers, transposes, operand copies
    b += ((n + 255) / 256 + k) * d * 16;           // centroid chunk partials
    return b + (8ull << 20);
}

struct Ticket {
    mc_job_desc desc{};
    mc_job_result res{};
    bool done = false;
    Clock::time_point t_submit, t_admit, t_done;
    uint64_t bytes = 0;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// linear interpolation between closest ranks
double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * double(v.size() - 1);
    const size_t i = size_t(pos);
    const double f = pos - double(i);
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

struct mc_server {
    int device = 0;
    uint64_t budget = 0, reserved = 0, running = 0, max_running = 0;
    uint64_t completed = 0, failed = 0, next_id = 1;
    bool stop = false;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Ticket *> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Ticket>> tickets;
    std::vector<mc_context *> ctxs;
    std::vector<std::thread> workers;
    std::vector<double> lat_total, lat_queue, lat_run;
};

namespace {

int run_job(mc_context *ctx, Ticket &t) {
    const mc_job_desc &j = t.desc;
    mc_job *job = nullptr;
    const Clock::time_point t0 = Clock::now();
    if (j.centers)
        MC_TRY(mc_job_create(ctx, &j.X, j.centers, j.k, j.msr, j.prior, j.weights, j.precision, j.seed, &job));
    else
        MC_TRY(mc_job_create_kmeanspp(ctx, &j.X, j.k, j.msr, j.prior, j.weights, j.precision, j.seed,
                                      j.center_ids_out, &job));
    std::unique_ptr<mc_job, int (*)(mc_job *)> guard(job, mc_job_destroy);
    const Clock::time_point t1 = Clock::now();
    MC_TRY(mc_job_run(job, j.eps, j.maxiter, &t.res.initcost, &t.res.finalcost, &t.res.numiter));
    const Clock::time_point t2 = Clock::now();
    const int rc = mc_job_read(job, j.centers_out, j.asn_out, j.costs_out);
    const Clock::time_point t3 = Clock::now();
    t.res.setup_ms = ms_between(t0, t1);
    t.res.loop_ms = ms_between(t1, t2);
    t.res.read_ms = ms_between(t2, t3);
    return rc;
}

// bytes the device can still hand out: free memory plus what the stream-ordered pool holds
// but does not use (its release threshold keeps freed blocks)
uint64_t device_available(int device) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
    uint64_t slack = 0;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t resv = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &resv) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && resv > used)
            slack = resv - used;
    }
    return uint64_t(free_b) + slack;
}

void worker_main(mc_server *s, int slot) {
    cudaSetDevice(s->device);
    // the host loop: with several jobs in flight the GPU stays busy through each job's host
    // round trips, while capturing and instantiating a loop graph per job costs more
    // (measured on the serving stream: 201 jobs/s host loop against 154 with graphs)
    set_thread_loop_graph(0);
    mc_context *ctx = s->ctxs[size_t(slot)];
    for (;;) {
        Ticket *t = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (s->stop && s->queue.empty()) return;
                if (!s->queue.empty()) {
                    const uint64_t avail = s->running ? device_available(s->device) : ~0ull;
                    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
                        Ticket *c = *it;
                        if (s->running == 0 || (s->reserved + c->bytes <= s->budget && c->bytes <= avail)) {
                            t = c;
                            s->queue.erase(it);
                            break;
                        }
                    }
                    if (t) break;
                }
                // woken by a submission or a completion; the timeout re-reads free memory
                s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
            }
            s->reserved += t->bytes;
            s->running += 1;
            s->max_running = std::max(s->max_running, s->running);
            t->t_admit = Clock::now();
        }
        const int rc = run_job(ctx, *t);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            t->t_done = Clock::now();
            t->res.status = rc;
            if (rc != MC_OK) std::snprintf(t->res.error, sizeof(t->res.error), "%s", mc_last_error());
            t->res.queue_ms = ms_between(t->t_submit, t->t_admit);
            t->res.run_ms = ms_between(t->t_admit, t->t_done);
            t->res.total_ms = ms_between(t->t_submit, t->t_done);
            t->done = true;
            s->reserved -= t->bytes;
            s->running -= 1;
            if (rc == MC_OK) {
                s->completed += 1;
                s->lat_total.push_back(t->res.total_ms);
                s->lat_queue.push_back(t->res.queue_ms);
                s->lat_run.push_back(t->res.run_ms);
            } else {
                s->failed += 1;
            }
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int mc_server_create(int device, uint32_t slots, uint64_t mem_budget_bytes, mc_server **out) {
    if (!out) return fail(MC_EINVAL, "out is null");
    *out = nullptr;
    if (slots == 0 || slots > 64) return fail(MC_EINVAL, "slots must be in [1, 64]");
    MC_CUDA_TRY(cudaSetDevice(device));
    size_t free_b = 0, total_b = 0;
    MC_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    std::unique_ptr<mc_server> s(new mc_server());
    s->device = device;
    s->budget = mem_budget_bytes ? mem_budget_bytes : uint64_t(double(free_b) * 0.9);
    for (uint32_t i = 0; i < slots; ++i) {
        mc_context *c = nullptr;
        const int rc = mc_context_create(device, &c);
        if (rc != MC_OK) {
            for (auto *p : s->ctxs) mc_context_destroy(p);
            return rc;
        }
        s->ctxs.push_back(c);
    }
    for (uint32_t i = 0; i < slots; ++i) s->workers.emplace_back(worker_main, s.get(), int(i));
    *out = s.release();
    return MC_OK;
}

int mc_server_submit(mc_server *s, const mc_job_desc *desc, uint64_t *ticket) {
    if (!s || !desc || !ticket) return fail(MC_EINVAL, "null argument");
    if (!measure_supported(desc->msr)) return fail(MC_EUNSUPPORTED, "measure not implemented on this path");
    if (desc->k == 0 || desc->X.nrows == 0 || desc->X.ncols == 0) return fail(MC_EINVAL, "empty job");
    if (!desc->centers && desc->k > desc->X.nrows)
        return fail(MC_EINVAL, "k-means++ seeding needs k <= number of rows");
    std::unique_ptr<Ticket> t(new Ticket());
    t->desc = *desc;
    t->bytes = job_footprint(*desc);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return fail(MC_EINVAL, "server is shutting down");
        t->t_submit = Clock::now();
        const uint64_t id = s->next_id++;
        s->queue.push_back(t.get());
        s->tickets.emplace(id, std::move(t));
        *ticket = id;
    }
    s->cv_work.notify_one();
    return MC_OK;
}

int mc_server_poll(mc_server *s, uint64_t ticket, mc_job_result *res) {
    if (!s) return fail(MC_EINVAL, "server is null");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(MC_EINVAL, "unknown ticket");
    if (!it->second->done) return MC_EBUSY;
    if (res) *res = it->second->res;
    s->tickets.erase(it);
    return MC_OK;
}

int mc_server_wait(mc_server *s, uint64_t ticket, uint64_t timeout_ms, mc_job_result *res) {
    if (!s) return fail(MC_EINVAL, "server is null");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(MC_EINVAL, "unknown ticket");
    Ticket *t = it->second.get();
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return t->done; }))
        return fail(MC_ETIMEOUT, "job not finished within the timeout");
    if (res) *res = t->res;
    s->tickets.erase(ticket);
    return MC_OK;
}

int mc_server_stats(mc_server *s, char *json, uint64_t capacity) {
    if (!s || !json || !capacity) return fail(MC_EINVAL, "null argument");
    std::string out;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        char buf[1024];
        std::snprintf(buf, sizeof(buf),
                      "{\"completed\": %llu, \"failed\": %llu, \"queued\": %llu, \"running\": %llu, "
                      "\"max_running\": %llu, \"slots\": %llu, \"budget_bytes\": %llu, "
                      "\"p50_total_ms\": %.6g, \"p99_total_ms\": %.6g, \"p50_queue_ms\": %.6g, "
                      "\"p99_queue_ms\": %.6g, \"p50_run_ms\": %.6g, \"p99_run_ms\": %.6g}",
                      (unsigned long long)s->completed, (unsigned long long)s->failed,
                      (unsigned long long)s->queue.size(), (unsigned long long)s->running,
                      (unsigned long long)s->max_running, (unsigned long long)s->ctxs.size(),
                      (unsigned long long)s->budget, percentile(s->lat_total, 0.5), percentile(s->lat_total, 0.99),
                      percentile(s->lat_queue, 0.5), percentile(s->lat_queue, 0.99), percentile(s->lat_run, 0.5),
                      percentile(s->lat_run, 0.99));
        out = buf;
    }
    if (out.size() + 1 > capacity) return fail(MC_EINVAL, "stats buffer too small");
    std::memcpy(json, out.c_str(), out.size() + 1);
    return MC_OK;
}

int mc_server_reset_stats(mc_server *s) {
    if (!s) return fail(MC_EINVAL, "server is null");
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_total.clear();
    s->lat_queue.clear();
    s->lat_run.clear();
    s->completed = s->failed = 0;
    s->max_running = s->running;
    return MC_OK;
}

int mc_server_destroy(mc_server *s) {
    if (!s) return MC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &w : s->workers) w.join();
    for (auto *c : s->ctxs) mc_context_destroy(c);
    delete s;
    return MC_OK;
}

}  // extern "C"
