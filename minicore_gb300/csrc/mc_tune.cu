// Kernel-variant autotuner.
//
// Tuned families (all variants bit-identical by construction):
//   csr_sparse   k_assign_sparse nonzero batch size (8, 4, 16)
//   dense_sqrl2  k_assign_tiled register tile for SQRL2 (8x8 / 128 rows, 4x4 / 64 rows)
//   kmpp_dense   kmeans++ distance update (cp.async-staged rows, direct loads)
// Keys carry the device (compute capability and SM count) and the shape bucket.  Decisions
// live in a process-wide table, loaded from and appended to a cache file:
//   MC_AUTOTUNE=0            tuning off (defaults only)
//   MC_AUTOTUNE_CACHE=path   cache file (default $XDG_CACHE_HOME or $HOME/.cache, then
//                            minicore_gb300/autotune.tsv); one "key<TAB>variant<TAB>ms,..."
//                            line per decision
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <vector>

#include "mc_tune.cuh"

namespace mc {

namespace {

struct Decision {
    int variant = 0;
    std::vector<float> ms;  // best time per variant (empty when loaded without timings)
};

std::mutex g_tune_mu;
std::map<std::string, Decision> g_tune;
int g_tune_on = -1;  // -1: from MC_AUTOTUNE
bool g_tune_loaded = false;
std::string g_tune_path;

bool tune_enabled_locked() {
    if (g_tune_on < 0) {
        const char *e = std::getenv("MC_AUTOTUNE");
        g_tune_on = (e && e[0] == '0') ? 0 : 1;
    }
    return g_tune_on == 1;
}

std::string default_cache_path() {
    if (const char *p = std::getenv("MC_AUTOTUNE_CACHE")) return p;
    std::string base;
    if (const char *x = std::getenv("XDG_CACHE_HOME")) base = x;
    else if (const char *h = std::getenv("HOME")) base = std::string(h) + "/.cache";
    if (base.empty()) return "";
    return base + "/minicore_gb300/autotune.tsv";
}

bool load_file_locked(const std::string &path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string key, var, times;
        if (!std::getline(ls, key, '\t') || !std::getline(ls, var, '\t')) continue;
        std::getline(ls, times);
        Decision d;
        char *end = nullptr;
        const long v = std::strtol(var.c_str(), &end, 10);
        if (end == var.c_str() || v < 0 || v > 64) continue;
        d.variant = int(v);
        std::istringstream ts(times);
        std::string t;
        while (std::getline(ts, t, ',')) d.ms.push_back(std::strtof(t.c_str(), nullptr));
        g_tune[key] = d;  // later lines win
    }
    return true;
}

void ensure_loaded_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    g_tune_path = default_cache_path();
    if (!g_tune_path.empty()) load_file_locked(g_tune_path);
}

std::string line_of(const std::string &key, const Decision &d) {
    std::ostringstream o;
    o << key << '\t' << d.variant << '\t';
    for (size_t i = 0; i < d.ms.size(); ++i) o << (i ? "," : "") << d.ms[i];
    return o.str();
}

void append_locked(const std::string &key, const Decision &d) {
    if (g_tune_path.empty()) return;
    const size_t slash = g_tune_path.find_last_of('/');
    if (slash != std::string::npos) {
        // create the directory chain (ignore failures: the table stays in memory)
        std::string dir = g_tune_path.substr(0, slash);
        for (size_t p = 1; p <= dir.size(); ++p)
            if (p == dir.size() || dir[p] == '/') mkdir(dir.substr(0, p).c_str(), 0755);
    }
    std::ofstream f(g_tune_path, std::ios::app);
    if (f) f << line_of(key, d) << '\n';
}

// attribute queries (cudaGetDeviceProperties fills the whole structure, far slower per call)
std::string device_tag() {
    int dev = 0, major = 0, minor = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return "dev?";
    return "sm" + std::to_string(major * 10 + minor) + "x" + std::to_string(sms);
}

}  // namespace

std::string tune_bucket(uint64_t v) {
    int b = 0;
    while ((uint64_t(1) << b) < v && b < 63) ++b;
    return "2^" + std::to_string(b);
}

int tune_launch(const std::string &key0, int nvariants, int default_variant, cudaStream_t st, bool allow,
                const std::function<int(int)> &launch) {
    if (nvariants <= 1) return launch(default_variant);
    std::string key;
    int known = -1;  // decided under the lock, launched outside it (a launch may tune a nested key)
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (!tune_enabled_locked()) {
            known = default_variant;
        } else {
            ensure_loaded_locked();
            key = key0 + "|" + device_tag();
            auto it = g_tune.find(key);
            if (it != g_tune.end() && it->second.variant < nvariants) known = it->second.variant;
        }
    }
    if (known >= 0) return launch(known);
    // a caller that may not time (a loop that must not synchronise, a stream being captured)
    // takes a recorded decision above, else the default
    if (!allow) return launch(default_variant);
    // a stream being captured into a graph cannot time anything: the default (the variants
    // give identical results)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusNone;
    if (cap != cudaStreamCaptureStatusNone) return launch(default_variant);
    // time every variant twice (the first run also warms caches); outputs are identical, so
    // whatever ran last leaves the right result
    cudaEvent_t e0, e1;
    MC_CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(MC_ECUDA, "cudaEventCreate failed");
    }
    Decision d;
    d.ms.assign(size_t(nvariants), 3.0e38f);
    int rc = MC_OK;
    for (int rep = 0; rep < 2 && rc == MC_OK; ++rep) {
        for (int v = 0; v < nvariants && rc == MC_OK; ++v) {
            cudaEventRecord(e0, st);
            rc = launch(v);
            cudaEventRecord(e1, st);
            if (rc != MC_OK) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = fail(MC_ECUDA, "autotune: cudaEventSynchronize failed");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < d.ms[size_t(v)]) d.ms[size_t(v)] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != MC_OK) return rc;
    d.variant = default_variant;
    for (int v = 0; v < nvariants; ++v)
        if (d.ms[size_t(v)] < d.ms[size_t(d.variant)]) d.variant = v;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (g_tune.find(key) == g_tune.end()) {
        g_tune[key] = d;
        append_locked(key, d);
    }
    return MC_OK;
}

}  // namespace mc

using namespace mc;

namespace mc {

// Measured logf throughput of this GPU, the compute roof of the CSR JSD sparse dot (two
// logf per nonzero and center): 8 independent chains per thread of x <- logf(x) + 4 (the
// inputs stay positive normal floats near the fixed point 5.75), full occupancy, best of
// three launches timed with CUDA events.
__global__ void __launch_bounds__(256) k_logf_rate(float seed, int iters, float *sink) {
    float x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = seed + 0.125f * float(c) + 1e-6f * float(threadIdx.x);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = logf(x[c]) + 4.0f;
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 123.456f) sink[0] = s;  // keeps the chains live
}

}  // namespace mc

extern "C" int mc_diag_logf_rate(int device, double *logs_per_s) {
    using namespace mc;
    if (!logs_per_s) return fail(MC_EINVAL, "null output");
    MC_CUDA_TRY(cudaSetDevice(device));
    int sms = 0;
    MC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st = nullptr;
    MC_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float *sink = nullptr;
    int rc = MC_OK;
    const int iters = 4096, blocks = sms * 8, threads = 256;
    float best = 0.f;
    if (cudaMallocAsync(&sink, sizeof(float), st) != cudaSuccess) rc = fail(MC_ENOMEM, "probe buffer");
    for (int rep = 0; rc == MC_OK && rep < 4; ++rep) {
        cudaEventRecord(e0, st);
        k_logf_rate<<<blocks, threads, 0, st>>>(1.5f, iters, sink), note_launch();
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = fail(MC_ECUDA, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // launch 0 warms up
    }
    if (sink) cudaFreeAsync(sink, st);
    cudaStreamSynchronize(st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (rc != MC_OK) return rc;
    *logs_per_s = double(blocks) * threads * 8.0 * iters / (double(best) * 1e-3);
    return MC_OK;
}

extern "C" {

int mc_autotune_enable(int on) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_on = on ? 1 : 0;
    return MC_OK;
}

int mc_autotune_reset(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
    g_tune_loaded = true;  // do not reload the cache file into the cleared table
    return MC_OK;
}

int mc_autotune_load(const char *path) {
    if (!path) return fail(MC_EINVAL, "path is null");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ensure_loaded_locked();  // the default cache first, so the given file's lines win
    if (!load_file_locked(path)) return fail(MC_EINVAL, std::string("cannot read ") + path);
    return MC_OK;
}

int mc_autotune_save(const char *path) {
    if (!path) return fail(MC_EINVAL, "path is null");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::ofstream f(path, std::ios::trunc);
    if (!f) return fail(MC_EINVAL, std::string("cannot write ") + path);
    for (const auto &kv : g_tune) f << line_of(kv.first, kv.second) << '\n';
    return f ? MC_OK : fail(MC_EINVAL, std::string("write failed: ") + path);
}

int mc_autotune_report(char *json, uint64_t capacity) {
    if (!json || !capacity) return fail(MC_EINVAL, "null buffer");
    std::ostringstream o;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        o << "{\"enabled\": " << (tune_enabled_locked() ? "true" : "false") << ", \"entries\": {";
        bool first = true;
        for (const auto &kv : g_tune) {
            o << (first ? "" : ", ") << "\"" << kv.first << "\": {\"variant\": " << kv.second.variant << ", \"ms\": [";
            for (size_t i = 0; i < kv.second.ms.size(); ++i) o << (i ? ", " : "") << kv.second.ms[i];
            o << "]}";
            first = false;
        }
        o << "}}";
    }
    const std::string s = o.str();
    if (s.size() + 1 > capacity) return fail(MC_EINVAL, "report buffer too small");
    std::memcpy(json, s.c_str(), s.size() + 1);
    return MC_OK;
}

}  // extern "C"
