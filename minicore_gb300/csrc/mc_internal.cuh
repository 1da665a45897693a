// Internal definitions shared by the minicore_gb300 CUDA translation units.
//
// Numerical contract (identical to the oracle's restatement):
//  * pair scalars follow cmp::msr_with_prior's prior setup, FT = float
//    (include/minicore/dist/applicator.h:1642-1656);
//  * element reductions run sequentially over columns in float, with fmaf only where
//    written out (the library is compiled with -fmad=false);
//  * FP64 totals and D^2 draws use the blocked order of det_* below.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/minicore_gb300.h"

namespace mc {

// ------------------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);

#define MC_CUDA_TRY(expr)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return ::mc::fail(e_ == cudaErrorMemoryAllocation ? MC_ENOMEM : MC_ECUDA,       \
                              std::string(#expr) + ": " + cudaGetErrorString(e_));          \
    } while (0)

#define MC_TRY(expr)                    \
    do {                                \
        int s_ = (expr);                \
        if (s_ != MC_OK) return s_;     \
    } while (0)

// ------------------------------------------------------------------------------------
// measure helpers
// ------------------------------------------------------------------------------------
enum Msr { L1 = 0, SQRL2 = 2, JSD = 4, MKL = 5, HELLINGER = 6 };

inline bool measure_supported(int msr) {
    return msr == L1 || msr == SQRL2 || msr == JSD || msr == MKL || msr == HELLINGER;
}
inline bool measure_uses_prior(int msr) { return msr != SQRL2; }

constexpr double kSqrt1_2 = 0.70710678118654752440;

struct PairScalars {
    float pv, lhrsi, rhrsi, lhinc, rhinc;
};

// One side of the prior setup: given the pair's pv, the scaled sum for a vector.
__host__ __device__ inline void side_scalars(float pv, double vsum, uint64_t nd, float &rsi, float &inc) {
    const float psum = pv * float(nd);
    const float s = float(vsum + double(psum));
    rsi = 1.f / s;
    float v = (pv != 0.f && s != 0.f) ? pv * rsi : 0.f;
    if (v != v) v = 0.f;
    inc = v;
}

// Full pair setup (applicator.h:1642-1656): lh = center, rh = data row.
__host__ __device__ inline PairScalars pair_scalars(double prior, double prior_sum_arg, double rowsum,
                                                     double ctrsum, uint64_t nd) {
    const float lhsum0 = float(ctrsum + prior_sum_arg);
    const float rhsum0 = float(rowsum + prior_sum_arg);
    const float smallest_pv = 7.0069e-42f * (lhsum0 + rhsum0);
    const float fp = float(prior);
    const float pv = (fp < smallest_pv) ? smallest_pv : fp;
    PairScalars s;
    s.pv = pv;
    side_scalars(pv, ctrsum, nd, s.lhrsi, s.lhinc);
    side_scalars(pv, rowsum, nd, s.rhrsi, s.rhinc);
    return s;
}

// post-processing of divergences (applicator.h:1754-1760), as a float value
__host__ __device__ inline float post_divergence(float r) {
    if (r != r) return r;
    if (r < 0.f) r = 0.f;
    if (r > 3.402823466e+38f) r = 3.402823466e+38f;  // +inf -> FLT_MAX
    return r;
}

// ------------------------------------------------------------------------------------
// splitmix64 uniforms (same stream as mc_uniforms / the oracle)
// ------------------------------------------------------------------------------------
__host__ __device__ inline double uniform_at(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return double(z >> 11) * (1.0 / 9007199254740992.0);
}

// ------------------------------------------------------------------------------------
// deterministic FP64 sums: chunks of 8192 consecutive elements, a pairwise tree inside each
// chunk and a pairwise tree over the chunk totals (padded to a power of two)
// ------------------------------------------------------------------------------------
constexpr int kDetChunk = 8192;
constexpr int kDetThreads = 256;
constexpr int kDetPer = 32;

__host__ __device__ inline uint64_t det_chunks(uint64_t n) { return (n + kDetChunk - 1) / kDetChunk; }

// from the root of a heap with P leaves (node j has children 2j, 2j + 1; leaves at [P, 2P)):
// left when r < L or R is not positive, else r -= L; returns the leaf
__device__ inline uint64_t det_heap_descend(const double *T, uint64_t P, double &r) {
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
// leaves of the tree over the chunk totals (a power of two, at least 1)
__host__ __device__ inline uint64_t det_leaves(uint64_t n) {
    uint64_t p = 1;
    while (p < det_chunks(n)) p <<= 1;
    return p;
}
// doubles of scratch that launch_det_sum / launch_det_draw need (the tree, heap layout)
__host__ __device__ inline uint64_t det_tmp_size(uint64_t n) { return 2 * det_leaves(n); }

// value sources for det sums
enum DetSrc : int {
    DET_F64 = 0,        // x[i]
    DET_F32 = 1,        // (double)xf[i]
    DET_F64_W = 2,      // x[i] * w[i]
    DET_F32_W = 3,      // (double)xf[i] * w[i]
    DET_F64_KEY = 4,    // key[i] == kval ? x[i] : 0
};

struct DetInput {
    int src;
    const double *x;
    const float *xf;
    const double *w;
    uint64_t n;
    const uint32_t *key = nullptr;
    uint32_t kval = 0;
    __device__ inline double get(uint64_t i) const {
        switch (src) {
            case DET_F64: return x[i];
            case DET_F32: return double(xf[i]);
            case DET_F64_W: return x[i] * w[i];
            case DET_F64_KEY: return key[i] == kval ? x[i] : 0.0;
            default: return double(xf[i]) * w[i];
        }
    }
};

// ------------------------------------------------------------------------------------
// device buffers
// ------------------------------------------------------------------------------------
// device allocations made through DBuf by the calling thread (a stream capture checks that
// it made none)
void note_device_alloc();
uint64_t device_allocs();

template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count, cudaStream_t stream) {
        if (count <= n && p) return MC_OK;
        release();
        st = stream;
        if (count == 0) count = 1;
        note_device_alloc();
        cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(T), stream);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(MC_ENOMEM, std::string("device allocation of ") + std::to_string(count * sizeof(T)) +
                                       " bytes failed: " + cudaGetErrorString(e));
        }
        n = count;
        return MC_OK;
    }
};

// managed memory, or device memory of the current device
bool is_device_ptr(const void *p);
// device memory of a GPU other than the current one
bool is_foreign_device_ptr(const void *p);

// process-wide count of kernel launches issued by this library
void note_launch();
// mc_job_run's loop graph for jobs run by the calling thread: 1 on, 0 off, -1 the process
// setting (mc_loop_graph_enable / MC_LOOP_GRAPH)
void set_thread_loop_graph(int on);

// Phase profiler (off by default): when enabled, Phase records a CUDA event pair on the
// stream around a scope; mc_profile_report() sums the elapsed times per phase name.
bool profiling_enabled();
void profile_record(const char *name, cudaEvent_t a, cudaEvent_t b);
struct Phase {
    const char *name;
    cudaStream_t st;
    cudaEvent_t a = nullptr, b = nullptr;
    Phase(const char *n, cudaStream_t s) : name(n), st(s) {
        if (profiling_enabled() && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
            cudaEventRecord(a, st);
        else
            a = b = nullptr;
    }
    ~Phase() {
        if (a && b) {
            cudaEventRecord(b, st);
            profile_record(name, a, b);
        }
    }
};

__host__ __device__ inline uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

// ------------------------------------------------------------------------------------
// kernel launchers (defined in the .cu files)
// ------------------------------------------------------------------------------------
// reductions / draws (mc_reduce.cu)
int launch_det_sum(const DetInput &in, double *chunk_tmp, double *out, cudaStream_t st);
int launch_det_draw(const DetInput &in, double *chunk_tmp, const double *u_dev, double u_host, int use_dev_u,
                    const double *fallback_vals, uint64_t *out_idx, cudaStream_t st);

// dense + CSR row statistics
int launch_row_sums_dense(const float *X, uint64_t n, uint64_t d, double *rowsum, float *rownorm, cudaStream_t st);
int launch_row_sums_csr(const float *vals, const uint64_t *indptr, uint64_t n, double *rowsum, cudaStream_t st);

}  // namespace mc
