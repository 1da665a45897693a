// Deterministic reductions, D^2 draws, row statistics, the stable counting sort of rows by
// cluster, and the chunked centroid sums.
//
// Reference behaviour these kernels implement:
//  * objective totals: perform_hard_clustering's compute_cost (clustering/solve.h:120-123);
//  * D^2 draws: kmeanspp's sampling step (optim/kmeans.h:115-135) and the empty-cluster
//    restart (clustering/centroid.h:687-713), as an FP64 inverse CDF on a supplied uniform;
//  * centroid sums: set_centroids_full_mean + set_center (clustering/centroid.h:81-178,
//    649-779): rows bucketed by assignment in ascending order, weighted mean per bucket.
#include "mc_reduce.cuh"

#include <algorithm>
#include <cstdlib>
#include <vector>

namespace mc {

// ------------------------------------------------------------------------------------
// Deterministic FP64 sums and draws.  Chunks of 8192 consecutive elements (zeros past n);
// inside a chunk a pairwise tree over consecutive elements (level 1 adds elements 2i and
// 2i+1, level 2 adds those sums pairwise, ... 13 levels); the chunk totals, padded with
// zeros to a power of two P, are the leaves of the same pairwise tree.  Every sum is a tree
// of depth log2(n), so no step waits on a long chain of dependent FP64 adds (each costs
// about 75 ns on this GPU).  The scratch holds the top tree in heap layout: node j has
// children 2j and 2j+1, the leaves (chunk totals) sit at [P, 2P).
// ------------------------------------------------------------------------------------
// pairwise sum of 32 consecutive elements held one per lane; the result is in lane 0
__device__ __forceinline__ double lane_pairwise32(double v) {
#pragma unroll
    for (int sft = 1; sft < 32; sft <<= 1) v = v + __shfl_down_sync(0xffffffffu, v, sft);
    return v;
}

// pairwise sum of the 32 consecutive elements [b, b + 32) in registers (31 adds: GB300 issues
// about two FP64 adds per SM clock, so no add is spent on idle lanes)
__device__ __forceinline__ double det_block32(const DetInput &in, uint64_t b) {
    double v[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) v[e] = b + e < in.n ? in.get(b + e) : 0.0;
#pragma unroll
    for (int sft = 1; sft < 32; sft <<= 1)
#pragma unroll
        for (int e = 0; e < 32; e += 2 * sft) v[e] = v[e] + v[e + sft];
    return v[0];
}

// one CTA of 256 threads per chunk: thread t sums elements [32t, 32t + 32) of the chunk, the
// lanes' block sums go pairwise to lane 0 (1024 elements per warp), the 8 warp totals
// pairwise to the chunk total in leaves[g]
__global__ void __launch_bounds__(kDetThreads) k_det_chunks(DetInput in, double *leaves) {
    __shared__ double wt[kDetThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double b = det_block32(in, uint64_t(blockIdx.x) * kDetChunk + uint64_t(threadIdx.x) * 32);
    b = lane_pairwise32(b);
    if (lane == 0) wt[w] = b;
    __syncthreads();
    if (threadIdx.x == 0)
        leaves[blockIdx.x] = ((wt[0] + wt[1]) + (wt[2] + wt[3])) + ((wt[4] + wt[5]) + (wt[6] + wt[7]));
}

// block-wide: zero-pads the leaves [P + G, 2P) and builds the internal nodes [1, P) of the
// heap T (shared or global memory; every thread of the block calls it)
__device__ void det_heap_build(double *T, uint64_t P, uint64_t G) {
    for (uint64_t j = P + G + threadIdx.x; j < 2 * P; j += blockDim.x) T[j] = 0.0;
    __syncthreads();
    for (uint64_t lv = P >> 1; lv >= 1; lv >>= 1) {
        for (uint64_t j = lv + threadIdx.x; j < 2 * lv; j += blockDim.x) T[j] = T[2 * j] + T[2 * j + 1];
        __syncthreads();
    }
}

constexpr uint64_t kDetSmemLeaves = 2048;  // tree in shared memory up to this many leaves

__global__ void __launch_bounds__(kDetThreads) k_det_final(double *tree, uint64_t P, uint64_t G, double *out) {
    __shared__ double sT[2 * kDetSmemLeaves];
    double *T = tree;
    if (P <= kDetSmemLeaves) {
        for (uint64_t g = threadIdx.x; g < G; g += blockDim.x) sT[P + g] = tree[P + g];
        T = sT;
    }
    det_heap_build(T, P, G);
    if (threadIdx.x == 0) *out = T[1];
}

int launch_det_sum(const DetInput &in, double *chunk_tmp, double *out, cudaStream_t st) {
    const uint64_t G = det_chunks(in.n), P = det_leaves(in.n);
    if (G == 0) {
        MC_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), st));
        return MC_OK;
    }
    k_det_chunks<<<unsigned(G), kDetThreads, 0, st>>>(in, chunk_tmp + P), note_launch();
    k_det_final<<<1, kDetThreads, 0, st>>>(chunk_tmp, P, G, out), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// det draw: chunk totals (k_det_chunks), then one CTA builds the top tree, descends it with
// r = u * S to a chunk, recomputes that chunk's 256 sums of 32 elements (the same pairwise
// arithmetic as k_det_chunks), descends their tree to a 32-element block and that block's
// tree to one element.  If the total is not positive, the first maximum of fallback_vals
// (or index 0) is taken, as kmeanspp's argmax fallback does (kmeans.h:179-186).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kDetThreads) k_det_draw(DetInput in, double *tree, const double *u_dev,
                                                          double u_host, int use_dev_u, const double *fallback_vals,
                                                          uint64_t *out_idx) {
    __shared__ double sT[2 * kDetSmemLeaves];
    __shared__ double H[2 * kDetThreads];
    __shared__ double E[64];
    __shared__ uint64_t sm_g, sm_b;
    __shared__ double sm_r;
    __shared__ int sm_pos;
    const int t = threadIdx.x;
    const uint64_t G = det_chunks(in.n), P = det_leaves(in.n);
    double *T = tree;
    if (P <= kDetSmemLeaves) {
        for (uint64_t g = t; g < G; g += blockDim.x) sT[P + g] = tree[P + g];
        T = sT;
    }
    det_heap_build(T, P, G);
    if (t == 0) {
        const double S = T[1];
        sm_pos = S > 0.0;
        if (S > 0.0) {
            double r = (use_dev_u ? *u_dev : u_host) * S;
            sm_g = det_heap_descend(T, P, r);
            sm_r = r;
        }
    }
    __syncthreads();
    if (!sm_pos) {  // total not positive: argmax fallback (first maximum) over fallback_vals
        if (t == 0) {
            uint64_t am = 0;
            if (fallback_vals) {
                for (uint64_t i = 1; i < in.n; ++i)
                    if (fallback_vals[i] > fallback_vals[am]) am = i;
            }
            *out_idx = am;
        }
        return;
    }
    // the chosen chunk: thread t sums its 32 consecutive elements pairwise (as k_det_chunks)
    const uint64_t base = sm_g * kDetChunk;
    H[kDetThreads + t] = det_block32(in, base + uint64_t(t) * 32);
    __syncthreads();
    det_heap_build(H, kDetThreads, kDetThreads);
    if (t == 0) {
        double r = sm_r;
        sm_b = det_heap_descend(H, kDetThreads, r);
        sm_r = r;
    }
    __syncthreads();
    if (t < 32) {  // the chosen block's 32 elements and their tree
        const uint64_t i = base + sm_b * 32 + t;
        E[32 + t] = i < in.n ? in.get(i) : 0.0;
        __syncwarp();
        for (int lv = 16; lv >= 1; lv >>= 1) {
            if (t < lv) E[lv + t] = E[2 * (lv + t)] + E[2 * (lv + t) + 1];
            __syncwarp();
        }
        if (t == 0) {
            double r = sm_r;
            uint64_t res = base + sm_b * 32 + det_heap_descend(E, 32, r);
            if (res >= in.n) res = 0;
            *out_idx = res;
        }
    }
}

int launch_det_draw(const DetInput &in, double *chunk_tmp, const double *u_dev, double u_host, int use_dev_u,
                    const double *fallback_vals, uint64_t *out_idx, cudaStream_t st) {
    const uint64_t G = det_chunks(in.n), P = det_leaves(in.n);
    if (G > 0) k_det_chunks<<<unsigned(G), kDetThreads, 0, st>>>(in, chunk_tmp + P), note_launch();
    k_det_draw<<<1, kDetThreads, 0, st>>>(in, chunk_tmp, u_dev, u_host, use_dev_u, fallback_vals, out_idx), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// row statistics: sequential FP64 row sums (and float squared norms for dense rows)
// ------------------------------------------------------------------------------------
__global__ void k_row_sums_dense(const float *__restrict__ X, uint64_t n, uint64_t d, double *rowsum,
                                 float *rownorm) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const float *r = X + i * d;
    float q = 0.f;
    if (rowsum) {
        double s = 0.0;
        for (uint64_t j = 0; j < d; ++j) {
            const float v = r[j];
            s = s + double(v);
            q = fmaf(v, v, q);
        }
        rowsum[i] = s;
    } else {  // norms only: no FP64 work (about two FP64 adds per SM clock on this GPU)
        for (uint64_t j = 0; j < d; ++j) q = fmaf(r[j], r[j], q);
    }
    if (rownorm) rownorm[i] = q;
}

__global__ void k_row_sums_csr(const float *__restrict__ vals, const uint64_t *__restrict__ indptr, uint64_t n,
                               double *rowsum) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (uint64_t p = indptr[i]; p < indptr[i + 1]; ++p) s = s + double(vals[p]);
    rowsum[i] = s;
}

// norms only, rows of d % 4 == 0 floats at 16-byte alignment: the CTA's 128 rows are staged
// 32 columns at a time through shared memory with coalesced cp.async (double buffered), and
// each thread keeps its row's sequential fmaf chain (k_row_sums_dense reads a row per thread
// straight from global memory: 32 rows per load instruction, about 1.2 TB/s)
__global__ void __launch_bounds__(128) k_row_norms_staged(const float *__restrict__ X, uint64_t n, uint64_t d,
                                                          float *rownorm) {
    __shared__ __align__(16) float xs[2][128][36];
    const int t = threadIdx.x;
    const uint64_t row0 = uint64_t(blockIdx.x) * 128;
    const uint64_t nchunk = (d + 31) / 32;
    auto stage = [&](uint64_t ci, int buf) {
        const uint64_t k0 = ci * 32;
        const int kmax = int(umin64(32, d - k0));
        for (int e = t; e < 128 * 8; e += 128) {
            const int r = e >> 3, q4 = e & 7;
            const bool ok = row0 + r < n && 4 * q4 < kmax;
            const float *src = ok ? X + (row0 + r) * d + k0 + 4 * q4 : X;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(uint32_t(__cvta_generic_to_shared(
                             &xs[buf][r][4 * q4]))),
                         "l"(src), "r"(ok ? 16 : 0)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    float q = 0.f;
    stage(0, 0);
    for (uint64_t ci = 0; ci < nchunk; ++ci) {
        const int buf = int(ci & 1);
        if (ci + 1 < nchunk) {
            stage(ci + 1, buf ^ 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const int kmax = int(umin64(32, d - ci * 32));
        for (int kk = 0; kk < kmax; ++kk) {
            const float v = xs[buf][t][kk];
            q = fmaf(v, v, q);
        }
        __syncthreads();
    }
    if (row0 + t < n) rownorm[row0 + t] = q;
}

int launch_row_sums_dense(const float *X, uint64_t n, uint64_t d, double *rowsum, float *rownorm, cudaStream_t st) {
    if (n == 0) return MC_OK;
    if (!rowsum && rownorm && d % 4 == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0) {
        k_row_norms_staged<<<unsigned((n + 127) / 128), 128, 0, st>>>(X, n, d, rownorm), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    }
    k_row_sums_dense<<<unsigned((n + 127) / 128), 128, 0, st>>>(X, n, d, rowsum, rownorm), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

int launch_row_sums_csr(const float *vals, const uint64_t *indptr, uint64_t n, double *rowsum, cudaStream_t st) {
    if (n == 0) return MC_OK;
    k_row_sums_csr<<<unsigned((n + 127) / 128), 128, 0, st>>>(vals, indptr, n, rowsum), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// Stable counting sort of rows by cluster id.
// keys[i] in [0,k); optional keys2[i] (second membership, 0xffffffff = none).
// Tiles of kSortTile rows; per-tile counts (key-major: tile_counts[key][tile]) -> per
// (key, tile) offsets by a parallel scan per key -> one warp per tile scatters its rows in
// order (match_any ranks), so each bucket lists rows ascending.
// ------------------------------------------------------------------------------------
// per-tile counts; a shared-memory histogram when k is small enough
constexpr uint32_t kSmemKeys = 8192;

__global__ void k_sort_count(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ keys2, uint64_t n,
                             uint32_t k, uint64_t ntiles, uint32_t *tile_counts /* [k][ntiles] */) {
    __shared__ uint32_t hist[kSmemKeys];
    const uint64_t tile = blockIdx.x;
    const uint64_t b = tile * kSortTile, e = umin64(n, b + kSortTile);
    const bool sm = k <= kSmemKeys;
    if (sm) {
        for (uint32_t j = threadIdx.x; j < k; j += blockDim.x) hist[j] = 0;
        __syncthreads();
    }
    for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const uint32_t k1 = keys[i];
        if (sm) atomicAdd(&hist[k1], 1u);
        else atomicAdd(&tile_counts[uint64_t(k1) * ntiles + tile], 1u);
        if (keys2) {
            const uint32_t k2 = keys2[i];
            if (k2 != 0xffffffffu) {
                if (sm) atomicAdd(&hist[k2], 1u);
                else atomicAdd(&tile_counts[uint64_t(k2) * ntiles + tile], 1u);
            }
        }
    }
    if (sm) {
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < k; j += blockDim.x) tile_counts[uint64_t(j) * ntiles + tile] = hist[j];
    }
}

// one CTA per key: exclusive scan of the key's tile counts (in place: per-tile offsets
// relative to the bucket start) and the bucket total
__global__ void __launch_bounds__(256) k_sort_key_scan(uint32_t *tile_counts, uint64_t ntiles, uint32_t k,
                                                       uint64_t *bucket_count) {
    __shared__ uint64_t wsum[8];
    const uint32_t key = blockIdx.x;
    if (key >= k) return;
    uint32_t *row = tile_counts + uint64_t(key) * ntiles;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint64_t per = (ntiles + 255) / 256;
    const uint64_t b = uint64_t(t) * per, e = umin64(ntiles, b + per);
    uint64_t s = 0;
    for (uint64_t i = b; i < e; ++i) s += row[i];
    // exclusive scan of the 256 thread sums
    uint64_t incl = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint64_t v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    uint64_t wbase = 0;
    for (int i = 0; i < w; ++i) wbase += wsum[i];
    uint64_t acc = wbase + incl - s;
    for (uint64_t i = b; i < e; ++i) {
        const uint32_t c = row[i];
        row[i] = uint32_t(acc);
        acc += c;
    }
    if (t == 255) bucket_count[key] = acc;
}

// exclusive scan of up to a few thousand counts (single CTA of 1024 threads): per-thread
// sequential runs, then a parallel scan of the 1024 run totals (warp shuffles, 32 warp
// totals); out[m] = total.  div > 0 scans ceil(in[i] / div) instead (chunks per bucket).
__global__ void __launch_bounds__(1024) k_exclusive_scan_u64(const uint64_t *in, uint64_t *out, uint64_t m,
                                                             uint64_t div) {
    __shared__ uint64_t wtot[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint64_t per = (m + blockDim.x - 1) / blockDim.x;
    const uint64_t b = t * per, e = umin64(m, b + per);
    uint64_t s = 0;
    for (uint64_t i = b; i < e; ++i) s += div ? (in[i] + div - 1) / div : in[i];
    uint64_t inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint64_t v = lane < int(blockDim.x >> 5) ? wtot[lane] : 0, vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < int(blockDim.x >> 5)) wtot[lane] = vi - v;  // exclusive warp offsets
        if (lane == 31) out[m] = vi;
    }
    __syncthreads();
    uint64_t acc = wtot[w] + inc - s;
    for (uint64_t i = b; i < e; ++i) {
        const uint64_t v = div ? (in[i] + div - 1) / div : in[i];
        out[i] = acc;
        acc += v;
    }
}

__global__ void k_sort_scatter(const uint32_t *__restrict__ keys, uint64_t n, uint32_t k, uint64_t ntiles,
                               uint32_t *tile_offsets, const uint64_t *__restrict__ bucket_start, uint32_t *perm) {
    // one warp per tile; rows in order, 32 at a time; ranks from match_any.  Cursors live in
    // dynamic shared memory sized to k when k <= kSmemKeys (so that many one-warp blocks fit
    // on an SM), else in the tile's column of tile_offsets (stride ntiles).  The keys of 16
    // rounds are loaded ahead of their use.
    extern __shared__ uint32_t scur[];
    const uint64_t tile = blockIdx.x;
    const int lane = threadIdx.x & 31;
    const uint64_t b = tile * kSortTile;
    if (b >= n) return;
    const uint64_t e = umin64(n, b + kSortTile);
    const bool sm = k <= kSmemKeys;
    if (sm) {
        for (uint32_t j = lane; j < k; j += 32) scur[j] = tile_offsets[uint64_t(j) * ntiles + tile];
        __syncwarp();
    }
    uint32_t *cur = sm ? scur : tile_offsets + tile;
    const uint64_t cstride = sm ? 1 : ntiles;
    const unsigned lt = (1u << lane) - 1u;
    for (uint64_t base0 = b; base0 < e; base0 += 32 * 16) {
        uint32_t kr[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const uint64_t i = base0 + uint64_t(r) * 32 + lane;
            kr[r] = i < e ? keys[i] : 0xffffffffu;
        }
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const uint64_t i = base0 + uint64_t(r) * 32 + lane;
            const bool act = i < e;
            const uint32_t key = kr[r];
            const unsigned actmask = __ballot_sync(0xffffffffu, act);
            if (!actmask) break;
            const unsigned peers = __match_any_sync(0xffffffffu, key) & actmask;
            uint32_t off = 0;
            if (act) off = cur[uint64_t(key) * cstride];
            __syncwarp();
            if (act) {
                perm[bucket_start[key] + off + __popc(peers & lt)] = uint32_t(i);
                if ((peers & lt) == 0) cur[uint64_t(key) * cstride] = off + __popc(peers);
            }
            __syncwarp();
        }
    }
}

// Rare path (rows with a second membership after an empty-cluster restart): one thread
// per tile walks its rows in order so that every bucket stays ascending.
__global__ void k_sort_scatter2(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ keys2, uint64_t n,
                                uint32_t k, uint64_t ntiles, uint32_t *tile_offsets,
                                const uint64_t *__restrict__ bucket_start, uint32_t *perm) {
    const uint64_t tile = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    const uint64_t b = tile * kSortTile;
    if (b >= n) return;
    const uint64_t e = umin64(n, b + kSortTile);
    uint32_t *cur = tile_offsets + tile;
    for (uint64_t i = b; i < e; ++i) {
        const uint32_t k1 = keys[i], k2 = keys2[i];
        perm[bucket_start[k1] + cur[uint64_t(k1) * ntiles]++] = uint32_t(i);
        if (k2 != 0xffffffffu) perm[bucket_start[k2] + cur[uint64_t(k2) * ntiles]++] = uint32_t(i);
    }
}

// long integer scans (row lists, flags over n rows): tiles of 4096 values, 16 consecutive per
// thread; tile totals, one CTA scans them, then every tile writes its values
constexpr int kScanTile = 4096;

__device__ __forceinline__ uint64_t block_exclusive_scan_u64(uint64_t v, uint64_t *warp_tot) {
    // exclusive scan over the 256 threads of the block; warp_tot: 8 slots of shared memory
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    uint64_t before = 0;
    for (int q = 0; q < w; ++q) before += warp_tot[q];
    __syncthreads();
    return before + inc - v;
}

__global__ void __launch_bounds__(256) k_scan_tile_sums(const uint64_t *__restrict__ in, uint64_t m, uint64_t *tile_sum) {
    __shared__ uint64_t wt[8];
    const uint64_t b = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * 16;
    uint64_t s = 0;
#pragma unroll
    for (int e = 0; e < 16; ++e)
        if (b + e < m) s += in[b + e];
    const uint64_t ex = block_exclusive_scan_u64(s, wt);
    if (threadIdx.x == 255) tile_sum[blockIdx.x] = ex + s;
}

__global__ void __launch_bounds__(256) k_scan_tile_write(const uint64_t *__restrict__ in, uint64_t m,
                                                         const uint64_t *__restrict__ tile_off, uint64_t *out) {
    __shared__ uint64_t wt[8];
    const uint64_t b = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * 16;
    uint64_t v[16], s = 0;
#pragma unroll
    for (int e = 0; e < 16; ++e) {
        v[e] = b + e < m ? in[b + e] : 0;
        s += v[e];
    }
    uint64_t acc = tile_off[blockIdx.x] + block_exclusive_scan_u64(s, wt);
#pragma unroll
    for (int e = 0; e < 16; ++e) {
        if (b + e < m) out[b + e] = acc;
        acc += v[e];
    }
}

int launch_exclusive_scan_u64(const uint64_t *in, uint64_t *out, uint64_t m, cudaStream_t st, DBuf<uint64_t> *scratch) {
    if (m <= 16 * 1024) {  // one CTA
        k_exclusive_scan_u64<<<1, 1024, 0, st>>>(in, out, m, 0), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    }
    const uint64_t nt = (m + kScanTile - 1) / kScanTile;
    DBuf<uint64_t> own;  // freed in stream order
    DBuf<uint64_t> &buf = scratch ? *scratch : own;
    MC_TRY(buf.alloc(2 * nt + 1, st));
    uint64_t *tsum = buf.p, *toff = buf.p + nt;
    k_scan_tile_sums<<<unsigned(nt), 256, 0, st>>>(in, m, tsum), note_launch();
    k_exclusive_scan_u64<<<1, 1024, 0, st>>>(tsum, toff, nt, 0), note_launch();
    k_scan_tile_write<<<unsigned(nt), 256, 0, st>>>(in, m, toff, out), note_launch();
    MC_CUDA_TRY(cudaMemcpyAsync(out + m, toff + nt, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

int launch_sort_by_key(const uint32_t *keys, const uint32_t *keys2, uint64_t n, uint32_t k, SortWork &w,
                       cudaStream_t st) {
    const uint64_t ntiles = (n + kSortTile - 1) / kSortTile;
    MC_TRY(w.tile_counts.alloc(ntiles * k, st));
    MC_TRY(w.bucket_count.alloc(k, st));
    MC_TRY(w.bucket_start.alloc(uint64_t(k) + 1, st));
    MC_TRY(w.perm.alloc(keys2 ? 2 * n : n, st));
    if (k > kSmemKeys) MC_CUDA_TRY(cudaMemsetAsync(w.tile_counts.p, 0, ntiles * k * sizeof(uint32_t), st));
    if (ntiles)
        k_sort_count<<<unsigned(ntiles), 256, 0, st>>>(keys, keys2, n, k, ntiles, w.tile_counts.p), note_launch();
    else
        MC_CUDA_TRY(cudaMemsetAsync(w.bucket_count.p, 0, k * sizeof(uint64_t), st));
    if (ntiles) k_sort_key_scan<<<k, 256, 0, st>>>(w.tile_counts.p, ntiles, k, w.bucket_count.p), note_launch();
    k_exclusive_scan_u64<<<1, 1024, 0, st>>>(w.bucket_count.p, w.bucket_start.p, k, 0), note_launch();
    if (ntiles) {
        if (!keys2)
            k_sort_scatter<<<unsigned(ntiles), 32, k <= kSmemKeys ? k * sizeof(uint32_t) : 0, st>>>(
                keys, n, k, ntiles, w.tile_counts.p, w.bucket_start.p,
                                                            w.perm.p), note_launch();
        else
            k_sort_scatter2<<<unsigned((ntiles + 63) / 64), 64, 0, st>>>(keys, keys2, n, k, ntiles,
                                                                         w.tile_counts.p, w.bucket_start.p,
                                                                         w.perm.p), note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// Centroid sums.  Chunks: bucket c is split into ceil(cnt_c / ch) chunks of ch rows.
// chunk_start[c] = exclusive scan of the chunk counts (computed on device); a grid of
// ceil(n/ch)+k CTAs maps its chunk id by binary search, extra CTAs exit.
// ------------------------------------------------------------------------------------
__device__ inline uint32_t find_bucket(const uint64_t *chunk_start, uint32_t k, uint64_t q) {
    // largest c with chunk_start[c] <= q (chunk_start has k+1 entries, nondecreasing)
    uint32_t lo = 0, hi = k;  // invariant: chunk_start[lo] <= q < chunk_start[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (chunk_start[mid] <= q) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ inline void two_sum_add(float &s, float &e, float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    s = t;
    e = __fadd_rn(e, err);
}

// dense: one CTA per chunk (at most kDenseChunk rows of one cluster), threads over
// columns, rows sequential.  The chunk's row ids are staged in shared memory and each
// thread loads 8 rows' values ahead of its sequential sum, so the loads overlap.
constexpr uint64_t kDenseChunk = 256;

__global__ void __launch_bounds__(128) k_centroid_chunks_dense(const float *__restrict__ X, uint64_t d,
                                                               const uint32_t *__restrict__ perm,
                                                               const uint64_t *__restrict__ bucket_start,
                                                               const uint64_t *__restrict__ bucket_count,
                                                               const uint64_t *__restrict__ chunk_start, uint32_t k,
                                                               uint64_t ch, const double *__restrict__ w,
                                                               double *partial /* [chunk][d] */,
                                                               double *partial_w /* [chunk] */) {
    __shared__ uint32_t srows[kDenseChunk];
    __shared__ double sw[kDenseChunk];
    const uint64_t q = blockIdx.x;
    if (q >= chunk_start[k]) return;
    const uint32_t c = find_bucket(chunk_start, k, q);
    const uint64_t local = q - chunk_start[c];
    const uint64_t r0 = local * ch, r1 = umin64(bucket_count[c], r0 + ch);
    const int cnt = int(r1 - r0);
    const uint32_t *rows = perm + bucket_start[c] + r0;
    for (int r = threadIdx.x; r < cnt; r += blockDim.x) {
        srows[r] = rows[r];
        if (w) sw[r] = w[rows[r]];
    }
    __syncthreads();
    constexpr int U = 8;
    for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) {
        if (w) {
            double acc = 0.0;
            for (int r = 0; r < cnt; r += U) {
                float xv[U];
#pragma unroll
                for (int u = 0; u < U; ++u) xv[u] = (r + u < cnt) ? X[uint64_t(srows[r + u]) * d + j] : 0.f;
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (r + u < cnt) acc = fma(sw[r + u], double(xv[u]), acc);
            }
            partial[q * d + j] = acc;
        } else {
            float s = 0.f, e = 0.f;
            for (int r = 0; r < cnt; r += U) {
                float xv[U];
#pragma unroll
                for (int u = 0; u < U; ++u) xv[u] = (r + u < cnt) ? X[uint64_t(srows[r + u]) * d + j] : 0.f;
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (r + u < cnt) two_sum_add(s, e, xv[u]);
            }
            partial[q * d + j] = double(s) + double(e);
        }
    }
    if (w && threadIdx.x == 0) {
        double wq = 0.0;
        for (int r = 0; r < cnt; ++r) wq = wq + sw[r];
        partial_w[q] = wq;
    }
}

// CSR: one CTA per (chunk, column band); dense band accumulator in shared memory.
// Rows are visited in order; within a row every nonzero touches a distinct column, so
// each column's additions happen in row order.  The rows are software-pipelined: a row's
// nonzeros (up to 256 * kCsrRowRegs of them) are loaded into registers while the previous
// row is added, and the row bounds two rows ahead, so that the DRAM latency of the next
// row overlaps the work on the current one (a third buffer measured no faster).
constexpr int kCsrRowRegs = 8;

struct CsrRowRegs {
    uint32_t ci[kCsrRowRegs];
    float cv[kCsrRowRegs];
};

__device__ __forceinline__ void csr_row_bounds(const uint32_t *rows, const uint64_t *indptr, const double *w,
                                               uint64_t r, uint64_t r1, uint64_t &pb, uint64_t &pe, double &wr) {
    pb = pe = 0;
    wr = 0.0;
    if (r < r1) {
        const uint32_t row = rows[r];
        pb = indptr[row];
        pe = indptr[row + 1];
        if (w) wr = w[row];
    }
}

__device__ __forceinline__ void csr_row_load(const float *vals, const uint32_t *idx, uint64_t pb, uint64_t pe,
                                             CsrRowRegs &b) {
#pragma unroll
    for (int i = 0; i < kCsrRowRegs; ++i) {
        const uint64_t p = pb + threadIdx.x + 256u * i;
        if (p < pe) {
            b.ci[i] = idx[p];
            b.cv[i] = vals[p];
        }
    }
}

// adds one row into the band accumulator (weighted: FP64 fma into acc; else float TwoSum
// into s/e); nonzeros past the register window come straight from memory
__device__ __forceinline__ void csr_row_add(const float *vals, const uint32_t *idx, uint64_t pb, uint64_t pe,
                                            const CsrRowRegs &b, uint64_t j0, uint64_t j1, bool weighted,
                                            double wr, double *acc, float *s, float *e) {
#pragma unroll
    for (int i = 0; i < kCsrRowRegs; ++i) {
        const uint64_t p = pb + threadIdx.x + 256u * i;
        if (p < pe) {
            const uint32_t col = b.ci[i];
            if (col >= j0 && col < j1) {
                if (weighted) acc[col - j0] = fma(wr, double(b.cv[i]), acc[col - j0]);
                else two_sum_add(s[col - j0], e[col - j0], b.cv[i]);
            }
        }
    }
    for (uint64_t p = pb + threadIdx.x + 256u * kCsrRowRegs; p < pe; p += 256) {
        const uint32_t col = idx[p];
        if (col >= j0 && col < j1) {
            if (weighted) acc[col - j0] = fma(wr, double(vals[p]), acc[col - j0]);
            else two_sum_add(s[col - j0], e[col - j0], vals[p]);
        }
    }
}

__global__ void __launch_bounds__(256) k_centroid_chunks_csr(const float *__restrict__ vals,
                                                             const uint32_t *__restrict__ idx,
                                                             const uint64_t *__restrict__ indptr, uint64_t d,
                                                             uint64_t band, const uint32_t *__restrict__ perm,
                                                             const uint64_t *__restrict__ bucket_start,
                                                             const uint64_t *__restrict__ bucket_count,
                                                             const uint64_t *__restrict__ chunk_start, uint32_t k,
                                                             uint64_t ch, const double *__restrict__ w,
                                                             double *partial, double *partial_w) {
    extern __shared__ unsigned char smraw[];
    const uint64_t q = blockIdx.x;
    if (q >= chunk_start[k]) return;
    const uint32_t c = find_bucket(chunk_start, k, q);
    const uint64_t local = q - chunk_start[c];
    const uint64_t r0 = local * ch, r1 = umin64(bucket_count[c], r0 + ch);
    const uint32_t *rows = perm + bucket_start[c];
    const uint64_t j0 = blockIdx.y * band, j1 = umin64(d, j0 + band);
    const uint64_t bw = j1 - j0;
    const bool weighted = w != nullptr;
    double *acc = reinterpret_cast<double *>(smraw);
    float *s = reinterpret_cast<float *>(smraw);
    float *e = s + band;
    if (weighted) {
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x) acc[j] = 0.0;
    } else {
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x) { s[j] = 0.f; e[j] = 0.f; }
    }
    __syncthreads();
    CsrRowRegs A, B;
    uint64_t pbA, peA, pbB, peB, pbN, peN;
    double wA, wB, wN;
    csr_row_bounds(rows, indptr, w, r0, r1, pbA, peA, wA);
    csr_row_load(vals, idx, pbA, peA, A);
    csr_row_bounds(rows, indptr, w, r0 + 1, r1, pbB, peB, wB);
    for (uint64_t r = r0; r < r1; r += 2) {
        // A holds row r; B's bounds are row r + 1's
        csr_row_load(vals, idx, pbB, peB, B);
        csr_row_bounds(rows, indptr, w, r + 2, r1, pbN, peN, wN);
        csr_row_add(vals, idx, pbA, peA, A, j0, j1, weighted, wA, acc, s, e);
        __syncthreads();
        if (r + 1 >= r1) break;
        csr_row_load(vals, idx, pbN, peN, A);
        pbA = pbN, peA = peN, wA = wN;
        csr_row_bounds(rows, indptr, w, r + 3, r1, pbN, peN, wN);
        csr_row_add(vals, idx, pbB, peB, B, j0, j1, weighted, wB, acc, s, e);
        __syncthreads();
        pbB = pbN, peB = peN, wB = wN;
    }
    if (weighted) {
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x) partial[q * d + j0 + j] = acc[j];
        if (blockIdx.y == 0 && threadIdx.x == 0) {
            double wq = 0.0;
            for (uint64_t r = r0; r < r1; ++r) wq = wq + w[rows[r]];
            partial_w[q] = wq;
        }
    } else {
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x)
            partial[q * d + j0 + j] = double(s[j]) + double(e[j]);
    }
}

// The same for short rows (a few nonzeros each, where the register pipeline below costs
// more instructions per row than it saves): rows one after the other.
__global__ void k_centroid_chunks_csr_short(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                                      const uint64_t *__restrict__ indptr, uint64_t d, uint64_t band,
                                      const uint32_t *__restrict__ perm, const uint64_t *__restrict__ bucket_start,
                                      const uint64_t *__restrict__ bucket_count,
                                      const uint64_t *__restrict__ chunk_start, uint32_t k, uint64_t ch,
                                      const double *__restrict__ w, double *partial, double *partial_w) {
    extern __shared__ unsigned char smraw[];
    const uint64_t q = blockIdx.x;
    if (q >= chunk_start[k]) return;
    const uint32_t c = find_bucket(chunk_start, k, q);
    const uint64_t local = q - chunk_start[c];
    const uint64_t r0 = local * ch, r1 = umin64(bucket_count[c], r0 + ch);
    const uint32_t *rows = perm + bucket_start[c];
    const uint64_t j0 = blockIdx.y * band, j1 = umin64(d, j0 + band);
    const uint64_t bw = j1 - j0;
    if (w) {
        double *acc = reinterpret_cast<double *>(smraw);
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x) acc[j] = 0.0;
        __syncthreads();
        for (uint64_t r = r0; r < r1; ++r) {
            const uint32_t row = rows[r];
            const double wr = w[row];
            for (uint64_t p = indptr[row] + threadIdx.x; p < indptr[row + 1]; p += blockDim.x) {
                const uint32_t col = idx[p];
                if (col >= j0 && col < j1) acc[col - j0] = fma(wr, double(vals[p]), acc[col - j0]);
            }
            __syncthreads();
        }
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x) partial[q * d + j0 + j] = acc[j];
        if (blockIdx.y == 0 && threadIdx.x == 0) {
            double wq = 0.0;
            for (uint64_t r = r0; r < r1; ++r) wq = wq + w[rows[r]];
            partial_w[q] = wq;
        }
    } else {
        float *s = reinterpret_cast<float *>(smraw);
        float *e = s + band;
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x) { s[j] = 0.f; e[j] = 0.f; }
        __syncthreads();
        for (uint64_t r = r0; r < r1; ++r) {
            const uint32_t row = rows[r];
            for (uint64_t p = indptr[row] + threadIdx.x; p < indptr[row + 1]; p += blockDim.x) {
                const uint32_t col = idx[p];
                if (col >= j0 && col < j1) two_sum_add(s[col - j0], e[col - j0], vals[p]);
            }
            __syncthreads();
        }
        for (uint64_t j = threadIdx.x; j < bw; j += blockDim.x)
            partial[q * d + j0 + j] = double(s[j]) + double(e[j]);
    }
}

// The same sums for short rows and narrow bands (d <= 2048): the chunk's rows are taken
// kCsrTileRows at a time and scattered into a dense [rows][512 columns] tile in shared
// memory (rows in parallel, one warp each); then each thread walks its column down the tile
// in row order.  A column's additions are the same as in k_centroid_chunks_csr_short (every
// stored value of the column, rows ascending; a zero added by TwoSum or by the weighted fma
// leaves the sum unchanged, so empty tile cells are skipped), so the partials are
// bit-identical, but the rows of a batch are loaded concurrently instead of one dependent
// round trip per row.
constexpr int kCsrTileRows = 32, kCsrTileBand = 512;

__global__ void __launch_bounds__(kCsrTileBand) k_centroid_chunks_csr_tile(
    const float *__restrict__ vals, const uint32_t *__restrict__ idx, const uint64_t *__restrict__ indptr, uint64_t d,
    const uint32_t *__restrict__ perm, const uint64_t *__restrict__ bucket_start,
    const uint64_t *__restrict__ bucket_count, const uint64_t *__restrict__ chunk_start, uint32_t k, uint64_t ch,
    const double *__restrict__ w, double *partial, double *partial_w) {
    extern __shared__ __align__(16) float tile[];  // [kCsrTileRows][kCsrTileBand]
    __shared__ uint64_t rb[kCsrTileRows], re[kCsrTileRows];
    __shared__ double rw[kCsrTileRows];
    const uint64_t q = blockIdx.x;
    if (q >= chunk_start[k]) return;
    const uint32_t c = find_bucket(chunk_start, k, q);
    const uint64_t local = q - chunk_start[c];
    const uint64_t r0 = local * ch, r1 = umin64(bucket_count[c], r0 + ch);
    const uint32_t *rows = perm + bucket_start[c];
    const uint64_t j0 = uint64_t(blockIdx.y) * kCsrTileBand, j1 = umin64(d, j0 + kCsrTileBand);
    const int t = threadIdx.x, lane = t & 31, wp = t >> 5;
    constexpr int NW = kCsrTileBand / 32;
    const bool weighted = w != nullptr;
    for (int e = t; e < kCsrTileRows * kCsrTileBand; e += kCsrTileBand) tile[e] = 0.f;
    const uint64_t j = j0 + uint64_t(t);
    float s = 0.f, er = 0.f;
    double acc = 0.0, wq = 0.0;
    for (uint64_t b0 = r0; b0 < r1; b0 += kCsrTileRows) {
        const int nb = int(umin64(kCsrTileRows, r1 - b0));
        if (t < nb) {
            const uint32_t row = rows[b0 + t];
            rb[t] = indptr[row];
            re[t] = indptr[row + 1];
            if (weighted) rw[t] = w[row];
        }
        __syncthreads();
        for (int rr = wp; rr < nb; rr += NW)
            for (uint64_t p = rb[rr] + lane; p < re[rr]; p += 32) {
                const uint32_t col = idx[p];
                if (col >= j0 && col < j1) tile[rr * kCsrTileBand + int(col - j0)] = vals[p];
            }
        __syncthreads();
        if (j < j1) {
            for (int rr = 0; rr < nb; ++rr) {
                const float v = tile[rr * kCsrTileBand + t];
                if (v != 0.f) {
                    if (weighted) acc = fma(rw[rr], double(v), acc);
                    else two_sum_add(s, er, v);
                }
            }
        }
        if (weighted && t == 0 && blockIdx.y == 0)
            for (int rr = 0; rr < nb; ++rr) wq = wq + rw[rr];
        __syncthreads();
        for (int rr = wp; rr < nb; rr += NW)
            for (uint64_t p = rb[rr] + lane; p < re[rr]; p += 32) {
                const uint32_t col = idx[p];
                if (col >= j0 && col < j1) tile[rr * kCsrTileBand + int(col - j0)] = 0.f;
            }
        __syncthreads();
    }
    if (j < j1) partial[q * d + j] = weighted ? acc : double(s) + double(er);
    if (weighted && t == 0 && blockIdx.y == 0) partial_w[q] = wq;
}

// finalize: per (bucket, column): FP64 sum of chunk partials in order, divide, round.
// Buckets with one row copy the row (here for dense rows X; CSR rows in
// k_centroid_singletons_csr); empty buckets keep the old center.
__global__ void k_centroid_finalize(const double *__restrict__ partial, const double *__restrict__ partial_w,
                                    const uint64_t *__restrict__ chunk_start, const uint64_t *__restrict__ bucket_count,
                                    uint32_t k, uint64_t d, int weighted, float *centers, int *nan_flag,
                                    const float *__restrict__ X, const uint32_t *__restrict__ perm,
                                    const uint64_t *__restrict__ bucket_start) {
    const uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (j >= d) return;
    for (uint32_t c = blockIdx.y; c < k; c += gridDim.y) {
        const uint64_t cnt = bucket_count[c];
        if (cnt == 1 && X) centers[uint64_t(c) * d + j] = X[uint64_t(perm[bucket_start[c]]) * d + j];
        if (cnt <= 1) continue;  // empty: keep
        const uint64_t q0 = chunk_start[c], q1 = chunk_start[c + 1];
        double S = partial[q0 * d + j];
        for (uint64_t q = q0 + 1; q < q1; ++q) S = S + partial[q * d + j];
        double den;
        if (weighted) {
            den = partial_w[q0];
            for (uint64_t q = q0 + 1; q < q1; ++q) den = den + partial_w[q];
        } else {
            den = double(cnt);
        }
        const float v = float(S / den);
        centers[uint64_t(c) * d + j] = v;
        if (v != v) atomicExch(nan_flag, 1);
    }
}

// singleton buckets of CSR rows copy the row verbatim (centroid.h:761-768)
__global__ void k_centroid_singletons_csr(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                                          const uint64_t *__restrict__ indptr, uint64_t d, const uint32_t *perm,
                                          const uint64_t *bucket_start, const uint64_t *bucket_count, uint32_t k,
                                          float *centers) {
    for (uint32_t c = blockIdx.x; c < k; c += gridDim.x) {
        if (bucket_count[c] != 1) continue;
        const uint32_t row = perm[bucket_start[c]];
        float *dst = centers + uint64_t(c) * d;
        for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) dst[j] = 0.f;
        __syncthreads();
        for (uint64_t p = indptr[row] + threadIdx.x; p < indptr[row + 1]; p += blockDim.x) dst[idx[p]] = vals[p];
        __syncthreads();
    }
}

int launch_centroids(const CentroidArgs &a, SortWork &w, cudaStream_t st, bool presorted) {
    const uint64_t n = a.n, d = a.d;
    const uint32_t k = a.k;
    const uint64_t ch = a.csr ? 4096 : kDenseChunk;
    if (!presorted) MC_TRY(launch_sort_by_key(a.keys, a.keys2, n, k, w, st));
    MC_TRY(w.chunk_start.alloc(uint64_t(k) + 1, st));
    // chunk starts: exclusive scan of ceil(bucket count / ch)
    k_exclusive_scan_u64<<<1, 1024, 0, st>>>(w.bucket_count.p, w.chunk_start.p, k, ch), note_launch();
    const uint64_t members = n + (a.keys2 ? a.extra_members : 0);
    const uint64_t max_chunks = (members + ch - 1) / ch + k;
    MC_TRY(w.partial.alloc(max_chunks * d, st));
    MC_TRY(w.partial_w.alloc(max_chunks, st));
    if (!a.csr) {
        k_centroid_chunks_dense<<<unsigned(max_chunks), 128, 0, st>>>(a.X, d, w.perm.p, w.bucket_start.p,
                                                                     w.bucket_count.p, w.chunk_start.p, k, ch, a.w,
                                                                     w.partial.p, w.partial_w.p), note_launch();
    } else {
        const uint64_t band = a.w ? 12288 : 24576;  // 96 KB (double) or 192 KB (two floats)
        const uint64_t bw = band < d ? band : d;
        const size_t smem = a.w ? bw * sizeof(double) : 2 * bw * sizeof(float);
        const unsigned nb = unsigned((d + band - 1) / band);
        // always the largest band's size: a per-call value could be lowered by another host
        // thread between this call's set and its launch
        // rows of 32 or more nonzeros on average: the register-pipelined kernel
        if (a.nnz < 32 * n && d <= 4 * uint64_t(kCsrTileBand)) {
            // short rows over at most four 512-column bands: rows of a batch scattered into a
            // dense shared-memory tile, columns walked in row order
            const size_t tsm = size_t(kCsrTileRows) * kCsrTileBand * sizeof(float);
            MC_CUDA_TRY(cudaFuncSetAttribute(k_centroid_chunks_csr_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(tsm)));
            k_centroid_chunks_csr_tile<<<dim3(unsigned(max_chunks), unsigned((d + kCsrTileBand - 1) / kCsrTileBand)),
                                         kCsrTileBand, tsm, st>>>(a.vals, a.idx, a.indptr, d, w.perm.p,
                                                                  w.bucket_start.p, w.bucket_count.p,
                                                                  w.chunk_start.p, k, ch, a.w, w.partial.p,
                                                                  w.partial_w.p), note_launch();
        } else {
            auto kern = (a.nnz >= 32 * n) ? k_centroid_chunks_csr : k_centroid_chunks_csr_short;
            MC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(2 * 24576 * sizeof(float))));
            kern<<<dim3(unsigned(max_chunks), nb), 256, smem, st>>>(
                a.vals, a.idx, a.indptr, d, bw, w.perm.p, w.bucket_start.p, w.bucket_count.p, w.chunk_start.p, k,
                ch, a.w, w.partial.p, w.partial_w.p), note_launch();
        }
    }
    k_centroid_finalize<<<dim3(unsigned((d + 127) / 128), k < 65535 ? k : 65535), 128, 0, st>>>(
        w.partial.p, w.partial_w.p, w.chunk_start.p, w.bucket_count.p, k, d, a.w ? 1 : 0, a.centers, a.nan_flag,
        a.csr ? nullptr : a.X, w.perm.p, w.bucket_start.p), note_launch();
    if (a.csr)
        k_centroid_singletons_csr<<<k < 65535 ? k : 65535, 256, 0, st>>>(a.vals, a.idx, a.indptr, d, w.perm.p, w.bucket_start.p,
                                                     w.bucket_count.p, k, a.centers), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// per-center sums (sequential FP64 over columns) and squared norms
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_center_sums(const float *__restrict__ C, uint32_t k, uint64_t d, double *csum,
                                                     float *cnorm) {
    // one warp per center.  csum: lane l adds columns l, l+32, l+64, ... in FP64, then the 32
    // lane partials are added in lane order (the canonical center-sum order).  cnorm: a FP32
    // fmaf chain in column order, by lane 0 from coalesced shared-memory chunks.
    __shared__ float t[4][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t c = blockIdx.x * 4 + w;
    if (c >= k) return;  // whole warp; the block has no barrier
    const float *r = C + uint64_t(c) * d;
    double s = 0.0;
    float q = 0.f;
    for (uint64_t j0 = 0; j0 < d; j0 += 256) {
        const int cnt = int(d - j0 < 256 ? d - j0 : 256);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = lane + 32 * u;
            if (i < cnt) {
                const float x = r[j0 + i];
                s = s + double(x);
                if (cnorm) t[w][i] = x;
            }
        }
        if (cnorm) {
            __syncwarp();
            if (lane == 0) {
                if (cnt == 256) {
#pragma unroll 16
                    for (int i = 0; i < 256; ++i) q = fmaf(t[w][i], t[w][i], q);
                } else {
                    for (int i = 0; i < cnt; ++i) q = fmaf(t[w][i], t[w][i], q);
                }
            }
            __syncwarp();
        }
    }
    double tot = 0.0;
#pragma unroll
    for (int l = 0; l < 32; ++l) tot = tot + __shfl_sync(0xffffffffu, s, l);
    if (lane == 0) {
        csum[c] = tot;
        if (cnorm) cnorm[c] = q;
    }
}

int launch_center_sums(const float *C, uint32_t k, uint64_t d, double *csum, float *cnorm, cudaStream_t st) {
    if (k == 0) return MC_OK;
    k_center_sums<<<(k + 3) / 4, 128, 0, st>>>(C, k, d, csum, cnorm), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// L1 medians: one CTA (8 warps) per (cluster, 32 columns).  Unweighted: a 4-pass radix select
// (one byte of the order-preserving key per pass, histograms in shared memory) for the ranks
// (m - 1) / 2 and m / 2 at once.  Weighted: the largest weight of the cluster, then per
// column the smallest value among the rows that carry it.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t f2ord(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void __launch_bounds__(256) k_l1_median_dense(const float *__restrict__ X, uint64_t d,
                                                         const uint32_t *__restrict__ perm,
                                                         const uint64_t *__restrict__ bstart,
                                                         const uint64_t *__restrict__ bcount, float *centers) {
    extern __shared__ uint32_t hist[];  // [2][32][256]
    __shared__ uint32_t prefix[2][32];
    __shared__ uint64_t rank[2][32];
    const uint32_t c = blockIdx.x;
    const uint64_t c0 = uint64_t(blockIdx.y) * 32;
    const uint64_t m = bcount[c], b = bstart[c];
    if (m == 0) return;  // whole block
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint64_t col = c0 + lane;
    if (t < 64) {
        const int s = t >> 5;
        prefix[s][lane] = 0;
        rank[s][lane] = s == 0 ? (m - 1) / 2 : m / 2;
    }
    for (int pass = 3; pass >= 0; --pass) {
        for (int e = t; e < 2 * 32 * 256; e += 256) hist[e] = 0;
        __syncthreads();
        if (col < d) {
            const uint32_t p0 = prefix[0][lane], p1 = prefix[1][lane];
            for (uint64_t r = warp; r < m; r += 8) {
                const uint32_t key = f2ord(X[uint64_t(perm[b + r]) * d + col]);
                const uint32_t bin = (key >> (8 * pass)) & 255u;
                const bool top = pass == 3;
                if (top || (key >> (8 * (pass + 1))) == p0) atomicAdd(&hist[(0 * 32 + lane) * 256 + bin], 1u);
                if (top || (key >> (8 * (pass + 1))) == p1) atomicAdd(&hist[(1 * 32 + lane) * 256 + bin], 1u);
            }
        }
        __syncthreads();
        if (t < 64) {
            const int s = t >> 5;
            const uint32_t *h = hist + (s * 32 + lane) * 256;
            uint64_t rk = rank[s][lane], cum = 0;
            uint32_t bin = 255;
            for (uint32_t q = 0; q < 256; ++q) {
                if (cum + h[q] > rk) { bin = q; break; }
                cum += h[q];
            }
            rank[s][lane] = rk - cum;
            prefix[s][lane] = (prefix[s][lane] << 8) | bin;
        }
        __syncthreads();
    }
    if (t < 32 && col < d) {
        const float lo = ord2f(prefix[0][lane]), hi = ord2f(prefix[1][lane]);
        centers[uint64_t(c) * d + col] = (m & 1) ? hi : 0.5f * (lo + hi);
    }
}

__global__ void __launch_bounds__(256) k_l1_median_weighted(const float *__restrict__ X, uint64_t d,
                                                            const uint32_t *__restrict__ perm,
                                                            const uint64_t *__restrict__ bstart,
                                                            const uint64_t *__restrict__ bcount,
                                                            const double *__restrict__ w, uint64_t nw_local,
                                                            float *centers) {
    __shared__ double wmax[8];
    __shared__ uint32_t best[8][32];
    const uint32_t c = blockIdx.x;
    const uint64_t c0 = uint64_t(blockIdx.y) * 32;
    const uint64_t m = bcount[c], b = bstart[c];
    if (m == 0) return;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // nw_local > 0: the r-th row of the cluster weighs w[r] (w holds nw_local entries)
    auto wt = [&](uint64_t r) {
        if (nw_local) return r < nw_local ? w[r] : -1.7976931348623157e308;
        return w[perm[b + r]];
    };
    double mx = -1.7976931348623157e308;
    for (uint64_t r = t; r < m; r += 256) mx = fmax(mx, wt(r));
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) wmax[warp] = mx;
    __syncthreads();
    mx = wmax[0];
    for (int q = 1; q < 8; ++q) mx = fmax(mx, wmax[q]);
    const uint64_t col = c0 + lane;
    uint32_t bk = 0xffffffffu;
    if (col < d)
        for (uint64_t r = warp; r < m; r += 8) {
            const uint32_t row = perm[b + r];
            if (wt(r) == mx) bk = min(bk, f2ord(X[uint64_t(row) * d + col]));
        }
    best[warp][lane] = bk;
    __syncthreads();
    if (t < 32 && col < d) {
        uint32_t v = best[0][lane];
        for (int q = 1; q < 8; ++q) v = min(v, best[q][lane]);
        centers[uint64_t(c) * d + col] = ord2f(v);
    }
}

int launch_l1_medians(const float *X, uint64_t d, uint32_t k, const SortWork &w, const double *weights,
                      float *centers, cudaStream_t st, uint64_t nw_local) {
    if (k == 0 || d == 0) return MC_OK;
    const dim3 g(k, unsigned((d + 31) / 32));
    if (weights) {
        k_l1_median_weighted<<<g, 256, 0, st>>>(X, d, w.perm.p, w.bucket_start.p, w.bucket_count.p, weights,
                                               nw_local, centers), note_launch();
    } else {
        const int smem = 2 * 32 * 256 * int(sizeof(uint32_t));
        MC_CUDA_TRY(cudaFuncSetAttribute(k_l1_median_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        k_l1_median_dense<<<g, 256, smem, st>>>(X, d, w.perm.p, w.bucket_start.p, w.bucket_count.p, centers),
            note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

__global__ void k_l1_reseed_update(const float *__restrict__ X, uint64_t n, uint64_t d,
                                   const float *__restrict__ center, uint32_t id, uint32_t *asn, double *costs) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        const float *x = X + i * d;
        float a = 0.f;
        for (uint64_t j = 0; j < d; ++j) a = a + fabsf(center[j] - x[j]);
        if (double(a) < costs[i]) {
            asn[i] = id;
            costs[i] = double(a);
        }
    }
}

int launch_l1_reseed_update(const float *X, uint64_t n, uint64_t d, const float *center, uint32_t id,
                            uint32_t *asn, double *costs, cudaStream_t st) {
    if (n == 0) return MC_OK;
    k_l1_reseed_update<<<unsigned(umin64((n + 255) / 256, 4096)), 256, 0, st>>>(X, n, d, center, id, asn, costs),
        note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// ------------------------------------------------------------------------------------
// L1 medians over CSR rows
// ------------------------------------------------------------------------------------
// the new center is CSR row *rsel: the sequential sum over the union of the two rows' columns
// (a column where both are zero adds exactly 0), one thread per row
__global__ void k_l1_reseed_update_csr(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                                       const uint64_t *__restrict__ indptr, uint64_t n,
                                       const uint64_t *__restrict__ rsel, uint32_t id, uint32_t *asn,
                                       double *costs) {
    const uint64_t cb = indptr[*rsel], ce = indptr[*rsel + 1];
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += gridDim.x * uint64_t(blockDim.x)) {
        uint64_t p = indptr[i], q = cb;
        const uint64_t pe = indptr[i + 1];
        float a = 0.f;
        while (p < pe || q < ce) {
            const uint32_t rc = p < pe ? idx[p] : 0xffffffffu, cc = q < ce ? idx[q] : 0xffffffffu;
            const float x = rc <= cc ? vals[p] : 0.f, c = cc <= rc ? vals[q] : 0.f;
            a = a + fabsf(c - x);
            p += rc <= cc;
            q += cc <= rc;
        }
        if (double(a) < costs[i]) {
            asn[i] = id;
            costs[i] = double(a);
        }
    }
}

int launch_l1_reseed_update_csr(const float *vals, const uint32_t *idx, const uint64_t *indptr, uint64_t n,
                                const uint64_t *rsel, uint32_t id, uint32_t *asn, double *costs, cudaStream_t st) {
    if (n == 0) return MC_OK;
    k_l1_reseed_update_csr<<<unsigned(umin64((n + 255) / 256, 4096)), 256, 0, st>>>(vals, idx, indptr, n, rsel, id,
                                                                                   asn, costs), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

// one warp per row: the row's nonzeros as (cluster << 32 | column, value key), CSR order
__global__ void k_l1csr_fill(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                             const uint64_t *__restrict__ indptr, uint64_t n, const uint32_t *__restrict__ asn,
                             uint64_t *key, uint32_t *val) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    for (uint64_t r = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; r < n; r += nw) {
        const uint64_t hi = uint64_t(asn[r]) << 32, e = indptr[r + 1];
        for (uint64_t p = indptr[r] + lane; p < e; p += 32) {
            key[p] = hi | idx[p];
            val[p] = f2ord(vals[p]);
        }
    }
}

__global__ void k_l1csr_digit(const uint64_t *__restrict__ key, const uint32_t *__restrict__ val, uint64_t m,
                              int from_key, int shift, uint32_t mask, uint32_t *digit) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m; i += gridDim.x * uint64_t(blockDim.x))
        digit[i] = from_key ? uint32_t(key[i] >> shift) & mask : (val[i] >> shift) & mask;
}

__global__ void k_l1csr_gather(const uint32_t *__restrict__ perm, uint64_t m, const uint64_t *__restrict__ key,
                               const uint32_t *__restrict__ val, uint64_t *key2, uint32_t *val2) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < m; i += gridDim.x * uint64_t(blockDim.x)) {
        const uint32_t s = perm[i];
        key2[i] = key[s];
        val2[i] = val[s];
    }
}

// clusters of two or more rows start from zero (the median writes only the columns that
// have nonzeros); a cluster of one row takes that row
__global__ void k_l1csr_init(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                             const uint64_t *__restrict__ indptr, uint64_t d, const uint32_t *__restrict__ perm,
                             const uint64_t *__restrict__ bstart, const uint64_t *__restrict__ bcount,
                             float *centers) {
    const uint32_t c = blockIdx.x;
    const uint64_t m = bcount[c];
    if (m == 0) return;  // whole block
    float *dst = centers + uint64_t(c) * d;
    for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) dst[j] = 0.f;
    if (m != 1) return;  // whole block
    __syncthreads();
    const uint32_t r = perm[bstart[c]];
    for (uint64_t p = indptr[r] + threadIdx.x; p < indptr[r + 1]; p += blockDim.x) dst[idx[p]] = vals[p];
}

// the sparse median of one (cluster, column) run: v = the run's nel value keys, ascending;
// m = the cluster's rows.  Follows util/csc.h:856-890, including its choices: with more
// than m/2 nonzeros and m even it averages the sorted positions m/2 and m/2 + 1 (counting
// the zeros), the all-negative case reads one position past the middle, and an odd m with
// exactly m/2 nonzeros of one sign gives half the smallest (largest) of them.  Where the
// reference's position runs past the end of its vector (m = 2, or the all-negative case with
// nel = m/2 + 1) the last element stands in.
__device__ float l1csr_median(const uint32_t *__restrict__ v, uint64_t nel, uint64_t m) {
    const uint64_t h = m / 2;
    const float front = ord2f(v[0]), back = ord2f(v[nel - 1]);
    auto nz = [&](uint64_t q) { return ord2f(v[q < nel ? q : nel - 1]); };
    if (nel > h) {
        if (front > 0.f || back < 0.f) {
            const uint64_t t = front > 0.f ? nel + h - m : m - h;
            return (m & 1) ? nz(t) : 0.5f * (nz(t) + nz(t + 1));
        }
        // mixed signs (or stored zeros): the negatives, then m - nel zeros, then the rest
        uint64_t lo = 0, hi = nel;  // first key >= f2ord(-0.0)
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (v[mid] < 0x7fffffffu) lo = mid + 1;
            else hi = mid;
        }
        const uint64_t nneg = lo, z = m - nel;
        auto full = [&](uint64_t q) {
            if (q >= m) q = m - 1;
            return q < nneg ? ord2f(v[q]) : (q < nneg + z ? 0.f : ord2f(v[q - z]));
        };
        return (m & 1) ? full(h) : 0.5f * (full(h) + full(h + 1));
    }
    if ((m & 1) && nel == h) {
        if (front > 0.f) return 0.5f * front;
        if (back < 0.f) return 0.5f * back;
    }
    return 0.f;
}

__global__ void k_l1csr_runs(const uint64_t *__restrict__ key, const uint32_t *__restrict__ val, uint64_t nnz,
                             uint64_t d, const uint64_t *__restrict__ bcount, float *centers) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < nnz;
         i += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t kk = key[i];
        if (i > 0 && key[i - 1] == kk) continue;
        const uint32_t c = uint32_t(kk >> 32);
        const uint64_t m = bcount[c];
        if (m < 2) continue;
        // end of the run: galloping, then bisection (key[lo] == kk, key[hi] != kk or hi == nnz)
        uint64_t lo = i, hi = i + 1, step = 1;
        while (hi < nnz && key[hi] == kk) {
            lo = hi;
            step <<= 1;
            hi = lo + step;
        }
        if (hi > nnz) hi = nnz;
        while (hi - lo > 1) {
            const uint64_t mid = lo + (hi - lo) / 2;
            if (key[mid] == kk) lo = mid;
            else hi = mid;
        }
        centers[uint64_t(c) * d + uint32_t(kk)] = l1csr_median(val + i, hi - i, m);
    }
}

// Bucket path (k * d <= kL1BucketMax): the nonzeros of clusters with two or more rows are
// counted per (cluster, column) bucket, the counts scanned to offsets, and the value keys
// scattered into their bucket with atomic cursors (order within a bucket is irrelevant: only
// order statistics are read).  Buckets that need one (more than m/2 nonzeros, or an odd m
// with exactly m/2) are listed, and one CTA per listed bucket takes the minimum, maximum and
// negative count, then a 4-pass radix select of the (at most two) ranks the rule reads.
constexpr uint64_t kL1BucketMax = 1ull << 28;

__global__ void k_l1b_count(const uint32_t *__restrict__ idx, const uint64_t *__restrict__ indptr, uint64_t n,
                            uint64_t d, const uint32_t *__restrict__ asn, const uint64_t *__restrict__ bcount,
                            unsigned long long *cnt) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    for (uint64_t r = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; r < n; r += nw) {
        const uint32_t c = asn[r];
        if (bcount[c] < 2) continue;
        const uint64_t base = uint64_t(c) * d, e = indptr[r + 1];
        for (uint64_t p = indptr[r] + lane; p < e; p += 32) atomicAdd(&cnt[base + idx[p]], 1ull);
    }
}

__global__ void k_l1b_scatter(const float *__restrict__ vals, const uint32_t *__restrict__ idx,
                              const uint64_t *__restrict__ indptr, uint64_t n, uint64_t d,
                              const uint32_t *__restrict__ asn, const uint64_t *__restrict__ bcount,
                              unsigned long long *cur, uint32_t *keys) {
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (gridDim.x * uint64_t(blockDim.x)) >> 5;
    for (uint64_t r = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; r < n; r += nw) {
        const uint32_t c = asn[r];
        if (bcount[c] < 2) continue;
        const uint64_t base = uint64_t(c) * d, e = indptr[r + 1];
        for (uint64_t p = indptr[r] + lane; p < e; p += 32) keys[atomicAdd(&cur[base + idx[p]], 1ull)] = f2ord(vals[p]);
    }
}

__global__ void k_l1b_list(const unsigned long long *__restrict__ cnt, uint64_t nb, uint64_t d,
                           const uint64_t *__restrict__ bcount, unsigned long long *nrun, uint64_t *runs) {
    for (uint64_t b = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; b < nb; b += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t nel = cnt[b];
        if (!nel) continue;
        const uint64_t m = bcount[b / d], h = m / 2;
        if (m >= 2 && (nel > h || ((m & 1) && nel == h))) runs[atomicAdd(nrun, 1ull)] = b;
    }
}

__global__ void __launch_bounds__(256) k_l1b_select(const unsigned long long *__restrict__ nrun,
                                                    const uint64_t *__restrict__ runs,
                                                    const uint64_t *__restrict__ off,
                                                    const unsigned long long *__restrict__ cnt,
                                                    const uint32_t *__restrict__ keys, uint64_t d,
                                                    const uint64_t *__restrict__ bcount, float *centers) {
    __shared__ uint32_t hist[2][256];
    __shared__ uint32_t wmin[8], wmax[8];
    __shared__ uint64_t wneg[8];
    __shared__ uint32_t prefix[2];
    __shared__ uint64_t rank[2];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint64_t total = *nrun;
    for (uint64_t ri = blockIdx.x; ri < total; ri += gridDim.x) {
        const uint64_t b = runs[ri];
        const uint64_t c = b / d, col = b - c * d;
        const uint64_t m = bcount[c], h = m / 2, nel = cnt[b];
        const uint32_t *v = keys + off[b];
        uint32_t mn = 0xffffffffu, mx = 0u;
        uint64_t ng = 0;
        for (uint64_t i = t; i < nel; i += 256) {
            const uint32_t kv = v[i];
            mn = min(mn, kv);
            mx = max(mx, kv);
            ng += kv < 0x7fffffffu;  // strictly negative values
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            ng += __shfl_xor_sync(0xffffffffu, ng, o);
        }
        if (lane == 0) wmin[warp] = mn, wmax[warp] = mx, wneg[warp] = ng;
        __syncthreads();
        mn = wmin[0], mx = wmax[0], ng = wneg[0];
        for (int q = 1; q < 8; ++q) mn = min(mn, wmin[q]), mx = max(mx, wmax[q]), ng += wneg[q];
        const float front = ord2f(mn), back = ord2f(mx);
        // the ranks the rule reads, among the bucket's nonzeros (ascending); zero[s]: the
        // position falls on one of the m - nel implicit zeros
        uint64_t r[2] = {0, 0};
        bool zero[2] = {false, false};
        int nsel = 0;
        float result = 0.f;
        if (nel > h) {
            nsel = (m & 1) ? 1 : 2;
            if (front > 0.f || back < 0.f) {
                const uint64_t tt = front > 0.f ? nel + h - m : m - h;
                r[0] = tt < nel ? tt : nel - 1;
                r[1] = tt + 1 < nel ? tt + 1 : nel - 1;
            } else {
                const uint64_t z = m - nel, qq[2] = {h, h + 1 < m ? h + 1 : m - 1};
                for (int s2 = 0; s2 < 2; ++s2) {
                    const uint64_t q = qq[s2];
                    if (q < ng) r[s2] = q;
                    else if (q < ng + z) zero[s2] = true;
                    else r[s2] = q - z;
                }
            }
        } else {
            result = front > 0.f ? 0.5f * front : (back < 0.f ? 0.5f * back : 0.f);
        }
        if (nsel) {
            if (t < 2) prefix[t] = 0, rank[t] = r[t];
            for (int pass = 3; pass >= 0; --pass) {
                for (int e = t; e < 512; e += 256) (&hist[0][0])[e] = 0;
                __syncthreads();
                const uint32_t p0 = prefix[0], p1 = prefix[1];
                for (uint64_t i0 = 0; i0 < nel; i0 += 256) {
                    const uint64_t i = i0 + t;
                    const bool in = i < nel;
                    const uint32_t kv = in ? v[i] : 0u;
                    const uint32_t bin = (kv >> (8 * pass)) & 255u, hi = pass == 3 ? 0u : kv >> (8 * (pass + 1));
#pragma unroll
                    for (int s2 = 0; s2 < 2; ++s2) {
                        const bool hit = in && (pass == 3 || hi == (s2 ? p1 : p0));
                        // equal bins of a warp add once (count data repeats values)
                        const unsigned grp = __match_any_sync(0xffffffffu, hit ? bin : 0xffffffffu);
                        if (hit && (grp & ((1u << lane) - 1u)) == 0) atomicAdd(&hist[s2][bin], __popc(grp));
                    }
                }
                __syncthreads();
                if (t < 2) {
                    const uint32_t *hh = hist[t];
                    uint64_t rk = rank[t], cum = 0;
                    uint32_t bin = 255;
                    for (uint32_t q = 0; q < 256; ++q) {
                        if (cum + hh[q] > rk) { bin = q; break; }
                        cum += hh[q];
                    }
                    rank[t] = rk - cum;
                    prefix[t] = (prefix[t] << 8) | bin;
                }
                __syncthreads();
            }
            const float x0 = zero[0] ? 0.f : ord2f(prefix[0]), x1 = zero[1] ? 0.f : ord2f(prefix[1]);
            result = nsel == 1 ? x0 : 0.5f * (x0 + x1);
        }
        if (t == 0) centers[c * d + col] = result;
        __syncthreads();  // shared memory is reused by the next bucket
    }
}

namespace {
int bit_width(uint64_t x) {  // bits needed for values 0..x
    int b = 0;
    while (x >> b) ++b;
    return b;
}
}  // namespace

int launch_l1_medians_csr(const float *vals, const uint32_t *idx, const uint64_t *indptr, uint64_t n, uint64_t d,
                          uint64_t nnz, uint32_t k, const uint32_t *asn, const SortWork &rows, L1CsrWork &w,
                          float *centers, cudaStream_t st) {
    if (k == 0 || d == 0) return MC_OK;
    if (nnz >= (1ull << 32)) return fail(MC_EUNSUPPORTED, "CSR L1 medians take at most 2^32-1 nonzeros");
    k_l1csr_init<<<k, 256, 0, st>>>(vals, idx, indptr, d, rows.perm.p, rows.bucket_start.p, rows.bucket_count.p,
                                    centers), note_launch();
    if (nnz == 0) {
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    }
    const uint64_t nb = uint64_t(k) * d;
    const char *force = std::getenv("MC_L1CSR_SORT");
    if (nb <= kL1BucketMax && !(force && force[0] == '1')) {
        MC_TRY(w.cnt.alloc(nb, st));
        MC_TRY(w.off.alloc(nb + 1, st));
        MC_TRY(w.cur.alloc(nb, st));
        MC_TRY(w.runs.alloc(nb + 1, st));
        MC_TRY(w.val.alloc(nnz, st));
        unsigned long long *cnt = reinterpret_cast<unsigned long long *>(w.cnt.p);
        unsigned long long *cur = reinterpret_cast<unsigned long long *>(w.cur.p);
        unsigned long long *nrun = reinterpret_cast<unsigned long long *>(w.runs.p + nb);
        const unsigned gr = unsigned(umin64((n + 7) / 8, 152 * 16));
        MC_CUDA_TRY(cudaMemsetAsync(w.cnt.p, 0, nb * sizeof(uint64_t), st));
        k_l1b_count<<<gr, 256, 0, st>>>(idx, indptr, n, d, asn, rows.bucket_count.p, cnt), note_launch();
        MC_TRY(launch_exclusive_scan_u64(w.cnt.p, w.off.p, nb, st, &w.scan));
        MC_CUDA_TRY(cudaMemcpyAsync(w.cur.p, w.off.p, nb * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        k_l1b_scatter<<<gr, 256, 0, st>>>(vals, idx, indptr, n, d, asn, rows.bucket_count.p, cur, w.val.p),
            note_launch();
        MC_CUDA_TRY(cudaMemsetAsync(nrun, 0, sizeof(uint64_t), st));
        k_l1b_list<<<unsigned(umin64((nb + 255) / 256, 152 * 16)), 256, 0, st>>>(cnt, nb, d, rows.bucket_count.p,
                                                                                  nrun, w.runs.p), note_launch();
        k_l1b_select<<<152 * 8, 256, 0, st>>>(nrun, w.runs.p, w.off.p, cnt, w.val.p, d, rows.bucket_count.p,
                                              centers), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        return MC_OK;
    }
    MC_TRY(w.key.alloc(nnz, st));
    MC_TRY(w.key2.alloc(nnz, st));
    MC_TRY(w.val.alloc(nnz, st));
    MC_TRY(w.val2.alloc(nnz, st));
    MC_TRY(w.digit.alloc(nnz, st));
    const unsigned g = unsigned(umin64((nnz + 255) / 256, 152 * 16));
    k_l1csr_fill<<<unsigned(umin64((n + 7) / 8, 152 * 16)), 256, 0, st>>>(vals, idx, indptr, n, asn, w.key.p,
                                                                         w.val.p), note_launch();
    // LSD passes: (from_key, shift, bits), least significant field first
    struct Pass { int from_key, shift, bits; };
    std::vector<Pass> passes;
    auto field = [&](int from_key, int base, int bits) {
        const int np = (bits + 10) / 11;
        for (int q = 0, done = 0; q < np; ++q) {
            const int b = (bits - done + (np - q) - 1) / (np - q);
            passes.push_back({from_key, base + done, b});
            done += b;
        }
    };
    field(0, 0, 32);
    field(1, 0, std::max(1, bit_width(d - 1)));
    field(1, 32, std::max(1, bit_width(uint64_t(k) - 1)));
    for (const Pass &p : passes) {
        k_l1csr_digit<<<g, 256, 0, st>>>(w.key.p, w.val.p, nnz, p.from_key, p.shift, (1u << p.bits) - 1u,
                                         w.digit.p), note_launch();
        MC_TRY(launch_sort_by_key(w.digit.p, nullptr, nnz, 1u << p.bits, w.sort, st));
        k_l1csr_gather<<<g, 256, 0, st>>>(w.sort.perm.p, nnz, w.key.p, w.val.p, w.key2.p, w.val2.p), note_launch();
        std::swap(w.key.p, w.key2.p), std::swap(w.key.n, w.key2.n);
        std::swap(w.val.p, w.val2.p), std::swap(w.val.n, w.val2.n);
    }
    k_l1csr_runs<<<g, 256, 0, st>>>(w.key.p, w.val.p, nnz, d, rows.bucket_count.p, centers), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

}  // namespace mc
