// Tensor-core SQRL2 assignment for dense rows (tcgen05, sm_103a).
//
// For SQRL2 the argmin over centers of ||x - c||^2 equals the argmin of
// v_j = ||c_j||^2 - 2 x.c_j.  The dot products x.c_j come from a BF16 (or TF32) GEMM with
// FP32 accumulation: A = rows (128-row tiles, K-major), B = centers (256-center chunks,
// K-major), both staged in shared memory by TMA (128-byte swizzle), accumulators in TMEM
// (two 256-column buffers so the epilogue drains one while the MMA fills the other).
//
// Rounding bound.  With per-operand relative rounding u (BF16 round-to-nearest, 8-bit
// significand: 2^-8; TF32 operands taken by truncation, 11-bit significand: 2^-10) and FP32
// accumulation over d products,
//   |v_j - v*_j| <= 2 eta ||x|| ||c_j||,   eta = 2u + u^2 + d 2^-22.
// Every center whose exact distance can be the row's minimum satisfies v_j <= b1 + Delta,
//   Delta = 4 eta ||x|| Cmax + 4 gamma_d (||x|| + Cmax)^2,
// where b1 is the row's smallest tensor-core value, Cmax = max_j ||c_j|| and the gamma term
// covers FP32 rounding of the norms and of the exact sequential distance
// (gamma_d = d 2^-24 / (1 - d 2^-24)).
//
// Pass 1 (branch-free epilogue) takes the minimum of every subgroup of 8 consecutive
// centers and keeps, per row, the two smallest subgroup minima m1 <= m2 and the subgroup
// of m1.  If m2 > m1 + Delta, every candidate lies in that subgroup ("single" rows: m1 is
// the row's b1).  The other rows ("multi", about 12 % of the 4M x 128 mixture) are gathered
// into a compact operand copy, and pass 2 (the same MMAs over those rows; the tensor cores
// are deterministic) lists every center with v_j <= m1 + Delta (up to 3 per column part).
// The finalize pass walks the rows sorted by their subgroup (so a warp's center loads are
// mostly one broadcast), evaluates the exact FP32 distance (sequential fmaf over columns,
// the FP32 path's expression) of the 8 centers of a single row's subgroup or of a multi
// row's candidates, and keeps the smallest, lowest index on ties; rows with more
// candidates than slots, or with a non-finite minimum or bound, are rescanned exactly over
// all centers.  So the assignment equals the FP32 path's on every row and costs are exact
// FP32 distances.
//
// Every mbarrier wait is bounded (about one second of clock64 cycles); on a timeout the
// kernel records an error code, stops issuing, waits (bounded) for its copies and MMAs in
// flight, frees its TMEM and returns.
#include <cuda.h>

#include <atomic>

#include <cmath>

#include "mc_assign.cuh"
#include "mc_tc.cuh"
#include "mc_tune.cuh"

namespace mc {

namespace tc {

constexpr int BM = 128;           // rows per tile (MMA M)
constexpr int KBYTES = 128;       // bytes of K per k-block (one 128B swizzle row)
constexpr int A_STAGE = BM * KBYTES;   // 16 KB
constexpr int PARTS = 4;          // column parts of a chunk: one epilogue warp per (lane quarter, part)
// Tile shapes (the autotuner picks one per shape bucket): BN centers per chunk (MMA N,
// 128 or 256) and STAGES shared-memory stages of (A 16 KB + B BN x 128 B).  Centers are
// padded to a multiple of 128; the BN = 256 shapes need a multiple of 256.
template <int BN, int STAGES>
struct Shape {
    static constexpr int B_STAGE = BN * KBYTES;
    static constexpr int STAGE_BYTES = A_STAGE + B_STAGE;
    static constexpr int PCOLS = BN / PARTS;  // columns per epilogue warp and chunk
    static_assert(PCOLS % 32 == 0, "epilogue reads TMEM in 32-column groups");
};
constexpr int KP_ALIGN = 128;
constexpr int NCAND = 3;          // pass 2 candidate slots per row and column part
constexpr int EPI_WARPS = 4 * PARTS;
constexpr int THREADS = 64 + 32 * EPI_WARPS;  // warp 0 TMA, warp 1 MMA (+TMEM alloc), warps 2-17 epilogue
constexpr int CN_SMEM = 4096;     // center norms staged in shared memory when kp <= CN_SMEM
constexpr uint32_t TMEM_COLS = 512;
constexpr long long WAIT_CYCLES = 2000000000ll;  // ~1 s at 2 GHz

template <int STAGES>
struct Smem {
    uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], drain;
    uint64_t nrows;      // rows of this launch (pass 2: the compact row count read on the device)
    uint32_t ntiles;
    uint32_t tmem_base;
    int abort;
    int outstanding[STAGES];
    uint32_t out_parity[STAGES];
};

__device__ inline uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ inline void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ inline void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ inline void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ inline bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; returns false on timeout or when another role aborted
template <class SM>
__device__ inline bool mbar_wait(uint64_t *bar, uint32_t parity, SM *sm, int *err, int code) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 255u) == 0) {
            if (*(volatile int *)&sm->abort) return false;
            if (clock64() - t0 > WAIT_CYCLES) {
                atomicExch(&sm->abort, 1);
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}

// wait with a bound but without the abort check (used while draining after an abort)
__device__ inline void mbar_drain(uint64_t *bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > WAIT_CYCLES) return;
    }
}

__device__ inline void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
        : "memory");
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row atoms 1024 B apart
__device__ inline uint64_t sdesc(const void *p) {
    const uint64_t addr = smem_u32(p);
    uint64_t d = 0;
    d |= (addr >> 4) & 0x3FFFull;          // start address
    d |= uint64_t(1) << 16;                // leading byte offset (unused for K-major swizzle)
    d |= uint64_t(1024 >> 4) << 32;        // stride byte offset: 8 rows x 128 B
    d |= uint64_t(1) << 46;                // descriptor version
    d |= uint64_t(2) << 61;                // 128-byte swizzle
    return d;
}

template <bool TF32, int BN>
__device__ inline uint32_t idesc() {
    // D = F32 (bits 4-5 = 1); A/B format BF16 = 1 or TF32 = 2 (bits 7-9, 10-12); both
    // K-major; N >> 3 at bits 17-22; M >> 4 at bits 24-28
    const uint32_t fmt = TF32 ? 2u : 1u;
    return (1u << 4) | (fmt << 7) | (fmt << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);
}

template <bool TF32, int BN>
__device__ inline void mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    const uint32_t id = idesc<TF32, BN>();
    if (TF32) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(id), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(id), "r"(accumulate)
            : "memory");
    }
}

__device__ inline void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ inline void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ inline void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ inline void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// UMMA shared-memory descriptor for the 32-byte-swizzled K = 16 (BF16) / 8 (TF32) operand
// tiles (one 32-byte row per M/N row, 8-row atoms 256 B apart)
__device__ inline uint64_t sdesc32(const void *p) {
    const uint64_t addr = smem_u32(p);
    uint64_t d = 0;
    d |= (addr >> 4) & 0x3FFFull;          // start address
    d |= uint64_t(1) << 16;                // leading byte offset (unused for K-major swizzle)
    d |= uint64_t(256 >> 4) << 32;         // stride byte offset: 8 rows x 32 B
    d |= uint64_t(1) << 46;                // descriptor version
    d |= uint64_t(6) << 61;                // 32-byte swizzle
    return d;
}

__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// three-input minimum (sm_100 family)
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// three-input maximum (sm_100 family)
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// The same over accumulators that already hold D_j = x.c_j - ||c_j||^2 / 2 (the norm enters
// the accumulator through one more MMA, k_tc_top2_res): v_j = -2 D_j exactly, so the smallest
// v are the largest D.  Keeps the two largest subgroup maxima (M1 >= M2) and the first
// subgroup holding M1; padding centers (j >= k) at -inf.
__device__ __forceinline__ void top2max_group32(float (&v)[32], uint32_t j0, uint32_t k, float &M1, float &M2,
                                                uint32_t &sg1) {
    const float NINF = __int_as_float(0xff800000);
    if (j0 + 32 > k) {
#pragma unroll
        for (int i = 0; i < 32; ++i)
            if (j0 + uint32_t(i) >= k) v[i] = NINF;
    }
#pragma unroll
    for (int sg = 0; sg < 4; ++sg) {
        const float *w = v + 8 * sg;
        const float sv = fmax3(fmax3(w[0], w[1], w[2]), fmax3(w[3], w[4], w[5]), fmaxf(w[6], w[7]));
        const bool higher = sv > M1;
        M2 = fmaxf(M2, fminf(M1, sv));
        sg1 = higher ? (j0 >> 3) + uint32_t(sg) : sg1;
        M1 = fmaxf(M1, sv);
    }
}

// Pass 1 epilogue over 32 accumulator columns (centers j0 .. j0 + 31, norms cn32[0 .. 31]):
// v_j = ||c_j||^2 - 2 acc_j
// (packed f32x2 FMA, each half the IEEE fmaf(-2, acc, ||c||^2)), padding centers (j >= k) at
// +inf, the minimum of each 8-center subgroup, merged into the row's (m1, m2, sg1): the two
// smallest subgroup minima and the first subgroup holding m1.
__device__ __forceinline__ void top2_group32(float (&v)[32], const float *cn32, uint32_t j0, uint32_t k, float &m1,
                                             float &m2, uint32_t &sg1) {
    const float INF = __int_as_float(0x7f800000);
    const unsigned long long m2x = pk2(-2.f, -2.f);
    const float4 *c4 = reinterpret_cast<const float4 *>(cn32);
#pragma unroll
    for (int q4 = 0; q4 < 8; ++q4) {
        const float4 c = c4[q4];
        unsigned long long r0, r1;
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r0) : "l"(pk2(v[4 * q4 + 0], v[4 * q4 + 1])), "l"(m2x), "l"(pk2(c.x, c.y)));
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r1) : "l"(pk2(v[4 * q4 + 2], v[4 * q4 + 3])), "l"(m2x), "l"(pk2(c.z, c.w)));
        upk2(r0, v[4 * q4 + 0], v[4 * q4 + 1]);
        upk2(r1, v[4 * q4 + 2], v[4 * q4 + 3]);
    }
    if (j0 + 32 > k) {  // padding centers take no part
#pragma unroll
        for (int i = 0; i < 32; ++i)
            if (j0 + uint32_t(i) >= k) v[i] = INF;
    }
#pragma unroll
    for (int sg = 0; sg < 4; ++sg) {
        const float *w = v + 8 * sg;
        const float sv = fmin3(fmin3(w[0], w[1], w[2]), fmin3(w[3], w[4], w[5]), fminf(w[6], w[7]));
        const bool lower = sv < m1;
        m2 = fminf(m2, fmaxf(m1, sv));
        sg1 = lower ? (j0 >> 3) + uint32_t(sg) : sg1;
        m1 = fminf(m1, sv);
    }
}

// Column-part exchange of a row tile: each epilogue warp leaves its rows' (m1, m2, subgroup)
// for its column part; the part-0 warp of each lane quarter merges the four parts in part order
// (the first part holding the minimum gives the subgroup) after a named barrier of the quarter's
// four warps (ids 1-4).  Two tile slots alternate, so one barrier per tile suffices: a warp
// rewrites a slot only after the next tile's barrier, which the merging warp reaches after its
// reads.
struct PartX {
    float m1[2][PARTS][BM], m2[2][PARTS][BM];
    uint32_t sg[2][PARTS][BM];
};

__device__ __forceinline__ void quarter_sync(int quarter) {
    asm volatile("bar.sync %0, 128;" ::"r"(1 + quarter) : "memory");
}

// leaves this part's entry, merges on the part-0 warp; returns true there (m1, m2, sg1 merged)
__device__ __forceinline__ bool part_merge(PartX *px, uint32_t tile, int quarter, int part, int rloc, float &m1,
                                           float &m2, uint32_t &sg1) {
    const int sl = int(tile & 1u);
    px->m1[sl][part][rloc] = m1;
    px->m2[sl][part][rloc] = m2;
    px->sg[sl][part][rloc] = m1 < __int_as_float(0x7f800000) ? sg1 : 0xffffffffu;
    quarter_sync(quarter);
    if (part != 0) return false;
    float a1 = __int_as_float(0x7f800000), a2 = a1;
    uint32_t gr = 0xffffffffu;
#pragma unroll
    for (int p = 0; p < PARTS; ++p) {
        const float c1 = px->m1[sl][p][rloc], c2 = px->m2[sl][p][rloc];
        if (c1 < a1) gr = px->sg[sl][p][rloc];
        a2 = fminf(fminf(a2, c2), fmaxf(a1, c1));
        a1 = fminf(a1, c1);
    }
    m1 = a1;
    m2 = a2;
    sg1 = gr;
    return true;
}

}  // namespace tc

struct TcArgs {
    uint64_t n, d;
    uint32_t k, kb, nchunks, ntiles;
    const float *rownorm;  // [n] row squared norms
    float eta, gamma;
    const float *cnp;      // [kp] center norms, +inf past k; [kp] holds Cmax
    uint32_t kp;
    float *b1;             // [n][entries] pass 1: smallest subgroup minimum per row (per group and part)
    float *b2;             // [n][entries] pass 1: second smallest subgroup minimum
    uint32_t *j1;          // [n][entries] pass 1: first subgroup (8 centers) holding b1 (0xffffffff: none)
    const unsigned *count; // pass 2: device count of compact rows (rows = min(*count, n))
    const float *thrc;     // [rows] pass 2: candidate threshold per compact row
    uint8_t *cnt;          // [rows][PARTS] pass 2: candidates per column part (255: too many)
    uint32_t *cand;        // [rows][PARTS][NCAND] pass 2: candidate centers
    int *err;
    int stall_test;        // test hook: the MMA issuer first waits on a barrier nothing completes
};

enum TcMode { TC_TOP2 = 0, TC_CAND = 1 };

// (a1, a2) <- top-2 of the union of (a1, a2) and (b1, b2)
__device__ __forceinline__ void top2_merge(float &a1, float &a2, float b1, float b2) {
    a2 = fminf(fminf(a2, b2), fmaxf(a1, b1));
    a1 = fminf(a1, b1);
}

template <bool TF32, int MODE, int BN, int STAGES>
__global__ void __launch_bounds__(tc::THREADS, 1)
    k_tc_assign(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a) {
    using namespace tc;
    using SH = Shape<BN, STAGES>;
    constexpr int STAGE_BYTES = SH::STAGE_BYTES, PCOLS = SH::PCOLS;
    using Smem = tc::Smem<STAGES>;
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *base = reinterpret_cast<unsigned char *>((uintptr_t(smraw) + 1023) & ~uintptr_t(1023));
    unsigned char *stages = base;
    float *cn_s = reinterpret_cast<float *>(base + STAGES * STAGE_BYTES);
    PartX *px = reinterpret_cast<PartX *>(base + STAGES * STAGE_BYTES + CN_SMEM * sizeof(float));
    Smem *sm = reinterpret_cast<Smem *>(reinterpret_cast<unsigned char *>(px) + (MODE == TC_TOP2 ? sizeof(PartX) : 0));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool cn_in_smem = a.kp <= CN_SMEM;
    if (cn_in_smem)
        for (uint32_t j = threadIdx.x; j < a.kp; j += THREADS) cn_s[j] = a.cnp[j];
    const float *cnp = cn_in_smem ? cn_s : a.cnp;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&sm->full[s], 1);
            mbar_init(&sm->empty[s], 1);
            sm->outstanding[s] = 0;
            sm->out_parity[s] = 0;
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sm->acc_full[b], 1);
            mbar_init(&sm->acc_empty[b], 32 * EPI_WARPS);
        }
        mbar_init(&sm->drain, 1);
        sm->abort = 0;
        uint64_t rows = a.n;
        if (a.count) rows = umin64(uint64_t(*a.count), a.n);
        sm->nrows = rows;
        sm->ntiles = uint32_t((rows + BM - 1) / BM);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm->tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sm->tmem_base;
    const uint32_t total_it = a.nchunks * a.kb;  // k-block iterations per row tile
    const uint32_t ntiles = sm->ntiles;
    const uint64_t nrows = sm->nrows;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t s = 0, ph = 0;
            bool ok = true;
            for (uint32_t m = blockIdx.x; m < ntiles && ok; m += gridDim.x) {
                for (uint32_t it = 0; it < total_it && ok; ++it) {
                    const uint32_t nc = it / a.kb, kb = it % a.kb;
                    if (!mbar_wait(&sm->empty[s], ph ^ 1, sm, a.err, 1)) { ok = false; break; }
                    unsigned char *st = stages + s * STAGE_BYTES;
                    mbar_expect_tx(&sm->full[s], STAGE_BYTES);
                    sm->outstanding[s] = 1;
                    sm->out_parity[s] = ph;
                    const int kcoord = int(kb) * (TF32 ? 32 : 64);
                    tma_load_2d(st, &tmA, &sm->full[s], kcoord, int(m * BM));
                    tma_load_2d(st + A_STAGE, &tmB, &sm->full[s], kcoord, int(nc * BN));
                    if (++s == STAGES) { s = 0; ph ^= 1; }
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t s = 0, ph = 0;
            uint32_t acc_it = 0;
            bool ok = true;
            // test hook (mc_test_tc_stall): `drain` completes only after this thread's own
            // commit below, so this wait runs out its bound, sets the abort flag and error
            // code 5, and every role then takes the bounded drain-and-return path
            if (a.stall_test && !mbar_wait(&sm->drain, 0, sm, a.err, 5)) ok = false;
            for (uint32_t m = blockIdx.x; m < ntiles && ok; m += gridDim.x) {
                for (uint32_t nc = 0; nc < a.nchunks && ok; ++nc, ++acc_it) {
                    const uint32_t buf = acc_it & 1, use = acc_it >> 1;
                    if (!mbar_wait(&sm->acc_empty[buf], (use & 1) ^ 1, sm, a.err, 2)) { ok = false; break; }
                    fence_after();
                    const uint32_t d_tmem = tmem + buf * BN;
                    for (uint32_t kb = 0; kb < a.kb; ++kb) {
                        if (!mbar_wait(&sm->full[s], ph, sm, a.err, 3)) { ok = false; break; }
                        sm->outstanding[s] = 0;
                        fence_after();
                        unsigned char *st = stages + s * STAGE_BYTES;
                        const uint64_t ad = sdesc(st), bd = sdesc(st + A_STAGE);
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {
                            // +32 bytes of K per MMA within the 128-byte swizzle row
                            mma<TF32, BN>(d_tmem, ad + uint64_t(ks * 2), bd + uint64_t(ks * 2), (kb | ks) ? 1u : 0u);
                        }
                        mma_commit(&sm->empty[s]);
                        if (++s == STAGES) { s = 0; ph ^= 1; }
                    }
                    if (ok) mma_commit(&sm->acc_full[buf]);
                }
            }
            // all MMAs issued by this thread complete before the drain barrier fires (a CTA
            // without tiles, possible in pass 2, issued none and has nothing to drain)
            if (blockIdx.x < ntiles) {
                mma_commit(&sm->drain);
                mbar_drain(&sm->drain, 0);
            }
        }
    } else {
        // ---------------- epilogue (warps 2-17) ----------------
        const int quarter = warp & 3;                 // TMEM lanes 32*quarter .. +31
        const int part = (warp - 2) >> 2;             // columns [64*part, 64*part + 64) of a chunk
        const uint32_t lane_base = uint32_t(quarter * 32) << 16;
        const int rloc = quarter * 32 + lane;
        const float INF = __int_as_float(0x7f800000);
        uint32_t acc_it = 0, tcount = 0;
        bool ok = true;
        for (uint32_t m = blockIdx.x; m < ntiles && ok; m += gridDim.x) {
            const uint64_t row = uint64_t(m) * BM + rloc;  // pass 2: compact row
            const bool valid = row < nrows;
            float m1 = INF, m2 = INF;                      // pass 1: top-2 of the subgroup minima
            uint32_t sg1 = 0xffffffffu;                    // pass 1: subgroup (8 centers) of m1
            float thr = __int_as_float(0xff800000);        // pass 2: fixed candidate threshold
            int ncand = 0;
            if (MODE == TC_CAND && valid) thr = a.thrc[row];
            uint32_t *cdst = a.cand + (row * PARTS + part) * NCAND;
            for (uint32_t nc = 0; nc < a.nchunks; ++nc, ++acc_it) {
                const uint32_t buf = acc_it & 1, use = acc_it >> 1;
                // one lane waits, the warp follows converged (tcgen05.ld is warp-collective)
                int got = 0;
                if (lane == 0) got = mbar_wait(&sm->acc_full[buf], use & 1, sm, a.err, 4) ? 1 : 0;
                got = __shfl_sync(0xffffffffu, got, 0);
                __syncwarp();
                if (!got) { ok = false; break; }
                fence_after();
                const uint32_t taddr = tmem + lane_base + buf * BN + part * PCOLS;
#pragma unroll 1
                for (int g = 0; g < PCOLS / 32; ++g) {
                    float v[32];
                    tmem_ld32(taddr + g * 32, v);
                    const uint32_t j0 = nc * BN + part * PCOLS + g * 32;
                    if (MODE == TC_TOP2) {
                        top2_group32(v, cnp + j0, j0, a.k, m1, m2, sg1);
                    } else {
                        const float4 *c4 = reinterpret_cast<const float4 *>(cnp + j0);
#pragma unroll
                        for (int q4 = 0; q4 < 8; ++q4) {
                            const float4 c = c4[q4];
                            v[4 * q4 + 0] = fmaf(-2.f, v[4 * q4 + 0], c.x);
                            v[4 * q4 + 1] = fmaf(-2.f, v[4 * q4 + 1], c.y);
                            v[4 * q4 + 2] = fmaf(-2.f, v[4 * q4 + 2], c.z);
                            v[4 * q4 + 3] = fmaf(-2.f, v[4 * q4 + 3], c.w);
                        }
                        float smin[4];
#pragma unroll
                        for (int sg = 0; sg < 4; ++sg) {
                            const float *w = v + 8 * sg;
                            smin[sg] = fminf(fminf(fminf(w[0], w[1]), fminf(w[2], w[3])),
                                             fminf(fminf(w[4], w[5]), fminf(w[6], w[7])));
                        }
                        const float gmin = fminf(fminf(smin[0], smin[1]), fminf(smin[2], smin[3]));
                        if (gmin <= thr) {  // candidates in this group
#pragma unroll
                            for (int sg = 0; sg < 4; ++sg) {
                                if (smin[sg] <= thr) {
#pragma unroll
                                    for (int q8 = 0; q8 < 8; ++q8) {
                                        if (v[8 * sg + q8] <= thr) {
                                            if (ncand < NCAND) cdst[ncand] = j0 + uint32_t(8 * sg + q8);
                                            ++ncand;
                                        }
                                    }
                                }
                            }
                        }
                    }
                }
                fence_before();
                mbar_arrive(&sm->acc_empty[buf]);
            }
            if (!ok) break;
            if (MODE == TC_TOP2) {
                // one merged entry per row (all four part warps of the quarter take part)
                if (part_merge(px, tcount++, quarter, part, rloc, m1, m2, sg1) && valid) {
                    a.b1[row] = m1;
                    a.b2[row] = m2;
                    a.j1[row] = sg1;
                }
            } else if (valid) {
                a.cnt[row * PARTS + part] = ncand > NCAND ? uint8_t(255) : uint8_t(ncand);
            }
        }
    }
    // ---------------- teardown ----------------
    __syncthreads();
    if (threadIdx.x == 0 && sm->abort) {
        // copies still in flight into this CTA's shared memory: wait for them (bounded)
        for (int s = 0; s < STAGES; ++s)
            if (sm->outstanding[s]) mbar_drain(&sm->full[s], sm->out_parity[s]);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// Pass 1 with the centers resident in shared memory.  Streaming the center operand for every
// row tile (k_tc_assign) moves (128 + 256) x K operand elements through L2 per 128 x 256 x K
// MMA block, about 16 TB/s at this kernel's pace; here the centers are split into groups of
// `gch` 256-center chunks that fit shared memory next to two row-tile stages, each CTA loads
// its group's centers once and then streams row tiles only, and the rows' tiles are read once
// per group.  CTA b serves group b % G and row tiles b / G, b / G + T, ... (T = grid / G).
// The norms enter the accumulators instead of the epilogue: every chunk starts with one more
// MMA (K = 16 BF16 / 8 TF32, 32-byte swizzled operands) of A = (1, 1, 1, 0, ...) against
// B_j = -||c_j||^2 / 2 split into three parts, so D_j = x.c_j - ||c_j||^2 / 2 and
// v_j = -2 D_j exactly.  Adding the norm in the epilogue took one 4-byte broadcast per
// (warp, center) from shared memory, which kept the load/store pipe about 80 % busy.  The
// norm now shares the accumulator's FP32 rounding: with T = d / 16 + 1 accumulation steps of
// relative error <= 2^-22 each over partial sums of magnitude <= ||x|| ||c|| + Cmax^2 / 2, and
// the three-part split exact to 2^-24, v_j moves by at most (d + 1) 2^-22 Cmax^2 beyond the
// dot-product bound, which k_tc_select adds twice to Delta.  The epilogue keeps the two
// largest subgroup maxima of D.  Each group writes its own column parts unmerged (a merge
// across the part warps, as k_tc_assign does, measured slower here), so a row has G x PARTS
// (m1, m2, subgroup) entries at [row][g][part] for k_tc_select to merge in that order.
namespace tc {
template <int KB>
struct ResShape {
    static constexpr int A_TILE = KB * A_STAGE;                  // a row tile's k-blocks
    static constexpr int ASTAGES = KB == 1 ? 3 : 2;
    static constexpr int GCH = KB == 1 ? 4 : 2;                  // 256-center chunks per group
    static constexpr int B_CHUNK = KB * 256 * KBYTES;            // 32 KB per k-block
    static constexpr int AUXA = BM * 32;                         // norm MMA: ones, 32 B per row
    static constexpr int AUXB = 256 * 32;                        // norm MMA: -||c||^2 / 2 split, per chunk
    static constexpr int SMEM = ASTAGES * A_TILE + GCH * B_CHUNK + AUXA + GCH * AUXB;
};
struct ResSmem {
    uint64_t afull[4], aempty[4], bfull, acc_full[2], acc_empty[2], drain;
    uint32_t tmem_base;
    int abort;
    int a_out[4], b_out;
    uint32_t a_par[4];
};
}  // namespace tc

template <bool TF32, int KB>
__global__ void __launch_bounds__(tc::THREADS, 1)
    k_tc_top2_res(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ CUtensorMap tmAuxA, const __grid_constant__ CUtensorMap tmAuxB, TcArgs a,
                  uint32_t G, uint32_t nchunks) {
    using namespace tc;
    using RS = ResShape<KB>;
    constexpr int BN = 256, PCOLS = BN / PARTS, ASTAGES = RS::ASTAGES;
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *base = reinterpret_cast<unsigned char *>((uintptr_t(smraw) + 1023) & ~uintptr_t(1023));
    unsigned char *astages = base;
    unsigned char *bres = base + ASTAGES * RS::A_TILE;
    unsigned char *auxa = bres + RS::GCH * RS::B_CHUNK;
    unsigned char *auxb = auxa + RS::AUXA;
    ResSmem *sm = reinterpret_cast<ResSmem *>(auxb + RS::GCH * RS::AUXB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g = blockIdx.x % G, T = gridDim.x / G, t0 = blockIdx.x / G;
    const uint32_t c0 = g * RS::GCH;                                   // first chunk of the group
    const uint32_t gch = umin64(RS::GCH, nchunks - c0);                // chunks of this group
    const uint32_t ntiles = a.ntiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < ASTAGES; ++s) {
            mbar_init(&sm->afull[s], 1);
            mbar_init(&sm->aempty[s], 1);
            sm->a_out[s] = 0;
            sm->a_par[s] = 0;
        }
        mbar_init(&sm->bfull, 1);
        sm->b_out = 0;
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sm->acc_full[b], 1);
            mbar_init(&sm->acc_empty[b], 32 * EPI_WARPS);
        }
        mbar_init(&sm->drain, 1);
        sm->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm->tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sm->tmem_base;

    if (warp == 0) {
        // ---------------- TMA producer: the group's centers once, then row tiles ----------------
        if (lane == 0 && t0 < ntiles) {
            mbar_expect_tx(&sm->bfull, gch * RS::B_CHUNK + RS::AUXA + gch * RS::AUXB);
            sm->b_out = 1;
            for (uint32_t nc = 0; nc < gch; ++nc)
                for (int kb = 0; kb < KB; ++kb)
                    tma_load_2d(bres + (nc * KB + kb) * (256 * KBYTES), &tmB, &sm->bfull, kb * (TF32 ? 32 : 64),
                                int((c0 + nc) * BN));
            tma_load_2d(auxa, &tmAuxA, &sm->bfull, 0, 0);
            for (uint32_t nc = 0; nc < gch; ++nc)
                tma_load_2d(auxb + nc * RS::AUXB, &tmAuxB, &sm->bfull, 0, int((c0 + nc) * BN));
            uint32_t s = 0, ph = 0;
            for (uint32_t m = t0; m < ntiles; m += T) {
                if (!mbar_wait(&sm->aempty[s], ph ^ 1, sm, a.err, 1)) break;
                unsigned char *st = astages + s * RS::A_TILE;
                mbar_expect_tx(&sm->afull[s], RS::A_TILE);
                sm->a_out[s] = 1;
                sm->a_par[s] = ph;
                for (int kb = 0; kb < KB; ++kb)
                    tma_load_2d(st + kb * A_STAGE, &tmA, &sm->afull[s], kb * (TF32 ? 32 : 64), int(m * BM));
                if (++s == ASTAGES) { s = 0; ph ^= 1; }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0 && t0 < ntiles) {
            bool ok = true;
            if (a.stall_test && !mbar_wait(&sm->drain, 0, sm, a.err, 5)) ok = false;
            if (ok && !mbar_wait(&sm->bfull, 0, sm, a.err, 6)) ok = false;
            if (ok) sm->b_out = 0;
            uint32_t s = 0, ph = 0, acc_it = 0;
            for (uint32_t m = t0; m < ntiles && ok; m += T) {
                if (!mbar_wait(&sm->afull[s], ph, sm, a.err, 3)) { ok = false; break; }
                sm->a_out[s] = 0;
                fence_after();
                const uint64_t ad0 = sdesc(astages + s * RS::A_TILE);
                for (uint32_t nc = 0; nc < gch && ok; ++nc, ++acc_it) {
                    const uint32_t buf = acc_it & 1, use = acc_it >> 1;
                    if (!mbar_wait(&sm->acc_empty[buf], (use & 1) ^ 1, sm, a.err, 2)) { ok = false; break; }
                    fence_after();
                    const uint32_t d_tmem = tmem + buf * BN;
                    // D = 1 . (-||c||^2 / 2, split in three) ... then += x . c
                    mma<TF32, BN>(d_tmem, sdesc32(auxa), sdesc32(auxb + nc * RS::AUXB), 0u);
#pragma unroll
                    for (int kb = 0; kb < KB; ++kb) {
                        const uint64_t ad = ad0 + uint64_t((kb * A_STAGE) >> 4);
                        const uint64_t bd = sdesc(bres + (nc * KB + kb) * (256 * KBYTES));
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks)
                            mma<TF32, BN>(d_tmem, ad + uint64_t(ks * 2), bd + uint64_t(ks * 2), 1u);
                    }
                    mma_commit(&sm->acc_full[buf]);
                }
                if (!ok) break;
                mma_commit(&sm->aempty[s]);  // the row tile's stage is free once these MMAs finish
                if (++s == ASTAGES) { s = 0; ph ^= 1; }
            }
            mma_commit(&sm->drain);
            mbar_drain(&sm->drain, 0);
        }
    } else {
        // ---------------- epilogue (warps 2-17) ----------------
        const int quarter = warp & 3;
        const int part = (warp - 2) >> 2;
        const uint32_t lane_base = uint32_t(quarter * 32) << 16;
        const int rloc = quarter * 32 + lane;
        const float INF = __int_as_float(0x7f800000);
        uint32_t acc_it = 0;
        bool ok = true;
        for (uint32_t m = t0; m < ntiles && ok; m += T) {
            const uint64_t row = uint64_t(m) * BM + rloc;
            float M1 = -INF, M2 = -INF;  // the two largest subgroup maxima of D
            uint32_t sg1 = 0xffffffffu;
            for (uint32_t nc = 0; nc < gch; ++nc, ++acc_it) {
                const uint32_t buf = acc_it & 1, use = acc_it >> 1;
                int got = 0;
                if (lane == 0) got = mbar_wait(&sm->acc_full[buf], use & 1, sm, a.err, 4) ? 1 : 0;
                got = __shfl_sync(0xffffffffu, got, 0);
                __syncwarp();
                if (!got) { ok = false; break; }
                fence_after();
                const uint32_t taddr = tmem + lane_base + buf * BN + part * PCOLS;
                float v0[32], v1[32];
                tmem_ld32(taddr, v0);
                tmem_ld32(taddr + 32, v1);
                fence_before();
                mbar_arrive(&sm->acc_empty[buf]);  // both column groups are in registers
                const uint32_t j0 = (c0 + nc) * BN + part * PCOLS;
                top2max_group32(v0, j0, a.k, M1, M2, sg1);
                top2max_group32(v1, j0 + 32, a.k, M1, M2, sg1);
            }
            if (!ok) break;
            if (row < a.n) {
                // v = -2 D exactly: the smallest and second smallest subgroup minima of v
                const uint64_t o = (row * G + g) * PARTS + part;
                a.b1[o] = -2.f * M1;
                a.b2[o] = -2.f * M2;
                a.j1[o] = M1 > -INF ? sg1 : 0xffffffffu;
            }
        }
    }
    // ---------------- teardown ----------------
    __syncthreads();
    if (threadIdx.x == 0 && sm->abort) {
        if (sm->b_out) mbar_drain(&sm->bfull, 0);
        for (int s = 0; s < ASTAGES; ++s)
            if (sm->a_out[s]) mbar_drain(&sm->afull[s], sm->a_par[s]);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// ------------------------------------------------------------------------------------
// support kernels
// ------------------------------------------------------------------------------------
__global__ void k_to_bf16_pad(const float *__restrict__ X, uint64_t n, uint64_t d, uint64_t dp,
                              __nv_bfloat16 *__restrict__ Y) {
    const uint64_t total = n * dp;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t r = e / dp, c = e % dp;
        Y[e] = __float2bfloat16_rn(c < d ? X[r * d + c] : 0.f);
    }
}

// rows without padding (d % 8 == 0, 16-byte aligned): eight floats per thread, two float4
// loads and one 16-byte store of four bf16 pairs (the same round-to-nearest conversion)
__global__ void k_to_bf16_flat8(const float4 *__restrict__ X, uint64_t n8, uint4 *__restrict__ Y) {
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < n8; e += gridDim.x * uint64_t(blockDim.x)) {
        const float4 a = X[2 * e], b = X[2 * e + 1];
        const __nv_bfloat162 p0 = __floats2bfloat162_rn(a.x, a.y), p1 = __floats2bfloat162_rn(a.z, a.w);
        const __nv_bfloat162 p2 = __floats2bfloat162_rn(b.x, b.y), p3 = __floats2bfloat162_rn(b.z, b.w);
        uint4 o;
        o.x = *reinterpret_cast<const uint32_t *>(&p0);
        o.y = *reinterpret_cast<const uint32_t *>(&p1);
        o.z = *reinterpret_cast<const uint32_t *>(&p2);
        o.w = *reinterpret_cast<const uint32_t *>(&p3);
        Y[e] = o;
    }
}

int launch_to_bf16_flat8(const float *X, uint64_t n8, void *Y, int sms, cudaStream_t st) {
    if (n8 == 0) return MC_OK;
    k_to_bf16_flat8<<<unsigned(umin64((n8 + 255) / 256, uint64_t(sms) * 16)), 256, 0, st>>>(
        reinterpret_cast<const float4 *>(X), n8, reinterpret_cast<uint4 *>(Y)), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

__global__ void k_pad_f32(const float *__restrict__ X, uint64_t n, uint64_t d, uint64_t dp, float *__restrict__ Y) {
    const uint64_t total = n * dp;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t r = e / dp, c = e % dp;
        Y[e] = c < d ? X[r * d + c] : 0.f;
    }
}

__global__ void k_center_prep_tc(const float *__restrict__ C, uint32_t k, uint32_t kp, uint64_t d, uint64_t dp,
                                 int tf32, __nv_bfloat16 *Cb, float *Ct, const float *cn, float *cnp) {
    const uint64_t total = uint64_t(kp) * dp;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += gridDim.x * uint64_t(blockDim.x)) {
        const uint64_t r = e / dp, c = e % dp;
        const float v = (r < k && c < d) ? C[r * d + c] : 0.f;
        if (tf32) Ct[e] = v;
        else Cb[e] = __float2bfloat16_rn(v);
    }
    // padded norms (+inf past k) and the max center norm at cnp[kp] (norms are non-negative,
    // so their bit patterns order like the values)
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < kp; j += gridDim.x * blockDim.x) {
        cnp[j] = j < k ? cn[j] : __int_as_float(0x7f800000);
        if (j < k) atomicMax(reinterpret_cast<int *>(cnp + kp), __float_as_int(sqrtf(cn[j])));
    }
}

// Row status after pass 1 (k_tc_select): the subgroup holding every candidate (< 2^31),
// MULTI | compact slot, or OVER (rescanned over all centers).  key[] orders the finalize:
// the subgroup for single rows, nsg for multi rows, nsg + 1 for OVER rows.
constexpr uint32_t ST_MULTI = 0x80000000u;
constexpr uint32_t ST_OVER = 0xffffffffu;

// Combines the column parts' top-2 of every row, decides single / multi / over, and for
// multi rows takes a compact slot: the row's operand copy goes to Xc[slot], its pass 2
// threshold to thrc[slot].  Slots come from warp-aggregated atomics, so their order varies
// from run to run; no result depends on it.
__global__ void __launch_bounds__(256) k_tc_select(uint64_t n, const float *__restrict__ b1,
                                                    const float *__restrict__ b2, const uint32_t *__restrict__ j1,
                                                    const float *__restrict__ rownorm, const float *__restrict__ cmaxp,
                                                    float eta, float gamma, uint32_t nsg, uint32_t *status,
                                                    uint32_t *key, uint32_t *crow, float *thrc, unsigned *count,
                                                    uint32_t cap, const uint4 *__restrict__ A, uint64_t row_u4,
                                                    uint4 *Xc, uint32_t *over_rows, unsigned long long *nover,
                                                    unsigned long long *nmulti, uint32_t ngroups, float nerr) {
    __shared__ uint32_t mrow[8][32], mslot[8][32];  // the warp's multi rows and their slots
    const uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const float INF = __int_as_float(0x7f800000);
    bool over = false, multi = false;
    float thr = 0.f;
    if (row < n) {
        float m1 = INF, m2 = INF;
        uint32_t gr = ST_OVER;
        // the row's pass 1 entries (one, or one per center group and column part), in order
        for (uint32_t g = 0; g < ngroups; ++g) {
            const uint64_t o = row * ngroups + g;
            const float c1 = b1[o], c2 = b2[o];
            if (c1 < m1) gr = j1[o];
            top2_merge(m1, m2, c1, c2);
        }
        const float cmax = *cmaxp;
        const float xn = sqrtf(rownorm[row]);
        const float delta =
            4.f * eta * xn * cmax * 1.0001f + 4.f * gamma * (xn + cmax) * (xn + cmax) + nerr * cmax * cmax;
        // no finite minimum or a non-finite bound proves nothing: exact rescan
        if (!(m1 < INF) || !(delta <= 3.402823466e+38f) || gr >= nsg) {
            over = true;
        } else if (m2 > m1 + delta) {
            status[row] = gr;
            key[row] = gr;
        } else {
            multi = true;
            thr = m1 + delta;
        }
    }
    const unsigned mb = __ballot_sync(0xffffffffu, multi);
    unsigned base = 0;
    if (lane == 0 && mb) base = atomicAdd(count, unsigned(__popc(mb)));
    base = __shfl_sync(0xffffffffu, base, 0);
    const unsigned slot = base + unsigned(__popc(mb & ((1u << lane) - 1u)));
    if (multi) {
        if (slot < cap) {
            status[row] = ST_MULTI | slot;
            key[row] = nsg;
            crow[slot] = uint32_t(row);
            thrc[slot] = thr;
        } else {
            over = true;  // compact buffer full: exact rescan
        }
    }
    // operand copies of the warp's multi rows: the (row, 16-byte word) items spread over the
    // lanes, so the copies of several rows are in flight at once
    if (multi) {
        const int r = __popc(mb & ((1u << lane) - 1u));
        mrow[wib][r] = uint32_t(row);
        mslot[wib][r] = slot;
    }
    __syncwarp();
    const uint32_t ru4 = uint32_t(row_u4), items = uint32_t(__popc(mb)) * ru4;
    for (uint32_t it = lane; it < items; it += 32) {
        const uint32_t r = it / ru4, q = it - r * ru4;
        const unsigned sl = mslot[wib][r];
        if (sl < cap) Xc[uint64_t(sl) * row_u4 + q] = A[uint64_t(mrow[wib][r]) * row_u4 + q];
    }
    const unsigned ob = __ballot_sync(0xffffffffu, over);
    unsigned long long obase = 0;
    if (lane == 0) {
        if (ob) obase = atomicAdd(nover, (unsigned long long)__popc(ob));
        if (mb) atomicAdd(nmulti, (unsigned long long)__popc(mb));
    }
    obase = __shfl_sync(0xffffffffu, obase, 0);
    if (over) {
        status[row] = ST_OVER;
        key[row] = nsg + 1;
        over_rows[obase + __popc(ob & ((1u << lane) - 1u))] = uint32_t(row);
    }
}

// Exact FP32 distances for the candidate centers of every row (sequential fmaf over the
// columns: the FP32 path's expression).  Rows are taken in `order` (sorted by subgroup).
// A CTA handles 128 consecutive rows of that order: it stages the centers of the first two
// subgroups it meets in shared memory (when 16 d floats fit), and 32 columns of its rows
// at a time; each thread keeps its row's staged columns in registers and walks its
// candidates: the 8 centers of a single row's subgroup, or a multi row's pass 2 list (up
// to 3 per column part).  A warp whose rows all use staged centers reads them from shared
// memory (one broadcast per warp); any other warp reads its candidates from global memory.
// Multi rows with too many candidates, or none, are listed for an exact scan over all
// centers; OVER rows were listed by k_tc_select.
constexpr int NSLOT = tc::PARTS * tc::NCAND;
constexpr int FIN_ROWS = 128;
constexpr int FIN_SG = 2;  // subgroups whose centers a CTA stages
constexpr int FIN_COLS = 16;  // columns per cp.async stage (smaller stages: more CTAs per SM)

__device__ __forceinline__ void cp_async16(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::smem_u32(dst)), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// FIN_COLS columns of one candidate: c - x for the staged columns, sequential fmaf
__device__ __forceinline__ void fin_chunk32(const float *cr, const float (&xr)[FIN_COLS], float &a) {
    const float4 *c4 = reinterpret_cast<const float4 *>(cr);
#pragma unroll
    for (int k4 = 0; k4 < FIN_COLS / 4; ++k4) {
        const float4 c = c4[k4];
        float df = c.x - xr[4 * k4 + 0];
        a = fmaf(df, df, a);
        df = c.y - xr[4 * k4 + 1];
        a = fmaf(df, df, a);
        df = c.z - xr[4 * k4 + 2];
        a = fmaf(df, df, a);
        df = c.w - xr[4 * k4 + 3];
        a = fmaf(df, df, a);
    }
}

// the same for a chunk of kmax < 32 columns or unaligned rows (columns read from shared memory)
__device__ __forceinline__ void fin_chunk_scalar(const float *cr, const float *xrow, int kmax, float &a) {
    for (int kk = 0; kk < kmax; ++kk) {
        const float df = cr[kk] - xrow[kk];
        a = fmaf(df, df, a);
    }
}

// staged centers: two subgroups of 8, stored as 4 pairs per subgroup with the pair's two
// values of a column side by side, so that one 64-bit word feeds a packed f32x2 operation
// (center q of subgroup s, column j) -> ((4 s + q / 2) d + j) 2 + q % 2
__device__ __forceinline__ const float *fin_pair_col(const float *sub_base, int q, uint64_t d, uint64_t j) {
    return sub_base + ((uint64_t(q >> 1) * d + j) << 1) + (q & 1);
}

// fin_chunk_scalar over the pair layout (stride 2)
__device__ __forceinline__ void fin_chunk_scalar2(const float *cr, const float *xrow, int kmax, float &a) {
    for (int kk = 0; kk < kmax; ++kk) {
        const float df = cr[2 * kk] - xrow[kk];
        a = fmaf(df, df, a);
    }
}

// packed f32x2 (sm_100 family): each half is the IEEE single operation of the scalar code
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// a = fma(c - x, c - x, a) in both halves
__device__ __forceinline__ unsigned long long f2_sqdiff_acc(unsigned long long c, unsigned long long x,
                                                           unsigned long long a) {
    unsigned long long df, r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(df) : "l"(c), "l"(x));
    asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(r) : "l"(df), "l"(a));
    return r;
}

template <bool VEC4>
__global__ void __launch_bounds__(FIN_ROWS) k_tc_finalize(const float *__restrict__ X, uint64_t n, uint64_t d,
                                                           const float *__restrict__ C, uint32_t k, uint32_t nsg,
                                                           int stage_centers, uint32_t *asn,
                                                           const uint32_t *__restrict__ order,
                                                           const uint32_t *__restrict__ status,
                                                           const uint8_t *__restrict__ cnt,
                                                           const uint32_t *__restrict__ cand, double *costs,
                                                           uint32_t *over_rows, unsigned long long *nover) {
    constexpr int R = FIN_ROWS;
    extern __shared__ __align__(16) float cs[];  // [FIN_SG][4 pairs][d][2] staged centers
    __shared__ __align__(16) float xs4[2][R][FIN_COLS + 4];  // two column stages (rows padded by 16 B)
    __shared__ uint32_t rows_s[R];
    __shared__ uint32_t sg_first;
    const int t = threadIdx.x, lane = t & 31;
    const uint64_t pos = uint64_t(blockIdx.x) * R + t;
    const uint64_t row = pos < n ? order[pos] : n;
    rows_s[t] = uint32_t(row < n ? row : 0xffffffffu);
    const uint32_t st = row < n ? status[row] : ST_OVER;
    if (t == 0) sg_first = (stage_centers && st != ST_OVER && !(st & ST_MULTI)) ? st : 0xffffffffu;
    // cj[q] == 0xffffffff marks an unused slot
    uint32_t cj[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) cj[q] = 0xffffffffu;
    bool over = false;
    if (st != ST_OVER && (st & ST_MULTI)) {
        const uint64_t slot = st & ~ST_MULTI;
        int tot = 0;
#pragma unroll
        for (int p = 0; p < tc::PARTS; ++p) {
            const int c = cnt[slot * tc::PARTS + p];
            if (c == 255) over = true;
            tot += c;
#pragma unroll
            for (int q = 0; q < tc::NCAND; ++q) {
                if (q < c && c != 255) {
                    const uint32_t j = cand[(slot * tc::PARTS + p) * tc::NCAND + q];
                    cj[p * tc::NCAND + q] = j < k ? j : 0xffffffffu;
                }
            }
        }
        if (tot == 0) over = true;
    } else if (st != ST_OVER) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint32_t j = st * 8u + uint32_t(q);
            cj[q] = j < k ? j : 0xffffffffu;
        }
    }
    // warp-aggregated counter: one atomic per warp
    const unsigned ob = __ballot_sync(0xffffffffu, over);
    unsigned long long obase = 0;
    if (lane == 0 && ob) obase = atomicAdd(nover, (unsigned long long)__popc(ob));
    obase = __shfl_sync(0xffffffffu, obase, 0);
    if (over) {
        over_rows[obase + __popc(ob & ((1u << lane) - 1u))] = uint32_t(row);
#pragma unroll
        for (int q = 0; q < NSLOT; ++q) cj[q] = 0xffffffffu;
    }
    __syncthreads();
    const uint64_t nchunk = (d + FIN_COLS - 1) / FIN_COLS;
    auto stage = [&](uint64_t ci, int buf) {
        const uint64_t k0 = ci * FIN_COLS;
        const int kmax = int(umin64(FIN_COLS, d - k0));
        for (int e = t; e < R * (FIN_COLS / 4); e += R) {
            const int r = e / (FIN_COLS / 4), q4 = e % (FIN_COLS / 4);
            const uint32_t rr = rows_s[r];
            const bool ok = rr != 0xffffffffu && 4 * q4 < kmax;
            const float *src = ok ? X + uint64_t(rr) * d + k0 + 4 * q4 : X;
            cp_async16(&xs4[buf][r][4 * q4], src, ok ? 16 : 0);
        }
        cp_async_commit();
    };
    // the rows' first column chunk is in flight while the centers are staged
    if (VEC4) stage(0, 0);
    // staged centers: subgroups sg_first .. sg_first + FIN_SG - 1
    const uint32_t sgf = sg_first;
    if (sgf != 0xffffffffu) {
        // the staged centers are contiguous rows of C: copy them as one run (zeros past k)
        const uint64_t j0 = uint64_t(sgf) * 8;
        const uint64_t jend = umin64(j0 + uint64_t(FIN_SG) * 8, k);
        const uint32_t valid = uint32_t((jend > j0 ? jend - j0 : 0) * d);
        const uint32_t tot = uint32_t(FIN_SG * 8 * d);
        const float *src = C + j0 * d;
        if (VEC4) {
            // float4 items (center cl, columns 4 j4 .. 4 j4 + 3), R apart, four loads in flight
            const uint32_t dq = uint32_t(d / 4), items = tot / 4;
            for (uint32_t e0 = t; e0 < items; e0 += 4 * R) {
                float4 v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t e = e0 + uint32_t(u) * R;
                    v[u] = (e < items && 4 * e < valid) ? __ldg(reinterpret_cast<const float4 *>(src) + e)
                                                        : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t e = e0 + uint32_t(u) * R;
                    if (e < items) {
                        const uint32_t cl = e / dq, j = 4 * (e - cl * dq);
                        float *dst = cs + uint64_t(cl >> 3) * 8 * d + ((uint64_t((cl & 7) >> 1) * d + j) << 1) + (cl & 1);
                        dst[0] = v[u].x;
                        dst[2] = v[u].y;
                        dst[4] = v[u].z;
                        dst[6] = v[u].w;
                    }
                }
            }
        } else {
            for (uint32_t e = t; e < tot; e += R) {
                const uint32_t cl = e / uint32_t(d), j = e - cl * uint32_t(d);
                cs[uint64_t(cl >> 3) * 8 * d + ((uint64_t((cl & 7) >> 1) * d + j) << 1) + (cl & 1)] =
                    e < valid ? src[e] : 0.f;
            }
        }
    }
    const bool mine_local = sgf != 0xffffffffu && st != ST_OVER && !(st & ST_MULTI) && !over && st - sgf < FIN_SG;
    const bool warp_local = __all_sync(0xffffffffu, mine_local || st == ST_OVER || over || row >= n);
    const float *lbase = cs + uint64_t(mine_local ? st - sgf : 0) * 8 * d;
    float acc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) acc[q] = 0.f;
    if (VEC4) {
        // d % 4 == 0: FIN_COLS-column chunks (the last one may be narrower) double-buffered
        // with cp.async, so the next chunk's rows load while this one is evaluated (chunk 0 was
        // issued before the centers were staged)
        for (uint64_t ci = 0; ci < nchunk; ++ci) {
            const int buf = int(ci & 1);
            if (ci + 1 < nchunk) {
                stage(ci + 1, buf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            const uint64_t k0 = ci * FIN_COLS;
            const int kmax = int(umin64(FIN_COLS, d - k0));
            if (kmax == FIN_COLS) {
                // the row's 32 staged columns in registers, reused by every candidate
                float xr[FIN_COLS];
#pragma unroll
                for (int c4 = 0; c4 < FIN_COLS / 4; ++c4) {
                    const float4 v = *reinterpret_cast<const float4 *>(&xs4[buf][t][4 * c4]);
                    xr[4 * c4 + 0] = v.x;
                    xr[4 * c4 + 1] = v.y;
                    xr[4 * c4 + 2] = v.z;
                    xr[4 * c4 + 3] = v.w;
                }
                if (warp_local) {
                    if (mine_local) {
                        // all 8 subgroup centers at once (padding centers are zeros and are
                        // ignored below): 8 independent sequential chains per thread, two per
                        // packed f32x2 accumulator (pairs of centers side by side in shared memory)
                        unsigned long long a2[4];
#pragma unroll
                        for (int pq = 0; pq < 4; ++pq) a2[pq] = f2_pack(acc[2 * pq], acc[2 * pq + 1]);
#pragma unroll
                        for (int k2 = 0; k2 < FIN_COLS / 2; ++k2) {
                            const unsigned long long x0 = f2_pack(xr[2 * k2], xr[2 * k2]);
                            const unsigned long long x1 = f2_pack(xr[2 * k2 + 1], xr[2 * k2 + 1]);
#pragma unroll
                            for (int pq = 0; pq < 4; ++pq) {
                                const ulonglong2 c = *reinterpret_cast<const ulonglong2 *>(
                                    lbase + ((uint64_t(pq) * d + k0 + 2 * k2) << 1));
                                a2[pq] = f2_sqdiff_acc(c.x, x0, a2[pq]);
                                a2[pq] = f2_sqdiff_acc(c.y, x1, a2[pq]);
                            }
                        }
#pragma unroll
                        for (int pq = 0; pq < 4; ++pq) f2_unpack(a2[pq], acc[2 * pq], acc[2 * pq + 1]);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < NSLOT; ++q)
                        if (cj[q] != 0xffffffffu) fin_chunk32(C + uint64_t(cj[q]) * d + k0, xr, acc[q]);
                }
            } else {
                if (warp_local) {
                    if (mine_local) {
#pragma unroll
                        for (int q = 0; q < 8; ++q)
                            if (cj[q] != 0xffffffffu)
                                fin_chunk_scalar2(fin_pair_col(lbase, q, d, k0), xs4[buf][t], kmax, acc[q]);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < NSLOT; ++q)
                        if (cj[q] != 0xffffffffu)
                            fin_chunk_scalar(C + uint64_t(cj[q]) * d + k0, xs4[buf][t], kmax, acc[q]);
                }
            }
            __syncthreads();  // buffer buf is restaged two chunks later
        }
    } else {
        for (uint64_t k0 = 0; k0 < d; k0 += FIN_COLS) {
            const int kmax = int(umin64(FIN_COLS, d - k0));
            __syncthreads();
            for (int e = t; e < R * FIN_COLS; e += R) {
                const int r = e / FIN_COLS, kk = e % FIN_COLS;
                const uint32_t rr = rows_s[r];
                xs4[0][r][kk] = (rr != 0xffffffffu && kk < kmax) ? X[uint64_t(rr) * d + k0 + kk] : 0.f;
            }
            __syncthreads();
            if (warp_local) {
                if (mine_local) {
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        if (cj[q] != 0xffffffffu)
                            fin_chunk_scalar2(fin_pair_col(lbase, q, d, k0), xs4[0][t], kmax, acc[q]);
                }
            } else {
#pragma unroll
                for (int q = 0; q < NSLOT; ++q)
                    if (cj[q] != 0xffffffffu) fin_chunk_scalar(C + uint64_t(cj[q]) * d + k0, xs4[0][t], kmax, acc[q]);
            }
        }
    }
    uint32_t best = 0xffffffffu;
    float bv = __int_as_float(0x7f800000);
#pragma unroll
    for (int q = 0; q < NSLOT; ++q) {
        if (cj[q] != 0xffffffffu && (best == 0xffffffffu || acc[q] < bv || (acc[q] == bv && cj[q] < best))) {
            bv = acc[q];
            best = cj[q];
        }
    }
    if (best == 0xffffffffu) return;
    asn[row] = best;
    costs[row] = double(bv);
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// looked up once per process (thread-safe static initialisation: server slots call this
// from several threads)
static EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(p);
        return EncodeTiledFn(nullptr);
    }();
    return fn;
}

static int make_map(CUtensorMap *map, const void *ptr, bool tf32, uint64_t rows, uint64_t cols, uint64_t pitch_elems,
                    uint32_t box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return fail(MC_ECUDA, "cuTensorMapEncodeTiled unavailable");
    const uint64_t esz = tf32 ? 4 : 2;
    cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
    cuuint64_t strides[1] = {cuuint64_t(pitch_elems * esz)};
    cuuint32_t box[2] = {cuuint32_t(tc::KBYTES / esz), box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                    const_cast<void *>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MC_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(int(r)));
    return MC_OK;
}

// Operands of the norm MMA of k_tc_top2_res, 32 bytes per row: A = (1, 1, 1, 0, ...) for every
// row; B row j = (h, m, l, 0, ...) with h + m + l = -||c_j||^2 / 2 in three BF16 (round to
// nearest) or TF32 (truncated) parts, each the remainder of the one before (exact in FP32);
// padding centers (j >= k) are zero rows (the epilogue sets their values to -inf).
__device__ inline float tf32_trunc(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__global__ void k_tc_aux_prep(const float *__restrict__ cnorm, uint32_t k, uint32_t kp, int tf32, uint32_t *auxa,
                              uint32_t *auxb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < tc::BM) {
        uint32_t *r = auxa + i * 8;
        for (int q = 0; q < 8; ++q) r[q] = 0u;
        if (tf32) {
            r[0] = r[1] = r[2] = __float_as_uint(1.f);
        } else {
            r[0] = 0x3F803F80u;  // bf16 1.0, 1.0
            r[1] = 0x00003F80u;  // bf16 1.0, 0
        }
    }
    if (i < kp) {
        uint32_t *r = auxb + uint64_t(i) * 8;
        for (int q = 0; q < 8; ++q) r[q] = 0u;
        if (i < k) {
            const float t = -0.5f * cnorm[i];
            if (tf32) {
                const float h = tf32_trunc(t), r1 = t - h, m = tf32_trunc(r1), l = tf32_trunc(r1 - m);
                r[0] = __float_as_uint(h);
                r[1] = __float_as_uint(m);
                r[2] = __float_as_uint(l);
            } else {
                const __nv_bfloat16 h = __float2bfloat16_rn(t);
                const float r1 = t - __bfloat162float(h);
                const __nv_bfloat16 m = __float2bfloat16_rn(r1);
                const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
                r[0] = uint32_t(__bfloat16_as_ushort(h)) | (uint32_t(__bfloat16_as_ushort(m)) << 16);
                r[1] = uint32_t(__bfloat16_as_ushort(l));
            }
        }
    }
}

// tensor map of a [rows][32 bytes] operand tile with the 32-byte swizzle (box: 32 bytes x box_rows)
static int make_map_aux(CUtensorMap *map, const void *ptr, bool tf32, uint64_t rows, uint32_t box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return fail(MC_ECUDA, "cuTensorMapEncodeTiled unavailable");
    const uint64_t esz = tf32 ? 4 : 2;
    cuuint64_t dims[2] = {cuuint64_t(32 / esz), cuuint64_t(rows)};
    cuuint64_t strides[1] = {32};
    cuuint32_t box[2] = {cuuint32_t(32 / esz), box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                    const_cast<void *>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MC_ECUDA, "cuTensorMapEncodeTiled (norm operands) failed: " + std::to_string(int(r)));
    return MC_OK;
}

// test hook: the next tensor-core pass 1 launched by this process stalls on purpose (one shot)
static std::atomic<int> g_tc_stall_next{0};
void tc_stall_next() { g_tc_stall_next.store(1); }

// Tile shapes of the tensor-core passes, as (BN, STAGES); the first kTcWideOnly need the
// padded center count to be a multiple of 256.  Every shape issues, per output element, the
// same chain of K-steps, and the exact FP32 finalize decides every assignment from the
// rounding bound, so all shapes give identical assignments and costs.
constexpr int kTcShapes = 4, kTcWideOnly = 2;

template <bool TF32, int MODE, int BN, int STAGES>
static int tc_launch_t(unsigned grid, const CUtensorMap &mA, const CUtensorMap &mB, TcArgs a, cudaStream_t st) {
    a.nchunks = a.kp / BN;
    const size_t smem = size_t(STAGES) * tc::Shape<BN, STAGES>::STAGE_BYTES + tc::CN_SMEM * sizeof(float) +
                        (MODE == TC_TOP2 ? sizeof(tc::PartX) : 0) + sizeof(tc::Smem<STAGES>) + 1024;
    auto kern = k_tc_assign<TF32, MODE, BN, STAGES>;
    MC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    kern<<<grid, tc::THREADS, smem, st>>>(mA, mB, a), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

template <bool TF32, int MODE>
static int tc_shape_launch(int shape, unsigned grid, const CUtensorMap &mA, const CUtensorMap &mB128,
                           const CUtensorMap &mB256, const TcArgs &a, cudaStream_t st) {
    switch (shape) {
        case 0: return tc_launch_t<TF32, MODE, 256, 4>(grid, mA, mB256, a, st);
        case 1: return tc_launch_t<TF32, MODE, 256, 3>(grid, mA, mB256, a, st);
        case 2: return tc_launch_t<TF32, MODE, 128, 4>(grid, mA, mB128, a, st);
        default: return tc_launch_t<TF32, MODE, 128, 6>(grid, mA, mB128, a, st);
    }
}

// Pass 1 with resident centers (k_tc_top2_res): usable when a row has at most two k-blocks
// and the centers fill whole 256-center chunks; G groups of GCH chunks, T = sms / G CTAs each.
struct ResPlan {
    bool ok = false;
    uint32_t G = 1, grid = 0, nchunks = 0;
    size_t smem = 0;
};

static ResPlan res_plan(uint32_t kb, uint32_t kp, int sms) {
    ResPlan p;
    if (kb < 1 || kb > 2 || kp % 256 != 0) return p;
    const uint32_t gch = kb == 1 ? tc::ResShape<1>::GCH : tc::ResShape<2>::GCH;
    p.nchunks = kp / 256;
    p.G = (p.nchunks + gch - 1) / gch;
    const uint32_t T = uint32_t(sms) / p.G;
    if (T < 2) return p;
    p.grid = T * p.G;
    p.smem = size_t(kb == 1 ? tc::ResShape<1>::SMEM : tc::ResShape<2>::SMEM) + sizeof(tc::ResSmem) + 1024;
    p.ok = true;
    return p;
}

template <bool TF32>
static int tc_res_launch(const ResPlan &p, uint32_t kb, const CUtensorMap &mA, const CUtensorMap &mB256,
                         const CUtensorMap &mAuxA, const CUtensorMap &mAuxB, TcArgs a, cudaStream_t st) {
    a.nchunks = p.nchunks;
    auto kern = kb == 1 ? k_tc_top2_res<TF32, 1> : k_tc_top2_res<TF32, 2>;
    MC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(p.smem)));
    kern<<<p.grid, tc::THREADS, p.smem, st>>>(mA, mB256, mAuxA, mAuxB, a, p.G, p.nchunks), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    return MC_OK;
}

int tc_assign(TcState &s, const float *X, uint64_t n, uint64_t d, const float *C, const float *cnorm, uint32_t k,
              int precision, const float *rownorm, uint32_t *asn, double *costs, int sms, cudaStream_t st,
              uint64_t *recheck_count, bool graph_mode) {
    const bool tf32 = precision == MC_TF32;
    const uint64_t esz = tf32 ? 4 : 2;
    const uint64_t kelems = tc::KBYTES / esz;            // K elements per k-block
    const uint64_t dp = (d + 7) / 8 * 8;                 // 16-byte row pitch for both types
    const uint32_t kb = uint32_t((d + kelems - 1) / kelems);
    const uint32_t kp = (k + tc::KP_ALIGN - 1) / tc::KP_ALIGN * tc::KP_ALIGN;
    const unsigned cg = unsigned(umin64((n * dp + 255) / 256, uint64_t(sms) * 64));
    // resident operand copy of the rows (once per matrix / precision)
    if (s.X_src != X || s.prec != precision || s.n != n || s.d != d) {
        if (tf32) {
            if (d % 4 == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0) {
                s.Xt.release();
            } else {
                MC_TRY(s.Xt.alloc(n * dp, st));
                k_pad_f32<<<cg, 256, 0, st>>>(X, n, d, dp, s.Xt.p), note_launch();
            }
        } else {
            MC_TRY(s.Xb.alloc(n * dp, st));
            if (dp == d && (reinterpret_cast<uintptr_t>(X) & 15) == 0)
                k_to_bf16_flat8<<<unsigned(umin64((n * d / 8 + 255) / 256, uint64_t(sms) * 16)), 256, 0, st>>>(
                    reinterpret_cast<const float4 *>(X), n * d / 8, reinterpret_cast<uint4 *>(s.Xb.p)), note_launch();
            else
                k_to_bf16_pad<<<cg, 256, 0, st>>>(X, n, d, dp, s.Xb.p), note_launch();
        }
        MC_CUDA_TRY(cudaGetLastError());
        s.X_src = X;
        s.prec = precision;
        s.n = n;
        s.d = d;
        s.dp = dp;
    }
    const void *Aptr = tf32 ? (s.Xt.p ? (const void *)s.Xt.p : (const void *)X) : (const void *)s.Xb.p;
    const uint64_t apitch = tf32 ? (s.Xt.p ? dp : d) : dp;
    // centers: padded operand copy + max norm
    MC_TRY(s.cnorm_p.alloc(uint64_t(kp) + 1, st));  // padded norms + Cmax
    MC_CUDA_TRY(cudaMemsetAsync(s.cnorm_p.p + kp, 0, sizeof(float), st));
    if (tf32) MC_TRY(s.Ct.alloc(uint64_t(kp) * dp, st));
    else MC_TRY(s.Cb.alloc(uint64_t(kp) * dp, st));
    k_center_prep_tc<<<unsigned(umin64((uint64_t(kp) * dp + 255) / 256, 4096)), 256, 0, st>>>(
        C, k, kp, d, dp, tf32 ? 1 : 0, s.Cb.p, s.Ct.p, cnorm, s.cnorm_p.p), note_launch();
    MC_CUDA_TRY(cudaGetLastError());
    CUtensorMap mA, mB128, mB256;
    const bool wide = kp % 256 == 0;  // the BN = 256 shapes need whole 256-center chunks
    MC_TRY(make_map(&mA, Aptr, tf32, n, d, apitch, tc::BM));
    const void *Bptr = tf32 ? (const void *)s.Ct.p : (const void *)s.Cb.p;
    MC_TRY(make_map(&mB128, Bptr, tf32, kp, d, dp, 128));
    if (wide) MC_TRY(make_map(&mB256, Bptr, tf32, kp, d, dp, 256));
    using tc::PARTS;
    const ResPlan rp = res_plan(kb, kp, sms);
    // pass 1 writes one merged entry per row (k_tc_assign) or one per center group and column
    // part (k_tc_top2_res)
    const uint64_t ngmax = rp.ok ? uint64_t(rp.G) * PARTS : 1;
    MC_TRY(s.b1.alloc(n * ngmax, st));
    MC_TRY(s.b2.alloc(n * ngmax, st));
    MC_TRY(s.j1.alloc(n * ngmax, st));
    CUtensorMap mAuxA, mAuxB;
    if (rp.ok) {
        MC_TRY(s.auxa.alloc(uint64_t(tc::BM) * 8, st));
        MC_TRY(s.auxb.alloc(uint64_t(kp) * 8, st));
        k_tc_aux_prep<<<(kp > tc::BM ? kp : tc::BM) / 128 + 1, 128, 0, st>>>(cnorm, k, kp, tf32 ? 1 : 0, s.auxa.p,
                                                                          s.auxb.p), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        MC_TRY(make_map_aux(&mAuxA, s.auxa.p, tf32, tc::BM, tc::BM));
        MC_TRY(make_map_aux(&mAuxB, s.auxb.p, tf32, kp, 256));
    }
    MC_TRY(s.status.alloc(n, st));
    MC_TRY(s.key.alloc(n, st));
    const uint32_t nsg = kp / 8;  // subgroups of 8 centers
    // compact buffer for the multi rows: all rows up to 2^20, else half of them (rows
    // beyond the capacity are rescanned exactly)
    const uint64_t cap = n <= (1u << 20) ? n : (n / 2 > (1u << 20) ? n / 2 : (1u << 20));
    const uint64_t row_u4 = apitch * esz / 16;
    MC_TRY(s.crow.alloc(cap, st));
    MC_TRY(s.thrc.alloc(cap, st));
    MC_TRY(s.Xc.alloc(cap * row_u4, st));
    MC_TRY(s.cnt.alloc(PARTS * cap, st));
    MC_TRY(s.cand.alloc(cap * NSLOT, st));
    MC_TRY(s.count.alloc(1, st));
    MC_TRY(s.err.alloc(1, st));
    MC_TRY(s.nrecheck.alloc(2, st));
    MC_TRY(s.over_rows.alloc(n, st));
    MC_CUDA_TRY(cudaMemsetAsync(s.err.p, 0, sizeof(int), st));
    MC_CUDA_TRY(cudaMemsetAsync(s.count.p, 0, sizeof(unsigned), st));
    MC_CUDA_TRY(cudaMemsetAsync(s.nrecheck.p, 0, 2 * sizeof(unsigned long long), st));
    CUtensorMap mC;
    MC_TRY(make_map(&mC, s.Xc.p, tf32, cap, d, apitch, tc::BM));
    TcArgs a;
    a.n = n;
    a.d = d;
    a.k = k;
    a.kb = kb;
    a.nchunks = 0;  // set per tile shape
    a.ntiles = uint32_t((n + tc::BM - 1) / tc::BM);
    a.rownorm = rownorm;
    a.cnp = s.cnorm_p.p;
    a.kp = kp;
    const double u = tf32 ? 1.0 / 1024.0 : 1.0 / 256.0;  // unit roundoff of the operands (see above)
    a.eta = float(2 * u + u * u + double(d) * std::ldexp(1.0, -22));
    const double g = double(d) * std::ldexp(1.0, -24);
    a.gamma = float(g / (1.0 - g) * 2.0);
    a.b1 = s.b1.p;
    a.b2 = s.b2.p;
    a.j1 = s.j1.p;
    a.count = nullptr;
    a.thrc = nullptr;
    a.cnt = nullptr;
    a.cand = nullptr;
    a.err = s.err.p;
    a.stall_test = 0;
    TcArgs a2 = a;  // pass 2: compact rows, count read on the device
    a.stall_test = g_tc_stall_next.exchange(0);
    a2.n = cap;
    a2.count = s.count.p;
    a2.thrc = s.thrc.p;
    a2.cnt = s.cnt.p;
    a2.cand = s.cand.p;
    const unsigned grid = unsigned(umin64(a.ntiles, uint64_t(sms)));
    const unsigned grid2 = unsigned(umin64((cap + tc::BM - 1) / tc::BM, uint64_t(sms)));
    // tile shape per shape bucket (tc_shape_launch); the stall test hook and graph capture
    // take the recorded decision or the default
    const int nvar = wide ? kTcShapes : kTcShapes - kTcWideOnly;
    auto shape_of = [&](int v) { return wide ? v : v + kTcWideOnly; };
    const bool allow = !graph_mode && !a.stall_test;
    const std::string bucket = std::string(tf32 ? "|tf32" : "|bf16") + "|kp" + std::to_string(kp) + "|d" +
                               tune_bucket(d) + "|n" + tune_bucket(n);
    // pass 1 variants: the tile shapes, then (where it fits) the resident-centers kernel; the
    // output layout is that of the variant launched last
    uint32_t ngroups = 1;
    float nerr = 0.f;  // extra bound term (times Cmax^2) of pass 1 values that carry the norms
    {
        Phase ph("tc_pass1_top2", st);
        const int nvar1 = nvar + (rp.ok ? 1 : 0);
        MC_TRY(tune_launch("tc1" + bucket, nvar1, 0, st, allow, [&](int v) -> int {
            if (v == nvar) {
                ngroups = rp.G * PARTS;
                nerr = float(double(d + 1) * std::ldexp(1.0, -21) * 1.0001);
                return tf32 ? tc_res_launch<true>(rp, kb, mA, mB256, mAuxA, mAuxB, a, st)
                            : tc_res_launch<false>(rp, kb, mA, mB256, mAuxA, mAuxB, a, st);
            }
            ngroups = 1;
            nerr = 0.f;
            return tf32 ? tc_shape_launch<true, TC_TOP2>(shape_of(v), grid, mA, mB128, mB256, a, st)
                        : tc_shape_launch<false, TC_TOP2>(shape_of(v), grid, mA, mB128, mB256, a, st);
        }));
    }
    MC_CUDA_TRY(cudaGetLastError());
    {
        Phase ph("tc_select", st);
        k_tc_select<<<unsigned((n + 255) / 256), 256, 0, st>>>(
            n, s.b1.p, s.b2.p, s.j1.p, rownorm, s.cnorm_p.p + kp, a.eta, a.gamma, nsg, s.status.p, s.key.p,
            s.crow.p, s.thrc.p, s.count.p, uint32_t(cap), static_cast<const uint4 *>(Aptr), row_u4, s.Xc.p,
            s.over_rows.p, s.nrecheck.p + 1, s.nrecheck.p, ngroups, nerr), note_launch();
        MC_CUDA_TRY(cudaGetLastError());
        // finalize order: rows grouped by subgroup, then multi rows, then OVER rows
        MC_TRY(launch_sort_by_key(s.key.p, nullptr, n, nsg + 2, s.sort, st));
    }
    MC_CUDA_TRY(cudaGetLastError());
    {
        Phase ph("tc_pass2_candidates", st);
        MC_TRY(tune_launch("tc2" + bucket, nvar, 0, st, allow, [&](int v) -> int {
            return tf32 ? tc_shape_launch<true, TC_CAND>(shape_of(v), grid2, mC, mB128, mB256, a2, st)
                        : tc_shape_launch<false, TC_CAND>(shape_of(v), grid2, mC, mB128, mB256, a2, st);
        }));
    }
    MC_CUDA_TRY(cudaGetLastError());
    {
        Phase phf("tc_finalize_exact", st);
        const bool vec4 = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0) &&
                          ((reinterpret_cast<uintptr_t>(X) & 15) == 0);
        const size_t cs_bytes = size_t(FIN_SG) * 8 * d * sizeof(float);
        const int stage = cs_bytes <= 48 * 1024 ? 1 : 0;
        const size_t dyn = stage ? cs_bytes : 0;
        const unsigned fg = unsigned((n + FIN_ROWS - 1) / FIN_ROWS);
        // static (37 KB) + staged centers (up to 48 KB) exceeds the 48 KB default; always the
        // largest value, so concurrent callers never lower it under another's launch
        MC_CUDA_TRY(cudaFuncSetAttribute(k_tc_finalize<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 48 * 1024));
        MC_CUDA_TRY(cudaFuncSetAttribute(k_tc_finalize<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 48 * 1024));
        if (vec4)
            k_tc_finalize<true><<<fg, FIN_ROWS, dyn, st>>>(X, n, d, C, k, nsg, stage, asn, s.sort.perm.p, s.status.p,
                                                           s.cnt.p, s.cand.p, costs, s.over_rows.p, s.nrecheck.p + 1),
                note_launch();
        else
            k_tc_finalize<false><<<fg, FIN_ROWS, dyn, st>>>(X, n, d, C, k, nsg, stage, asn, s.sort.perm.p,
                                                            s.status.p, s.cnt.p, s.cand.p, costs, s.over_rows.p,
                                                            s.nrecheck.p + 1), note_launch();
    }
    MC_CUDA_TRY(cudaGetLastError());
    if (graph_mode) {
        // no host round trip: the FP32 rescan is launched for every row and reads the count
        // of rows without a candidate list on the device; s.err is read by the caller
        AssignArgs b;
        b.msr = SQRL2;
        b.n = n;
        b.n_dev = s.nrecheck.p + 1;
        b.d = d;
        b.k = k;
        b.kp = tiled_center_pad(k, false, SQRL2);
        b.X = X;
        b.rows = s.over_rows.p;
        MC_TRY(s.CT0.alloc(uint64_t(b.kp) * d, st));
        b.CT0 = s.CT0.p;
        b.asn = asn;
        b.costs = costs;
        MC_TRY(launch_prep_centers(b, C, false, false, st));
        MC_TRY(launch_assign_tiled(b, false, false, st, /*tune=*/false));
        if (recheck_count) *recheck_count = 0;
        return MC_OK;
    }
    int err = 0;
    unsigned long long nr[2] = {0, 0};
    MC_CUDA_TRY(cudaMemcpyAsync(&err, s.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaMemcpyAsync(nr, s.nrecheck.p, sizeof(nr), cudaMemcpyDeviceToHost, st));
    MC_CUDA_TRY(cudaStreamSynchronize(st));
    if (err) return fail(MC_ETIMEOUT, "tensor-core assignment: bounded wait expired (code " + std::to_string(err) + ")");
    if (nr[1]) {
        // rows without a usable candidate list: exact FP32 scan over all centers
        AssignArgs b;
        b.msr = SQRL2;
        b.n = nr[1];
        b.d = d;
        b.k = k;
        b.kp = tiled_center_pad(k, false, SQRL2);
        b.X = X;
        b.rows = s.over_rows.p;
        MC_TRY(s.CT0.alloc(uint64_t(b.kp) * d, st));
        b.CT0 = s.CT0.p;
        b.asn = asn;
        b.costs = costs;
        Phase ph("tc_rescan_fp32", st);
        MC_TRY(launch_prep_centers(b, C, false, false, st));
        MC_TRY(launch_assign_tiled(b, false, false, st, /*tune=*/false));
    }
    if (recheck_count) *recheck_count = nr[0] + nr[1];
    return MC_OK;
}

}  // namespace mc
