// Tensor-core (tcgen05) SQRL2 assignment: BF16 / TF32 GEMM with FP32 accumulation in
// TMEM, fused ||x||^2 - 2 x.c + ||c||^2 epilogue with row min / second min / argmin, and
// an exact FP32 re-check of the rows whose margin falls below the rounding bound.
#pragma once
#include "mc_internal.cuh"
#include "mc_reduce.cuh"

namespace mc {

struct TcState {
    DBuf<__nv_bfloat16> Xb;      // [n][dp] bf16 copy of the rows (BF16 path)
    DBuf<float> Xt;              // [n][dp] tf32-ready copy (TF32 path, d padded)
    DBuf<__nv_bfloat16> Cb;      // [kp][dp]
    DBuf<float> Ct;              // [kp][dp]
    DBuf<float> cnorm_p;         // device scalar: max center norm
    DBuf<float> b1, b2;          // [n][entries] pass 1 top-2 subgroup minima per row (per group and part)
    DBuf<uint32_t> j1;           // [n][entries] subgroup of b1
    DBuf<uint32_t> status;       // [n] candidate subgroup / multi slot / rescan
    DBuf<uint32_t> key;          // [n] finalize order key (subgroup, multi, rescan)
    SortWork sort;               // rows sorted by key
    DBuf<uint32_t> crow;         // [cap] original row of each compact (multi) row
    DBuf<float> thrc;            // [cap] pass 2 threshold of each compact row
    DBuf<uint4> Xc;              // [cap][pitch] operand copy of the compact rows
    DBuf<unsigned> count;        // compact rows taken
    DBuf<uint8_t> cnt;           // [cap][4] pass 2 candidates per column part (255: too many)
    DBuf<uint32_t> cand;         // [cap][4][3] pass 2 candidate centers
    DBuf<int> err;               // bounded-wait error code
    DBuf<unsigned long long> nrecheck;   // [0] multi rows (pass 2), [1] rows rescanned
    DBuf<uint32_t> over_rows;    // rows rescanned over all centers
    DBuf<float> CT0;             // transposed centers for that rescan
    DBuf<uint32_t> auxa, auxb;   // norm MMA operands of the resident pass 1 (32 bytes per row)
    const float *X_src = nullptr;
    uint64_t n = 0, d = 0, dp = 0;
    int prec = -1;
};

int tc_assign(TcState &s, const float *X, uint64_t n, uint64_t d, const float *C, const float *cnorm, uint32_t k,
              int precision, const float *rownorm, uint32_t *asn, double *costs, int sms, cudaStream_t st,
              uint64_t *recheck_count, bool graph_mode = false);
// test hook: the next tensor-core pass 1 waits on a barrier nothing completes (one shot)
void tc_stall_next();
// BF16 copy (round to nearest) of n8 groups of eight floats: X and Y 16-byte aligned
int launch_to_bf16_flat8(const float *X, uint64_t n8, void *Y, int sms, cudaStream_t st);

}  // namespace mc
