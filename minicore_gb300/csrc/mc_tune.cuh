// Kernel-variant autotuner (mc_tune.cu).
#pragma once
#include <functional>
#include <string>

#include "mc_internal.cuh"

namespace mc {

// Launches one of `nvariants` variants of a kernel for the shape bucket `key`.  Every
// variant must write the same results (same per-element arithmetic and summation order)
// and be idempotent, so timing them changes nothing but speed.  On the first call for a
// key, unless the cache holds it, each variant runs twice on `st` (CUDA events) and the
// fastest is kept; later calls launch the kept variant only.  With tuning off, the default
// runs; when `allow` is false (callers that must not synchronise: the loops that run without
// host round trips, stream capture), a recorded decision runs, else the default.
int tune_launch(const std::string &key, int nvariants, int default_variant, cudaStream_t st, bool allow,
                const std::function<int(int)> &launch);

// log2 bucket of a size ("2^k", the next power of two at or above v)
std::string tune_bucket(uint64_t v);

}  // namespace mc
