#include "mc_tc.cuh"

namespace mc {

int tc_assign(TcState &, const float *, uint64_t, uint64_t, const float *, const float *, uint32_t, int,
              const float *, uint32_t *, double *, int, cudaStream_t, uint64_t *) {
    return fail(MC_EUNSUPPORTED, "tensor-core assignment not built");
}

}  // namespace mc
