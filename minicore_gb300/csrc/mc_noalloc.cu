// mc_assign_sqrl2_noalloc: the dense SQRL2 FP32 assignment pass without any device
// allocation.
//
// Some callers cannot allocate device memory on the call path: hosts that reserve their
// whole GPU memory budget at start-up and forbid later allocations (fixed-footprint
// services, memory pools owned by another runtime), or callers that only hand the library
// buffers they already own.  For them this entry point keeps its one scratch buffer (the
// centers transposed to [d][kp]) in a fixed file-scope device array, so a call allocates
// nothing: the caller passes device pointers for the rows, the centers and both outputs.
//
// Rules of use:
//  * scratch capacity: kp * d <= MC_NOALLOC_SCRATCH_FLOATS (4 MiB of floats), where kp is k
//    rounded up to a multiple of 64 (k < 128) or 128 (k >= 128); larger shapes are rejected
//    with MC_EINVAL;
//  * the first call on a device looks up the array's device address for that device
//    (cudaGetSymbolAddress with the device current), which may load this file's module and
//    with it the 4 MiB array: a one-time cost of the first call.  Make that first call
//    before any stream capture; a first call on a stream that is being captured is
//    refused with MC_EINVAL before it touches the runtime's module state;
//  * every pointer must be device memory of the current device (or managed memory), and
//    the stream must belong to the current device: memory of another GPU is refused rather
//    than read across the link;
//  * every call on a device shares the one array, and it keeps the last call's contents:
//    two calls whose kernels overlap on the GPU (different streams, no ordering between
//    them) race on it.  Order such calls on one stream or with events.
//  * every scratch element the kernel reads is written by the same call first, so nothing
//    has to start at zero.
// The array stays resident on every GPU that loads this library until the process exits.
#include <mutex>

#include "mc_assign.cuh"

namespace mc {

constexpr uint64_t kNoallocScratchFloats = 1ull << 20;  // == MC_NOALLOC_SCRATCH_FLOATS

static __device__ __align__(256) float g_noalloc_scratch[kNoallocScratchFloats];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
float *g_noalloc_ptr[kMaxDevices] = {};

// device address of the scratch array for the current device (set up once per device,
// never while `st` is being captured into a graph)
int noalloc_scratch(float **out, cudaStream_t st) {
    int dev = 0;
    MC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(MC_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        MC_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(MC_EINVAL, "mc_assign_sqrl2_noalloc: the first call on a device sets up its scratch "
                                   "address and must not run inside a stream capture");
        void *p = nullptr;
        MC_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (!p) return fail(MC_ECUDA, "scratch array has no device address");
        g_noalloc_ptr[dev] = static_cast<float *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return MC_OK;
}
}  // namespace

}  // namespace mc

extern "C" int mc_assign_sqrl2_noalloc(const float *X, uint64_t n, uint64_t d, const float *centers, uint32_t k,
                                       uint32_t *asn, double *costs, void *cuda_stream) {
    using namespace mc;
    if (!X || !centers || !asn || !costs) return fail(MC_EINVAL, "null pointer argument");
    if (n == 0 || d == 0 || k == 0) return fail(MC_EINVAL, "empty rows, columns or centers");
    if (n >= (1ull << 32)) return fail(MC_EINVAL, "more than 2^32-1 rows");
    if (!is_device_ptr(X) || !is_device_ptr(centers) || !is_device_ptr(asn) || !is_device_ptr(costs))
        return fail(MC_EINVAL, "mc_assign_sqrl2_noalloc takes device pointers of the current device only");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    if (st) {
        int dev = -1, sdev = -1;
        MC_CUDA_TRY(cudaGetDevice(&dev));
        MC_CUDA_TRY(cudaStreamGetDevice(st, &sdev));
        if (sdev != dev) return fail(MC_EINVAL, "mc_assign_sqrl2_noalloc: the stream belongs to another device");
    }
    const uint32_t kp = tiled_center_pad(k, false, SQRL2);
    if (uint64_t(kp) * d > kNoallocScratchFloats)
        return fail(MC_EINVAL, "mc_assign_sqrl2_noalloc: padded centers x columns (" +
                                   std::to_string(uint64_t(kp) * d) + ") exceed the scratch capacity of " +
                                   std::to_string(kNoallocScratchFloats) + " floats");
    float *scratch = nullptr;
    MC_TRY(noalloc_scratch(&scratch, st));
    AssignArgs a;
    a.msr = SQRL2;
    a.n = n;
    a.d = d;
    a.k = k;
    a.kp = kp;
    a.X = X;
    a.CT0 = scratch;
    a.asn = asn;
    a.costs = costs;
    MC_TRY(launch_prep_centers(a, centers, false, false, st));
    return launch_assign_tiled(a, false, false, st, /*tune=*/false);
}
