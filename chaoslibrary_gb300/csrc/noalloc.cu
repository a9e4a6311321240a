// Allocation-free entry point: the per-point interval clustering of the 2-D
// bifurcation (the kernel behind chaos_point_dbscan) with its scratch rows in
// a fixed array compiled into the library instead of memory allocated per call.
//
// Who needs it: callers that cannot call cudaMalloc while they run -- hosts
// that reserve all device memory up front through their own allocator and
// budget (a framework's caching allocator, an MPS client with a memory limit),
// where a library-side cudaMalloc can fail or break the host's accounting, and
// latency-critical loops where cudaMalloc / cudaFree would synchronise the
// device. The caller provides every input and output in device memory; this
// call allocates nothing.
//
// The scratch array costs kNoAllocMaxEntries * 2 * 4 bytes = 8 MiB on every
// GPU that loads the library, held until the process exits. All calls share
// it: two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.
// The kernel clears each row it uses before reading it, so the contents left
// by a previous call do not matter.
#include <cuda_runtime.h>

#include "../../include/chaos_gb300.h"
#include "capi_internal.h"
#include "launch.h"

namespace {

constexpr long long kNoAllocMaxEntries = 1LL << 20;  // n * stride limit: label and slot rows, int each

static __device__ __align__(256) int g_noalloc_scratch[2 * kNoAllocMaxEntries];

// Device address of the scratch array in the current device's context. The
// array's host-side name is only a stand-in, not a device address, so the
// address is looked up on every call (the lookup allocates nothing): a cached
// address would dangle after a cudaDeviceReset, which reloads the module.
int scratch_address(int** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return chaos::cuda_error(e, "scratch address");
    *out = static_cast<int*>(p);
    return CHAOS_OK;
}

}  // namespace

extern "C" int chaos_point_dbscan_noalloc(const chaos_exec* ex, const double* intervals, const int* counts,
                                          long long n, int stride, double eps, int* labels) {
    using namespace chaos;
    if (!ex || ex->memory != CHAOS_MEM_DEVICE)
        return set_error(CHAOS_E_ARGS, "chaos_point_dbscan_noalloc needs chaos_exec.memory = CHAOS_MEM_DEVICE "
                                       "(all arrays in device memory)");
    if (n < 0 || stride < 1 || (n > 0 && (!intervals || !counts || !labels)))
        return set_error(CHAOS_E_ARGS, "bad point dbscan arguments");
    if (n > 0 && n > kNoAllocMaxEntries / stride)
        return set_error(CHAOS_E_ARGS, "n * stride = %lld exceeds the fixed scratch of %lld entries of "
                                       "chaos_point_dbscan_noalloc; use chaos_point_dbscan",
                         n * (long long)stride, kNoAllocMaxEntries);
    if (n == 0) return CHAOS_OK;
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return cuda_error(e, "get device");
    const int dev = ex->device >= 0 ? ex->device : prev;
    if (dev != prev && (e = cudaSetDevice(dev)) != cudaSuccess) return cuda_error(e, "set device");
    int* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc == CHAOS_OK) {
        // NULL selects the legacy default stream here: this entry creates no stream of its own
        cudaStream_t st = ex->stream ? (cudaStream_t)ex->stream : cudaStreamLegacy;
        e = launch_point_dbscan(intervals, counts, n, stride, eps, scratch, scratch + kNoAllocMaxEntries, labels, st);
        if (e != cudaSuccess) rc = cuda_error(e, "point dbscan kernel");
    }
    if (dev != prev) cudaSetDevice(prev);
    return rc;
}
