// FP32 FMA-pipe probe: the denominator of the integration kernels' roofline.
// Every thread runs 8 independent fmaf chains; the result is stored so the
// work cannot be removed. flops = threads * iters * 8 * 2.
#include <cuda_runtime.h>

#include "../../include/chaos_gb300.h"
#include "capi_internal.h"

namespace {
__global__ void __launch_bounds__(256) fma_probe_kernel(long long iters, float* sink) {
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 1.0f + 1e-7f * (threadIdx.x + j);
    const float b = 0.9999999f, c = 1e-7f;
    for (long long i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == 12345.678f) sink[threadIdx.x] = s;  // practically never taken
}
}  // namespace

extern "C" int chaos_fma_probe(const chaos_exec* ex, long long iters, double* seconds, double* flops) {
    using namespace chaos;
    if (iters < 1 || !seconds || !flops) return set_error(CHAOS_E_ARGS, "bad probe arguments");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const unsigned grid = (unsigned)sms * 8;  // 8 blocks x 256 threads = 2048 threads per SM
    float* sink = (float*)c.alloc(256 * sizeof(float));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_probe_kernel<<<grid, 256, 0, c.stream>>>(iters / 8 + 1, sink);  // warm-up
    note_launch();
    cudaEventRecord(e0, c.stream);
    fma_probe_kernel<<<grid, 256, 0, c.stream>>>(iters, sink);
    note_launch();
    cudaEventRecord(e1, c.stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return c.finish(cuda_error(e, "fma probe"));
    *seconds = ms * 1e-3;
    *flops = (double)grid * 256.0 * (double)iters * 16.0;
    return c.finish(CHAOS_OK);
}

extern "C" int chaos_device_code_version(int device, int* binaryVersion, int* ptxVersion) {
    using namespace chaos;
    if (!binaryVersion || !ptxVersion) return set_error(CHAOS_E_ARGS, "bad version arguments");
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return cuda_error(e, "get device");
    const int dev = device >= 0 ? device : prev;
    if (dev != prev && (e = cudaSetDevice(dev)) != cudaSuccess) return cuda_error(e, "set device");
    cudaFuncAttributes fa{};
    e = cudaFuncGetAttributes(&fa, fma_probe_kernel);
    if (dev != prev) cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_error(e, "function attributes");
    *binaryVersion = fa.binaryVersion;
    *ptxVersion = fa.ptxVersion;
    return CHAOS_OK;
}
