// Batched execution of many independent sweeps in one submission.
//
// A batch is a list of jobs (1-D bifurcation, LLE map or basins features;
// any built-in system; uneven sizes and transients). The host cuts every job
// into block-sized chunks of points and groups the chunks by (kind, system),
// each group ordered longest-work-per-point first. Every group gets one
// persistent kernel (resident blocks x SMs, at most one block per chunk)
// that pulls its chunks from a device counter (the work queue); the groups'
// kernels run concurrently on forked streams. A block works on one chunk at
// a time, so every warp runs one job's code path. Each point runs the same
// device function as the single-sweep kernels, so its result does not depend
// on the batch, chunk or block it ran in.
//
// Batches are FP32 (trajectories in FP32 registers, FP64 accumulation) but
// for the float-float LLE jobs, whose group kernel lives with the other FF
// kernels (kern_ff.cu, compiled without contraction); the
// jobs of the RK4 systems run two points per thread (packed FP32x2 lanes; the
// bifurcation jobs in the hybrid form), the others one. A prepared batch is
// replayed from a captured CUDA graph (counter reset + the group kernels).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "batch.h"
#include "capi_internal.h"
#include "engine.cuh"

namespace chaos {

namespace {

constexpr int kBatchBlock = 128;

template <int S> struct FieldOf;
template <> struct FieldOf<SYS_LORENZ_RK4> { using F = Lorenz; };
template <> struct FieldOf<SYS_ROSSLER_RK4> { using F = Rossler; };
template <> struct FieldOf<SYS_CHEN_RK4> { using F = Chen; };

// Bifurcation chunks: the RK4 systems as hybrid pairs (packed transient,
// recorded part lane by lane; chunks of two blocks' worth of points), the
// others one point per thread.
template <int S>
__device__ __forceinline__ void run_bif(const JobDesc& J, long long b, int cnt) {
    __shared__ SweepParams sP;
    if (threadIdx.x == 0) sP = J.sp;
    __syncthreads();
    if constexpr (S <= SYS_CHEN_RK4) {
#pragma unroll 1
        for (int t = 2 * threadIdx.x; t < cnt; t += 2 * blockDim.x) {
            const long long p = b + t;
            const bool two = t + 1 < cnt;
            bif_hybrid_point<typename FieldOf<S>::F>(sP, J.bif, p, two ? p + 1 : p, p, two ? p + 1 : p, two);
        }
    } else {
#pragma unroll 1
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) bif_point<S, float>(sP, J.bif, b + t, b + t);
    }
}

// Basins chunks: the RK4 systems as packed pairs (the single sweep's default
// form for large maps), the others one point per thread.
template <int S, bool PRE1>
__device__ __forceinline__ void run_basins_as(const SweepParams& sP, const JobDesc& J, long long b, int cnt) {
    if constexpr (S <= SYS_CHEN_RK4) {
#pragma unroll 1
        for (int t = 2 * threadIdx.x; t < cnt; t += 2 * blockDim.x) {
            const long long p = b + t;
            const bool two = t + 1 < cnt;
            basins_pair_point<typename FieldOf<S>::F, PRE1>(sP, J.bas, p, two ? p + 1 : p, p, two ? p + 1 : p,
                                                            two);
        }
    } else {
#pragma unroll 1
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) basins_point<S, float, PRE1>(sP, J.bas, b + t, b + t);
    }
}

template <int S>
__device__ __forceinline__ void run_basins(const JobDesc& J, long long b, int cnt) {
    __shared__ SweepParams sP;
    if (threadIdx.x == 0) sP = J.sp;
    __syncthreads();
    if (sP.preScaller == 1) run_basins_as<S, true>(sP, J, b, cnt);
    else run_basins_as<S, false>(sP, J, b, cnt);
}

// The job's parameter block is staged in shared memory for the chunk: read
// from there, the step loop keeps fewer values in registers than when it
// reads them through the global descriptor.
template <class F>
__device__ __forceinline__ void run_lle(const JobDesc& J, long long b, int cnt) {
    __shared__ LleParams sL;
    if (threadIdx.x == 0) sL = J.lp;
    __syncthreads();
    const LleParams& L = sL;
#pragma unroll 1
    for (int t = 2 * threadIdx.x; t < cnt; t += 2 * blockDim.x) {
        const long long p = b + t;
        const bool two = t + 1 < cnt;
        lle_pair_twin<F>(L, p, two ? p + 1 : p, J.lle + p, two ? J.lle + p + 1 : nullptr);
    }
}

// Chameleon LLE chunks: one point per thread, the twin as the difference of
// chameleon_step_twin (lle_point_twin_chameleon, as the single-sweep kernel).
__device__ __forceinline__ void run_lle_chameleon(const JobDesc& J, long long b, int cnt) {
    __shared__ LleParams sL;
    if (threadIdx.x == 0) sL = J.lp;
    __syncthreads();
#pragma unroll 1
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) J.lle[b + t] = lle_point_twin_chameleon(sL, b + t);
}

// Persistent kernel of one (kind, system) group: pulls chunks [0, count) of
// the group's range from its counter until none is left. One kernel per
// group keeps each code path's register allocation as small as the
// single-sweep kernel's (a kernel that switched over every kind and system
// would be sized for the largest of them).
template <int KIND, int S>
__global__ void __launch_bounds__(kBatchBlock) group_kernel(const JobDesc* __restrict__ jobs,
                                                            const Chunk* __restrict__ chunks, int count,
                                                            int* counter) {
    __shared__ int slot;
    for (;;) {
        if (threadIdx.x == 0) slot = atomicAdd(counter, 1);
        __syncthreads();
        const int c = slot;
        __syncthreads();
        if (c >= count) return;
        const Chunk ch = chunks[c];
        const JobDesc& J = jobs[ch.job];
        if (KIND == CHAOS_JOB_BIF1D) run_bif<S>(J, ch.begin, ch.count);
        else if (KIND == CHAOS_JOB_BASINS) run_basins<S>(J, ch.begin, ch.count);
        else if constexpr (S <= SYS_CHEN_RK4) run_lle<typename FieldOf<S>::F>(J, ch.begin, ch.count);
        else if constexpr (S == SYS_CHAMELEON) run_lle_chameleon(J, ch.begin, ch.count);
    }
}

__global__ void reset_counters_kernel(int* counters, int n) {
    if ((int)threadIdx.x < n) counters[threadIdx.x] = 0;
}

using GroupKernel = void (*)(const JobDesc*, const Chunk*, int, int*);

template <int KIND>
GroupKernel kernel_for_system(int s) {
    switch (s) {
        case SYS_LORENZ_RK4: return group_kernel<KIND, SYS_LORENZ_RK4>;
        case SYS_ROSSLER_RK4: return group_kernel<KIND, SYS_ROSSLER_RK4>;
        case SYS_CHEN_RK4: return group_kernel<KIND, SYS_CHEN_RK4>;
        case SYS_CHAMELEON: return group_kernel<KIND, SYS_CHAMELEON>;
        case SYS_ROSSLER_CD: return KIND == CHAOS_JOB_LLE2D ? nullptr : group_kernel<KIND, SYS_ROSSLER_CD>;
        case SYS_SIN3: return KIND == CHAOS_JOB_LLE2D ? nullptr : group_kernel<KIND, SYS_SIN3>;
        case SYS_SIN2: return KIND == CHAOS_JOB_LLE2D ? nullptr : group_kernel<KIND, SYS_SIN2>;
        case SYS_MEMRISTOR: return KIND == CHAOS_JOB_LLE2D ? nullptr : group_kernel<KIND, SYS_MEMRISTOR>;
        default: return nullptr;
    }
}

GroupKernel group_kernel_for(int kind, int system) {
    switch (kind) {
        case CHAOS_JOB_BIF1D: return kernel_for_system<CHAOS_JOB_BIF1D>(system);
        case CHAOS_JOB_BASINS: return kernel_for_system<CHAOS_JOB_BASINS>(system);
        case CHAOS_JOB_LLE2D: return kernel_for_system<CHAOS_JOB_LLE2D>(system);
        default: return nullptr;
    }
}

}  // namespace

int batch_block_size() { return kBatchBlock; }

int group_resident_blocks(int kind, int system, int device) {
    if (kind == CHAOS_JOB_LLE2D_FF32) return group_ff_resident_blocks(system, device);
    GroupKernel k = group_kernel_for(kind, system);
    if (!k) return 0;
    int perSm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, kBatchBlock, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return std::max(perSm, 1) * std::max(sms, 1);
}

cudaError_t reset_counters(int* counters, int n, cudaStream_t st) {
    reset_counters_kernel<<<1, 32, 0, st>>>(counters, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_group(int kind, int system, const JobDesc* jobs, const Chunk* chunks, int count, int* counter,
                         int gridBlocks, cudaStream_t st) {
    if (kind == CHAOS_JOB_LLE2D_FF32) return launch_group_ff(system, jobs, chunks, count, counter, gridBlocks, st);
    GroupKernel k = group_kernel_for(kind, system);
    if (!k) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    k<<<gridBlocks, kBatchBlock, 0, st>>>(jobs, chunks, count, counter);
    note_launch();
    return cudaGetLastError();
}

}  // namespace chaos
