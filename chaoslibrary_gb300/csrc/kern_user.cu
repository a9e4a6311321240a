// FP64 kernels of a user plug-in: a header in the reference's systems.cuh
// format (it defines SIZE_X, SIZE_A and CALC_DISCRETE_MODEL(X, a, h), one
// step of a discrete map on doubles; systems/systems.cuh:12-38 in the
// reference), compiled in as system CHAOS_SYS_USER. The build passes the
// header as CHAOS_USER_SYSTEM_HEADER and compiles this file with
// --fmad=false, like the built-in FP64 kernels.
#define CHAOS_USER_SYSTEM 1
#define CHAOS_USER_NX SIZE_X  // expanded after the header below has defined them
#define CHAOS_USER_NA SIZE_A

#include CHAOS_USER_SYSTEM_HEADER

#include "engine.cuh"
#include "legacy_lle.cuh"

namespace chaos {

template <> __device__ void user_step<double>(double* x, const double* a, double h) { CALC_DISCRETE_MODEL(x, a, h); }

namespace {
constexpr int kBlock = 128;
inline unsigned grid_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

__global__ void __launch_bounds__(kBlock) bif_kernel_user(SweepParams P, BifOut O) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.nPoints) return;
    if (P.legacyLoop) bif_point_legacy<SYS_USER>(P, O, P.pBegin + o, o);
    else bif_point<SYS_USER, double>(P, O, P.pBegin + o, o);
}
__global__ void __launch_bounds__(kBlock) basins_kernel_user(SweepParams P, BasinsOut O) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.nPoints) return;
    basins_point<SYS_USER, double>(P, O, P.pBegin + o, o);
}
__global__ void __launch_bounds__(kBlock) lle_kernel_user(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = L.legacyLoop  ? lle_point_legacy<SYS_USER>(L, L.pBegin + o)
             : L.twin == 2 ? lle_point_reftwin<SYS_USER>(L, L.pBegin + o)
                           : lle_point_full<SYS_USER, double>(L, L.pBegin + o);
}
__global__ void __launch_bounds__(kBlock) trajectory_kernel_user(const double* x0, const double* a0, double h,
                                                                 int nSteps, double* out, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    trajectory_point<SYS_USER, double>(x0, a0, h, nSteps, out, t);
}
}  // namespace

bool user_system_available() { return true; }
void user_system_sizes(int* nx, int* na) {
    *nx = SIZE_X;
    *na = SIZE_A;
}
cudaError_t launch_bif_user(const SweepParams& P, const BifOut& O, cudaStream_t st) {
    if (P.nPoints > 0) {
        bif_kernel_user<<<grid_for(P.nPoints), kBlock, 0, st>>>(P, O);
        note_launch();
    }
    return cudaGetLastError();
}
cudaError_t launch_basins_user(const SweepParams& P, const BasinsOut& O, cudaStream_t st) {
    if (P.nPoints > 0) {
        basins_kernel_user<<<grid_for(P.nPoints), kBlock, 0, st>>>(P, O);
        note_launch();
    }
    return cudaGetLastError();
}
cudaError_t launch_lle_user(const LleParams& L, double* out, cudaStream_t st) {
    if (L.nPoints > 0) {
        lle_kernel_user<<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out);
        note_launch();
    }
    return cudaGetLastError();
}
cudaError_t launch_trajectory_user(const double* x0, const double* a0, double h, int nSteps, double* out,
                                   long long n, cudaStream_t st) {
    if (n > 0) {
        trajectory_kernel_user<<<grid_for(n), kBlock, 0, st>>>(x0, a0, h, nSteps, out, n);
        note_launch();
    }
    return cudaGetLastError();
}

}  // namespace chaos
