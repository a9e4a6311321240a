// Stand-in for kern_user.cu in builds without a user plug-in header:
// CHAOS_SYS_USER is then reported as unsupported.
#include "launch.h"

namespace chaos {
bool user_system_available() { return false; }
void user_system_sizes(int* nx, int* na) {
    *nx = 0;
    *na = 0;
}
cudaError_t launch_bif_user(const SweepParams&, const BifOut&, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_basins_user(const SweepParams&, const BasinsOut&, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_lle_user(const LleParams&, double*, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_trajectory_user(const double*, const double*, double, int, double*, long long, cudaStream_t) {
    return cudaErrorNotSupported;
}
}  // namespace chaos
