/* vp_geometry_r3.cu — the shell and geometry kernels for chunks of 8^3
 * (k_shell<3>, k_geometry<3>) and their host launchers. */
#include "vp_geometry_dev.cuh"

namespace vp {

cudaError_t launch_geometry_r3(const GeoLaunch &L, cudaStream_t st) { return launch_rb<3>(L, st); }
int geometry_ctas_per_sm_r3(int threads) { return ctas_per_sm<3>(threads); }

} // namespace vp
