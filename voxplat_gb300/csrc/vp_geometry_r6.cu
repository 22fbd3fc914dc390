/* vp_geometry_r6.cu — the shell and geometry kernels for chunks of 64^3
 * (k_shell<6>, k_geometry<6>) and their host launchers. */
#include "vp_geometry_dev.cuh"

namespace vp {

cudaError_t launch_geometry_r6(const GeoLaunch &L, cudaStream_t st) { return launch_rb<6>(L, st); }
int geometry_ctas_per_sm_r6(int threads) { return ctas_per_sm<6>(threads); }

} // namespace vp
