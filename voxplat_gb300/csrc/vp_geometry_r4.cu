/* vp_geometry_r4.cu — the shell and geometry kernels for chunks of 16^3
 * (k_shell<4>, k_geometry<4>) and their host launchers. */
#include "vp_geometry_dev.cuh"

namespace vp {

cudaError_t launch_geometry_r4(const GeoLaunch &L, cudaStream_t st) { return launch_rb<4>(L, st); }
int geometry_ctas_per_sm_r4(int threads) { return ctas_per_sm<4>(threads); }

} // namespace vp
