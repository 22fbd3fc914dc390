/* vp_geometry_r5.cu — the shell and geometry kernels for chunks of 32^3
 * (k_shell<5>, k_geometry<5>) and their host launchers. */
#include "vp_geometry_dev.cuh"

namespace vp {

cudaError_t launch_geometry_r5(const GeoLaunch &L, cudaStream_t st) { return launch_rb<5>(L, st); }
int geometry_ctas_per_sm_r5(int threads) { return ctas_per_sm<5>(threads); }

} // namespace vp
