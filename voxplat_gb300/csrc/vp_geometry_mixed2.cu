/* vp_geometry_mixed2.cu — k_geometry_mixed<2>, the persistent kernel over
 * work items of every root size, registers capped for two CTAs per SM. */
#include "vp_geometry_dev.cuh"

namespace vp {

int geometry_mixed_ctas_per_sm_b2(int threads)
{
	int n = 0;
	cudaFuncSetAttribute(k_geometry_mixed<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo<6>::bytes);
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_geometry_mixed<2>, threads, Geo<6>::bytes) !=
	    cudaSuccess)
		return 1;
	return n;
}

cudaError_t launch_geometry_mixed_b2(uint32_t grid, const GeoLaunch &L, cudaStream_t st)
{
	cudaError_t e = cudaFuncSetAttribute(k_geometry_mixed<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
					     (int)Geo<6>::bytes);
	if (e != cudaSuccess) return e;
	k_geometry_mixed<2><<<grid, L.threads, Geo<6>::bytes, st>>>(L.sets, L.items, L.n_items, L.queue, L.outs, L.svl,
								     L.vbo, L.ibo, L.lod_max, L.big_scratch,
								     L.grain ? L.grain : 1u);
	return cudaGetLastError();
}

} // namespace vp
