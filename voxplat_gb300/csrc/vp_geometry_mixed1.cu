/* vp_geometry_mixed1.cu — k_geometry_mixed<1>, the persistent kernel over
 * work items of every root size, registers uncapped (one CTA per SM). */
#include "vp_geometry_dev.cuh"

namespace vp {

int geometry_mixed_ctas_per_sm_b1(int threads)
{
	int n = 0;
	cudaFuncSetAttribute(k_geometry_mixed<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo<6>::bytes);
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_geometry_mixed<1>, threads, Geo<6>::bytes) !=
	    cudaSuccess)
		return 1;
	return n;
}

cudaError_t launch_geometry_mixed_b1(uint32_t grid, const GeoLaunch &L, cudaStream_t st)
{
	cudaError_t e = cudaFuncSetAttribute(k_geometry_mixed<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
					     (int)Geo<6>::bytes);
	if (e != cudaSuccess) return e;
	k_geometry_mixed<1><<<grid, L.threads, Geo<6>::bytes, st>>>(L.sets, L.items, L.n_items, L.queue, L.outs, L.svl,
								     L.vbo, L.ibo, L.lod_max, L.big_scratch,
								     L.grain ? L.grain : 1u);
	return cudaGetLastError();
}

} // namespace vp
