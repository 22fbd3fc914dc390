/* vp_raycast.h — launch interface of the picking-ray kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

struct RayWorld {
	const uint32_t *pool;
	const uint64_t *off;
	const uint32_t *len;
	const uint32_t *runidx;   /* run-start index, parallel to pool */
	uint32_t root_bitw, max_bitw[3];
};

cudaError_t launch_run_starts(const uint32_t *pool, const uint64_t *off, const uint32_t *len, uint32_t nchunks,
			      uint32_t *runidx, cudaStream_t st);
/* origins / vectors: n x 3 floats; voxels n, coords n x 3, normals n x 3 */
cudaError_t launch_raycast(const RayWorld &W, const float *origins, const float *vectors, uint32_t n, uint8_t *voxels,
			   uint32_t *coords, int8_t *normals, cudaStream_t st);

} // namespace vp
