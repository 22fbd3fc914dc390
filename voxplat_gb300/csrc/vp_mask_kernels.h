/* vp_mask_kernels.h — launch interface of the dense-mask kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

/* work[c] = last nonzero child of c in scan order, for children in
 * [0, range)^3 of an S^3 mask (S = R + 1). */
cudaError_t launch_downsample(const uint8_t *mask, uint8_t *work, uint32_t S, uint32_t range, cudaStream_t st);

/* Splats of the nonzero cells of [0, range)^3, in scan order, for LOD
 * `level` of the chunk whose first voxel is at world wbase; *count cells. */
cudaError_t launch_splatlist(const uint8_t *mask, uint32_t S, uint32_t range, uint32_t level, const uint32_t wbase[3],
			     const SetDesc &sd, int16_t *out, uint32_t *count, cudaStream_t st);

} // namespace vp
