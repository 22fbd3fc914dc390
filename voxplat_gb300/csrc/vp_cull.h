/* vp_cull.h — launch interface of the draw-cull / LOD-selection kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

struct CullArgs {
	float view_proj[16];            /* column-major */
	float origin[3];                /* LOD origin (camera position) */
	uint32_t root_bitw, max_bitw[3];
	uint32_t top;                   /* LOD level the walk starts from */
	uint32_t roots[3];              /* (max >> top) + 1 per axis */
	uint32_t nodes[kMaxLevels][3];  /* in-world octree nodes per level and axis */
	const ChunkOut *outs;           /* a chunk's mesh is drawn when vbo_items > 0 */
	const uint32_t *node_items;     /* [levels][nchunks] grouped items per node */
	uint32_t nchunks;
	uint32_t *slots;                /* cull_slots(a) words of scratch */
};

uint64_t cull_slots(const CullArgs &a);
/* block_counts: 2 * ceil(slots / 1024) words; totals: 2 words (mesh, splat) */
cudaError_t launch_cull(const CullArgs &a, uint32_t *block_counts, uint32_t *totals, uint32_t *mesh_out,
			uint32_t mesh_cap, uint32_t *svl_out, uint32_t svl_cap, cudaStream_t st);
cudaError_t launch_mesh_flags(const CullArgs &a, uint8_t *flags, cudaStream_t st);

} // namespace vp
