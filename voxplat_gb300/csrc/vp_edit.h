/* vp_edit.h — launch interface of the sphere-edit kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

struct EditDesc {
	int32_t c[3];     /* sphere centre (world voxels) */
	uint32_t r;       /* radius */
	uint32_t voxel;   /* value written; 0 carves */
	uint32_t nlist;   /* chunks in the edit's AABB list */
};

struct EditChunk {
	int32_t cv[3];    /* chunk coordinates */
	uint32_t vol_slot; /* decoded volume of this chunk in the batch */
};

/* One edit: voxel writes into the decoded volumes of its chunks and, for
 * fills, the shadow-map updates of its rows. `chunks` holds the edit's AABB
 * chunk list in the reference's order (x outer, y, z inner). */
cudaError_t launch_edit(const EditDesc &e, const EditChunk *chunks, uint32_t nchunks, uint8_t *vols,
			uint32_t root_bitw, uint16_t *shadow, uint64_t shadow_len, uint32_t shadow_w, cudaStream_t st);

cudaError_t launch_scatter_streams(const uint32_t *chunk_ids, uint32_t n, const uint64_t *new_off,
				   const uint32_t *new_len, uint64_t base, uint64_t *off, uint32_t *len, cudaStream_t st);

} // namespace vp
