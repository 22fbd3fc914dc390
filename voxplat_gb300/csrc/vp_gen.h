/* vp_gen.h — launch interface of the device world generator. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

enum : uint32_t { kGenTerrainSmall = 1, kGenTerrainCaves = 2 };

struct GenArgs {
	uint32_t kind;
	uint64_t seed;
	int hshift;
	uint32_t root_bitw;
	uint32_t max_bitw[3];
	uint32_t shadow_w;
};

/* Voxel volumes of the slab cz (all chunks with that cz, index cy*nx+cx). */
cudaError_t launch_gen_slab(const GenArgs &a, uint32_t cz, uint8_t *vols, cudaStream_t st);
/* Shadow-map rows of slab cz from its volumes. */
cudaError_t launch_gen_shadow(const GenArgs &a, uint32_t cz, const uint8_t *vols, uint16_t *shadow,
			      uint64_t shadow_len, cudaStream_t st);

cudaError_t launch_scatter_slab(const uint64_t *new_off, const uint32_t *new_len, uint32_t n, uint32_t first,
				uint64_t base, uint64_t *off, uint32_t *len, cudaStream_t st);

} // namespace vp
