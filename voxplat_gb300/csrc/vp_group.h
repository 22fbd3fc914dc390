/* vp_group.h — launch interface of the LOD/octree grouping kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

struct GroupArgs {
	uint32_t max_bitw[3];
	uint64_t *counts;      /* [levels][nchunks] scratch: counts, then prefixes */
	uint64_t *level_total; /* [levels] int16 items per level */
	uint64_t *node_off;    /* [levels][nchunks] node start (int16 units): level 0 in the
	                        * splat arena, levels >= 1 in `out` */
	uint32_t *node_items;  /* [levels][nchunks] node length (int16 units) */
	const int16_t *svl;    /* per-chunk splat lists (the splat arena) */
	int16_t *out;          /* grouped lists of levels >= 1: level 1 nodes, then level 2 ... */
	const unsigned long long *svl_cursor; /* the splat arena's bump cursor (16 B units) */
	uint64_t svl_cap_units;               /* the splat arena's capacity (16 B units) */
	uint64_t out_cap;                     /* capacity of `out` (int16 units) */
};

cudaError_t launch_group(const ChunkOut *outs, uint32_t nchunks, int lod_max, const GroupArgs &a, cudaStream_t st);

} // namespace vp
