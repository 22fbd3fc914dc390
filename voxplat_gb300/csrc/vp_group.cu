/*
 * vp_group.cu — LOD/octree grouping of the splat lists (gfx_update_svl,
 * src/gfx/vsplat.c:209-331, without the GL upload).
 *
 * For LOD l, chunk c belongs to octree node offset >> l, whose members are
 * the chunks [node << l, min((node+1) << l, max)) scanned x outer, y, z
 * inner; the node's buffer is the concatenation of its members' level-l
 * splat segments in that order. Nodes are numbered flatten3(node,
 * max_bitw - min(l, max_bitw)) as in the reference.
 *
 * At LOD 0 every node is one chunk, so a node's buffer is that chunk's
 * level-0 segment as the geometry pass wrote it: the node table points into
 * the splat arena and nothing is copied (level 0 holds most of the splats).
 *
 * For LOD >= 1, with power-of-two chunk counts every node is full, so
 *   key(c) = node_index(c) * members + member_rank(c)
 * is a bijection onto [0, nchunks): the prefix sum of the level-l item
 * counts in key order gives every segment's destination, and node i's
 * buffer starts at the prefix of its first key. One pass writes the
 * level-0 node table and scatters the counts of the levels above into key
 * order, one CTA per level scans them, and a warp per segment (in a
 * small world, per eighth of a large level-1 segment) copies it with
 * 8-byte vector moves (one splat per lane per step, eight loads in flight
 * per lane) into the group arena.
 *
 * A rebuild whose splat arena overflowed left some chunks without lists
 * (their records carry the overflow status); the copy is then skipped as a
 * whole, and the host grows the arena and runs the rebuild and the grouping
 * again.
 */
#include <algorithm>

#include "vp_dev.cuh"
#include "vp_group.h"

namespace vp {

struct GroupGeom {
	uint32_t mb[3];   /* chunk count exponents */
	uint32_t eb[3];   /* member extent exponents: min(l, mb) */
	uint32_t ob[3];   /* node count exponents: mb - eb */
};

__device__ __forceinline__ GroupGeom group_geom(const uint32_t mb[3], int l)
{
	GroupGeom g;
	for (int i = 0; i < 3; i++) {
		g.mb[i] = mb[i];
		g.eb[i] = min((uint32_t)l, mb[i]);
		g.ob[i] = mb[i] - g.eb[i];
	}
	return g;
}

__device__ __forceinline__ uint32_t group_key(const GroupGeom &g, uint32_t c, uint32_t *node_index, uint32_t *rank)
{
	const uint32_t x = c & ((1u << g.mb[0]) - 1u);
	const uint32_t y = (c >> g.mb[0]) & ((1u << g.mb[1]) - 1u);
	const uint32_t z = c >> (g.mb[0] + g.mb[1]);
	const uint32_t nx = x >> g.eb[0], ny = y >> g.eb[1], nz = z >> g.eb[2];
	const uint32_t lx = x & ((1u << g.eb[0]) - 1u), ly = y & ((1u << g.eb[1]) - 1u), lz = z & ((1u << g.eb[2]) - 1u);
	*node_index = ((nz << g.ob[1] | ny) << g.ob[0]) | nx; /* flatten3 */
	*rank = ((lx << g.eb[1] | ly) << g.eb[2]) | lz;       /* x outer, z inner */
	return (*node_index << (g.eb[0] + g.eb[1] + g.eb[2])) | *rank;
}

/* One thread per chunk c and level l (all kMaxLevels levels):
 *   level 0: node c is chunk c, its list the chunk's level-0 segment in the
 *   splat arena;
 *   levels 1..lod_max: counts[l][key(c)] = the chunk's level-l splat items
 *   (int16 units), and the node table entry cleared (k_group_copy records
 *   the nodes that exist);
 *   levels above lod_max: the node table entry cleared. */
__global__ void k_group_tables(const ChunkOut *__restrict__ outs, uint32_t nchunks, int lod_max, GroupArgs a)
{
	grid_wait(); /* the geometry pass's result records */
	grid_release();
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	const int l = blockIdx.y;
	if (c >= nchunks) return;
	if (l == 0) {
		a.node_off[c] = outs[c].svl_off;
		a.node_items[c] = outs[c].svl_items[0];
		return;
	}
	a.node_items[(size_t)l * nchunks + c] = 0;
	if (l > lod_max) return;
	const GroupGeom g = group_geom(a.max_bitw, l);
	uint32_t node, rank;
	const uint32_t key = group_key(g, c, &node, &rank);
	a.counts[(size_t)l * nchunks + key] = outs[c].svl_items[l];
}

/* exclusive prefix sum of each level's counts, one CTA per level >= 1 */
__global__ void __launch_bounds__(1024) k_group_scan(uint32_t n, GroupArgs a)
{
	__shared__ uint64_t wsum[32];
	__shared__ uint64_t wexcl[32];
	__shared__ uint64_t s_tile, s_carry;
	grid_wait(); /* the scattered counts */
	grid_release();
	const int l = 1 + (int)blockIdx.x;
	uint64_t *v = a.counts + (size_t)l * n;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	if (threadIdx.x == 0) s_carry = 0;
	__syncthreads();
	/* four consecutive counts a thread per tile */
	constexpr uint32_t K = 4;
	for (uint32_t base = 0; base < n; base += K * blockDim.x) {
		const uint32_t i0 = base + K * threadIdx.x;
		uint64_t xs[K];
		uint64_t x = 0;
#pragma unroll
		for (uint32_t k = 0; k < K; k++) {
			xs[k] = i0 + k < n ? v[i0 + k] : 0ull;
			x += xs[k];
		}
		uint64_t inc = x;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint64_t t = __shfl_up_sync(kFull, inc, d);
			if (lane >= d) inc += t;
		}
		if (lane == 31) wsum[warp] = inc;
		__syncthreads();
		if (warp == 0) {
			const uint64_t w = lane < nw ? wsum[lane] : 0ull;
			uint64_t wi = w;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const uint64_t t = __shfl_up_sync(kFull, wi, d);
				if (lane >= d) wi += t;
			}
			wexcl[lane] = wi - w;
			if (lane == 31) s_tile = wi;
		}
		__syncthreads();
		uint64_t run = s_carry + wexcl[warp] + inc - x;
#pragma unroll
		for (uint32_t k = 0; k < K; k++) {
			if (i0 + k < n) v[i0 + k] = run;
			run += xs[k];
		}
		__syncthreads();
		if (threadIdx.x == 0) s_carry += s_tile;
		__syncthreads();
	}
	if (threadIdx.x == 0) a.level_total[l] = s_carry;
}

/* A level-1 segment (the largest) of at least kSliceMin splats is copied in
 * up to kL1Slices slices, one warp each, when the world has few segments for
 * the GPU's warps (the largest segments then set the copy's time); other
 * segments, and every segment of a large world, by one warp each. */
constexpr uint32_t kL1Slices = 8, kSliceMin = 1024;

/* levels >= 1: one warp per work unit, grid-stride: a slice of a chunk's
 * level-1 segment (l1_slices per chunk), or a chunk's whole segment of a
 * level >= 2. The warp copies it to its node's place, one splat (8 bytes)
 * per lane per step; the first unit of each node's first member also
 * records the node's offset and length. (A CTA per segment spent most of
 * its time on launching CTAs for the many empty segments of worlds with air
 * layers.) */
__global__ void __launch_bounds__(256) k_group_copy(const ChunkOut *__restrict__ outs, uint32_t nchunks, int levels,
						    uint32_t l1_slices, GroupArgs a)
{
	grid_wait(); /* the scanned counts */
	const int lane = threadIdx.x & 31;
	const uint32_t per_chunk = l1_slices + (uint32_t)(levels - 1);
	const uint64_t nwork = (uint64_t)nchunks * per_chunk;
	const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
	if (*a.svl_cursor > a.svl_cap_units) return; /* overflowed rebuild: rerun follows */
	for (uint64_t wu = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wu < nwork; wu += nwarps) {
		const uint32_t c = (uint32_t)(wu / per_chunk), j = (uint32_t)(wu % per_chunk);
		const int l = j < l1_slices ? 1 : 1 + (int)(j - l1_slices + 1u);
		const uint32_t slice = j < l1_slices ? j : 0u;
		const uint32_t items = outs[c].svl_items[l];
		const uint32_t n = items / 4u; /* splats */
		const uint32_t nslices = (l == 1 && n >= kSliceMin) ? l1_slices : 1u;
		if (slice >= nslices) continue; /* a small segment: its first slice copies it */
		const GroupGeom g = group_geom(a.max_bitw, l);
		uint32_t node, rank;
		const uint32_t key = group_key(g, c, &node, &rank);
		uint64_t lbase = 0;
		for (int k = 1; k < l; k++) lbase += a.level_total[k];
		const uint64_t *cnt = a.counts + (size_t)l * nchunks;
		const uint64_t dst_off = lbase + cnt[key];
		if (slice == 0 && rank == 0 && lane == 0) {
			const uint32_t mbits = g.eb[0] + g.eb[1] + g.eb[2];
			const uint32_t next_key = (node + 1u) << mbits;
			const uint64_t end = next_key < nchunks ? cnt[next_key] : a.level_total[l];
			a.node_off[(size_t)l * nchunks + node] = dst_off;
			a.node_items[(size_t)l * nchunks + node] = (uint32_t)(end - cnt[key]);
		}
		if (!items) continue;
		uint64_t src_off = outs[c].svl_off;
		for (int k = 0; k < l; k++) src_off += outs[c].svl_items[k];
		if (src_off + items > a.svl_cap_units * 8u || dst_off + items > a.out_cap) continue;
		const uint2 *src = (const uint2 *)(a.svl + src_off);
		uint2 *dst = (uint2 *)(a.out + dst_off);
		const uint32_t lo = (uint32_t)((uint64_t)n * slice / nslices);
		const uint32_t hi = (uint32_t)((uint64_t)n * (slice + 1u) / nslices);
		/* eight loads in flight per lane before their stores */
		uint32_t s = lo + (uint32_t)lane;
		for (; s + 224u < hi; s += 256u) {
			uint2 v[8];
#pragma unroll
			for (int u = 0; u < 8; u++) v[u] = __ldg(src + s + 32u * u);
#pragma unroll
			for (int u = 0; u < 8; u++) dst[s + 32u * u] = v[u];
		}
		for (; s < hi; s += 32u) dst[s] = __ldg(src + s);
	}
}

cudaError_t launch_group(const ChunkOut *outs, uint32_t nchunks, int lod_max, const GroupArgs &a, cudaStream_t st)
{
	if (!nchunks) return cudaSuccess;
	const int L = lod_max + 1;
	cudaError_t e = launch_dependent(k_group_tables, dim3((nchunks + 255) / 256, kMaxLevels), dim3(256), 0, st,
					 outs, nchunks, lod_max, a);
	if (e != cudaSuccess) return e;
	if (L > 1) {
		e = launch_dependent(k_group_scan, dim3(L - 1), dim3(1024), 0, st, nchunks, a);
		if (e != cudaSuccess) return e;
		/* 8 warps per CTA, up to 8 CTAs per SM of a 152-SM GPU; level-1
		 * slices while the segments are fewer than eight per warp */
		const uint64_t nseg = (uint64_t)nchunks * (uint64_t)(L - 1);
		const uint32_t max_grid = 152u * 8u;
		const uint32_t l1_slices = nseg <= (uint64_t)max_grid * 8u * 8u ? kL1Slices : 1u;
		const uint64_t nwork = (uint64_t)nchunks * (l1_slices + (uint64_t)(L - 2));
		const uint32_t grid = (uint32_t)std::min<uint64_t>((nwork + 7) / 8, max_grid);
		e = launch_dependent(k_group_copy, dim3(grid), dim3(256), 0, st, outs, nchunks, L - 1, l1_slices, a);
		if (e != cudaSuccess) return e;
	}
	return cudaGetLastError();
}

} // namespace vp
