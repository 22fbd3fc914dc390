/*
 * vp_cull.cu — draw culling and LOD selection on the device: the octree walk
 * of octree_cull (src/game.c:319-395, started from LOD `top` at
 * src/game.c:517-524), the frustum test of src/gfx/fcull.c, and the
 * mesh-or-splat choice of src/game.c:612-625.
 *
 * The recursive walk becomes one thread per octree node of every level:
 * a node is drawn when every ancestor is inside the frustum and nearer than
 * its level's LOD distance (so the walk descended), and the node itself is
 * inside the frustum and farther than its own (or is a chunk). Drawn nodes
 * scatter into a slot array indexed by their depth-first position (root
 * index in x, y, z loop order, then one octal digit per level, child order
 * x, y, z), so compacting the slots yields the walk's queue order.
 *
 * Float arithmetic uses explicitly rounded operations (no contraction into
 * fused multiply-adds), in the reference's order of evaluation, so every
 * comparison comes out as on the host.
 */
#include "vp_cull.h"

namespace vp {

/* gfx_fcull_extract_planes (src/gfx/fcull.c:20-35) on one thread */
__device__ void extract_planes(const float *m, float *planes)
{
	int n = 0;
	for (int i = 0; i < 3; i++) {
		for (int j = 0; j < 4; j++) planes[n++] = __fsub_rn(m[3 + 4 * j], m[4 * j + i]);
		for (int j = 0; j < 4; j++) planes[n++] = __fadd_rn(m[3 + 4 * j], m[4 * j + i]);
	}
	for (int p = 0; p < 6; p++) {
		float *q = planes + 4 * p;
		const float s = __fadd_rn(__fadd_rn(__fmul_rn(q[0], q[0]), __fmul_rn(q[1], q[1])), __fmul_rn(q[2], q[2]));
		const float len = __double2float_rn(__dsqrt_rn((double)s));
		for (int k = 0; k < 4; k++) q[k] = __fdiv_rn(q[k], len);
	}
}

/* gfx_fcull_visible (src/gfx/fcull.c:38-45) */
__device__ __forceinline__ bool visible(const float *planes, const float c[3], float radius)
{
	for (int p = 0; p < 6; p++) {
		const float *q = planes + 4 * p;
		const float d = __fadd_rn(
			__fadd_rn(__fadd_rn(__fmul_rn(q[0], c[0]), __fmul_rn(q[1], c[1])), __fmul_rn(q[2], c[2])), q[3]);
		if (d < -radius) return false;
	}
	return true;
}

/* Euclidean distance in float (glm_vec_distance) */
__device__ __forceinline__ float distance3(const float a[3], const float b[3])
{
	const float d0 = __fsub_rn(b[0], a[0]), d1 = __fsub_rn(b[1], a[1]), d2 = __fsub_rn(b[2], a[2]);
	return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1)), __fmul_rn(d2, d2)));
}

/* Octree node (x, y, z) of level l: centre, visibility and distance. */
struct NodeTest {
	bool visible;
	float distance;
};

__device__ __forceinline__ NodeTest node_test(const CullArgs &a, const float *planes, uint32_t l, uint32_t x,
					      uint32_t y, uint32_t z)
{
	const uint32_t ws_root = (1u << a.root_bitw) << l;
	const float c[3] = {__uint2float_rn(x * ws_root + ws_root / 2), __uint2float_rn(y * ws_root + ws_root / 2),
			    __uint2float_rn(z * ws_root + ws_root / 2)};
	const float radius = __double2float_rn(__dmul_rn((double)ws_root, 0.85));
	NodeTest t;
	t.visible = visible(planes, c, radius);
	t.distance = distance3(a.origin, c);
	return t;
}

__global__ void __launch_bounds__(256) k_cull_nodes(CullArgs a)
{
	__shared__ float planes[24];
	if (threadIdx.x == 0) extract_planes(a.view_proj, planes);
	__syncthreads();
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	/* level of node i: levels top..0 are laid out one after another */
	uint32_t l = 0;
	uint64_t base = 0;
	for (;; l++) {
		if (l > a.top) return;
		const uint64_t n = (uint64_t)a.nodes[l][0] * a.nodes[l][1] * a.nodes[l][2];
		if (i < base + n) break;
		base += n;
	}
	const uint64_t j = i - base;
	const uint32_t x = (uint32_t)(j % a.nodes[l][0]);
	const uint32_t y = (uint32_t)((j / a.nodes[l][0]) % a.nodes[l][1]);
	const uint32_t z = (uint32_t)(j / ((uint64_t)a.nodes[l][0] * a.nodes[l][1]));
	/* the walk reaches this node only through ancestors it descended from */
	for (uint32_t k = a.top; k > l; k--) {
		const uint32_t s = k - l;
		const NodeTest t = node_test(a, planes, k, x >> s, y >> s, z >> s);
		if (!t.visible || t.distance > __uint2float_rn(k * 1024u)) return;
	}
	const NodeTest t = node_test(a, planes, l, x, y, z);
	if (!t.visible) return;
	if (l != 0 && !(t.distance > __uint2float_rn(l * 1024u))) return; /* the walk descends */
	uint32_t code = 0;
	if (l == 0) {
		const uint32_t c = ((z << a.max_bitw[1] | y) << a.max_bitw[0]) | x;
		if (a.outs[c].vbo_items) code = 0x80000000u | c;
	}
	if (!code) {
		uint32_t ob[3];
		for (int d = 0; d < 3; d++) ob[d] = a.max_bitw[d] - min(l, a.max_bitw[d]);
		const uint32_t node = ((z << ob[1] | y) << ob[0]) | x;
		if (!a.node_items[(size_t)l * a.nchunks + node]) return;
		code = ((l << 24) | node) + 1u;
	}
	/* depth-first position: root index, then one octal digit per level */
	const uint32_t s = a.top - l;
	const uint32_t rx = x >> s, ry = y >> s, rz = z >> s;
	uint64_t key = ((uint64_t)rx * a.roots[1] + ry) * a.roots[2] + rz;
	for (uint32_t k = a.top; k > 0; k--) {
		uint32_t d = 0;
		if (k > l) {
			const uint32_t sh = k - 1 - l;
			d = (((x >> sh) & 1u) << 2) | (((y >> sh) & 1u) << 1) | ((z >> sh) & 1u);
		}
		key = key * 8u + d;
	}
	a.slots[key] = code;
}

constexpr int kCompactBlock = 1024;

__device__ __forceinline__ bool is_mesh_code(uint32_t v) { return (v & 0x80000000u) != 0; }

/* per block of slots: number of mesh and splat entries */
__global__ void __launch_bounds__(kCompactBlock) k_cull_count(const uint32_t *__restrict__ slots, uint64_t n,
							      uint32_t *block_counts)
{
	__shared__ uint32_t s_m, s_s;
	if (threadIdx.x == 0) s_m = s_s = 0;
	__syncthreads();
	const uint64_t i = blockIdx.x * (uint64_t)kCompactBlock + threadIdx.x;
	const uint32_t v = i < n ? slots[i] : 0u;
	const uint32_t bm = __ballot_sync(kFull, v && is_mesh_code(v));
	const uint32_t bs = __ballot_sync(kFull, v && !is_mesh_code(v));
	if ((threadIdx.x & 31) == 0) {
		if (bm) atomicAdd(&s_m, (uint32_t)__popc(bm));
		if (bs) atomicAdd(&s_s, (uint32_t)__popc(bs));
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		block_counts[2 * blockIdx.x] = s_m;
		block_counts[2 * blockIdx.x + 1] = s_s;
	}
}

/* exclusive scan of the (mesh, splat) block counts in one CTA; totals[0..1] */
__global__ void __launch_bounds__(1024) k_cull_scan(uint32_t *block_counts, uint32_t nblocks, uint32_t *totals)
{
	__shared__ uint32_t carry[2], tile[2];
	__shared__ uint32_t wsum[2][32], wexcl[2][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	if (threadIdx.x < 2) carry[threadIdx.x] = 0;
	__syncthreads();
	for (uint32_t b0 = 0; b0 < nblocks; b0 += blockDim.x) {
		const uint32_t b = b0 + threadIdx.x;
		uint32_t x[2], inc[2];
		for (int k = 0; k < 2; k++) {
			x[k] = b < nblocks ? block_counts[2 * b + k] : 0u;
			inc[k] = warp_incl_add(x[k]);
			if (lane == 31) wsum[k][warp] = inc[k];
		}
		__syncthreads();
		if (warp == 0) {
			for (int k = 0; k < 2; k++) {
				const uint32_t w = lane < nw ? wsum[k][lane] : 0u;
				const uint32_t wi = warp_incl_add(w);
				wexcl[k][lane] = wi - w;
				if (lane == 31) tile[k] = wi;
			}
		}
		__syncthreads();
		if (b < nblocks)
			for (int k = 0; k < 2; k++) block_counts[2 * b + k] = carry[k] + wexcl[k][warp] + inc[k] - x[k];
		__syncthreads();
		if (threadIdx.x < 2) carry[threadIdx.x] += tile[threadIdx.x];
		__syncthreads();
	}
	if (threadIdx.x < 2) totals[threadIdx.x] = carry[threadIdx.x];
}

/* entries in slot order: mesh queue (chunk index), splat queue
 * (lod << 24 | node); writes past a capacity are dropped (the host sees the
 * totals) */
__global__ void __launch_bounds__(kCompactBlock) k_cull_write(const uint32_t *__restrict__ slots, uint64_t n,
							      const uint32_t *__restrict__ block_base, uint32_t *mesh_out,
							      uint32_t mesh_cap, uint32_t *svl_out, uint32_t svl_cap)
{
	__shared__ uint32_t wm[32], ws[32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t i = blockIdx.x * (uint64_t)kCompactBlock + threadIdx.x;
	const uint32_t v = i < n ? slots[i] : 0u;
	const bool m = v && is_mesh_code(v), sp = v && !is_mesh_code(v);
	const uint32_t bm = __ballot_sync(kFull, m), bs = __ballot_sync(kFull, sp);
	if (lane == 0) {
		wm[warp] = __popc(bm);
		ws[warp] = __popc(bs);
	}
	__syncthreads();
	if (warp == 0) {
		const uint32_t a = wm[lane], b = ws[lane];
		const uint32_t ai = warp_incl_add(a), bi = warp_incl_add(b);
		wm[lane] = ai - a;
		ws[lane] = bi - b;
	}
	__syncthreads();
	const uint32_t lt = (1u << lane) - 1u;
	if (m) {
		const uint32_t pos = block_base[2 * blockIdx.x] + wm[warp] + __popc(bm & lt);
		if (pos < mesh_cap) mesh_out[pos] = v & 0x7FFFFFFFu;
	}
	if (sp) {
		const uint32_t pos = block_base[2 * blockIdx.x + 1] + ws[warp] + __popc(bs & lt);
		if (pos < svl_cap) svl_out[pos] = v - 1u;
	}
}

/* make_mesh per chunk (src/game.c:612-625): centre within 512 of origin */
__global__ void k_mesh_flags(CullArgs a, uint8_t *flags)
{
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= a.nchunks) return;
	const uint32_t R = 1u << a.root_bitw;
	const uint32_t v[3] = {c & ((1u << a.max_bitw[0]) - 1u), (c >> a.max_bitw[0]) & ((1u << a.max_bitw[1]) - 1u),
			       c >> (a.max_bitw[0] + a.max_bitw[1])};
	float centre[3];
	for (int i = 0; i < 3; i++) centre[i] = __uint2float_rn((v[i] << a.root_bitw) + R / 2);
	flags[c] = distance3(centre, a.origin) < 512.0f ? 1 : 0;
}

uint64_t cull_slots(const CullArgs &a)
{
	return (uint64_t)a.roots[0] * a.roots[1] * a.roots[2] << (3 * a.top);
}

cudaError_t launch_cull(const CullArgs &a, uint32_t *block_counts, uint32_t *totals, uint32_t *mesh_out,
			uint32_t mesh_cap, uint32_t *svl_out, uint32_t svl_cap, cudaStream_t st)
{
	const uint64_t nslots = cull_slots(a);
	cudaError_t e = cudaMemsetAsync(a.slots, 0, nslots * sizeof(uint32_t), st);
	if (e != cudaSuccess) return e;
	uint64_t nodes = 0;
	for (uint32_t l = 0; l <= a.top; l++) nodes += (uint64_t)a.nodes[l][0] * a.nodes[l][1] * a.nodes[l][2];
	k_cull_nodes<<<(unsigned)((nodes + 255) / 256), 256, 0, st>>>(a);
	const uint32_t nb = (uint32_t)((nslots + kCompactBlock - 1) / kCompactBlock);
	k_cull_count<<<nb, kCompactBlock, 0, st>>>(a.slots, nslots, block_counts);
	k_cull_scan<<<1, 1024, 0, st>>>(block_counts, nb, totals);
	k_cull_write<<<nb, kCompactBlock, 0, st>>>(a.slots, nslots, block_counts, mesh_out, mesh_cap, svl_out, svl_cap);
	return cudaGetLastError();
}

cudaError_t launch_mesh_flags(const CullArgs &a, uint8_t *flags, cudaStream_t st)
{
	k_mesh_flags<<<(a.nchunks + 255) / 256, 256, 0, st>>>(a, flags);
	return cudaGetLastError();
}

} // namespace vp
