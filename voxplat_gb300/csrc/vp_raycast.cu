/*
 * vp_raycast.cu — picking rays on a device-resident RLE world
 * (chunkset_edit_raycast_until_solid, src/chunkset/edit.c:248-314, reading
 * voxels as chunkset_edit_read, src/chunkset/edit.c:10-36).
 *
 * One thread per ray runs the reference's float DDA with explicitly rounded
 * operations in its order of evaluation. A voxel is read from the chunk's
 * stream by binary search over a run-start index (voxel index at which each
 * run starts, built once per version of the pool); the ray keeps the last run
 * it found, so consecutive steps inside one run cost no search.
 *
 * `coord += step` goes through float as in the reference; below 0 it takes
 * x86-64's float->unsigned conversion (a 64-bit signed conversion truncated
 * to 32 bits): 0 - 1 gives 0xFFFFFFFF, and 0xFFFFFFFF - 1 rounds to 2^32,
 * which truncates to 0.
 */
#include "vp_raycast.h"

namespace vp {

/* runidx[off[c] + k] = voxel index where run k of chunk c starts */
__global__ void __launch_bounds__(256) k_run_starts(const uint32_t *__restrict__ pool, const uint64_t *__restrict__ off,
						    const uint32_t *__restrict__ len, uint32_t nchunks, uint32_t *runidx)
{
	__shared__ uint32_t tmp[40];
	const uint32_t c = blockIdx.x;
	if (c >= nchunks) return;
	const uint32_t *s = pool + off[c];
	uint32_t *o = runidx + off[c];
	const uint32_t n = len[c] - 1u; /* validated streams: len >= 2 */
	uint32_t carry = 0;
	for (uint32_t base = 0; base < n; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		const uint32_t v = i < n ? (s[i] & 0xFFFFFFu) : 0u;
		uint32_t tot;
		const uint32_t excl = block_excl_add(v, tmp, &tot);
		if (i < n) o[i] = carry + excl;
		carry += tot;
	}
}

struct RunCache {
	uint32_t chunk, lo, hi, colour;
};

__device__ __forceinline__ uint32_t read_voxel(const RayWorld &W, const uint32_t ws[3], RunCache &rc)
{
	for (int i = 0; i < 3; i++)
		if (ws[i] >= (1u << (W.max_bitw[i] + W.root_bitw))) return 0;
	const uint32_t rb = W.root_bitw, mask = (1u << rb) - 1u;
	const uint32_t c = (((ws[2] >> rb) << W.max_bitw[1] | (ws[1] >> rb)) << W.max_bitw[0]) | (ws[0] >> rb);
	const uint32_t p = (ws[0] & mask) | ((ws[1] & mask) << rb) | ((ws[2] & mask) << (2 * rb));
	if (c == rc.chunk && p >= rc.lo && p < rc.hi) return rc.colour;
	const uint64_t o = W.off[c];
	const uint32_t n = W.len[c] - 1u;
	const uint32_t *st = W.runidx + o;
	uint32_t lo = 0, hi = n; /* st[lo] <= p < st[hi] (st[n] = R^3) */
	while (hi - lo > 1u) {
		const uint32_t mid = (lo + hi) >> 1;
		if (__ldg(st + mid) <= p) lo = mid;
		else hi = mid;
	}
	rc.chunk = c;
	rc.lo = __ldg(st + lo);
	rc.hi = lo + 1u < n ? __ldg(st + lo + 1u) : (1u << (3 * rb));
	rc.colour = __ldg(W.pool + o + lo) >> 24;
	return rc.colour;
}

__global__ void __launch_bounds__(128) k_raycast(RayWorld W, const float *__restrict__ origins,
						 const float *__restrict__ vectors, uint32_t n, uint8_t *voxels,
						 uint32_t *coords, int8_t *normals)
{
	const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= n) return;
	float org[3], vec[3], delta[3], next[3], step[3];
	uint32_t coord[3];
	for (int i = 0; i < 3; i++) {
		org[i] = origins[3 * r + i];
		vec[i] = vectors[3 * r + i];
		coord[i] = (uint32_t)__float2int_rz(org[i]);
	}
	for (int i = 0; i < 3; i++) {
		const float t0 = __fdiv_rn(vec[0], vec[i]), t1 = __fdiv_rn(vec[1], vec[i]), t2 = __fdiv_rn(vec[2], vec[i]);
		const float s = __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(t1, t1)), __fmul_rn(t2, t2));
		delta[i] = __double2float_rn(__dsqrt_rn((double)s));
		if (vec[i] < 0.0f) {
			step[i] = -1.0f;
			next[i] = __fmul_rn(__fsub_rn(org[i], __uint2float_rn(coord[i])), delta[i]);
		} else {
			step[i] = 1.0f;
			next[i] = __fmul_rn(__fsub_rn(__fadd_rn(__uint2float_rn(coord[i]), 1.0f), org[i]), delta[i]);
		}
	}
	RunCache rc = {0xFFFFFFFFu, 0, 0, 0};
	uint8_t hit = 0;
	int8_t nrm[3] = {0, 0, 0};
	for (int loops = 4096; loops-- > 1;) {
		int side = 0;
		for (int j = 1; j < 3; j++)
			if (next[side] > next[j]) side = j;
		next[side] = __fadd_rn(next[side], delta[side]);
		coord[side] = (uint32_t)__float2ll_rz(__fadd_rn(__uint2float_rn(coord[side]), step[side]));
		const uint32_t v = read_voxel(W, coord, rc);
		if (v) {
			nrm[side] = (-vec[side] > 0.0f) ? 1 : -1;
			hit = (uint8_t)v;
			break;
		}
	}
	voxels[r] = hit;
	for (int i = 0; i < 3; i++) {
		coords[3 * r + i] = coord[i];
		normals[3 * r + i] = nrm[i];
	}
}

cudaError_t launch_run_starts(const uint32_t *pool, const uint64_t *off, const uint32_t *len, uint32_t nchunks,
			      uint32_t *runidx, cudaStream_t st)
{
	if (!nchunks) return cudaSuccess;
	k_run_starts<<<nchunks, 256, 0, st>>>(pool, off, len, nchunks, runidx);
	return cudaGetLastError();
}

cudaError_t launch_raycast(const RayWorld &W, const float *origins, const float *vectors, uint32_t n, uint8_t *voxels,
			   uint32_t *coords, int8_t *normals, cudaStream_t st)
{
	if (!n) return cudaSuccess;
	k_raycast<<<(n + 127) / 128, 128, 0, st>>>(W, origins, vectors, n, voxels, coords, normals);
	return cudaGetLastError();
}

} // namespace vp
