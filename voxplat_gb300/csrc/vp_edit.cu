/*
 * vp_edit.cu — sphere edits on a device-resident world
 * (chunkset_edit_sphere, src/chunkset/edit.c:179-244, with chunk_ws_write
 * :143-176 and shadow_place_update, src/chunkset/shadow.h:77-89).
 *
 * One launch per edit, in arrival order:
 *   - blocks [0, nchunks): one per chunk of the edit's AABB list; every
 *     voxel u of the AABB inside that chunk with |u - c|^2 < r^2 and
 *     u.y >= 2 gets the edit's voxel (voxel writes do not depend on order);
 *   - blocks [nchunks, nchunks + rows): fill edits only, one per world z
 *     row of the AABB. shadow_place_update reads and writes map entries
 *     (x + y) + W*z and its +1 neighbour, always inside row z, so rows are
 *     independent; inside a row the updates are order dependent: they run
 *     in the reference's order (chunks x-outer then y, then u.x, then u.y)
 *     on a shared-memory copy of the row segment, one column (all u.y of one
 *     u.x) at a time, which is exact because no update of a column reads an
 *     entry an earlier update of the same column wrote.
 * The reference's test sqrtf(d0^2 + d1^2 + d2^2) < (float)r equals
 * d0^2 + d1^2 + d2^2 < r^2 for integer d and r < 4096: the squares are exact
 * in float and sqrtf is correctly rounded.
 */
#include "vp_dev.cuh"
#include "vp_edit.h"

namespace vp {

__device__ __forceinline__ bool in_sphere(int32_t ux, int32_t uy, int32_t uz, const EditDesc &e)
{
	const int64_t dx = ux - e.c[0], dy = uy - e.c[1], dz = uz - e.c[2];
	return dx * dx + dy * dy + dz * dz < (int64_t)e.r * e.r;
}

__global__ void __launch_bounds__(256) k_edit(EditDesc e, const EditChunk *__restrict__ chunks, uint32_t nchunks,
					      uint8_t *vols, uint32_t root_bitw, uint16_t *shadow, uint64_t shadow_len,
					      uint32_t shadow_w)
{
	const int32_t R = 1 << root_bitw;
	const int32_t mn[3] = {e.c[0] - (int32_t)e.r - 1, e.c[1] - (int32_t)e.r - 1, e.c[2] - (int32_t)e.r - 1};
	const int32_t mx[3] = {e.c[0] + (int32_t)e.r + 1, e.c[1] + (int32_t)e.r + 1, e.c[2] + (int32_t)e.r + 1};
	if (blockIdx.x < nchunks) {
		const EditChunk ch = chunks[blockIdx.x];
		int32_t lo[3], hi[3];
		for (int i = 0; i < 3; i++) {
			const int32_t o = ch.cv[i] * R;
			lo[i] = max(mn[i], o);
			hi[i] = min(mx[i], o + R);
		}
		if (lo[0] >= hi[0] || lo[1] >= hi[1] || lo[2] >= hi[2]) return;
		const uint32_t ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
		const uint32_t n = ex * ey * ez;
		uint8_t *vol = vols + ((size_t)ch.vol_slot << (3 * root_bitw));
		for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
			const int32_t ux = lo[0] + (int32_t)(i % ex);
			const int32_t uy = lo[1] + (int32_t)((i / ex) % ey);
			const int32_t uz = lo[2] + (int32_t)(i / (ex * ey));
			if (uy < 2 || !in_sphere(ux, uy, uz, e)) continue;
			const uint32_t lx = ux - ch.cv[0] * R, ly = uy - ch.cv[1] * R, lz = uz - ch.cv[2] * R;
			vol[lx | (ly << root_bitw) | (lz << (2 * root_bitw))] = e.voxel;
		}
		return;
	}
	/* shadow rows: fill edits only (the carve path calls a stub) */
	if (!e.voxel) return;
	const int32_t z = mn[2] + (int32_t)(blockIdx.x - nchunks);
	if (z >= mx[2]) return;
	__shared__ uint16_t seg[1024];
	__shared__ uint32_t s_base;
	/* indices touched in row z: (x + y) for x in [mn0, mx0), y in [mn1, mx1),
	 * plus one */
	const int64_t row = (int64_t)shadow_w * (uint32_t)z;
	const int64_t first = row + (int64_t)(uint32_t)mn[0] + (uint32_t)mn[1];
	const uint32_t span = (uint32_t)((mx[0] - mn[0]) + (mx[1] - mn[1]) + 1);
	if (span > 1024) return; /* radii are limited so that this never happens */
	for (uint32_t i = threadIdx.x; i < span; i += blockDim.x) {
		const uint64_t idx = (uint64_t)(uint32_t)(first + i);
		seg[i] = idx < shadow_len ? shadow[idx] : 0;
	}
	if (threadIdx.x == 0) s_base = (uint32_t)first;
	__syncthreads();
	/* Updates along one column (fixed chunk and x, y ascending) read
	 * entries x+y and x+y+1 and write x+y: no step reads an entry an earlier
	 * step of the same column wrote, so a column is applied at once (warp 0,
	 * lane per y); columns follow the reference's order. */
	if (threadIdx.x < 32) {
		const uint32_t base = s_base;
		const int lane = threadIdx.x;
		for (uint32_t k = 0; k < e.nlist; k++) {
			const EditChunk ch = chunks[k];
			if (ch.cv[2] * R > z || z >= ch.cv[2] * R + R) continue;
			const int32_t x0 = max(mn[0], ch.cv[0] * R), x1 = min(mx[0], ch.cv[0] * R + R);
			const int32_t y0 = max(mn[1], ch.cv[1] * R), y1 = min(mx[1], ch.cv[1] * R + R);
			for (int32_t x = x0; x < x1; x++)
				for (int32_t yb = y0; yb < y1; yb += 32) {
					const int32_t y = yb + lane;
					bool upd = false;
					uint32_t j = 0;
					if (y < y1 && in_sphere(x, y, z, e)) {
						/* shadow_sample: shadowed unless both entries < y + 1 */
						j = (((uint32_t)x + (uint32_t)y) + shadow_w * (uint32_t)z) - base;
						const uint32_t lim = (uint32_t)y + 1u;
						upd = seg[j] < lim && seg[j + 1] < lim;
					}
					__syncwarp();
					if (upd) seg[j] = (uint16_t)y;
					__syncwarp();
				}
		}
	}
	__syncthreads();
	for (uint32_t i = threadIdx.x; i < span; i += blockDim.x) {
		const uint64_t idx = (uint64_t)(uint32_t)(first + i);
		if (idx < shadow_len) shadow[idx] = seg[i];
	}
}

/* off[chunk_k] / len[chunk_k] = the freshly encoded streams */
__global__ void k_scatter_streams(const uint32_t *__restrict__ chunk_ids, uint32_t n, const uint64_t *__restrict__ new_off,
				  const uint32_t *__restrict__ new_len, uint64_t base, uint64_t *off, uint32_t *len)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	off[chunk_ids[k]] = base + new_off[k];
	len[chunk_ids[k]] = new_len[k];
}

cudaError_t launch_edit(const EditDesc &e, const EditChunk *chunks, uint32_t nchunks, uint8_t *vols,
			uint32_t root_bitw, uint16_t *shadow, uint64_t shadow_len, uint32_t shadow_w, cudaStream_t st)
{
	const uint32_t rows = e.voxel ? 2u * e.r + 2u : 0u;
	if (nchunks + rows == 0) return cudaSuccess;
	k_edit<<<nchunks + rows, 256, 0, st>>>(e, chunks, nchunks, vols, root_bitw, shadow, shadow_len, shadow_w);
	return cudaGetLastError();
}

cudaError_t launch_scatter_streams(const uint32_t *chunk_ids, uint32_t n, const uint64_t *new_off,
				   const uint32_t *new_len, uint64_t base, uint64_t *off, uint32_t *len, cudaStream_t st)
{
	if (!n) return cudaSuccess;
	k_scatter_streams<<<(n + 255) / 256, 256, 0, st>>>(chunk_ids, n, new_off, new_len, base, off, len);
	return cudaGetLastError();
}

} // namespace vp
