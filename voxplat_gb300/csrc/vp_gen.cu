/*
 * vp_gen.cu — the seeded synthetic worlds generated on the device, bit-
 * identical to the host generator (vp_worldgen.c): same integer hashing
 * (vp_noise.h), same interpolation order, same canonical shadow-map order.
 *
 * The world is produced one z-slab of chunks (all chunks with the same cz)
 * at a time:
 *   k_gen_chunk    one CTA per chunk fills its R^3 voxel volume: column
 *                  heights and colours per (x, z), cave noise from the
 *                  chunk's lattice values staged in shared memory;
 *   k_gen_shadow   one CTA per map row z of the slab: the row is staged in
 *                  shared memory and shadow_place_update (src/chunkset/
 *                  shadow.h:77-89) runs for every solid voxel of the row in
 *                  the canonical order (chunk index ascending, then x, then
 *                  y ascending), a column of 32 voxels at a time;
 *   the RLE encoder then appends the slab's streams to the world's pool.
 */
#include "vp_dev.cuh"
#include "vp_gen.h"
#include "vp_noise.h"

namespace vp {

constexpr int32_t kCaveThreshold = 36045; /* 0.55 in 16-bit fixed point */

struct Lat {
	int s, x0, y0, z0, n;
	const uint16_t *v;
};

__device__ __forceinline__ int32_t lat_eval(const Lat &L, int x, int y, int z)
{
	const int s = L.s, m = (1 << s) - 1;
	const int i = (x >> s) - L.x0, j = (y >> s) - L.y0, k = (z >> s) - L.z0;
	const int64_t wx = vp_smooth16((int64_t)(x & m) << (16 - s));
	const int64_t wy = vp_smooth16((int64_t)(y & m) << (16 - s));
	const int64_t wz = vp_smooth16((int64_t)(z & m) << (16 - s));
	int64_t c[2][2];
	for (int dz = 0; dz < 2; dz++)
		for (int dy = 0; dy < 2; dy++) {
			const uint16_t *row = L.v + ((k + dz) * L.n + (j + dy)) * L.n + i;
			c[dz][dy] = vp_lerp16(row[0], row[1], wx);
		}
	const int64_t e0 = vp_lerp16(c[0][0], c[0][1], wy);
	const int64_t e1 = vp_lerp16(c[1][0], c[1][1], wy);
	return (int32_t)vp_lerp16(e0, e1, wz);
}

template <int RB>
__global__ void __launch_bounds__(256) k_gen_chunk(GenArgs a, uint32_t cz, uint8_t *vols)
{
	constexpr int R = 1 << RB;
	const uint32_t cx = blockIdx.x & ((1u << a.max_bitw[0]) - 1u);
	const uint32_t cy = blockIdx.x >> a.max_bitw[0];
	const int ox = (int)cx << RB, oy = (int)cy << RB, oz = (int)cz << RB;
	uint8_t *vol = vols + ((size_t)blockIdx.x << (3 * RB));
	__shared__ int16_t hcol[R * R];
	__shared__ int16_t offc[R * R];
	__shared__ uint8_t colc[R * R];
	__shared__ uint16_t lat5[((R - 1) / 32 + 3) * ((R - 1) / 32 + 3) * ((R - 1) / 32 + 3)];
	__shared__ uint16_t lat4[((R - 1) / 16 + 3) * ((R - 1) / 16 + 3) * ((R - 1) / 16 + 3)];
	__shared__ int s_maxh;
	if (threadIdx.x == 0) s_maxh = 0;
	__syncthreads();
	for (int i = threadIdx.x; i < R * R; i += blockDim.x) {
		const int x = i & (R - 1), z = i >> RB;
		const int X = ox + x, Z = oz + z;
		int h;
		if (a.kind == kGenTerrainSmall)
			h = 8 + (int)(((int64_t)vp_fractal2(a.seed, X, Z, 5 + a.hshift, 4) * 49) >> 16);
		else
			h = 40 + (int)(((int64_t)vp_fractal2(a.seed, X, Z, 8 + a.hshift, 6) * 161) >> 16);
		hcol[i] = (int16_t)h;
		if (a.kind == kGenTerrainSmall) {
			colc[i] = (uint8_t)(1 + h / 4 + (vp_hash3(a.seed ^ 0xC01u, X, 0, Z) & 3));
		} else {
			offc[i] = (int16_t)(vp_value2(a.seed + 13, X, Z, 6) >> 12);
		}
		atomicMax(&s_maxh, h);
	}
	const bool caves = a.kind == kGenTerrainCaves;
	const int n5 = ((R - 1) >> 5) + 3, n4 = ((R - 1) >> 4) + 3;
	if (caves) {
		for (int i = threadIdx.x; i < n5 * n5 * n5; i += blockDim.x) {
			const int di = i % n5, dj = (i / n5) % n5, dk = i / (n5 * n5);
			lat5[i] = (uint16_t)(vp_hash3(a.seed + 11, (ox >> 5) + di, (oy >> 5) + dj, (oz >> 5) + dk) & 0xFFFF);
		}
		for (int i = threadIdx.x; i < n4 * n4 * n4; i += blockDim.x) {
			const int di = i % n4, dj = (i / n4) % n4, dk = i / (n4 * n4);
			lat4[i] = (uint16_t)(vp_hash3(a.seed + 12, (ox >> 4) + di, (oy >> 4) + dj, (oz >> 4) + dk) & 0xFFFF);
		}
	}
	__syncthreads();
	const bool empty = s_maxh <= oy;
	const Lat L5 = {5, ox >> 5, oy >> 5, oz >> 5, n5, lat5};
	const Lat L4 = {4, ox >> 4, oy >> 4, oz >> 4, n4, lat4};
	/* voxel (x, y, z) at x + R*(y + R*z); a thread writes 4 consecutive x */
	for (int q = threadIdx.x; q < R * R * R / 4; q += blockDim.x) {
		const int p = q * 4;
		const int x0 = p & (R - 1), y = (p >> RB) & (R - 1), z = p >> (2 * RB);
		uint32_t word = 0;
		if (!empty) {
			for (int k = 0; k < 4; k++) {
				const int x = x0 + k;
				const int ci = z * R + x;
				const int h = hcol[ci];
				const int Y = oy + y;
				uint32_t c = 0;
				if (Y < h) {
					if (!caves) {
						c = colc[ci];
					} else {
						const int X = ox + x, Z = oz + z;
						const int32_t d = (2 * lat_eval(L5, X, Y, Z) + lat_eval(L4, X, Y, Z)) / 3;
						if (d <= kCaveThreshold) {
							if (Y == h - 1)
								c = h < 120 ? 42u : 63u;
							else
								c = 1u + (uint32_t)((((Y + offc[ci]) >> 4) * 23 + 7) % 62);
						}
					}
				}
				word |= c << (8 * k);
			}
		}
		*(uint32_t *)(vol + p) = word;
	}
}

/* Shadow rows of one slab. Candidates in canonical order: chunk index
 * ascending (cy outer, cx inner for a fixed cz), x ascending, y ascending.
 * Each chunk's plane z is staged in shared memory (coalesced), then warp 0
 * walks it column by column and applies each column's updates to the
 * staged map row at once. */
__global__ void __launch_bounds__(256) k_gen_shadow(GenArgs a, uint32_t cz, const uint8_t *__restrict__ vols,
						    uint16_t *shadow, uint64_t shadow_len)
{
	extern __shared__ uint16_t row[];
	const int RB = a.root_bitw, R = 1 << RB;
	uint8_t *plane = (uint8_t *)(row + ((a.shadow_w + 7u) & ~7u));
	const uint32_t zl = blockIdx.x, z = (cz << RB) + zl;
	const uint32_t W = a.shadow_w;
	const uint64_t base = (uint64_t)W * z;
	for (uint32_t i = threadIdx.x; i < W; i += blockDim.x) row[i] = (base + i < shadow_len) ? shadow[base + i] : 0;
	const int lane = threadIdx.x & 31;
	const uint32_t ny = 1u << a.max_bitw[1], nx = 1u << a.max_bitw[0];
	for (uint32_t cy = 0; cy < ny; cy++)
		for (uint32_t cx = 0; cx < nx; cx++) {
			const uint8_t *vol = vols + ((size_t)((cy << a.max_bitw[0]) | cx) << (3 * RB)) + ((size_t)zl << (2 * RB));
			__syncthreads();
			for (int i = threadIdx.x * 4; i < R * R; i += blockDim.x * 4)
				*(uint32_t *)(plane + i) = *(const uint32_t *)(vol + i);
			__syncthreads();
			if (threadIdx.x >= 32) continue;
			/* one column (x) at a time: its updates read entries x+y and
			 * x+y+1, which no earlier update of the column wrote, so the
			 * lanes apply the whole column at once */
			for (int x = 0; x < R; x++)
				for (int yb = 0; yb < R; yb += 32) {
					const int y = yb + lane;
					bool upd = false;
					uint32_t j = 0, Y = 0;
					if (y < R && plane[x + R * y] != 0) {
						const uint32_t X = (cx << RB) + x;
						Y = (cy << RB) + y;
						j = X + Y; /* index within the row */
						const uint32_t lim = Y + 1;
						const uint32_t v1 = j + 1 < W ? row[j + 1] : 0u;
						upd = row[j] < lim && v1 < lim;
					}
					__syncwarp();
					if (upd) row[j] = (uint16_t)Y;
					__syncwarp();
				}
		}
	__syncthreads();
	for (uint32_t i = threadIdx.x; i < W; i += blockDim.x)
		if (base + i < shadow_len) shadow[base + i] = row[i];
}

/* off/len of the slab's chunks [first, first + n) = the encoded streams */
__global__ void k_scatter_slab(const uint64_t *__restrict__ new_off, const uint32_t *__restrict__ new_len, uint32_t n,
			       uint32_t first, uint64_t base, uint64_t *off, uint32_t *len)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	off[first + k] = base + new_off[k];
	len[first + k] = new_len[k];
}

cudaError_t launch_scatter_slab(const uint64_t *new_off, const uint32_t *new_len, uint32_t n, uint32_t first,
				uint64_t base, uint64_t *off, uint32_t *len, cudaStream_t st)
{
	k_scatter_slab<<<(n + 255) / 256, 256, 0, st>>>(new_off, new_len, n, first, base, off, len);
	return cudaGetLastError();
}

cudaError_t launch_gen_slab(const GenArgs &a, uint32_t cz, uint8_t *vols, cudaStream_t st)
{
	const uint32_t n = 1u << (a.max_bitw[0] + a.max_bitw[1]);
	switch (a.root_bitw) {
	case 3: k_gen_chunk<3><<<n, 256, 0, st>>>(a, cz, vols); break;
	case 4: k_gen_chunk<4><<<n, 256, 0, st>>>(a, cz, vols); break;
	case 5: k_gen_chunk<5><<<n, 256, 0, st>>>(a, cz, vols); break;
	case 6: k_gen_chunk<6><<<n, 256, 0, st>>>(a, cz, vols); break;
	default: return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

cudaError_t launch_gen_shadow(const GenArgs &a, uint32_t cz, const uint8_t *vols, uint16_t *shadow,
			      uint64_t shadow_len, cudaStream_t st)
{
	const size_t smem = (((size_t)a.shadow_w + 7u) & ~(size_t)7u) * sizeof(uint16_t) + ((size_t)1 << (2 * a.root_bitw));
	cudaError_t e = cudaFuncSetAttribute(k_gen_shadow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	k_gen_shadow<<<1u << a.root_bitw, 256, smem, st>>>(a, cz, vols, shadow, shadow_len);
	return cudaGetLastError();
}

} // namespace vp
