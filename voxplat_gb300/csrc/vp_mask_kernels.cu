/*
 * vp_mask_kernels.cu — kernels for the per-call drop-ins that work on dense
 * (R+1)^3 mask arrays the caller owns:
 *
 *   k_downsample   chunk_mask_downsample (src/chunkset/mesher.c:460-493):
 *                  each coarse cell receives the last nonzero child in z,y,x
 *                  scan order, i.e. the child with the largest (z, y, x);
 *                  cells with no nonzero child keep their value.
 *   k_splatlist    chunk_make_splatlist (src/chunkset/mesher.c:497-536): one
 *                  CTA compacts the nonzero cells of [0, (R>>l)+1)^3 in scan
 *                  order (tile counts, block prefix sum, in-order stores) and
 *                  emits {x, y, z, colour | shadow << 6} per cell.
 */
#include "vp_dev.cuh"
#include "vp_mask_kernels.h"

namespace vp {

__global__ void k_downsample(const uint8_t *__restrict__ mask, uint8_t *work, uint32_t S, uint32_t range)
{
	const uint32_t half = (range + 1u) / 2u;
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= half * half * half) return;
	const uint32_t x = i % half, y = (i / half) % half, z = i / (half * half);
	for (int d = 7; d >= 0; d--) {
		const uint32_t X = 2 * x + (d & 1), Y = 2 * y + ((d >> 1) & 1), Z = 2 * z + (d >> 2);
		if (X >= range || Y >= range || Z >= range) continue;
		const uint8_t v = mask[((size_t)Z * S + Y) * S + X];
		if (v) {
			work[((size_t)z * S + y) * S + x] = v;
			return;
		}
	}
}

__global__ void __launch_bounds__(1024) k_splatlist(const uint8_t *__restrict__ mask, uint32_t S, uint32_t range,
						    uint32_t level, uint32_t wx0, uint32_t wy0, uint32_t wz0, SetDesc sd,
						    int16_t *out, uint32_t *count)
{
	__shared__ uint32_t tmp[64];
	const uint32_t n = range * range * range;
	uint32_t base = 0;
	for (uint32_t t0 = 0; t0 < n; t0 += blockDim.x) {
		const uint32_t i = t0 + threadIdx.x;
		uint32_t x = 0, y = 0, z = 0;
		uint8_t m = 0;
		if (i < n) {
			x = i % range;
			y = (i / range) % range;
			z = i / (range * range);
			m = mask[((size_t)z * S + y) * S + x];
		}
		uint32_t tot;
		const uint32_t k = base + block_excl_add(m ? 1u : 0u, tmp, &tot);
		if (m) {
			const uint32_t wx = wx0 + (x << level), wy = wy0 + (y << level), wz = wz0 + (z << level);
			const uint32_t sh = level ? (1u << level) : 0u;
			const uint32_t shadow = (uint32_t)shadow_sample(sd, wx + sh, wy + sh, wz + sh);
			const uint32_t w = (uint32_t)m | (shadow << 6);
			uint2 v;
			v.x = (wx & 0xFFFFu) | ((wy & 0xFFFFu) << 16);
			v.y = (wz & 0xFFFFu) | ((w & 0xFFFFu) << 16);
			*(uint2 *)(out + (size_t)k * 4) = v;
		}
		base += tot;
	}
	if (threadIdx.x == 0) *count = base;
}

cudaError_t launch_downsample(const uint8_t *mask, uint8_t *work, uint32_t S, uint32_t range, cudaStream_t st)
{
	const uint32_t half = (range + 1u) / 2u;
	const uint32_t n = half * half * half;
	k_downsample<<<(n + 255) / 256, 256, 0, st>>>(mask, work, S, range);
	return cudaGetLastError();
}

cudaError_t launch_splatlist(const uint8_t *mask, uint32_t S, uint32_t range, uint32_t level, const uint32_t wbase[3],
			     const SetDesc &sd, int16_t *out, uint32_t *count, cudaStream_t st)
{
	k_splatlist<<<1, 1024, 0, st>>>(mask, S, range, level, wbase[0], wbase[1], wbase[2], sd, out, count);
	return cudaGetLastError();
}

} // namespace vp
