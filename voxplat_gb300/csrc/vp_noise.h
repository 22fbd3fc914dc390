/*
 * vp_noise.h — integer-only hashing and value noise for the seeded synthetic
 * worlds (host C and CUDA device code share this header, so a world generated
 * on the CPU and one generated on the GPU are bit-identical).
 *
 * The reference generates terrain with FastNoise simplex noise
 * (src/cpp/noise.cpp:6-27, called from src/chunkset/gen.c:89-142); that
 * library is not vendored and its floating point output is not reproducible
 * across compilers, so the synthetic worlds here are defined with splitmix64
 * lattice hashing and fixed-point smoothstep interpolation instead.
 */
#ifndef VP_NOISE_H
#define VP_NOISE_H

#include <stdint.h>

#if defined(__CUDACC__)
#define VP_HD static __host__ __device__ __forceinline__
#else
#define VP_HD static inline
#endif

/* splitmix64 finaliser (Steele, Lea, Flood 2014). */
VP_HD uint64_t vp_mix64(uint64_t z)
{
	z += 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

/* 32-bit hash of a seed and an integer lattice point. */
VP_HD uint32_t vp_hash3(uint64_t seed, int32_t x, int32_t y, int32_t z)
{
	uint64_t k = seed * 0xD1B54A32D192ED03ull;
	k ^= (uint64_t)(uint32_t)x * 0x9E3779B97F4A7C15ull;
	k = vp_mix64(k);
	k ^= (uint64_t)(uint32_t)y * 0xC2B2AE3D27D4EB4Full;
	k = vp_mix64(k);
	k ^= (uint64_t)(uint32_t)z * 0x165667B19E3779F9ull;
	return (uint32_t)(vp_mix64(k) >> 32);
}

/* Fixed-point smoothstep: t in [0, 65535] -> w in [0, 65535]. */
VP_HD int64_t vp_smooth16(int64_t t)
{
	return (t * t * (196608 - 2 * t)) >> 32;
}

VP_HD int64_t vp_lerp16(int64_t a, int64_t b, int64_t w)
{
	return a + (((b - a) * w) >> 16);
}

/* 2-D value noise with a power-of-two cell size 2^sb; result in [0, 65535]. */
VP_HD int32_t vp_value2(uint64_t seed, int32_t x, int32_t z, int sb)
{
	int32_t ix = x >> sb, iz = z >> sb;
	int64_t tx = (int64_t)(x & ((1 << sb) - 1)) << (16 - sb);
	int64_t tz = (int64_t)(z & ((1 << sb) - 1)) << (16 - sb);
	int64_t wx = vp_smooth16(tx), wz = vp_smooth16(tz);
	int64_t v00 = vp_hash3(seed, ix, 0, iz) & 0xFFFF;
	int64_t v10 = vp_hash3(seed, ix + 1, 0, iz) & 0xFFFF;
	int64_t v01 = vp_hash3(seed, ix, 0, iz + 1) & 0xFFFF;
	int64_t v11 = vp_hash3(seed, ix + 1, 0, iz + 1) & 0xFFFF;
	int64_t a = vp_lerp16(v00, v10, wx);
	int64_t b = vp_lerp16(v01, v11, wx);
	return (int32_t)vp_lerp16(a, b, wz);
}

/* Fractal sum of `oct` octaves of 2-D value noise, cell sizes 2^sb, 2^(sb-1),
 * ... with amplitudes halving; normalised back to [0, 65535]. */
VP_HD int32_t vp_fractal2(uint64_t seed, int32_t x, int32_t z, int sb, int oct)
{
	int64_t acc = 0, norm = 0;
	int64_t amp = 1 << 10;
	for (int o = 0; o < oct; o++) {
		int s = sb - o;
		if (s < 1) s = 1;
		acc += amp * vp_value2(seed + 0x1000u * (uint64_t)o, x, z, s);
		norm += amp;
		amp >>= 1;
	}
	return (int32_t)(acc / norm);
}

/* 3-D value noise with cell size 2^sb; result in [0, 65535]. */
VP_HD int32_t vp_value3(uint64_t seed, int32_t x, int32_t y, int32_t z, int sb)
{
	int32_t ix = x >> sb, iy = y >> sb, iz = z >> sb;
	int64_t m = (1 << sb) - 1;
	int64_t wx = vp_smooth16((int64_t)(x & m) << (16 - sb));
	int64_t wy = vp_smooth16((int64_t)(y & m) << (16 - sb));
	int64_t wz = vp_smooth16((int64_t)(z & m) << (16 - sb));
	int64_t c[2][2];
	for (int dz = 0; dz < 2; dz++)
		for (int dy = 0; dy < 2; dy++) {
			int64_t a = vp_hash3(seed, ix, iy + dy, iz + dz) & 0xFFFF;
			int64_t b = vp_hash3(seed, ix + 1, iy + dy, iz + dz) & 0xFFFF;
			c[dz][dy] = vp_lerp16(a, b, wx);
		}
	int64_t e0 = vp_lerp16(c[0][0], c[0][1], wy);
	int64_t e1 = vp_lerp16(c[1][0], c[1][1], wy);
	return (int32_t)vp_lerp16(e0, e1, wz);
}

#endif
