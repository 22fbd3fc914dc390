/*
 * vp_worldgen.h — seeded synthetic voxel worlds, produced directly in the
 * resident format the GPU pipeline consumes: one RLE stream per chunk in a
 * 16-byte aligned word pool, plus the padded u16 shadow map.
 *
 * World kinds (voxel = uint8, 0 = air):
 *   VPG_TERRAIN_SMALL  2-D value-noise heightmap, 4 octaves, heights 8..56,
 *                      colour 1 + h/4 + per-column jitter 0..3.
 *   VPG_TERRAIN_CAVES  6-octave fractal heightmap 40..200, 3-D value-noise
 *                      caves carved where density > 0.55, colour from
 *                      wavy height bands with a two-colour surface layer.
 *   VPG_UNEVEN         one standalone chunk: noise blobs plus uniform random
 *                      voxels, occupancy log-uniform 0.1%..100%, colours
 *                      uniform over 1..255.
 *
 * The shadow map is built the way the reference's generator does it
 * (src/chunkset/gen.c:298-306 calls shadow_place_update for each solid voxel,
 * src/chunkset/shadow.h:77-89), but in one canonical serial order per map row
 * (chunk index ascending; inside a chunk x outer, z, y ascending), because the
 * reference's OpenMP generator races on it.
 */
#ifndef VP_WORLDGEN_H
#define VP_WORLDGEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { VPG_TERRAIN_SMALL = 1, VPG_TERRAIN_CAVES = 2, VPG_UNEVEN = 3 };

typedef struct vpg_world {
	int root_bitw;
	int max_bitw[3];
	int max[3];
	uint32_t nchunks;
	uint32_t *pool;        /* RLE words, each stream starts on a 4-word boundary */
	uint64_t pool_words;
	uint64_t pool_cap;
	uint64_t *off;         /* per chunk: word offset of its stream */
	uint32_t *len;         /* per chunk: words including the 0 terminator */
	uint16_t *shadow;      /* shadow_w * (shadow_z + pad rows), zero padded */
	uint64_t shadow_len;
	uint32_t shadow_w, shadow_z;
} vpg_world;

/* Allocate an empty (all-air) world; `pad_rows` zero rows follow the map. */
int vpg_world_alloc(vpg_world *w, int root_bitw, const int max_bitw[3], uint32_t pad_rows);
void vpg_world_free(vpg_world *w);

/* Fill `w` with terrain of `kind`; `hshift` scales the horizontal noise by
 * 2^hshift. Uses up to `nthreads` OpenMP threads (0 = all). */
int vpg_gen_terrain(vpg_world *w, int kind, uint64_t seed, int hshift, int nthreads);

/* Chunk size exponent (5, 6 or 7 in ratio 1:6:1) of standalone chunk k. */
int vpg_uneven_root_bitw(uint64_t seed, uint32_t k);
/* Occupancy target of standalone chunk k, in millionths. */
uint32_t vpg_uneven_occupancy_ppm(uint64_t seed, uint32_t k);
/* Fill a 1x1x1 world (allocated with vpg_uneven_root_bitw) with chunk k. */
int vpg_gen_uneven(vpg_world *w, uint64_t seed, uint32_t k);

/* Decode-free helpers used by the generators and tests. */
uint32_t vpg_rle_encode(const uint8_t *vox, uint32_t n, uint32_t *out);
void vpg_chunk_voxels(const vpg_world *w, uint32_t chunk, uint8_t *out);

/* Replace chunk `c`'s stream (appends to the pool). */
int vpg_set_chunk_rle(vpg_world *w, uint32_t c, const uint32_t *words, uint32_t nwords);

#ifdef __cplusplus
}
#endif
#endif
