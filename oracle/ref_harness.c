/*
 * oracle/ref_harness.c — drives the UNMODIFIED reference hot-path sources
 * (src/chunkset.c, src/chunkset/rle.c, src/chunkset/mesher.c,
 * src/chunkset/edit.c of kosshi-net/voxplat 0.11), compiled together with
 * this file by oracle/build_ref.sh into oracle/_ref/libvpref.so.
 *
 * TEST INFRASTRUCTURE ONLY: it generates golden fixtures and pins the C
 * restatement in oracle/vpo.c. Harness rules (each avoids reference
 * behaviour that is undefined or nondeterministic, without changing results
 * where the reference is defined):
 *   - per-chunk functions are called directly with worst-case sized buffers,
 *     in the order chunkset_manage uses (src/chunkset.c:318-459), instead of
 *     chunkset_manage itself (its gating reads the clock and its buffers
 *     overflow on dense meshes);
 *   - every chunk gets a private RLE copy, so chunk_make_mask's early-out
 *     (src/chunkset/mesher.c:404-409, which reads uninitialised neighbour
 *     copies) is never taken;
 *   - the shadow map is replaced by a zeroed buffer with padding rows,
 *     placed at the start of a 2^32-element zero mapping: a shadow sample
 *     taken one voxel below y = 0 at the world origin wraps its uint32 index
 *     to 0xFFFFFFFF (src/chunkset/mesher.c:315-316 with
 *     src/chunkset/shadow.h:50), which faults on an ordinary allocation. The
 *     value read there never matters (the compare is against ws[1]+1 == 0);
 *     the mapping only lets the reference run to completion;
 *   - rle_work_buf_len is set to root^3 before every decode.
 */
#include "chunkset.h"
#include "chunkset/edit.h"
#include "chunkset/mesher.h"
#include "chunkset/rle.h"

#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>

extern uint32_t rle_work_buf_len;
void shadow_init(struct ChunkSet *set);

static uint64_t shadow_padded_len;

struct ChunkSet *vpref_world_new(int root_bitw, int bx, int by, int bz, uint32_t pad_rows)
{
	uint8_t mb[3] = {(uint8_t)bx, (uint8_t)by, (uint8_t)bz};
	struct ChunkSet *set = chunkset_create((uint8_t)root_bitw, mb);
	chunkset_clear(set);
	shadow_init(set);
	free(set->shadow_map);
	shadow_padded_len = (uint64_t)set->shadow_map_size[0] * (set->shadow_map_size[1] + pad_rows);
	size_t span = ((size_t)1 << 32) + 2 + (size_t)shadow_padded_len;
	void *m = mmap(NULL, span * sizeof(uint16_t), PROT_READ | PROT_WRITE,
		       MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
	set->shadow_map = (m == MAP_FAILED) ? NULL : (uint16_t *)m;
	return set;
}

uint64_t vpref_shadow_len(struct ChunkSet *set) { (void)set; return shadow_padded_len; }

void vpref_set_shadow(struct ChunkSet *set, const uint16_t *map, uint64_t n)
{
	if (n > shadow_padded_len) n = shadow_padded_len;
	memcpy(set->shadow_map, map, n * sizeof(uint16_t));
}

void vpref_get_shadow(struct ChunkSet *set, uint16_t *out, uint64_t n)
{
	if (n > shadow_padded_len) n = shadow_padded_len;
	memcpy(out, set->shadow_map, n * sizeof(uint16_t));
}

void vpref_set_chunk_rle(struct ChunkSet *set, uint32_t c, const uint32_t *words, uint32_t n)
{
	struct ChunkMD *m = &set->chunks[c];
	uint32_t *copy = (uint32_t *)calloc((size_t)n + 16, sizeof(uint32_t));
	memcpy(copy, words, (size_t)n * sizeof(uint32_t));
	m->rle = (Voxel *)copy;
	m->voxels = NULL;
}

static void prime_rle(struct ChunkSet *set)
{
	rle_work_buf_len = (uint32_t)set->root * set->root * set->root;
}

/* src/chunkset.c:318-459, far-chunk branch, generalised to lod_max levels. */
uint32_t vpref_chunk_splats(struct ChunkSet *set, uint32_t c, int lod_max, int16_t *geom,
			    uint32_t *items, uint8_t *mask, uint8_t *work)
{
	struct ChunkMD *m = &set->chunks[c];
	size_t S3 = (size_t)(set->root + 1) * (set->root + 1) * (set->root + 1);
	prime_rle(set);
	chunk_open_ro(set, m);
	memset(work, 0, S3);
	memset(mask, 0, S3);
	chunk_make_mask(set, m, mask);
	uint32_t geom_items = 0;
	chunk_make_splatlist(set, m, 0, mask, geom, &geom_items);
	items[0] = geom_items;
	for (int l = 1; l <= lod_max; l++) {
		uint8_t *src = (l & 1) ? mask : work;
		uint8_t *dst = (l & 1) ? work : mask;
		if (l >= 2) memset(dst, 0, S3);
		chunk_mask_downsample(set, (int8_t)l, src, dst);
		uint32_t g2 = 0;
		chunk_make_splatlist(set, m, (uint8_t)l, dst, geom + geom_items, &g2);
		items[l] = g2;
		geom_items += g2;
	}
	chunk_close_ro(set, m);
	return geom_items;
}

/* src/chunkset.c:318-345, near-chunk branch. */
void vpref_chunk_mesh(struct ChunkSet *set, uint32_t c, int16_t *vbo, uint32_t *nv, uint32_t *ibo,
		      uint32_t *ni)
{
	struct ChunkMD *m = &set->chunks[c];
	prime_rle(set);
	chunk_open_ro(set, m);
	*nv = 0;
	*ni = 0;
	chunk_make_mesh(set, m, vbo, nv, ibo, ni);
	chunk_close_ro(set, m);
}

void vpref_edit_sphere(struct ChunkSet *set, int32_t x, int32_t y, int32_t z, uint32_t r, uint8_t v)
{
	int32_t ws[3] = {x, y, z};
	prime_rle(set);
	chunkset_edit_sphere(set, ws, r, v);
}

/* The reference's DDA picking ray (src/chunkset/edit.c:248-314). */
Voxel chunkset_edit_raycast_until_solid(struct ChunkSet *set, float *origin, float *vector, uint32_t *coord,
					int8_t *normal);

uint8_t vpref_raycast(struct ChunkSet *set, const float *origin, const float *vector, uint32_t *coord, int8_t *normal)
{
	float o[3] = {origin[0], origin[1], origin[2]}, v[3] = {vector[0], vector[1], vector[2]};
	prime_rle(set);
	normal[0] = normal[1] = normal[2] = 0;
	return chunkset_edit_raycast_until_solid(set, o, v, coord, normal);
}

void vpref_chunk_voxels(struct ChunkSet *set, uint32_t c, uint8_t *out)
{
	struct ChunkMD *m = &set->chunks[c];
	prime_rle(set);
	chunk_open_ro(set, m);
	memcpy(out, m->voxels, (size_t)set->root * set->root * set->root);
	chunk_close_ro(set, m);
}

int vpref_chunk_dirty(struct ChunkSet *set, uint32_t c) { return set->chunks[c].dirty; }
void vpref_clear_dirty(struct ChunkSet *set)
{
	for (uint32_t c = 0; c < set->count; c++) set->chunks[c].dirty = 0;
}

uint32_t vpref_rle_compress(const uint8_t *vox, uint32_t n, uint32_t *out)
{
	uint32_t *r = (uint32_t *)rle_compress((Voxel *)vox, n);
	uint32_t k = 0;
	while (r[k]) {
		out[k] = r[k];
		k++;
	}
	out[k++] = 0;
	free(r);
	return k;
}

uint32_t vpref_rle_decompress(const uint32_t *words, uint8_t *out, uint32_t n)
{
	rle_work_buf_len = n;
	uint8_t *v = (uint8_t *)rle_decompress((void *)words);
	memcpy(out, v, n);
	free(v);
	return n;
}

/* Timed CPU baseline on the reference's own code: chunkset_manage's
 * per-chunk work (src/chunkset.c:251-459) for a list of chunks, OpenMP over
 * chunks like the reference (there: 4 threads, 8 chunks per 5 ms tick, a
 * 100 ms rate limit; here: `nthreads` threads and no throttles). Cold: the
 * decoded voxels of every chunk are dropped first, as chunk_compress leaves
 * idle chunks (src/chunkset.c:213-230), so each chunk_open_ro decodes from
 * RLE. Each chunk's output is copied into an exact-size buffer, as the
 * reference publishes it (src/chunkset.c:347-358, 472-480). Returns the
 * output bytes produced. */
uint64_t vpref_rebuild(struct ChunkSet *set, const uint32_t *chunks, uint32_t n, const uint8_t *make_mesh,
		       int lod_max, int nthreads)
{
	for (uint32_t c = 0; c < set->count; c++) {
		struct ChunkMD *m = &set->chunks[c];
		if (m->voxels && m->voxels != set->null_chunk->voxels && m->rle) {
			free(m->voxels);
			m->voxels = NULL;
		}
	}
	prime_rle(set);
	const size_t R = set->root, S3 = (R + 1) * (R + 1) * (R + 1);
	size_t geom_cap = 16;
	for (int l = 0; l <= lod_max; l++) geom_cap += 4 * (((R >> l) + 1) * ((R >> l) + 1) * ((R >> l) + 1));
	uint64_t total = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : total)
	{
		int16_t *geom = NULL, *vbo = NULL;
		uint32_t *ibo = NULL;
		uint8_t *mask = (uint8_t *)malloc(S3), *work = (uint8_t *)malloc(S3);
#pragma omp for schedule(dynamic, 1)
		for (uint32_t k = 0; k < n; k++) {
			const uint32_t c = chunks[k];
			if (make_mesh && make_mesh[c]) {
				if (!vbo) {
					vbo = (int16_t *)malloc(3 * R * R * R * 16 * sizeof(int16_t));
					ibo = (uint32_t *)malloc(3 * R * R * R * 6 * sizeof(uint32_t));
				}
				uint32_t nv = 0, ni = 0;
				vpref_chunk_mesh(set, c, vbo, &nv, ibo, &ni);
				int16_t *pv = (int16_t *)malloc((size_t)nv * sizeof(int16_t) + 1);
				uint32_t *pi = (uint32_t *)malloc((size_t)ni * sizeof(uint32_t) + 1);
				memcpy(pv, vbo, (size_t)nv * sizeof(int16_t));
				memcpy(pi, ibo, (size_t)ni * sizeof(uint32_t));
				total += (uint64_t)nv * 2 + (uint64_t)ni * 4;
				free(pv);
				free(pi);
			} else {
				if (!geom) geom = (int16_t *)malloc(geom_cap * sizeof(int16_t));
				uint32_t items[8];
				const uint32_t t = vpref_chunk_splats(set, c, lod_max, geom, items, mask, work);
				int16_t *ps = (int16_t *)malloc((size_t)t * sizeof(int16_t) + 1);
				memcpy(ps, geom, (size_t)t * sizeof(int16_t));
				total += (uint64_t)t * 2;
				free(ps);
			}
		}
		free(geom);
		free(vbo);
		free(ibo);
		free(mask);
		free(work);
	}
	return total;
}
