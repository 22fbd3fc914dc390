/*
 * Test driver for the drop-in entry points (include/voxgpu_dropin.h): a
 * caller written against the reference's own ChunkSet/ChunkMD layout, doing
 * what src/chunkset.c does around the mesher — per-chunk mask, splat and
 * downsample calls in chunkset_manage's order (src/chunkset.c:318-459),
 * chunk_make_mesh, and the batched chunkset_manage with its flags.
 * Built by tests/test_gpu_dropin.py and driven through ctypes.
 */
#include "voxgpu_dropin.h"

#include <stdlib.h>
#include <string.h>

struct harness {
	struct ChunkSet *set;
	uint32_t N;
};

static uint32_t flat3(const struct ChunkSet *s, uint32_t x, uint32_t y, uint32_t z)
{
	return ((z << s->max_bitw[1] | y) << s->max_bitw[0]) | x;
}

/* A set like chunkset_create + chunkset_clear (src/chunkset.c:31-121), with
 * every chunk holding its RLE stream, or its decoded voxels if `decoded`. */
struct harness *harness_new(int root_bitw, const int mb[3], const uint32_t *pool, const uint64_t *off,
			    const uint32_t *len, const uint16_t *shadow, uint64_t shadow_len, uint32_t sw, uint32_t sz,
			    int decoded)
{
	struct harness *h = calloc(1, sizeof(*h));
	const uint32_t n = 1u << (mb[0] + mb[1] + mb[2]);
	struct ChunkSet *s = calloc(1, sizeof(struct ChunkSet) + n * sizeof(struct ChunkMD));
	s->count = n;
	s->root_bitw = (uint8_t)root_bitw;
	s->root = (uint16_t)(1u << root_bitw);
	for (int i = 0; i < 3; i++) {
		s->max_bitw[i] = (uint8_t)mb[i];
		s->max[i] = (uint16_t)(1u << mb[i]);
	}
	s->chunks = (struct ChunkMD *)(s + 1);
	h->N = 1u << (3 * root_bitw);
	s->null_chunk = calloc(1, sizeof(struct ChunkMD));
	s->null_chunk->voxels = calloc(h->N, 1);
	s->null_chunk->rle = (Voxel *)calloc(2, sizeof(uint32_t));
	((uint32_t *)s->null_chunk->rle)[0] = h->N;
	uint32_t i = 0;
	for (uint32_t z = 0; z < s->max[2]; z++)
		for (uint32_t y = 0; y < s->max[1]; y++)
			for (uint32_t x = 0; x < s->max[0]; x++, i++) {
				struct ChunkMD *c = &s->chunks[i];
				pthread_mutex_init(&c->mutex_read, NULL);
				pthread_mutex_init(&c->mutex_write, NULL);
				pthread_mutex_init(&c->mutex_svl, NULL);
				c->offset[0] = (uint16_t)x;
				c->offset[1] = (uint16_t)y;
				c->offset[2] = (uint16_t)z;
				c->count = h->N;
				uint32_t *copy = malloc(len[i] * sizeof(uint32_t));
				memcpy(copy, pool + off[i], len[i] * sizeof(uint32_t));
				c->rle = (Voxel *)copy;
				if (decoded) {
					c->voxels = rle_decompress(c->rle);
					free(c->rle);
					c->rle = NULL;
				}
			}
	s->shadow_map_size[0] = sw;
	s->shadow_map_size[1] = sz;
	s->shadow_map_length = (uint32_t)shadow_len;
	s->shadow_map = malloc(shadow_len * sizeof(uint16_t));
	memcpy(s->shadow_map, shadow, shadow_len * sizeof(uint16_t));
	h->set = s;
	return h;
}

/* src/chunkset.c:318-459 for chunk c, far branch; returns int16 items, or
 * -1 on a drop-in error. items[] gets the per-level counts. */
long harness_splats(struct harness *h, uint32_t c, int lod_max, int16_t *geom, uint32_t *items)
{
	struct ChunkSet *s = h->set;
	struct ChunkMD *m = &s->chunks[c];
	const size_t S3 = (size_t)(s->root + 1) * (s->root + 1) * (s->root + 1);
	uint8_t *mask = calloc(S3, 1), *work = calloc(S3, 1);
	chunk_make_mask(s, m, mask);
	if (vp_dropin_last_error()) return -1;
	uint32_t geom_items = 0;
	chunk_make_splatlist(s, m, 0, mask, geom, &geom_items);
	items[0] = geom_items;
	for (int l = 1; l <= lod_max; l++) {
		uint8_t *src = (l & 1) ? mask : work;
		uint8_t *dst = (l & 1) ? work : mask;
		if (l >= 2) memset(dst, 0, S3);
		chunk_mask_downsample(s, (int8_t)l, src, dst);
		uint32_t g2 = 0;
		chunk_make_splatlist(s, m, (uint8_t)l, dst, geom + geom_items, &g2);
		if (vp_dropin_last_error()) return -1;
		items[l] = g2;
		geom_items += g2;
	}
	free(mask);
	free(work);
	return geom_items;
}

long harness_mesh(struct harness *h, uint32_t c, int16_t *vbo, uint32_t *nv, uint32_t *ibo, uint32_t *ni)
{
	chunk_make_mesh(h->set, &h->set->chunks[c], vbo, nv, ibo, ni);
	return vp_dropin_last_error() ? -1 : (long)*nv;
}

/* Mark every chunk dirty with the given near/far modes and run the batched
 * chunkset_manage once. */
int harness_manage(struct harness *h, const uint8_t *make_mesh)
{
	for (uint32_t i = 0; i < h->set->count; i++) {
		h->set->chunks[i].dirty = 1;
		h->set->chunks[i].make_mesh = make_mesh[i];
		h->set->chunks[i].svl_dirty = 0;
		h->set->chunks[i].mesh_dirty = 0;
	}
	chunkset_manage(h->set);
	return vp_dropin_last_error();
}

/* Published results of chunk c after harness_manage. */
void harness_published(struct harness *h, uint32_t c, uint32_t *svl_items, uint32_t *nv, uint32_t *ni,
		       uint32_t *flags)
{
	struct ChunkMD *m = &h->set->chunks[c];
	for (int l = 0; l < MAX_LOD_LEVEL; l++) svl_items[l] = m->svl_items[l];
	*nv = m->mesh_vbo_items;
	*ni = m->mesh_ibo_items;
	*flags = (uint32_t)m->svl_dirty | ((uint32_t)m->mesh_dirty << 1) | ((uint32_t)m->no_geometry << 2) |
		 ((uint32_t)m->dirty << 3) | ((uint32_t)m->changing << 4);
}

void harness_copy_published(struct harness *h, uint32_t c, int16_t *svl, int16_t *vbo, uint32_t *ibo)
{
	struct ChunkMD *m = &h->set->chunks[c];
	if (m->svl && svl) memcpy(svl, m->svl, m->svl_items_total * sizeof(int16_t));
	if (m->mesh_vbo && vbo) memcpy(vbo, m->mesh_vbo, m->mesh_vbo_items * sizeof(int16_t));
	if (m->mesh_ibo && ibo) memcpy(ibo, m->mesh_ibo, m->mesh_ibo_items * sizeof(uint32_t));
}

/* rle_compress / rle_decompress round trip through the drop-ins */
uint32_t harness_rle(const uint8_t *vox, uint32_t n, uint32_t *out, uint8_t *back)
{
	Voxel *r = rle_compress((Voxel *)vox, n);
	if (!r) return 0;
	uint32_t k = 0;
	while (((uint32_t *)r)[k]) k++;
	memcpy(out, r, (k + 1) * sizeof(uint32_t));
	Voxel *d = rle_decompress(r);
	if (d) memcpy(back, d, n);
	free(r);
	free(d);
	return k + 1;
}

size_t harness_sizeof_chunkmd(void) { return sizeof(struct ChunkMD); }
size_t harness_sizeof_chunkset(void) { return sizeof(struct ChunkSet); }
uint32_t harness_flat3(struct harness *h, uint32_t x, uint32_t y, uint32_t z) { return flat3(h->set, x, y, z); }
