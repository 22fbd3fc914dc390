/*
 * oracle/vpo.c — CPU restatement of voxplat's per-chunk geometry pipeline.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle; see vpo.h). Scalar C that
 * follows the reference loop by loop; each function cites the reference
 * function it restates (kosshi-net/voxplat 0.11, paths relative to the
 * project root).
 */
#include "vpo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define RLE_MASK 0xFFFFFFu
#define RLE_SHIFT 24

/* src/chunkset/rle.c:44-87 */
uint32_t vpo_rle_encode(const uint8_t *vox, uint32_t n, uint32_t *out)
{
	uint32_t count = 1, b = 0;
	uint8_t last = vox[0];
	for (uint32_t i = 1; i < n; i++) {
		uint8_t cur = vox[i];
		if (cur == last && count < RLE_MASK) {
			count++;
			continue;
		}
		out[b++] = count | ((uint32_t)last << RLE_SHIFT);
		count = 1;
		last = cur;
	}
	out[b++] = count | ((uint32_t)last << RLE_SHIFT);
	out[b++] = 0;
	return b;
}

/* src/chunkset/rle.c:90-117. The first word is always consumed (do-while);
 * decoding stops at the first zero word after it. Writes past `cap` are
 * dropped (the reference sizes its buffer from the last encoded length). */
uint32_t vpo_rle_decode(const uint32_t *words, uint8_t *out, uint32_t cap)
{
	uint32_t i = 0, b = 0;
	do {
		uint32_t count = words[i] & RLE_MASK;
		uint8_t item = (uint8_t)(words[i] >> RLE_SHIFT);
		uint32_t n = count;
		if (b >= cap) n = 0;
		else if (n > cap - b) n = cap - b;
		memset(out + b, item, n);
		b += count;
	} while (words[++i]);
	return b;
}

vpo_world *vpo_world_new(int root_bitw, const int max_bitw[3], uint32_t pad_rows)
{
	vpo_world *w = (vpo_world *)calloc(1, sizeof(*w));
	w->root_bitw = root_bitw;
	w->R = 1 << root_bitw;
	for (int i = 0; i < 3; i++) {
		w->max_bitw[i] = max_bitw[i];
		w->max[i] = 1 << max_bitw[i];
	}
	w->nchunks = (uint32_t)w->max[0] * w->max[1] * w->max[2];
	w->rle = (uint32_t **)calloc(w->nchunks, sizeof(uint32_t *));
	w->rle_len = (uint32_t *)calloc(w->nchunks, sizeof(uint32_t));
	w->vox = (uint8_t **)calloc(w->nchunks, sizeof(uint8_t *));
	/* src/chunkset/shadow.h:26-43 sizes; padded and zeroed here. */
	w->shadow_w = ((uint32_t)w->max[0] << root_bitw) + ((uint32_t)w->max[1] << root_bitw);
	w->shadow_z = (uint32_t)w->max[2] << root_bitw;
	w->shadow_len = (uint64_t)w->shadow_w * (w->shadow_z + pad_rows);
	w->shadow = (uint16_t *)calloc(w->shadow_len, sizeof(uint16_t));
	/* chunkset_clear (src/chunkset.c:85-121): every chunk starts as air. */
	uint32_t N = (uint32_t)w->R * w->R * w->R;
	for (uint32_t c = 0; c < w->nchunks; c++) {
		w->rle[c] = (uint32_t *)malloc(2 * sizeof(uint32_t));
		w->rle[c][0] = N;
		w->rle[c][1] = 0;
		w->rle_len[c] = 2;
	}
	return w;
}

void vpo_world_free(vpo_world *w)
{
	if (!w) return;
	for (uint32_t c = 0; c < w->nchunks; c++) {
		free(w->rle[c]);
		free(w->vox[c]);
	}
	free(w->rle);
	free(w->rle_len);
	free(w->vox);
	free(w->shadow);
	free(w);
}

void vpo_world_set_rle(vpo_world *w, uint32_t c, const uint32_t *words, uint32_t n)
{
	free(w->rle[c]);
	free(w->vox[c]);
	w->vox[c] = NULL;
	w->rle[c] = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
	memcpy(w->rle[c], words, (size_t)n * sizeof(uint32_t));
	w->rle_len[c] = n;
}

void vpo_world_set_shadow(vpo_world *w, const uint16_t *map, uint64_t n)
{
	if (n > w->shadow_len) n = w->shadow_len;
	memcpy(w->shadow, map, n * sizeof(uint16_t));
}

/* chunk_open_ro (src/chunkset.c:133-152): decode lazily and keep the voxels.
 * Safe to call from several threads: a racing decode loses the swap. */
const uint8_t *vpo_world_voxels(vpo_world *w, uint32_t c)
{
	uint8_t *v = __atomic_load_n(&w->vox[c], __ATOMIC_ACQUIRE);
	if (v) return v;
	uint32_t N = (uint32_t)w->R * w->R * w->R;
	uint8_t *d = (uint8_t *)malloc(N);
	vpo_rle_decode(w->rle[c], d, N);
	uint8_t *expected = NULL;
	if (!__atomic_compare_exchange_n(&w->vox[c], &expected, d, 0, __ATOMIC_ACQ_REL,
					 __ATOMIC_ACQUIRE)) {
		free(d);
		return expected;
	}
	return d;
}

/* chunk_compress (src/chunkset.c:213-230): re-encode the decoded voxels. */
void vpo_world_compress(vpo_world *w, uint32_t c)
{
	if (!w->vox[c]) return;
	uint32_t N = (uint32_t)w->R * w->R * w->R;
	uint32_t *tmp = (uint32_t *)malloc(((size_t)N + 2) * sizeof(uint32_t));
	uint32_t n = vpo_rle_encode(w->vox[c], N, tmp);
	free(w->rle[c]);
	w->rle[c] = (uint32_t *)realloc(tmp, (size_t)n * sizeof(uint32_t));
	w->rle_len[c] = n;
}

/* flatten3 (src/chunkset.c:124-126) */
uint32_t vpo_flatten3(const vpo_world *w, const uint32_t cv[3])
{
	return ((cv[2] << w->max_bitw[1] | cv[1]) << w->max_bitw[0]) | cv[0];
}

/* chunkset_edit_read (src/chunkset/edit.c:10-36): out of world reads air. */
uint8_t vpo_world_read(vpo_world *w, const uint32_t ws[3])
{
	for (int i = 0; i < 3; i++)
		if (ws[i] >= ((uint32_t)w->max[i] << w->root_bitw)) return 0;
	uint32_t cv[3], vv[3];
	for (int i = 0; i < 3; i++) {
		cv[i] = ws[i] >> w->root_bitw;
		vv[i] = ws[i] - (cv[i] << w->root_bitw);
	}
	const uint8_t *v = vpo_world_voxels(w, vpo_flatten3(w, cv));
	return v[(vv[2] << (2 * w->root_bitw)) | (vv[1] << w->root_bitw) | vv[0]];
}

static inline uint16_t shadow_at(const vpo_world *w, uint32_t idx)
{
	return (uint64_t)idx < w->shadow_len ? w->shadow[idx] : 0;
}

/* shadow_index + shadow_sample (src/chunkset/shadow.h:45-63); all index
 * arithmetic in uint32 as in the reference. */
int vpo_shadow_sample(const vpo_world *w, const uint32_t ws[3])
{
	uint32_t idx = (ws[0] + ws[1]) + w->shadow_w * ws[2];
	uint32_t lim = ws[1] + 1;
	return !(shadow_at(w, idx) < lim && shadow_at(w, idx + 1) < lim);
}

/* shadow_sample_normal (src/chunkset/shadow.h:65-75) */
int vpo_shadow_sample_normal(const vpo_world *w, const uint32_t ws[3])
{
	uint32_t idx = (ws[0] + ws[1]) + w->shadow_w * ws[2];
	uint32_t lim = ws[1] + 1;
	return !(shadow_at(w, idx) < lim && shadow_at(w, idx - 1) < lim);
}

/* shadow_place_update (src/chunkset/shadow.h:77-89) */
void vpo_shadow_place_update(vpo_world *w, const uint32_t ws[3])
{
	if (vpo_shadow_sample(w, ws)) return;
	uint32_t idx = (ws[0] + ws[1]) + w->shadow_w * ws[2];
	if ((uint64_t)idx < w->shadow_len) w->shadow[idx] = (uint16_t)ws[1];
}

/* The +x/+y/+z neighbours of chunk c, or NULL past the world edge
 * (src/chunkset/mesher.c:391-402 / 200-211). */
static void plus_neighbours(vpo_world *w, uint32_t c, const uint8_t *nb[3], uint32_t off[3])
{
	uint32_t cv[3];
	cv[0] = c & (uint32_t)(w->max[0] - 1);
	cv[1] = (c >> w->max_bitw[0]) & (uint32_t)(w->max[1] - 1);
	cv[2] = c >> (w->max_bitw[0] + w->max_bitw[1]);
	for (int i = 0; i < 3; i++) off[i] = cv[i];
	for (int i = 0; i < 3; i++) {
		cv[i]++;
		if (cv[i] + 1 > (uint32_t)w->max[i])
			nb[i] = NULL;
		else
			nb[i] = vpo_world_voxels(w, vpo_flatten3(w, cv));
		cv[i]--;
	}
}

/* chunk_make_mask (src/chunkset/mesher.c:377-456) */
void vpo_make_mask(vpo_world *w, uint32_t c, uint8_t *mask)
{
	const uint8_t *nb[3];
	uint32_t off[3];
	plus_neighbours(w, c, nb, off);
	const uint8_t *v = vpo_world_voxels(w, c);
	const uint32_t R = (uint32_t)w->R, rb = (uint32_t)w->root_bitw, S = R + 1;
	uint32_t AC[3], Ai = 0;
	for (AC[2] = 0; AC[2] < R; AC[2]++)
		for (AC[1] = 0; AC[1] < R; AC[1]++)
			for (AC[0] = 0; AC[0] < R; AC[0]++, Ai++) {
				uint8_t A = v[Ai];
				uint32_t shift = 0;
				for (int i = 0; i < 3; i++, shift += rb) {
					uint8_t B;
					if (AC[i] + 1 == R)
						B = nb[i] ? nb[i][Ai - ((R - 1) << shift)] : 0;
					else
						B = v[Ai + (1u << shift)];
					if (!A == !B) continue;
					uint32_t MC[3] = {AC[0], AC[1], AC[2]};
					MC[i] += (A == 0);
					mask[(MC[2] * S + MC[1]) * S + MC[0]] = A | B;
				}
			}
}

/* chunk_mask_downsample (src/chunkset/mesher.c:460-493): the last nonzero
 * child in z,y,x scan order wins. */
void vpo_mask_downsample(int R, int level, const uint8_t *mask, uint8_t *work)
{
	const uint32_t S = (uint32_t)R + 1;
	const uint32_t range = ((uint32_t)R >> (level - 1)) + 1;
	for (uint32_t z = 0; z < range; z++)
		for (uint32_t y = 0; y < range; y++)
			for (uint32_t x = 0; x < range; x++) {
				uint8_t m = mask[(z * S + y) * S + x];
				if (!m) continue;
				work[((z >> 1) * S + (y >> 1)) * S + (x >> 1)] = m;
			}
}

/* chunk_make_splatlist (src/chunkset/mesher.c:497-536). Returns items
 * written (the reference adds them to *geometry_items). */
uint32_t vpo_make_splatlist(vpo_world *w, uint32_t c, int level, const uint8_t *mask, int16_t *geom)
{
	uint32_t cv[3];
	cv[0] = c & (uint32_t)(w->max[0] - 1);
	cv[1] = (c >> w->max_bitw[0]) & (uint32_t)(w->max[1] - 1);
	cv[2] = c >> (w->max_bitw[0] + w->max_bitw[1]);
	const uint32_t R = (uint32_t)w->R, S = R + 1;
	const uint32_t range = (R >> level) + 1;
	uint32_t v = 0;
	for (uint32_t z = 0; z < range; z++)
		for (uint32_t y = 0; y < range; y++)
			for (uint32_t x = 0; x < range; x++) {
				uint8_t m = mask[(z * S + y) * S + x];
				if (!m) continue;
				uint32_t AC[3] = {x, y, z}, ws[3];
				for (int j = 0; j < 3; j++) {
					ws[j] = (cv[j] << w->root_bitw) + (AC[j] << level);
					geom[v++] = (int16_t)(uint16_t)ws[j];
				}
				if (level)
					for (int j = 0; j < 3; j++) ws[j] += 1u << level;
				geom[v++] = (int16_t)(uint16_t)(m | (vpo_shadow_sample(w, ws) << 6));
			}
	return v;
}

/* chunkset_manage's far-chunk sequence (src/chunkset.c:321-459). */
uint32_t vpo_chunk_splats(vpo_world *w, uint32_t c, int lod_max, int16_t *geom, uint32_t *items,
			  uint8_t *mask, uint8_t *work)
{
	const size_t S3 = (size_t)(w->R + 1) * (w->R + 1) * (w->R + 1);
	memset(mask, 0, S3);
	memset(work, 0, S3);
	vpo_make_mask(w, c, mask);
	uint32_t total = vpo_make_splatlist(w, c, 0, mask, geom);
	items[0] = total;
	for (int l = 1; l <= lod_max; l++) {
		uint8_t *src = (l & 1) ? mask : work;
		uint8_t *dst = (l & 1) ? work : mask;
		if (l >= 2) memset(dst, 0, S3);
		vpo_mask_downsample(w->R, l, src, dst);
		items[l] = vpo_make_splatlist(w, c, l, dst, geom + total);
		total += items[l];
	}
	return total;
}

/* Vertex offsets of the three visible quad orientations (the first 36
 * entries of lutv, src/chunkset/mesher.c:19-33) and the index pattern with
 * AO rotation and back-face variants (luti, src/chunkset/mesher.c:53-66). */
static const uint8_t quad_offset[3][4][3] = {
	{{1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}},
	{{0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}},
	{{1, 0, 1}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}},
};
static const uint8_t quad_index[24] = {0, 3, 1, 2, 1, 3, 3, 2, 0, 1, 0, 2,
				       1, 3, 0, 3, 1, 2, 0, 2, 3, 2, 0, 1};

/* sample_ao (mesher.c:72-116) and sample_ao_border (mesher.c:119-171):
 * edge samples -u, -v, +u, +v and corner samples (-,-), (+,-), (+,+), (-,+)
 * around the air voxel, in the two axes other than the face axis. Interior
 * voxels read the chunk; border voxels read the world. */
static void sample_ao(vpo_world *w, const uint8_t *v, const uint32_t off[3], const uint32_t AIR[3],
		      int face, int border, uint8_t aon[4], uint8_t aoc[4])
{
	int uv[2], d = 0;
	const uint32_t rb = (uint32_t)w->root_bitw;
	uint32_t base[3];
	for (int k = 0; k < 3; k++) base[k] = border ? (off[k] << rb) + AIR[k] : AIR[k];
#define AO_READ(O) (border ? !!vpo_world_read(w, O) \
			   : !!v[((O)[2] << (2 * rb)) | ((O)[1] << rb) | (O)[0]])
	for (int a = 0; a < 3; a++) {
		if (a == face) continue;
		uv[d] = a;
		uint32_t O[3];
		memcpy(O, base, sizeof(O));
		O[a]++;
		aon[d + 2] = AO_READ(O);
		memcpy(O, base, sizeof(O));
		O[a]--;
		aon[d] = AO_READ(O);
		d++;
	}
	static const int cs[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
	for (int k = 0; k < 4; k++) {
		uint32_t O[3];
		memcpy(O, base, sizeof(O));
		O[uv[0]] += (uint32_t)cs[k][0];
		O[uv[1]] += (uint32_t)cs[k][1];
		aoc[k] = AO_READ(O);
	}
#undef AO_READ
}

/* chunk_make_mesh (src/chunkset/mesher.c:184-357) */
void vpo_make_mesh(vpo_world *w, uint32_t c, int16_t *geom, uint32_t *vbo_items, uint32_t *index,
		   uint32_t *ibo_items)
{
	const uint8_t *nb[3];
	uint32_t off[3];
	plus_neighbours(w, c, nb, off);
	const uint8_t *vx = vpo_world_voxels(w, c);
	const uint32_t R = (uint32_t)w->R, rb = (uint32_t)w->root_bitw;
	uint32_t v = 0, nidx = 0, vertices = 0;
	uint32_t AC[3], Ai = 0;
	for (AC[2] = 0; AC[2] < R; AC[2]++)
		for (AC[1] = 0; AC[1] < R; AC[1]++)
			for (AC[0] = 0; AC[0] < R; AC[0]++, Ai++) {
				uint8_t A = vx[Ai];
				uint32_t shift = 0;
				for (int i = 0; i < 3; i++, shift += rb) {
					uint8_t B;
					if (AC[i] == R - 1)
						B = nb[i] ? nb[i][Ai - ((R - 1) << shift)] : 0;
					else
						B = vx[Ai + (1u << shift)];
					if (!A == !B) continue;
					uint32_t AIR[3] = {AC[0], AC[1], AC[2]};
					AIR[i] += (B == 0);
					uint32_t BLOCK[3] = {AC[0], AC[1], AC[2]};
					BLOCK[i] += (A == 0);
					int border = 0;
					for (int k = 0; k < 3; k++)
						if (AC[k] == 0 || AC[k] == R - 1) border = 1;
					uint8_t aon[4], aoc[4];
					sample_ao(w, vx, off, AIR, i, border, aon, aoc);
					uint8_t va[4];
					uint8_t e0 = (uint8_t)((aon[0] + aon[1]) | aoc[0]);
					uint8_t e1 = (uint8_t)((aon[1] + aon[2]) | aoc[1]);
					uint8_t e2 = (uint8_t)((aon[2] + aon[3]) | aoc[2]);
					uint8_t e3 = (uint8_t)((aon[3] + aon[0]) | aoc[3]);
					if (i == 0) {
						va[0] = e0; va[3] = e1; va[2] = e2; va[1] = e3;
					} else if (i == 1) {
						va[0] = e0; va[1] = e1; va[2] = e2; va[3] = e3;
					} else {
						va[1] = e0; va[0] = e1; va[3] = e2; va[2] = e3;
					}
					int rotate = (va[0] + va[2] < va[1] + va[3]) ? 6 : 0;
					uint32_t ws[3];
					for (int k = 0; k < 3; k++) ws[k] = (off[k] << rb) + BLOCK[k];
					int normal = (A == 0);
					int shadow = 0;
					if (i == 0 && normal)
						shadow = vpo_shadow_sample_normal(w, ws);
					else if (i == 1 && !normal)
						shadow = vpo_shadow_sample(w, ws);
					ws[i] -= (uint32_t)normal;
					int diamond = 3;
					if (i == 2) {
						shadow = 0;
						uint32_t sws[3] = {ws[0], ws[1], ws[2]};
						if (!B) sws[2] += 1;
						diamond = (!vpo_shadow_sample(w, sws)) << 1;
						sws[1] -= 1;
						diamond |= !vpo_shadow_sample(w, sws);
					}
					for (int vert = 0; vert < 4; vert++) {
						for (int k = 0; k < 3; k++)
							geom[v++] = (int16_t)(uint16_t)(ws[k] + quad_offset[i][vert][k]);
						int word = (A | B) | (va[vert] << 6) | ((i + 3 * normal) << 8) |
							   (vert << 11) | (shadow << 13) | (diamond << 14);
						geom[v++] = (int16_t)(uint16_t)word;
					}
					for (int k = 0; k < 6; k++)
						index[nidx++] = vertices + quad_index[normal * 12 + k + rotate];
					vertices += 4;
				}
			}
	*vbo_items = v;
	*ibo_items = nidx;
}

/* chunkset_get_chunks_in_aabb (src/chunkset/edit.c:89-126), chunk_ws_inside
 * (:129-140), chunk_ws_write (:143-176) and chunkset_edit_sphere
 * (:179-244). The distance test is the reference's float sqrtf compare. */
uint32_t vpo_edit_sphere(vpo_world *w, const int32_t ws[3], uint32_t radius, uint8_t voxel,
			 uint8_t *dirty)
{
	const int rb = w->root_bitw, R = w->R;
	int32_t mn[3], mx[3];
	for (int i = 0; i < 3; i++) {
		mn[i] = ws[i] - (int32_t)radius - 1;
		mx[i] = ws[i] + (int32_t)radius + 1;
	}
	int16_t cmin[3], cmax[3];
	for (int i = 0; i < 3; i++) {
		cmax[i] = (int16_t)(mx[i] >> rb);
		cmin[i] = (int16_t)(mn[i] >> rb);
	}
	uint32_t list[1024];
	uint32_t n = 0;
	int16_t cs[3];
	for (cs[0] = cmin[0]; cs[0] <= cmax[0]; ++cs[0])
		for (cs[1] = cmin[1]; cs[1] <= cmax[1]; ++cs[1])
			for (cs[2] = cmin[2]; cs[2] <= cmax[2]; ++cs[2]) {
				int ok = 1;
				for (int i = 0; i < 3; i++)
					if (cs[i] < 0 || cs[i] >= w->max[i]) ok = 0;
				if (!ok || n >= 1024) continue;
				uint32_t cv[3] = {(uint16_t)cs[0], (uint16_t)cs[1], (uint16_t)cs[2]};
				list[n++] = vpo_flatten3(w, cv);
			}
	if (!n) return 0;
	const float fr = (float)radius;
	for (uint32_t k = 0; k < n; k++) {
		uint32_t c = list[k];
		uint8_t *vx = (uint8_t *)vpo_world_voxels(w, c);
		int32_t lo[3];
		lo[0] = (int32_t)((c & (uint32_t)(w->max[0] - 1)) << rb);
		lo[1] = (int32_t)(((c >> w->max_bitw[0]) & (uint32_t)(w->max[1] - 1)) << rb);
		lo[2] = (int32_t)((c >> (w->max_bitw[0] + w->max_bitw[1])) << rb);
		int32_t u[3];
		for (u[0] = mn[0]; u[0] < mx[0]; u[0]++)
			for (u[1] = mn[1]; u[1] < mx[1]; u[1]++)
				for (u[2] = mn[2]; u[2] < mx[2]; u[2]++) {
					float d0 = (float)ws[0] - (float)u[0];
					float d1 = (float)ws[1] - (float)u[1];
					float d2 = (float)ws[2] - (float)u[2];
					float dist = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
					if (!(dist < fr)) continue;
					int inside = 1;
					for (int i = 0; i < 3; i++)
						if (u[i] < lo[i] || u[i] + 1 > lo[i] + R) inside = 0;
					if (!inside) continue;
					if (u[1] >= 2)
						vx[(uint32_t)(u[0] - lo[0]) |
						   ((uint32_t)(u[1] - lo[1]) << rb) |
						   ((uint32_t)(u[2] - lo[2]) << (2 * rb))] = voxel;
					if (voxel) {
						uint32_t uu[3] = {(uint32_t)u[0], (uint32_t)u[1], (uint32_t)u[2]};
						vpo_shadow_place_update(w, uu);
					}
				}
		vpo_world_compress(w, c);
	}
	if (dirty)
		for (uint32_t k = 0; k < n; k++) dirty[list[k]] = 1;
	return n;
}

/* gfx_update_svl's per-node concatenation (src/gfx/vsplat.c:209-331). */
uint64_t vpo_group_node(const vpo_world *w, int lod, const uint32_t node[3], int16_t *const *svl,
			const uint32_t *const *svl_items, int16_t *out)
{
	uint32_t lo[3], hi[3];
	for (int i = 0; i < 3; i++) {
		lo[i] = node[i] << lod;
		hi[i] = (node[i] + 1) << lod;
		if (hi[i] > (uint32_t)w->max[i]) hi[i] = (uint32_t)w->max[i];
	}
	uint64_t total = 0;
	uint32_t s[3];
	for (s[0] = lo[0]; s[0] < hi[0]; s[0]++)
		for (s[1] = lo[1]; s[1] < hi[1]; s[1]++)
			for (s[2] = lo[2]; s[2] < hi[2]; s[2]++) {
				uint32_t c = vpo_flatten3(w, s);
				uint32_t n = svl_items[c][lod];
				if (!n) continue;
				uint32_t start = 0;
				for (int k = 0; k < lod; k++) start += svl_items[c][k];
				memcpy(out + total, svl[c] + start, (size_t)n * sizeof(int16_t));
				total += n;
			}
	return total;
}

/* Drop every decoded chunk (the reference compresses idle chunks again,
 * src/chunkset.c:298-306); the next access decodes from RLE. */
void vpo_world_drop_voxels(vpo_world *w)
{
	for (uint32_t c = 0; c < w->nchunks; c++) {
		free(w->vox[c]);
		w->vox[c] = NULL;
	}
}

/* chunkset_manage's per-chunk work (src/chunkset.c:251-505) for a list of
 * chunks, OpenMP-parallel over chunks like the reference (there: 4 threads,
 * 8 chunks per 5 ms tick; here: `nthreads` threads, no throttles). Each
 * chunk is opened (decoded on first use), meshed or masked + splatted, and
 * its output copied into an exact-size buffer, as the reference publishes
 * it. Returns the total number of output bytes produced. */
uint64_t vpo_rebuild(vpo_world *w, const uint32_t *chunks, uint32_t n, const uint8_t *make_mesh, int lod_max,
		     int nthreads)
{
	const size_t R = (size_t)w->R, S3 = (R + 1) * (R + 1) * (R + 1);
	size_t geom_cap = 0;
	for (int l = 0; l <= lod_max; l++) geom_cap += 4 * (((R >> l) + 1) * ((R >> l) + 1) * ((R >> l) + 1));
	uint64_t total = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : total)
	{
		int16_t *geom = NULL;
		int16_t *vbo = NULL;
		uint32_t *ibo = NULL;
		uint8_t *mask = (uint8_t *)malloc(S3), *work = (uint8_t *)malloc(S3);
#pragma omp for schedule(dynamic, 1)
		for (uint32_t k = 0; k < n; k++) {
			uint32_t c = chunks[k];
			vpo_world_voxels(w, c);
			if (make_mesh && make_mesh[c]) {
				if (!vbo) {
					vbo = (int16_t *)malloc(3 * R * R * R * 16 * sizeof(int16_t));
					ibo = (uint32_t *)malloc(3 * R * R * R * 6 * sizeof(uint32_t));
				}
				uint32_t nv = 0, ni = 0;
				vpo_make_mesh(w, c, vbo, &nv, ibo, &ni);
				int16_t *pv = (int16_t *)malloc((size_t)nv * sizeof(int16_t) + 1);
				uint32_t *pi = (uint32_t *)malloc((size_t)ni * sizeof(uint32_t) + 1);
				memcpy(pv, vbo, (size_t)nv * sizeof(int16_t));
				memcpy(pi, ibo, (size_t)ni * sizeof(uint32_t));
				total += (uint64_t)nv * 2 + (uint64_t)ni * 4;
				free(pv);
				free(pi);
			} else {
				if (!geom) geom = (int16_t *)malloc(geom_cap * sizeof(int16_t));
				uint32_t items[VPO_MAX_LEVELS];
				uint32_t t = vpo_chunk_splats(w, c, lod_max, geom, items, mask, work);
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

/* Bulk form of vpo_world_set_rle for every chunk: chunk c's stream is
 * pool[off[c] .. off[c] + len[c]). */
void vpo_world_set_pool(vpo_world *w, const uint32_t *pool, const uint64_t *off, const uint32_t *len)
{
	for (uint32_t c = 0; c < w->nchunks; c++) vpo_world_set_rle(w, c, pool + off[c], len[c]);
}

/* Parity check of a candidate rebuild (the checker of the tests): for each
 * of the n chunks in `chunks`, OpenMP over chunks, run the same per-chunk
 * sequence as vpo_rebuild (the reference's src/chunkset.c:337-459: mesh, or
 * mask + L0 splats + downsample/splat per level) and compare with the
 * candidate's output of chunk c: svl[svl_off[c] ..] with per-level counts
 * svl_items[c * 8 + l] (int16 items), or vbo[vbo_off[c] ..] / ibo[ibo_off[c]
 * ..] with vbo_items[c] / ibo_items[c]. A chunk whose status[c] is nonzero,
 * whose ranges fall outside the given arrays, or whose bytes differ is a
 * mismatch. Returns the number of mismatching chunks; the first bad_cap of
 * them (in no particular order) go to bad[]. */
uint32_t vpo_check_chunks(vpo_world *w, const uint32_t *chunks, uint32_t n, const uint8_t *make_mesh, int lod_max,
			  int nthreads, const int16_t *svl, uint64_t svl_len, const int16_t *vbo, uint64_t vbo_len,
			  const uint32_t *ibo, uint64_t ibo_len, const uint64_t *svl_off, const uint32_t *svl_items,
			  const uint64_t *vbo_off, const uint32_t *vbo_items, const uint64_t *ibo_off,
			  const uint32_t *ibo_items, const uint32_t *status, uint32_t *bad, uint32_t bad_cap)
{
	const size_t R = (size_t)w->R, S3 = (R + 1) * (R + 1) * (R + 1);
	size_t geom_cap = 16;
	for (int l = 0; l <= lod_max; l++) geom_cap += 4 * (((R >> l) + 1) * ((R >> l) + 1) * ((R >> l) + 1));
	uint32_t nbad = 0;
#pragma omp parallel num_threads(nthreads)
	{
		int16_t *geom = NULL, *v = NULL;
		uint32_t *ix = NULL;
		uint8_t *mask = (uint8_t *)malloc(S3), *work = (uint8_t *)malloc(S3);
#pragma omp for schedule(dynamic, 1)
		for (uint32_t k = 0; k < n; k++) {
			const uint32_t c = chunks[k];
			int ok = status[c] == 0;
			if (ok && make_mesh && make_mesh[c]) {
				if (!v) {
					v = (int16_t *)malloc(3 * R * R * R * 16 * sizeof(int16_t));
					ix = (uint32_t *)malloc(3 * R * R * R * 6 * sizeof(uint32_t));
				}
				uint32_t nv = 0, ni = 0;
				vpo_make_mesh(w, c, v, &nv, ix, &ni);
				ok = nv == vbo_items[c] && ni == ibo_items[c] && vbo_off[c] + nv <= vbo_len &&
				     ibo_off[c] + ni <= ibo_len &&
				     !memcmp(vbo + vbo_off[c], v, (size_t)nv * sizeof(int16_t)) &&
				     !memcmp(ibo + ibo_off[c], ix, (size_t)ni * sizeof(uint32_t));
			} else if (ok) {
				if (!geom) geom = (int16_t *)malloc(geom_cap * sizeof(int16_t));
				uint32_t items[VPO_MAX_LEVELS];
				const uint32_t t = vpo_chunk_splats(w, c, lod_max, geom, items, mask, work);
				for (int l = 0; l <= lod_max; l++) ok &= items[l] == svl_items[(size_t)c * 8 + l];
				ok = ok && svl_off[c] + t <= svl_len &&
				     !memcmp(svl + svl_off[c], geom, (size_t)t * sizeof(int16_t));
			}
			if (!ok) {
				uint32_t slot;
#pragma omp atomic capture
				slot = nbad++;
				if (slot < bad_cap) bad[slot] = c;
			}
		}
		free(geom);
		free(v);
		free(ix);
		free(mask);
		free(work);
	}
	return nbad;
}

/* ------------------------------------------------------------------ */
/* Draw culling and LOD selection                                      */
/* ------------------------------------------------------------------ */

/* gfx_fcull_extract_planes (src/gfx/fcull.c:20-35): six planes from the
 * column-major view-projection matrix, normalised by the length of their
 * normal (float products and sums, the square root in double). */
void vpo_fcull_extract_planes(const float *m, float *planes)
{
	int n = 0;
	for (int i = 0; i < 3; i++) {
		for (int j = 0; j < 4; j++) planes[n++] = m[3 + 4 * j] - m[4 * j + i];
		for (int j = 0; j < 4; j++) planes[n++] = m[3 + 4 * j] + m[4 * j + i];
	}
	for (int p = 0; p < 6; p++) {
		float *q = planes + 4 * p;
		const float len = (float)sqrt((double)(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]));
		for (int k = 0; k < 4; k++) q[k] /= len;
	}
}

/* gfx_fcull_visible (src/gfx/fcull.c:38-45) */
int vpo_fcull_visible(const float *planes, const float *loc, float radius)
{
	for (int p = 0; p < 6; p++) {
		const float *q = planes + 4 * p;
		if ((q[0] * loc[0]) + (q[1] * loc[1]) + (q[2] * loc[2]) + q[3] < -radius) return 0;
	}
	return 1;
}

static float cull_distance(const float *a, const float *b)
{
	const float d0 = b[0] - a[0], d1 = b[1] - a[1], d2 = b[2] - a[2];
	return sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
}

typedef struct {
	int root_bitw, max_bitw[3];
	const float *planes, *origin;
	const uint8_t *has_mesh;
	const uint32_t *const *svl_items;
	uint32_t *mesh_out, *n_mesh, *svl_out, *n_svl;
	uint64_t visits;
} cull_ctx;

/* octree_cull (src/game.c:319-395). Level 0 is always a leaf: the
 * reference recurses below it only for a camera exactly at a chunk centre,
 * with a wrapped level. */
static void octree_cull_rec(cull_ctx *c, int lod, uint32_t x, uint32_t y, uint32_t z)
{
	c->visits++;
	const uint32_t ws_root = (uint32_t)(1u << c->root_bitw) << lod;
	const uint32_t v[3] = {x, y, z};
	float center[3];
	for (int i = 0; i < 3; i++) center[i] = (float)(v[i] * ws_root + ws_root / 2);
	for (int i = 0; i < 3; i++)
		if ((v[i] << lod) >= (1u << c->max_bitw[i])) return;
	if (!vpo_fcull_visible(c->planes, center, (float)(ws_root * 0.85))) return;
	const float distance = cull_distance(c->origin, center);
	if (lod == 0 || distance > (float)(lod * 1024)) {
		uint32_t ob[3];
		for (int i = 0; i < 3; i++) ob[i] = (uint32_t)(c->max_bitw[i] - (lod < c->max_bitw[i] ? lod : c->max_bitw[i]));
		const uint32_t node = ((z << ob[1] | y) << ob[0]) | x;
		if (lod == 0) {
			const uint32_t idx = ((z << c->max_bitw[1] | y) << c->max_bitw[0]) | x;
			if (c->has_mesh[idx]) {
				c->mesh_out[(*c->n_mesh)++] = idx;
				return;
			}
		}
		if (!c->svl_items[lod][node]) return;
		c->svl_out[(*c->n_svl)++] = ((uint32_t)lod << 24) | node;
		return;
	}
	for (uint32_t nx = 0; nx < 2; nx++)
		for (uint32_t ny = 0; ny < 2; ny++)
			for (uint32_t nz = 0; nz < 2; nz++)
				octree_cull_rec(c, lod - 1, 2 * x + nx, 2 * y + ny, 2 * z + nz);
}

/* The draw-queue walk of src/game.c:517-524. */
uint64_t vpo_octree_cull(int root_bitw, const int max_bitw[3], const float *planes, const float *origin, int top,
			 const uint8_t *has_mesh, const uint32_t *const *svl_items, uint32_t *mesh_out,
			 uint32_t *n_mesh, uint32_t *svl_out, uint32_t *n_svl)
{
	cull_ctx c = {root_bitw, {max_bitw[0], max_bitw[1], max_bitw[2]}, planes, origin, has_mesh, svl_items,
		      mesh_out, n_mesh, svl_out, n_svl, 0};
	*n_mesh = *n_svl = 0;
	const uint32_t rx = ((1u << max_bitw[0]) >> top) + 1, ry = ((1u << max_bitw[1]) >> top) + 1,
		       rz = ((1u << max_bitw[2]) >> top) + 1;
	for (uint32_t x = 0; x < rx; x++)
		for (uint32_t y = 0; y < ry; y++)
			for (uint32_t z = 0; z < rz; z++) octree_cull_rec(&c, top, x, y, z);
	return c.visits;
}

/* make_mesh (src/game.c:612-625): chunk centre within 512 of the LOD origin. */
void vpo_mesh_flags(int root_bitw, const int max_bitw[3], const float *origin, uint8_t *make_mesh)
{
	const uint32_t R = 1u << root_bitw;
	const uint32_t n = 1u << (max_bitw[0] + max_bitw[1] + max_bitw[2]);
	for (uint32_t c = 0; c < n; c++) {
		const uint32_t v[3] = {c & ((1u << max_bitw[0]) - 1u), (c >> max_bitw[0]) & ((1u << max_bitw[1]) - 1u),
				       c >> (max_bitw[0] + max_bitw[1])};
		float center[3];
		for (int i = 0; i < 3; i++) center[i] = (float)((v[i] << root_bitw) + (R / 2));
		make_mesh[c] = cull_distance(center, origin) < 512;
	}
}

/* chunkset_edit_raycast_until_solid (src/chunkset/edit.c:248-314). Float
 * DDA; a step moves a coordinate through float, as the reference's
 * `coord += step` does. Stepping below 0 takes the float->unsigned
 * conversion of x86-64 (through a 64-bit signed integer, truncated to 32
 * bits), written out explicitly here so every host computes the same: 0 - 1
 * gives 0xFFFFFFFF, and 0xFFFFFFFF - 1 rounds to 2^32, which truncates to 0. */
uint8_t vpo_raycast(vpo_world *w, const float *origin, const float *vector, uint32_t *coord, int8_t *normal)
{
	float delta[3], next[3], step[3], t[3][3];
	normal[0] = normal[1] = normal[2] = 0;
	for (int i = 0; i < 3; i++) coord[i] = (uint32_t)(int)origin[i];
	for (int i = 0; i < 3; i++)
		for (int j = 0; j < 3; j++) t[i][j] = vector[j] / vector[i];
	for (int i = 0; i < 3; i++) {
		delta[i] = (float)sqrt((double)(t[i][0] * t[i][0] + t[i][1] * t[i][1] + t[i][2] * t[i][2]));
		if (vector[i] < 0) {
			step[i] = -1.0f;
			next[i] = (origin[i] - (float)coord[i]) * delta[i];
		} else {
			step[i] = 1.0f;
			next[i] = ((float)coord[i] + 1.0f - origin[i]) * delta[i];
		}
	}
	for (int loops = 4096; loops-- > 1;) {
		int side = 0;
		for (int j = 1; j < 3; j++)
			if (next[side] > next[j]) side = j;
		next[side] += delta[side];
		coord[side] = (uint32_t)(int64_t)((float)coord[side] + step[side]);
		const uint8_t v = vpo_world_read(w, coord);
		if (v > 0) {
			normal[side] = (-vector[side] > 0) ? 1 : -1;
			return v;
		}
	}
	return 0;
}

/* ------------------------------------------------------------------ */
/* Software rasteriser (resources/splat.*.glsl, resources/mesh.*.glsl) */
/* ------------------------------------------------------------------ */

/* row `row` of m (column-major) times v, summed left to right */
static float mv_row(const float *m, int row, const float *v)
{
	return ((m[row] * v[0] + m[4 + row] * v[1]) + m[8 + row] * v[2]) + m[12 + row] * v[3];
}

static void mat_vec(const float *m, const float *v, float *out)
{
	for (int i = 0; i < 4; i++) out[i] = mv_row(m, i, v);
}

static float signf_(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

static uint32_t to8(float c)
{
	c = fminf(fmaxf(c, 0.0f), 1.0f);
	return (uint32_t)(c * 255.0f + 0.5f);
}

static uint32_t float_bits(float f)
{
	uint32_t u;
	memcpy(&u, &f, 4);
	return u;
}

static void frame_put(uint64_t *frame, int width, int px, int py, float depth, const float rgb[3])
{
	const uint32_t rgba = to8(rgb[0]) | (to8(rgb[1]) << 8) | (to8(rgb[2]) << 16) | (255u << 24);
	const float d = depth < 0.0f ? 0.0f : depth;
	const uint64_t v = ((uint64_t)float_bits(d) << 32) | rgba;
	uint64_t *p = frame + (size_t)py * width + px;
	if (v < *p) *p = v;
}

/* fog (pow(max(d - 256 / far, 0.0001), 0.5) as a square root) and mix */
static void fog_mix(const float col[3], float depth, float far_plane, float out[3])
{
	const float fog_start = 256.0f / far_plane;
	const float fog = sqrtf(fmaxf(depth - fog_start, 0.0001f));
	const float fc[3] = {0.5f, 0.5f, 0.7f};
	for (int i = 0; i < 3; i++) out[i] = col[i] * (1.0f - fog) + fc[i] * fog;
}

void vpo_frame_clear(uint64_t *frame, int width, int height)
{
	const float bg[3] = {0.5f, 0.5f, 0.7f};
	const uint32_t rgba = to8(bg[0]) | (to8(bg[1]) << 8) | (to8(bg[2]) << 16) | (255u << 24);
	const uint64_t v = ((uint64_t)float_bits(1.0f) << 32) | rgba;
	for (size_t i = 0; i < (size_t)width * height; i++) frame[i] = v;
}

/* splat.vert.glsl:34-54 + point rasterisation + splat.frag.glsl:25-157 */
void vpo_draw_splats(const vpo_camera *cam, const int16_t *svl, uint64_t n, int lod_level, uint64_t *frame)
{
	const float lod = (float)(1 << lod_level);
	const float W = (float)cam->width, H = (float)cam->height;
	const float llen = sqrtf(1.0f + 1.0f);
	const float light[3] = {-1.0f / llen, 1.0f / llen, 0.0f / llen};
	for (uint64_t k = 0; k < n; k++) {
		const int16_t *sp = svl + 4 * k;
		const float a[4] = {(float)sp[0] + 0.5f * lod, (float)sp[1] + 0.5f * lod, (float)sp[2] + 0.5f * lod, 1.0f};
		float vv[4], clip[4];
		mat_vec(cam->view_translation, a, vv);
		mat_vec(cam->proj_view_rot, vv, clip);
		if (!(clip[3] > 0.0f) || fabsf(clip[0]) > clip[3] || fabsf(clip[1]) > clip[3] || fabsf(clip[2]) > clip[3])
			continue;
		const float ratio = W / H;
		const float reduce = fmaxf(fabsf(clip[0] * ratio / clip[3]), fabsf(clip[1] / clip[3])) + 0.03f;
		const float size = (H * 1.1f) / clip[2] * fmaxf(reduce, 1.0f);
		const float ps = fminf(fmaxf(size * lod, 1.0f), 64.0f);
		const float xw = (clip[0] / clip[3] * 0.5f + 0.5f) * W, yw = (clip[1] / clip[3] * 0.5f + 0.5f) * H;
		const int c = sp[3];
		const float shadow = (float)((c >> 6) & 1);
		const float f = fmaxf(0.7f, 1.0f - shadow);
		const float vcol[3] = {(float)((c >> 4) & 3) / 3.0f * f, (float)((c >> 2) & 3) / 3.0f * f,
				       (float)(c & 3) / 3.0f * f};
		int x0 = (int)ceilf(xw - ps * 0.5f - 0.5f), x1 = (int)ceilf(xw + ps * 0.5f - 0.5f) - 1;
		int y0 = (int)ceilf(yw - ps * 0.5f - 0.5f), y1 = (int)ceilf(yw + ps * 0.5f - 0.5f) - 1;
		if (x0 < 0) x0 = 0;
		if (y0 < 0) y0 = 0;
		if (x1 > cam->width - 1) x1 = cam->width - 1;
		if (y1 > cam->height - 1) y1 = cam->height - 1;
		for (int py = y0; py <= y1; py++)
			for (int px = x0; px <= x1; px++) {
				const float rc[4] = {((float)px + 0.5f) / W * 2.0f - 1.0f, ((float)py + 0.5f) / H * 2.0f - 1.0f,
						     -1.0f, 1.0f};
				float r4[4];
				mat_vec(cam->inv_proj_view_rot, rc, r4);
				const float rv[3] = {r4[0] / r4[3], r4[1] / r4[3], r4[2] / r4[3]};
				const float len = sqrtf((rv[0] * rv[0] + rv[1] * rv[1]) + rv[2] * rv[2]);
				const float ray[3] = {rv[0] / len, rv[1] / len, rv[2] / len};
				float tmin[3], tmax[3];
				for (int i = 0; i < 3; i++) {
					const float inv = 1.0f / ray[i];
					const float tb = (vv[i] - 0.5f * lod) * inv, tt = (vv[i] + 0.5f * lod) * inv;
					tmin[i] = fminf(tt, tb);
					tmax[i] = fmaxf(tt, tb);
				}
				const float t0 = fmaxf(fmaxf(tmin[0], tmin[1]), fmaxf(tmin[0], tmin[2]));
				const float t1 = fminf(fminf(tmax[0], tmax[1]), fminf(tmax[0], tmax[2]));
				if (!(t0 <= t1)) continue;
				const float depth = t0 / cam->far_plane;
				if (!(depth < 1.0f)) continue;
				float hit[3], habs[3];
				for (int i = 0; i < 3; i++) {
					hit[i] = vv[i] - ray[i] * t0;
					habs[i] = fabsf(hit[i]);
				}
				const float md = fmaxf(fmaxf(habs[0], habs[1]), habs[2]);
				float r[3];
				for (int i = 0; i < 3; i++) r[i] = -((habs[i] == md ? 1.0f : 0.0f) * signf_(hit[i]));
				const float s = signf_((r[0] * light[0] + r[1] * light[1]) + r[2] * light[2]);
				const float g = fmaxf(fmaxf(0.7f, shadow), s);
				const float col[3] = {vcol[0] * g, vcol[1] * g, vcol[2] * g};
				float out[3];
				fog_mix(col, depth, cam->far_plane, out);
				frame_put(frame, cam->width, px, py, depth, out);
			}
	}
}

typedef struct {
	float xw, yw, w;       /* window position, clip w */
	float depth, col[3], uv[2], nrm[3];
	int diamond;
} mesh_vert;

static void mesh_vertex(const vpo_camera *cam, const int16_t *v, mesh_vert *o, int *ok)
{
	static const float nlut[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
	static const float ulut[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
	const float a[4] = {(float)v[0], (float)v[1], (float)v[2], 1.0f};
	float clip[4], vt[4];
	mat_vec(cam->view_projection, a, clip);
	mat_vec(cam->view_translation, a, vt);
	*ok = clip[3] > 0.0f;
	o->w = clip[3];
	o->xw = (clip[0] / clip[3] * 0.5f + 0.5f) * (float)cam->width;
	o->yw = (clip[1] / clip[3] * 0.5f + 0.5f) * (float)cam->height;
	const float d = sqrtf(((vt[0] * vt[0] + vt[1] * vt[1]) + vt[2] * vt[2]) + vt[3] * vt[3]);
	o->depth = d / cam->far_plane;
	const float aow = 1.0f - fminf(d / 180.0f, 1.0f);
	const int c = v[3];
	const float shadow = (float)((c >> 13) & 1);
	const float ao = fminf((float)((c >> 6) & 3), 2.0f) / 12.0f;
	const float f = fmaxf(1.0f - shadow, 0.6f);
	const float g = 1.0f - ao * aow;
	o->col[0] = (float)((c >> 4) & 3) / 3.0f * f * g;
	o->col[1] = (float)((c >> 2) & 3) / 3.0f * f * g;
	o->col[2] = (float)(c & 3) / 3.0f * f * g;
	const int ni = (c >> 8) & 7;
	for (int i = 0; i < 3; i++) o->nrm[i] = ni < 6 ? nlut[ni][i] : 0.0f;
	o->uv[0] = ulut[(c >> 11) & 3][0];
	o->uv[1] = ulut[(c >> 11) & 3][1];
	o->diamond = (c >> 14) & 3;
}

/* edge (a -> b) owns pixel centres exactly on it when it is a top or left
 * edge of a counter-clockwise triangle (y up) */
static int top_left(float ax, float ay, float bx, float by)
{
	const float dx = bx - ax, dy = by - ay;
	return dy < 0.0f || (dy == 0.0f && dx < 0.0f);
}

static float edge_fn(float ax, float ay, float bx, float by, float px, float py)
{
	return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

/* mesh.vert.glsl + back-face culling + triangle rasterisation with
 * perspective-correct varyings + mesh.frag.glsl */
void vpo_draw_mesh(const vpo_camera *cam, const int16_t *vbo, const uint32_t *ibo, uint64_t nfaces, uint64_t *frame)
{
	for (uint64_t t = 0; t < 2 * nfaces; t++) {
		mesh_vert v[3];
		int ok = 1;
		for (int k = 0; k < 3; k++) {
			int okk;
			mesh_vertex(cam, vbo + 4 * (size_t)ibo[3 * t + k], &v[k], &okk);
			ok &= okk;
		}
		if (!ok) continue; /* a vertex behind the eye: the triangle is dropped */
		const float area = edge_fn(v[0].xw, v[0].yw, v[1].xw, v[1].yw, v[2].xw, v[2].yw);
		if (!(area > 0.0f)) continue; /* back-facing (GL_BACK, CCW front) or degenerate */
		float mnx = fminf(fminf(v[0].xw, v[1].xw), v[2].xw), mxx = fmaxf(fmaxf(v[0].xw, v[1].xw), v[2].xw);
		float mny = fminf(fminf(v[0].yw, v[1].yw), v[2].yw), mxy = fmaxf(fmaxf(v[0].yw, v[1].yw), v[2].yw);
		int x0 = (int)fmaxf(floorf(mnx), 0.0f), x1 = (int)fminf(ceilf(mxx), (float)(cam->width - 1));
		int y0 = (int)fmaxf(floorf(mny), 0.0f), y1 = (int)fminf(ceilf(mxy), (float)(cam->height - 1));
		const int tl0 = top_left(v[1].xw, v[1].yw, v[2].xw, v[2].yw);
		const int tl1 = top_left(v[2].xw, v[2].yw, v[0].xw, v[0].yw);
		const int tl2 = top_left(v[0].xw, v[0].yw, v[1].xw, v[1].yw);
		for (int py = y0; py <= y1; py++)
			for (int px = x0; px <= x1; px++) {
				const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
				const float e0 = edge_fn(v[1].xw, v[1].yw, v[2].xw, v[2].yw, fx, fy);
				const float e1 = edge_fn(v[2].xw, v[2].yw, v[0].xw, v[0].yw, fx, fy);
				const float e2 = edge_fn(v[0].xw, v[0].yw, v[1].xw, v[1].yw, fx, fy);
				if (!(e0 > 0.0f || (e0 == 0.0f && tl0)) || !(e1 > 0.0f || (e1 == 0.0f && tl1)) ||
				    !(e2 > 0.0f || (e2 == 0.0f && tl2)))
					continue;
				const float q0 = e0 / area / v[0].w, q1 = e1 / area / v[1].w, q2 = e2 / area / v[2].w;
				const float qs = (q0 + q1) + q2;
				const float b0 = q0 / qs, b1 = q1 / qs, b2 = q2 / qs;
#define INTERP(f) ((b0 * v[0].f + b1 * v[1].f) + b2 * v[2].f)
				const float depth = INTERP(depth);
				if (!(depth < 1.0f)) continue;
				float col[3], uv[2], nrm[3];
				for (int i = 0; i < 3; i++) {
					col[i] = INTERP(col[i]);
					nrm[i] = INTERP(nrm[i]);
				}
				uv[0] = INTERP(uv[0]);
				uv[1] = INTERP(uv[1]);
#undef INTERP
				float c2[3] = {col[0], col[1], col[2]};
				if (!((v[2].diamond >> (uv[0] < uv[1] ? 1 : 0)) & 1))
					for (int i = 0; i < 3; i++) c2[i] = col[i] * 0.6f;
				if (nrm[1] < -0.9f || nrm[0] > 0.9f)
					for (int i = 0; i < 3; i++) c2[i] = col[i] * 0.6f;
				float out[3];
				fog_mix(c2, depth, cam->far_plane, out);
				frame_put(frame, cam->width, px, py, depth, out);
			}
	}
}
