/*
 * vp_worldgen.c — seeded synthetic worlds for tests and benchmarks (host C).
 * See vp_worldgen.h for the world definitions.
 */
#include "vp_worldgen.h"
#include "vp_noise.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RLE_COUNT_MAX 0xFFFFFFu

/* Run-length encode with the reference format (src/chunkset/rle.c:14-22,
 * 44-87): word = count | colour << 24, runs capped at 0xFFFFFF, then a 0
 * terminator. Returns words written. `out` holds n + 1 words at most. */
uint32_t vpg_rle_encode(const uint8_t *vox, uint32_t n, uint32_t *out)
{
	uint32_t b = 0, count = 1;
	uint8_t last = vox[0];
	for (uint32_t i = 1; i < n; i++) {
		if (vox[i] == last && count < RLE_COUNT_MAX) {
			count++;
		} else {
			out[b++] = count | ((uint32_t)last << 24);
			count = 1;
			last = vox[i];
		}
	}
	out[b++] = count | ((uint32_t)last << 24);
	out[b++] = 0;
	return b;
}

void vpg_chunk_voxels(const vpg_world *w, uint32_t chunk, uint8_t *out)
{
	const uint32_t *s = w->pool + w->off[chunk];
	uint64_t p = 0;
	for (uint32_t i = 0; s[i]; i++) {
		uint32_t cnt = s[i] & RLE_COUNT_MAX;
		memset(out + p, (int)(s[i] >> 24), cnt);
		p += cnt;
	}
}

static int pool_reserve(vpg_world *w, uint64_t extra)
{
	if (w->pool_words + extra <= w->pool_cap) return 0;
	uint64_t cap = w->pool_cap ? w->pool_cap : 1024;
	while (cap < w->pool_words + extra) cap *= 2;
	uint32_t *p = (uint32_t *)realloc(w->pool, cap * sizeof(uint32_t));
	if (!p) return -1;
	w->pool = p;
	w->pool_cap = cap;
	return 0;
}

/* Append a stream and pad the pool to the next 4-word boundary. */
static int pool_append(vpg_world *w, uint32_t c, const uint32_t *words, uint32_t n)
{
	uint32_t padded = (n + 3u) & ~3u;
	if (pool_reserve(w, padded)) return -1;
	memcpy(w->pool + w->pool_words, words, n * sizeof(uint32_t));
	memset(w->pool + w->pool_words + n, 0, (padded - n) * sizeof(uint32_t));
	w->off[c] = w->pool_words;
	w->len[c] = n;
	w->pool_words += padded;
	return 0;
}

int vpg_set_chunk_rle(vpg_world *w, uint32_t c, const uint32_t *words, uint32_t nwords)
{
	return pool_append(w, c, words, nwords);
}

int vpg_world_alloc(vpg_world *w, int root_bitw, const int max_bitw[3], uint32_t pad_rows)
{
	memset(w, 0, sizeof(*w));
	w->root_bitw = root_bitw;
	for (int i = 0; i < 3; i++) {
		w->max_bitw[i] = max_bitw[i];
		w->max[i] = 1 << max_bitw[i];
	}
	w->nchunks = (uint32_t)w->max[0] * w->max[1] * w->max[2];
	w->off = (uint64_t *)calloc(w->nchunks, sizeof(uint64_t));
	w->len = (uint32_t *)calloc(w->nchunks, sizeof(uint32_t));
	uint32_t R = 1u << root_bitw;
	/* shadow_init: width X + Y, depth Z (src/chunkset/shadow.h:26-43). */
	w->shadow_w = ((uint32_t)w->max[0] << root_bitw) + ((uint32_t)w->max[1] << root_bitw);
	w->shadow_z = (uint32_t)w->max[2] << root_bitw;
	w->shadow_len = (uint64_t)w->shadow_w * (w->shadow_z + pad_rows);
	w->shadow = (uint16_t *)calloc(w->shadow_len, sizeof(uint16_t));
	if (!w->off || !w->len || !w->shadow) return -1;
	/* Every chunk starts as the all-air stream {R^3, 0}. One shared copy. */
	uint32_t air[2] = {R * R * R, 0};
	if (pool_append(w, 0, air, 2)) return -1;
	for (uint32_t c = 1; c < w->nchunks; c++) {
		w->off[c] = w->off[0];
		w->len[c] = 2;
	}
	return 0;
}

void vpg_world_free(vpg_world *w)
{
	free(w->pool);
	free(w->off);
	free(w->len);
	free(w->shadow);
	memset(w, 0, sizeof(*w));
}

/* shadow_sample + shadow_place_update (src/chunkset/shadow.h:45-89) with
 * reads past the padded map returning 0. */
static void shadow_place(vpg_world *w, uint32_t x, uint32_t y, uint32_t z)
{
	uint32_t idx = (x + y) + w->shadow_w * z;
	uint32_t a = idx < w->shadow_len ? w->shadow[idx] : 0;
	uint32_t b = (uint64_t)idx + 1 < w->shadow_len ? w->shadow[idx + 1] : 0;
	if (!(a < y + 1 && b < y + 1)) return;
	if (idx < w->shadow_len) w->shadow[idx] = (uint16_t)y;
}

/* Build map rows [z0, z1) from a slab of decoded chunks covering those rows.
 * `slab[cy][cx]` points at the R^3 voxels of chunk (cx, cy, z0 >> R_b). */
static void shadow_rows(vpg_world *w, uint8_t **slab, uint32_t z0, uint32_t z1, int nthreads)
{
	const int rb = w->root_bitw;
	const uint32_t R = 1u << rb;
	(void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
	for (int64_t zz = z0; zz < (int64_t)z1; zz++) {
		uint32_t z = (uint32_t)zz, zl = z & (R - 1);
		for (int cy = 0; cy < w->max[1]; cy++)
			for (int cx = 0; cx < w->max[0]; cx++) {
				const uint8_t *v = slab[cy * w->max[0] + cx];
				if (!v) continue;
				for (uint32_t x = 0; x < R; x++)
					for (uint32_t y = 0; y < R; y++)
						if (v[x + R * (y + R * zl)])
							shadow_place(w, ((uint32_t)cx << rb) + x, ((uint32_t)cy << rb) + y, z);
			}
	}
}

typedef struct {
	int s;            /* cell size exponent */
	int x0, y0, z0;   /* first lattice index */
	int n;            /* lattice points per axis */
	uint16_t *v;
} lattice3;

static void lattice_init(lattice3 *L, uint64_t seed, int s, int ox, int oy, int oz, int R)
{
	L->s = s;
	L->x0 = ox >> s;
	L->y0 = oy >> s;
	L->z0 = oz >> s;
	L->n = ((R - 1) >> s) + 2 + 1;
	L->v = (uint16_t *)malloc((size_t)L->n * L->n * L->n * sizeof(uint16_t));
	for (int k = 0; k < L->n; k++)
		for (int j = 0; j < L->n; j++)
			for (int i = 0; i < L->n; i++)
				L->v[(k * L->n + j) * L->n + i] =
					(uint16_t)(vp_hash3(seed, L->x0 + i, L->y0 + j, L->z0 + k) & 0xFFFF);
}

/* Same arithmetic as vp_value3, with lattice values from the table. */
static inline int32_t lattice_eval(const lattice3 *L, int x, int y, int z)
{
	int s = L->s;
	int m = (1 << s) - 1;
	int i = (x >> s) - L->x0, j = (y >> s) - L->y0, k = (z >> s) - L->z0;
	int64_t wx = vp_smooth16((int64_t)(x & m) << (16 - s));
	int64_t wy = vp_smooth16((int64_t)(y & m) << (16 - s));
	int64_t wz = vp_smooth16((int64_t)(z & m) << (16 - s));
	const int n = L->n;
	int64_t c[2][2];
	for (int dz = 0; dz < 2; dz++)
		for (int dy = 0; dy < 2; dy++) {
			const uint16_t *row = L->v + ((k + dz) * n + (j + dy)) * n + i;
			c[dz][dy] = vp_lerp16(row[0], row[1], wx);
		}
	int64_t e0 = vp_lerp16(c[0][0], c[0][1], wy);
	int64_t e1 = vp_lerp16(c[1][0], c[1][1], wy);
	return (int32_t)vp_lerp16(e0, e1, wz);
}

#define CAVE_THRESHOLD 36045 /* 0.55 in 16-bit fixed point */

/* Fill one chunk of a terrain world; returns 1 if any voxel is solid. */
static int terrain_chunk(const vpg_world *w, int kind, uint64_t seed, int hshift,
			 int cx, int cy, int cz, uint8_t *vox, int32_t *hcol)
{
	const int rb = w->root_bitw, R = 1 << rb;
	const int ox = cx << rb, oy = cy << rb, oz = cz << rb;
	int any = 0, maxh = 0;
	for (int z = 0; z < R; z++)
		for (int x = 0; x < R; x++) {
			int X = ox + x, Z = oz + z, h;
			if (kind == VPG_TERRAIN_SMALL)
				h = 8 + (int)(((int64_t)vp_fractal2(seed, X, Z, 5 + hshift, 4) * 49) >> 16);
			else
				h = 40 + (int)(((int64_t)vp_fractal2(seed, X, Z, 8 + hshift, 6) * 161) >> 16);
			hcol[z * R + x] = h;
			if (h > maxh) maxh = h;
		}
	memset(vox, 0, (size_t)R * R * R);
	if (maxh <= oy) return 0;
	lattice3 L5 = {0}, L4 = {0};
	if (kind == VPG_TERRAIN_CAVES) {
		lattice_init(&L5, seed + 11, 5, ox, oy, oz, R);
		lattice_init(&L4, seed + 12, 4, ox, oy, oz, R);
	}
	for (int z = 0; z < R; z++)
		for (int x = 0; x < R; x++) {
			int X = ox + x, Z = oz + z, h = hcol[z * R + x];
			int top = h - oy;
			if (top <= 0) continue;
			if (top > R) top = R;
			uint8_t col_small = 0;
			int off = 0;
			if (kind == VPG_TERRAIN_SMALL)
				col_small = (uint8_t)(1 + h / 4 + (vp_hash3(seed ^ 0xC01u, X, 0, Z) & 3));
			else
				off = vp_value2(seed + 13, X, Z, 6) >> 12;
			for (int y = 0; y < top; y++) {
				int Y = oy + y;
				uint8_t c;
				if (kind == VPG_TERRAIN_SMALL) {
					c = col_small;
				} else {
					int32_t d = (2 * lattice_eval(&L5, X, Y, Z) + lattice_eval(&L4, X, Y, Z)) / 3;
					if (d > CAVE_THRESHOLD) continue;
					if (Y == h - 1)
						c = (uint8_t)(h < 120 ? 42 : 63);
					else
						c = (uint8_t)(1 + ((((Y + off) >> 4) * 23 + 7) % 62));
				}
				vox[x + R * (y + R * z)] = c;
				any = 1;
			}
		}
	free(L5.v);
	free(L4.v);
	return any;
}

int vpg_gen_terrain(vpg_world *w, int kind, uint64_t seed, int hshift, int nthreads)
{
	const int rb = w->root_bitw, R = 1 << rb;
	const size_t N = (size_t)R * R * R;
	const int sx = w->max[0], sy = w->max[1];
	const int per_slab = sx * sy;
#ifdef _OPENMP
	if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
	nthreads = 1;
#endif
	uint8_t **slab = (uint8_t **)calloc(per_slab, sizeof(uint8_t *));
	uint32_t **enc = (uint32_t **)calloc(per_slab, sizeof(uint32_t *));
	uint32_t *enc_n = (uint32_t *)calloc(per_slab, sizeof(uint32_t));
	if (!slab || !enc || !enc_n) return -1;
	int err = 0;
	for (int cz = 0; cz < w->max[2] && !err; cz++) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
		for (int i = 0; i < per_slab; i++) {
			int cx = i % sx, cy = i / sx;
			uint8_t *vox = (uint8_t *)malloc(N);
			int32_t *hcol = (int32_t *)malloc((size_t)R * R * sizeof(int32_t));
			int any = terrain_chunk(w, kind, seed, hshift, cx, cy, cz, vox, hcol);
			free(hcol);
			if (!any) {
				free(vox);
				slab[i] = NULL;
				enc[i] = NULL;
				continue;
			}
			uint32_t *e = (uint32_t *)malloc((N + 2) * sizeof(uint32_t));
			enc_n[i] = vpg_rle_encode(vox, (uint32_t)N, e);
			enc[i] = e;
			slab[i] = vox;
		}
		for (int i = 0; i < per_slab; i++) {
			if (!enc[i]) continue;
			uint32_t c = (uint32_t)(((cz << w->max_bitw[1]) | (i / sx)) << w->max_bitw[0] | (i % sx));
			if (pool_append(w, c, enc[i], enc_n[i])) err = -1;
			free(enc[i]);
			enc[i] = NULL;
		}
		shadow_rows(w, slab, (uint32_t)cz << rb, (uint32_t)(cz + 1) << rb, nthreads);
		for (int i = 0; i < per_slab; i++) {
			free(slab[i]);
			slab[i] = NULL;
		}
	}
	free(slab);
	free(enc);
	free(enc_n);
	return err;
}

/* round(1000 * 10^(j/64)) for j = 0..192: occupancy in ppm, log-uniform
 * between 0.1% and 100%. */
static const uint32_t pow10_ppm[193] = {
	1000, 1037, 1075, 1114, 1155, 1197, 1241, 1286, 1334, 1382, 1433, 1486, 1540, 1596, 1655,
	1715, 1778, 1843, 1911, 1981, 2054, 2129, 2207, 2288, 2371, 2458, 2548, 2642, 2738, 2839,
	2943, 3051, 3162, 3278, 3398, 3523, 3652, 3786, 3924, 4068, 4217, 4371, 4532, 4698, 4870,
	5048, 5233, 5425, 5623, 5829, 6043, 6264, 6494, 6732, 6978, 7234, 7499, 7774, 8058, 8354,
	8660, 8977, 9306, 9647, 10000, 10366, 10746, 11140, 11548, 11971, 12409, 12864, 13335,
	13824, 14330, 14855, 15399, 15963, 16548, 17154, 17783, 18434, 19110, 19810, 20535, 21288,
	22067, 22876, 23714, 24582, 25483, 26416, 27384, 28387, 29427, 30505, 31623, 32781, 33982,
	35227, 36517, 37855, 39242, 40679, 42170, 43714, 45316, 46976, 48697, 50481, 52330, 54247,
	56234, 58294, 60430, 62643, 64938, 67317, 69783, 72339, 74989, 77737, 80584, 83536, 86596,
	89769, 93057, 96466, 100000, 103663, 107461, 111397, 115478, 119709, 124094, 128640,
	133352, 138237, 143301, 148551, 153993, 159634, 165482, 171544, 177828, 184342, 191095,
	198096, 205353, 212875, 220673, 228757, 237137, 245824, 254830, 264165, 273842, 283874,
	294273, 305053, 316228, 327812, 339821, 352269, 365174, 378552, 392419, 406794, 421697,
	437144, 453158, 469759, 486968, 504807, 523299, 542469, 562341, 582942, 604296, 626434,
	649382, 673170, 697831, 723394, 749894, 777365, 805842, 835363, 865964, 897687, 930572,
	964662, 1000000};

int vpg_uneven_root_bitw(uint64_t seed, uint32_t k)
{
	uint32_t r = vp_hash3(seed, (int32_t)k, 0, 0x55) & 7;
	return r == 0 ? 5 : (r == 7 ? 7 : 6);
}

uint32_t vpg_uneven_occupancy_ppm(uint64_t seed, uint32_t k)
{
	return pow10_ppm[vp_hash3(seed, (int32_t)k, 1, 0x55) % 193];
}

int vpg_gen_uneven(vpg_world *w, uint64_t seed, uint32_t k)
{
	const int rb = w->root_bitw, R = 1 << rb;
	const uint32_t N = (uint32_t)R * R * R;
	const uint64_t p = vpg_uneven_occupancy_ppm(seed, k);
	/* Half of the target from blobs, the rest from uniform random voxels
	 * with probability q chosen so that both together reach p. */
	const uint64_t half = p / 2;
	const uint64_t q = half * 1000000ull / (1000000ull - half);
	const int nb = 1 + (int)(vp_hash3(seed, (int32_t)k, 2, 0x55) % 6);
	const uint64_t vb = (uint64_t)N * half / 1000000ull / (uint64_t)nb; /* per blob */
	int64_t r = 0;
	while ((uint64_t)(4189 * (r + 1) * (r + 1) * (r + 1) / 1000) <= vb) r++;
	int32_t bc[6][3];
	uint8_t bcol[6];
	for (int b = 0; b < nb; b++) {
		for (int a = 0; a < 3; a++)
			bc[b][a] = (int32_t)(vp_hash3(seed, (int32_t)k, 16 + b, a) & (uint32_t)(R - 1));
		bcol[b] = (uint8_t)(1 + vp_hash3(seed, (int32_t)k, 32 + b, 0) % 255);
	}
	uint8_t *vox = (uint8_t *)calloc(N, 1);
	uint32_t *e = (uint32_t *)malloc((N + 2) * sizeof(uint32_t));
	if (!vox || !e) return -1;
	for (int z = 0; z < R; z++)
		for (int y = 0; y < R; y++)
			for (int x = 0; x < R; x++) {
				uint8_t c = 0;
				uint32_t hsh = vp_hash3(seed ^ ((uint64_t)k << 20), x, y, z);
				if ((uint64_t)(hsh % 1000000u) < q) {
					c = (uint8_t)(1 + vp_hash3(seed + 77, (int32_t)k, x, y + (z << 8)) % 255);
				} else {
					for (int b = 0; b < nb; b++) {
						int64_t dx = x - bc[b][0], dy = y - bc[b][1], dz = z - bc[b][2];
						if (dx * dx + dy * dy + dz * dz < r * r) {
							c = bcol[b];
							break;
						}
					}
				}
				vox[x + R * (y + R * z)] = c;
			}
	uint32_t n = vpg_rle_encode(vox, N, e);
	int err = pool_append(w, 0, e, n);
	uint8_t *slab[1] = {vox};
	shadow_rows(w, slab, 0, (uint32_t)R, 1);
	free(vox);
	free(e);
	return err;
}
