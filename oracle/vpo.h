/*
 * oracle/vpo.h — CPU restatement of voxplat's per-chunk geometry pipeline.
 *
 * TEST INFRASTRUCTURE ONLY. This is the parity oracle: tests, the smoke
 * check and the benchmark's CPU-baseline leg call it to check or time the
 * CUDA path. The product never links it.
 *
 * Each function restates one reference function (file:line in
 * kosshi-net/voxplat 0.11) in plain scalar C. The restatement is pinned
 * against the unmodified reference sources, compiled by oracle/build_ref.sh
 * into oracle/_ref/, through golden fixtures under tests/golden/.
 *
 * Conventions that make the reference's undefined corners deterministic (the
 * same conventions hold on the GPU):
 *   - the shadow map is zero padded after its last row, and a read at an
 *     index at or past the padded length returns 0;
 *   - a chunk's +x/+y/+z neighbour past the world edge is all air (the
 *     reference's null chunk, src/chunkset/mesher.c:391-402);
 *   - chunk_make_mask's early-out (src/chunkset/mesher.c:404-409), which
 *     reads an uninitialised neighbour copy, is not taken: the full face
 *     scan runs, which is what the early-out is meant to be equivalent to.
 */
#ifndef VPO_H
#define VPO_H

#define VPO_MAX_LEVELS 8

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vpo_world {
	int root_bitw, R;
	int max_bitw[3], max[3];
	uint32_t nchunks;
	uint32_t **rle;      /* per chunk: owned stream incl. terminator */
	uint32_t *rle_len;   /* words incl. terminator */
	uint8_t **vox;       /* per chunk: decoded voxels, filled lazily */
	uint16_t *shadow;    /* padded map */
	uint64_t shadow_len; /* padded length in elements */
	uint32_t shadow_w;   /* X + Y world extent */
	uint32_t shadow_z;
} vpo_world;

/* rle.c */
uint32_t vpo_rle_encode(const uint8_t *vox, uint32_t n, uint32_t *out);
uint32_t vpo_rle_decode(const uint32_t *words, uint8_t *out, uint32_t cap);

/* world state */
vpo_world *vpo_world_new(int root_bitw, const int max_bitw[3], uint32_t pad_rows);
void vpo_world_free(vpo_world *w);
void vpo_world_set_rle(vpo_world *w, uint32_t chunk, const uint32_t *words, uint32_t n);
void vpo_world_set_shadow(vpo_world *w, const uint16_t *map, uint64_t n);
const uint8_t *vpo_world_voxels(vpo_world *w, uint32_t chunk);
void vpo_world_compress(vpo_world *w, uint32_t chunk);
uint32_t vpo_flatten3(const vpo_world *w, const uint32_t cv[3]);
uint8_t vpo_world_read(vpo_world *w, const uint32_t ws[3]);

/* shadow.h */
int vpo_shadow_sample(const vpo_world *w, const uint32_t ws[3]);
int vpo_shadow_sample_normal(const vpo_world *w, const uint32_t ws[3]);
void vpo_shadow_place_update(vpo_world *w, const uint32_t ws[3]);

/* mesher.c */
void vpo_make_mask(vpo_world *w, uint32_t chunk, uint8_t *mask);
void vpo_mask_downsample(int R, int level, const uint8_t *mask, uint8_t *work);
uint32_t vpo_make_splatlist(vpo_world *w, uint32_t chunk, int level, const uint8_t *mask,
			    int16_t *geom);
void vpo_make_mesh(vpo_world *w, uint32_t chunk, int16_t *vbo, uint32_t *vbo_items,
		   uint32_t *ibo, uint32_t *ibo_items);

/* chunkset.c:367-459 splat sequence: mask, L0, then downsample + splat per
 * level up to lod_max. Returns total int16 items; per-level counts in items.
 * `mask` and `work` are (R+1)^3 bytes of caller scratch. */
uint32_t vpo_chunk_splats(vpo_world *w, uint32_t chunk, int lod_max, int16_t *geom,
			  uint32_t *items, uint8_t *mask, uint8_t *work);

/* edit.c:179-244 sphere edit; marks dirty[c] = 1 for every chunk in the
 * edit's AABB (dirty may be NULL). Returns the number of such chunks. */
uint32_t vpo_edit_sphere(vpo_world *w, const int32_t ws[3], uint32_t radius, uint8_t voxel,
			 uint8_t *dirty);

/* vsplat.c:209-331 grouping: concatenation of LOD-`lod` segments of the
 * member chunks of octree node `node`. seg_off/seg_items give, per chunk, the
 * int16 offset and item count of that chunk's level-`lod` segment in `svl`
 * (segment pointers may differ per chunk, so svl is an array of pointers).
 * Returns int16 items written. */
uint64_t vpo_group_node(const vpo_world *w, int lod, const uint32_t node[3],
			int16_t *const *svl, const uint32_t *const *svl_items, int16_t *out);

/* Timed CPU baseline: the reference's per-chunk mesher work for `chunks`,
 * OpenMP over chunks; returns output bytes. */
void vpo_world_drop_voxels(vpo_world *w);

/* Draw culling and LOD selection (src/gfx/fcull.c, src/game.c:319-395,
 * 517-524, 612-625). */
void vpo_fcull_extract_planes(const float *m, float *planes);
int vpo_fcull_visible(const float *planes, const float *loc, float radius);
/* Octree walk from LOD `top` over the roots (x, y, z) < (max >> top) + 1,
 * x outer: chunks whose mesh is drawn go to mesh_out (chunk index), octree
 * nodes whose grouped splats are drawn to svl_out (lod << 24 | node index).
 * has_mesh[c] and svl_items[lod][node] describe the uploaded geometry.
 * Returns the number of nodes visited. */
uint64_t vpo_octree_cull(int root_bitw, const int max_bitw[3], const float *planes, const float *origin, int top,
			 const uint8_t *has_mesh, const uint32_t *const *svl_items, uint32_t *mesh_out,
			 uint32_t *n_mesh, uint32_t *svl_out, uint32_t *n_svl);
/* chunkset_edit_raycast_until_solid (src/chunkset/edit.c:248-314): the
 * first solid voxel along the ray (0 if none within 4095 steps), its
 * coordinates and the normal of the face entered (normal zeroed first). */
uint8_t vpo_raycast(vpo_world *w, const float *origin, const float *vector, uint32_t *coord, int8_t *normal);
/* Software rasteriser of the splat and mesh shaders (resources/splat.vert.glsl,
 * splat.frag.glsl, mesh.vert.glsl, mesh.frag.glsl), the semantics the CUDA
 * rasteriser implements. Matrices are column-major float[16]. The frame is
 * width x height packed words, (depth bits << 32) | RGBA8, initialised by
 * vpo_frame_clear; a fragment keeps the minimum (GL_LESS; equal depths keep
 * the smaller colour word). */
typedef struct vpo_camera {
	float projection[16], view_rotation[16], view_translation[16];
	float view_projection[16];   /* projection x view_rotation x view_translation */
	float inv_proj_view_rot[16]; /* inverse of projection x view_rotation */
	float proj_view_rot[16];     /* projection x view_rotation */
	float far_plane;
	int width, height;
} vpo_camera;
void vpo_frame_clear(uint64_t *frame, int width, int height);
/* n splats (4 int16 each) drawn with u_lod = 2^lod */
void vpo_draw_splats(const vpo_camera *cam, const int16_t *svl, uint64_t n, int lod, uint64_t *frame);
/* nfaces quads: 16 int16 of vertices and 6 u32 indices (relative to the
 * chunk's vertices) per face */
void vpo_draw_mesh(const vpo_camera *cam, const int16_t *vbo, const uint32_t *ibo, uint64_t nfaces, uint64_t *frame);
/* make_mesh per chunk: distance from the chunk centre to origin < 512. */
void vpo_mesh_flags(int root_bitw, const int max_bitw[3], const float *origin, uint8_t *make_mesh);
uint64_t vpo_rebuild(vpo_world *w, const uint32_t *chunks, uint32_t n, const uint8_t *make_mesh, int lod_max,
		     int nthreads);
/* every chunk's stream at once: chunk c = pool[off[c] .. off[c] + len[c]) */
void vpo_world_set_pool(vpo_world *w, const uint32_t *pool, const uint64_t *off, const uint32_t *len);
/* Parity check of a candidate rebuild's outputs against vpo_rebuild's
 * per-chunk sequence, OpenMP over the listed chunks; returns the number of
 * mismatching chunks and lists up to bad_cap of them. */
uint32_t vpo_check_chunks(vpo_world *w, const uint32_t *chunks, uint32_t n, const uint8_t *make_mesh, int lod_max,
			  int nthreads, const int16_t *svl, uint64_t svl_len, const int16_t *vbo, uint64_t vbo_len,
			  const uint32_t *ibo, uint64_t ibo_len, const uint64_t *svl_off, const uint32_t *svl_items,
			  const uint64_t *vbo_off, const uint32_t *vbo_items, const uint64_t *ibo_off,
			  const uint32_t *ibo_items, const uint32_t *status, uint32_t *bad, uint32_t bad_cap);

#ifdef __cplusplus
}
#endif
#endif
