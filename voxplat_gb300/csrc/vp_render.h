/* vp_render.h — launch interface of the headless rasteriser. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

constexpr int kBlockFootprint = 256; /* pixels; larger footprints go to whole blocks */

struct RenderCam {
	float projection[16], view_rotation[16], view_translation[16];
	float view_projection[16];   /* projection x view_rotation x view_translation */
	float inv_proj_view_rot[16]; /* inverse of projection x view_rotation */
	float proj_view_rot[16];     /* projection x view_rotation */
	float far_plane;
	int width, height;
};

struct RenderSeg {
	uint64_t off;   /* int16 offset of a drawn node's splats in `splats` */
	uint32_t lod;
	uint32_t pad;
};

struct RenderMesh {
	uint64_t vbo_off, ibo_off; /* a drawn chunk's vertices (int16) and indices (u32) */
};

struct RenderArgs {
	RenderCam cam;
	float light[3];                 /* normalize(-1, 1, 0) */
	float fog_start;                /* 256 / far_plane (mesh.frag.glsl, splat.frag.glsl fog) */
	const int16_t *splats;     /* grouped lists of LOD >= 1 nodes */
	const int16_t *splats_l0;  /* the splat arena: LOD 0 nodes are chunks' level-0 segments */
	const RenderSeg *segs;
	const uint64_t *seg_first;      /* first splat of each segment */
	uint32_t nseg;
	uint64_t nsplats;
	const int16_t *vbo;
	const uint32_t *ibo;
	const RenderMesh *meshes;
	const uint64_t *mesh_first;     /* first triangle of each mesh */
	uint32_t nmesh;
	uint64_t ntris;
	unsigned long long *frame;      /* width x height, (depth << 32) | RGBA8 */
	/* per pixel, from the camera alone: the splat fragments' ray direction
	 * and its reciprocals, ray_a = (dx, dy, dz, 1/dx), ray_b = (1/dy, 1/dz) */
	float4 *ray_a;
	float2 *ray_b;
	uint64_t *big;                  /* [2][big_cap]: large splats, large triangles */
	uint32_t *big_count;            /* [2] */
	uint32_t big_cap;
};

/* Segments of the drawn queues: svl entries (lod << 24 | node) from the
 * grouped node tables, mesh chunks from the result records; totals[0] =
 * splats, totals[1] = triangles. */
cudaError_t launch_render_prep(const uint32_t *svl_q, uint32_t n_svl, const uint64_t *node_off,
			       const uint32_t *node_items, uint32_t nchunks, const uint32_t *mesh_q, uint32_t n_mesh,
			       const ChunkOut *outs, RenderSeg *segs, uint64_t *seg_first, RenderMesh *meshes,
			       uint64_t *mesh_first, uint64_t *totals, cudaStream_t st);
cudaError_t launch_render(const RenderArgs &a, uint32_t *rgba, float *depth, int sm_count, cudaStream_t st);

} // namespace vp
