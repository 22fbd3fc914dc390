/*
 * vp_render.cu — a headless CUDA rasteriser for the drawn octree nodes'
 * splats and the drawn chunks' meshes: a restatement of the reference's
 * shaders (resources/splat.vert.glsl:34-54, resources/splat.frag.glsl:25-157,
 * resources/mesh.vert.glsl, resources/mesh.frag.glsl) into a device frame.
 *
 * Semantics (the CPU restatement in the oracle computes the same bits):
 *   - splats: the vertex stage gives the point size, clamped to [1, 64]
 *     pixels; the point covers the pixel centres in [x - s/2, x + s/2) on both
 *     axes; each fragment casts the pixel's ray against the splat's box
 *     (slab test), shades by the box face it enters, fogs, and writes depth
 *     t0 / far;
 *   - meshes: triangles with a vertex behind the eye are dropped, back faces
 *     culled (counter-clockwise front), pixel centres inside (top-left rule
 *     on edges) get perspective-correct varyings, the diamond/normal darkening
 *     and fog; the provoking vertex is the last;
 *   - every fragment with depth < 1 keeps min((depth bits << 32) | RGBA8) in
 *     the frame word (GL_LESS; equal depths keep the smaller colour word), so
 *     the result does not depend on the order fragments arrive in;
 *   - float operations are rounded one by one in the shaders' order of
 *     evaluation; pow(x, 0.5) is evaluated as sqrt(x).
 * One thread per splat or triangle; footprints above 256 pixels go to a
 * list that whole blocks work through.
 */
#include "vp_render.h"

namespace vp {

__device__ __forceinline__ float mv_row(const float *m, int row, const float *v)
{
	return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[row], v[0]), __fmul_rn(m[4 + row], v[1])),
				   __fmul_rn(m[8 + row], v[2])),
			 __fmul_rn(m[12 + row], v[3]));
}

__device__ __forceinline__ void mat_vec(const float *m, const float *v, float *o)
{
	for (int i = 0; i < 4; i++) o[i] = mv_row(m, i, v);
}

__device__ __forceinline__ float signf_(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

__device__ __forceinline__ uint32_t to8(float c)
{
	c = fminf(fmaxf(c, 0.0f), 1.0f);
	return __float2uint_rz(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f));
}

__device__ __forceinline__ void frame_put(unsigned long long *frame, int width, int px, int py, float depth,
					  const float rgb[3])
{
	const uint32_t rgba = to8(rgb[0]) | (to8(rgb[1]) << 8) | (to8(rgb[2]) << 16) | (255u << 24);
	const float d = depth < 0.0f ? 0.0f : depth;
	const unsigned long long v = ((unsigned long long)__float_as_uint(d) << 32) | rgba;
	atomicMin(frame + (size_t)py * width + px, v);
}

/* fog_start = 256 / far, rounded once per frame on the host */
__device__ __forceinline__ void fog_mix(const float col[3], float depth, float fog_start, float out[3])
{
	const float fog = __fsqrt_rn(fmaxf(__fsub_rn(depth, fog_start), 0.0001f));
	const float fc[3] = {0.5f, 0.5f, 0.7f};
	for (int i = 0; i < 3; i++) out[i] = __fadd_rn(__fmul_rn(col[i], __fsub_rn(1.0f, fog)), __fmul_rn(fc[i], fog));
}

/* Clears the frame and fills the per-pixel ray table: the ray through the
 * pixel's centre (splat.frag.glsl's ray from the inverse projection and
 * rotation, normalised) and its reciprocals, the same for every splat. */
__global__ void k_frame_clear(RenderArgs a, uint64_t n)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float bg[3] = {0.5f, 0.5f, 0.7f};
	const uint32_t rgba = to8(bg[0]) | (to8(bg[1]) << 8) | (to8(bg[2]) << 16) | (255u << 24);
	a.frame[i] = ((unsigned long long)__float_as_uint(1.0f) << 32) | rgba;
	const int px = (int)(i % (uint64_t)a.cam.width), py = (int)(i / (uint64_t)a.cam.width);
	const float W = __int2float_rn(a.cam.width), H = __int2float_rn(a.cam.height);
	const float rc[4] = {__fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(__int2float_rn(px), 0.5f), W), 2.0f), 1.0f),
			     __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(__int2float_rn(py), 0.5f), H), 2.0f), 1.0f), -1.0f,
			     1.0f};
	float r4[4];
	mat_vec(a.cam.inv_proj_view_rot, rc, r4);
	const float rv[3] = {__fdiv_rn(r4[0], r4[3]), __fdiv_rn(r4[1], r4[3]), __fdiv_rn(r4[2], r4[3])};
	const float len =
		__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(rv[0], rv[0]), __fmul_rn(rv[1], rv[1])), __fmul_rn(rv[2], rv[2])));
	const float ray[3] = {__fdiv_rn(rv[0], len), __fdiv_rn(rv[1], len), __fdiv_rn(rv[2], len)};
	a.ray_a[i] = make_float4(ray[0], ray[1], ray[2], __fdiv_rn(1.0f, ray[0]));
	a.ray_b[i] = make_float2(__fdiv_rn(1.0f, ray[1]), __fdiv_rn(1.0f, ray[2]));
}

/* ---------------- splats ---------------- */

struct SplatSetup {
	float vv[3], vcol[3], shadow, lod;
	int x0, x1, y0, y1;
};

__device__ bool splat_setup(const RenderArgs &a, const int16_t *sp, float lod, SplatSetup &s)
{
	const float W = __int2float_rn(a.cam.width), H = __int2float_rn(a.cam.height);
	const float hl = __fmul_rn(0.5f, lod);
	const float p[4] = {__fadd_rn(__int2float_rn(sp[0]), hl), __fadd_rn(__int2float_rn(sp[1]), hl),
			    __fadd_rn(__int2float_rn(sp[2]), hl), 1.0f};
	float vv[4], clip[4];
	mat_vec(a.cam.view_translation, p, vv);
	mat_vec(a.cam.proj_view_rot, vv, clip);
	if (!(clip[3] > 0.0f) || fabsf(clip[0]) > clip[3] || fabsf(clip[1]) > clip[3] || fabsf(clip[2]) > clip[3])
		return false;
	const float ratio = __fdiv_rn(W, H);
	const float reduce = __fadd_rn(
		fmaxf(fabsf(__fdiv_rn(__fmul_rn(clip[0], ratio), clip[3])), fabsf(__fdiv_rn(clip[1], clip[3]))), 0.03f);
	const float size = __fmul_rn(__fdiv_rn(__fmul_rn(H, 1.1f), clip[2]), fmaxf(reduce, 1.0f));
	const float ps = fminf(fmaxf(__fmul_rn(size, lod), 1.0f), 64.0f);
	const float xw = __fmul_rn(__fadd_rn(__fmul_rn(__fdiv_rn(clip[0], clip[3]), 0.5f), 0.5f), W);
	const float yw = __fmul_rn(__fadd_rn(__fmul_rn(__fdiv_rn(clip[1], clip[3]), 0.5f), 0.5f), H);
	const float hp = __fmul_rn(ps, 0.5f);
	s.x0 = max(__float2int_rz(ceilf(__fsub_rn(__fsub_rn(xw, hp), 0.5f))), 0);
	s.x1 = min(__float2int_rz(ceilf(__fsub_rn(__fadd_rn(xw, hp), 0.5f))) - 1, a.cam.width - 1);
	s.y0 = max(__float2int_rz(ceilf(__fsub_rn(__fsub_rn(yw, hp), 0.5f))), 0);
	s.y1 = min(__float2int_rz(ceilf(__fsub_rn(__fadd_rn(yw, hp), 0.5f))) - 1, a.cam.height - 1);
	const int c = sp[3];
	s.shadow = __int2float_rn((c >> 6) & 1);
	const float f = fmaxf(0.7f, __fsub_rn(1.0f, s.shadow));
	s.vcol[0] = __fmul_rn(__fdiv_rn(__int2float_rn((c >> 4) & 3), 3.0f), f);
	s.vcol[1] = __fmul_rn(__fdiv_rn(__int2float_rn((c >> 2) & 3), 3.0f), f);
	s.vcol[2] = __fmul_rn(__fdiv_rn(__int2float_rn(c & 3), 3.0f), f);
	for (int i = 0; i < 3; i++) s.vv[i] = vv[i];
	s.lod = lod;
	return s.x0 <= s.x1 && s.y0 <= s.y1;
}

__device__ void splat_fragment(const RenderArgs &a, const SplatSetup &s, int px, int py)
{
	const size_t p = (size_t)py * a.cam.width + px;
	const float4 ra = a.ray_a[p];
	const float2 rb = a.ray_b[p];
	const float ray[3] = {ra.x, ra.y, ra.z}, inv[3] = {ra.w, rb.x, rb.y};
	const float hl = __fmul_rn(0.5f, s.lod);
	float tmin[3], tmax[3];
	for (int i = 0; i < 3; i++) {
		const float tb = __fmul_rn(__fsub_rn(s.vv[i], hl), inv[i]), tt = __fmul_rn(__fadd_rn(s.vv[i], hl), inv[i]);
		tmin[i] = fminf(tt, tb);
		tmax[i] = fmaxf(tt, tb);
	}
	const float t0 = fmaxf(fmaxf(tmin[0], tmin[1]), fmaxf(tmin[0], tmin[2]));
	const float t1 = fminf(fminf(tmax[0], tmax[1]), fminf(tmax[0], tmax[2]));
	if (!(t0 <= t1)) return;
	const float depth = __fdiv_rn(t0, a.cam.far_plane);
	if (!(depth < 1.0f)) return;
	float hit[3], habs[3];
	for (int i = 0; i < 3; i++) {
		hit[i] = __fsub_rn(s.vv[i], __fmul_rn(ray[i], t0));
		habs[i] = fabsf(hit[i]);
	}
	const float md = fmaxf(fmaxf(habs[0], habs[1]), habs[2]);
	float r[3];
	for (int i = 0; i < 3; i++) r[i] = -__fmul_rn(habs[i] == md ? 1.0f : 0.0f, signf_(hit[i]));
	const float s_ = signf_(__fadd_rn(__fadd_rn(__fmul_rn(r[0], a.light[0]), __fmul_rn(r[1], a.light[1])),
					  __fmul_rn(r[2], a.light[2])));
	const float g = fmaxf(fmaxf(0.7f, s.shadow), s_);
	const float col[3] = {__fmul_rn(s.vcol[0], g), __fmul_rn(s.vcol[1], g), __fmul_rn(s.vcol[2], g)};
	float out[3];
	fog_mix(col, depth, a.fog_start, out);
	frame_put(a.frame, a.cam.width, px, py, depth, out);
}

/* splat k of the drawn nodes: the node (segment) by binary search */
__device__ __forceinline__ const int16_t *splat_of(const RenderArgs &a, uint64_t k, float &lod)
{
	uint32_t lo = 0, hi = a.nseg;
	while (hi - lo > 1u) {
		const uint32_t mid = (lo + hi) >> 1;
		if (a.seg_first[mid] <= k) lo = mid;
		else hi = mid;
	}
	const RenderSeg sg = a.segs[lo];
	lod = __int2float_rn(1 << sg.lod);
	return (sg.lod ? a.splats : a.splats_l0) + sg.off + (k - a.seg_first[lo]) * 4u;
}

__global__ void __launch_bounds__(256) k_draw_splats(RenderArgs a)
{
	const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (k >= a.nsplats) return;
	float lod;
	const int16_t *sp = splat_of(a, k, lod);
	SplatSetup s;
	if (!splat_setup(a, sp, lod, s)) return;
	const int area = (s.x1 - s.x0 + 1) * (s.y1 - s.y0 + 1);
	if (area > kBlockFootprint) {
		const uint32_t slot = atomicAdd(a.big_count, 1u);
		if (slot < a.big_cap) a.big[slot] = k;
		return;
	}
	for (int py = s.y0; py <= s.y1; py++)
		for (int px = s.x0; px <= s.x1; px++) splat_fragment(a, s, px, py);
}

__global__ void __launch_bounds__(256) k_draw_splats_big(RenderArgs a)
{
	const uint32_t n = min(*a.big_count, a.big_cap);
	for (uint32_t b = blockIdx.x; b < n; b += gridDim.x) {
		float lod;
		const int16_t *sp = splat_of(a, a.big[b], lod);
		SplatSetup s;
		if (!splat_setup(a, sp, lod, s)) continue;
		const int w = s.x1 - s.x0 + 1, area = w * (s.y1 - s.y0 + 1);
		for (int i = threadIdx.x; i < area; i += blockDim.x) splat_fragment(a, s, s.x0 + i % w, s.y0 + i / w);
	}
}

/* ---------------- meshes ---------------- */

struct MeshVert {
	float xw, yw, w, depth, col[3], uv[2], nrm[3];
	int diamond;
};

/* The vertex stage in two parts: the window position, which decides
 * whether the triangle is drawn at all, and the varyings, computed only for
 * triangles that are. */
__device__ bool mesh_vertex_pos(const RenderArgs &a, const int16_t *v, MeshVert &o)
{
	const float a4[4] = {__int2float_rn(v[0]), __int2float_rn(v[1]), __int2float_rn(v[2]), 1.0f};
	float clip[4];
	mat_vec(a.cam.view_projection, a4, clip);
	o.w = clip[3];
	const float W = __int2float_rn(a.cam.width), H = __int2float_rn(a.cam.height);
	o.xw = __fmul_rn(__fadd_rn(__fmul_rn(__fdiv_rn(clip[0], clip[3]), 0.5f), 0.5f), W);
	o.yw = __fmul_rn(__fadd_rn(__fmul_rn(__fdiv_rn(clip[1], clip[3]), 0.5f), 0.5f), H);
	return clip[3] > 0.0f;
}

__device__ void mesh_vertex_attr(const RenderArgs &a, const int16_t *v, MeshVert &o)
{
	const float a4[4] = {__int2float_rn(v[0]), __int2float_rn(v[1]), __int2float_rn(v[2]), 1.0f};
	float vt[4];
	mat_vec(a.cam.view_translation, a4, vt);
	const float d = __fsqrt_rn(__fadd_rn(
		__fadd_rn(__fadd_rn(__fmul_rn(vt[0], vt[0]), __fmul_rn(vt[1], vt[1])), __fmul_rn(vt[2], vt[2])),
		__fmul_rn(vt[3], vt[3])));
	o.depth = __fdiv_rn(d, a.cam.far_plane);
	const float aow = __fsub_rn(1.0f, fminf(__fdiv_rn(d, 180.0f), 1.0f));
	const int c = v[3];
	const float shadow = __int2float_rn((c >> 13) & 1);
	const float ao = __fdiv_rn(fminf(__int2float_rn((c >> 6) & 3), 2.0f), 12.0f);
	const float f = fmaxf(__fsub_rn(1.0f, shadow), 0.6f);
	const float g = __fsub_rn(1.0f, __fmul_rn(ao, aow));
	o.col[0] = __fmul_rn(__fmul_rn(__fdiv_rn(__int2float_rn((c >> 4) & 3), 3.0f), f), g);
	o.col[1] = __fmul_rn(__fmul_rn(__fdiv_rn(__int2float_rn((c >> 2) & 3), 3.0f), f), g);
	o.col[2] = __fmul_rn(__fmul_rn(__fdiv_rn(__int2float_rn(c & 3), 3.0f), f), g);
	const int ni = (c >> 8) & 7;
	/* normal table (mesh.vert.glsl unpack_normal): +x, +y, +z, -x, -y, -z */
	for (int i = 0; i < 3; i++) o.nrm[i] = ni < 6 ? (ni % 3 == i ? (ni < 3 ? 1.0f : -1.0f) : 0.0f) : 0.0f;
	/* uv table (mesh.vert.glsl clut): (0,0) (1,0) (1,1) (0,1) */
	const int ui = (c >> 11) & 3;
	o.uv[0] = (ui == 1 || ui == 2) ? 1.0f : 0.0f;
	o.uv[1] = ui >= 2 ? 1.0f : 0.0f;
	o.diamond = (c >> 14) & 3;
}

__device__ __forceinline__ float edge_fn(float ax, float ay, float bx, float by, float px, float py)
{
	return __fsub_rn(__fmul_rn(__fsub_rn(bx, ax), __fsub_rn(py, ay)), __fmul_rn(__fsub_rn(by, ay), __fsub_rn(px, ax)));
}

__device__ __forceinline__ bool top_left(float ax, float ay, float bx, float by)
{
	const float dx = __fsub_rn(bx, ax), dy = __fsub_rn(by, ay);
	return dy < 0.0f || (dy == 0.0f && dx < 0.0f);
}

struct TriSetup {
	MeshVert v[3];
	float area;
	bool tl[3];
	int x0, x1, y0, y1;
};

/* triangle t of the drawn meshes: the chunk (segment) by binary search */
__device__ bool tri_setup(const RenderArgs &a, uint64_t t, TriSetup &s)
{
	uint32_t lo = 0, hi = a.nmesh;
	while (hi - lo > 1u) {
		const uint32_t mid = (lo + hi) >> 1;
		if (a.mesh_first[mid] <= t) lo = mid;
		else hi = mid;
	}
	const RenderMesh m = a.meshes[lo];
	const uint64_t local = t - a.mesh_first[lo];
	const uint32_t *ib = a.ibo + m.ibo_off + local * 3u;
	const int16_t *vb = a.vbo + m.vbo_off;
	const int16_t *vp[3];
	for (int k = 0; k < 3; k++) {
		vp[k] = vb + 4u * (size_t)ib[k];
		if (!mesh_vertex_pos(a, vp[k], s.v[k])) return false;
	}
	s.area = edge_fn(s.v[0].xw, s.v[0].yw, s.v[1].xw, s.v[1].yw, s.v[2].xw, s.v[2].yw);
	if (!(s.area > 0.0f)) return false;
	const float mnx = fminf(fminf(s.v[0].xw, s.v[1].xw), s.v[2].xw), mxx = fmaxf(fmaxf(s.v[0].xw, s.v[1].xw), s.v[2].xw);
	const float mny = fminf(fminf(s.v[0].yw, s.v[1].yw), s.v[2].yw), mxy = fmaxf(fmaxf(s.v[0].yw, s.v[1].yw), s.v[2].yw);
	/* clamp in float before converting: far-off vertices give huge boxes */
	s.x0 = __float2int_rz(fmaxf(floorf(mnx), 0.0f));
	s.x1 = __float2int_rz(fminf(ceilf(mxx), __int2float_rn(a.cam.width - 1)));
	s.y0 = __float2int_rz(fmaxf(floorf(mny), 0.0f));
	s.y1 = __float2int_rz(fminf(ceilf(mxy), __int2float_rn(a.cam.height - 1)));
	s.tl[0] = top_left(s.v[1].xw, s.v[1].yw, s.v[2].xw, s.v[2].yw);
	s.tl[1] = top_left(s.v[2].xw, s.v[2].yw, s.v[0].xw, s.v[0].yw);
	s.tl[2] = top_left(s.v[0].xw, s.v[0].yw, s.v[1].xw, s.v[1].yw);
	if (!(s.x0 <= s.x1 && s.y0 <= s.y1)) return false;
	for (int k = 0; k < 3; k++) mesh_vertex_attr(a, vp[k], s.v[k]);
	return true;
}

/* Whether the pixel centre (px, py) is inside the triangle (top-left rule
 * on edges), and its three edge values. */
__device__ __forceinline__ bool tri_inside(const TriSetup &s, int px, int py, float e[3])
{
	const MeshVert *v = s.v;
	const float fx = __fadd_rn(__int2float_rn(px), 0.5f), fy = __fadd_rn(__int2float_rn(py), 0.5f);
	e[0] = edge_fn(v[1].xw, v[1].yw, v[2].xw, v[2].yw, fx, fy);
	e[1] = edge_fn(v[2].xw, v[2].yw, v[0].xw, v[0].yw, fx, fy);
	e[2] = edge_fn(v[0].xw, v[0].yw, v[1].xw, v[1].yw, fx, fy);
	return (e[0] > 0.0f || (e[0] == 0.0f && s.tl[0])) && (e[1] > 0.0f || (e[1] == 0.0f && s.tl[1])) &&
	       (e[2] > 0.0f || (e[2] == 0.0f && s.tl[2]));
}

__device__ void tri_fragment(const RenderArgs &a, const TriSetup &s, int px, int py)
{
	const MeshVert *v = s.v;
	float e[3];
	if (!tri_inside(s, px, py, e)) return;
	const float e0 = e[0], e1 = e[1], e2 = e[2];
	const float q0 = __fdiv_rn(__fdiv_rn(e0, s.area), v[0].w);
	const float q1 = __fdiv_rn(__fdiv_rn(e1, s.area), v[1].w);
	const float q2 = __fdiv_rn(__fdiv_rn(e2, s.area), v[2].w);
	const float qs = __fadd_rn(__fadd_rn(q0, q1), q2);
	const float b0 = __fdiv_rn(q0, qs), b1 = __fdiv_rn(q1, qs), b2 = __fdiv_rn(q2, qs);
#define INTERP(f) __fadd_rn(__fadd_rn(__fmul_rn(b0, v[0].f), __fmul_rn(b1, v[1].f)), __fmul_rn(b2, v[2].f))
	const float depth = INTERP(depth);
	if (!(depth < 1.0f)) return;
	float col[3], nrm[3];
	for (int i = 0; i < 3; i++) {
		col[i] = INTERP(col[i]);
		nrm[i] = INTERP(nrm[i]);
	}
	const float u0 = INTERP(uv[0]), u1 = INTERP(uv[1]);
#undef INTERP
	float c2[3] = {col[0], col[1], col[2]};
	if (!((v[2].diamond >> (u0 < u1 ? 1 : 0)) & 1))
		for (int i = 0; i < 3; i++) c2[i] = __fmul_rn(col[i], 0.6f);
	if (nrm[1] < -0.9f || nrm[0] > 0.9f)
		for (int i = 0; i < 3; i++) c2[i] = __fmul_rn(col[i], 0.6f);
	float out[3];
	fog_mix(c2, depth, a.fog_start, out);
	frame_put(a.frame, a.cam.width, px, py, depth, out);
}

__global__ void __launch_bounds__(256) k_draw_tris(RenderArgs a)
{
	const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (t >= a.ntris) return;
	TriSetup s;
	if (!tri_setup(a, t, s)) return;
	const int64_t area = (int64_t)(s.x1 - s.x0 + 1) * (s.y1 - s.y0 + 1);
	if (area > kBlockFootprint) {
		const uint32_t slot = atomicAdd(a.big_count + 1, 1u);
		if (slot < a.big_cap) a.big[a.big_cap + slot] = t;
		return;
	}
	for (int py = s.y0; py <= s.y1; py++)
		for (int px = s.x0; px <= s.x1; px++) tri_fragment(a, s, px, py);
}

__global__ void __launch_bounds__(256) k_draw_tris_big(RenderArgs a)
{
	const uint32_t n = min(a.big_count[1], a.big_cap);
	for (uint32_t b = blockIdx.x; b < n; b += gridDim.x) {
		TriSetup s;
		if (!tri_setup(a, a.big[a.big_cap + b], s)) continue;
		const int w = s.x1 - s.x0 + 1;
		const int64_t area = (int64_t)w * (s.y1 - s.y0 + 1);
		for (int64_t i = threadIdx.x; i < area; i += blockDim.x)
			tri_fragment(a, s, s.x0 + (int)(i % w), s.y0 + (int)(i / w));
	}
}

__global__ void k_frame_resolve(const unsigned long long *frame, uint64_t n, uint32_t *rgba, float *depth)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= n) return;
	const unsigned long long v = frame[i];
	rgba[i] = (uint32_t)v;
	if (depth) depth[i] = __uint_as_float((uint32_t)(v >> 32));
}

cudaError_t launch_render(const RenderArgs &a, uint32_t *rgba, float *depth, int sm_count, cudaStream_t st)
{
	const uint64_t npx = (uint64_t)a.cam.width * a.cam.height;
	k_frame_clear<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(a, npx);
	cudaError_t e = cudaMemsetAsync(a.big_count, 0, 2 * sizeof(uint32_t), st);
	if (e != cudaSuccess) return e;
	if (a.ntris) {
		k_draw_tris<<<(unsigned)((a.ntris + 255) / 256), 256, 0, st>>>(a);
		k_draw_tris_big<<<sm_count * 4, 256, 0, st>>>(a);
	}
	if (a.nsplats) {
		k_draw_splats<<<(unsigned)((a.nsplats + 255) / 256), 256, 0, st>>>(a);
		k_draw_splats_big<<<sm_count * 4, 256, 0, st>>>(a);
	}
	k_frame_resolve<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(a.frame, npx, rgba, depth);
	return cudaGetLastError();
}

} // namespace vp

namespace vp {

/* block 0: splat segments of the drawn nodes; block 1: drawn meshes; each an
 * exclusive scan of the item counts in one CTA */
__global__ void __launch_bounds__(1024) k_render_prep(const uint32_t *__restrict__ svl_q, uint32_t n_svl,
						      const uint64_t *__restrict__ node_off,
						      const uint32_t *__restrict__ node_items, uint32_t nchunks,
						      const uint32_t *__restrict__ mesh_q, uint32_t n_mesh,
						      const ChunkOut *__restrict__ outs, RenderSeg *segs,
						      uint64_t *seg_first, RenderMesh *meshes, uint64_t *mesh_first,
						      uint64_t *totals)
{
	__shared__ unsigned long long wsum[32], wexcl[32], carry, tile;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const bool svl = blockIdx.x == 0;
	const uint32_t n = svl ? n_svl : n_mesh;
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	for (uint32_t b0 = 0; b0 < n; b0 += blockDim.x) {
		const uint32_t i = b0 + threadIdx.x;
		unsigned long long cnt = 0;
		if (i < n) {
			if (svl) {
				const uint32_t e = svl_q[i], l = e >> 24, node = e & 0xFFFFFFu;
				const size_t k = (size_t)l * nchunks + node;
				segs[i].off = node_off[k];
				segs[i].lod = l;
				segs[i].pad = 0;
				cnt = node_items[k] / 4u;
			} else {
				const ChunkOut o = outs[mesh_q[i]];
				meshes[i].vbo_off = o.vbo_off;
				meshes[i].ibo_off = o.ibo_off;
				cnt = (o.ibo_items / 6u) * 2u;
			}
		}
		unsigned long long inc = cnt;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const unsigned long long t = __shfl_up_sync(kFull, inc, d);
			if (lane >= d) inc += t;
		}
		if (lane == 31) wsum[warp] = inc;
		__syncthreads();
		if (warp == 0) {
			const unsigned long long w = lane < nw ? wsum[lane] : 0ull;
			unsigned long long wi = w;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const unsigned long long t = __shfl_up_sync(kFull, wi, d);
				if (lane >= d) wi += t;
			}
			wexcl[lane] = wi - w;
			if (lane == 31) tile = wi;
		}
		__syncthreads();
		if (i < n) (svl ? seg_first : mesh_first)[i] = carry + wexcl[warp] + inc - cnt;
		__syncthreads();
		if (threadIdx.x == 0) carry += tile;
		__syncthreads();
	}
	if (threadIdx.x == 0) totals[svl ? 0 : 1] = carry;
}

cudaError_t launch_render_prep(const uint32_t *svl_q, uint32_t n_svl, const uint64_t *node_off,
			       const uint32_t *node_items, uint32_t nchunks, const uint32_t *mesh_q, uint32_t n_mesh,
			       const ChunkOut *outs, RenderSeg *segs, uint64_t *seg_first, RenderMesh *meshes,
			       uint64_t *mesh_first, uint64_t *totals, cudaStream_t st)
{
	k_render_prep<<<2, 1024, 0, st>>>(svl_q, n_svl, node_off, node_items, nchunks, mesh_q, n_mesh, outs, segs,
					  seg_first, meshes, mesh_first, totals);
	return cudaGetLastError();
}

} // namespace vp
