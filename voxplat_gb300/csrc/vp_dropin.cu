/*
 * vp_dropin.cu — the reference's hot-path entry points (include/
 * voxgpu_dropin.h) on top of the device pipeline.
 *
 * Per-chunk calls (chunk_make_mask, chunk_make_mesh) build a small device
 * world around the chunk: a 4x4x4 set with the chunk at (1,1,1) and its
 * existing neighbours around it, each taken from the host ChunkMD as
 * decoded voxels (encoded on the device) or as its RLE stream, plus the
 * window of the host shadow map the chunk can read. The set's origin maps
 * it back to world coordinates, so emitted positions and shadow indices are
 * the reference's. chunk_mask_downsample and chunk_make_splatlist work on
 * the caller's dense mask arrays. chunkset_manage rebuilds every eligible
 * chunk of the set in one batched pass over a device mirror of the set and
 * publishes into the ChunkMD fields like src/chunkset.c:463-501.
 */
#include "voxgpu_dropin.h"
#include "vp_internal.h"
#include "vp_mask_kernels.h"
#include "vp_rle.h"

#include <cstdlib>
#include <cstring>
#include <mutex>

namespace {

std::mutex g_mu;
vp_ctx *g_ctx = nullptr;
int g_device = 0;
void *(*g_alloc)(size_t) = malloc;
void (*g_free)(void *) = free;
thread_local int g_err = VP_OK;

struct TempWorld {
	vp_world *w = nullptr;
	int root_bitw = -1;
};
TempWorld g_tmp;

/* mirror of a whole ChunkSet for chunkset_manage */
struct Mirror {
	vp_world *w = nullptr;
	const struct ChunkSet *set = nullptr;
};
Mirror g_mirror;

int ctx_get(vp_ctx **out)
{
	if (!g_ctx) {
		int rc = vp_ctx_create(g_device, &g_ctx);
		if (rc) return rc;
	}
	*out = g_ctx;
	return VP_OK;
}

uint32_t stream_words(const uint32_t *s)
{
	uint32_t n = 1;
	while (s[n]) n++;
	return n + 1;
}

/* The chunk's data as the reference reads it after chunk_open_ro
 * (src/chunkset.c:133-152): decoded voxels when present, else its RLE. */
VpiChunkSrc chunk_src(const struct ChunkSet *set, const struct ChunkMD *c)
{
	VpiChunkSrc s = {nullptr, nullptr, 0};
	if (c->voxels && !(set->null_chunk && c->voxels == set->null_chunk->voxels)) {
		s.bytes = c->voxels;
	} else if (c->rle && !(set->null_chunk && c->rle == set->null_chunk->rle)) {
		s.words = (const uint32_t *)c->rle;
		s.nwords = stream_words(s.words);
	}
	return s;
}

int tmp_world(int root_bitw, vp_world **out)
{
	if (g_tmp.w && g_tmp.root_bitw == root_bitw) {
		*out = g_tmp.w;
		return VP_OK;
	}
	vp_ctx *ctx;
	int rc = ctx_get(&ctx);
	if (rc) return rc;
	if (g_tmp.w) vp_world_destroy(g_tmp.w);
	g_tmp.w = nullptr;
	const int mb[3] = {2, 2, 2};
	rc = vp_world_create(ctx, root_bitw, mb, &g_tmp.w);
	if (rc) return rc;
	g_tmp.root_bitw = root_bitw;
	*out = g_tmp.w;
	return VP_OK;
}

uint32_t chunk_index(const struct ChunkSet *set, const uint16_t v[3])
{
	return ((uint32_t)v[2] << set->max_bitw[1] | v[1]) << set->max_bitw[0] | v[0];
}

/* Load the 4x4x4 neighbourhood of c (c at (1,1,1)) and, when `shadow` is
 * set, the window of the shadow map the chunk's mesh can read (rows z-1 ..
 * z+R+1 of the chunk's footprint). */
int load_neighbourhood(struct ChunkSet *set, struct ChunkMD *c, bool shadow, vp_world **out)
{
	vp_world *w;
	int rc = tmp_world(set->root_bitw, &w);
	if (rc) return rc;
	VpiChunkSrc src[64];
	memset(src, 0, sizeof(src));
	for (int dz = -1; dz <= 1; dz++)
		for (int dy = -1; dy <= 1; dy++)
			for (int dx = -1; dx <= 1; dx++) {
				const int d[3] = {dx, dy, dz};
				uint16_t v[3];
				bool inside = true;
				for (int i = 0; i < 3; i++) {
					const int t = (int)c->offset[i] + d[i];
					if (t < 0 || t >= (int)set->max[i]) inside = false;
					v[i] = (uint16_t)t;
				}
				if (!inside) continue;
				const struct ChunkMD *n = &set->chunks[chunk_index(set, v)];
				src[((dz + 1) * 4 + (dy + 1)) * 4 + (dx + 1)] = chunk_src(set, n);
			}
	if ((rc = vpi_world_load(w, src))) return rc;
	const uint64_t R = set->root, W = set->shadow_map_size[0];
	const uint64_t X = (uint64_t)c->offset[0] * R, Y = (uint64_t)c->offset[1] * R, Z = (uint64_t)c->offset[2] * R;
	const uint64_t base = W * Z + X + Y;
	uint64_t lo = base > 1 ? base - 1 : 0;
	uint64_t hi = W * (Z + R + 2) + X + Y + 2 * R + 4;
	if (!shadow) lo = hi = 0;
	const int32_t origin[3] = {(int32_t)c->offset[0] - 1, (int32_t)c->offset[1] - 1, (int32_t)c->offset[2] - 1};
	rc = vpi_world_shadow_window(w, set->shadow_map, set->shadow_map_length, lo, hi - lo, (uint32_t)W, origin);
	*out = w;
	return rc;
}

constexpr uint32_t kCenter = (1 * 4 + 1) * 4 + 1; /* (1,1,1) in the 4x4x4 set */

} // namespace

extern "C" {

VP_API void vp_dropin_set_allocator(void *(*alloc_fn)(size_t), void (*free_fn)(void *))
{
	std::lock_guard<std::mutex> lk(g_mu);
	g_alloc = alloc_fn ? alloc_fn : malloc;
	g_free = free_fn ? free_fn : free;
}

VP_API int vp_dropin_set_device(int device)
{
	std::lock_guard<std::mutex> lk(g_mu);
	if (g_ctx) return VP_EINVAL;
	g_device = device;
	return VP_OK;
}

VP_API int vp_dropin_last_error(void) { return g_err; }

VP_API void chunk_make_mask(struct ChunkSet *setp, struct ChunkMD *cp, uint8_t *mask)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_world *w;
	int rc = load_neighbourhood(setp, cp, false, &w);
	const size_t S = (size_t)setp->root + 1, S3 = S * S * S;
	if (!rc) rc = vpi_ensure_arenas(w);
	if (!rc && w->cap[0] * 16u < S3) rc = VP_ENOMEM;
	if (!rc) {
		cudaStream_t st = w->ctx->stream;
		cudaError_t e = cudaMemcpyAsync(w->d_arena[0], mask, S3, cudaMemcpyHostToDevice, st);
		const WorkItem it = {0, kCenter, kItemMaskDense, 0};
		if (e != cudaSuccess) rc = cuda_fail(e, "mask upload");
		if (!rc) rc = vpi_world_run(w, &it, 1, 0);
		if (!rc) {
			e = cudaMemcpyAsync(mask, w->d_arena[0], S3, cudaMemcpyDeviceToHost, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			if (e != cudaSuccess) rc = cuda_fail(e, "mask readback");
		}
	}
	g_err = rc;
}

VP_API void chunk_make_mesh(struct ChunkSet *setp, struct ChunkMD *cp, int16_t *geometry, uint32_t *geometry_items,
			    uint32_t *index, uint32_t *index_items)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_world *w;
	int rc = load_neighbourhood(setp, cp, true, &w);
	if (!rc) {
		const WorkItem it = {0, kCenter, kItemMesh, kCenter};
		rc = vpi_world_run(w, &it, 1, 0);
	}
	if (!rc) {
		vp_chunk_result r;
		cudaStream_t st = w->ctx->stream;
		cudaError_t e = cudaMemcpyAsync(&r, w->d_outs + kCenter, sizeof(r), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e == cudaSuccess && r.vbo_items)
			e = cudaMemcpyAsync(geometry, (const int16_t *)w->d_arena[1] + r.vbo_off, r.vbo_items * 2u,
					    cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess && r.ibo_items)
			e = cudaMemcpyAsync(index, (const uint32_t *)w->d_arena[2] + r.ibo_off, r.ibo_items * 4u,
					    cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e != cudaSuccess) {
			rc = cuda_fail(e, "mesh readback");
		} else {
			*geometry_items = r.vbo_items;
			*index_items = r.ibo_items;
		}
	}
	g_err = rc;
}

VP_API void chunk_mask_downsample(struct ChunkSet *setp, int8_t lod, Voxel *mask, Voxel *work)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_ctx *ctx;
	int rc = ctx_get(&ctx);
	const uint32_t S = (uint32_t)setp->root + 1u;
	const size_t S3 = (size_t)S * S * S;
	if (!rc && lod < 1) rc = VP_EINVAL;
	uint8_t *d = nullptr;
	if (!rc) rc = dev_alloc(&d, 2 * S3);
	if (!rc) {
		cudaStream_t st = ctx->stream;
		const uint32_t range = ((uint32_t)setp->root >> (lod - 1)) + 1u;
		cudaError_t e = cudaMemcpyAsync(d, mask, S3, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(d + S3, work, S3, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = launch_downsample(d, d + S3, S, range, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(work, d + S3, S3, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e != cudaSuccess) rc = cuda_fail(e, "downsample");
	}
	dev_free(d);
	g_err = rc;
}

VP_API void chunk_make_splatlist(struct ChunkSet *setp, struct ChunkMD *cp, uint8_t level, Voxel *mask,
				 int16_t *geometry, uint32_t *geometry_items)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_ctx *ctx;
	int rc = ctx_get(&ctx);
	const uint32_t R = setp->root, S = R + 1u;
	const size_t S3 = (size_t)S * S * S;
	const uint32_t range = (R >> level) + 1u;
	const size_t cap = (size_t)range * range * range;
	uint8_t *dmask = nullptr;
	int16_t *dout = nullptr;
	uint32_t *dcnt = nullptr;
	uint16_t *dmap = nullptr;
	if (!rc) rc = dev_alloc(&dmask, S3);
	if (!rc) rc = dev_alloc(&dout, cap * 4u);
	if (!rc) rc = dev_alloc(&dcnt, 1);
	/* the shadow rows the chunk's splats can read, as a window */
	const uint64_t W = setp->shadow_map_size[0];
	const uint64_t X = (uint64_t)cp->offset[0] * R, Y = (uint64_t)cp->offset[1] * R, Z = (uint64_t)cp->offset[2] * R;
	uint64_t lo = W * Z + X + Y;
	uint64_t hi = W * (Z + R + (1u << level) + 2) + X + Y + 2 * R + (2u << level) + 4;
	const uint64_t len = setp->shadow_map_length;
	if (lo > len) lo = len;
	if (hi > len) hi = len;
	if (!rc) rc = dev_alloc(&dmap, (size_t)(hi - lo) + 8u);
	if (!rc) {
		cudaStream_t st = ctx->stream;
		SetDesc sd;
		memset(&sd, 0, sizeof(sd));
		sd.shadow = dmap;
		sd.shadow_len = hi - lo;
		sd.shadow_base = lo;
		sd.shadow_w = (uint32_t)W;
		const uint32_t wb[3] = {(uint32_t)X, (uint32_t)Y, (uint32_t)Z};
		uint32_t n = 0;
		cudaError_t e = cudaMemcpyAsync(dmask, mask, S3, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess && hi > lo)
			e = cudaMemcpyAsync(dmap, setp->shadow_map + lo, (hi - lo) * 2u, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = launch_splatlist(dmask, S, range, level, wb, sd, dout, dcnt, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(&n, dcnt, 4, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e == cudaSuccess && n)
			e = cudaMemcpyAsync(geometry + *geometry_items, dout, (size_t)n * 8u, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e != cudaSuccess) {
			rc = cuda_fail(e, "splatlist");
		} else {
			/* the reference adds its running item index to the count
			 * (src/chunkset/mesher.c:510,533) */
			*geometry_items += *geometry_items + n * 4u;
		}
	}
	dev_free(dmask);
	dev_free(dout);
	dev_free(dcnt);
	dev_free(dmap);
	g_err = rc;
}

VP_API Voxel *rle_compress(Voxel *data, uint32_t length)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_ctx *ctx;
	int rc = ctx_get(&ctx);
	Voxel *out = nullptr;
	if (!rc) {
		uint32_t *tmp = (uint32_t *)malloc(((size_t)length + 2u) * sizeof(uint32_t));
		uint32_t n = 0;
		rc = tmp ? vp_rle_encode(ctx, data, length, tmp, length + 2u, &n) : VP_ENOMEM;
		if (!rc) {
			out = (Voxel *)g_alloc((size_t)n * sizeof(uint32_t));
			if (out)
				memcpy(out, tmp, (size_t)n * sizeof(uint32_t));
			else
				rc = VP_ENOMEM;
		}
		free(tmp);
	}
	g_err = rc;
	return out;
}

VP_API Voxel *rle_decompress(void *vdata)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_ctx *ctx;
	int rc = ctx_get(&ctx);
	Voxel *out = nullptr;
	if (!rc) {
		const uint32_t *s = (const uint32_t *)vdata;
		const uint32_t nw = stream_words(s);
		uint64_t total = 0;
		for (uint32_t i = 0; i + 1 < nw; i++) total += s[i] & 0xFFFFFFu;
		out = (Voxel *)g_alloc(total ? (size_t)total : 1u);
		uint32_t n = 0;
		if (!out)
			rc = VP_ENOMEM;
		else
			rc = vp_rle_decode(ctx, s, nw, out, (uint32_t)total, &n);
		if (rc && out) {
			g_free(out);
			out = nullptr;
		}
	}
	g_err = rc;
	return out;
}

VP_API void chunkset_manage(struct ChunkSet *set)
{
	std::lock_guard<std::mutex> lk(g_mu);
	vp_ctx *ctx;
	int rc = ctx_get(&ctx);
	if (rc) {
		g_err = rc;
		return;
	}
	if (g_mirror.set != set || !g_mirror.w || g_mirror.w->root_bitw != set->root_bitw) {
		if (g_mirror.w) vp_world_destroy(g_mirror.w);
		g_mirror.w = nullptr;
		const int mb[3] = {set->max_bitw[0], set->max_bitw[1], set->max_bitw[2]};
		rc = vp_world_create(ctx, set->root_bitw, mb, &g_mirror.w);
		if (rc) {
			g_err = rc;
			return;
		}
		g_mirror.set = set;
	}
	vp_world *w = g_mirror.w;
	/* gating of src/chunkset.c:281-313: skip chunks whose last geometry is
	 * not consumed yet; rebuild the ones with remesh or dirty set */
	std::vector<WorkItem> items;
	for (uint32_t i = 0; i < set->count; i++) {
		struct ChunkMD *c = &set->chunks[i];
		if (c->svl_dirty || c->mesh_dirty) continue;
		c->remesh = c->remesh | c->dirty;
		if (!c->remesh) continue;
		c->changing = c->dirty;
		c->dirty = 0;
		c->remesh = 0;
		items.push_back(WorkItem{0, i, c->make_mesh ? kItemMesh : 0u, i});
	}
	if (items.empty()) {
		g_err = VP_OK;
		return;
	}
	std::vector<VpiChunkSrc> src(set->count);
	for (uint32_t i = 0; i < set->count; i++) src[i] = chunk_src(set, &set->chunks[i]);
	rc = vpi_world_load(w, src.data());
	const int32_t origin[3] = {0, 0, 0};
	if (!rc)
		rc = vpi_world_shadow_window(w, set->shadow_map, set->shadow_map_length, 0, set->shadow_map_length,
					     set->shadow_map_size[0], origin);
	if (!rc) rc = vpi_world_run(w, items.data(), (uint32_t)items.size(), MAX_LOD_LEVEL - 1);
	std::vector<vp_chunk_result> res(set->count);
	if (!rc) rc = vp_world_results(w, res.data(), set->count);
	for (size_t k = 0; k < items.size() && !rc; k++) {
		struct ChunkMD *c = &set->chunks[items[k].chunk];
		const vp_chunk_result &r = res[items[k].chunk];
		if (items[k].flags & kItemMesh) {
			/* src/chunkset.c:347-366 */
			if (c->mesh_vbo) g_free(c->mesh_vbo);
			if (c->mesh_ibo) g_free(c->mesh_ibo);
			c->mesh_vbo_items = r.vbo_items;
			c->mesh_vbo = g_alloc((size_t)r.vbo_items * 2u + 1u);
			c->mesh_ibo_items = r.ibo_items;
			c->mesh_ibo = g_alloc((size_t)r.ibo_items * 4u + 1u);
			if (r.vbo_items) rc = vp_world_read_vbo(w, r.vbo_off, r.vbo_items, (int16_t *)c->mesh_vbo);
			if (!rc && r.ibo_items) rc = vp_world_read_ibo(w, r.ibo_off, r.ibo_items, (uint32_t *)c->mesh_ibo);
			c->no_geometry = !r.vbo_items;
			c->mesh_dirty = 1;
			if (c->no_geometry) {
				pthread_mutex_lock(&c->mutex_svl);
				if (c->svl) g_free(c->svl);
				c->svl = nullptr;
				memset(c->svl_items, 0, sizeof(c->svl_items));
				c->svl_items_total = 0;
				c->svl_dirty = 1;
				pthread_mutex_unlock(&c->mutex_svl);
			}
		} else {
			/* src/chunkset.c:463-501 */
			pthread_mutex_lock(&c->mutex_svl);
			c->no_geometry = !r.svl_total;
			if (c->svl) g_free(c->svl);
			c->svl = nullptr;
			if (!c->no_geometry) {
				for (int l = 0; l < MAX_LOD_LEVEL; l++) c->svl_items[l] = r.svl_items[l];
				c->svl = (uint16_t *)g_alloc((size_t)r.svl_total * 2u);
				rc = vp_world_read_svl(w, r.svl_off, r.svl_total, (int16_t *)c->svl);
				c->svl_items_total = r.svl_total;
			} else {
				memset(c->svl_items, 0, sizeof(c->svl_items));
				c->svl_items_total = 0;
			}
			c->svl_dirty = 1;
			pthread_mutex_unlock(&c->mutex_svl);
		}
		c->changing = 0;
	}
	g_err = rc;
}

} // extern "C"
