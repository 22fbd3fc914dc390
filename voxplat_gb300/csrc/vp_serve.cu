/*
 * vp_serve.cu — world edits and the edit-serving loop.
 *
 * An edit batch (edits applied in arrival order, src/chunkset/edit.c:
 * 179-244 per edit) runs entirely on the device:
 *   1. every chunk in any edit's AABB list (the reference marks exactly
 *      these dirty, edit.c:241-242) is decoded into a volume (tile-parallel:
 *      many CTAs per chunk, so a few long streams still fill the GPU);
 *   2. one k_edit launch per edit, in order (voxels + shadow rows);
 *   3. the volumes are re-encoded (rle_compress, tile-parallel) and appended
 *      at the pool's tail, and the chunks' stream offsets are redirected;
 *   4. the dirty chunks' shells are rewritten and their geometry rebuilt
 *      (mesh or splats by their mode), appended to the output arenas; the
 *      chunk records point at the new geometry.
 * The serving loop (vp_world_serve) replays a timed edit trace: edits that
 * arrive while a batch is on the GPU queue up; when the GPU is free the
 * queued edits (up to max_batch, and as many as the free-HBM budget
 * admits) form the next batch. Latency = batch completion - arrival.
 */
#include "vp_edit.h"
#include "vp_internal.h"
#include "vp_rle.h"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace {

constexpr uint32_t kMaxListPerEdit = 1024; /* the reference's list[1024], edit.c:195 */
constexpr uint32_t kMaxRadius = 250;        /* one shadow row segment fits 1 KiB */

double now_s()
{
	using clk = std::chrono::steady_clock;
	return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

/* chunkset_get_chunks_in_aabb (edit.c:89-126): x outer, y, z inner */
void aabb_chunks(const vp_world *w, const vp_edit &e, std::vector<EditChunk> &out)
{
	const int rb = w->root_bitw;
	int32_t mn[3] = {e.x - (int32_t)e.radius - 1, e.y - (int32_t)e.radius - 1, e.z - (int32_t)e.radius - 1};
	int32_t mx[3] = {e.x + (int32_t)e.radius + 1, e.y + (int32_t)e.radius + 1, e.z + (int32_t)e.radius + 1};
	int32_t lo[3], hi[3];
	for (int i = 0; i < 3; i++) {
		lo[i] = mn[i] >> rb;
		hi[i] = mx[i] >> rb;
	}
	uint32_t n = 0;
	for (int32_t x = lo[0]; x <= hi[0]; x++)
		for (int32_t y = lo[1]; y <= hi[1]; y++)
			for (int32_t z = lo[2]; z <= hi[2]; z++) {
				if (x < 0 || y < 0 || z < 0 || x >= (1 << w->max_bitw[0]) || y >= (1 << w->max_bitw[1]) ||
				    z >= (1 << w->max_bitw[2]))
					continue;
				if (n++ >= kMaxListPerEdit - 1) continue;
				EditChunk c;
				c.cv[0] = x;
				c.cv[1] = y;
				c.cv[2] = z;
				c.vol_slot = 0;
				out.push_back(c);
			}
}

uint32_t chunk_of(const vp_world *w, const EditChunk &c)
{
	return (((uint32_t)c.cv[2] << w->max_bitw[1] | (uint32_t)c.cv[1]) << w->max_bitw[0]) | (uint32_t)c.cv[0];
}

template <typename T>
int grow(T **p, size_t &cap, size_t need)
{
	if (need <= cap && *p) return VP_OK;
	dev_free(*p);
	cap = 0;
	const size_t n = std::max(need, (size_t)64) + need / 2;
	int rc = dev_alloc(p, n);
	if (rc) return rc;
	cap = n;
	return VP_OK;
}

/* Copy the live streams into a fresh pool with new headroom (one copy
 * kernel; the old pool is freed afterwards). */
int compact_pool(vp_world *w, uint64_t extra_words)
{
	cudaStream_t st = w->ctx->stream;
	std::vector<uint32_t> len(w->nchunks);
	CK(cudaMemcpyAsync(len.data(), w->d_len, w->nchunks * 4u, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	std::vector<uint64_t> noff(w->nchunks);
	uint64_t total = 0;
	for (uint32_t c = 0; c < w->nchunks; c++) {
		noff[c] = total;
		total += (len[c] + 3u) & ~3u;
	}
	const uint64_t cap = total + total / 4 + extra_words + (16u << 20);
	uint32_t *np = nullptr;
	uint64_t *d_noff = nullptr;
	int rc = dev_alloc(&np, cap);
	if (!rc) rc = dev_alloc(&d_noff, w->nchunks);
	if (rc) {
		dev_free(np);
		return rc;
	}
	cudaError_t e = cudaMemcpyAsync(d_noff, noff.data(), w->nchunks * 8u, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = launch_copy_streams(w->d_pool, w->d_off, w->d_len, d_noff, np, w->nchunks, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(w->d_off, d_noff, w->nchunks * 8u, cudaMemcpyDeviceToDevice, st);
	w->pool_version++;
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	dev_free(d_noff);
	if (e != cudaSuccess) {
		dev_free(np);
		return cuda_fail(e, "pool compaction");
	}
	dev_free(w->d_pool);
	w->d_pool = np;
	w->pool_cap = cap;
	w->pool_tail = total;
	return vpi_upload_setdesc(w);
}

/* Bytes of device memory one batch over `dirty` chunks needs on top of
 * what the world holds: volumes, worst-case streams and the lists. */
uint64_t batch_bytes(const vp_world *w, size_t dirty, size_t listed)
{
	const uint64_t N = 1ull << (3 * w->root_bitw);
	return dirty * (N + 64u) + dirty * (N + 8u) * 4u + listed * sizeof(EditChunk);
}

int grow_arena_keep(vp_world *w, int a, uint64_t need_units)
{
	cudaStream_t st = w->ctx->stream;
	const uint64_t units = need_units + need_units / 2 + 1024;
	void *np = nullptr;
	cudaError_t e = cudaMalloc(&np, units * 16u);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(arena growth)");
	if (w->d_arena[a]) CK(cudaMemcpyAsync(np, w->d_arena[a], w->cap[a] * 16u, cudaMemcpyDeviceToDevice, st));
	CK(cudaStreamSynchronize(st));
	dev_free(w->d_arena[a]);
	w->d_arena[a] = np;
	w->cap[a] = units;
	return VP_OK;
}

/* Remesh the batch's dirty chunks (shells, then geometry appended to the
 * arenas), then queue the readback of the cursors. */
int enqueue_remesh(vp_world *w, uint32_t ndirty)
{
	cudaStream_t st = w->ctx->stream;
	GeoLaunch L;
	memset(&L, 0, sizeof(L));
	L.big_scratch = w->d_big;
	L.big_slots = w->big_slots;
	L.sets = w->d_set;
	L.threads = 512;
	L.outs = w->d_outs;
	L.lod_max = w->last_lod;
	Arena *ar[3] = {&L.svl, &L.vbo, &L.ibo};
	for (int a = 0; a < 3; a++) {
		ar[a]->base = w->d_arena[a];
		ar[a]->cap_units = w->cap[a];
		ar[a]->cursor = w->d_cursors + a;
	}
	GeoLaunch Ls = L;
	Ls.shell_items = w->d_edit_items;
	Ls.n_shell = ndirty;
	Ls.run_shell = 1;
	cudaError_t e = launch_geometry(w->root_bitw, Ls, st);
	if (e != cudaSuccess) return cuda_fail(e, "edit shell launch");
	GeoLaunch Lg = L;
	Lg.items = w->d_edit_items;
	Lg.n_items = ndirty;
	e = launch_geometry(w->root_bitw, Lg, st);
	if (e != cudaSuccess) return cuda_fail(e, "edit geometry launch");
	CK(cudaMemcpyAsync(w->h_pin + 2, w->d_cursors, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
	return VP_OK;
}

/* Queue one batch (edits in arrival order). */
int enqueue_batch(vp_world *w, const vp_edit *edits, uint32_t n)
{
	cudaStream_t st = w->ctx->stream;
	const uint32_t N = 1u << (3 * w->root_bitw);
	int rc;
	for (uint32_t i = 0; i < n; i++)
		if (edits[i].radius > kMaxRadius) return VP_EUNSUPPORTED;
	if (w->slot_of.size() != w->nchunks) w->slot_of.assign(w->nchunks, -1);
	std::vector<EditChunk> lists;
	std::vector<uint32_t> start(n + 1);
	std::vector<uint32_t> dirty;
	for (uint32_t i = 0; i < n; i++) {
		start[i] = (uint32_t)lists.size();
		aabb_chunks(w, edits[i], lists);
	}
	start[n] = (uint32_t)lists.size();
	for (auto &c : lists) {
		const uint32_t id = chunk_of(w, c);
		if (w->slot_of[id] < 0) {
			w->slot_of[id] = (int32_t)dirty.size();
			dirty.push_back(id);
		}
		c.vol_slot = (uint32_t)w->slot_of[id];
	}
	for (uint32_t id : dirty) w->slot_of[id] = -1;
	w->last_dirty = dirty;
	const uint32_t nd = (uint32_t)dirty.size();
	if (!nd) return VP_OK;
	/* room for the worst-case streams at the pool's tail */
	const uint64_t need_words = (uint64_t)nd * ((uint64_t)N + 8u);
	if (w->pool_tail + need_words > w->pool_cap)
		if ((rc = compact_pool(w, need_words))) return rc;
	size_t cap;
	cap = w->vols_cap;
	if ((rc = grow(&w->d_vols, cap, (size_t)nd * N + 16u))) return rc;
	w->vols_cap = cap;
	size_t ecap = w->edit_chunks_cap;
	EditChunk *dec = (EditChunk *)w->d_edit_chunks;
	if ((rc = grow(&dec, ecap, lists.size()))) return rc;
	w->d_edit_chunks = dec;
	w->edit_chunks_cap = ecap;
	if (nd > w->dirty_cap) {
		dev_free(w->d_dirty);
		dev_free(w->d_edit_items);
		dev_free(w->d_new_off);
		dev_free(w->d_new_len);
		w->dirty_cap = 0;
		const size_t m = nd + nd / 2 + 64;
		if ((rc = dev_alloc(&w->d_dirty, m)) || (rc = dev_alloc(&w->d_edit_items, m)) ||
		    (rc = dev_alloc(&w->d_new_off, m)) || (rc = dev_alloc(&w->d_new_len, m)))
			return rc;
		w->dirty_cap = m;
	}
	if (!w->d_edit_sc && (rc = dev_alloc(&w->d_edit_sc, 2))) return rc;
	{
		size_t c1 = w->tile_cap, c2 = w->nruns_cap, c3 = w->run_scratch_cap;
		if ((rc = grow(&w->d_tile_scratch, c1, (size_t)nd * (N / 4096u + 2u)))) return rc;
		if ((rc = grow(&w->d_nruns, c2, nd))) return rc;
		if ((rc = grow(&w->d_run_scratch, c3, (size_t)nd * (N + 1u)))) return rc;
		w->tile_cap = c1;
		w->nruns_cap = c2;
		w->run_scratch_cap = c3;
	}
	if (!w->h_pin) CK(cudaMallocHost((void **)&w->h_pin, 8 * sizeof(unsigned long long)));
	if (!w->edit_done) CK(cudaEventCreateWithFlags(&w->edit_done, cudaEventDisableTiming));
	if ((rc = vpi_ensure_arenas(w))) return rc;
	std::vector<WorkItem> items(nd);
	for (uint32_t k = 0; k < nd; k++) items[k] = WorkItem{0, dirty[k], w->modes[dirty[k]] ? kItemMesh : 0u, dirty[k]};
	CK(cudaMemcpyAsync(w->d_edit_chunks, lists.data(), lists.size() * sizeof(EditChunk), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(w->d_dirty, dirty.data(), nd * 4u, cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(w->d_edit_items, items.data(), nd * sizeof(WorkItem), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(w->d_edit_sc, 0, 2 * sizeof(unsigned long long), st));
	/* 1. decode */
	cudaError_t e = launch_rle_decode_tiles(w->d_pool, w->d_off, w->d_len, w->d_dirty, nd, N, w->d_vols,
						w->d_tile_scratch, st);
	if (e != cudaSuccess) return cuda_fail(e, "edit decode");
	/* 2. edits in order */
	for (uint32_t i = 0; i < n; i++) {
		EditDesc d;
		d.c[0] = edits[i].x;
		d.c[1] = edits[i].y;
		d.c[2] = edits[i].z;
		d.r = edits[i].radius;
		d.voxel = edits[i].voxel;
		d.nlist = start[i + 1] - start[i];
		e = launch_edit(d, (const EditChunk *)w->d_edit_chunks + start[i], d.nlist, w->d_vols, w->root_bitw,
				w->d_shadow, w->shadow_len, w->shadow_w, st);
		if (e != cudaSuccess) return cuda_fail(e, "edit launch");
	}
	/* 3. re-encode at the pool's tail and redirect the streams */
	e = launch_rle_encode_tiles(w->d_vols, nd, N, w->d_pool + w->pool_tail, w->pool_cap - w->pool_tail, w->d_edit_sc,
				    w->d_new_off, w->d_new_len, (uint32_t *)(w->d_edit_sc + 1), w->d_tile_scratch,
				    w->d_nruns, w->d_run_scratch, st);
	if (e == cudaSuccess)
		w->pool_version++;
		e = launch_scatter_streams(w->d_dirty, nd, w->d_new_off, w->d_new_len, w->pool_tail, w->d_off, w->d_len,
					   st);
	if (e != cudaSuccess) return cuda_fail(e, "edit re-encode");
	CK(cudaMemcpyAsync(w->h_pin, w->d_edit_sc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
	/* 4. remesh */
	if ((rc = enqueue_remesh(w, nd))) return rc;
	CK(cudaEventRecord(w->edit_done, st));
	w->pool_tail += need_words; /* reserved until the batch reports its size */
	w->launches += 2 * n + 4;
	return VP_OK;
}

/* After the batch's event: settle the pool tail, retry the remesh on arena
 * overflow. */
int finish_batch(vp_world *w)
{
	const uint32_t N = 1u << (3 * w->root_bitw);
	const uint32_t nd = (uint32_t)w->last_dirty.size();
	if (!nd) return VP_OK;
	CK(cudaEventSynchronize(w->edit_done));
	const uint64_t used = w->h_pin[0];
	const uint32_t status = (uint32_t)w->h_pin[1];
	w->pool_tail = w->pool_tail - (uint64_t)nd * ((uint64_t)N + 8u) + used;
	if (status & (kStatusOverflow | kStatusBadStream)) return VP_ECUDA;
	for (int attempt = 0; attempt < 3; attempt++) {
		bool grew = false;
		for (int a = 0; a < 3; a++) {
			if (w->h_pin[2 + a] <= w->cap[a]) continue;
			int rc = grow_arena_keep(w, a, w->h_pin[2 + a]);
			if (rc) return rc;
			grew = true;
		}
		if (!grew) return VP_OK;
		/* the chunks that did not fit wrote nothing: remesh the batch again
		 * behind the already used part of the arenas */
		int rc = enqueue_remesh(w, nd);
		if (rc) return rc;
		CK(cudaEventRecord(w->edit_done, w->ctx->stream));
		CK(cudaEventSynchronize(w->edit_done));
	}
	return VP_EOVERFLOW;
}

} // namespace

extern "C" {

VP_API int vp_world_edit(vp_world *w, const vp_edit *edits, uint32_t n)
{
	if (!w || (!edits && n) || !w->uploaded) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	int rc = vpi_pipe_drain(w);
	if (rc) return rc;
	rc = enqueue_batch(w, edits, n);
	if (!rc) rc = finish_batch(w);
	return rc;
}

VP_API int vp_world_chunk_rle(vp_world *w, uint32_t chunk, uint32_t *dst, uint32_t cap, uint32_t *n)
{
	if (!w || !n || chunk >= w->nchunks || !w->uploaded) return VP_EINVAL;
	cudaStream_t st = w->ctx->stream;
	uint64_t off = 0;
	uint32_t len = 0;
	CK(cudaMemcpyAsync(&off, w->d_off + chunk, 8, cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(&len, w->d_len + chunk, 4, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	*n = len;
	if (len > cap || !dst) return VP_EOVERFLOW;
	CK(cudaMemcpyAsync(dst, w->d_pool + off, len * 4u, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

VP_API int vp_world_rle_words(vp_world *w, uint64_t *words)
{
	if (!w || !words || !w->uploaded) return VP_EINVAL;
	std::vector<uint32_t> len(w->nchunks);
	CK(cudaMemcpyAsync(len.data(), w->d_len, w->nchunks * 4u, cudaMemcpyDeviceToHost, w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	uint64_t t = 0;
	for (uint32_t l : len) t += l;
	*words = t;
	return VP_OK;
}

VP_API int vp_world_read_shadow(vp_world *w, uint16_t *dst, uint64_t n)
{
	if (!w || !dst || n > w->shadow_len) return VP_EINVAL;
	CK(cudaMemcpyAsync(dst, w->d_shadow, n * 2u, cudaMemcpyDeviceToHost, w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	return VP_OK;
}

VP_API int vp_world_dirty(vp_world *w, uint32_t *chunks, uint32_t cap, uint32_t *n)
{
	if (!w || !n) return VP_EINVAL;
	*n = (uint32_t)w->last_dirty.size();
	if (chunks)
		for (uint32_t k = 0; k < *n && k < cap; k++) chunks[k] = w->last_dirty[k];
	return VP_OK;
}

VP_API int vp_world_serve(vp_world *w, const vp_edit *edits, uint32_t n, uint32_t max_batch, uint64_t hbm_reserve,
			  double *latency_ms, vp_serve_stats *stats)
{
	if (!w || (!edits && n) || !latency_ms || !stats || !w->uploaded || !max_batch) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	memset(stats, 0, sizeof(*stats));
	const int rc0 = vpi_pipe_drain(w);
	if (rc0) return rc0;
	std::vector<uint32_t> queue, batch;
	size_t qhead = 0;
	uint32_t next = 0, done = 0;
	bool inflight = false;
	double t_launch = 0;
	const double t0 = now_s();
	while (done < n) {
		const double now = now_s();
		while (next < n && edits[next].arrival_s <= now - t0) queue.push_back(next++);
		if (inflight) {
			if (cudaEventQuery(w->edit_done) == cudaSuccess) {
				const double t_done = now_s();
				int rc = finish_batch(w);
				if (rc) return rc;
				for (uint32_t i : batch) latency_ms[i] = (t_done - (t0 + edits[i].arrival_s)) * 1e3;
				stats->busy_s += t_done - t_launch;
				stats->chunks_remeshed += (uint32_t)w->last_dirty.size();
				done += (uint32_t)batch.size();
				inflight = false;
			}
			continue;
		}
		if (qhead == queue.size()) continue;
		/* admission: take queued edits while their chunks fit the free HBM
		 * left above the reserve */
		size_t free_b = 0, total_b = 0;
		if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return VP_ECUDA;
		batch.clear();
		std::vector<EditChunk> probe;
		while (qhead < queue.size() && batch.size() < max_batch) {
			probe.clear();
			for (uint32_t i : batch) aabb_chunks(w, edits[i], probe);
			aabb_chunks(w, edits[queue[qhead]], probe);
			const uint64_t need = batch_bytes(w, probe.size(), probe.size());
			if (need + hbm_reserve > free_b && !batch.empty()) break;
			if (need + hbm_reserve > free_b) {
				stats->deferred++;
				break;
			}
			batch.push_back(queue[qhead++]);
		}
		if (batch.empty()) continue; /* wait for memory to free up */
		std::vector<vp_edit> be(batch.size());
		for (size_t k = 0; k < batch.size(); k++) be[k] = edits[batch[k]];
		t_launch = now_s();
		int rc = enqueue_batch(w, be.data(), (uint32_t)be.size());
		if (rc) return rc;
		inflight = true;
		stats->batches++;
		stats->edits += (uint32_t)batch.size();
		if (batch.size() > stats->max_batch) stats->max_batch = (uint32_t)batch.size();
	}
	stats->wall_s = now_s() - t0;
	return VP_OK;
}

} // extern "C"
