/*
 * vp_serve.cu — world edits, the edit server and the edit-serving loop.
 *
 * An edit batch (edits applied in arrival order, src/chunkset/edit.c:
 * 179-244 per edit) runs entirely on the device, on one stream:
 *   1. every chunk in any edit's AABB list (the reference marks exactly
 *      these dirty, edit.c:241-242) is decoded into a volume (tile-parallel:
 *      many CTAs per chunk, so a few long streams still fill the GPU);
 *   2. one k_edit launch per edit, in order (voxels + shadow rows);
 *   3. the volumes are re-encoded (rle_compress, tile-parallel) and appended
 *      to the pool through a device-side tail cursor shared by every batch,
 *      and the chunks' stream offsets are redirected;
 *   4. the dirty chunks' shells are rewritten and their geometry rebuilt
 *      (mesh or splats by their mode), appended to the output arenas; the
 *      chunk records point at the new geometry.
 * A batch's buffers, stream and bookkeeping form an EditSlot. vp_world_edit
 * runs one batch on the context stream and waits for it.
 *
 * The edit server (vp_server) keeps several batches on the GPU at once, one
 * per slot, each on its own stream: the reference's flow of edit -> dirty ->
 * next mesher tick (src/chunkset.c:246-309, src/game.c:706-713) as a request
 * loop with continuous batching. Batches in flight are pairwise
 * independent: a batch is admitted only when none of its dirty chunks lies
 * within one chunk of an in-flight batch's dirty chunks (so neither reads
 * the other's voxels, shells or stream table entries) and the sun-shadow
 * map entries it writes (fills) or reads (its remesh, its fills' updates)
 * overlap nothing an in-flight batch writes, and vice versa. Independent
 * batches commute, so the result of every batch equals serial application
 * in submission order. A batch that would conflict waits at the head of the
 * queue until the batches it conflicts with have retired.
 */
#include "vp_edit.h"
#include "vp_internal.h"
#include "vp_rle.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <thread>

namespace {

constexpr uint32_t kMaxListPerEdit = 1024; /* the reference's list[1024], edit.c:195 */
constexpr uint32_t kMaxRadius = 250;        /* one shadow row segment fits 1 KiB */
constexpr uint32_t kMaxSlots = 8;

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
	uint64_t cap = total + total / 4 + extra_words + (16u << 20);
	uint32_t *np = nullptr;
	int rc;
	if (w->d_pool_spare && w->pool_spare_cap >= cap) {
		/* the spare pool holds it: no allocation */
		np = w->d_pool_spare;
		cap = w->pool_spare_cap;
		w->d_pool_spare = nullptr;
		w->pool_spare_cap = 0;
	} else if ((rc = dev_alloc(&np, cap))) {
		return rc;
	}
	if (!w->d_noff && (rc = dev_alloc(&w->d_noff, w->nchunks))) {
		dev_free(np);
		return rc;
	}
	cudaError_t e = cudaMemcpyAsync(w->d_noff, noff.data(), w->nchunks * 8u, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = launch_copy_streams(w->d_pool, w->d_off, w->d_len, w->d_noff, np, w->nchunks, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(w->d_off, w->d_noff, w->nchunks * 8u, cudaMemcpyDeviceToDevice, st);
	w->pool_version++;
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) {
		dev_free(np);
		return cuda_fail(e, "pool compaction");
	}
	/* the old pool is the next spare (a smaller one than the spare it
	 * replaces is freed) */
	if (w->pool_cap >= w->pool_spare_cap) {
		dev_free(w->d_pool_spare);
		w->d_pool_spare = w->d_pool;
		w->pool_spare_cap = w->pool_cap;
	} else {
		dev_free(w->d_pool);
	}
	w->d_pool = np;
	w->pool_cap = cap;
	w->pool_tail = total;
	return vpi_upload_setdesc(w);
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


/* A rectangle of sun-shadow map entries, u = x + y (column) by z (row),
 * inclusive bounds. */
struct Rect {
	int64_t u0, u1, z0, z1;
};

/* The map index is (u + W z) in uint32 arithmetic: a column past the row's
 * end is the next row's start and a negative column the previous row's end,
 * so such rectangles are split into the entries they really address. */
void add_rect(std::vector<Rect> &v, int64_t u0, int64_t u1, int64_t z0, int64_t z1, int64_t W)
{
	if (u0 < 0) {
		v.push_back(Rect{std::max<int64_t>(W + u0, 0), W - 1, z0 - 1, z1 - 1});
		u0 = 0;
	}
	if (u1 >= W) {
		v.push_back(Rect{0, std::min<int64_t>(u1 - W, W - 1), z0 + 1, z1 + 1});
		u1 = W - 1;
	}
	if (u0 <= u1) v.push_back(Rect{u0, u1, z0, z1});
}

bool overlaps(const std::vector<Rect> &a, const std::vector<Rect> &b)
{
	for (const Rect &p : a)
		for (const Rect &q : b)
			if (p.u0 <= q.u1 && q.u0 <= p.u1 && p.z0 <= q.z1 && q.z0 <= p.z1) return true;
	return false;
}

/* Shadow entries a fill edit reads and writes: rows [cz - r - 1, cz + r],
 * columns (x + y) over its AABB plus one (k_edit, shadow_place_update). */
void fill_rect(const vp_world *w, const vp_edit &e, std::vector<Rect> &v)
{
	if (!e.voxel) return;
	const int64_t r = e.radius;
	add_rect(v, (int64_t)e.x + e.y - 2 * r - 2, (int64_t)e.x + e.y + 2 * r + 2, (int64_t)e.z - r - 1, (int64_t)e.z + r,
		 (int64_t)w->shadow_w);
}

/* Shadow entries the remesh of chunk cv may sample: splat samples at the
 * chunk's cells plus 2^l, both entries of shadow_sample and the normal
 * variant's idx - 1, the mesh's diamond samples (src/chunkset/mesher.c:
 * 289-318, 497-536), with a margin. */
void remesh_rect(const vp_world *w, const int32_t cv[3], std::vector<Rect> &v)
{
	const int64_t R = 1 << w->root_bitw, m = 2 * (1 << std::max(w->last_lod, 0)) + 4;
	add_rect(v, R * (cv[0] + cv[1]) - 4, R * (cv[0] + cv[1]) + 2 * R + m, R * cv[2] - 4, R * cv[2] + R + m,
		 (int64_t)w->shadow_w);
}

} // namespace

/* One edit batch's device buffers, its stream and its bookkeeping. */
struct EditSlot {
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	cudaEvent_t done = nullptr;
	uint8_t *d_vols = nullptr;             /* decoded volumes of the batch's dirty chunks */
	size_t vols_cap = 0;                   /* bytes */
	EditChunk *d_lists = nullptr;          /* the edits' AABB chunk lists */
	size_t lists_cap = 0;
	uint32_t *d_dirty = nullptr;           /* dirty chunk ids */
	WorkItem *d_items = nullptr;
	uint64_t *d_new_off = nullptr;
	uint32_t *d_new_len = nullptr;
	size_t dirty_cap = 0;
	unsigned long long *d_status = nullptr; /* encoder status */
	uint32_t *d_tile = nullptr;            /* tile sums of the tile-parallel codec */
	size_t tile_cap = 0;
	uint32_t *d_nruns = nullptr;
	size_t nruns_cap = 0;
	uint32_t *d_runs = nullptr;            /* packed run starts while re-encoding */
	size_t runs_cap = 0;
	/* pinned: [0] pool tail after the encode, [1] encoder status, [2..4]
	 * arena cursors after the remesh, [5] the tail the batch starts from */
	unsigned long long *h_pin = nullptr;
	/* the batch on this slot */
	bool busy = false;
	uint32_t seq = 0;
	std::vector<uint32_t> dirty;
	std::vector<uint64_t> tickets;
	std::vector<double> submit_s;
	std::vector<uint32_t> near;            /* dirty chunks and their 26 neighbours, sorted */
	std::vector<Rect> sh_read, sh_write;   /* shadow entries the batch reads / writes */
	uint64_t worst_words = 0;              /* pool words the batch may append */
	double t_start = 0;
};

namespace {

int slot_init(EditSlot *s, cudaStream_t borrow)
{
	if (borrow) {
		s->stream = borrow;
	} else {
		CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
		s->own_stream = true;
	}
	CK(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming));
	CK(cudaMallocHost((void **)&s->h_pin, 8 * sizeof(unsigned long long)));
	return dev_alloc(&s->d_status, 2);
}

void slot_free(EditSlot *s)
{
	if (!s) return;
	if (s->stream) cudaStreamSynchronize(s->stream);
	dev_free(s->d_vols);
	dev_free(s->d_lists);
	dev_free(s->d_dirty);
	dev_free(s->d_items);
	dev_free(s->d_new_off);
	dev_free(s->d_new_len);
	dev_free(s->d_status);
	dev_free(s->d_tile);
	dev_free(s->d_nruns);
	dev_free(s->d_runs);
	if (s->h_pin) cudaFreeHost(s->h_pin);
	if (s->done) cudaEventDestroy(s->done);
	if (s->own_stream) cudaStreamDestroy(s->stream);
	delete s;
}

/* Buffers for nd dirty chunks and nlists AABB list entries (allocates:
 * only while no batch of this world is on the GPU, or at server creation). */
int slot_size(vp_world *w, EditSlot *s, size_t nd, size_t nlists)
{
	const size_t N = (size_t)1 << (3 * w->root_bitw);
	int rc;
	if ((rc = grow(&s->d_vols, s->vols_cap, nd * N + 16u))) return rc;
	if ((rc = grow(&s->d_lists, s->lists_cap, nlists))) return rc;
	if (nd > s->dirty_cap || !s->d_dirty) {
		dev_free(s->d_dirty);
		dev_free(s->d_items);
		dev_free(s->d_new_off);
		dev_free(s->d_new_len);
		s->dirty_cap = 0;
		const size_t m = nd + nd / 2 + 64;
		if ((rc = dev_alloc(&s->d_dirty, m)) || (rc = dev_alloc(&s->d_items, m)) ||
		    (rc = dev_alloc(&s->d_new_off, m)) || (rc = dev_alloc(&s->d_new_len, m)))
			return rc;
		s->dirty_cap = m;
	}
	if ((rc = grow(&s->d_tile, s->tile_cap, nd * (N / 4096u + 2u)))) return rc;
	if ((rc = grow(&s->d_nruns, s->nruns_cap, nd))) return rc;
	if ((rc = grow(&s->d_runs, s->runs_cap, nd * (N + 1u)))) return rc;
	return VP_OK;
}

/* Device bytes of a slot sized for nd dirty chunks and nlists list entries. */
uint64_t slot_bytes(const vp_world *w, size_t nd, size_t nlists)
{
	const uint64_t N = 1ull << (3 * w->root_bitw);
	const uint64_t m = nd + nd / 2 + 64, g = nd + nd / 2 + 64;
	return (nd * N + 16u) * 3 / 2 + nlists * sizeof(EditChunk) * 3 / 2 + m * (4 + sizeof(WorkItem) + 8 + 4) +
	       g * ((N / 4096u + 2u) * 4 + 4 + (N + 1u) * 4) * 3 / 2;
}

/* A batch's chunk lists: every edit's AABB list in the reference's order,
 * each entry pointing at its chunk's volume, and the distinct dirty chunks
 * in first-seen order. */
struct Plan {
	std::vector<EditChunk> lists;
	std::vector<uint32_t> start;
	std::vector<uint32_t> dirty;
};

void plan_batch(vp_world *w, const vp_edit *edits, uint32_t n, Plan &p)
{
	p.lists.clear();
	p.dirty.clear();
	p.start.assign(n + 1, 0);
	for (uint32_t i = 0; i < n; i++) {
		p.start[i] = (uint32_t)p.lists.size();
		aabb_chunks(w, edits[i], p.lists);
	}
	p.start[n] = (uint32_t)p.lists.size();
	std::vector<int32_t> &slot_of = w->slot_of;
	if (slot_of.size() != w->nchunks) slot_of.assign(w->nchunks, -1);
	for (auto &c : p.lists) {
		const uint32_t id = chunk_of(w, c);
		if (slot_of[id] < 0) {
			slot_of[id] = (int32_t)p.dirty.size();
			p.dirty.push_back(id);
		}
		c.vol_slot = (uint32_t)slot_of[id];
	}
	for (uint32_t id : p.dirty) slot_of[id] = -1;
}

/* Remesh the batch's dirty chunks on the slot's stream (shells, then
 * geometry appended to the arenas), then queue the readback of the arena
 * cursors. */
int enqueue_remesh(vp_world *w, EditSlot *s, uint32_t ndirty)
{
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
	Ls.shell_items = s->d_items;
	Ls.n_shell = ndirty;
	Ls.run_shell = 1;
	cudaError_t e = launch_geometry(w->root_bitw, Ls, s->stream);
	if (e != cudaSuccess) return cuda_fail(e, "edit shell launch");
	GeoLaunch Lg = L;
	Lg.items = s->d_items;
	Lg.n_items = ndirty;
	e = launch_geometry(w->root_bitw, Lg, s->stream);
	if (e != cudaSuccess) return cuda_fail(e, "edit geometry launch");
	CK(cudaMemcpyAsync(s->h_pin + 2, w->d_cursors, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
			   s->stream));
	return VP_OK;
}

/* Queue one batch on its slot (edits in arrival order). The slot's buffers
 * must hold the plan. With set_tail, the shared pool cursor is first set to
 * the host's pool tail (no other batch may be in flight then). */
int enqueue_batch(vp_world *w, EditSlot *s, const vp_edit *edits, uint32_t n, const Plan &p, bool set_tail)
{
	cudaStream_t st = s->stream;
	const uint32_t N = 1u << (3 * w->root_bitw);
	const uint32_t nd = (uint32_t)p.dirty.size();
	std::vector<WorkItem> items(nd);
	for (uint32_t k = 0; k < nd; k++)
		items[k] = WorkItem{0, p.dirty[k], w->modes[p.dirty[k]] ? kItemMesh : 0u, p.dirty[k]};
	CK(cudaMemcpyAsync(s->d_lists, p.lists.data(), p.lists.size() * sizeof(EditChunk), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(s->d_dirty, p.dirty.data(), nd * 4u, cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(s->d_items, items.data(), nd * sizeof(WorkItem), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(s->d_status, 0, 2 * sizeof(unsigned long long), st));
	if (set_tail) {
		s->h_pin[5] = w->pool_tail;
		CK(cudaMemcpyAsync(w->d_pool_cursor, s->h_pin + 5, sizeof(unsigned long long), cudaMemcpyHostToDevice, st));
	}
	/* 1. decode */
	cudaError_t e = launch_rle_decode_tiles(w->d_pool, w->d_off, w->d_len, s->d_dirty, nd, N, s->d_vols, s->d_tile, st);
	if (e != cudaSuccess) return cuda_fail(e, "edit decode");
	/* 2. edits in order */
	for (uint32_t i = 0; i < n; i++) {
		EditDesc d;
		d.c[0] = edits[i].x;
		d.c[1] = edits[i].y;
		d.c[2] = edits[i].z;
		d.r = edits[i].radius;
		d.voxel = edits[i].voxel;
		d.nlist = p.start[i + 1] - p.start[i];
		e = launch_edit(d, s->d_lists + p.start[i], d.nlist, s->d_vols, w->root_bitw, w->d_shadow, w->shadow_len,
				w->shadow_w, st);
		if (e != cudaSuccess) return cuda_fail(e, "edit launch");
	}
	/* 3. re-encode at the pool's tail (shared cursor) and redirect the streams */
	e = launch_rle_encode_tiles(s->d_vols, nd, N, w->d_pool, w->pool_cap, w->d_pool_cursor, s->d_new_off, s->d_new_len,
				    (uint32_t *)s->d_status, s->d_tile, s->d_nruns, s->d_runs, st);
	if (e == cudaSuccess) e = launch_scatter_streams(s->d_dirty, nd, s->d_new_off, s->d_new_len, 0, w->d_off, w->d_len, st);
	w->lens_stale = true; /* the full rebuilds' work orders follow the new lengths */
	if (e != cudaSuccess) return cuda_fail(e, "edit re-encode");
	w->pool_version++;
	CK(cudaMemcpyAsync(s->h_pin, w->d_pool_cursor, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(s->h_pin + 1, s->d_status, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
	/* 4. remesh */
	int rc = enqueue_remesh(w, s, nd);
	if (rc) return rc;
	CK(cudaEventRecord(s->done, st));
	s->dirty = p.dirty;
	w->launches += 2 * n + 6;
	return VP_OK;
}

/* Arena cursors past their capacity after a batch: grow the arenas (nothing
 * may be on the GPU) and remesh the batch again behind the used part. With
 * force the batch is remeshed even when the arenas have grown already (its
 * chunks overflowed against the capacity its remesh saw). */
int regrow_and_remesh(vp_world *w, EditSlot *s, bool force = false)
{
	for (int attempt = 0; attempt < 3; attempt++) {
		bool grew = false;
		for (int a = 0; a < 3; a++) {
			if (s->h_pin[2 + a] <= w->cap[a]) continue;
			int rc = grow_arena_keep(w, a, s->h_pin[2 + a]);
			if (rc) return rc;
			grew = true;
		}
		if (!grew && !force) return VP_OK;
		force = false;
		/* the chunks that did not fit wrote nothing: remesh them again */
		int rc = enqueue_remesh(w, s, (uint32_t)s->dirty.size());
		if (rc) return rc;
		CK(cudaEventRecord(s->done, s->stream));
		CK(cudaEventSynchronize(s->done));
	}
	return VP_EOVERFLOW;
}

bool arena_overflow(const vp_world *w, const EditSlot *s)
{
	for (int a = 0; a < 3; a++)
		if (s->h_pin[2 + a] > w->cap[a]) return true;
	return false;
}

int ensure_edit_state(vp_world *w)
{
	if (!w->d_pool_cursor) {
		int rc = dev_alloc(&w->d_pool_cursor, 1);
		if (rc) return rc;
	}
	if (!w->eslot) {
		EditSlot *s = new EditSlot();
		int rc = slot_init(s, w->ctx->stream);
		if (rc) {
			slot_free(s);
			return rc;
		}
		w->eslot = s;
	}
	return vpi_ensure_arenas(w);
}

uint64_t worst_words(const vp_world *w, size_t nd)
{
	return (uint64_t)nd * ((1ull << (3 * w->root_bitw)) + 8u);
}

} // namespace

/* ------------------------------------------------------------------ */
/* the edit server                                                     */
/* ------------------------------------------------------------------ */

struct vp_server {
	vp_world *w = nullptr;
	vp_server_config cfg = {};
	std::vector<EditSlot *> slots;
	struct Pending {
		uint64_t ticket;
		vp_edit e;
		double submit_s;
	};
	std::deque<Pending> queue;
	std::deque<vp_edit_done> done;
	uint64_t next_ticket = 0;
	uint32_t next_seq = 0;
	uint32_t inflight = 0;
	uint64_t tail_known = 0;   /* pool tail bound from retired batches */
	double t0 = 0, busy_since = 0, last_change = 0;
	bool held = false;         /* the queue head is waiting (counted once) */
	vp_serve_stats st = {};
	Plan plan;                 /* scratch */
	cudaEvent_t ctx_ev = nullptr; /* orders each batch after the world's own stream */
};

namespace {

double srv_now(const vp_server *s) { return now_s() - s->t0; }

void note_inflight(vp_server *s, int delta)
{
	const double t = srv_now(s);
	s->st.inflight_s += (double)s->inflight * (t - s->last_change);
	s->last_change = t;
	if (s->inflight == 0 && delta > 0) s->busy_since = t;
	s->inflight = (uint32_t)((int)s->inflight + delta);
	if (s->inflight == 0 && delta < 0) s->st.busy_s += t - s->busy_since;
	s->st.max_inflight = std::max(s->st.max_inflight, s->inflight);
}

/* Retire the slot's finished batch: pool tail, completions. Arena overflow
 * is handled by the caller (it needs the GPU idle). */
int retire(vp_server *s, EditSlot *sl)
{
	vp_world *w = s->w;
	const uint32_t status = (uint32_t)sl->h_pin[1];
	if (status & (kStatusOverflow | kStatusBadStream)) return VP_ECUDA;
	s->tail_known = std::max<uint64_t>(s->tail_known, sl->h_pin[0]);
	const double t = srv_now(s);
	for (size_t k = 0; k < sl->tickets.size(); k++)
		s->done.push_back(vp_edit_done{sl->tickets[k], VP_OK, sl->seq, sl->submit_s[k], sl->t_start, t});
	s->st.chunks_remeshed += sl->dirty.size();
	w->last_dirty = sl->dirty;
	sl->busy = false;
	sl->tickets.clear();
	sl->submit_s.clear();
	note_inflight(s, -1);
	if (s->inflight == 0) w->pool_tail = s->tail_known;
	return VP_OK;
}

/* Retire every finished batch (or, with wait, every batch), in admission
 * order; an arena overflow waits for all batches, grows and remeshes. */
int retire_finished(vp_server *s, bool wait)
{
	vp_world *w = s->w;
	std::vector<EditSlot *> busy;
	for (EditSlot *sl : s->slots)
		if (sl->busy) busy.push_back(sl);
	std::sort(busy.begin(), busy.end(), [](const EditSlot *a, const EditSlot *b) { return a->seq < b->seq; });
	bool overflow = false;
	std::vector<EditSlot *> fin;
	for (EditSlot *sl : busy) {
		if (wait) {
			CK(cudaEventSynchronize(sl->done));
		} else {
			const cudaError_t q = cudaEventQuery(sl->done);
			if (q == cudaErrorNotReady) continue;
			if (q != cudaSuccess) return cuda_fail(q, "edit batch");
		}
		fin.push_back(sl);
		overflow |= arena_overflow(w, sl);
	}
	if (overflow) {
		/* independent batches: wait for all, then grow and remesh those
		 * whose remesh saw its cursors pass the capacity, in admission
		 * order (flags taken before any growth) */
		fin.clear();
		for (EditSlot *sl : busy) {
			CK(cudaEventSynchronize(sl->done));
			fin.push_back(sl);
		}
		std::vector<bool> need(fin.size());
		for (size_t k = 0; k < fin.size(); k++) need[k] = arena_overflow(w, fin[k]);
		for (size_t k = 0; k < fin.size(); k++)
			if (need[k]) {
				int rc = regrow_and_remesh(w, fin[k], true);
				if (rc) return rc;
			}
	}
	for (EditSlot *sl : fin) {
		int rc = retire(s, sl);
		if (rc) return rc;
	}
	return VP_OK;
}

bool near_hit(const std::vector<uint32_t> &near, uint32_t c) { return std::binary_search(near.begin(), near.end(), c); }

/* Admit queued edits into free slots while they are independent of the
 * batches in flight. */
int admit(vp_server *s)
{
	vp_world *w = s->w;
	while (!s->queue.empty()) {
		EditSlot *sl = nullptr;
		for (EditSlot *c : s->slots)
			if (!c->busy) {
				sl = c;
				break;
			}
		if (!sl) {
			if (!s->held) s->st.deferred++;
			s->held = true;
			return VP_OK;
		}
		/* form the batch from the queue head */
		std::vector<vp_edit> be;
		std::vector<EditChunk> one;
		std::vector<uint32_t> dirty;
		std::vector<Rect> rd, wr;
		const bool big = w->root_bitw == 7; /* 128^3 remesh uses per-SM scratch: one batch at a time */
		size_t take = 0;
		bool wait = false;
		while (take < s->queue.size() && be.size() < s->cfg.max_batch) {
			const vp_edit &e = s->queue[take].e;
			one.clear();
			aabb_chunks(w, e, one);
			std::vector<uint32_t> nd = dirty;
			for (const EditChunk &c : one) nd.push_back(chunk_of(w, c));
			std::sort(nd.begin(), nd.end());
			nd.erase(std::unique(nd.begin(), nd.end()), nd.end());
			if (nd.size() > s->cfg.slot_chunks) {
				if (be.empty()) {
					/* alone it needs more than a slot holds: refused */
					const auto &pe = s->queue.front();
					const double t = srv_now(s);
					s->done.push_back(vp_edit_done{pe.ticket, VP_ENOMEM, 0, pe.submit_s, t, t});
					s->st.rejected++;
					s->queue.pop_front();
					continue;
				}
				break;
			}
			/* independence from every batch in flight */
			std::vector<Rect> er, ew;
			fill_rect(w, e, ew);
			er = ew;
			for (const EditChunk &c : one) remesh_rect(w, c.cv, er);
			bool conflict = big && s->inflight > 0;
			for (EditSlot *o : s->slots) {
				if (conflict) break;
				if (!o->busy) continue;
				for (const EditChunk &c : one)
					if (near_hit(o->near, chunk_of(w, c))) {
						conflict = true;
						break;
					}
				if (!conflict) conflict = overlaps(ew, o->sh_read) || overlaps(ew, o->sh_write) || overlaps(er, o->sh_write);
			}
			if (conflict) {
				if (be.empty()) wait = true;
				break;
			}
			be.push_back(e);
			dirty.swap(nd);
			rd.insert(rd.end(), er.begin(), er.end());
			wr.insert(wr.end(), ew.begin(), ew.end());
			take++;
		}
		if (be.empty()) { /* the queue head waits for the batches it conflicts with */
			if (wait && !s->held) s->st.deferred++;
			s->held = wait;
			return VP_OK;
		}
		/* room for the worst-case streams at the pool's tail */
		const uint64_t worst = worst_words(w, dirty.size());
		uint64_t bound = s->tail_known;
		for (EditSlot *o : s->slots)
			if (o->busy) bound += o->worst_words;
		if (bound + worst > w->pool_cap) {
			if (s->inflight) {
				if (!s->held) s->st.deferred++;
				s->held = true;
				return VP_OK;
			}
			int rc = compact_pool(w, worst);
			if (rc) return rc;
			s->tail_known = w->pool_tail;
		}
		s->held = false;
		plan_batch(w, be.data(), (uint32_t)be.size(), s->plan);
		/* after whatever the world's own stream holds (a rebuild, an upload) */
		CK(cudaEventRecord(s->ctx_ev, w->ctx->stream));
		CK(cudaStreamWaitEvent(sl->stream, s->ctx_ev, 0));
		const bool first = s->inflight == 0;
		if (first) s->tail_known = w->pool_tail;
		int rc = enqueue_batch(w, sl, be.data(), (uint32_t)be.size(), s->plan, first);
		if (rc) return rc;
		sl->busy = true;
		sl->seq = s->next_seq++;
		sl->worst_words = worst;
		sl->sh_read.swap(rd);
		sl->sh_write.swap(wr);
		sl->near.clear();
		const int mx[3] = {1 << w->max_bitw[0], 1 << w->max_bitw[1], 1 << w->max_bitw[2]};
		for (uint32_t c : sl->dirty) {
			const int cx = (int)(c & (uint32_t)(mx[0] - 1)), cy = (int)((c >> w->max_bitw[0]) & (uint32_t)(mx[1] - 1)),
				  cz = (int)(c >> (w->max_bitw[0] + w->max_bitw[1]));
			for (int dz = -1; dz <= 1; dz++)
				for (int dy = -1; dy <= 1; dy++)
					for (int dx = -1; dx <= 1; dx++) {
						const int x = cx + dx, y = cy + dy, z = cz + dz;
						if (x < 0 || y < 0 || z < 0 || x >= mx[0] || y >= mx[1] || z >= mx[2]) continue;
						sl->near.push_back(((uint32_t)z << w->max_bitw[1] | (uint32_t)y) << w->max_bitw[0] | (uint32_t)x);
					}
		}
		std::sort(sl->near.begin(), sl->near.end());
		sl->near.erase(std::unique(sl->near.begin(), sl->near.end()), sl->near.end());
		sl->t_start = srv_now(s);
		for (size_t k = 0; k < take; k++) {
			sl->tickets.push_back(s->queue.front().ticket);
			sl->submit_s.push_back(s->queue.front().submit_s);
			s->queue.pop_front();
		}
		note_inflight(s, +1);
		s->st.batches++;
		s->st.edits += (uint32_t)be.size();
		s->st.max_batch = std::max(s->st.max_batch, (uint32_t)be.size());
	}
	return VP_OK;
}

int pump(vp_server *s)
{
	int rc = retire_finished(s, false);
	if (!rc) rc = admit(s);
	return rc;
}

} // namespace

int vpi_server_quiesce(vp_world *w)
{
	if (!w->server || !w->server->inflight) return VP_OK;
	cudaSetDevice(w->ctx->device);
	return retire_finished(w->server, true);
}

void vpi_edit_state_free(vp_world *w)
{
	if (w->server) {
		vp_server_destroy(w->server);
		w->server = nullptr;
	}
	slot_free(w->eslot);
	w->eslot = nullptr;
	dev_free(w->d_pool_cursor);
}

extern "C" {

VP_API int vp_world_edit(vp_world *w, const vp_edit *edits, uint32_t n)
{
	if (!w || (!edits && n) || !w->uploaded) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	int rc = vpi_pipe_drain(w);
	if (rc) return rc;
	for (uint32_t i = 0; i < n; i++)
		if (edits[i].radius > kMaxRadius) return VP_EUNSUPPORTED;
	if ((rc = ensure_edit_state(w))) return rc;
	Plan p;
	plan_batch(w, edits, n, p);
	w->last_dirty = p.dirty;
	const size_t nd = p.dirty.size();
	if (!nd) return VP_OK;
	const uint64_t worst = worst_words(w, nd);
	if (w->pool_tail + worst > w->pool_cap)
		if ((rc = compact_pool(w, worst))) return rc;
	EditSlot *s = w->eslot;
	if ((rc = slot_size(w, s, nd, p.lists.size()))) return rc;
	if ((rc = enqueue_batch(w, s, edits, n, p, true))) return rc;
	CK(cudaEventSynchronize(s->done));
	if ((uint32_t)s->h_pin[1] & (kStatusOverflow | kStatusBadStream)) return VP_ECUDA;
	w->pool_tail = s->h_pin[0];
	return arena_overflow(w, s) ? regrow_and_remesh(w, s) : VP_OK;
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

VP_API int vp_server_create(vp_world *w, const vp_server_config *cfg, vp_server **out)
{
	if (!w || !cfg || !out || !w->uploaded || !cfg->slots || cfg->slots > kMaxSlots || !cfg->max_batch ||
	    !cfg->slot_chunks)
		return VP_EINVAL;
	if (w->server) return VP_EBUSY;
	CK(cudaSetDevice(w->ctx->device));
	int rc = vpi_pipe_drain(w);
	if (rc) return rc;
	if ((rc = ensure_edit_state(w))) return rc;
	*out = nullptr;
	/* slots sized for slot_chunks dirty chunks; as many as the free device
	 * memory above the reserve holds */
	const size_t nlists = (size_t)cfg->max_batch * kMaxListPerEdit;
	const uint64_t per = slot_bytes(w, cfg->slot_chunks, nlists);
	size_t free_b = 0, total_b = 0;
	CK(cudaMemGetInfo(&free_b, &total_b));
	const uint64_t avail = free_b > cfg->hbm_reserve ? free_b - cfg->hbm_reserve : 0;
	const uint32_t nslots = (uint32_t)std::min<uint64_t>(cfg->slots, avail / std::max<uint64_t>(per, 1));
	if (!nslots) return VP_ENOMEM;
	vp_server *s = new vp_server();
	s->w = w;
	s->cfg = *cfg;
	if (cudaEventCreateWithFlags(&s->ctx_ev, cudaEventDisableTiming) != cudaSuccess) {
		delete s;
		return cuda_fail(cudaGetLastError(), "cudaEventCreate");
	}
	for (uint32_t k = 0; k < nslots; k++) {
		EditSlot *sl = new EditSlot();
		s->slots.push_back(sl);
		if ((rc = slot_init(sl, nullptr)) || (rc = slot_size(w, sl, cfg->slot_chunks, nlists))) {
			vp_server_destroy(s);
			return rc == VP_ECUDA || rc == VP_ENOMEM ? VP_ENOMEM : rc;
		}
	}
	/* a spare pool for compactions while serving (without the room, a
	 * compaction allocates one then) */
	const uint64_t spare = w->pool_cap + w->pool_cap / 4 + (16u << 20);
	if (w->pool_spare_cap < spare && free_b > cfg->hbm_reserve + spare * 4u + nslots * per) {
		dev_free(w->d_pool_spare);
		w->pool_spare_cap = 0;
		if (dev_alloc(&w->d_pool_spare, spare) == VP_OK) w->pool_spare_cap = spare;
	}
	if (!w->d_noff && dev_alloc(&w->d_noff, w->nchunks) != VP_OK) w->d_noff = nullptr;
	s->t0 = now_s();
	s->tail_known = w->pool_tail;
	w->server = s;
	*out = s;
	return VP_OK;
}

VP_API void vp_server_destroy(vp_server *s)
{
	if (!s) return;
	cudaSetDevice(s->w->ctx->device);
	if (s->inflight) retire_finished(s, true);
	if (s->w->server == s) s->w->server = nullptr;
	for (EditSlot *sl : s->slots) slot_free(sl);
	if (s->ctx_ev) cudaEventDestroy(s->ctx_ev);
	delete s;
}

VP_API int vp_edit_submit(vp_server *s, const vp_edit *edits, uint32_t n, uint64_t *first_ticket)
{
	if (!s || (!edits && n)) return VP_EINVAL;
	for (uint32_t i = 0; i < n; i++)
		if (edits[i].radius > kMaxRadius) return VP_EUNSUPPORTED;
	CK(cudaSetDevice(s->w->ctx->device));
	if (first_ticket) *first_ticket = s->next_ticket;
	const double t = srv_now(s);
	for (uint32_t i = 0; i < n; i++) s->queue.push_back(vp_server::Pending{s->next_ticket++, edits[i], t});
	return pump(s);
}

VP_API int vp_poll_results(vp_server *s, vp_edit_done *out, uint32_t cap, uint32_t *n, uint32_t wait_us)
{
	if (!s || !n || (!out && cap)) return VP_EINVAL;
	CK(cudaSetDevice(s->w->ctx->device));
	int rc = pump(s);
	if (rc) return rc;
	const double until = now_s() + wait_us * 1e-6;
	while (s->done.empty() && (s->inflight || !s->queue.empty()) && now_s() < until) {
		std::this_thread::sleep_for(std::chrono::microseconds(20));
		if ((rc = pump(s))) return rc;
	}
	uint32_t k = 0;
	while (k < cap && !s->done.empty()) {
		out[k++] = s->done.front();
		s->done.pop_front();
	}
	*n = k;
	return VP_OK;
}

VP_API int vp_server_drain(vp_server *s)
{
	if (!s) return VP_EINVAL;
	CK(cudaSetDevice(s->w->ctx->device));
	int rc;
	while (!s->queue.empty() || s->inflight) {
		if ((rc = pump(s))) return rc;
		if (s->inflight && (rc = retire_finished(s, true))) return rc;
	}
	return VP_OK;
}

VP_API int vp_server_stats(vp_server *s, vp_serve_stats *stats, uint32_t *slots_out)
{
	if (!s || !stats) return VP_EINVAL;
	*stats = s->st;
	const double t = srv_now(s);
	stats->inflight_s += (double)s->inflight * (t - s->last_change);
	if (s->inflight) stats->busy_s += t - s->busy_since;
	stats->wall_s = t;
	if (slots_out) *slots_out = (uint32_t)s->slots.size();
	return VP_OK;
}

VP_API int vp_world_serve(vp_world *w, const vp_edit *edits, uint32_t n, uint32_t max_batch, uint32_t slots,
			  uint64_t hbm_reserve, double *latency_ms, vp_serve_stats *stats)
{
	if (!w || (!edits && n) || !latency_ms || !stats || !w->uploaded || !max_batch || !slots) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	memset(stats, 0, sizeof(*stats));
	vp_server_config cfg = {slots, max_batch, 512, hbm_reserve};
	vp_server *s = nullptr;
	int rc = vp_server_create(w, &cfg, &s);
	if (rc) return rc;
	std::vector<vp_edit_done> got(256);
	uint32_t next = 0, finished = 0;
	while (finished < n) {
		/* submit what has arrived */
		const double t = srv_now(s);
		uint32_t k = next;
		while (k < n && edits[k].arrival_s <= t) k++;
		if (k > next) {
			for (uint32_t i = next; i < k; i++) s->queue.push_back(vp_server::Pending{s->next_ticket++, edits[i], edits[i].arrival_s});
			next = k;
		}
		uint32_t m = 0;
		if ((rc = vp_poll_results(s, got.data(), (uint32_t)got.size(), &m, 0))) break;
		for (uint32_t j = 0; j < m; j++) {
			const vp_edit_done &d = got[j];
			const double a = edits[d.ticket].arrival_s;
			latency_ms[d.ticket] = d.status == VP_OK ? (d.done_s - a) * 1e3 : -1.0;
			finished++;
		}
		if (m) continue;
		/* nothing finished: sleep a little, never past the next arrival */
		const double gap = next < n ? edits[next].arrival_s - srv_now(s) : 1.0;
		if (gap > 0) std::this_thread::sleep_for(std::chrono::microseconds(gap > 20e-6 ? 20 : 1));
	}
	if (!rc) rc = vp_server_stats(s, stats, nullptr);
	vp_server_destroy(s);
	return rc;
}

} // extern "C"
