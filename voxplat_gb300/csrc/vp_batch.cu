/*
 * vp_batch.cu — batches of standalone chunks of mixed root sizes (8..128):
 * each chunk is its own 1x1x1 ChunkSet with its own shadow map, as the
 * reference meshes a chunk whose neighbours are the air null chunk
 * (src/chunkset.c:233-507 over such sets, src/chunkset/mesher.c:377-536).
 *
 * A rebuild runs in one of three forms:
 *   plain      one launch per chunk of the kernel for its root size;
 *   direct     the tuned batched configuration, launched directly;
 *   graph      the same configuration captured once into a CUDA graph and
 *              replayed (one cudaGraphLaunch per rebuild).
 * Batched configurations (chosen by vp_batch_autotune, which times each):
 *   MIXED      one persistent launch whose CTAs take items of every root
 *              size from one device queue (register cap for 2 CTAs/SM, or
 *              none);
 *   SPLIT      one persistent launch per root size, on forked streams so
 *              they run concurrently;
 * each with items ordered longest stream first, or by root size then
 * longest first.
 */
#include "voxgpu.h"
#include "vp_geometry.h"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "vp_internal.h"

using namespace vp;

struct vp_batch {
	vp_ctx *ctx = nullptr;
	uint32_t n = 0;
	std::vector<int> rb;             /* root_bitw per chunk */
	std::vector<uint32_t> hlen;      /* stream words per chunk */
	uint32_t *d_pool = nullptr;
	uint64_t *d_off = nullptr;
	uint32_t *d_len = nullptr;
	uint16_t *d_shadow = nullptr;
	SetDesc *d_sets = nullptr;
	WorkItem *d_items = nullptr;
	std::vector<WorkItem> items;     /* host copy in launch order */
	uint32_t group_start[9] = {0};   /* SPLIT: items of root size r at [start[r], start[r+1]) */
	ChunkOut *d_outs = nullptr;
	unsigned int *d_queue = nullptr; /* [8] */
	unsigned long long *d_cursors = nullptr;
	void *d_arena[3] = {nullptr, nullptr, nullptr};
	uint64_t cap[3] = {0, 0, 0};
	uint8_t *d_big = nullptr;
	uint32_t big_slots = 0;
	std::vector<uint8_t> modes;
	bool uploaded = false;
	vp_batch_tune tune;
	int items_order = -1;            /* order the device items are in */
	/* graph of the tuned configuration */
	cudaGraphExec_t gexec = nullptr;
	int graph_lod = -1;
	cudaStream_t side[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	PlainStreams plain;              /* VP_REBUILD_CONCURRENT */
	cudaEvent_t fork = nullptr, join[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	/* timing */
	std::vector<cudaEvent_t> ev;
	double ms = 0;
	uint32_t launches = 0;
	int last_lod = 4;
	unsigned last_flags = 0;
};

static void drop_graph(vp_batch *b)
{
	if (b->gexec) cudaGraphExecDestroy(b->gexec);
	b->gexec = nullptr;
	b->graph_lod = -1;
}

VP_API int vp_batch_create(vp_ctx *ctx, uint32_t n, const int *root_bitw, vp_batch **out)
{
	if (!ctx || !out || !root_bitw || n == 0 || n > (1u << 24)) return VP_EINVAL;
	*out = nullptr;
	for (uint32_t k = 0; k < n; k++)
		if (root_bitw[k] < 3 || root_bitw[k] > 7) return VP_EUNSUPPORTED;
	CK(cudaSetDevice(ctx->device));
	vp_batch *b = new vp_batch();
	b->ctx = ctx;
	b->n = n;
	b->rb.assign(root_bitw, root_bitw + n);
	b->modes.assign(n, 0);
	b->tune.strategy = VP_BATCH_MIXED;
	b->tune.min_blocks = 2;
	b->tune.order = 0;
	b->tune.ctas = 0;
	b->tune.ms = 0.f;
	b->tune.threads = 512;
	b->tune.grain = 1;
	int rc;
	if ((rc = dev_alloc(&b->d_off, n)) || (rc = dev_alloc(&b->d_len, n)) || (rc = dev_alloc(&b->d_sets, n)) ||
	    (rc = dev_alloc(&b->d_items, n)) || (rc = dev_alloc(&b->d_outs, n)) || (rc = dev_alloc(&b->d_queue, 8)) ||
	    (rc = dev_alloc(&b->d_cursors, 3))) {
		vp_batch_destroy(b);
		return rc;
	}
	if (std::find(b->rb.begin(), b->rb.end(), 7) != b->rb.end()) {
		/* a 128^3 item may land on any CTA of a two-per-SM launch */
		b->big_slots = 2u * (uint32_t)ctx->sm_count;
		if ((rc = dev_alloc(&b->d_big, (size_t)b->big_slots * big_scratch_slot_bytes()))) {
			vp_batch_destroy(b);
			return rc;
		}
	}
	for (int i = 0; i < 5; i++) {
		if (cudaStreamCreateWithFlags(&b->side[i], cudaStreamNonBlocking) != cudaSuccess ||
		    cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) != cudaSuccess) {
			vp_batch_destroy(b);
			return VP_ECUDA;
		}
	}
	if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
		vp_batch_destroy(b);
		return VP_ECUDA;
	}
	*out = b;
	return VP_OK;
}

VP_API void vp_batch_destroy(vp_batch *b)
{
	if (!b) return;
	cudaSetDevice(b->ctx->device);
	cudaStreamSynchronize(b->ctx->stream);
	drop_graph(b);
	for (int i = 0; i < 5; i++) {
		if (b->side[i]) {
			cudaStreamSynchronize(b->side[i]);
			cudaStreamDestroy(b->side[i]);
		}
		if (b->join[i]) cudaEventDestroy(b->join[i]);
	}
	if (b->fork) cudaEventDestroy(b->fork);
	vpi_plain_free(b->plain);
	for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
	dev_free(b->d_pool);
	dev_free(b->d_off);
	dev_free(b->d_len);
	dev_free(b->d_shadow);
	dev_free(b->d_sets);
	dev_free(b->d_items);
	dev_free(b->d_outs);
	dev_free(b->d_queue);
	dev_free(b->d_cursors);
	dev_free(b->d_big);
	for (int a = 0; a < 3; a++) dev_free(b->d_arena[a]);
	delete b;
}

/* Items in launch order for an ordering: 0 = longest stream first (work
 * weighted by the chunk volume as well), 1 = by root size (largest first),
 * then longest first. Records the per-root ranges for SPLIT. */
static int upload_items(vp_batch *b, int order)
{
	std::vector<uint32_t> idx(b->n);
	std::iota(idx.begin(), idx.end(), 0u);
	auto weight = [&](uint32_t k) { return (uint64_t)b->hlen[k] + (1ull << (3 * b->rb[k] - 6)); };
	if (order == 0)
		std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t c) { return weight(a) > weight(c); });
	else
		std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t c) {
			if (b->rb[a] != b->rb[c]) return b->rb[a] > b->rb[c];
			return weight(a) > weight(c);
		});
	b->items.resize(b->n);
	for (uint32_t i = 0; i < b->n; i++) {
		const uint32_t k = idx[i];
		b->items[i] = WorkItem{k, 0u, b->modes[k] ? kItemMesh : 0u, k};
	}
	/* per-root ranges (meaningful for order 1: roots descending) */
	for (int r = 0; r <= 8; r++) b->group_start[r] = 0;
	if (order == 1) {
		uint32_t pos = 0;
		for (int r = 7; r >= 3; r--) {
			b->group_start[r] = pos;
			while (pos < b->n && b->rb[b->items[pos].set] == r) pos++;
		}
		b->group_start[8] = pos; /* end of root 3 = n */
	}
	CK(cudaMemcpyAsync(b->d_items, b->items.data(), b->n * sizeof(WorkItem), cudaMemcpyHostToDevice,
			   b->ctx->stream));
	b->items_order = order;
	return VP_OK;
}

/* range of root size r in SPLIT order: [lo, hi) */
static void group_range(const vp_batch *b, int r, uint32_t &lo, uint32_t &hi)
{
	lo = b->group_start[r];
	hi = r == 3 ? b->group_start[8] : b->group_start[r - 1];
	if (r > 3 && hi < lo) hi = lo;
}

VP_API int vp_batch_upload(vp_batch *b, const uint32_t *pool, uint64_t pool_words, const uint64_t *off,
			   const uint32_t *len, const uint16_t *shadow, const uint64_t *shadow_off,
			   const uint64_t *shadow_len)
{
	if (!b || !pool || !off || !len || !shadow || !shadow_off || !shadow_len) return VP_EINVAL;
	std::vector<uint64_t> noff(b->n);
	uint64_t total = 0, sh_total = 0;
	for (uint32_t k = 0; k < b->n; k++) {
		if (off[k] + len[k] > pool_words) return VP_EINVAL;
		int rc = vpi_validate_stream(pool + off[k], len[k], 1ull << (3 * b->rb[k]));
		if (rc) return rc;
		noff[k] = total;
		total += (len[k] + 3u) & ~3u;
		sh_total = std::max<uint64_t>(sh_total, shadow_off[k] + shadow_len[k]);
	}
	total += 8; /* vector loads may read up to 7 words past a terminator */
	std::vector<uint32_t> packed(total, 0u);
	for (uint32_t k = 0; k < b->n; k++) memcpy(&packed[noff[k]], pool + off[k], (size_t)len[k] * sizeof(uint32_t));
	CK(cudaSetDevice(b->ctx->device));
	cudaStream_t st = b->ctx->stream;
	CK(cudaStreamSynchronize(st));
	drop_graph(b);
	dev_free(b->d_pool);
	dev_free(b->d_shadow);
	int rc;
	if ((rc = dev_alloc(&b->d_pool, total)) || (rc = dev_alloc(&b->d_shadow, sh_total + 8))) return rc;
	CK(cudaMemcpyAsync(b->d_pool, packed.data(), total * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(b->d_off, noff.data(), b->n * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(b->d_len, len, b->n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(b->d_shadow, 0, (sh_total + 8) * sizeof(uint16_t), st));
	CK(cudaMemcpyAsync(b->d_shadow, shadow, sh_total * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
	std::vector<SetDesc> sets(b->n);
	for (uint32_t k = 0; k < b->n; k++) {
		SetDesc &d = sets[k];
		memset(&d, 0, sizeof(d));
		d.pool = b->d_pool;
		d.off = b->d_off + k;
		d.len = b->d_len + k;
		d.shadow = b->d_shadow + shadow_off[k];
		d.shadow_len = shadow_len[k];
		d.shell_bits = nullptr; /* no neighbours: no shell is ever read */
		d.shell_col = nullptr;
		d.shadow_w = 2u << b->rb[k];
		d.nchunks = 1;
		d.root_bitw = (uint32_t)b->rb[k];
	}
	CK(cudaMemcpyAsync(b->d_sets, sets.data(), b->n * sizeof(SetDesc), cudaMemcpyHostToDevice, st));
	b->hlen.assign(len, len + b->n);
	b->uploaded = true;
	if ((rc = upload_items(b, b->tune.order))) return rc;
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

VP_API int vp_batch_set_modes(vp_batch *b, const uint8_t *make_mesh)
{
	if (!b) return VP_EINVAL;
	for (uint32_t k = 0; k < b->n; k++) b->modes[k] = make_mesh ? (make_mesh[k] ? 1 : 0) : 0;
	if (!b->uploaded) return VP_OK;
	/* the graph reads the items from device memory: no recapture needed */
	return upload_items(b, b->items_order < 0 ? b->tune.order : b->items_order);
}

static int ensure_arenas(vp_batch *b)
{
	for (int a = 0; a < 3; a++) {
		if (b->d_arena[a]) continue;
		const uint64_t units = std::max<uint64_t>((uint64_t)b->n * 1024u, 1u << 20);
		cudaError_t e = cudaMalloc(&b->d_arena[a], units * 16u);
		if (e != cudaSuccess) {
			b->d_arena[a] = nullptr;
			return cuda_fail(e, "cudaMalloc(batch arena)");
		}
		b->cap[a] = units;
	}
	return VP_OK;
}

static GeoLaunch base_launch(vp_batch *b, int lod_max)
{
	GeoLaunch L;
	memset(&L, 0, sizeof(L));
	L.sets = b->d_sets;
	L.threads = b->tune.threads ? b->tune.threads : 512u;
	L.grain = b->tune.grain ? b->tune.grain : 1u;
	L.outs = b->d_outs;
	L.lod_max = lod_max;
	L.big_scratch = b->d_big;
	L.big_slots = b->big_slots;
	Arena *ar[3] = {&L.svl, &L.vbo, &L.ibo};
	for (int a = 0; a < 3; a++) {
		ar[a]->base = b->d_arena[a];
		ar[a]->cap_units = b->cap[a];
		ar[a]->cursor = b->d_cursors + a;
	}
	return L;
}

/* The batched configuration's stream work (memsets + launches) on `st`. */
static int enqueue_batched(vp_batch *b, int lod_max, cudaStream_t st)
{
	CK(cudaMemsetAsync(b->d_cursors, 0, 3 * sizeof(unsigned long long), st));
	CK(cudaMemsetAsync(b->d_queue, 0, 8 * sizeof(unsigned int), st));
	GeoLaunch L = base_launch(b, lod_max);
	const int sm = b->ctx->sm_count;
	if (b->tune.strategy == VP_BATCH_MIXED) {
		L.items = b->d_items;
		L.n_items = b->n;
		L.queue = b->d_queue;
		const int per_sm = geometry_mixed_ctas_per_sm(b->tune.min_blocks, (int)L.threads);
		L.ctas = b->tune.ctas ? b->tune.ctas : (uint32_t)(sm * std::max(per_sm, 1));
		cudaError_t e = launch_geometry_mixed(b->tune.min_blocks, L, st);
		if (e != cudaSuccess) return cuda_fail(e, "mixed launch");
		b->launches += 1;
		return VP_OK;
	}
	/* SPLIT: one persistent launch per root size, forked side streams */
	CK(cudaEventRecord(b->fork, st));
	int used = 0;
	for (int r = 7; r >= 3; r--) {
		uint32_t lo, hi;
		group_range(b, r, lo, hi);
		if (hi <= lo) continue;
		cudaStream_t s2 = b->side[used];
		CK(cudaStreamWaitEvent(s2, b->fork, 0));
		GeoLaunch G = L;
		G.items = b->d_items + lo;
		G.n_items = hi - lo;
		G.queue = b->d_queue + r;
		G.ctas = (uint32_t)(sm * std::max(geometry_ctas_per_sm(r, (int)G.threads), 1));
		cudaError_t e = launch_geometry(r, G, s2);
		if (e != cudaSuccess) return cuda_fail(e, "split launch");
		CK(cudaEventRecord(b->join[used], s2));
		used++;
		b->launches += 1;
	}
	for (int i = 0; i < used; i++) CK(cudaStreamWaitEvent(st, b->join[i], 0));
	return VP_OK;
}

/* One launch per chunk, on `st` or (conc) round-robin over forked streams;
 * a 128^3 chunk then uses the scratch slot of its stream, so two of them
 * never share a slot. */
static int enqueue_plain(vp_batch *b, int lod_max, cudaStream_t st, bool conc)
{
	CK(cudaMemsetAsync(b->d_cursors, 0, 3 * sizeof(unsigned long long), st));
	GeoLaunch L = base_launch(b, lod_max);
	int rc;
	if (conc && (rc = vpi_plain_fork(b->plain, st))) return rc;
	for (uint32_t i = 0; i < b->n; i++) {
		GeoLaunch G = L;
		G.items = b->d_items + i;
		G.n_items = 1;
		G.queue = nullptr;
		const int k = (int)(i % kPlainStreams);
		const int rb = b->rb[b->items[i].set];
		if (conc && rb == 7) {
			G.big_scratch = b->d_big + (size_t)k * big_scratch_slot_bytes();
			G.big_slots = 1;
		}
		cudaError_t e = launch_geometry(rb, G, conc ? b->plain.s[k] : st);
		if (e != cudaSuccess) return cuda_fail(e, "plain launch");
	}
	if (conc && (rc = vpi_plain_join(b->plain, st))) return rc;
	b->launches += b->n;
	return VP_OK;
}

static int capture_graph(vp_batch *b, int lod_max)
{
	drop_graph(b);
	cudaStream_t st = b->ctx->stream;
	/* occupancy queries and attribute setup outside the capture */
	geometry_mixed_ctas_per_sm(b->tune.min_blocks, 512);
	for (int r = 3; r <= 6; r++) geometry_ctas_per_sm(r, 512);
	CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
	const uint32_t launches = b->launches;
	int rc = enqueue_batched(b, lod_max, st);
	b->launches = launches;
	cudaGraph_t g = nullptr;
	cudaError_t e = cudaStreamEndCapture(st, &g);
	if (rc) {
		if (g) cudaGraphDestroy(g);
		return rc;
	}
	if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
	e = cudaGraphInstantiate(&b->gexec, g, 0);
	cudaGraphDestroy(g);
	if (e != cudaSuccess) {
		b->gexec = nullptr;
		return cuda_fail(e, "cudaGraphInstantiate");
	}
	b->graph_lod = lod_max;
	return VP_OK;
}

static int enqueue_rebuild(vp_batch *b, int lod_max, unsigned flags)
{
	vp_ctx *ctx = b->ctx;
	cudaStream_t st = ctx->stream;
	int rc;
	if ((rc = ensure_arenas(b))) return rc;
	const bool plain = (flags & (VP_REBUILD_PLAIN | VP_REBUILD_CONCURRENT)) != 0;
	if (!plain && b->items_order != b->tune.order) {
		drop_graph(b);
		if ((rc = upload_items(b, b->tune.order))) return rc;
	}
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	if (ctx->timing) {
		cudaEventCreate(&e0);
		cudaEventCreate(&e1);
		cudaEventRecord(e0, st);
	}
	if (plain) {
		rc = enqueue_plain(b, lod_max, st, (flags & VP_REBUILD_CONCURRENT) != 0);
	} else if (flags & VP_REBUILD_GRAPH) {
		if (!b->gexec || b->graph_lod != lod_max) rc = capture_graph(b, lod_max);
		if (!rc) {
			cudaError_t e = cudaGraphLaunch(b->gexec, st);
			if (e != cudaSuccess) rc = cuda_fail(e, "cudaGraphLaunch");
			b->launches += b->tune.strategy == VP_BATCH_MIXED ? 1u : 0u;
			if (b->tune.strategy == VP_BATCH_SPLIT)
				for (int r = 3; r <= 7; r++) {
					uint32_t lo, hi;
					group_range(b, r, lo, hi);
					b->launches += hi > lo;
				}
		}
	} else {
		rc = enqueue_batched(b, lod_max, st);
	}
	if (ctx->timing) {
		cudaEventRecord(e1, st);
		b->ev.push_back(e0);
		b->ev.push_back(e1);
	}
	if (rc) return rc;
	b->last_lod = lod_max;
	b->last_flags = flags;
	return VP_OK;
}

VP_API int vp_batch_rebuild(vp_batch *b, int lod_max, unsigned flags)
{
	if (!b || !b->uploaded) return VP_EINVAL;
	if (lod_max < 0 || lod_max >= VP_MAX_LEVELS) return VP_EUNSUPPORTED;
	CK(cudaSetDevice(b->ctx->device));
	return enqueue_rebuild(b, lod_max, flags);
}

VP_API int vp_batch_finish(vp_batch *b)
{
	if (!b) return VP_EINVAL;
	cudaStream_t st = b->ctx->stream;
	for (int attempt = 0; attempt < 4; attempt++) {
		unsigned long long cur[3];
		CK(cudaMemcpyAsync(cur, b->d_cursors, sizeof(cur), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		bool grow = false;
		for (int a = 0; a < 3; a++) {
			if (cur[a] <= b->cap[a]) continue;
			grow = true;
			const uint64_t units = cur[a] + cur[a] / 4 + 1024;
			dev_free(b->d_arena[a]);
			cudaError_t e = cudaMalloc(&b->d_arena[a], units * 16u);
			if (e != cudaSuccess) {
				b->d_arena[a] = nullptr;
				b->cap[a] = 0;
				return cuda_fail(e, "cudaMalloc(batch arena growth)");
			}
			b->cap[a] = units;
		}
		if (!grow) return VP_OK;
		drop_graph(b); /* the graph holds the old arena pointers */
		int rc = enqueue_rebuild(b, b->last_lod, b->last_flags);
		if (rc) return rc;
	}
	return VP_EOVERFLOW;
}

VP_API int vp_batch_set_tune(vp_batch *b, const vp_batch_tune *t)
{
	if (!b || !t) return VP_EINVAL;
	if (t->strategy != VP_BATCH_MIXED && t->strategy != VP_BATCH_SPLIT) return VP_EINVAL;
	if (t->order != 0 && t->order != 1) return VP_EINVAL;
	if (t->strategy == VP_BATCH_SPLIT && t->order != 1) return VP_EINVAL; /* SPLIT needs root-grouped items */
	if (t->min_blocks != 1 && t->min_blocks != 2) return VP_EINVAL;
	if (b->big_slots && t->ctas > b->big_slots) return VP_EINVAL;
	if (t->threads != 0 && t->threads != 256 && t->threads != 512) return VP_EINVAL;
	if (t->grain > 64) return VP_EINVAL;
	CK(cudaStreamSynchronize(b->ctx->stream));
	b->tune = *t;
	drop_graph(b);
	return VP_OK;
}

/* Time one configuration: the first replay sizes the arenas and captures
 * the graph, then `reps` replays are timed. */
static int time_tune(vp_batch *b, int lod_max, vp_batch_tune *t, cudaEvent_t t0, cudaEvent_t t1)
{
	cudaStream_t st = b->ctx->stream;
	int rc;
	if ((rc = vp_batch_set_tune(b, t))) return rc;
	if ((rc = enqueue_rebuild(b, lod_max, VP_REBUILD_GRAPH)) || (rc = vp_batch_finish(b))) return rc;
	if ((rc = enqueue_rebuild(b, lod_max, VP_REBUILD_GRAPH))) return rc;
	CK(cudaEventRecord(t0, st));
	const int reps = 3;
	for (int k = 0; k < reps; k++)
		if ((rc = enqueue_rebuild(b, lod_max, VP_REBUILD_GRAPH))) return rc;
	CK(cudaEventRecord(t1, st));
	CK(cudaEventSynchronize(t1));
	float ms = 0.f;
	CK(cudaEventElapsedTime(&ms, t0, t1));
	t->ms = ms / reps;
	return VP_OK;
}

VP_API int vp_batch_autotune(vp_batch *b, int lod_max, vp_batch_tune *best, vp_batch_tune *tried, int *ntried)
{
	if (!b || !b->uploaded || !best) return VP_EINVAL;
	CK(cudaSetDevice(b->ctx->device));
	/* stage 1: strategy, order, register cap */
	const vp_batch_tune stage1[] = {
		{VP_BATCH_MIXED, 2, 0, 0, 0.f, 512, 1},
		{VP_BATCH_MIXED, 2, 1, 0, 0.f, 512, 1},
		{VP_BATCH_MIXED, 1, 0, 0, 0.f, 512, 1},
		{VP_BATCH_SPLIT, 2, 1, 0, 0.f, 512, 1},
	};
	cudaEvent_t t0, t1;
	CK(cudaEventCreate(&t0));
	CK(cudaEventCreate(&t1));
	const int timing = b->ctx->timing;
	b->ctx->timing = 0;
	std::vector<vp_batch_tune> res;
	int rc = VP_OK, bi = -1;
	for (const vp_batch_tune &c : stage1) {
		vp_batch_tune t = c;
		if ((rc = time_tune(b, lod_max, &t, t0, t1))) break;
		res.push_back(t);
		if (bi < 0 || t.ms < res[bi].ms) bi = (int)res.size() - 1;
	}
	/* stage 2: threads per chunk, chunks per dequeue and the persistent
	 * grid around the best of stage 1 */
	if (!rc) {
		const vp_batch_tune base = res[bi];
		const uint32_t sm = (uint32_t)b->ctx->sm_count;
		for (uint32_t threads : {256u, 512u})
			for (uint32_t grain : {1u, 2u, 4u})
				for (uint32_t ctas : {0u, sm}) {
					if (rc) break;
					if (ctas && base.strategy != VP_BATCH_MIXED) continue;
					if (threads == base.threads && grain == base.grain && ctas == base.ctas) continue;
					if (b->big_slots && ctas > b->big_slots) continue;
					vp_batch_tune t = base;
					t.threads = threads;
					t.grain = grain;
					t.ctas = ctas;
					if ((rc = time_tune(b, lod_max, &t, t0, t1))) break;
					res.push_back(t);
					if (t.ms < res[bi].ms) bi = (int)res.size() - 1;
				}
	}
	b->ctx->timing = timing;
	cudaEventDestroy(t0);
	cudaEventDestroy(t1);
	if (rc) return rc;
	if (tried && ntried) {
		const int m = std::min(*ntried, (int)res.size());
		for (int c = 0; c < m; c++) tried[c] = res[c];
		*ntried = (int)res.size();
	}
	*best = res[bi];
	return vp_batch_set_tune(b, &res[bi]);
}

VP_API int vp_batch_get_tune(vp_batch *b, vp_batch_tune *t)
{
	if (!b || !t) return VP_EINVAL;
	*t = b->tune;
	return VP_OK;
}

VP_API int vp_batch_results(vp_batch *b, vp_chunk_result *out, uint32_t n)
{
	static_assert(sizeof(vp_chunk_result) == sizeof(ChunkOut), "result record layout");
	if (!b || !out || n > b->n) return VP_EINVAL;
	CK(cudaMemcpyAsync(out, b->d_outs, (size_t)n * sizeof(ChunkOut), cudaMemcpyDeviceToHost, b->ctx->stream));
	CK(cudaStreamSynchronize(b->ctx->stream));
	return VP_OK;
}

static int read_arena(vp_batch *b, int a, uint64_t off_bytes, uint64_t nbytes, void *dst)
{
	if (!b || (!dst && nbytes)) return VP_EINVAL;
	if (off_bytes + nbytes > b->cap[a] * 16u) return VP_EINVAL;
	if (!nbytes) return VP_OK;
	CK(cudaMemcpyAsync(dst, (const char *)b->d_arena[a] + off_bytes, nbytes, cudaMemcpyDeviceToHost,
			   b->ctx->stream));
	CK(cudaStreamSynchronize(b->ctx->stream));
	return VP_OK;
}

VP_API int vp_batch_read_svl(vp_batch *b, uint64_t off, uint64_t n, int16_t *dst)
{
	return read_arena(b, 0, off * 2u, n * 2u, dst);
}

VP_API int vp_batch_read_vbo(vp_batch *b, uint64_t off, uint64_t n, int16_t *dst)
{
	return read_arena(b, 1, off * 2u, n * 2u, dst);
}

VP_API int vp_batch_read_ibo(vp_batch *b, uint64_t off, uint64_t n, uint32_t *dst)
{
	return read_arena(b, 2, off * 4u, n * 4u, dst);
}

VP_API int vp_batch_kernel_ms(vp_batch *b, double *ms, uint32_t *launches)
{
	if (!b || !ms) return VP_EINVAL;
	CK(cudaStreamSynchronize(b->ctx->stream));
	double t = 0;
	for (size_t i = 0; i + 1 < b->ev.size(); i += 2) {
		float x = 0.f;
		cudaEventElapsedTime(&x, b->ev[i], b->ev[i + 1]);
		t += x;
	}
	for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
	b->ev.clear();
	*ms = t;
	if (launches) *launches = b->launches;
	b->launches = 0;
	return VP_OK;
}
