/*
 * vp_api.cu — the C ABI (include/voxgpu.h): contexts, device-resident worlds,
 * batched rebuilds, result readback and kernel timing.
 */
#include "voxgpu.h"
#include "vp_geometry.h"
#include "vp_rle.h"
#include "vp_group.h"
#include "vp_gen.h"
#include "vp_cull.h"
#include "vp_raycast.h"
#include "vp_render.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

using namespace vp;

#include "vp_internal.h"

thread_local std::string vpi_cuda_err;

int vpi_cuda_fail(cudaError_t e, const char *what)
{
	char buf[256];
	snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
	vpi_cuda_err = buf;
	return e == cudaErrorMemoryAllocation ? VP_ENOMEM : VP_ECUDA;
}

/* A few words between device and host as kernels: stores into mapped pinned
 * memory do not queue behind bulk transfers on the copy engines, as a small
 * cudaMemcpyAsync would while an output readback is in flight. */
template <typename T> __global__ void k_fetch_words(const T *src, T *dst, uint32_t n)
{
	if (threadIdx.x < n) dst[threadIdx.x] = src[threadIdx.x];
}

__global__ void k_put_cursors(unsigned long long *cur, unsigned long long a, unsigned long long b, unsigned long long c)
{
	if (threadIdx.x == 0) {
		cur[0] = a;
		cur[1] = b;
		cur[2] = c;
	}
}

extern "C" {

VP_API const char *vp_strerror(int code)
{
	switch (code) {
	case VP_OK: return "ok";
	case VP_EINVAL: return "invalid argument";
	case VP_ENOMEM: return "out of memory";
	case VP_ECUDA: return "CUDA error";
	case VP_EOVERFLOW: return "output overflow";
	case VP_ETIMEOUT: return "device wait timed out";
	case VP_EUNSUPPORTED: return "unsupported configuration";
	case VP_EBUSY: return "admission refused";
	default: return "unknown error";
	}
}

VP_API const char *vp_last_cuda_error(void) { return vpi_cuda_err.c_str(); }

VP_API int vp_ctx_create(int device, vp_ctx **out)
{
	if (!out) return VP_EINVAL;
	*out = nullptr;
	CK(cudaSetDevice(device));
	vp_ctx *c = new vp_ctx();
	c->device = device;
	c->timing = 0;
	cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
	if (e != cudaSuccess) {
		delete c;
		return cuda_fail(e, "cudaStreamCreate");
	}
	cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
	*out = c;
	return VP_OK;
}

VP_API void vp_ctx_destroy(vp_ctx *c)
{
	if (!c) return;
	cudaSetDevice(c->device);
	cudaStreamSynchronize(c->stream);
	dev_free(c->d_bytes);
	dev_free(c->d_words);
	dev_free(c->d_scalars);
	cudaStreamDestroy(c->stream);
	delete c;
}

static int ensure_stage(vp_ctx *c, size_t nbytes, size_t nwords)
{
	if (nbytes > c->bytes_cap) {
		dev_free(c->d_bytes);
		c->bytes_cap = 0;
		int rc = dev_alloc(&c->d_bytes, nbytes);
		if (rc) return rc;
		c->bytes_cap = nbytes;
	}
	if (nwords > c->words_cap) {
		dev_free(c->d_words);
		c->words_cap = 0;
		int rc = dev_alloc(&c->d_words, nwords);
		if (rc) return rc;
		c->words_cap = nwords;
	}
	if (!c->d_scalars) {
		int rc = dev_alloc(&c->d_scalars, 4);
		if (rc) return rc;
	}
	return VP_OK;
}

VP_API int vp_rle_encode(vp_ctx *c, const uint8_t *vox, uint32_t length, uint32_t *out, uint32_t out_cap,
			 uint32_t *out_len)
{
	if (!c || !vox || !out || !out_len || length == 0) return VP_EINVAL;
	if (length >= 0xFFFFFFu) return VP_EUNSUPPORTED;
	CK(cudaSetDevice(c->device));
	const size_t padded = ((size_t)length + 15u) & ~(size_t)15u;
	int rc = ensure_stage(c, padded, (size_t)length + 8u);
	if (rc) return rc;
	cudaStream_t st = c->stream;
	CK(cudaMemcpyAsync(c->d_bytes, vox, length, cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(c->d_scalars, 0, 4 * sizeof(uint64_t), st));
	cudaError_t e = launch_rle_encode(c->d_bytes, 1, length, c->d_words, c->words_cap,
					  (unsigned long long *)c->d_scalars, c->d_scalars + 1,
					  (uint32_t *)(c->d_scalars + 2), (uint32_t *)(c->d_scalars + 3), st);
	if (e != cudaSuccess) return cuda_fail(e, "rle encode launch");
	uint64_t sc[4];
	CK(cudaMemcpyAsync(sc, c->d_scalars, sizeof(sc), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	const uint32_t n = (uint32_t)sc[2];
	if ((uint32_t)sc[3] & kStatusOverflow) return VP_EOVERFLOW;
	*out_len = n;
	if (n > out_cap) return VP_EOVERFLOW;
	CK(cudaMemcpyAsync(out, c->d_words + sc[1], (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

VP_API int vp_rle_decode(vp_ctx *c, const uint32_t *words, uint32_t nwords, uint8_t *out, uint32_t out_cap,
			 uint32_t *out_len)
{
	if (!c || !words || !out || !out_len || nwords == 0) return VP_EINVAL;
	/* the reference consumes the first word, then stops at the first 0 */
	uint32_t n = 1;
	uint64_t total = words[0] & 0xFFFFFFu;
	while (n < nwords && words[n]) {
		total += words[n] & 0xFFFFFFu;
		n++;
	}
	if (n >= nwords && nwords > 1 && words[nwords - 1] != 0) return VP_EINVAL; /* no terminator */
	*out_len = (uint32_t)total;
	if (total > out_cap) return VP_EOVERFLOW;
	if (total == 0) return VP_OK;
	CK(cudaSetDevice(c->device));
	int rc = ensure_stage(c, (total + 15u) & ~(uint64_t)15u, (size_t)n + 9u);
	if (rc) return rc;
	cudaStream_t st = c->stream;
	CK(cudaMemsetAsync(c->d_words, 0, ((size_t)n + 9u) * sizeof(uint32_t), st));
	CK(cudaMemcpyAsync(c->d_words, words, (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	const uint64_t off0 = 0;
	const uint32_t len0 = n + 1u; /* runs + terminator */
	CK(cudaMemcpyAsync(c->d_scalars, &off0, sizeof(off0), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(c->d_scalars + 1, &len0, sizeof(len0), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(c->d_scalars + 2, 0, sizeof(uint64_t), st));
	cudaError_t e = launch_rle_decode_bytes(c->d_words, c->d_scalars, (const uint32_t *)(c->d_scalars + 1), nullptr,
						1, (uint32_t)total, c->d_bytes, (uint32_t *)(c->d_scalars + 2), st);
	if (e != cudaSuccess) return cuda_fail(e, "rle decode launch");
	CK(cudaMemcpyAsync(out, c->d_bytes, total, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

VP_API void *vp_ctx_stream(vp_ctx *c) { return c ? (void *)c->stream : nullptr; }

VP_API int vp_ctx_sync(vp_ctx *c)
{
	if (!c) return VP_EINVAL;
	CK(cudaStreamSynchronize(c->stream));
	return VP_OK;
}

VP_API int vp_ctx_set_timing(vp_ctx *c, int on)
{
	if (!c) return VP_EINVAL;
	c->timing = on ? 1 : 0;
	return VP_OK;
}

VP_API int vp_world_create(vp_ctx *ctx, int root_bitw, const int max_bitw[3], vp_world **out)
{
	if (!ctx || !out || !max_bitw) return VP_EINVAL;
	*out = nullptr;
	if (geometry_smem_bytes(root_bitw) == 0) return VP_EUNSUPPORTED;
	for (int i = 0; i < 3; i++)
		if (max_bitw[i] < 0 || max_bitw[i] > 12) return VP_EINVAL;
	if (max_bitw[0] + max_bitw[1] + max_bitw[2] > 24) return VP_EUNSUPPORTED;
	CK(cudaSetDevice(ctx->device));
	vp_world *w = new vp_world();
	w->ctx = ctx;
	w->root_bitw = root_bitw;
	for (int i = 0; i < 3; i++) w->max_bitw[i] = max_bitw[i];
	w->nchunks = 1u << (max_bitw[0] + max_bitw[1] + max_bitw[2]);
	w->modes.assign(w->nchunks, 0);
	int rc = VP_OK;
	if ((rc = dev_alloc(&w->d_off, w->nchunks)) || (rc = dev_alloc(&w->d_len, w->nchunks)) ||
	    (rc = dev_alloc(&w->d_shell_bits, (size_t)w->nchunks * shell_words_per_chunk(root_bitw))) ||
	    (rc = dev_alloc(&w->d_shell_col, (size_t)w->nchunks * shell_cols_per_chunk(root_bitw))) ||
	    (rc = dev_alloc(&w->d_set, 1)) || (rc = dev_alloc(&w->d_items, w->nchunks)) ||
	    (rc = dev_alloc(&w->d_outs, w->nchunks)) || (rc = dev_alloc(&w->d_queue, 1)) ||
	    (rc = dev_alloc(&w->d_cursors, 3))) {
		vp_world_destroy(w);
		return rc;
	}
	if (root_bitw == 7) {
		/* one working set per SM: the 128^3 kernels run one CTA per SM */
		w->big_slots = (uint32_t)ctx->sm_count;
		if ((rc = dev_alloc(&w->d_big, (size_t)w->big_slots * big_scratch_slot_bytes()))) {
			vp_world_destroy(w);
			return rc;
		}
	}
	*out = w;
	return VP_OK;
}

VP_API void vp_world_destroy(vp_world *w)
{
	if (!w) return;
	cudaSetDevice(w->ctx->device);
	cudaStreamSynchronize(w->ctx->stream);
	dev_free(w->d_pool);
	dev_free(w->d_off);
	dev_free(w->d_len);
	dev_free(w->d_shadow);
	dev_free(w->d_shell_bits);
	dev_free(w->d_shell_col);
	dev_free(w->d_big);
	dev_free(w->d_check);
	dev_free(w->d_dec);
	dev_free(w->d_dec_slot);
	dev_free(w->d_cull_slots);
	dev_free(w->d_cull_blocks);
	dev_free(w->d_cull_out);
	dev_free(w->d_flags);
	dev_free(w->d_runidx);
	dev_free(w->d_rays);
	dev_free(w->d_render);
	dev_free(w->d_frame);
	dev_free(w->d_stream_items);
	dev_free(w->d_slab_q);
	if (w->copy_stream) {
		cudaStreamSynchronize(w->copy_stream);
		cudaStreamDestroy(w->copy_stream);
	}
	vpi_plain_free(w->plain);
	for (int h = 0; h < 2; h++)
		if (w->half_done[h]) cudaEventDestroy(w->half_done[h]);
	if (w->outs_alt[1]) {
		/* one of the two record buffers is d_outs (freed below) */
		if (w->outs_alt[1] != w->d_outs) dev_free(w->outs_alt[1]);
		else dev_free(w->outs_alt[0]);
	}
	for (int k = 0; k < kMaxStreamSlabs; k++)
		if (w->slab_ev[k]) cudaEventDestroy(w->slab_ev[k]);
	if (w->h_snap) cudaFreeHost(w->h_snap);
	if (w->h_check) cudaFreeHost(w->h_check);
	dev_free(w->d_set);
	dev_free(w->d_items);
	dev_free(w->d_shell_items);
	dev_free(w->d_null);
	dev_free(w->d_pool_spare);
	dev_free(w->d_noff);
	dev_free(w->d_outs);
	dev_free(w->d_queue);
	dev_free(w->d_cursors);
	for (int a = 0; a < 3; a++) dev_free(w->d_arena[a]);
	dev_free(w->d_gcounts);
	dev_free(w->d_gtotal);
	dev_free(w->d_node_off);
	dev_free(w->d_node_items);
	dev_free(w->d_garena);
	vpi_edit_state_free(w);
	for (cudaEvent_t e : w->ev) cudaEventDestroy(e);
	delete w;
}

int vpi_plain_fork(PlainStreams &p, cudaStream_t main)
{
	if (!p.fork) {
		for (int k = 0; k < kPlainStreams; k++) {
			CK(cudaStreamCreateWithFlags(&p.s[k], cudaStreamNonBlocking));
			CK(cudaEventCreateWithFlags(&p.ev[k], cudaEventDisableTiming));
		}
		CK(cudaEventCreateWithFlags(&p.fork, cudaEventDisableTiming));
	}
	CK(cudaEventRecord(p.fork, main));
	for (int k = 0; k < kPlainStreams; k++) CK(cudaStreamWaitEvent(p.s[k], p.fork, 0));
	return VP_OK;
}

int vpi_plain_join(PlainStreams &p, cudaStream_t main)
{
	for (int k = 0; k < kPlainStreams; k++) {
		CK(cudaEventRecord(p.ev[k], p.s[k]));
		CK(cudaStreamWaitEvent(main, p.ev[k], 0));
	}
	return VP_OK;
}

void vpi_plain_free(PlainStreams &p)
{
	for (int k = 0; k < kPlainStreams; k++) {
		if (p.s[k]) {
			cudaStreamSynchronize(p.s[k]);
			cudaStreamDestroy(p.s[k]);
		}
		if (p.ev[k]) cudaEventDestroy(p.ev[k]);
		p.s[k] = nullptr;
		p.ev[k] = nullptr;
	}
	if (p.fork) cudaEventDestroy(p.fork);
	p.fork = nullptr;
}

int vpi_validate_stream(const uint32_t *s, uint32_t n, uint64_t N)
{
	if (n < 2 || s[n - 1] != 0) return VP_EINVAL;
	uint64_t sum = 0;
	for (uint32_t i = 0; i + 1 < n; i++) {
		uint32_t c = s[i] & 0xFFFFFFu;
		if (c == 0) return VP_EINVAL;
		sum += c;
	}
	return sum == N ? VP_OK : VP_EINVAL;
}

int vpi_upload_setdesc(vp_world *w)
{
	SetDesc d;
	memset(&d, 0, sizeof(d));
	d.pool = w->d_pool;
	d.off = w->d_off;
	d.len = w->d_len;
	d.shadow = w->d_shadow;
	d.shadow_len = w->shadow_len;
	d.shell_bits = w->d_shell_bits;
	d.shell_col = w->d_shell_col;
	d.shadow_w = w->shadow_w;
	d.nchunks = w->nchunks;
	d.root_bitw = (uint32_t)w->root_bitw;
	for (int i = 0; i < 3; i++) d.max_bitw[i] = (uint32_t)w->max_bitw[i];
	for (int i = 0; i < 3; i++) d.origin[i] = w->origin[i];
	d.shadow_base = w->shadow_base;
	CK(cudaMemcpyAsync(w->d_set, &d, sizeof(d), cudaMemcpyHostToDevice, w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	return VP_OK;
}

VP_API int vp_world_upload(vp_world *w, const uint32_t *pool, uint64_t pool_words, const uint64_t *off,
			   const uint32_t *len, const uint16_t *shadow, uint64_t shadow_len, uint32_t shadow_w)
{
	if (!w || !pool || !off || !len || (!shadow && shadow_len)) return VP_EINVAL;
	const uint64_t N = 1ull << (3 * w->root_bitw);
	/* streams already on 16-byte boundaries are copied as laid out;
	 * otherwise they are repacked */
	bool aligned = true;
	for (uint32_t c = 0; c < w->nchunks; c++) {
		if (len[c] < 2 || off[c] + len[c] > pool_words) return VP_EINVAL;
		if (off[c] & 3u) aligned = false;
	}
	std::vector<uint64_t> noff;
	std::vector<uint32_t> packed;
	const uint32_t *src = pool;
	const uint64_t *src_off = off;
	uint64_t words = pool_words;
	if (!aligned) {
		noff.resize(w->nchunks);
		uint64_t total = 0;
		for (uint32_t c = 0; c < w->nchunks; c++) {
			noff[c] = total;
			total += (len[c] + 3u) & ~3u;
		}
		packed.assign(total, 0u);
		for (uint32_t c = 0; c < w->nchunks; c++)
			memcpy(&packed[noff[c]], pool + off[c], (size_t)len[c] * sizeof(uint32_t));
		src = packed.data();
		src_off = noff.data();
		words = total;
	}
	const uint64_t total = words + 8; /* vector loads may read up to 7 words past a terminator */
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	CK(cudaStreamSynchronize(st));
	int rc;
	/* reuse the allocations when they fit; keep headroom at the pool's tail
	 * for streams re-encoded by edits */
	if (!w->d_pool || w->pool_cap < total) {
		dev_free(w->d_pool);
		w->pool_cap = 0;
		const uint64_t cap = total + total / 4 + (16u << 20);
		if ((rc = dev_alloc(&w->d_pool, cap))) return rc;
		w->pool_cap = cap;
	}
	if (!w->d_shadow || w->shadow_cap < shadow_len + 8) {
		dev_free(w->d_shadow);
		w->shadow_cap = 0;
		if ((rc = dev_alloc(&w->d_shadow, shadow_len + 8))) return rc;
		w->shadow_cap = shadow_len + 8;
	}
	if (!w->d_check) {
		if ((rc = dev_alloc(&w->d_check, 2))) return rc;
		CK(cudaHostAlloc((void **)&w->h_check, 2 * sizeof(uint32_t), cudaHostAllocMapped));
		CK(cudaHostGetDevicePointer((void **)&w->h_check_dev, w->h_check, 0));
	}
	CK(cudaMemcpyAsync(w->d_pool, src, words * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(w->d_pool + words, 0, 8 * sizeof(uint32_t), st));
	w->pool_tail = total;
	w->pool_version++;
	CK(cudaMemcpyAsync(w->d_off, src_off, w->nchunks * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(w->d_len, len, w->nchunks * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	if (shadow_len)
		CK(cudaMemcpyAsync(w->d_shadow, shadow, shadow_len * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(w->d_shadow + shadow_len, 0, 8 * sizeof(uint16_t), st));
	/* every stream checked on the device before any kernel decodes it */
	CK(cudaMemsetAsync(w->d_check, 0, sizeof(uint32_t), st));
	CK(cudaMemsetAsync(w->d_check + 1, 0xFF, sizeof(uint32_t), st));
	cudaError_t e = launch_validate_streams(w->d_pool, w->d_off, w->d_len, w->nchunks, N, w->d_check,
						w->d_check + 1, st);
	if (e != cudaSuccess) return cuda_fail(e, "stream validation");
	k_fetch_words<<<1, 32, 0, st>>>(w->d_check, w->h_check_dev, 2u);
	CK(cudaGetLastError());
	CK(cudaStreamSynchronize(st));
	if (w->h_check[0]) {
		w->uploaded = false;
		return VP_EINVAL;
	}
	w->pool_words = total;
	/* the work orders depend on the lengths and on which chunks are all
	 * air: an upload that changes neither keeps them */
	std::vector<uint8_t> null(w->nchunks);
	for (uint32_t c = 0; c < w->nchunks; c++) null[c] = (len[c] == 2u && pool[off[c]] == N) ? 1u : 0u;
	const bool same = w->hlen.size() == w->nchunks && std::equal(len, len + w->nchunks, w->hlen.begin()) &&
			  w->hnull == null && !w->lens_stale;
	w->hlen.assign(len, len + w->nchunks);
	w->hnull.swap(null);
	if (!same) w->items_dirty = true;
	w->shadow_len = shadow_len;
	w->shadow_w = shadow_w;
	w->uploaded = true;
	return vpi_upload_setdesc(w);
}

VP_API int vp_world_generate(vp_world *w, int kind, uint64_t seed, int hshift, uint32_t pad_rows)
{
	if (!w || (kind != 1 && kind != 2) || hshift < 0 || hshift > 8) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	const uint32_t rb = (uint32_t)w->root_bitw, R = 1u << rb, N = R * R * R;
	const uint32_t nslab = 1u << (w->max_bitw[0] + w->max_bitw[1]);
	const uint32_t nz = 1u << w->max_bitw[2];
	GenArgs a;
	a.kind = (uint32_t)kind;
	a.seed = seed;
	a.hshift = hshift;
	a.root_bitw = rb;
	for (int i = 0; i < 3; i++) a.max_bitw[i] = (uint32_t)w->max_bitw[i];
	a.shadow_w = ((1u << w->max_bitw[0]) + (1u << w->max_bitw[1])) * R;
	const uint64_t Z = (uint64_t)nz * R;
	CK(cudaStreamSynchronize(st));
	dev_free(w->d_shadow);
	dev_free(w->d_pool);
	int rc;
	const uint64_t slen = (uint64_t)a.shadow_w * (Z + pad_rows);
	w->shadow_cap = 0;
	if ((rc = dev_alloc(&w->d_shadow, slen + 8))) return rc;
	w->shadow_cap = slen + 8;
	CK(cudaMemsetAsync(w->d_shadow, 0, (slen + 8) * 2u, st));
	/* pool: a first guess, grown (with copy) when a slab does not fit */
	uint64_t cap = (uint64_t)w->nchunks * 2048u + (uint64_t)nslab * (N + 8u) + (1u << 20);
	if ((rc = dev_alloc(&w->d_pool, cap))) return rc;
	uint8_t *vols = nullptr;
	uint64_t *noff = nullptr, *sc = nullptr;
	uint32_t *nlen = nullptr;
	if ((rc = dev_alloc(&vols, (size_t)nslab * N + 16u)) || (rc = dev_alloc(&noff, nslab)) ||
	    (rc = dev_alloc(&nlen, nslab)) || (rc = dev_alloc(&sc, 2))) {
		dev_free(vols);
		dev_free(noff);
		dev_free(nlen);
		return rc;
	}
	uint64_t tail = 0;
	cudaError_t e = cudaSuccess;
	for (uint32_t cz = 0; cz < nz && e == cudaSuccess && !rc; cz++) {
		e = launch_gen_slab(a, cz, vols, st);
		if (e == cudaSuccess) e = launch_gen_shadow(a, cz, vols, w->d_shadow, slen, st);
		for (int attempt = 0; attempt < 2 && e == cudaSuccess; attempt++) {
			unsigned long long h[2] = {0, 0};
			e = cudaMemsetAsync(sc, 0, 2 * sizeof(uint64_t), st);
			if (e == cudaSuccess)
				e = launch_rle_encode(vols, nslab, N, w->d_pool + tail, cap - tail, (unsigned long long *)sc,
						      noff, nlen, (uint32_t *)(sc + 1), st);
			if (e == cudaSuccess) e = cudaMemcpyAsync(h, sc, sizeof(h), cudaMemcpyDeviceToHost, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			if (e != cudaSuccess) break;
			if (!((uint32_t)h[1] & kStatusOverflow)) {
				e = launch_scatter_slab(noff, nlen, nslab, cz * nslab, tail, w->d_off, w->d_len, st);
				w->pool_version++;
				tail += h[0];
				break;
			}
			/* grow the pool, keeping what is written */
			const uint64_t ncap = cap + cap / 2 + (uint64_t)nslab * (N + 8u);
			uint32_t *np = nullptr;
			if ((rc = dev_alloc(&np, ncap))) break;
			e = cudaMemcpyAsync(np, w->d_pool, tail * 4u, cudaMemcpyDeviceToDevice, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			dev_free(w->d_pool);
			w->d_pool = np;
			cap = ncap;
		}
	}
	dev_free(vols);
	dev_free(noff);
	dev_free(nlen);
	dev_free(sc);
	if (rc) return rc;
	if (e != cudaSuccess) return cuda_fail(e, "world generation");
	/* headroom at the tail for streams re-encoded by edits */
	const uint64_t want = tail + tail / 4 + (64u << 20);
	if (cap < want) {
		uint32_t *np = nullptr;
		if ((rc = dev_alloc(&np, want))) return rc;
		CK(cudaMemcpyAsync(np, w->d_pool, tail * 4u, cudaMemcpyDeviceToDevice, st));
		CK(cudaStreamSynchronize(st));
		dev_free(w->d_pool);
		w->d_pool = np;
		cap = want;
	}
	w->pool_cap = cap;
	w->pool_tail = tail;
	w->pool_words = tail;
	w->shadow_len = slen;
	w->shadow_w = a.shadow_w;
	w->shadow_base = 0;
	w->hlen.resize(w->nchunks);
	CK(cudaMemcpyAsync(w->hlen.data(), w->d_len, w->nchunks * 4u, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	w->hnull.clear();
	w->uploaded = true;
	w->items_dirty = true;
	return vpi_upload_setdesc(w);
}

VP_API int vp_world_set_handoff(vp_world *w, int on)
{
	if (!w) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	int rc = vpi_pipe_drain(w);
	if (rc) return rc;
	CK(cudaStreamSynchronize(w->ctx->stream));
	w->handoff = on != 0;
	w->dec_failed = false;
	if (!w->handoff) {
		dev_free(w->d_dec);
		dev_free(w->d_dec_slot);
		w->dec_bytes = 0;
		w->h_dec_slot.clear();
	}
	return VP_OK;
}

VP_API int vp_world_handoff_bytes(vp_world *w, uint64_t *bytes)
{
	if (!w || !bytes) return VP_EINVAL;
	*bytes = w->d_dec ? w->dec_bytes : 0u;
	return VP_OK;
}

VP_API int vp_world_set_modes(vp_world *w, const uint8_t *make_mesh)
{
	if (!w) return VP_EINVAL;
	for (uint32_t c = 0; c < w->nchunks; c++) w->modes[c] = make_mesh ? (make_mesh[c] ? 1 : 0) : 0;
	w->items_dirty = true;
	return VP_OK;
}

/* flags[c] = 1 when chunk c is all air (one air run and the terminator) */
__global__ void k_null_flags(const SetDesc *__restrict__ set, uint32_t n, uint32_t N, uint8_t *flags)
{
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c < n) flags[c] = (set->len[c] == 2u && set->pool[set->off[c]] == N) ? 1u : 0u;
}

/* The shell pass of a full rebuild: the decoding shell kernel over the
 * chunks of more than one run, the single-run ones without decoding (<=
 * 64^3; the 128^3 shell kernel is persistent and takes every chunk). Call
 * after ensure_items. */
static void set_shell_items(vp_world *w, GeoLaunch &L)
{
	if (w->root_bitw <= 6 && w->d_shell_items) {
		L.shell_items = w->d_shell_items;
		L.n_shell = w->n_shell_multi;
		L.uni_items = w->d_shell_items + w->n_shell_multi;
		L.n_uni = w->nchunks - w->n_shell_multi;
	} else {
		L.shell_items = w->d_items;
		L.n_shell = w->nchunks;
	}
}

static int ensure_items(vp_world *w)
{
	if (w->lens_stale) {
		/* edits re-encoded streams on the device: refresh the lengths the
		 * work orders are built from */
		w->hlen.resize(w->nchunks);
		CK(cudaMemcpyAsync(w->hlen.data(), w->d_len, w->nchunks * 4u, cudaMemcpyDeviceToHost, w->ctx->stream));
		CK(cudaStreamSynchronize(w->ctx->stream));
		w->lens_stale = false;
		w->hnull.clear();
		w->items_dirty = true;
	}
	if (!w->items_dirty) return VP_OK;
	/* which chunks are all air (known on the host after an upload; after a
	 * generation, a file load or edits, read from the device once) */
	if (w->hnull.size() != w->nchunks) {
		int rc0;
		if (!w->d_null && (rc0 = dev_alloc(&w->d_null, w->nchunks))) return rc0;
		w->hnull.resize(w->nchunks);
		k_null_flags<<<(w->nchunks + 255) / 256, 256, 0, w->ctx->stream>>>(w->d_set, w->nchunks,
										    1u << (3 * w->root_bitw), w->d_null);
		CK(cudaGetLastError());
		CK(cudaMemcpyAsync(w->hnull.data(), w->d_null, w->nchunks, cudaMemcpyDeviceToHost, w->ctx->stream));
		CK(cudaStreamSynchronize(w->ctx->stream));
	}
	/* those whose +x, +y and +z neighbours are all air (or outside) too
	 * have no geometry */
	const std::vector<uint8_t> &null = w->hnull;
	const uint32_t bx = w->max_bitw[0], by = w->max_bitw[1], bz = w->max_bitw[2];
	auto air = [&](uint32_t c, int dx, int dy, int dz) {
		const uint32_t x = (c & ((1u << bx) - 1u)) + dx, y = ((c >> bx) & ((1u << by) - 1u)) + dy,
			       z = (c >> (bx + by)) + dz;
		if (x >> bx || y >> by || z >> bz) return true; /* outside the world */
		return null[(z << (bx + by)) | (y << bx) | x] != 0;
	};
	/* longest first: a chunk's cost grows with its run count, and a meshed
	 * chunk costs about three times a splatted one; chunks without geometry
	 * last */
	std::vector<uint32_t> order(w->nchunks);
	std::vector<uint64_t> cost(w->nchunks);
	uint32_t n_geo = 0;
	for (uint32_t c = 0; c < w->nchunks; c++) {
		order[c] = c;
		const uint64_t len = c < w->hlen.size() ? w->hlen[c] : 2u;
		/* (a chunk holding a handoff slot is in the decoding shell list,
		 * which does not zero records: it keeps its geometry pass) */
		const bool slot = c < w->h_dec_slot.size() && w->h_dec_slot[c] != kNoSlot;
		const bool empty = w->root_bitw <= 6 && !slot && null[c] && air(c, 1, 0, 0) && air(c, 0, 1, 0) &&
				   air(c, 0, 0, 1);
		cost[c] = empty ? 0u : (len + 64u) * (w->modes[c] ? 3u : 1u);
		n_geo += empty ? 0u : 1u;
	}
	std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
	w->n_geo = n_geo;
	std::vector<uint8_t> no_geometry(w->nchunks, 0);
	for (uint32_t k = n_geo; k < w->nchunks; k++) no_geometry[order[k]] = 1;
	std::vector<WorkItem> it(w->nchunks);
	for (uint32_t k = 0; k < w->nchunks; k++) {
		const uint32_t c = order[k];
		it[k].set = 0;
		it[k].chunk = c;
		it[k].flags = w->modes[c] ? kItemMesh : 0u;
		it[k].slot = c;
	}
	CK(cudaMemcpyAsync(w->d_items, it.data(), it.size() * sizeof(WorkItem), cudaMemcpyHostToDevice,
			   w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	w->h_items.swap(it);
	/* shell order: chunks of more than one run, and any chunk with a
	 * handoff slot (the shell pass stores its decoded state), longest
	 * first; then the single-run chunks */
	{
		std::vector<uint32_t> multi, uni;
		for (uint32_t c = 0; c < w->nchunks; c++) {
			const uint32_t len = c < w->hlen.size() ? w->hlen[c] : 2u;
			const bool slot = c < w->h_dec_slot.size() && w->h_dec_slot[c] != kNoSlot;
			(len > 2u || slot ? multi : uni).push_back(c);
		}
		std::stable_sort(multi.begin(), multi.end(), [&](uint32_t a, uint32_t b) {
			const uint32_t la = a < w->hlen.size() ? w->hlen[a] : 2u, lb = b < w->hlen.size() ? w->hlen[b] : 2u;
			return la > lb;
		});
		std::vector<WorkItem> sh;
		sh.reserve(w->nchunks);
		for (uint32_t c : multi) sh.push_back(WorkItem{0u, c, 0u, c});
		for (uint32_t c : uni) sh.push_back(WorkItem{0u, c, no_geometry[c] ? kItemEmpty : 0u, c});
		int rc;
		if (!w->d_shell_items && (rc = dev_alloc(&w->d_shell_items, w->nchunks))) return rc;
		CK(cudaMemcpyAsync(w->d_shell_items, sh.data(), sh.size() * sizeof(WorkItem), cudaMemcpyHostToDevice,
				   w->ctx->stream));
		CK(cudaStreamSynchronize(w->ctx->stream));
		w->n_shell_multi = (uint32_t)multi.size();
	}
	w->items_dirty = false;
	w->stream_slabs = 0; /* the slab orders follow the work order */
	return VP_OK;
}

uint8_t *vpi_decoded(vp_world *w)
{
	const size_t per = decoded_bytes_per_chunk(w->root_bitw);
	if (!per || !w->handoff || w->dec_failed) return nullptr;
	if (w->d_dec) return w->d_dec;
	/* one slot per chunk of more than one run (single-run chunks decode in
	 * no time); chunks whose length changes later keep or lack a slot,
	 * which only decides whether the geometry pass loads or decodes */
	std::vector<uint32_t> slot(w->nchunks, kNoSlot);
	uint32_t k = 0;
	for (uint32_t c = 0; c < w->nchunks; c++)
		if (c < w->hlen.size() && w->hlen[c] > 2u) slot[c] = k++;
	const size_t need = (size_t)k * per;
	size_t free_b = 0, total_b = 0;
	/* keep 4 GiB free for arenas and the rest, and at most a quarter of the
	 * device; without room, decode twice */
	if (!k || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < need + (4ull << 30) ||
	    need > total_b / 4 || cudaMalloc(&w->d_dec, need) != cudaSuccess) {
		cudaGetLastError();
		w->d_dec = nullptr;
		w->dec_failed = true;
		return nullptr;
	}
	if (dev_alloc(&w->d_dec_slot, w->nchunks) ||
	    cudaMemcpy(w->d_dec_slot, slot.data(), w->nchunks * 4u, cudaMemcpyHostToDevice) != cudaSuccess) {
		cudaGetLastError();
		dev_free(w->d_dec);
		dev_free(w->d_dec_slot);
		w->dec_failed = true;
		return nullptr;
	}
	w->dec_bytes = need;
	w->h_dec_slot.swap(slot);
	return w->d_dec;
}

int vpi_ensure_arenas(vp_world *w)
{
	/* first guess: 16 KiB of each output per chunk, at least 16 MiB; an
	 * overflowing rebuild grows the arena to what it needed and reruns */
	for (int a = 0; a < 3; a++) {
		if (w->d_arena[a]) continue;
		uint64_t units = std::max<uint64_t>((uint64_t)w->nchunks * 1024u, 1u << 20);
		cudaError_t e = cudaMalloc(&w->d_arena[a], units * 16u);
		if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(arena)");
		w->cap[a] = units;
	}
	return VP_OK;
}

VP_API int vp_world_reserve(vp_world *w, const uint64_t bytes[3])
{
	if (!w || !bytes) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	CK(cudaStreamSynchronize(w->ctx->stream));
	int rc0 = vpi_pipe_drain(w);
	if (rc0) return rc0;
	for (int a = 0; a < 3; a++) {
		const uint64_t units = std::max<uint64_t>((bytes[a] + 15u) / 16u, 1u);
		dev_free(w->d_arena[a]);
		w->cap[a] = 0;
		cudaError_t e = cudaMalloc(&w->d_arena[a], units * 16u);
		if (e != cudaSuccess) {
			w->d_arena[a] = nullptr;
			return cuda_fail(e, "cudaMalloc(arena)");
		}
		w->cap[a] = units;
	}
	return VP_OK;
}

static_assert(kMaxLevels == VP_MAX_LEVELS, "the node tables hold every level k_group_tables writes");

static int enqueue_group(vp_world *w, int lod_max, uint64_t svl_cap_units)
{
	cudaStream_t st = w->ctx->stream;
	const size_t L = (size_t)VP_MAX_LEVELS, n = w->nchunks;
	int rc;
	if (!w->d_gcounts) {
		if ((rc = dev_alloc(&w->d_gcounts, L * n)) || (rc = dev_alloc(&w->d_gtotal, L)) ||
		    (rc = dev_alloc(&w->d_node_off, L * n)) || (rc = dev_alloc(&w->d_node_items, L * n)))
			return rc;
	}
	if (w->garena_units < w->cap[0]) {
		dev_free(w->d_garena);
		w->garena_units = 0;
		if ((rc = dev_alloc(&w->d_garena, (size_t)w->cap[0] * 8u))) return rc;
		w->garena_units = w->cap[0];
	}
	GroupArgs a;
	for (int i = 0; i < 3; i++) a.max_bitw[i] = (uint32_t)w->max_bitw[i];
	a.counts = w->d_gcounts;
	a.level_total = w->d_gtotal;
	a.node_off = w->d_node_off;
	a.node_items = w->d_node_items;
	a.svl = (const int16_t *)w->d_arena[0];
	a.out = w->d_garena;
	a.svl_cursor = w->d_cursors;
	a.svl_cap_units = svl_cap_units;
	a.out_cap = (uint64_t)w->garena_units * 8u;
	cudaError_t e = launch_group(w->d_outs, w->nchunks, lod_max, a, st);
	if (e != cudaSuccess) return cuda_fail(e, "group launch");
	w->launches += lod_max >= 1 ? 3 : 1; /* node tables and counts, then scan and copy */
	w->grouped_lod = lod_max;
	return VP_OK;
}

static int enqueue_rebuild(vp_world *w, int lod_max, unsigned flags)
{
	vp_ctx *ctx = w->ctx;
	cudaStream_t st = ctx->stream;
	int rc;
	if ((rc = vpi_pipe_drain(w))) return rc;
	if ((rc = ensure_items(w)) || (rc = vpi_ensure_arenas(w))) return rc;
	CK(cudaMemsetAsync(w->d_cursors, 0, 3 * sizeof(unsigned long long), st));
	CK(cudaMemsetAsync(w->d_queue, 0, sizeof(unsigned int), st));
	GeoLaunch L;
	memset(&L, 0, sizeof(L));
	L.big_scratch = w->d_big;
	L.big_slots = w->big_slots;
	L.sets = w->d_set;
	L.items = w->d_items;
	L.n_items = w->nchunks;
	set_shell_items(w, L);
	L.threads = 512;
	L.outs = w->d_outs;
	L.lod_max = lod_max;
	L.decoded = vpi_decoded(w); /* every chunk is shelled before any geometry */
	L.dec_slot = w->d_dec_slot;
	Arena *ar[3] = {&L.svl, &L.vbo, &L.ibo};
	for (int a = 0; a < 3; a++) {
		ar[a]->base = w->d_arena[a];
		ar[a]->cap_units = w->cap[a];
		ar[a]->cursor = w->d_cursors + a;
	}
	if (flags & VP_REBUILD_PERSISTENT) {
		const int per_sm = geometry_ctas_per_sm(w->root_bitw, (int)L.threads);
		L.queue = w->d_queue;
		L.ctas = (uint32_t)(ctx->sm_count * std::max(per_sm, 1));
	}
	cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
	if (ctx->timing) {
		cudaEventCreate(&e0);
		cudaEventCreate(&e1);
		cudaEventCreate(&e2);
		cudaEventCreate(&e3);
		cudaEventRecord(e0, st);
	}
	cudaError_t e = cudaSuccess;
	if (flags & (VP_REBUILD_PLAIN | VP_REBUILD_CONCURRENT)) {
		/* one launch per chunk and pass: every shell, then every chunk's
		 * geometry (a chunk reads its neighbours' shells); on the context
		 * stream, or round-robin over forked streams */
		const bool conc = (flags & VP_REBUILD_CONCURRENT) != 0;
		if (conc && (rc = vpi_plain_fork(w->plain, st))) return rc;
		for (uint32_t k = 0; k < w->nchunks && e == cudaSuccess; k++) {
			GeoLaunch Ls = L;
			Ls.n_items = 0;
			Ls.shell_items = w->d_items + k;
			Ls.n_shell = 1;
			Ls.n_uni = 0; /* every chunk its own shell launch, single-run ones too */
			Ls.run_shell = 1;
			if (conc && w->root_bitw == 7) { /* a scratch slot per stream */
				Ls.big_scratch = w->d_big + (size_t)(k % kPlainStreams) * big_scratch_slot_bytes();
				Ls.big_slots = 1;
			}
			e = launch_geometry(w->root_bitw, Ls, conc ? w->plain.s[k % kPlainStreams] : st);
		}
		if (conc && e == cudaSuccess && ((rc = vpi_plain_join(w->plain, st)) || (rc = vpi_plain_fork(w->plain, st))))
			return rc;
		if (ctx->timing) cudaEventRecord(e1, st);
		for (uint32_t k = 0; k < w->nchunks && e == cudaSuccess; k++) {
			GeoLaunch Lg = L;
			Lg.run_shell = 0;
			Lg.items = w->d_items + k;
			Lg.n_items = 1;
			Lg.queue = nullptr;
			if (conc && w->root_bitw == 7) {
				Lg.big_scratch = w->d_big + (size_t)(k % kPlainStreams) * big_scratch_slot_bytes();
				Lg.big_slots = 1;
			}
			e = launch_geometry(w->root_bitw, Lg, conc ? w->plain.s[k % kPlainStreams] : st);
		}
		if (e != cudaSuccess) return cuda_fail(e, "plain launches");
		if (conc && (rc = vpi_plain_join(w->plain, st))) return rc;
		w->launches += 2 * w->nchunks;
	} else {
		L.run_shell = 1;
		GeoLaunch Ls = L;
		Ls.n_items = 0;
		e = launch_geometry(w->root_bitw, Ls, st);
		if (e != cudaSuccess) return cuda_fail(e, "shell launch");
		if (ctx->timing) cudaEventRecord(e1, st);
		GeoLaunch Lg = L;
		Lg.run_shell = 0;
		Lg.n_items = w->n_geo;
		e = launch_geometry(w->root_bitw, Lg, st);
		if (e != cudaSuccess) return cuda_fail(e, "geometry launch");
		w->launches += 2; /* shell (single-run chunks in its last CTAs), geometry */
	}
	if (ctx->timing) cudaEventRecord(e2, st);
	w->grouped_lod = -1;
	if (flags & VP_REBUILD_GROUP) {
		int rc2 = enqueue_group(w, lod_max, w->cap[0]);
		if (rc2) return rc2;
	}
	if (ctx->timing) {
		cudaEventRecord(e3, st);
		w->ev.push_back(e0);
		w->ev.push_back(e1);
		w->ev.push_back(e2);
		w->ev.push_back(e3);
	}
	w->last_lod = lod_max;
	w->last_flags = flags;
	return VP_OK;
}

VP_API int vp_world_rebuild(vp_world *w, int lod_max, unsigned flags)
{
	if (!w || !w->uploaded) return VP_EINVAL;
	if (lod_max < 0 || lod_max >= VP_MAX_LEVELS) return VP_EUNSUPPORTED;
	CK(cudaSetDevice(w->ctx->device));
	return enqueue_rebuild(w, lod_max, flags);
}

VP_API int vp_world_finish(vp_world *w)
{
	if (!w) return VP_EINVAL;
	cudaStream_t st = w->ctx->stream;
	for (int attempt = 0; attempt < 4; attempt++) {
		unsigned long long cur[3];
		CK(cudaMemcpyAsync(cur, w->d_cursors, sizeof(cur), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		bool grow = false;
		for (int a = 0; a < 3; a++) {
			if (cur[a] <= w->cap[a]) continue;
			grow = true;
			uint64_t units = cur[a] + cur[a] / 4 + 1024;
			dev_free(w->d_arena[a]);
			cudaError_t e = cudaMalloc(&w->d_arena[a], units * 16u);
			if (e != cudaSuccess) {
				w->cap[a] = 0;
				return cuda_fail(e, "cudaMalloc(arena growth)");
			}
			w->cap[a] = units;
		}
		if (!grow) return VP_OK;
		int rc = enqueue_rebuild(w, w->last_lod, w->last_flags);
		if (rc) return rc;
	}
	return VP_EOVERFLOW;
}

VP_API int vp_world_read_outputs(vp_world *w, void *svl, uint64_t svl_bytes, void *vbo, uint64_t vbo_bytes, void *ibo,
				 uint64_t ibo_bytes, uint64_t used_bytes[3])
{
	if (!w || !used_bytes) return VP_EINVAL;
	cudaStream_t st = w->ctx->stream;
	unsigned long long cur[3];
	CK(cudaMemcpyAsync(cur, w->d_cursors, sizeof(cur), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	void *dst[3] = {svl, vbo, ibo};
	const uint64_t cap[3] = {svl_bytes, vbo_bytes, ibo_bytes};
	int rc = VP_OK;
	for (int a = 0; a < 3; a++) {
		used_bytes[a] = (uint64_t)cur[a] * 16u;
		if (cur[a] > w->cap[a]) return VP_EOVERFLOW; /* an unfinished, overflowed rebuild */
		if (!dst[a] || !used_bytes[a]) continue;
		if (used_bytes[a] > cap[a]) {
			rc = VP_EOVERFLOW;
			continue;
		}
		CK(cudaMemcpyAsync(dst[a], w->d_arena[a], used_bytes[a], cudaMemcpyDeviceToHost, st));
	}
	CK(cudaStreamSynchronize(st));
	return rc;
}

static CullArgs cull_args(const vp_world *w, const float *origin, int top)
{
	CullArgs a;
	memset(&a, 0, sizeof(a));
	for (int i = 0; i < 3; i++) a.origin[i] = origin[i];
	a.root_bitw = (uint32_t)w->root_bitw;
	for (int i = 0; i < 3; i++) {
		a.max_bitw[i] = (uint32_t)w->max_bitw[i];
		a.roots[i] = ((1u << w->max_bitw[i]) >> top) + 1u;
	}
	a.top = (uint32_t)top;
	for (int l = 0; l < kMaxLevels; l++)
		for (int i = 0; i < 3; i++) a.nodes[l][i] = 1u << (w->max_bitw[i] - std::min(l, w->max_bitw[i]));
	a.outs = w->d_outs;
	a.node_items = w->d_node_items;
	a.nchunks = w->nchunks;
	return a;
}

VP_API int vp_world_cull(vp_world *w, const float view_proj[16], const float lod_origin[3], int top_lod,
			 uint32_t *mesh_out, uint32_t mesh_cap, uint32_t *n_mesh, uint32_t *svl_out, uint32_t svl_cap,
			 uint32_t *n_svl)
{
	if (!w || !view_proj || !lod_origin || !n_mesh || !n_svl) return VP_EINVAL;
	if ((mesh_cap && !mesh_out) || (svl_cap && !svl_out)) return VP_EINVAL;
	/* the drawn nodes' splats are the grouped lists of the last rebuild */
	if (top_lod < 0 || top_lod > w->grouped_lod || top_lod >= kMaxLevels) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	CullArgs a = cull_args(w, lod_origin, top_lod);
	memcpy(a.view_proj, view_proj, sizeof(a.view_proj));
	const uint64_t nslots = cull_slots(a);
	const uint64_t nblocks = (nslots + 1023) / 1024;
	int rc;
	if (w->cull_slots_cap < nslots) {
		dev_free(w->d_cull_slots);
		w->cull_slots_cap = 0;
		if ((rc = dev_alloc(&w->d_cull_slots, nslots))) return rc;
		w->cull_slots_cap = nslots;
	}
	if (w->cull_blocks_cap < 2 * nblocks) {
		dev_free(w->d_cull_blocks);
		w->cull_blocks_cap = 0;
		if ((rc = dev_alloc(&w->d_cull_blocks, 2 * nblocks))) return rc;
		w->cull_blocks_cap = 2 * nblocks;
	}
	/* the drawn nodes cover every chunk at most once: nchunks entries each */
	if (!w->d_cull_out && (rc = dev_alloc(&w->d_cull_out, 2 * (size_t)w->nchunks + 2))) return rc;
	a.slots = w->d_cull_slots;
	uint32_t *mq = w->d_cull_out, *sq = w->d_cull_out + w->nchunks, *tot = w->d_cull_out + 2 * (size_t)w->nchunks;
	cudaError_t e = launch_cull(a, w->d_cull_blocks, tot, mq, w->nchunks, sq, w->nchunks, st);
	if (e != cudaSuccess) return cuda_fail(e, "cull launch");
	w->launches += 4;
	uint32_t t[2];
	CK(cudaMemcpyAsync(t, tot, sizeof(t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	*n_mesh = t[0];
	*n_svl = t[1];
	const uint32_t cm = std::min(t[0], mesh_cap), cs = std::min(t[1], svl_cap);
	if (cm) CK(cudaMemcpyAsync(mesh_out, mq, cm * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	if (cs) CK(cudaMemcpyAsync(svl_out, sq, cs * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return (t[0] > mesh_cap || t[1] > svl_cap) ? VP_EOVERFLOW : VP_OK;
}

VP_API int vp_world_camera_modes(vp_world *w, const float lod_origin[3], uint8_t *make_mesh_out)
{
	if (!w || !lod_origin) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	int rc;
	if (!w->d_flags && (rc = dev_alloc(&w->d_flags, w->nchunks))) return rc;
	const CullArgs a = cull_args(w, lod_origin, 0);
	cudaError_t e = launch_mesh_flags(a, w->d_flags, st);
	if (e != cudaSuccess) return cuda_fail(e, "mesh flags");
	w->launches += 1;
	CK(cudaMemcpyAsync(w->modes.data(), w->d_flags, w->nchunks, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	w->items_dirty = true;
	if (make_mesh_out) memcpy(make_mesh_out, w->modes.data(), w->nchunks);
	return VP_OK;
}

VP_API int vp_world_raycast(vp_world *w, uint32_t n, const float *origins, const float *vectors, uint8_t *voxels,
			    uint32_t *coords, int8_t *normals)
{
	if (!w || !w->uploaded || (n && (!origins || !vectors || !voxels || !coords || !normals))) return VP_EINVAL;
	if (!n) return VP_OK;
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	int rc;
	if (w->runidx_version != w->pool_version) {
		if (w->runidx_cap < w->pool_cap) {
			dev_free(w->d_runidx);
			w->runidx_cap = 0;
			if ((rc = dev_alloc(&w->d_runidx, w->pool_cap))) return rc;
			w->runidx_cap = w->pool_cap;
		}
		cudaError_t e = launch_run_starts(w->d_pool, w->d_off, w->d_len, w->nchunks, w->d_runidx, st);
		if (e != cudaSuccess) return cuda_fail(e, "run-start index");
		w->launches += 1;
		w->runidx_version = w->pool_version;
	}
	/* ray buffers: origins, vectors (12 B each), coords (12 B), voxel, normal (3 B) */
	const size_t need = (size_t)n * 40u;
	if (w->rays_cap < need) {
		dev_free(w->d_rays);
		w->rays_cap = 0;
		if ((rc = dev_alloc(&w->d_rays, need))) return rc;
		w->rays_cap = need;
	}
	float *d_o = (float *)w->d_rays, *d_v = d_o + 3 * (size_t)n;
	uint32_t *d_c = (uint32_t *)(d_v + 3 * (size_t)n);
	uint8_t *d_vox = (uint8_t *)(d_c + 3 * (size_t)n);
	int8_t *d_n = (int8_t *)(d_vox + n);
	CK(cudaMemcpyAsync(d_o, origins, 12u * n, cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(d_v, vectors, 12u * n, cudaMemcpyHostToDevice, st));
	RayWorld W;
	W.pool = w->d_pool;
	W.off = w->d_off;
	W.len = w->d_len;
	W.runidx = w->d_runidx;
	W.root_bitw = (uint32_t)w->root_bitw;
	for (int i = 0; i < 3; i++) W.max_bitw[i] = (uint32_t)w->max_bitw[i];
	cudaError_t e = launch_raycast(W, d_o, d_v, n, d_vox, d_c, d_n, st);
	if (e != cudaSuccess) return cuda_fail(e, "raycast");
	w->launches += 1;
	CK(cudaMemcpyAsync(voxels, d_vox, n, cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(coords, d_c, 12u * n, cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(normals, d_n, 3u * n, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

static_assert(sizeof(vp_camera) == sizeof(RenderCam), "camera layout");

static size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

VP_API int vp_world_render(vp_world *w, const vp_camera *cam, const uint32_t *mesh_queue, uint32_t n_mesh,
			   const uint32_t *svl_queue, uint32_t n_svl, uint32_t *rgba, float *depth, uint64_t *stats)
{
	if (!w || !cam || !rgba || cam->width <= 0 || cam->height <= 0) return VP_EINVAL;
	const uint64_t npx = (uint64_t)cam->width * (uint64_t)cam->height;
	if (npx > (1ull << 26) || !(cam->far_plane > 0.0f)) return VP_EINVAL;
	if ((n_mesh && !mesh_queue) || (n_svl && !svl_queue)) return VP_EINVAL;
	for (uint32_t i = 0; i < n_mesh; i++)
		if (mesh_queue[i] >= w->nchunks) return VP_EINVAL;
	for (uint32_t i = 0; i < n_svl; i++) {
		const uint32_t l = svl_queue[i] >> 24, node = svl_queue[i] & 0xFFFFFFu;
		if ((int)l > w->grouped_lod || node >= w->nchunks) return VP_EINVAL;
	}
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	int rc;
	/* scratch: queues, segments + first splat, meshes + first triangle, totals */
	const size_t o_sq = 0, o_mq = a256(o_sq + 4u * (size_t)n_svl);
	const size_t o_seg = a256(o_mq + 4u * (size_t)n_mesh);
	const size_t o_sf = a256(o_seg + sizeof(RenderSeg) * n_svl);
	const size_t o_me = a256(o_sf + 8u * (size_t)n_svl);
	const size_t o_mf = a256(o_me + sizeof(RenderMesh) * n_mesh);
	const size_t o_tot = a256(o_mf + 8u * (size_t)n_mesh);
	const size_t o_bc = a256(o_tot + 16u);
	const size_t prep_bytes = a256(o_bc + 8u);
	if (w->render_cap < prep_bytes) {
		dev_free(w->d_render);
		w->render_cap = 0;
		if ((rc = dev_alloc(&w->d_render, prep_bytes))) return rc;
		w->render_cap = prep_bytes;
	}
	uint8_t *R = w->d_render;
	if (n_svl) CK(cudaMemcpyAsync(R + o_sq, svl_queue, 4u * (size_t)n_svl, cudaMemcpyHostToDevice, st));
	if (n_mesh) CK(cudaMemcpyAsync(R + o_mq, mesh_queue, 4u * (size_t)n_mesh, cudaMemcpyHostToDevice, st));
	uint64_t *tot = (uint64_t *)(R + o_tot);
	CK(cudaMemsetAsync(tot, 0, 16, st));
	cudaError_t e = launch_render_prep((const uint32_t *)(R + o_sq), n_svl, w->d_node_off, w->d_node_items,
					   w->nchunks, (const uint32_t *)(R + o_mq), n_mesh, w->d_outs,
					   (RenderSeg *)(R + o_seg), (uint64_t *)(R + o_sf), (RenderMesh *)(R + o_me),
					   (uint64_t *)(R + o_mf), tot, st);
	if (e != cudaSuccess) return cuda_fail(e, "render prep");
	uint64_t totals[2];
	CK(cudaMemcpyAsync(totals, tot, 16, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	/* frame words, RGBA, depth, and the two lists of large footprints */
	const uint32_t big_cap = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(totals[0] + totals[1], 1), 4u << 20);
	const size_t f_rgba = a256(8u * npx), f_depth = a256(f_rgba + 4u * npx), f_raya = a256(f_depth + 4u * npx);
	const size_t f_rayb = a256(f_raya + 16u * npx), f_big = a256(f_rayb + 8u * npx);
	const size_t frame_bytes = a256(f_big + 16u * (size_t)big_cap);
	if (w->frame_cap < frame_bytes) {
		dev_free(w->d_frame);
		w->frame_cap = 0;
		if ((rc = dev_alloc(&w->d_frame, frame_bytes))) return rc;
		w->frame_cap = frame_bytes;
	}
	RenderArgs a;
	memset(&a, 0, sizeof(a));
	memcpy(&a.cam, cam, sizeof(a.cam));
	const float llen = sqrtf(1.0f + 1.0f);
	a.light[0] = -1.0f / llen;
	a.light[1] = 1.0f / llen;
	a.light[2] = 0.0f / llen;
	/* one IEEE single-precision division (both hosts evaluate float
	 * expressions in float), the value every fragment computed before */
	a.fog_start = 256.0f / cam->far_plane;
	a.splats = w->d_garena;
	a.splats_l0 = (const int16_t *)w->d_arena[0];
	a.segs = (const RenderSeg *)(R + o_seg);
	a.seg_first = (const uint64_t *)(R + o_sf);
	a.nseg = n_svl;
	a.nsplats = totals[0];
	a.vbo = (const int16_t *)w->d_arena[1];
	a.ibo = (const uint32_t *)w->d_arena[2];
	a.meshes = (const RenderMesh *)(R + o_me);
	a.mesh_first = (const uint64_t *)(R + o_mf);
	a.nmesh = n_mesh;
	a.ntris = totals[1];
	a.frame = (unsigned long long *)w->d_frame;
	a.ray_a = (float4 *)(w->d_frame + f_raya);
	a.ray_b = (float2 *)(w->d_frame + f_rayb);
	a.big = (uint64_t *)(w->d_frame + f_big);
	a.big_count = (uint32_t *)(R + o_bc);
	a.big_cap = big_cap;
	if (n_svl && !a.splats) return VP_EINVAL;
	uint32_t *d_rgba = (uint32_t *)(w->d_frame + f_rgba);
	float *d_depth = (float *)(w->d_frame + f_depth);
	e = launch_render(a, d_rgba, depth ? d_depth : nullptr, w->ctx->sm_count, st);
	if (e != cudaSuccess) return cuda_fail(e, "render");
	w->launches += 7;
	uint32_t big[2];
	CK(cudaMemcpyAsync(rgba, d_rgba, 4u * npx, cudaMemcpyDeviceToHost, st));
	if (depth) CK(cudaMemcpyAsync(depth, d_depth, 4u * npx, cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(big, a.big_count, 8, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (stats) {
		stats[0] = totals[0];
		stats[1] = totals[1];
		stats[2] = big[0];
		stats[3] = big[1];
	}
	return (big[0] > big_cap || big[1] > big_cap) ? VP_EOVERFLOW : VP_OK;
}

/* Pipelined rebuild into half h: wait for its copies and rebase the result
 * records they delivered (device offsets index the whole arena; host
 * offsets index the host buffers, which start at the half's base). */
static int settle_half(vp_world *w, int h)
{
	if (!w->half_busy[h]) return VP_OK;
	CK(cudaEventSynchronize(w->half_done[h]));
	vp_world::Rebase &rb = w->rebase[h];
	for (uint32_t c = 0; c < rb.n; c++) {
		vp_chunk_result &r = rb.res[c];
		if (r.svl_total) r.svl_off -= rb.base[0] * 8u;
		if (r.vbo_items) r.vbo_off -= rb.base[1] * 8u;
		if (r.ibo_items) r.ibo_off -= rb.base[2] * 4u;
	}
	rb.res = nullptr;
	rb.n = 0;
	w->half_busy[h] = false;
	return VP_OK;
}

int vpi_pipe_drain(vp_world *w)
{
	int rc;
	if ((rc = vpi_server_quiesce(w))) return rc;
	const int older = w->pipe_half; /* the next half to be used was written first */
	if ((rc = settle_half(w, older)) || (rc = settle_half(w, older ^ 1))) return rc;
	return VP_OK;
}

VP_API int vp_world_outputs_wait(vp_world *w)
{
	if (!w) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	return vpi_pipe_drain(w);
}

/* The streamed rebuild. Synchronous: the whole arenas, everything finished
 * on return. Pipelined: the arenas' half `pipe_half` and its own result
 * records; returns once this call's copies are issued and the previous
 * call's copies (which ran under this call's compute) have finished. */
static int stream_rebuild(vp_world *w, int lod_max, unsigned flags, int slabs, void *svl, uint64_t svl_bytes,
			  void *vbo, uint64_t vbo_bytes, void *ibo, uint64_t ibo_bytes, vp_chunk_result *results,
			  uint64_t used_bytes[3], bool pipelined)
{
	CK(cudaSetDevice(w->ctx->device));
	vp_ctx *ctx = w->ctx;
	cudaStream_t st = ctx->stream;
	int rc;
	if ((rc = ensure_items(w)) || (rc = vpi_ensure_arenas(w))) return rc;
	if (!w->copy_stream) {
		CK(cudaStreamCreateWithFlags(&w->copy_stream, cudaStreamNonBlocking));
		for (int k = 0; k < kMaxStreamSlabs; k++) CK(cudaEventCreateWithFlags(&w->slab_ev[k], cudaEventDisableTiming));
		for (int h = 0; h < 2; h++) CK(cudaEventCreateWithFlags(&w->half_done[h], cudaEventDisableTiming));
		CK(cudaHostAlloc((void **)&w->h_snap, 3u * kMaxStreamSlabs * sizeof(unsigned long long),
				 cudaHostAllocMapped));
		CK(cudaHostGetDevicePointer((void **)&w->h_snap_dev, w->h_snap, 0));
		if ((rc = dev_alloc(&w->d_slab_q, kMaxStreamSlabs)) || (rc = dev_alloc(&w->d_stream_items, w->nchunks)))
			return rc;
	}
	if (!pipelined && (rc = vpi_pipe_drain(w))) return rc;
	const int h = pipelined ? w->pipe_half : 0;
	uint64_t base[3] = {0, 0, 0}, limit[3];
	for (int a = 0; a < 3; a++) {
		const uint64_t half = w->cap[a] / 2u;
		base[a] = pipelined ? (uint64_t)h * half : 0u;
		limit[a] = pipelined ? base[a] + half : w->cap[a];
	}
	if (pipelined) {
		if (!w->outs_alt[1]) {
			w->outs_alt[0] = w->d_outs;
			if ((rc = dev_alloc(&w->outs_alt[1], w->nchunks))) return rc;
		}
		/* this half was last written two calls ago: its copies end first */
		if ((rc = settle_half(w, h))) return rc;
		/* a caller that passes the previous call's result records again gets
		 * that call finished (and rebased) before they are overwritten */
		if (w->rebase[h ^ 1].res == results && (rc = settle_half(w, h ^ 1))) return rc;
		w->d_outs = w->outs_alt[h];
	}
	/* slab k takes ranks k, k + S, k + 2S, ... of the longest-first order, so
	 * every slab holds a similar mix and is itself longest first */
	std::vector<uint32_t> first(slabs + 1, 0);
	if (w->stream_slabs != slabs) {
		std::vector<WorkItem> order;
		order.reserve(w->nchunks);
		for (int k = 0; k < slabs; k++)
			for (uint32_t i = (uint32_t)k; i < w->n_geo; i += (uint32_t)slabs) order.push_back(w->h_items[i]);
		CK(cudaMemcpyAsync(w->d_stream_items, order.data(), order.size() * sizeof(WorkItem), cudaMemcpyHostToDevice,
				   st));
		CK(cudaStreamSynchronize(st));
		w->stream_slabs = slabs;
	}
	for (int k = 0; k < slabs; k++) first[k + 1] = first[k] + (w->n_geo - (uint32_t)k + (uint32_t)slabs - 1) / slabs;
	k_put_cursors<<<1, 32, 0, st>>>(w->d_cursors, base[0], base[1], base[2]);
	CK(cudaGetLastError());
	CK(cudaMemsetAsync(w->d_slab_q, 0, kMaxStreamSlabs * sizeof(unsigned int), st));
	GeoLaunch L;
	memset(&L, 0, sizeof(L));
	L.big_scratch = w->d_big;
	L.big_slots = w->big_slots;
	L.sets = w->d_set;
	set_shell_items(w, L);
	L.threads = 512;
	L.outs = w->d_outs;
	L.lod_max = lod_max;
	L.decoded = vpi_decoded(w); /* every chunk is shelled before the slabs */
	L.dec_slot = w->d_dec_slot;
	Arena *ar[3] = {&L.svl, &L.vbo, &L.ibo};
	for (int a = 0; a < 3; a++) {
		ar[a]->base = w->d_arena[a];
		ar[a]->cap_units = limit[a];
		ar[a]->cursor = w->d_cursors + a;
	}
	const int per_sm = geometry_ctas_per_sm(w->root_bitw, (int)L.threads);
	L.ctas = (uint32_t)(ctx->sm_count * std::max(per_sm, 1));
	GeoLaunch Ls = L;
	Ls.run_shell = 1;
	cudaError_t e = launch_geometry(w->root_bitw, Ls, st);
	if (e != cudaSuccess) return cuda_fail(e, "shell launch");
	for (int k = 0; k < slabs; k++) {
		GeoLaunch Lg = L;
		Lg.items = w->d_stream_items + first[k];
		Lg.n_items = first[k + 1] - first[k];
		Lg.queue = w->d_slab_q + k;
		e = launch_geometry(w->root_bitw, Lg, st);
		if (e != cudaSuccess) return cuda_fail(e, "geometry launch");
		k_fetch_words<<<1, 32, 0, st>>>(w->d_cursors, w->h_snap_dev + 3 * k, 3u);
		CK(cudaGetLastError());
		CK(cudaEventRecord(w->slab_ev[k], st));
	}
	/* cursors, shell (single-run chunks in its last CTAs), and per slab
	 * geometry and the cursor snapshot */
	w->launches += 2 + 2 * slabs;
	w->grouped_lod = -1;
	if ((flags & VP_REBUILD_GROUP) && (rc = enqueue_group(w, lod_max, limit[0]))) return rc;
	w->last_lod = lod_max;
	w->last_flags = flags;
	/* each slab's new output ranges go back while the next slab computes */
	void *dst[3] = {svl, vbo, ibo};
	const uint64_t cap_b[3] = {svl_bytes, vbo_bytes, ibo_bytes};
	uint64_t prev[3] = {base[0], base[1], base[2]};
	bool overflow = false, short_buf = false;
	for (int k = 0; k < slabs; k++) {
		CK(cudaEventSynchronize(w->slab_ev[k]));
		for (int a = 0; a < 3; a++) {
			const uint64_t cur = w->h_snap[3 * k + a];
			if (cur > limit[a]) overflow = true;
			if (overflow || cur <= prev[a]) continue;
			const uint64_t end_b = (cur - base[a]) * 16u;
			if (!dst[a] || end_b > cap_b[a]) {
				short_buf = short_buf || (dst[a] && end_b > cap_b[a]);
				prev[a] = cur;
				continue;
			}
			CK(cudaMemcpyAsync((uint8_t *)dst[a] + (prev[a] - base[a]) * 16u,
					   (const uint8_t *)w->d_arena[a] + prev[a] * 16u, (cur - prev[a]) * 16u,
					   cudaMemcpyDeviceToHost, w->copy_stream));
			prev[a] = cur;
		}
	}
	if (overflow) {
		/* an arena (half) was too small: size each arena for twice what
		 * this rebuild asked for and run it again */
		uint64_t need[3];
		for (int a = 0; a < 3; a++) need[a] = w->h_snap[3 * (slabs - 1) + a] - base[a];
		CK(cudaStreamSynchronize(st));
		CK(cudaStreamSynchronize(w->copy_stream));
		if ((rc = vpi_pipe_drain(w))) return rc;
		for (int a = 0; a < 3; a++) {
			const uint64_t want = (need[a] + need[a] / 4 + 1024) * (pipelined ? 2u : 1u);
			if (want <= w->cap[a]) continue;
			dev_free(w->d_arena[a]);
			w->cap[a] = 0;
			cudaError_t e2 = cudaMalloc(&w->d_arena[a], want * 16u);
			if (e2 != cudaSuccess) {
				w->d_arena[a] = nullptr;
				return cuda_fail(e2, "cudaMalloc(arena growth)");
			}
			w->cap[a] = want;
		}
		w->pipe_half = 0;
		return stream_rebuild(w, lod_max, flags, slabs, svl, svl_bytes, vbo, vbo_bytes, ibo, ibo_bytes, results,
				      used_bytes, pipelined);
	}
	CK(cudaMemcpyAsync(results, w->d_outs, (size_t)w->nchunks * sizeof(ChunkOut), cudaMemcpyDeviceToHost,
			   w->copy_stream));
	for (int a = 0; a < 3; a++) used_bytes[a] = (prev[a] - base[a]) * 16u;
	if (pipelined) {
		CK(cudaEventRecord(w->half_done[h], w->copy_stream));
		w->half_busy[h] = true;
		vp_world::Rebase &rb = w->rebase[h];
		rb.res = results;
		rb.n = w->nchunks;
		for (int a = 0; a < 3; a++) rb.base[a] = base[a];
		w->pipe_half = h ^ 1;
		/* the previous call's copies ran under this call's compute */
		if ((rc = settle_half(w, h ^ 1))) return rc;
		return short_buf ? VP_EOVERFLOW : VP_OK;
	}
	CK(cudaStreamSynchronize(w->copy_stream));
	CK(cudaStreamSynchronize(st));
	return short_buf ? VP_EOVERFLOW : VP_OK;
}

VP_API int vp_world_rebuild_to_host(vp_world *w, int lod_max, unsigned flags, int slabs, void *svl,
				    uint64_t svl_bytes, void *vbo, uint64_t vbo_bytes, void *ibo, uint64_t ibo_bytes,
				    vp_chunk_result *results, uint64_t used_bytes[3])
{
	if (!w || !w->uploaded || !results || !used_bytes) return VP_EINVAL;
	if (lod_max < 0 || lod_max >= VP_MAX_LEVELS || slabs < 1 || slabs > kMaxStreamSlabs) return VP_EINVAL;
	if ((flags & (VP_REBUILD_PLAIN | VP_REBUILD_CONCURRENT)) || w->root_bitw == 7) {
		/* per-chunk launches and 128^3 chunks take the plain sequence */
		int rc;
		if ((rc = vp_world_rebuild(w, lod_max, flags)) || (rc = vp_world_finish(w)) ||
		    (rc = vp_world_results(w, results, w->nchunks)))
			return rc;
		return vp_world_read_outputs(w, svl, svl_bytes, vbo, vbo_bytes, ibo, ibo_bytes, used_bytes);
	}
	return stream_rebuild(w, lod_max, flags, slabs, svl, svl_bytes, vbo, vbo_bytes, ibo, ibo_bytes, results,
			      used_bytes, false);
}

VP_API int vp_world_rebuild_to_host_async(vp_world *w, int lod_max, unsigned flags, int slabs, void *svl,
					  uint64_t svl_bytes, void *vbo, uint64_t vbo_bytes, void *ibo,
					  uint64_t ibo_bytes, vp_chunk_result *results, uint64_t used_bytes[3])
{
	if (!w || !w->uploaded || !results || !used_bytes) return VP_EINVAL;
	if (lod_max < 0 || lod_max >= VP_MAX_LEVELS || slabs < 1 || slabs > kMaxStreamSlabs) return VP_EINVAL;
	if ((flags & (VP_REBUILD_PLAIN | VP_REBUILD_CONCURRENT)) || w->root_bitw == 7)
		return vp_world_rebuild_to_host(w, lod_max, flags, slabs, svl, svl_bytes, vbo, vbo_bytes, ibo, ibo_bytes,
						results, used_bytes);
	return stream_rebuild(w, lod_max, flags, slabs, svl, svl_bytes, vbo, vbo_bytes, ibo, ibo_bytes, results,
			      used_bytes, true);
}

VP_API int vp_world_results(vp_world *w, vp_chunk_result *out, uint32_t n)
{
	static_assert(sizeof(vp_chunk_result) == sizeof(ChunkOut), "result record layout");
	if (!w || !out || n > w->nchunks) return VP_EINVAL;
	CK(cudaMemcpyAsync(out, w->d_outs, (size_t)n * sizeof(ChunkOut), cudaMemcpyDeviceToHost, w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	return VP_OK;
}

static int read_arena(vp_world *w, int a, uint64_t off_bytes, uint64_t nbytes, void *dst)
{
	if (!w || (!dst && nbytes)) return VP_EINVAL;
	if (off_bytes + nbytes > w->cap[a] * 16u) return VP_EINVAL;
	if (!nbytes) return VP_OK;
	CK(cudaMemcpyAsync(dst, (const char *)w->d_arena[a] + off_bytes, nbytes, cudaMemcpyDeviceToHost,
			   w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	return VP_OK;
}

VP_API int vp_world_read_svl(vp_world *w, uint64_t off, uint64_t n, int16_t *dst)
{
	return read_arena(w, 0, off * 2u, n * 2u, dst);
}

VP_API int vp_world_read_vbo(vp_world *w, uint64_t off, uint64_t n, int16_t *dst)
{
	return read_arena(w, 1, off * 2u, n * 2u, dst);
}

VP_API int vp_world_read_ibo(vp_world *w, uint64_t off, uint64_t n, uint32_t *dst)
{
	return read_arena(w, 2, off * 4u, n * 4u, dst);
}

VP_API int vp_world_group_nodes(vp_world *w, int lod, uint64_t *off, uint32_t *items, uint32_t n)
{
	if (!w || lod < 0 || lod > w->grouped_lod || !off || !items) return VP_EINVAL;
	if (n > w->nchunks) n = w->nchunks;
	cudaStream_t st = w->ctx->stream;
	CK(cudaMemcpyAsync(off, w->d_node_off + (size_t)lod * w->nchunks, (size_t)n * sizeof(uint64_t),
			   cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(items, w->d_node_items + (size_t)lod * w->nchunks, (size_t)n * sizeof(uint32_t),
			   cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

VP_API int vp_world_read_group(vp_world *w, int lod, uint64_t off, uint64_t n, int16_t *dst)
{
	if (!w || (!dst && n) || lod < 0 || lod > w->grouped_lod) return VP_EINVAL;
	if (lod == 0) return vp_world_read_svl(w, off, n, dst);
	if (!w->d_garena || (off + n) * 2u > w->garena_units * 16u) return VP_EINVAL;
	if (!n) return VP_OK;
	CK(cudaMemcpyAsync(dst, w->d_garena + off, n * 2u, cudaMemcpyDeviceToHost, w->ctx->stream));
	CK(cudaStreamSynchronize(w->ctx->stream));
	return VP_OK;
}

VP_API int vp_world_kernel_ms(vp_world *w, double *ms, int n, uint32_t *launches)
{
	if (!w || (n > 0 && !ms)) return VP_EINVAL;
	CK(cudaStreamSynchronize(w->ctx->stream));
	for (size_t i = 0; i + 3 < w->ev.size(); i += 4) {
		for (int k = 0; k < 3; k++) {
			float t = 0;
			cudaEventElapsedTime(&t, w->ev[i + k], w->ev[i + k + 1]);
			w->ms[k] += t;
		}
	}
	for (cudaEvent_t e : w->ev) cudaEventDestroy(e);
	w->ev.clear();
	for (int k = 0; k < n && k < 3; k++) ms[k] = w->ms[k];
	if (launches) *launches = w->launches;
	w->ms[0] = w->ms[1] = w->ms[2] = 0;
	w->launches = 0;
	return VP_OK;
}

} // extern "C"

/* ------------------------------------------------------------------ */
/* internal helpers for the drop-in layer                             */
/* ------------------------------------------------------------------ */

int vpi_world_load(vp_world *w, const VpiChunkSrc *src)
{
	const uint32_t N = 1u << (3 * w->root_bitw);
	cudaStream_t st = w->ctx->stream;
	std::vector<uint64_t> off(w->nchunks);
	std::vector<uint32_t> len(w->nchunks);
	std::vector<uint32_t> byte_chunks;
	uint64_t total = 0;
	for (uint32_t c = 0; c < w->nchunks; c++) {
		if (src[c].bytes) {
			byte_chunks.push_back(c);
			continue;
		}
		const uint32_t n = src[c].words ? src[c].nwords : 2u;
		off[c] = total;
		len[c] = n;
		total += (n + 3u) & ~3u;
	}
	const uint64_t rle_words = total;
	const uint64_t enc_cap = (uint64_t)byte_chunks.size() * ((uint64_t)N + 8u);
	total += enc_cap + 8u;
	std::vector<uint32_t> host(rle_words + 8u, 0u);
	for (uint32_t c = 0; c < w->nchunks; c++) {
		if (src[c].bytes) continue;
		if (src[c].words) {
			memcpy(&host[off[c]], src[c].words, (size_t)len[c] * sizeof(uint32_t));
		} else {
			host[off[c]] = N;
			host[off[c] + 1] = 0;
		}
	}
	CK(cudaStreamSynchronize(st));
	dev_free(w->d_pool);
	int rc;
	if ((rc = dev_alloc(&w->d_pool, total))) return rc;
	CK(cudaMemsetAsync(w->d_pool, 0, total * sizeof(uint32_t), st));
	CK(cudaMemcpyAsync(w->d_pool, host.data(), rle_words * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	if (!byte_chunks.empty()) {
		const size_t nb = byte_chunks.size();
		uint8_t *d_vox = nullptr;
		uint64_t *d_sc = nullptr, *d_eoff = nullptr;
		uint32_t *d_elen = nullptr;
		if ((rc = dev_alloc(&d_vox, nb * (size_t)N + 16u)) || (rc = dev_alloc(&d_sc, 2)) ||
		    (rc = dev_alloc(&d_eoff, nb)) || (rc = dev_alloc(&d_elen, nb))) {
			dev_free(d_vox);
			dev_free(d_sc);
			dev_free(d_eoff);
			dev_free(d_elen);
			return rc;
		}
		for (size_t k = 0; k < nb; k++)
			cudaMemcpyAsync(d_vox + k * N, src[byte_chunks[k]].bytes, N, cudaMemcpyHostToDevice, st);
		cudaMemsetAsync(d_sc, 0, 2 * sizeof(uint64_t), st);
		cudaError_t e = launch_rle_encode(d_vox, (uint32_t)nb, N, w->d_pool + rle_words, enc_cap,
						  (unsigned long long *)d_sc, d_eoff, d_elen, (uint32_t *)(d_sc + 1), st);
		std::vector<uint64_t> eoff(nb);
		std::vector<uint32_t> elen(nb);
		if (e == cudaSuccess) e = cudaMemcpyAsync(eoff.data(), d_eoff, nb * 8u, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(elen.data(), d_elen, nb * 4u, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		dev_free(d_vox);
		dev_free(d_sc);
		dev_free(d_eoff);
		dev_free(d_elen);
		if (e != cudaSuccess) return cuda_fail(e, "device encode");
		for (size_t k = 0; k < nb; k++) {
			off[byte_chunks[k]] = rle_words + eoff[k];
			len[byte_chunks[k]] = elen[k];
		}
	}
	w->pool_version++;
	CK(cudaMemcpyAsync(w->d_off, off.data(), w->nchunks * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(w->d_len, len.data(), w->nchunks * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
	w->hlen = len;
	w->hnull.clear();
	w->pool_words = total;
	w->pool_cap = total;
	w->pool_tail = total;
	w->uploaded = true;
	w->items_dirty = true;
	CK(cudaStreamSynchronize(st));
	return VP_OK;
}

int vpi_world_shadow_window(vp_world *w, const uint16_t *map, uint64_t map_len, uint64_t base, uint64_t n,
			    uint32_t shadow_w, const int32_t origin[3])
{
	if (base > map_len) base = map_len;
	if (base + n > map_len) n = map_len - base;
	cudaStream_t st = w->ctx->stream;
	CK(cudaStreamSynchronize(st));
	dev_free(w->d_shadow);
	int rc;
	w->shadow_cap = 0;
	if ((rc = dev_alloc(&w->d_shadow, n + 8u))) return rc;
	w->shadow_cap = n + 8u;
	if (n && map) CK(cudaMemcpyAsync(w->d_shadow, map + base, n * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
	w->shadow_len = n;
	w->shadow_base = base;
	w->shadow_w = shadow_w;
	for (int i = 0; i < 3; i++) w->origin[i] = origin[i];
	return vpi_upload_setdesc(w);
}

int vpi_world_run(vp_world *w, const WorkItem *items, uint32_t n, int lod_max)
{
	cudaStream_t st = w->ctx->stream;
	int rc;
	if ((rc = vpi_ensure_arenas(w))) return rc;
	for (int attempt = 0; attempt < 4; attempt++) {
		std::vector<WorkItem> all(w->nchunks);
		for (uint32_t c = 0; c < w->nchunks; c++) all[c] = WorkItem{0, c, 0, c};
		CK(cudaMemcpyAsync(w->d_items, all.data(), all.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, st));
		w->items_dirty = true; /* the full rebuilds' work order is rebuilt before the next one */
		WorkItem *d_run = nullptr;
		if ((rc = dev_alloc(&d_run, n))) return rc;
		cudaMemcpyAsync(d_run, items, n * sizeof(WorkItem), cudaMemcpyHostToDevice, st);
		cudaMemsetAsync(w->d_cursors, 0, 3 * sizeof(unsigned long long), st);
		GeoLaunch L;
		memset(&L, 0, sizeof(L));
		L.big_scratch = w->d_big;
		L.big_slots = w->big_slots;
		L.sets = w->d_set;
		L.shell_items = w->d_items;
		L.n_shell = w->nchunks;
		L.run_shell = 1;
		L.threads = 512;
		L.outs = w->d_outs;
		L.lod_max = lod_max;
		Arena *ar[3] = {&L.svl, &L.vbo, &L.ibo};
		for (int a = 0; a < 3; a++) {
			ar[a]->base = w->d_arena[a];
			ar[a]->cap_units = w->cap[a];
			ar[a]->cursor = w->d_cursors + a;
		}
		cudaError_t e = launch_geometry(w->root_bitw, L, st);
		if (e == cudaSuccess) {
			GeoLaunch Lg = L;
			Lg.run_shell = 0;
			Lg.items = d_run;
			Lg.n_items = n;
			e = launch_geometry(w->root_bitw, Lg, st);
		}
		unsigned long long cur[3] = {0, 0, 0};
		if (e == cudaSuccess) e = cudaMemcpyAsync(cur, w->d_cursors, sizeof(cur), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		dev_free(d_run);
		if (e != cudaSuccess) return cuda_fail(e, "drop-in launch");
		bool grow = false;
		for (int a = 0; a < 3; a++) {
			if (cur[a] <= w->cap[a]) continue;
			grow = true;
			const uint64_t units = cur[a] + cur[a] / 4 + 1024;
			dev_free(w->d_arena[a]);
			w->cap[a] = 0;
			cudaError_t e2 = cudaMalloc(&w->d_arena[a], units * 16u);
			if (e2 != cudaSuccess) return cuda_fail(e2, "cudaMalloc(arena growth)");
			w->cap[a] = units;
		}
		if (!grow) return VP_OK;
	}
	return VP_EOVERFLOW;
}
