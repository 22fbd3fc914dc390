/*
 * vp_noalloc.cu — vp_rebuild_noalloc: the batched geometry rebuild of a
 * small chunk set that allocates no memory.
 *
 * Some callers cannot allocate device memory at the moment they need
 * geometry: a render or input thread that must not stall on cudaMalloc's
 * implicit device synchronisation, or an engine that hands all device
 * memory to its own allocator up front. They pass device pointers for every
 * input and output; the pass-local working data (the set descriptor, the
 * checked stream table, the work list, the output cursors and the per-chunk
 * shells the neighbouring chunks read) lives in g_noalloc_scratch below, a
 * fixed 4 MiB array every GPU that loads the library holds until the process
 * exits.
 *
 * The caller's streams are not trusted: a set-up kernel checks every stream
 * (in bounds of the caller's pool, 16-byte aligned, nonzero counts summing
 * to R^3, one terminator) before any kernel decodes it. A chunk whose stream
 * fails is rebuilt as air (its neighbours see air too) and its result record
 * gets status VP_STATUS_BAD_STREAM.
 *
 * Set-up: the first call on a device looks up the scratch array's device
 * address with cudaGetSymbolAddress (with that device current) and caches
 * it; make that first call before any stream capture. All calls share the
 * one array and it keeps the previous call's contents: each call clears
 * what must start at zero, and calls whose work overlaps on the GPU (two
 * streams, or two host threads) race on it.
 */
#include "voxgpu.h"
#include "vp_geometry.h"

#include <mutex>

namespace vp {

static constexpr size_t kNoAllocScratchBytes = 4u << 20;
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_mu;
void *g_scratch_addr[64] = {nullptr};

constexpr uint32_t kAirWords = 16; /* {R^3, 0} and zero padding: 64 bytes */

size_t align256(size_t v) { return (v + 255u) & ~(size_t)255u; }

/* scratch layout for n chunks of 2^rb edge */
struct Layout {
	size_t set, items, cursors, air, off, len, bad, bits, cols, total;
};

Layout layout(uint32_t n, int rb)
{
	Layout L;
	L.set = 0;
	L.items = align256(sizeof(SetDesc));
	L.cursors = L.items + align256((size_t)n * sizeof(WorkItem));
	L.air = L.cursors + 256;
	L.off = L.air + 256;
	L.len = L.off + align256((size_t)n * sizeof(uint64_t));
	L.bad = L.len + align256((size_t)n * sizeof(uint32_t));
	L.bits = L.bad + align256(n);
	L.cols = L.bits + align256((size_t)n * shell_words_per_chunk(rb) * sizeof(uint64_t));
	L.total = L.cols + align256((size_t)n * shell_cols_per_chunk(rb));
	return L;
}

/* One warp per chunk. Checks chunk c's stream before anything decodes it:
 * length >= 2, start 16-byte aligned, the stream and the 8 words the decoder
 * may read after it inside the caller's pool (pool_words), every count
 * before the terminator nonzero, counts summing to N, a zero terminator.
 * Streams are addressed from `base` (the lower of the pool and the scratch
 * area): a good chunk keeps its stream, a failing one gets the all-air
 * stream in scratch and a bad flag. Also writes the set descriptor, the
 * work list, and clears the output cursors (fresh on every call: the area
 * keeps the previous call's contents). */
__global__ void __launch_bounds__(256) k_noalloc_setup(SetDesc d, uint8_t *scratch, Layout L, uint32_t n,
						       const uint32_t *pool, uint64_t pool_words, const uint64_t *off,
						       const uint32_t *len, const uint8_t *make_mesh, uint32_t N,
						       uint64_t pool_rel, uint64_t air_rel)
{
	const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (gw == 0 && lane == 0) {
		*(SetDesc *)(scratch + L.set) = d;
		unsigned long long *cur = (unsigned long long *)(scratch + L.cursors);
		cur[0] = cur[1] = cur[2] = 0ull;
		uint32_t *air = (uint32_t *)(scratch + L.air);
		air[0] = N; /* one air run, then the terminator and padding */
		for (uint32_t k = 1; k < kAirWords; k++) air[k] = 0u;
	}
	if (gw >= n) return;
	const uint32_t c = gw;
	const uint64_t o = off[c];
	const uint32_t ln = len[c];
	bool bad = ln < 2u || o > pool_words || (uint64_t)ln + 8u > pool_words - o ||
		   (((uintptr_t)(pool + o)) & 15u) != 0u;
	if (!bad) {
		const uint32_t *s = pool + o;
		uint64_t sum = 0;
		bool zero = false;
		for (uint32_t i = lane; i + 1u < ln; i += 32u) {
			const uint32_t cnt = s[i] & 0xFFFFFFu;
			zero |= cnt == 0u;
			sum += cnt;
		}
#pragma unroll
		for (int k = 16; k; k >>= 1) sum += __shfl_xor_sync(kFull, sum, k);
		zero = __any_sync(kFull, zero);
		bad = zero || sum != (uint64_t)N || s[ln - 1u] != 0u;
	}
	if (lane == 0) {
		((uint64_t *)(scratch + L.off))[c] = bad ? air_rel : pool_rel + o;
		((uint32_t *)(scratch + L.len))[c] = bad ? 2u : ln;
		(scratch + L.bad)[c] = bad ? 1u : 0u;
		WorkItem w;
		w.set = 0;
		w.chunk = c;
		w.flags = (make_mesh && make_mesh[c]) ? kItemMesh : 0u;
		w.slot = c;
		((WorkItem *)(scratch + L.items))[c] = w;
	}
}

/* After the geometry pass: mark the chunks whose streams failed the check. */
__global__ void k_noalloc_mark_bad(const uint8_t *bad, uint32_t n, ChunkOut *outs)
{
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c < n && bad[c]) outs[c].status |= kStatusBadStream;
}

} // namespace
} // namespace vp

using namespace vp;

extern "C" VP_API int vp_rebuild_noalloc(int device, void *stream, int root_bitw, const int max_bitw[3],
					   const uint32_t *pool, uint64_t pool_words, const uint64_t *off,
					   const uint32_t *len, const uint16_t *shadow, uint64_t shadow_len,
					   uint32_t shadow_w, const uint8_t *make_mesh, int lod_max, int16_t *svl,
					   uint64_t svl_bytes, int16_t *vbo, uint64_t vbo_bytes, uint32_t *ibo,
					   uint64_t ibo_bytes, vp_chunk_result *results)
{
	if (!max_bitw || !pool || !off || !len || !results || (!shadow && shadow_len)) return VP_EINVAL;
	if (((uintptr_t)pool & 3u) != 0u) return VP_EINVAL;
	if (root_bitw < 3 || root_bitw > 6) return VP_EUNSUPPORTED;
	if (lod_max < 0 || lod_max >= VP_MAX_LEVELS) return VP_EUNSUPPORTED;
	if (device < 0 || device >= 64) return VP_EINVAL;
	for (int i = 0; i < 3; i++)
		if (max_bitw[i] < 0 || max_bitw[i] > 12) return VP_EINVAL;
	/* as vp_world_create: at most 2^24 chunks (the shift below stays defined) */
	if (max_bitw[0] + max_bitw[1] + max_bitw[2] > 24) return VP_EUNSUPPORTED;
	const uint32_t n = 1u << (max_bitw[0] + max_bitw[1] + max_bitw[2]);
	const Layout L = layout(n, root_bitw);
	/* the set must fit the fixed scratch area (4 MiB: 256 chunks of 64^3,
	 * 512 of 32^3, 2048 of 16^3, 4096 of 8^3) */
	if (L.total > kNoAllocScratchBytes) return VP_EOVERFLOW;
	if (cudaSetDevice(device) != cudaSuccess) return VP_ECUDA;
	uint8_t *scratch;
	{
		std::lock_guard<std::mutex> lk(g_mu);
		if (!g_scratch_addr[device]) {
			void *p = nullptr;
			if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return VP_ECUDA;
			g_scratch_addr[device] = p;
		}
		scratch = (uint8_t *)g_scratch_addr[device];
	}
	cudaStream_t st = (cudaStream_t)stream;
	const uint32_t R = 1u << root_bitw;
	/* streams are addressed in words from the lower of the caller's pool
	 * and the scratch area's all-air stream, both 4-byte aligned */
	const uint32_t *air = (const uint32_t *)(scratch + L.air);
	const uint32_t *base = (uintptr_t)pool < (uintptr_t)air ? pool : air;
	const uint64_t pool_rel = ((uintptr_t)pool - (uintptr_t)base) / 4u;
	const uint64_t air_rel = ((uintptr_t)air - (uintptr_t)base) / 4u;
	SetDesc d = {};
	d.pool = base;
	d.off = (const uint64_t *)(scratch + L.off);
	d.len = (const uint32_t *)(scratch + L.len);
	d.shadow = shadow;
	d.shadow_len = shadow_len;
	d.shell_bits = (uint64_t *)(scratch + L.bits);
	d.shell_col = scratch + L.cols;
	d.shadow_w = shadow_w;
	d.nchunks = n;
	d.root_bitw = (uint32_t)root_bitw;
	for (int i = 0; i < 3; i++) d.max_bitw[i] = (uint32_t)max_bitw[i];
	k_noalloc_setup<<<(n + 7) / 8, 256, 0, st>>>(d, scratch, L, n, pool, pool_words, off, len, make_mesh,
						     R * R * R, pool_rel, air_rel);
	if (cudaGetLastError() != cudaSuccess) return VP_ECUDA;
	GeoLaunch G = {};
	G.sets = (const SetDesc *)(scratch + L.set);
	G.items = (const WorkItem *)(scratch + L.items);
	G.n_items = n;
	G.shell_items = G.items;
	G.n_shell = n;
	G.threads = 512;
	G.outs = (ChunkOut *)results;
	G.lod_max = lod_max;
	unsigned long long *cur = (unsigned long long *)(scratch + L.cursors);
	G.svl = Arena{svl, svl_bytes / 16u, cur};
	G.vbo = Arena{vbo, vbo_bytes / 16u, cur + 1};
	G.ibo = Arena{ibo, ibo_bytes / 16u, cur + 2};
	G.run_shell = 1;
	GeoLaunch Gs = G;
	Gs.n_items = 0;
	if (launch_geometry(root_bitw, Gs, st) != cudaSuccess) return VP_ECUDA;
	GeoLaunch Gg = G;
	Gg.run_shell = 0;
	if (launch_geometry(root_bitw, Gg, st) != cudaSuccess) return VP_ECUDA;
	k_noalloc_mark_bad<<<(n + 255) / 256, 256, 0, st>>>(scratch + L.bad, n, (ChunkOut *)results);
	if (cudaGetLastError() != cudaSuccess) return VP_ECUDA;
	return VP_OK;
}
