/*
 * vp_noalloc.cu — vp_rebuild_noalloc: the batched geometry rebuild of a
 * small chunk set that allocates no memory.
 *
 * Some callers cannot allocate device memory at the moment they need
 * geometry: a render or input thread that must not stall on cudaMalloc's
 * implicit device synchronisation, or an engine that hands all device
 * memory to its own allocator up front. They pass device pointers for every
 * input and output; the pass-local working data (the set descriptor, the
 * work list, the output cursors and the per-chunk shells the neighbouring
 * chunks read) lives in g_noalloc_scratch below, a fixed 4 MiB array every
 * GPU that loads the library holds until the process exits.
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

size_t align256(size_t v) { return (v + 255u) & ~(size_t)255u; }

/* scratch layout for n chunks of 2^rb edge */
struct Layout {
	size_t set, items, cursors, bits, cols, total;
};

Layout layout(uint32_t n, int rb)
{
	Layout L;
	L.set = 0;
	L.items = align256(sizeof(SetDesc));
	L.cursors = L.items + align256((size_t)n * sizeof(WorkItem));
	L.bits = L.cursors + 256;
	L.cols = L.bits + align256((size_t)n * shell_words_per_chunk(rb) * sizeof(uint64_t));
	L.total = L.cols + align256((size_t)n * shell_cols_per_chunk(rb));
	return L;
}

/* Writes the set descriptor and the work list into the scratch area and
 * clears the output cursors (fresh on every call: the area keeps the
 * previous call's contents). */
__global__ void k_noalloc_setup(SetDesc d, uint8_t *scratch, Layout L, uint32_t n, const uint8_t *make_mesh)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i == 0) {
		*(SetDesc *)(scratch + L.set) = d;
		unsigned long long *cur = (unsigned long long *)(scratch + L.cursors);
		cur[0] = cur[1] = cur[2] = 0ull;
	}
	if (i < n) {
		WorkItem w;
		w.set = 0;
		w.chunk = i;
		w.flags = (make_mesh && make_mesh[i]) ? kItemMesh : 0u;
		w.slot = i;
		((WorkItem *)(scratch + L.items))[i] = w;
	}
}

} // namespace
} // namespace vp

using namespace vp;

extern "C" VP_API int vp_rebuild_noalloc(int device, void *stream, int root_bitw, const int max_bitw[3],
					   const uint32_t *pool, const uint64_t *off, const uint32_t *len,
					   const uint16_t *shadow, uint64_t shadow_len, uint32_t shadow_w,
					   const uint8_t *make_mesh, int lod_max, int16_t *svl, uint64_t svl_bytes,
					   int16_t *vbo, uint64_t vbo_bytes, uint32_t *ibo, uint64_t ibo_bytes,
					   vp_chunk_result *results)
{
	if (!max_bitw || !pool || !off || !len || !results || (!shadow && shadow_len)) return VP_EINVAL;
	if (root_bitw < 3 || root_bitw > 6) return VP_EUNSUPPORTED;
	if (lod_max < 0 || lod_max >= VP_MAX_LEVELS) return VP_EUNSUPPORTED;
	if (device < 0 || device >= 64) return VP_EINVAL;
	for (int i = 0; i < 3; i++)
		if (max_bitw[i] < 0 || max_bitw[i] > 12) return VP_EINVAL;
	const uint32_t n = 1u << (max_bitw[0] + max_bitw[1] + max_bitw[2]);
	const Layout L = layout(n, root_bitw);
	/* the set must fit the fixed scratch area (4 MiB: e.g. 256 chunks of
	 * 64^3, 1024 of 32^3) */
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
	SetDesc d = {};
	d.pool = pool;
	d.off = off;
	d.len = len;
	d.shadow = shadow;
	d.shadow_len = shadow_len;
	d.shell_bits = (uint64_t *)(scratch + L.bits);
	d.shell_col = scratch + L.cols;
	d.shadow_w = shadow_w;
	d.nchunks = n;
	d.root_bitw = (uint32_t)root_bitw;
	for (int i = 0; i < 3; i++) d.max_bitw[i] = (uint32_t)max_bitw[i];
	k_noalloc_setup<<<(n + 255) / 256, 256, 0, st>>>(d, scratch, L, n, make_mesh);
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
	return VP_OK;
}
