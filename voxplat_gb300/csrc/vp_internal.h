/* vp_internal.h — host-side state shared by the C-ABI translation units. */
#pragma once
#include "voxgpu.h"
#include "vp_geometry.h"

#include <cstdio>
#include <string>
#include <vector>

using namespace vp;

int vpi_cuda_fail(cudaError_t e, const char *what);

#define CK(call)                                                     \
	do {                                                         \
		cudaError_t e_ = (call);                             \
		if (e_ != cudaSuccess) return vpi_cuda_fail(e_, #call); \
	} while (0)
#define cuda_fail vpi_cuda_fail

template <typename T>
static inline int dev_alloc(T **p, size_t n)
{
	*p = nullptr;
	if (n == 0) n = 1;
	cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
	if (e != cudaSuccess) return vpi_cuda_fail(e, "cudaMalloc");
	return VP_OK;
}

template <typename T>
static inline void dev_free(T *&p)
{
	if (p) cudaFree((void *)p);
	p = nullptr;
}

struct vp_ctx {
	int device;
	cudaStream_t stream;
	int timing;
	int sm_count;
	/* staging for the host-buffer codec calls */
	uint8_t *d_bytes = nullptr;
	size_t bytes_cap = 0;
	uint32_t *d_words = nullptr;
	size_t words_cap = 0;
	uint64_t *d_scalars = nullptr; /* [0] cursor, [1] off, [2] len|status */
};

constexpr int kMaxStreamSlabs = 16;

/* Streams for the concurrent plain comparison path: one launch per chunk,
 * spread round-robin over kPlainStreams streams forked from and joined back
 * into the caller's stream. */
constexpr int kPlainStreams = 16;
struct PlainStreams {
	cudaStream_t s[kPlainStreams] = {};
	cudaEvent_t ev[kPlainStreams] = {};
	cudaEvent_t fork = nullptr;
};
extern "C" int vpi_plain_fork(PlainStreams &p, cudaStream_t main); /* creates the streams on first use */
extern "C" int vpi_plain_join(PlainStreams &p, cudaStream_t main);
extern "C" void vpi_plain_free(PlainStreams &p);

struct EditSlot; /* one edit batch's device buffers, stream and bookkeeping (vp_serve.cu) */

struct vp_world {
	vp_ctx *ctx;
	int root_bitw;
	int max_bitw[3];
	uint32_t nchunks;
	uint32_t *d_pool = nullptr;
	uint64_t pool_words = 0;
	uint64_t *d_off = nullptr;
	uint32_t *d_len = nullptr;
	uint16_t *d_shadow = nullptr;
	uint64_t shadow_len = 0;
	uint64_t shadow_cap = 0;                 /* elements allocated in d_shadow */
	uint8_t *d_dec = nullptr;                /* decoded chunks, shell pass -> geometry pass */
	uint32_t *d_dec_slot = nullptr;          /* per chunk: its slot in d_dec, or kNoSlot */
	std::vector<uint32_t> h_dec_slot;        /* host copy */
	size_t dec_bytes = 0;
	bool dec_failed = false;                 /* no room: rebuilds decode twice */
	bool handoff = true;                     /* vp_world_set_handoff */
	uint32_t *d_check = nullptr;             /* upload validation: status, first bad chunk */
	uint32_t *h_check = nullptr;             /* its mapped pinned copy, and that copy's device address */
	uint32_t *h_check_dev = nullptr;
	/* draw culling */
	uint32_t *d_cull_slots = nullptr;
	uint64_t cull_slots_cap = 0;
	uint32_t *d_cull_blocks = nullptr;
	uint64_t cull_blocks_cap = 0;
	uint32_t *d_cull_out = nullptr;          /* [2][nchunks] mesh queue, splat queue; [2] totals after */
	uint8_t *d_flags = nullptr;
	/* picking rays: run-start index of the current pool version */
	uint64_t pool_version = 0, runidx_version = ~0ull;
	uint32_t *d_runidx = nullptr;
	uint64_t runidx_cap = 0;
	uint8_t *d_rays = nullptr;
	size_t rays_cap = 0;
	/* rasteriser */
	/* streamed rebuilds: work order by slab, per-slab queues, copy stream */
	std::vector<WorkItem> h_items;          /* longest-first work order */
	WorkItem *d_stream_items = nullptr;
	int stream_slabs = 0;
	unsigned int *d_slab_q = nullptr;
	cudaStream_t copy_stream = nullptr;
	cudaEvent_t slab_ev[kMaxStreamSlabs] = {};
	unsigned long long *h_snap = nullptr;   /* mapped pinned: 3 cursors per slab */
	unsigned long long *h_snap_dev = nullptr;
	/* pipelined streamed rebuilds: arena halves and result records alternate */
	ChunkOut *outs_alt[2] = {nullptr, nullptr};
	int pipe_half = 0;
	bool half_busy[2] = {false, false};
	cudaEvent_t half_done[2] = {nullptr, nullptr};
	struct Rebase {
		vp_chunk_result *res = nullptr;
		uint32_t n = 0;
		uint64_t base[3] = {0, 0, 0};
	} rebase[2];
	uint8_t *d_render = nullptr;            /* queues, segments, scans, big lists */
	size_t render_cap = 0;
	uint8_t *d_frame = nullptr;             /* frame words, RGBA, depth */
	size_t frame_cap = 0;
	uint32_t shadow_w = 0;
	uint64_t *d_shell_bits = nullptr;
	uint8_t *d_shell_col = nullptr;
	uint8_t *d_big = nullptr;                /* 128^3 chunks: per-CTA working sets */
	uint32_t big_slots = 0;
	SetDesc *d_set = nullptr;
	WorkItem *d_items = nullptr;
	/* d_items[0, n_geo): chunks with geometry to build, longest first;
	 * [n_geo, nchunks): chunks that are all air with all-air (or no) +x, +y
	 * and +z neighbours, whose result records a rebuild only zeroes */
	uint32_t n_geo = 0;
	uint8_t *d_null = nullptr;               /* per chunk: 1 = all air (one air run) */
	std::vector<uint8_t> hnull;              /* host copy; empty = to be fetched */
	/* shell pass order: the chunks of more than one run (or with a handoff
	 * slot), longest first, then the single-run chunks, whose shells (if
	 * not all air) the shell launch's last CTAs write a warp each */
	WorkItem *d_shell_items = nullptr;
	uint32_t n_shell_multi = 0;
	std::vector<uint8_t> modes;
	std::vector<uint32_t> hlen;              /* host copy of stream lengths */
	bool lens_stale = false;                 /* an edit changed lengths on the device since hlen */
	bool items_dirty = true;
	ChunkOut *d_outs = nullptr;
	unsigned int *d_queue = nullptr;
	unsigned long long *d_cursors = nullptr; /* svl, vbo, ibo */
	void *d_arena[3] = {nullptr, nullptr, nullptr};
	uint64_t cap[3] = {0, 0, 0};             /* 16-byte units */
	int last_lod = 4;
	unsigned last_flags = 0;
	bool uploaded = false;
	/* grouping */
	uint64_t *d_gcounts = nullptr, *d_gtotal = nullptr, *d_node_off = nullptr;
	uint32_t *d_node_items = nullptr;
	int16_t *d_garena = nullptr;
	uint64_t garena_units = 0;
	int grouped_lod = -1;
	int32_t origin[3] = {0, 0, 0};           /* world chunk coords of chunk 0 */
	/* edits: the pool grows at its tail, re-encoded streams are appended */
	uint64_t pool_cap = 0;                   /* words allocated in d_pool */
	/* the edit server's pool compaction copies into this spare pool and
	 * keeps the old one as the next spare: no device allocation while
	 * serving (set up with the server) */
	uint32_t *d_pool_spare = nullptr;
	uint64_t pool_spare_cap = 0;
	uint64_t *d_noff = nullptr;              /* compaction scratch, nchunks offsets */
	uint64_t pool_tail = 0;                  /* first free word */
	unsigned long long *d_pool_cursor = nullptr; /* device copy of the pool tail while edit batches append */
	EditSlot *eslot = nullptr;               /* the synchronous edit path's batch state (vp_world_edit) */
	vp_server *server = nullptr;             /* the edit server attached to this world, if any */
	std::vector<int32_t> slot_of;            /* chunk -> volume slot while a batch is planned */
	std::vector<uint32_t> last_dirty;
	uint64_t shadow_base = 0;                /* world index of d_shadow[0] */
	PlainStreams plain;                      /* VP_REBUILD_CONCURRENT */
	std::vector<cudaEvent_t> ev;             /* pairs per kernel */
	std::vector<int> ev_kind;                /* 0 shell, 1 geometry */
	double ms[3] = {0, 0, 0};
	uint32_t launches = 0;
};


/* internal helpers shared with the drop-in layer (vp_api.cu) */
extern "C" int vpi_upload_setdesc(vp_world *w); /* defined inside the C-ABI block */
extern "C" int vpi_ensure_arenas(vp_world *w);

/* One chunk's data for vpi_world_load: decoded voxels (R^3 bytes), or an
 * RLE stream, or neither (all air). */
struct VpiChunkSrc {
	const uint8_t *bytes;
	const uint32_t *words;
	uint32_t nwords; /* including the 0 terminator */
};
int vpi_world_load(vp_world *w, const VpiChunkSrc *src);
int vpi_world_shadow_window(vp_world *w, const uint16_t *map, uint64_t map_len, uint64_t base, uint64_t n,
			    uint32_t shadow_w, const int32_t origin[3]);
int vpi_world_run(vp_world *w, const WorkItem *items, uint32_t n, int lod_max);
/* A reference-format stream of n words (terminator included) covering N
 * voxels with nonzero run lengths. */
/* waits for the copies of pipelined streamed rebuilds and rebases their
 * results, and for the edit batches an attached server has in flight */
extern "C" int vpi_pipe_drain(vp_world *w);
/* vp_serve.cu: retire every in-flight batch of the world's server (no-op
 * without one) and free the edit path's state at world destruction */
int vpi_server_quiesce(vp_world *w);
void vpi_edit_state_free(vp_world *w);
/* the decoded-chunk handoff buffer of a full rebuild, or NULL (128^3 roots,
 * or not enough free device memory: the geometry pass then decodes) */
extern "C" uint8_t *vpi_decoded(vp_world *w);
extern "C" int vpi_validate_stream(const uint32_t *s, uint32_t n, uint64_t N);
