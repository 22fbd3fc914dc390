/*
 * voxgpu.h — C ABI of the GB300 (sm_103a) voxel geometry pipeline.
 *
 * Two groups of entry points:
 *
 * 1. The device-resident world API (vp_*). A world mirrors one reference
 *    ChunkSet (src/chunkset.h:29-55): chunk size 2^root_bitw, 2^max_bitw[i]
 *    chunks per axis, every chunk stored as its RLE stream in HBM, plus the
 *    sun-shadow map. vp_world_rebuild runs, for every chunk, what the
 *    reference's mesher thread does per chunk in chunkset_manage
 *    (src/chunkset.c:246-507): decode, then either the quad mesh
 *    (chunk_make_mesh, src/chunkset/mesher.c:184-357) or the exposure mask,
 *    LOD chain and splat lists (chunk_make_mask / chunk_mask_downsample /
 *    chunk_make_splatlist, src/chunkset/mesher.c:377-536) — in one batched
 *    launch instead of one OpenMP iteration per chunk.
 *
 * 2. Drop-in replacements with the reference's own names and signatures,
 *    declared in voxgpu_dropin.h.
 *
 * Every function returns 0 (VP_OK) or a negative VP_E* code; no function
 * aborts the process. Outputs are bit-identical to the reference C code.
 */
#ifndef VOXGPU_H
#define VOXGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define VP_API __attribute__((visibility("default")))
#else
#define VP_API
#endif

#define VP_OK 0
#define VP_EINVAL (-1)       /* bad argument or malformed RLE stream */
#define VP_ENOMEM (-2)       /* device or host allocation failed */
#define VP_ECUDA (-3)        /* a CUDA call failed; see vp_last_cuda_error */
#define VP_EOVERFLOW (-4)    /* output arena too small and growth refused */
#define VP_ETIMEOUT (-5)     /* a bounded device wait ran out */
#define VP_EUNSUPPORTED (-6) /* chunk size or level count not supported */
#define VP_EBUSY (-7)        /* admission refused: not enough free HBM */

#define VP_MAX_LEVELS 8      /* LOD levels 0..7 in one result record */

typedef struct vp_ctx vp_ctx;
typedef struct vp_world vp_world;
typedef struct vp_server vp_server;

/* Result of one chunk; offsets index the world's output arenas. Item counts
 * are in the reference's units: int16 elements for splats and vertices
 * (svl_items, mesh_vbo_items, src/chunkset.h:108-117), u32 for indices. */
typedef struct vp_chunk_result {
	uint64_t svl_off;
	uint64_t vbo_off;
	uint64_t ibo_off;
	uint32_t svl_items[VP_MAX_LEVELS];
	uint32_t svl_total;
	uint32_t vbo_items;
	uint32_t ibo_items;
	uint32_t status;
} vp_chunk_result;

/* Rebuild flags */
#define VP_REBUILD_PERSISTENT 1u /* persistent CTAs + device work queue */
#define VP_REBUILD_PLAIN 2u      /* one launch per chunk and pass (comparison path) */
#define VP_REBUILD_GROUP 4u      /* also build the LOD/octree draw groups */
#define VP_REBUILD_GRAPH 8u      /* batches: replay the tuned configuration's CUDA graph */
#define VP_REBUILD_CONCURRENT 16u /* one launch per chunk and pass, spread over 16 streams (comparison path) */

VP_API const char *vp_strerror(int code);
VP_API const char *vp_last_cuda_error(void);

/* A context owns one CUDA stream on `device`. */
VP_API int vp_ctx_create(int device, vp_ctx **out);
VP_API void vp_ctx_destroy(vp_ctx *ctx);
VP_API void *vp_ctx_stream(vp_ctx *ctx);       /* the cudaStream_t */
VP_API int vp_ctx_sync(vp_ctx *ctx);

/* Worlds. root_bitw 3..6 (chunks of 8^3 .. 64^3). */
VP_API int vp_world_create(vp_ctx *ctx, int root_bitw, const int max_bitw[3], vp_world **out);
VP_API void vp_world_destroy(vp_world *w);

/* Copy a whole world from host memory: the RLE streams of every chunk
 * (pool words, per-chunk word offsets and lengths including the 0
 * terminator) and the shadow map (shadow_len elements, zero padded past the
 * map; reads past shadow_len return 0). Streams are validated: every run
 * count >= 1, runs sum to root^3, a single 0 terminator. */
VP_API int vp_world_upload(vp_world *w, const uint32_t *pool, uint64_t pool_words, const uint64_t *off,
			   const uint32_t *len, const uint16_t *shadow, uint64_t shadow_len, uint32_t shadow_w);

/* Generate a seeded synthetic world directly in device memory (RLE pool
 * and shadow map), bit-identical to the host generator
 * (voxplat_gb300/csrc/vp_worldgen.h): kind 1 = small terrain (heights
 * 8..56), kind 2 = terrain + caves (heights 40..200); horizontal noise
 * scaled by 2^hshift; the shadow map gets pad_rows zero rows. */
VP_API int vp_world_generate(vp_world *w, int kind, uint64_t seed, int hshift, uint32_t pad_rows);

/* The decoded-chunk handoff of full rebuilds: the shell pass decodes every
 * chunk and, with the handoff on (the default), stores each multi-run
 * chunk's decoded rows (20 * root^2 bytes) for the geometry pass to load
 * instead of decoding again. The buffer is allocated at the first rebuild
 * when the device keeps 4 GiB free beside it and it is at most a quarter of
 * the device; otherwise, or with the handoff off, the geometry pass decodes.
 * Outputs are the same either way. vp_world_handoff_bytes reports the
 * buffer's size (0 when there is none). */
VP_API int vp_world_set_handoff(vp_world *w, int on);
VP_API int vp_world_handoff_bytes(vp_world *w, uint64_t *bytes);

/* Per chunk: 1 = quad mesh (near chunk, ChunkMD.make_mesh), 0 = splats.
 * NULL = every chunk splats. */
VP_API int vp_world_set_modes(vp_world *w, const uint8_t *make_mesh);

/* Size the three output arenas (splat lists, vertex and index buffers) to
 * bytes[0..2], rounded up to 16 B; a caller that knows its output sizes
 * avoids the grow-and-rerun of vp_world_finish. The default is 16 KiB per
 * chunk for each arena, at least 16 MiB. Not while a rebuild is in flight. */
VP_API int vp_world_reserve(vp_world *w, const uint64_t bytes[3]);

/* Enqueue a full rebuild on the context stream (asynchronous). */
VP_API int vp_world_rebuild(vp_world *w, int lod_max, unsigned flags);
/* Wait for the rebuild; grow the output arenas and rebuild again if any
 * chunk overflowed. */
VP_API int vp_world_finish(vp_world *w);

VP_API int vp_world_results(vp_world *w, vp_chunk_result *out, uint32_t n);
/* A full rebuild whose outputs stream into host buffers while the GPU
 * works (pinned buffers): the geometry pass runs as `slabs` launches (1..16)
 * over interleaved parts of the work order, and each part's output ranges
 * are copied back on a second stream while the next part computes; then the
 * result records. Same outputs and layout as vp_world_rebuild +
 * vp_world_finish + vp_world_results + vp_world_read_outputs, which it falls
 * back to when an arena has to grow. */
VP_API int vp_world_rebuild_to_host(vp_world *w, int lod_max, unsigned flags, int slabs, void *svl,
				    uint64_t svl_bytes, void *vbo, uint64_t vbo_bytes, void *ibo, uint64_t ibo_bytes,
				    vp_chunk_result *results, uint64_t used_bytes[3]);
/* The same rebuild, pipelined with the next one: returns once its copies
 * are issued and the previous call's copies have finished, so rebuild k+1
 * (and the upload before it) computes while rebuild k's outputs are being
 * copied. Calls alternate between two halves of each output arena and two
 * sets of result records, and so should the caller's host buffers: those of
 * call k (and `results`, whose offsets are then rebased to the host
 * buffers) are final once call k+1 or vp_world_outputs_wait returns, or a
 * synchronous rebuild, an edit or a reserve, which wait too. A call given
 * the previous call's `results` again first finishes that call (no
 * overlap). used_bytes[] is final on return. Outputs are identical to
 * vp_world_rebuild_to_host's. */
VP_API int vp_world_rebuild_to_host_async(vp_world *w, int lod_max, unsigned flags, int slabs, void *svl,
					  uint64_t svl_bytes, void *vbo, uint64_t vbo_bytes, void *ibo,
					  uint64_t ibo_bytes, vp_chunk_result *results, uint64_t used_bytes[3]);
VP_API int vp_world_outputs_wait(vp_world *w);
/* Copy the used part of the three output arenas (splats, vertices,
 * indices) into host buffers, with the arena layout the results' offsets
 * index (a NULL buffer is skipped). used_bytes[] gets each used size;
 * VP_EOVERFLOW when a buffer is smaller. Pinned buffers copy fastest. */
VP_API int vp_world_read_outputs(vp_world *w, void *svl, uint64_t svl_bytes, void *vbo, uint64_t vbo_bytes, void *ibo,
				 uint64_t ibo_bytes, uint64_t used_bytes[3]);
VP_API int vp_world_read_svl(vp_world *w, uint64_t off, uint64_t n, int16_t *dst);
VP_API int vp_world_read_vbo(vp_world *w, uint64_t off, uint64_t n, int16_t *dst);
VP_API int vp_world_read_ibo(vp_world *w, uint64_t off, uint64_t n, uint32_t *dst);

/* Sphere edits (chunkset_edit_sphere, src/chunkset/edit.c:179-244): fill
 * with `voxel`, or carve when voxel == 0; radius <= 250. Edits apply in
 * array order, exactly as the reference applies them one after the other:
 * voxel writes skip y < 2 (edit.c:151), fills update the shadow map in the
 * reference's loop order (src/chunkset/shadow.h:77-89), carves leave it.
 * Every chunk of an edit's AABB list (the chunks the reference marks dirty)
 * is re-encoded and its geometry rebuilt in the mode set by
 * vp_world_set_modes, with the LOD count of the last rebuild; its result
 * record then points at the new geometry. */
typedef struct vp_edit {
	int32_t x, y, z;    /* centre, world voxels */
	uint32_t radius;
	uint8_t voxel;
	uint8_t pad[7];
	double arrival_s;   /* vp_world_serve: arrival time from the start */
} vp_edit;

typedef struct vp_serve_stats {
	uint32_t batches;
	uint32_t edits;
	uint32_t max_batch;
	uint32_t deferred;  /* times the next batch waited: no free slot, or it touched in-flight work */
	uint64_t chunks_remeshed;
	double busy_s;      /* time with at least one batch on the GPU */
	double wall_s;
	uint32_t max_inflight; /* most batches on the GPU at once */
	uint32_t rejected;  /* edits refused: alone they need more than a slot holds */
	double inflight_s;  /* integral of batches on the GPU over time (/ busy_s = mean overlap) */
} vp_serve_stats;

/* Apply edits[0..n) as one batch and rebuild the dirty chunks (synchronous). */
VP_API int vp_world_edit(vp_world *w, const vp_edit *edits, uint32_t n);
/* Read back a chunk's current RLE stream (*n words incl. the terminator;
 * VP_EOVERFLOW when cap is short) and the shadow map (n elements). */
VP_API int vp_world_chunk_rle(vp_world *w, uint32_t chunk, uint32_t *dst, uint32_t cap, uint32_t *n);
VP_API int vp_world_read_shadow(vp_world *w, uint16_t *dst, uint64_t n);
/* Total words of all chunks' current RLE streams (terminators included). */
VP_API int vp_world_rle_words(vp_world *w, uint64_t *words);
/* The chunks the last edit batch rebuilt. */
VP_API int vp_world_dirty(vp_world *w, uint32_t *chunks, uint32_t cap, uint32_t *n);
/* Replay a timed edit trace (arrival_s ascending) in real time through an
 * edit server (vp_server_create with `slots` slots of slot_chunks = 512,
 * this max_batch and hbm_reserve): edits are submitted at their arrival
 * times and batches overlap on the device as the server admits them.
 * latency_ms[i] = the time edit i's batch was seen finished - its arrival
 * (negative for an edit the server refused). */
VP_API int vp_world_serve(vp_world *w, const vp_edit *edits, uint32_t n, uint32_t max_batch, uint32_t slots,
			  uint64_t hbm_reserve, double *latency_ms, vp_serve_stats *stats);

/* Edit server: continuous batching of world edits with requests in flight
 * on the device at once (the reference's edit -> dirty -> next mesher tick
 * flow, src/chunkset/edit.c:179-244, src/chunkset.c:246-309, as a request
 * loop). Edits are applied in submission order. The server keeps up to
 * `slots` batches on the GPU, each on its own stream with its own buffers
 * for `slot_chunks` dirty chunks; a new batch is formed from the queue head
 * (at most max_batch edits, at most slot_chunks dirty chunks) and admitted
 * when a slot is free and it touches nothing an in-flight batch touches
 * (chunks within one chunk of each other's dirty chunks, or sun-shadow map
 * rows both use), so every batch's result is the one serial application
 * gives. Slots are sized at creation from the device's free memory minus
 * hbm_reserve: fewer slots when memory is short, VP_ENOMEM when not even
 * one fits. An edit whose own dirty chunks exceed a slot completes with
 * status VP_ENOMEM and changes nothing. Other calls on the world first wait
 * for the server's in-flight batches. */
typedef struct vp_server_config {
	uint32_t slots;       /* batches on the GPU at once, 1..8 */
	uint32_t max_batch;   /* edits per batch */
	uint32_t slot_chunks; /* dirty chunks one batch may hold */
	uint64_t hbm_reserve; /* device bytes the slots must leave free */
} vp_server_config;

/* One finished edit: its ticket, status (VP_OK, or VP_ENOMEM when refused),
 * the batch it ran in, and host times in seconds since the server started:
 * submitted, its batch admitted to the GPU, its batch seen finished. */
typedef struct vp_edit_done {
	uint64_t ticket;
	int32_t status;
	uint32_t batch;
	double submit_s, start_s, done_s;
} vp_edit_done;

VP_API int vp_server_create(vp_world *w, const vp_server_config *cfg, vp_server **out);
/* Waits for the in-flight batches, then frees the server. */
VP_API void vp_server_destroy(vp_server *s);
/* Queue edits; they get consecutive tickets from *first_ticket. Does not
 * wait for the GPU: it retires finished batches and admits new ones. */
VP_API int vp_edit_submit(vp_server *s, const vp_edit *edits, uint32_t n, uint64_t *first_ticket);
/* Retire finished batches, admit queued edits, and return up to cap
 * finished edits (*n of them, in completion order). With wait_us > 0 it
 * keeps pumping for up to wait_us microseconds until at least one edit has
 * finished. */
VP_API int vp_poll_results(vp_server *s, vp_edit_done *out, uint32_t cap, uint32_t *n, uint32_t wait_us);
/* Run every queued and in-flight edit to completion. */
VP_API int vp_server_drain(vp_server *s);
VP_API int vp_server_stats(vp_server *s, vp_serve_stats *stats, uint32_t *slots_out);

/* LOD/octree draw groups of the last rebuild made with VP_REBUILD_GROUP
 * (gfx_update_svl, src/gfx/vsplat.c:209-331, minus the GL upload): for LOD
 * `lod`, node i (numbered flatten3(node, max_bitw - min(lod, max_bitw)))
 * holds the concatenated level-`lod` splats of its member chunks, scanned x
 * outer, y, z inner; off[i] / items[i] locate it, in int16 units. At LOD 0
 * every node is one chunk and its list is that chunk's level-0 segment, so
 * the LOD-0 offsets index the splat arena (nothing is copied); the lists of
 * LOD >= 1 nodes are concatenated in the group arena. n = number of nodes
 * to read (at most the chunk count). vp_world_read_group reads n items of
 * a LOD-`lod` node list at `off`. */
VP_API int vp_world_group_nodes(vp_world *w, int lod, uint64_t *off, uint32_t *items, uint32_t n);
VP_API int vp_world_read_group(vp_world *w, int lod, uint64_t off, uint64_t n, int16_t *dst);

/* RLE codec on host buffers (the device does the work). vp_rle_encode is
 * rle_compress (src/chunkset/rle.c:44-87): out receives the stream
 * including its 0 terminator, *out_len its word count; lengths below
 * 0xFFFFFF. vp_rle_decode is rle_decompress (src/chunkset/rle.c:90-117):
 * the first word is always consumed, decoding stops at the first 0 word;
 * *out_len receives the voxel count. VP_EOVERFLOW when out_cap is short
 * (*out_len then holds the size needed). */
VP_API int vp_rle_encode(vp_ctx *ctx, const uint8_t *vox, uint32_t length, uint32_t *out, uint32_t out_cap,
			 uint32_t *out_len);
VP_API int vp_rle_decode(vp_ctx *ctx, const uint32_t *words, uint32_t nwords, uint8_t *out, uint32_t out_cap,
			 uint32_t *out_len);

/* Geometry rebuild of a small chunk set that allocates no memory; it has
 * no counterpart in the reference. For callers that cannot allocate device
 * memory when they need geometry: a render or input thread that must not
 * stall on cudaMalloc's implicit device synchronisation, or an engine whose
 * own allocator owns all device memory. Every input and output is a device
 * pointer the caller provides: the chunks' RLE streams in `pool` (4-byte
 * aligned, pool_words readable words), their word offsets and lengths
 * (terminator included), the shadow map, optional per-chunk mesh flags,
 * three output buffers (splats, vertices, indices; bytes) and one result
 * record per chunk. Streams are laid out as vp_world_upload lays them out:
 * each starts on a 16-byte boundary and the pool holds at least 8 words
 * after each stream's terminator. They are checked on the device before
 * anything decodes them; a chunk whose stream is out of bounds, misaligned
 * or malformed (a zero count, counts not summing to the chunk's voxels, no
 * terminator) is built as air, its neighbours see air, and its result gets
 * status VP_STATUS_BAD_STREAM. The working data lives in a fixed 4 MiB
 * device array the library holds on every GPU that loads it (enough for 256
 * chunks of 64^3, 512 of 32^3, 2048 of 16^3 or 4096 of 8^3); larger sets
 * return VP_EOVERFLOW, more than 2^24 chunks VP_EUNSUPPORTED. The first call on a device looks the
 * array up (cudaGetSymbolAddress) and should come before any stream capture.
 * Calls share that array: each call resets it, and calls that overlap on the
 * GPU race. The work is queued on `stream` (asynchronous); a result whose
 * status is VP_STATUS_OVERFLOW means an output buffer was too small for
 * that chunk. */
#define VP_STATUS_OVERFLOW 1u   /* vp_chunk_result.status: output arena too small */
#define VP_STATUS_BAD_STREAM 2u /* vp_chunk_result.status: the chunk's stream failed the check */
#define VP_STATUS_TIMEOUT 4u    /* vp_chunk_result.status: a bounded device wait for its data ran out */

/* Self-test of the bounded wait behind VP_STATUS_TIMEOUT: one CTA arms the
 * decoded-chunk handoff's completion barrier for 16 bytes that no copy will
 * bring, waits as a geometry CTA does (2^16 tries) and records the outcome.
 * *status gets VP_STATUS_TIMEOUT when the wait gave up and the kernel
 * returned; the device stays usable. */
VP_API int vp_selftest_handoff_wait(int device, uint32_t *status);
VP_API int vp_rebuild_noalloc(int device, void *stream, int root_bitw, const int max_bitw[3], const uint32_t *pool,
			      uint64_t pool_words, const uint64_t *off, const uint32_t *len, const uint16_t *shadow,
			      uint64_t shadow_len, uint32_t shadow_w, const uint8_t *make_mesh, int lod_max,
			      int16_t *svl, uint64_t svl_bytes, int16_t *vbo, uint64_t vbo_bytes, uint32_t *ibo,
			      uint64_t ibo_bytes, vp_chunk_result *results);

/* Draw culling and LOD selection of the last rebuild made with
 * VP_REBUILD_GROUP (octree_cull, src/game.c:319-395, started from LOD
 * top_lod over the roots of src/game.c:517-524; frustum planes of
 * src/gfx/fcull.c from the column-major view-projection matrix). The walk's
 * draw queues, in its order: chunks whose mesh is drawn (chunk index) and
 * octree nodes whose grouped splats are drawn (lod << 24 | node index, node
 * numbered as in vp_world_group_nodes). *n_mesh / *n_svl get the queue
 * lengths; VP_EOVERFLOW when a capacity is short. top_lod must not exceed
 * the grouped LOD. */
VP_API int vp_world_cull(vp_world *w, const float view_proj[16], const float lod_origin[3], int top_lod,
			 uint32_t *mesh_out, uint32_t mesh_cap, uint32_t *n_mesh, uint32_t *svl_out, uint32_t svl_cap,
			 uint32_t *n_svl);
/* Mesh-or-splat mode of every chunk from the LOD origin (make_mesh =
 * chunk centre within 512 voxels, src/game.c:612-625), computed on the
 * device and applied to the next rebuild; make_mesh_out (optional) gets it. */
VP_API int vp_world_camera_modes(vp_world *w, const float lod_origin[3], uint8_t *make_mesh_out);

/* The world file / wire format: a 64-byte header (magic "VPW1", version 1,
 * root_bitw, max_bitw[3], nchunks, shadow_w, pool_words, shadow_len,
 * pad_rows), then off[nchunks] (u64), len[nchunks] (u32), the packed
 * streams (u32, each on a 16-byte boundary) and the u16 shadow map, all
 * little endian (layout in voxplat_gb300/csrc/vp_io.cu). vp_world_open
 * creates and uploads a world from a file (streams validated on the device). */
VP_API int vp_world_save(vp_world *w, const char *path);
VP_API int vp_world_open(vp_ctx *ctx, const char *path, vp_world **out);

/* Picking rays (chunkset_edit_raycast_until_solid, src/chunkset/edit.c:
 * 248-314), n at once: origins and vectors n x 3 floats; per ray the first
 * solid voxel (0 if none within 4095 steps), its coordinates (n x 3) and the
 * normal of the face entered (n x 3, one nonzero component on a hit). */
VP_API int vp_world_raycast(vp_world *w, uint32_t n, const float *origins, const float *vectors, uint8_t *voxels,
			    uint32_t *coords, int8_t *normals);

/* Headless rasteriser for the drawn geometry (resources/splat.vert.glsl,
 * splat.frag.glsl, mesh.vert.glsl, mesh.frag.glsl restated in CUDA): the
 * splats of the drawn octree nodes (svl_queue entries lod << 24 | node, the
 * grouped lists of the last VP_REBUILD_GROUP rebuild) and the meshes of the
 * drawn chunks (mesh_queue), e.g. vp_world_cull's queues. Matrices are
 * column-major. rgba gets width x height RGBA8 words (row 0 at the bottom),
 * depth (optional) the depth values. stats (optional, 4 values): splats and
 * triangles submitted, splats and triangles rasterised by whole blocks
 * (footprint above 256 pixels). */
typedef struct vp_camera {
	float projection[16], view_rotation[16], view_translation[16];
	float view_projection[16];   /* projection x view_rotation x view_translation */
	float inv_proj_view_rot[16]; /* inverse of projection x view_rotation */
	float proj_view_rot[16];     /* projection x view_rotation */
	float far_plane;
	int32_t width, height;
} vp_camera;
VP_API int vp_world_render(vp_world *w, const vp_camera *cam, const uint32_t *mesh_queue, uint32_t n_mesh,
			   const uint32_t *svl_queue, uint32_t n_svl, uint32_t *rgba, float *depth, uint64_t *stats);

/* Kernel timing: with timing on, every rebuild records CUDA events around
 * its passes on the context stream; vp_world_kernel_ms waits for the stream
 * and returns the summed milliseconds since the last call of ms[0] the shell
 * pass, ms[1] the geometry pass and ms[2] the grouping (n <= 3 values), and
 * the number of kernel launches, then resets them. */
VP_API int vp_ctx_set_timing(vp_ctx *ctx, int on);
VP_API int vp_world_kernel_ms(vp_world *w, double *ms, int n, uint32_t *launches);

/* Batches of standalone chunks of mixed root sizes (8..128): each chunk is
 * its own 1x1x1 ChunkSet (neighbours are the air null chunk) with its own
 * shadow map, 2R wide. This is how chunkset_manage (src/chunkset.c:233-507)
 * meshes chunks of unrelated sets, batched into one GPU pass. */
typedef struct vp_batch vp_batch;

#define VP_BATCH_MIXED 0 /* one persistent launch over items of every root size */
#define VP_BATCH_SPLIT 1 /* one persistent launch per root size, run concurrently */

typedef struct vp_batch_tune {
	int strategy;     /* VP_BATCH_MIXED or VP_BATCH_SPLIT */
	int min_blocks;   /* MIXED: 2 = registers capped for two CTAs per SM, 1 = uncapped */
	int order;        /* 0 = longest stream first, 1 = by root size then longest (SPLIT needs 1) */
	uint32_t ctas;    /* MIXED: persistent CTAs, 0 = as many as fit */
	float ms;         /* vp_batch_autotune: measured rebuild time of this configuration */
	uint32_t threads; /* threads per chunk (CTA) for chunks up to 64^3: 256 or 512 (0 = 512) */
	uint32_t grain;   /* MIXED and the 128^3 launch: chunks per dequeue from the work queue (0 = 1) */
} vp_batch_tune;

VP_API int vp_batch_create(vp_ctx *ctx, uint32_t n, const int *root_bitw, vp_batch **out);
VP_API void vp_batch_destroy(vp_batch *b);
/* Streams in the reference format, chunk k at pool[off[k] .. off[k]+len[k]),
 * and chunk k's shadow map at shadow[shadow_off[k] ..] (shadow_len[k]
 * entries, padded rows included). */
VP_API int vp_batch_upload(vp_batch *b, const uint32_t *pool, uint64_t pool_words, const uint64_t *off,
			   const uint32_t *len, const uint16_t *shadow, const uint64_t *shadow_off,
			   const uint64_t *shadow_len);
VP_API int vp_batch_set_modes(vp_batch *b, const uint8_t *make_mesh);
/* flags: VP_REBUILD_PLAIN = one launch per chunk; VP_REBUILD_GRAPH = replay
 * the CUDA graph of the tuned configuration (captured on first use and after
 * arena growth); otherwise the tuned configuration launched directly. */
VP_API int vp_batch_rebuild(vp_batch *b, int lod_max, unsigned flags);
VP_API int vp_batch_finish(vp_batch *b);
/* Time candidate configurations on this batch (graph replays) and keep the
 * fastest: first the strategies and orders, then, around the best of
 * those, threads per chunk (256, 512), chunks per dequeue (1, 2, 4) and,
 * for MIXED, the persistent grid (as many CTAs as fit, or one per SM).
 * `tried` (capacity *ntried) receives each with its time; *ntried gets the
 * number timed. */
VP_API int vp_batch_autotune(vp_batch *b, int lod_max, vp_batch_tune *best, vp_batch_tune *tried, int *ntried);
VP_API int vp_batch_set_tune(vp_batch *b, const vp_batch_tune *t);
VP_API int vp_batch_get_tune(vp_batch *b, vp_batch_tune *t);
VP_API int vp_batch_results(vp_batch *b, vp_chunk_result *out, uint32_t n);
VP_API int vp_batch_read_svl(vp_batch *b, uint64_t off, uint64_t n, int16_t *dst);
VP_API int vp_batch_read_vbo(vp_batch *b, uint64_t off, uint64_t n, int16_t *dst);
VP_API int vp_batch_read_ibo(vp_batch *b, uint64_t off, uint64_t n, uint32_t *dst);
/* Summed rebuild time (events around each rebuild while timing is on) and
 * kernel launches since the last call. */
VP_API int vp_batch_kernel_ms(vp_batch *b, double *ms, uint32_t *launches);

#ifdef __cplusplus
}
#endif
#endif
