/*
 * voxgpu_dropin.h — the reference's own hot-path entry points, same names,
 * same signatures, same results, computed on the GPU. Link libvoxgpu.so in
 * place of src/chunkset/mesher.c and src/chunkset/rle.c (and, for the
 * batched mesher, in place of chunkset_manage in src/chunkset.c).
 *
 * Data stays where the reference keeps it: voxels, RLE streams, masks,
 * geometry buffers and the shadow map are host memory. Each per-chunk call
 * copies its inputs to the device, runs the kernels and copies the results
 * back ("plain path"); chunkset_manage instead keeps a device mirror of the
 * whole set and rebuilds every eligible chunk in one batched launch.
 *
 * Conventions where the reference is undefined (same as the oracle):
 *   - shadow-map reads at or past shadow_map_length read 0;
 *   - chunk_make_mask always scans all faces (the reference's early-out
 *     reads uninitialised memory, src/chunkset/mesher.c:404-409);
 *   - rle_decompress sizes its output from the stream itself, not from the
 *     length of the last rle_compress call (src/chunkset/rle.c:32,95).
 * The functions return void like the reference's; errors are reported by
 * vp_dropin_last_error() (0 when the last call succeeded).
 */
#ifndef VOXGPU_DROPIN_H
#define VOXGPU_DROPIN_H

#include "voxgpu.h"
#include "voxgpu_chunkset.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/chunkset/mesher.h:7-14 */
VP_API void chunk_make_mesh(struct ChunkSet *setp, struct ChunkMD *cp, int16_t *geometry, uint32_t *geometry_items,
			    uint32_t *index, uint32_t *index_items);
/* src/chunkset/mesher.h:17-21 */
VP_API void chunk_make_mask(struct ChunkSet *setp, struct ChunkMD *cp, uint8_t *mask);
/* src/chunkset/mesher.h:23-28 */
VP_API void chunk_mask_downsample(struct ChunkSet *setp, int8_t lod, Voxel *mask, Voxel *work);
/* src/chunkset/mesher.h:30-37 */
VP_API void chunk_make_splatlist(struct ChunkSet *setp, struct ChunkMD *cp, uint8_t level, Voxel *mask,
				 int16_t *geometry, uint32_t *geometry_items);
/* src/chunkset/rle.h:7-8; the returned buffer comes from the allocator set
 * by vp_dropin_set_allocator (malloc by default) */
VP_API Voxel *rle_compress(Voxel *data, uint32_t length);
VP_API Voxel *rle_decompress(void *vdata);
/* src/chunkset.h:227 — batched: every chunk with remesh or dirty set and no
 * unconsumed geometry is rebuilt in one launch and published into its
 * ChunkMD fields as src/chunkset.c:311-505 does (without the 100 ms rate
 * limit, the 8-chunks-per-call cap and idle recompression). */
VP_API void chunkset_manage(struct ChunkSet *set);

/* Host allocator for the buffers the drop-in functions hand out (the
 * reference uses its labelled heap: _mem_alloc / _mem_free, src/mem.h). */
VP_API void vp_dropin_set_allocator(void *(*alloc_fn)(size_t), void (*free_fn)(void *));
/* Device used by the drop-in functions (default 0); call before the first. */
VP_API int vp_dropin_set_device(int device);
/* Status of the last drop-in call on this thread (VP_OK or a VP_E* code). */
VP_API int vp_dropin_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
