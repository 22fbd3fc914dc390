/* vp_geometry.h — host-side launch interface of the geometry kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

struct GeoLaunch {
	const SetDesc *sets;        /* device array */
	const WorkItem *items;      /* device array: geometry work */
	uint32_t n_items;
	const WorkItem *shell_items;/* device array: chunks whose shell to write */
	uint32_t n_shell;
	/* <= 64^3 chunks: single-run chunks (one run and the terminator) whose
	 * shells, unless all air, the shell pass writes without decoding */
	const WorkItem *uni_items;
	uint32_t n_uni;
	int run_shell;
	unsigned int *queue;        /* device counter for persistent CTAs, or NULL */
	uint32_t ctas;              /* persistent grid size */
	uint32_t threads;
	ChunkOut *outs;
	Arena svl, vbo, ibo;
	int lod_max;
	uint8_t *big_scratch;       /* 128^3 chunks: per-CTA working sets */
	uint32_t big_slots;         /* slots in big_scratch = CTAs of a launch */
	/* <= 64^3 chunks, or NULL: decoded chunks handed from the shell pass
	 * to the geometry pass, decoded_bytes_per_chunk() each, chunk c in slot
	 * dec_slot[c] (kNoSlot: not handed over, the geometry pass decodes it).
	 * The shell pass stores each chunk it decodes that has a slot; the
	 * geometry pass loads those instead of decoding, so a launch pair that
	 * passes it must shell every non-empty chunk whose geometry it builds. */
	uint8_t *decoded;
	const uint32_t *dec_slot;
	/* persistent mixed and 128^3 launches: items per dequeue (0 = 1) */
	uint32_t grain;
};

size_t geometry_smem_bytes(int root_bitw);
size_t big_scratch_slot_bytes();
size_t shell_words_per_chunk(int root_bitw);
size_t shell_cols_per_chunk(int root_bitw);
size_t decoded_bytes_per_chunk(int root_bitw);
int geometry_ctas_per_sm(int root_bitw, int threads);
cudaError_t launch_geometry(int root_bitw, const GeoLaunch &L, cudaStream_t st);
/* One persistent launch over items of any root size (sets may differ in
 * root_bitw); min_blocks 2 caps registers for two CTAs per SM, 1 leaves the
 * 128^3 path its registers. With 128^3 items, grid <= big_slots. */
int geometry_mixed_ctas_per_sm(int min_blocks, int threads);
cudaError_t launch_geometry_mixed(int min_blocks, const GeoLaunch &L, cudaStream_t st);

/* per-translation-unit launchers behind the dispatchers above (one root size
 * or one mixed variant per unit, so the kernels compile in parallel) */
cudaError_t launch_geometry_r3(const GeoLaunch &L, cudaStream_t st);
cudaError_t launch_geometry_r4(const GeoLaunch &L, cudaStream_t st);
cudaError_t launch_geometry_r5(const GeoLaunch &L, cudaStream_t st);
cudaError_t launch_geometry_r6(const GeoLaunch &L, cudaStream_t st);
cudaError_t launch_big(const GeoLaunch &L, cudaStream_t st);
int geometry_ctas_per_sm_r3(int threads);
int geometry_ctas_per_sm_r4(int threads);
int geometry_ctas_per_sm_r5(int threads);
int geometry_ctas_per_sm_r6(int threads);
int geometry_mixed_ctas_per_sm_b1(int threads);
int geometry_mixed_ctas_per_sm_b2(int threads);
cudaError_t launch_geometry_mixed_b1(uint32_t grid, const GeoLaunch &L, cudaStream_t st);
cudaError_t launch_geometry_mixed_b2(uint32_t grid, const GeoLaunch &L, cudaStream_t st);

} // namespace vp
