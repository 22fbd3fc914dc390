/* vp_geometry_r7.cu — the shell and geometry kernels for 128^3 chunks
 * (persistent CTAs, each with a slot of global scratch) and their host
 * launcher. */
#include "vp_geometry_dev.cuh"

namespace vp {

/* 128^3 chunks: persistent CTAs, each with its own scratch slot; items come
 * from the queue, or by a grid stride when there is none. */
__global__ void __launch_bounds__(512, 1) k_shell_big(const SetDesc *__restrict__ sets, const WorkItem *__restrict__ items,
						      uint32_t nitems, uint8_t *scratch)
{
	__shared__ uint32_t tmp[64];
	__shared__ int32_t nbr[28];
	const BigMem m = big_carve(scratch, blockIdx.x, tmp, nbr);
	const uint32_t N = (uint32_t)Big::R * Big::R * Big::R;
	for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x) {
		const WorkItem wi = items[it];
		const SetDesc S = sets[wi.set];
		if (chunk_is_null(S, wi.chunk, N)) continue;
		const uint32_t *stream = S.pool + S.off[wi.chunk];
		decode_big(stream, S.len[wi.chunk] - 1u, m);
		shell_big(stream, m, S.shell_bits + (size_t)wi.chunk * Big::shell_words,
			  S.shell_col + (size_t)wi.chunk * Big::shell_cols);
		__syncthreads();
	}
}

__global__ void __launch_bounds__(1024, 1) k_geometry_big(const SetDesc *__restrict__ sets,
							 const WorkItem *__restrict__ items, uint32_t nitems,
							 unsigned int *queue, ChunkOut *outs, Arena asvl, Arena avbo,
							 Arena aibo, int lod_max, uint8_t *scratch, uint32_t grain)
{
	__shared__ uint32_t tmp[64];
	__shared__ int32_t nbr[28];
	__shared__ uint32_t s_item;
	const BigMem m = big_carve(scratch, blockIdx.x, tmp, nbr);
	uint32_t next = blockIdx.x;
	for (;;) {
		/* `grain` consecutive items per dequeue */
		if (threadIdx.x == 0) s_item = queue ? atomicAdd(queue, grain) : next;
		__syncthreads();
		const uint32_t it0 = s_item;
		if (it0 >= nitems) break;
		next += gridDim.x;
		const uint32_t it1 = queue ? min(it0 + grain, nitems) : it0 + 1u;
		for (uint32_t it = it0; it < it1; it++) {
			const WorkItem wi = items[it];
			const SetDesc S = sets[wi.set];
			geometry_item_big(S, wi, outs + wi.slot, m, asvl, avbo, aibo, lod_max);
			__syncthreads();
		}
	}
}

/* 128^3 chunks: shells and geometry by persistent CTAs, one scratch slot
 * each (grid = min(items, slots)). */
cudaError_t launch_big(const GeoLaunch &L, cudaStream_t st)
{
	if (!L.big_scratch || !L.big_slots) return cudaErrorInvalidValue;
	cudaError_t e = cudaSuccess;
	if (L.run_shell && L.n_shell) {
		const uint32_t grid = std::min(L.n_shell, L.big_slots);
		k_shell_big<<<grid, 512, 0, st>>>(L.sets, L.shell_items, L.n_shell, L.big_scratch);
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	if (L.n_items) {
		const uint32_t grid = std::min(L.n_items, L.big_slots);
		/* 1024 threads at 64 registers: twice the warps of the small path's
		 * CTAs to hide the latency of the scratch, which lives in L2 */
		k_geometry_big<<<grid, 1024, 0, st>>>(L.sets, L.items, L.n_items, L.queue, L.outs, L.svl, L.vbo, L.ibo,
						    L.lod_max, L.big_scratch, L.grain ? L.grain : 1u);
		e = cudaGetLastError();
	}
	return e;
}

size_t big_scratch_slot_bytes() { return Big::slot_bytes; }

} // namespace vp
