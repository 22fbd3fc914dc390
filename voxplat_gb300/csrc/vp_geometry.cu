/*
 * vp_geometry.cu — host-side dispatch of the geometry kernels by root size.
 * The kernels live in vp_geometry_dev.cuh and are instantiated one root size
 * (or one mixed variant) per translation unit: vp_geometry_r{3..7}.cu,
 * vp_geometry_mixed{1,2}.cu.
 */
#include <algorithm>

#include "vp_geometry_dev.cuh"

namespace vp {

int geometry_mixed_ctas_per_sm(int min_blocks, int threads)
{
	return min_blocks >= 2 ? geometry_mixed_ctas_per_sm_b2(threads) : geometry_mixed_ctas_per_sm_b1(threads);
}

cudaError_t launch_geometry_mixed(int min_blocks, const GeoLaunch &L, cudaStream_t st)
{
	if (!L.n_items) return cudaSuccess;
	/* 128^3 items use the CTA's scratch slot: never more CTAs than slots */
	uint32_t grid = L.queue ? L.ctas : L.n_items;
	if (L.big_scratch) grid = std::min(grid, L.big_slots);
	return min_blocks >= 2 ? launch_geometry_mixed_b2(grid, L, st) : launch_geometry_mixed_b1(grid, L, st);
}

size_t geometry_smem_bytes(int root_bitw)
{
	switch (root_bitw) {
	case 3: return Geo<3>::bytes;
	case 4: return Geo<4>::bytes;
	case 5: return Geo<5>::bytes;
	case 6: return Geo<6>::bytes;
	case 7: return 1; /* working set in global scratch */
	default: return 0;
	}
}

int geometry_ctas_per_sm(int root_bitw, int threads)
{
	switch (root_bitw) {
	case 3: return geometry_ctas_per_sm_r3(threads);
	case 4: return geometry_ctas_per_sm_r4(threads);
	case 5: return geometry_ctas_per_sm_r5(threads);
	case 6: return geometry_ctas_per_sm_r6(threads);
	default: return 1;
	}
}

size_t shell_words_per_chunk(int root_bitw)
{
	return root_bitw == 7 ? Big::shell_words : 6u * (1u << root_bitw);
}
size_t shell_cols_per_chunk(int root_bitw) { return 3u * (1u << root_bitw) * (1u << root_bitw); }

size_t decoded_bytes_per_chunk(int root_bitw)
{
	switch (root_bitw) {
	case 3: return Geo<3>::dec_bytes;
	case 4: return Geo<4>::dec_bytes;
	case 5: return Geo<5>::dec_bytes;
	case 6: return Geo<6>::dec_bytes;
	default: return 0; /* 128^3 chunks are not handed over */
	}
}

cudaError_t launch_geometry(int root_bitw, const GeoLaunch &L, cudaStream_t st)
{
	switch (root_bitw) {
	case 3: return launch_geometry_r3(L, st);
	case 4: return launch_geometry_r4(L, st);
	case 5: return launch_geometry_r5(L, st);
	case 6: return launch_geometry_r6(L, st);
	case 7: return launch_big(L, st);
	default: return cudaErrorInvalidValue;
	}
}

} // namespace vp
