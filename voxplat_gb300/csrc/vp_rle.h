/* vp_rle.h — launch interface of the RLE codec kernels. */
#pragma once
#include "vp_dev.cuh"

namespace vp {

/* Encode nchunks voxel volumes of N bytes (contiguous, 16-byte aligned and
 * padded) into streams bump-allocated from `pool` (cap_words, cursor);
 * out_off/out_len per chunk; *status gets kStatusOverflow on lack of room. */
cudaError_t launch_rle_encode(const uint8_t *vox, uint32_t nchunks, uint32_t N, uint32_t *pool, uint64_t cap_words,
			      unsigned long long *cursor, uint64_t *out_off, uint32_t *out_len, uint32_t *status,
			      cudaStream_t st);

/* Decode the streams of `chunks` (or 0..n-1 when chunks is NULL) into
 * consecutive N-byte volumes; *status gets kStatusBadStream when a stream
 * does not cover exactly N voxels. */
cudaError_t launch_rle_decode_bytes(const uint32_t *pool, const uint64_t *off, const uint32_t *len,
				    const uint32_t *chunks, uint32_t n, uint32_t N, uint8_t *vox, uint32_t *status,
				    cudaStream_t st);

/* Tile-parallel variants for a few chunks (many CTAs per chunk).
 * Decode: tile_scratch holds n * (N/4096 + 2) words. Encode: tile_scratch
 * n * (N/8192 + 1) words, nruns n words, run_scratch n * (N + 1) words;
 * the voxel volumes must be padded to 16 bytes. */
cudaError_t launch_rle_decode_tiles(const uint32_t *pool, const uint64_t *off, const uint32_t *len, const uint32_t *chunks,
				    uint32_t n, uint32_t N, uint8_t *vox, uint32_t *tile_scratch, cudaStream_t st);
cudaError_t launch_rle_encode_tiles(const uint8_t *vox, uint32_t n, uint32_t N, uint32_t *pool, uint64_t cap_words,
				    unsigned long long *cursor, uint64_t *out_off, uint32_t *out_len, uint32_t *status,
				    uint32_t *tile_scratch, uint32_t *nruns, uint32_t *run_scratch, cudaStream_t st);

/* Check every stream on the device (status |= kStatusBadStream and
 * first_bad = lowest failing chunk); status and first_bad are set by the
 * caller (0 and ~0). */
cudaError_t launch_validate_streams(const uint32_t *pool, const uint64_t *off, const uint32_t *len, uint32_t nchunks,
				    uint64_t N, uint32_t *status, uint32_t *first_bad, cudaStream_t st);

/* dst[noff[c] ..] = src[off[c] ..], len[c] words, for every chunk c. */
cudaError_t launch_copy_streams(const uint32_t *src, const uint64_t *off, const uint32_t *len, const uint64_t *noff,
				uint32_t *dst, uint32_t nchunks, cudaStream_t st);

} // namespace vp
