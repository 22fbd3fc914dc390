/*
 * vp_rle.cu — RLE codec kernels (reference format, src/chunkset/rle.c:14-22:
 * u32 words `count | colour << 24`, runs capped at 0xFFFFFF, one 0 word
 * terminating the stream).
 *
 * Encode (rle_compress, src/chunkset/rle.c:44-87), one CTA per chunk:
 *   pass 1  run-boundary detection over the voxels (16 per thread, the
 *           previous byte from the neighbouring lane), block-wide count;
 *   alloc   the exact stream length is bump-allocated in the output pool
 *           (16-byte aligned);
 *   pass 2  every run start p writes `p | colour << 24` at its run index
 *           (block prefix sum of boundary counts);
 *   pass 3  in place, word r becomes (start[r+1] - start[r]) | colour << 24
 *           (reads of a tile complete before its writes), then the 0.
 * Chunks up to 128^3 voxels never reach the 0xFFFFFF run cap (inputs are
 * limited to 2^24 - 1 voxels). The voxel buffer is padded to 16 bytes.
 *
 * Decode to bytes (rle_decompress, src/chunkset/rle.c:90-117), one CTA per
 * chunk: tiles of 4096 runs get their start positions by a block prefix sum
 * into shared memory; each thread then fills 16-byte output segments,
 * finding the segment's first run by binary search and walking forward.
 */
#include "vp_dev.cuh"
#include "vp_rle.h"

namespace vp {

__device__ __forceinline__ uint32_t byte_of(const uint4 &q, int j)
{
	const uint32_t w = j < 4 ? q.x : (j < 8 ? q.y : (j < 12 ? q.z : q.w));
	return (w >> (8 * (j & 3))) & 0xFFu;
}

/* boundary bits of 16 voxels starting at p (bit j: voxel p+j starts a run) */
__device__ __forceinline__ uint32_t boundaries16(const uint4 &q, uint32_t prev_byte, bool first)
{
	uint32_t b = 0, prev = prev_byte;
#pragma unroll
	for (int j = 0; j < 16; j++) {
		const uint32_t v = byte_of(q, j);
		if (v != prev || (first && j == 0)) b |= 1u << j;
		prev = v;
	}
	return b;
}

/* boundary bits at or past N are not runs (the device buffer is padded) */
__device__ __forceinline__ uint32_t tail_mask(uint32_t p, uint32_t N)
{
	return p + 16u <= N ? 0xFFFFu : ((1u << (N - p)) - 1u);
}

__global__ void __launch_bounds__(512) k_rle_encode(const uint8_t *__restrict__ vox, uint32_t nchunks, uint32_t N,
						    uint32_t *pool, uint64_t cap_words, unsigned long long *cursor,
						    uint64_t *out_off, uint32_t *out_len, uint32_t *status)
{
	__shared__ uint32_t tmp[64];
	__shared__ unsigned long long s_base;
	__shared__ uint32_t s_ok;
	const uint32_t c = blockIdx.x;
	if (c >= nchunks) return;
	const uint8_t *v = vox + (size_t)c * N;
	const uint32_t T = 16u * blockDim.x;
	const int lane = threadIdx.x & 31;
	/* pass 1: count run starts */
	uint32_t cnt = 0;
	for (uint32_t base = 0; base < N; base += T) {
		const uint32_t p = base + 16u * threadIdx.x;
		uint4 q = make_uint4(0, 0, 0, 0);
		if (p < N) q = __ldg((const uint4 *)(v + p));
		const uint32_t last = byte_of(q, 15);
		uint32_t prev = __shfl_up_sync(kFull, last, 1);
		if (lane == 0 && p > 0 && p < N) prev = v[p - 1];
		if (p < N) cnt += __popc(boundaries16(q, prev, p == 0) & tail_mask(p, N));
	}
	uint32_t nruns;
	block_excl_add(cnt, tmp, &nruns);
	const uint32_t words = nruns + 1u;
	if (threadIdx.x == 0) {
		const uint64_t padded = (words + 3u) & ~3u;
		const unsigned long long b = atomicAdd(cursor, (unsigned long long)padded);
		const uint32_t ok = b + padded <= cap_words;
		s_base = b;
		s_ok = ok;
		out_off[c] = b;
		out_len[c] = ok ? words : 0u;
		if (!ok) atomicOr(status, kStatusOverflow);
	}
	__syncthreads();
	if (!s_ok) return;
	uint32_t *out = pool + s_base;
	/* pass 2: packed run starts */
	uint32_t run0 = 0;
	for (uint32_t base = 0; base < N; base += T) {
		const uint32_t p = base + 16u * threadIdx.x;
		uint4 q = make_uint4(0, 0, 0, 0);
		if (p < N) q = __ldg((const uint4 *)(v + p));
		const uint32_t last = byte_of(q, 15);
		uint32_t prev = __shfl_up_sync(kFull, last, 1);
		if (lane == 0 && p > 0 && p < N) prev = v[p - 1];
		const uint32_t b = p < N ? (boundaries16(q, prev, p == 0) & tail_mask(p, N)) : 0u;
		uint32_t tot;
		uint32_t r = run0 + block_excl_add(__popc(b), tmp, &tot);
		for (uint32_t m = b; m; m &= m - 1u) {
			const int j = __ffs(m) - 1;
			out[r++] = (p + (uint32_t)j) | (byte_of(q, j) << 24);
		}
		run0 += tot;
	}
	__syncthreads();
	/* pass 3: starts -> counts, tile by tile (8 runs per thread); every tile
	 * reads all its inputs (and the next tile's first start) before any
	 * write */
	for (uint32_t base = 0; base < nruns; base += 8u * blockDim.x) {
		const uint32_t r0 = base + 8u * threadIdx.x;
		uint32_t cur[9];
#pragma unroll
		for (int j = 0; j < 9; j++) {
			const uint32_t r = r0 + j;
			cur[j] = r < nruns ? out[r] : (N | 0u);
		}
		__syncthreads();
#pragma unroll
		for (int j = 0; j < 8; j++) {
			const uint32_t r = r0 + j;
			if (r < nruns) out[r] = ((cur[j + 1] & 0xFFFFFFu) - (cur[j] & 0xFFFFFFu)) | (cur[j] & 0xFF000000u);
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) out[nruns] = 0u;
}

/* ---------------------------------------------------------------- */

__global__ void __launch_bounds__(512) k_rle_decode_bytes(const uint32_t *__restrict__ pool,
							  const uint64_t *__restrict__ off, const uint32_t *__restrict__ len,
							  const uint32_t *__restrict__ chunks, uint32_t n, uint32_t N,
							  uint8_t *vox, uint32_t *status)
{
	/* generic over N: run starts by a block scan, then each thread fills
	 * 16-byte segments by a binary search over the tile's starts */
	__shared__ uint32_t tmp[64];
	__shared__ uint32_t s_start[4097];
	__shared__ uint32_t s_word[4096];
	const uint32_t k = blockIdx.x;
	if (k >= n) return;
	const uint32_t c = chunks ? chunks[k] : k;
	const uint32_t *s = pool + off[c];
	const uint32_t nruns = len[c] - 1u;
	uint8_t *dst = vox + (size_t)k * N;
	uint32_t start0 = 0;
	for (uint32_t base = 0; base < nruns; base += 4096u) {
		const uint32_t cnt_tile = min(4096u, nruns - base);
		/* starts of this tile's runs: 8 per thread */
		uint32_t w[8], sum = 0;
		for (int j = 0; j < 8; j++) {
			const uint32_t r = base + 8u * threadIdx.x + j;
			w[j] = r < base + cnt_tile ? __ldg(s + r) : 0u;
			sum += w[j] & 0xFFFFFFu;
		}
		uint32_t tot;
		uint32_t pos = start0 + block_excl_add(sum, tmp, &tot);
		for (int j = 0; j < 8; j++) {
			const uint32_t i = 8u * threadIdx.x + j;
			if (i < cnt_tile) {
				s_start[i] = pos;
				s_word[i] = w[j];
			}
			pos += w[j] & 0xFFFFFFu;
		}
		if (threadIdx.x == 0) s_start[cnt_tile] = start0 + tot;
		__syncthreads();
		/* fill bytes [start0, start0 + tot) in 16-byte segments; segment
		 * edges that straddle tiles are written bytewise */
		const uint32_t lo = start0, hi = start0 + tot;
		const uint32_t seg0 = lo & ~15u;
		for (uint32_t p = seg0 + 16u * threadIdx.x; p < hi; p += 16u * blockDim.x) {
			uint32_t a = 0, b = cnt_tile; /* last run with start <= p */
			if (p >= lo) {
				while (b - a > 1) {
					const uint32_t mid = (a + b) >> 1;
					if (s_start[mid] <= p) a = mid; else b = mid;
				}
			}
			uint8_t bytes[16];
			uint32_t r = a;
			for (int j = 0; j < 16; j++) {
				const uint32_t q = p + j;
				while (r + 1 < cnt_tile && s_start[r + 1] <= q) r++;
				bytes[j] = (uint8_t)(s_word[r] >> 24);
			}
			if (p >= lo && p + 16u <= hi && p + 16u <= N) {
				uint4 o;
				o.x = bytes[0] | (bytes[1] << 8) | (bytes[2] << 16) | ((uint32_t)bytes[3] << 24);
				o.y = bytes[4] | (bytes[5] << 8) | (bytes[6] << 16) | ((uint32_t)bytes[7] << 24);
				o.z = bytes[8] | (bytes[9] << 8) | (bytes[10] << 16) | ((uint32_t)bytes[11] << 24);
				o.w = bytes[12] | (bytes[13] << 8) | (bytes[14] << 16) | ((uint32_t)bytes[15] << 24);
				*(uint4 *)(dst + p) = o;
			} else {
				for (int j = 0; j < 16; j++)
					if (p + j >= lo && p + j < hi && p + j < N) dst[p + j] = bytes[j];
			}
		}
		start0 += tot;
		__syncthreads();
	}
	if (threadIdx.x == 0 && start0 != N) atomicOr(status, kStatusBadStream);
}

/* one CTA per chunk: copy its stream to its new offset */
__global__ void k_copy_streams(const uint32_t *__restrict__ src, const uint64_t *__restrict__ off,
			       const uint32_t *__restrict__ len, const uint64_t *__restrict__ noff, uint32_t *dst)
{
	const uint32_t c = blockIdx.x;
	const uint32_t n = len[c];
	const uint32_t *s = src + off[c];
	uint32_t *d = dst + noff[c];
	for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
}

cudaError_t launch_copy_streams(const uint32_t *src, const uint64_t *off, const uint32_t *len, const uint64_t *noff,
				uint32_t *dst, uint32_t nchunks, cudaStream_t st)
{
	if (!nchunks) return cudaSuccess;
	k_copy_streams<<<nchunks, 256, 0, st>>>(src, off, len, noff, dst);
	return cudaGetLastError();
}

cudaError_t launch_rle_encode(const uint8_t *vox, uint32_t nchunks, uint32_t N, uint32_t *pool, uint64_t cap_words,
			      unsigned long long *cursor, uint64_t *out_off, uint32_t *out_len, uint32_t *status,
			      cudaStream_t st)
{
	if (!nchunks) return cudaSuccess;
	k_rle_encode<<<nchunks, 512, 0, st>>>(vox, nchunks, N, pool, cap_words, cursor, out_off, out_len, status);
	return cudaGetLastError();
}

cudaError_t launch_rle_decode_bytes(const uint32_t *pool, const uint64_t *off, const uint32_t *len,
				    const uint32_t *chunks, uint32_t n, uint32_t N, uint8_t *vox, uint32_t *status,
				    cudaStream_t st)
{
	if (!n) return cudaSuccess;
	k_rle_decode_bytes<<<n, 512, 0, st>>>(pool, off, len, chunks, n, N, vox, status);
	return cudaGetLastError();
}

} // namespace vp

/* ------------------------------------------------------------------ */
/* Tile-parallel codec for a few chunks at a time (edit batches): each   */
/* chunk is split over many CTAs, so a handful of long streams still    */
/* fill the GPU. Tiles: kDecTile runs (decode), kEncTile voxels (encode).*/
/* ------------------------------------------------------------------ */

namespace vp {

constexpr uint32_t kDecTile = 4096;
constexpr uint32_t kEncTile = 8192;

/* per (tile, chunk): sum of the tile's run lengths */
__global__ void __launch_bounds__(512) k_dec_sums(const uint32_t *__restrict__ pool, const uint64_t *__restrict__ off,
						  const uint32_t *__restrict__ len, const uint32_t *__restrict__ chunks,
						  uint32_t *tile_sum, uint32_t max_tiles)
{
	__shared__ uint32_t tmp[64];
	const uint32_t t = blockIdx.x, k = blockIdx.y;
	const uint32_t c = chunks[k];
	const uint32_t nruns = len[c] - 1u;
	const uint32_t base = t * kDecTile;
	if (base >= nruns) {
		if (threadIdx.x == 0) tile_sum[k * max_tiles + t] = 0;
		return;
	}
	const uint32_t *s = pool + off[c];
	uint32_t sum = 0;
	for (uint32_t r = base + threadIdx.x; r < min(base + kDecTile, nruns); r += blockDim.x) sum += __ldg(s + r) & 0xFFFFFFu;
	uint32_t tot;
	block_excl_add(sum, tmp, &tot);
	if (threadIdx.x == 0) tile_sum[k * max_tiles + t] = tot;
}

/* per chunk: exclusive scan of its tile sums (one warp) */
__global__ void k_tile_scan(uint32_t *tile_sum, uint32_t max_tiles, uint32_t n)
{
	const uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	const int lane = threadIdx.x & 31;
	if (k >= n) return;
	uint32_t *v = tile_sum + (size_t)k * max_tiles;
	uint32_t carry = 0;
	for (uint32_t b = 0; b < max_tiles; b += 32) {
		const uint32_t i = b + lane;
		const uint32_t x = i < max_tiles ? v[i] : 0u;
		const uint32_t inc = warp_incl_add(x);
		if (i < max_tiles) v[i] = carry + inc - x;
		carry += __shfl_sync(kFull, inc, 31);
	}
}

/* per (tile, chunk): fill the voxels covered by the tile's runs */
__global__ void __launch_bounds__(512) k_dec_fill(const uint32_t *__restrict__ pool, const uint64_t *__restrict__ off,
						  const uint32_t *__restrict__ len, const uint32_t *__restrict__ chunks,
						  const uint32_t *__restrict__ tile_start, uint32_t max_tiles, uint32_t N,
						  uint8_t *vox)
{
	__shared__ uint32_t tmp[64];
	__shared__ uint32_t s_start[kDecTile + 1];
	__shared__ uint32_t s_word[kDecTile];
	const uint32_t t = blockIdx.x, k = blockIdx.y;
	const uint32_t c = chunks[k];
	const uint32_t nruns = len[c] - 1u;
	const uint32_t base = t * kDecTile;
	if (base >= nruns) return;
	const uint32_t *s = pool + off[c];
	uint8_t *dst = vox + (size_t)k * N;
	const uint32_t cnt_tile = min(kDecTile, nruns - base);
	uint32_t w[8], sum = 0;
	for (int j = 0; j < 8; j++) {
		const uint32_t r = base + 8u * threadIdx.x + j;
		w[j] = r < base + cnt_tile ? __ldg(s + r) : 0u;
		sum += w[j] & 0xFFFFFFu;
	}
	uint32_t tot;
	const uint32_t start0 = tile_start[k * max_tiles + t];
	uint32_t pos = start0 + block_excl_add(sum, tmp, &tot);
	for (int j = 0; j < 8; j++) {
		const uint32_t i = 8u * threadIdx.x + j;
		if (i < cnt_tile) {
			s_start[i] = pos;
			s_word[i] = w[j];
		}
		pos += w[j] & 0xFFFFFFu;
	}
	if (threadIdx.x == 0) s_start[cnt_tile] = start0 + tot;
	__syncthreads();
	const uint32_t lo = start0, hi = min(start0 + tot, N);
	for (uint32_t p = (lo & ~15u) + 16u * threadIdx.x; p < hi; p += 16u * blockDim.x) {
		uint32_t a = 0, b = cnt_tile;
		if (p >= lo) {
			while (b - a > 1) {
				const uint32_t mid = (a + b) >> 1;
				if (s_start[mid] <= p) a = mid; else b = mid;
			}
		}
		uint8_t bytes[16];
		uint32_t r = a;
		for (int j = 0; j < 16; j++) {
			const uint32_t q = p + j;
			while (r + 1 < cnt_tile && s_start[r + 1] <= q) r++;
			bytes[j] = (uint8_t)(s_word[r] >> 24);
		}
		if (p >= lo && p + 16u <= hi) {
			uint4 o;
			o.x = bytes[0] | (bytes[1] << 8) | (bytes[2] << 16) | ((uint32_t)bytes[3] << 24);
			o.y = bytes[4] | (bytes[5] << 8) | (bytes[6] << 16) | ((uint32_t)bytes[7] << 24);
			o.z = bytes[8] | (bytes[9] << 8) | (bytes[10] << 16) | ((uint32_t)bytes[11] << 24);
			o.w = bytes[12] | (bytes[13] << 8) | (bytes[14] << 16) | ((uint32_t)bytes[15] << 24);
			*(uint4 *)(dst + p) = o;
		} else {
			for (int j = 0; j < 16; j++)
				if (p + j >= lo && p + j < hi) dst[p + j] = bytes[j];
		}
	}
}

/* per (voxel tile, chunk): run starts in the tile */
__global__ void __launch_bounds__(512) k_enc_count(const uint8_t *__restrict__ vox, uint32_t N, uint32_t *tcount,
						   uint32_t max_tiles)
{
	__shared__ uint32_t tmp[64];
	const uint32_t t = blockIdx.x, k = blockIdx.y;
	const uint8_t *v = vox + (size_t)k * N;
	const uint32_t p = t * kEncTile + 16u * threadIdx.x;
	const int lane = threadIdx.x & 31;
	uint4 q = make_uint4(0, 0, 0, 0);
	if (p < N) q = __ldg((const uint4 *)(v + p));
	uint32_t prev = __shfl_up_sync(kFull, byte_of(q, 15), 1);
	if (lane == 0 && p > 0 && p < N) prev = v[p - 1];
	const uint32_t b = p < N ? (boundaries16(q, prev, p == 0) & tail_mask(p, N)) : 0u;
	uint32_t tot;
	block_excl_add(__popc(b), tmp, &tot);
	if (threadIdx.x == 0) tcount[k * max_tiles + t] = tot;
}

/* per chunk: scan tile counts, allocate the stream, write its terminator */
__global__ void k_enc_alloc(uint32_t *tcount, uint32_t max_tiles, uint32_t n, uint32_t N, uint32_t *pool,
			    uint64_t cap_words, unsigned long long *cursor, uint64_t *out_off, uint32_t *out_len,
			    uint32_t *nruns_out, uint32_t *status)
{
	const uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	const int lane = threadIdx.x & 31;
	if (k >= n) return;
	uint32_t *v = tcount + (size_t)k * max_tiles;
	uint32_t carry = 0;
	for (uint32_t b = 0; b < max_tiles; b += 32) {
		const uint32_t i = b + lane;
		const uint32_t x = i < max_tiles ? v[i] : 0u;
		const uint32_t inc = warp_incl_add(x);
		if (i < max_tiles) v[i] = carry + inc - x;
		carry += __shfl_sync(kFull, inc, 31);
	}
	if (lane == 0) {
		const uint32_t nruns = carry, words = nruns + 1u;
		const uint64_t padded = (words + 3u) & ~3u;
		const unsigned long long b = atomicAdd(cursor, (unsigned long long)padded);
		const bool ok = b + padded <= cap_words;
		out_off[k] = b;
		out_len[k] = ok ? words : 0u;
		nruns_out[k] = ok ? nruns : 0xFFFFFFFFu;
		if (ok)
			pool[b + nruns] = 0u;
		else
			atomicOr(status, kStatusOverflow);
	}
}

/* per (voxel tile, chunk): packed run starts (start | colour << 24) */
__global__ void __launch_bounds__(512) k_enc_starts(const uint8_t *__restrict__ vox, uint32_t N,
						    const uint32_t *__restrict__ tstart, uint32_t max_tiles,
						    const uint32_t *__restrict__ nruns, uint32_t *scratch)
{
	__shared__ uint32_t tmp[64];
	const uint32_t t = blockIdx.x, k = blockIdx.y;
	if (nruns[k] == 0xFFFFFFFFu) return;
	const uint8_t *v = vox + (size_t)k * N;
	uint32_t *S = scratch + (size_t)k * (N + 1u);
	const uint32_t p = t * kEncTile + 16u * threadIdx.x;
	const int lane = threadIdx.x & 31;
	uint4 q = make_uint4(0, 0, 0, 0);
	if (p < N) q = __ldg((const uint4 *)(v + p));
	uint32_t prev = __shfl_up_sync(kFull, byte_of(q, 15), 1);
	if (lane == 0 && p > 0 && p < N) prev = v[p - 1];
	const uint32_t b = p < N ? (boundaries16(q, prev, p == 0) & tail_mask(p, N)) : 0u;
	uint32_t tot;
	uint32_t r = tstart[k * max_tiles + t] + block_excl_add(__popc(b), tmp, &tot);
	for (uint32_t m = b; m; m &= m - 1u) {
		const int j = __ffs(m) - 1;
		S[r++] = (p + (uint32_t)j) | (byte_of(q, j) << 24);
	}
	if (t == 0 && threadIdx.x == 0) S[nruns[k]] = N; /* end of the last run */
}

/* per (run tile, chunk): words = (next start - start) | colour << 24 */
__global__ void k_enc_words(const uint32_t *__restrict__ scratch, uint32_t N, const uint32_t *__restrict__ nruns,
			    const uint64_t *__restrict__ out_off, uint32_t *pool)
{
	const uint32_t k = blockIdx.y;
	const uint32_t n = nruns[k];
	if (n == 0xFFFFFFFFu) return;
	const uint32_t *S = scratch + (size_t)k * (N + 1u);
	uint32_t *out = pool + out_off[k];
	for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
		const uint32_t a = S[r], b = S[r + 1];
		out[r] = ((b & 0xFFFFFFu) - (a & 0xFFFFFFu)) | (a & 0xFF000000u);
	}
}

cudaError_t launch_rle_decode_tiles(const uint32_t *pool, const uint64_t *off, const uint32_t *len, const uint32_t *chunks,
				    uint32_t n, uint32_t N, uint8_t *vox, uint32_t *tile_scratch, cudaStream_t st)
{
	if (!n) return cudaSuccess;
	const uint32_t T = (N + kDecTile - 1) / kDecTile + 1;
	k_dec_sums<<<dim3(T, n), 512, 0, st>>>(pool, off, len, chunks, tile_scratch, T);
	k_tile_scan<<<(n + 7) / 8, 256, 0, st>>>(tile_scratch, T, n);
	k_dec_fill<<<dim3(T, n), 512, 0, st>>>(pool, off, len, chunks, tile_scratch, T, N, vox);
	return cudaGetLastError();
}

cudaError_t launch_rle_encode_tiles(const uint8_t *vox, uint32_t n, uint32_t N, uint32_t *pool, uint64_t cap_words,
				    unsigned long long *cursor, uint64_t *out_off, uint32_t *out_len, uint32_t *status,
				    uint32_t *tile_scratch, uint32_t *nruns, uint32_t *run_scratch, cudaStream_t st)
{
	if (!n) return cudaSuccess;
	const uint32_t T = (N + kEncTile - 1) / kEncTile;
	k_enc_count<<<dim3(T, n), 512, 0, st>>>(vox, N, tile_scratch, T);
	k_enc_alloc<<<(n + 7) / 8, 256, 0, st>>>(tile_scratch, T, n, N, pool, cap_words, cursor, out_off, out_len, nruns,
						 status);
	k_enc_starts<<<dim3(T, n), 512, 0, st>>>(vox, N, tile_scratch, T, nruns, run_scratch);
	k_enc_words<<<dim3(64, n), 256, 0, st>>>(run_scratch, N, nruns, out_off, pool);
	return cudaGetLastError();
}

/* One warp per stream: at least two words, a zero terminator, no zero
 * count before it, counts summing to N (the checks a stream must pass before
 * the decoders see it). Failing streams OR kStatusBadStream into *status and
 * record the lowest failing chunk in *first_bad. */
__global__ void __launch_bounds__(256) k_validate_streams(const uint32_t *__restrict__ pool,
							  const uint64_t *__restrict__ off,
							  const uint32_t *__restrict__ len, uint32_t nchunks, uint64_t N,
							  uint32_t *status, uint32_t *first_bad)
{
	const uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	const int lane = threadIdx.x & 31;
	if (c >= nchunks) return;
	const uint32_t n = len[c];
	const uint32_t *s = pool + off[c];
	bool bad = n < 2;
	uint64_t sum = 0;
	if (!bad) {
		bool zero = false;
		for (uint32_t i = lane; i + 1 < n; i += 32) {
			const uint32_t cnt = __ldg(s + i) & 0xFFFFFFu;
			zero |= cnt == 0;
			sum += cnt;
		}
#pragma unroll
		for (int d = 16; d; d >>= 1) sum += __shfl_xor_sync(kFull, sum, d);
		zero = __any_sync(kFull, zero);
		bad = zero || sum != N || __ldg(s + n - 1) != 0;
	}
	if (bad && lane == 0) {
		atomicOr(status, kStatusBadStream);
		atomicMin(first_bad, c);
	}
}

cudaError_t launch_validate_streams(const uint32_t *pool, const uint64_t *off, const uint32_t *len, uint32_t nchunks,
				    uint64_t N, uint32_t *status, uint32_t *first_bad, cudaStream_t st)
{
	if (!nchunks) return cudaSuccess;
	k_validate_streams<<<(nchunks + 7) / 8, 256, 0, st>>>(pool, off, len, nchunks, N, status, first_bad);
	return cudaGetLastError();
}

} // namespace vp
