/*
 * vp_dev.cuh — device-side data layout and helpers shared by the pipeline
 * kernels.
 *
 * Resident world layout in HBM (one "set" = one reference ChunkSet):
 *   pool[]        every chunk's RLE stream (reference format, src/chunkset/
 *                 rle.c:14-22), each starting on a 16-byte boundary;
 *   off[c], len[c] word offset / length (incl. terminator) of chunk c;
 *   shadow[]      the u16 sun-shadow height map (src/chunkset/shadow.h:26-43),
 *                 zero padded after its last row;
 *   shell_bits[c] the six boundary planes of chunk c as occupancy bits, and
 *   shell_col[c]  the colours of its three low planes (x=0, y=0, z=0);
 *                 both are written by the shell pass of every rebuild, so a
 *                 chunk's pass reads its neighbours' halo without decoding
 *                 their streams.
 */
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace vp {

constexpr int kMaxLevels = 8;   /* LOD levels 0..7 */
constexpr unsigned kFull = 0xFFFFFFFFu;

/* Programmatic dependent launch (sm_90 and later): a kernel launched with
 * launch_dependent() may start while the kernel before it on the stream is
 * finishing; it calls grid_wait() before touching anything that kernel
 * writes (the wait returns at once for an ordinary launch). A kernel calls
 * grid_release() to let the next one start launching early. */
__device__ __forceinline__ void grid_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void grid_release() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

template <typename... P, typename... A>
static inline cudaError_t launch_dependent(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
					   A &&...args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = st;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, k, static_cast<P>(args)...);
}

struct SetDesc {
	const uint32_t *pool;
	const uint64_t *off;
	const uint32_t *len;
	const uint16_t *shadow;
	uint64_t shadow_len;   /* padded length, elements */
	uint64_t *shell_bits;  /* per chunk: 6 planes x R rows (u64, R <= 64) */
	uint8_t *shell_col;    /* per chunk: 3 planes x R*R bytes */
	uint32_t shadow_w;     /* world X + Y */
	uint32_t nchunks;
	uint32_t root_bitw;
	uint32_t max_bitw[3];
	int32_t origin[3];     /* chunk coordinates of this set's chunk 0 in the world */
	uint64_t shadow_base;  /* world index of shadow[0] (a window of the map) */
};

/* flags of a work item */
enum : uint32_t { kItemMesh = 1u, kItemMaskDense = 2u, kItemEmpty = 4u /* shell list: no geometry, zero the record */ };

struct WorkItem {
	uint32_t set;
	uint32_t chunk;
	uint32_t flags;
	uint32_t slot;   /* index of the ChunkOut record this item fills */
};

/* Per work item result record. Offsets are in elements of the arena type. */
struct ChunkOut {
	uint64_t svl_off;    /* int16 elements in the splat arena */
	uint64_t vbo_off;    /* int16 elements in the vertex arena */
	uint64_t ibo_off;    /* u32 elements in the index arena */
	uint32_t svl_items[kMaxLevels]; /* int16 items per LOD level */
	uint32_t svl_total;
	uint32_t vbo_items;
	uint32_t ibo_items;
	uint32_t status;     /* 0 ok, else a kStatus* bit set */
};

enum : uint32_t { kStatusOverflow = 1u, kStatusBadStream = 2u, kStatusTimeout = 4u };

/* no slot (handoff table of decoded chunks) */
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;

/* A bump-allocated output arena, allocation unit 16 bytes. */
struct Arena {
	void *base;
	uint64_t cap_units;
	unsigned long long *cursor;
};

/* Plane numbering inside a chunk's shell. */
enum : int { kPX0 = 0, kPX1 = 1, kPY0 = 2, kPY1 = 3, kPZ0 = 4, kPZ1 = 5 };

__device__ __forceinline__ uint64_t low_mask(int n)
{
	return n >= 64 ? ~0ull : ((1ull << n) - 1ull);
}

/* Inclusive prefix XOR of the bits of x (bit i = XOR of bits 0..i). */
__device__ __forceinline__ uint64_t prefix_xor64(uint64_t x)
{
	x ^= x << 1;
	x ^= x << 2;
	x ^= x << 4;
	x ^= x << 8;
	x ^= x << 16;
	x ^= x << 32;
	return x;
}

/* OR each bit pair (2k, 2k+1) of v into bit k of the result. */
__device__ __forceinline__ uint64_t compress_pairs(uint64_t v)
{
	uint64_t t = (v | (v >> 1)) & 0x5555555555555555ull;
	t = (t | (t >> 1)) & 0x3333333333333333ull;
	t = (t | (t >> 2)) & 0x0F0F0F0F0F0F0F0Full;
	t = (t | (t >> 4)) & 0x00FF00FF00FF00FFull;
	t = (t | (t >> 8)) & 0x0000FFFF0000FFFFull;
	t = (t | (t >> 16)) & 0x00000000FFFFFFFFull;
	return t;
}

__device__ __forceinline__ uint32_t warp_incl_add(uint32_t v)
{
	const int lane = threadIdx.x & 31;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		uint32_t n = __shfl_up_sync(kFull, v, d);
		if (lane >= d) v += n;
	}
	return v;
}

__device__ __forceinline__ uint32_t warp_incl_xor(uint32_t v)
{
	const int lane = threadIdx.x & 31;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		uint32_t n = __shfl_up_sync(kFull, v, d);
		if (lane >= d) v ^= n;
	}
	return v;
}

/* Block-wide exclusive sum of one value per thread. `tmp` holds 33 words.
 * Returns the exclusive prefix; *total gets the block sum. All threads of
 * the block must call it. */
__device__ __forceinline__ uint32_t block_excl_add(uint32_t v, uint32_t *tmp, uint32_t *total)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nw = (blockDim.x + 31) >> 5;
	uint32_t inc = warp_incl_add(v);
	if (lane == 31) tmp[warp] = inc;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = lane < nw ? tmp[lane] : 0;
		uint32_t wi = warp_incl_add(w);
		tmp[lane] = wi - w;
		if (lane == 31) tmp[32] = wi;
	}
	__syncthreads();
	uint32_t r = tmp[warp] + inc - v;
	*total = tmp[32];
	__syncthreads();
	return r;
}

/* Exclusive prefix sum, in place, of n u32 values in shared memory. Each
 * warp scans a contiguous segment. `tmp` holds 33 words. */
__device__ __forceinline__ uint32_t block_scan_array(uint32_t *a, int n, uint32_t *tmp)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nw = blockDim.x >> 5;
	const int seg = (n + nw - 1) / nw;
	const int lo = warp * seg;
	const int hi = min(n, lo + seg);
	uint32_t sum = 0;
	for (int i = lo + lane; i < hi; i += 32) sum += a[i];
#pragma unroll
	for (int d = 16; d; d >>= 1) sum += __shfl_xor_sync(kFull, sum, d);
	if (lane == 0) tmp[warp] = sum;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = lane < nw ? tmp[lane] : 0;
		uint32_t wi = warp_incl_add(w);
		tmp[lane] = wi - w;
		if (lane == 31) tmp[32] = wi;
	}
	__syncthreads();
	uint32_t carry = tmp[warp];
	for (int base = lo; base < hi; base += 32) {
		int i = base + lane;
		uint32_t v = i < hi ? a[i] : 0;
		uint32_t inc = warp_incl_add(v);
		if (i < hi) a[i] = carry + inc - v;
		carry += __shfl_sync(kFull, inc, 31);
	}
	uint32_t total = tmp[32];
	__syncthreads();
	return total;
}

/* Shadow map read with the padded-zero convention: reads at or past the
 * padded length return 0. */
__device__ __forceinline__ uint32_t shadow_at(const SetDesc &s, uint32_t idx)
{
	const uint64_t i = (uint64_t)idx - s.shadow_base; /* wraps when idx < base */
	return i < s.shadow_len ? (uint32_t)__ldg(s.shadow + i) : 0u;
}

/* shadow_sample (src/chunkset/shadow.h:45-63), uint32 index arithmetic. */
__device__ __forceinline__ int shadow_sample(const SetDesc &s, uint32_t x, uint32_t y, uint32_t z)
{
	uint32_t lim = y + 1u;
	if (lim == 0u) return 1; /* nothing is < 0: shadowed whatever is read */
	uint32_t idx = (x + y) + s.shadow_w * z;
	const uint32_t a = shadow_at(s, idx), b = shadow_at(s, idx + 1u); /* both loads in flight */
	return !((a < lim) & (b < lim));
}

/* shadow_sample_normal (src/chunkset/shadow.h:65-75) */
__device__ __forceinline__ int shadow_sample_normal(const SetDesc &s, uint32_t x, uint32_t y, uint32_t z)
{
	uint32_t lim = y + 1u;
	if (lim == 0u) return 1;
	uint32_t idx = (x + y) + s.shadow_w * z;
	const uint32_t a = shadow_at(s, idx), b = shadow_at(s, idx - 1u);
	return !((a < lim) & (b < lim));
}

} // namespace vp
