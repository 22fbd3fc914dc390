/*
 * vp_geometry.cu — the per-chunk geometry pipeline on sm_103a.
 *
 * One CTA owns one chunk at a time (grid = chunks, or persistent CTAs fed by
 * a device work queue). For chunk size R = 2^RB <= 64 the whole chunk lives
 * in shared memory as occupancy bits, one 64-bit word per x-row:
 *
 *   decode     RLE stream -> run starts (block scan of run lengths) ->
 *              run-start bitmap + solid/air toggle bitmap (warp-aggregated
 *              shared atomics) -> occupancy rows (prefix XOR over the bit
 *              stream) + per-row rank table, so the colour of any voxel is
 *              stream[rank(row) + popc(runstarts & bits<=x) - 1] >> 24.
 *   shell pass writes each chunk's six boundary planes (bits) and its three
 *              low planes' colours, so neighbours get their halo cheaply.
 *   geometry   halo rows from the neighbours' shells; then either
 *              - splats: exposure bits E0 = solid & ~(all six neighbours
 *                solid), with the reference's per-axis rules (src/chunkset/
 *                mesher.c:377-456), LOD rows by pairwise OR + bit compaction,
 *                and per-level emission in z,y,x order; the LOD colour is
 *                the last nonzero child in scan order (mesher.c:460-493),
 *                found by walking down the stored level bits;
 *              - mesh: face bits Fx/Fy/Fz = row XOR shifted row, in-order
 *                emission of 4 vertices + 6 indices per face with the
 *                reference's AO, shadow and diamond rules (mesher.c:184-357).
 *   Output space comes from bump-allocated arenas; counts are known before
 *   emission, so every chunk's output is contiguous and in reference order.
 */
#include "vp_dev.cuh"
#include "vp_geometry.h"

namespace vp {

template <int RB>
struct Geo {
	static constexpr int R = 1 << RB;
	static constexpr int H = R + 2;      /* halo row pitch */
	static constexpr int RR = R * R;
	static constexpr int S = R + 1;      /* mask extent per axis */
	static constexpr uint64_t MASK = (R == 64) ? ~0ull : ((1ull << R) - 1ull);
	static constexpr int n_at(int l) { return (R >> l) + 1; }
	static constexpr int lv_words()
	{
		int t = 0;
		for (int l = 1; l < kMaxLevels; l++) t += n_at(l) * n_at(l);
		return t;
	}
	static constexpr size_t a16(size_t v) { return (v + 15) & ~(size_t)15; }
	/* shared memory carve, byte offsets (every region 16-byte aligned) */
	static constexpr size_t o_occ = 0;
	static constexpr size_t o_rs = a16(o_occ + sizeof(uint64_t) * H * H);
	static constexpr size_t o_e0 = a16(o_rs + sizeof(uint64_t) * RR);
	static constexpr size_t o_e0p = a16(o_e0 + sizeof(uint64_t) * RR);
	static constexpr size_t o_lv = a16(o_e0p + sizeof(uint64_t) * 3 * R);
	static constexpr size_t o_rank = a16(o_lv + sizeof(uint64_t) * lv_words());
	static constexpr size_t o_rowoff = a16(o_rank + sizeof(uint32_t) * RR);
	static constexpr size_t o_xlo = a16(o_rowoff + sizeof(uint32_t) * S * S);
	static constexpr size_t o_xhi = a16(o_xlo + H * H);
	static constexpr size_t o_col = a16(o_xhi + H * H);
	static constexpr size_t o_tmp = a16(o_col + 3 * RR);
	static constexpr size_t bytes = a16(o_tmp + sizeof(uint32_t) * 64);
	static constexpr size_t shell_words = 6 * R;   /* u64 per chunk */
	static constexpr size_t shell_cols = 3 * RR;   /* bytes per chunk */
};

struct Smem {
	uint64_t *occ, *rs, *e0, *e0p, *lv;
	uint32_t *rank, *rowoff, *tmp;
	uint8_t *xlo, *xhi, *col;
};

template <int RB>
__device__ __forceinline__ Smem carve(uint8_t *base)
{
	using G = Geo<RB>;
	Smem s;
	s.occ = (uint64_t *)(base + G::o_occ);
	s.rs = (uint64_t *)(base + G::o_rs);
	s.e0 = (uint64_t *)(base + G::o_e0);
	s.e0p = (uint64_t *)(base + G::o_e0p);
	s.lv = (uint64_t *)(base + G::o_lv);
	s.rank = (uint32_t *)(base + G::o_rank);
	s.rowoff = (uint32_t *)(base + G::o_rowoff);
	s.xlo = base + G::o_xlo;
	s.xhi = base + G::o_xhi;
	s.col = base + G::o_col;
	s.tmp = (uint32_t *)(base + G::o_tmp);
	return s;
}

template <int RB>
__device__ __forceinline__ int hidx(int y, int z)
{
	return (z + 1) * Geo<RB>::H + (y + 1);
}

__device__ __forceinline__ void chunk_coords(const SetDesc &s, uint32_t c, uint32_t cv[3])
{
	cv[0] = c & ((1u << s.max_bitw[0]) - 1u);
	cv[1] = (c >> s.max_bitw[0]) & ((1u << s.max_bitw[1]) - 1u);
	cv[2] = c >> (s.max_bitw[0] + s.max_bitw[1]);
}

__device__ __forceinline__ bool chunk_is_null(const SetDesc &s, uint32_t c, uint32_t N)
{
	return s.len[c] == 2u && s.pool[s.off[c]] == N;
}

/* Index of the chunk at cv + d, or -1 outside the world. */
__device__ __forceinline__ int64_t neighbour(const SetDesc &s, const uint32_t cv[3], int dx, int dy, int dz)
{
	int64_t x = (int64_t)cv[0] + dx, y = (int64_t)cv[1] + dy, z = (int64_t)cv[2] + dz;
	if (x < 0 || y < 0 || z < 0) return -1;
	if (x >= (1 << s.max_bitw[0]) || y >= (1 << s.max_bitw[1]) || z >= (1 << s.max_bitw[2])) return -1;
	return (int64_t)(((uint32_t)z << s.max_bitw[1] | (uint32_t)y) << s.max_bitw[0] | (uint32_t)x);
}

/*
 * RLE stream -> occupancy rows (halo layout, interior only), run-start rows
 * and per-row run rank. `s` points at the stream (16-byte aligned, padded to
 * a multiple of 4 words), nruns = words before the terminator.
 */
template <int RB>
__device__ void decode_chunk(const uint32_t *__restrict__ s, uint32_t nruns, const Smem &m)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR;
	constexpr int KB = RB < 5 ? RB : 5;        /* key = p >> KB */
	const int lane = threadIdx.x & 31;
	for (int r = threadIdx.x; r < RR; r += blockDim.x) {
		m.occ[hidx<RB>(r & (R - 1), r >> RB)] = 0;
		m.rs[r] = 0;
	}
	__syncthreads();
	uint32_t *rs32 = (uint32_t *)m.rs;
	uint32_t *occ32 = (uint32_t *)m.occ;
	uint32_t tile_start = 0;
	for (uint32_t base = 0; base < nruns; base += 4u * blockDim.x) {
		const uint32_t k0 = base + 4u * threadIdx.x;
		uint32_t w[4] = {0, 0, 0, 0};
		if (k0 < nruns) {
			uint4 q = __ldg((const uint4 *)(s + k0));
			w[0] = q.x; w[1] = q.y; w[2] = q.z; w[3] = q.w;
#pragma unroll
			for (int j = 0; j < 4; j++)
				if (k0 + j >= nruns) w[j] = 0;
		}
		uint32_t c[4], sum = 0;
#pragma unroll
		for (int j = 0; j < 4; j++) {
			c[j] = w[j] & 0xFFFFFFu;
			sum += c[j];
		}
		uint32_t tot;
		uint32_t pos = tile_start + block_excl_add(sum, m.tmp, &tot);
		uint32_t prev = (k0 > 0 && k0 < nruns) ? __ldg(s + k0 - 1) : 0u;
#pragma unroll
		for (int j = 0; j < 4; j++) {
			const bool valid = k0 + j < nruns;
			const uint32_t p = pos;
			pos += c[j];
			const uint32_t pc = j ? w[j - 1] : prev;
			const bool tog = valid && (((w[j] >> 24) != 0) != ((pc >> 24) != 0));
			uint32_t key = valid ? (p >> KB) : 0xFFFFFFFFu;
			uint32_t vr = valid ? (1u << (p & ((1u << KB) - 1u))) : 0u;
			uint32_t vt = tog ? vr : 0u;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				uint32_t k2 = __shfl_up_sync(kFull, key, d);
				uint32_t a = __shfl_up_sync(kFull, vr, d);
				uint32_t b = __shfl_up_sync(kFull, vt, d);
				if (lane >= d && k2 == key) {
					vr |= a;
					vt |= b;
				}
			}
			uint32_t nk = __shfl_down_sync(kFull, key, 1);
			const bool last = (lane == 31) || nk != key;
			if (valid && last) {
				const uint32_t row = p >> RB;
				const uint32_t half = (p & (R - 1)) >> 5;
				atomicOr(rs32 + 2 * row + half, vr);
				if (vt) {
					const int y = row & (R - 1), z = row >> RB;
					atomicOr(occ32 + 2 * hidx<RB>(y, z) + half, vt);
				}
			}
		}
		tile_start += tot;
	}
	__syncthreads();
	/* prefix XOR of the toggle stream and run-start ranks, rows in scan
	 * order; each warp owns a contiguous row segment. */
	const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const int seg = (RR + nw - 1) / nw;
	const int lo = warp * seg, hi = min(RR, lo + seg);
	uint32_t par = 0, cnt = 0;
	for (int r = lo + lane; r < hi; r += 32) {
		par ^= __popcll(m.occ[hidx<RB>(r & (R - 1), r >> RB)]) & 1;
		cnt += __popcll(m.rs[r]);
	}
#pragma unroll
	for (int d = 16; d; d >>= 1) {
		par ^= __shfl_xor_sync(kFull, par, d);
		cnt += __shfl_xor_sync(kFull, cnt, d);
	}
	if (lane == 0) m.tmp[warp] = (cnt << 1) | par;
	__syncthreads();
	if (warp == 0) {
		uint32_t v = lane < nw ? m.tmp[lane] : 0u;
		uint32_t p = v & 1u, n = v >> 1;
		uint32_t pi = warp_incl_xor(p), ni = warp_incl_add(n);
		m.tmp[32 + lane] = ((ni - n) << 1) | (pi ^ p);
	}
	__syncthreads();
	uint32_t cv = m.tmp[32 + warp];
	uint32_t cpar = cv & 1u, ccnt = cv >> 1;
	for (int b = lo; b < hi; b += 32) {
		const int r = b + lane;
		uint64_t t = 0, q = 0;
		int hi_ = 0;
		if (r < hi) {
			hi_ = hidx<RB>(r & (R - 1), r >> RB);
			t = m.occ[hi_];
			q = m.rs[r];
		}
		uint32_t p = __popcll(t) & 1u, n = __popcll(q);
		uint32_t pi = warp_incl_xor(p), ni = warp_incl_add(n);
		if (r < hi) {
			uint64_t o = prefix_xor64(t);
			if (cpar ^ pi ^ p) o = ~o;
			m.occ[hi_] = o & G::MASK;
			m.rank[r] = ccnt + ni - n;
		}
		cpar ^= __shfl_sync(kFull, pi, 31);
		ccnt += __shfl_sync(kFull, ni, 31);
	}
	__syncthreads();
}

/* Colour of a solid voxel of the decoded chunk. */
template <int RB>
__device__ __forceinline__ uint32_t colour_at(const uint32_t *__restrict__ s, const Smem &m, int x, int y, int z)
{
	const int row = (z << RB) | y;
	const uint64_t bits = m.rs[row] & (~0ull >> (63 - x));
	const uint32_t run = m.rank[row] + __popcll(bits) - 1u;
	return __ldg(s + run) >> 24;
}

/* ------------------------------------------------------------------ */
/* Shell pass                                                          */
/* ------------------------------------------------------------------ */

template <int RB>
__global__ void __launch_bounds__(512) k_shell(const SetDesc *__restrict__ sets, const WorkItem *__restrict__ items,
					       uint32_t nitems)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR;
	extern __shared__ __align__(16) uint8_t smem[];
	const Smem m = carve<RB>(smem);
	const uint32_t it = blockIdx.x;
	if (it >= nitems) return;
	const WorkItem wi = items[it];
	const SetDesc S = sets[wi.set];
	const uint32_t N = (uint32_t)R * R * R;
	if (chunk_is_null(S, wi.chunk, N)) return;
	const uint32_t *stream = S.pool + S.off[wi.chunk];
	decode_chunk<RB>(stream, S.len[wi.chunk] - 1u, m);
	uint64_t *bits = S.shell_bits + (size_t)wi.chunk * G::shell_words;
	uint8_t *cols = S.shell_col + (size_t)wi.chunk * G::shell_cols;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	/* x planes: bit y of row z, via ballots over y */
	for (int z = warp; z < R; z += nw) {
		uint64_t b0 = 0, b1 = 0;
		for (int h = 0; h < (R + 31) / 32; h++) {
			const int y = 32 * h + lane;
			uint64_t o = y < R ? m.occ[hidx<RB>(y, z)] : 0ull;
			uint32_t lo = __ballot_sync(kFull, (o & 1ull) != 0);
			uint32_t hi = __ballot_sync(kFull, ((o >> (R - 1)) & 1ull) != 0);
			b0 |= (uint64_t)lo << (32 * h);
			b1 |= (uint64_t)hi << (32 * h);
		}
		if (lane == 0) {
			bits[kPX0 * R + z] = b0 & G::MASK;
			bits[kPX1 * R + z] = b1 & G::MASK;
		}
	}
	for (int v = threadIdx.x; v < R; v += blockDim.x) {
		bits[kPY0 * R + v] = m.occ[hidx<RB>(0, v)];
		bits[kPY1 * R + v] = m.occ[hidx<RB>(R - 1, v)];
		bits[kPZ0 * R + v] = m.occ[hidx<RB>(v, 0)];
		bits[kPZ1 * R + v] = m.occ[hidx<RB>(v, R - 1)];
	}
	/* low planes' colours: X0[z][y] = (0,y,z), Y0[z][x] = (x,0,z),
	 * Z0[y][x] = (x,y,0) */
	for (int i = threadIdx.x; i < RR; i += blockDim.x) {
		const int a = i & (R - 1), b = i >> RB;
		uint32_t c0 = 0, c1 = 0, c2 = 0;
		if ((m.occ[hidx<RB>(a, b)] & 1ull)) c0 = colour_at<RB>(stream, m, 0, a, b);
		if ((m.occ[hidx<RB>(0, b)] >> a) & 1ull) c1 = colour_at<RB>(stream, m, a, 0, b);
		if ((m.occ[hidx<RB>(b, 0)] >> a) & 1ull) c2 = colour_at<RB>(stream, m, a, b, 0);
		cols[i] = (uint8_t)c0;
		cols[RR + i] = (uint8_t)c1;
		cols[2 * RR + i] = (uint8_t)c2;
	}
}

/* ------------------------------------------------------------------ */
/* Geometry pass                                                       */
/* ------------------------------------------------------------------ */

/* Occupancy row (bits over x) of the neighbour-local row (ly, lz) of chunk
 * nc, taken from its shell. */
template <int RB>
__device__ __forceinline__ uint64_t shell_row(const SetDesc &S, int64_t nc, int ly, int lz, uint32_t N)
{
	constexpr int R = Geo<RB>::R;
	if (nc < 0 || chunk_is_null(S, (uint32_t)nc, N)) return 0ull;
	const uint64_t *b = S.shell_bits + (size_t)nc * Geo<RB>::shell_words;
	if (ly == 0) return b[kPY0 * R + lz];
	if (ly == R - 1) return b[kPY1 * R + lz];
	if (lz == 0) return b[kPZ0 * R + ly];
	return b[kPZ1 * R + ly];
}

/* One occupancy bit (x = 0 or R-1 side plane) of chunk nc. */
template <int RB>
__device__ __forceinline__ uint32_t shell_xbit(const SetDesc &S, int64_t nc, int lx, int ly, int lz, uint32_t N)
{
	constexpr int R = Geo<RB>::R;
	if (nc < 0 || chunk_is_null(S, (uint32_t)nc, N)) return 0u;
	const uint64_t *b = S.shell_bits + (size_t)nc * Geo<RB>::shell_words;
	const uint64_t w = (lx == 0) ? b[kPX0 * R + lz] : b[kPX1 * R + lz];
	return (uint32_t)((w >> ly) & 1ull);
}

template <int RB>
__device__ void load_halo(const SetDesc &S, const uint32_t cv[3], const Smem &m, bool need_minus)
{
	using G = Geo<RB>;
	constexpr int R = G::R, H = G::H, RR = G::RR;
	const uint32_t N = (uint32_t)R * R * R;
	/* halo rows: y in {-1, R} for z in [-1, R], and z in {-1, R} for y in
	 * [0, R). Minus-side rows are only needed by the mesh path. */
	const int nrow = 2 * H + 2 * R;
	for (int i = threadIdx.x; i < nrow; i += blockDim.x) {
		int y, z;
		if (i < 2 * H) {
			y = (i < H) ? -1 : R;
			z = (i % H) - 1;
		} else {
			const int j = i - 2 * H;
			y = j % R;
			z = (j < R) ? -1 : R;
		}
		const int dy = y < 0 ? -1 : (y >= R ? 1 : 0);
		const int dz = z < 0 ? -1 : (z >= R ? 1 : 0);
		uint64_t v = 0;
		if (need_minus || (dy >= 0 && dz >= 0)) {
			const int64_t nc = neighbour(S, cv, 0, dy, dz);
			v = shell_row<RB>(S, nc, y - dy * R, z - dz * R, N);
		}
		m.occ[hidx<RB>(y, z)] = v;
	}
	/* x = -1 and x = R columns for (y, z) in [-1, R]^2 */
	for (int i = threadIdx.x; i < 2 * H * H; i += blockDim.x) {
		const int side = i / (H * H), k = i % (H * H);
		const int y = (k % H) - 1, z = (k / H) - 1;
		const int dx = side ? 1 : -1;
		const int dy = y < 0 ? -1 : (y >= R ? 1 : 0);
		const int dz = z < 0 ? -1 : (z >= R ? 1 : 0);
		uint32_t v = 0;
		if (need_minus || (dx > 0 && dy >= 0 && dz >= 0)) {
			const int64_t nc = neighbour(S, cv, dx, dy, dz);
			v = shell_xbit<RB>(S, nc, side ? 0 : R - 1, y - dy * R, z - dz * R, N);
		}
		(side ? m.xhi : m.xlo)[k] = (uint8_t)v;
	}
	/* colours of the +x / +y / +z neighbour cells (their low planes) */
	const int64_t nb[3] = {neighbour(S, cv, 1, 0, 0), neighbour(S, cv, 0, 1, 0), neighbour(S, cv, 0, 0, 1)};
	for (int a = 0; a < 3; a++) {
		uint4 *dst = (uint4 *)(m.col + a * RR);
		const bool live = nb[a] >= 0 && !chunk_is_null(S, (uint32_t)nb[a], N);
		const uint4 *src = live ? (const uint4 *)(S.shell_col + (size_t)nb[a] * G::shell_cols + (size_t)a * RR) : nullptr;
		for (int i = threadIdx.x; i < RR / 16; i += blockDim.x)
			dst[i] = live ? __ldg(src + i) : make_uint4(0, 0, 0, 0);
	}
	__syncthreads();
}

template <int RB>
__device__ __forceinline__ uint32_t occ_at(const Smem &m, int x, int y, int z)
{
	constexpr int R = Geo<RB>::R;
	const int k = hidx<RB>(y, z);
	if (x < 0) return m.xlo[k];
	if (x >= R) return m.xhi[k];
	return (uint32_t)((m.occ[k] >> x) & 1ull);
}

/* L0 mask row (y, z) in [0, R]^2: bits x in [0, R) plus the x = R cell. */
template <int RB>
__device__ __forceinline__ uint64_t e0_row(const Smem &m, int y, int z, uint32_t &xr)
{
	constexpr int R = Geo<RB>::R;
	xr = 0;
	if (y < R && z < R) {
		xr = (uint32_t)((m.e0p[z] >> y) & 1ull);
		return m.e0[(z << RB) | y];
	}
	if (y == R && z < R) return m.e0p[R + z];
	if (z == R && y < R) return m.e0p[2 * R + y];
	return 0ull;
}

template <int RB>
__device__ __forceinline__ uint32_t level_bit(const Smem &m, const int *lvoff, int l, int x, int y, int z)
{
	constexpr int R = Geo<RB>::R;
	if (l == 0) {
		uint32_t xr;
		uint64_t row = e0_row<RB>(m, y, z, xr);
		return x == R ? xr : (uint32_t)((row >> x) & 1ull);
	}
	const int n = (R >> l) + 1;
	return (uint32_t)((m.lv[lvoff[l] + z * n + y] >> x) & 1ull);
}

/* Colour of the L0 mask cell (x, y, z) in [0, R]^3. */
template <int RB>
__device__ __forceinline__ uint32_t mask_colour(const uint32_t *__restrict__ s, const Smem &m, int x, int y, int z)
{
	constexpr int R = Geo<RB>::R, RR = Geo<RB>::RR;
	if (x == R) return m.col[(z << RB) | y];
	if (y == R) return m.col[RR + ((z << RB) | x)];
	if (z == R) return m.col[2 * RR + ((y << RB) | x)];
	return colour_at<RB>(s, m, x, y, z);
}

static __device__ __forceinline__ void store_splat(int16_t *dst, uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
	uint2 v;
	v.x = (x & 0xFFFFu) | ((y & 0xFFFFu) << 16);
	v.y = (z & 0xFFFFu) | ((w & 0xFFFFu) << 16);
	*(uint2 *)dst = v;
}

/* Quad vertex offsets per visible face axis (lutv, src/chunkset/mesher.c:19-33)
 * and the index pattern (luti, src/chunkset/mesher.c:53-66). */
__constant__ uint8_t c_quad_offset[3][4][3] = {
	{{1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}},
	{{0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}},
	{{1, 0, 1}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}},
};
__constant__ uint8_t c_quad_index[24] = {0, 3, 1, 2, 1, 3, 3, 2, 0, 1, 0, 2,
					 1, 3, 0, 3, 1, 2, 0, 2, 3, 2, 0, 1};

template <int RB>
__device__ void emit_face(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m, const uint32_t cv[3],
			  int x, int y, int z, int i, uint32_t ordinal, int16_t *vbo, uint32_t *ibo)
{
	constexpr int R = Geo<RB>::R;
	const int AC[3] = {x, y, z};
	int NB[3] = {x, y, z};
	NB[i] += 1;
	const uint32_t a_solid = occ_at<RB>(m, x, y, z);
	uint32_t colour;
	if (a_solid) {
		colour = colour_at<RB>(stream, m, x, y, z);
	} else {
		colour = mask_colour<RB>(stream, m, NB[0], NB[1], NB[2]);
	}
	const int normal = a_solid ? 0 : 1;
	const int *AIR = a_solid ? NB : AC;
	const int *BLK = a_solid ? AC : NB;
	const int u = (i == 0) ? 1 : 0;
	const int v = (i == 2) ? 1 : 2;
	int O[3];
#define OCC3(dU, dV) (O[0] = AIR[0], O[1] = AIR[1], O[2] = AIR[2], O[u] += (dU), O[v] += (dV), \
		      occ_at<RB>(m, O[0], O[1], O[2]))
	const uint32_t an0 = OCC3(-1, 0), an2 = OCC3(1, 0), an1 = OCC3(0, -1), an3 = OCC3(0, 1);
	const uint32_t ac0 = OCC3(-1, -1), ac1 = OCC3(1, -1), ac2 = OCC3(1, 1), ac3 = OCC3(-1, 1);
#undef OCC3
	const uint32_t e0 = (an0 + an1) | ac0, e1 = (an1 + an2) | ac1;
	const uint32_t e2 = (an2 + an3) | ac2, e3 = (an3 + an0) | ac3;
	uint32_t va[4];
	if (i == 0) {
		va[0] = e0; va[3] = e1; va[2] = e2; va[1] = e3;
	} else if (i == 1) {
		va[0] = e0; va[1] = e1; va[2] = e2; va[3] = e3;
	} else {
		va[1] = e0; va[0] = e1; va[3] = e2; va[2] = e3;
	}
	const int rotate = (va[0] + va[2] < va[1] + va[3]) ? 6 : 0;
	uint32_t ws[3];
	for (int k = 0; k < 3; k++) ws[k] = (cv[k] << RB) + (uint32_t)BLK[k];
	uint32_t shadow = 0;
	if (i == 0 && normal)
		shadow = shadow_sample_normal(S, ws[0], ws[1], ws[2]);
	else if (i == 1 && !normal)
		shadow = shadow_sample(S, ws[0], ws[1], ws[2]);
	ws[i] -= (uint32_t)normal;
	uint32_t diamond = 3;
	if (i == 2) {
		shadow = 0;
		const uint32_t b_solid = a_solid ? 0u : 1u;
		const uint32_t sz = ws[2] + (b_solid ? 0u : 1u);
		diamond = (uint32_t)(!shadow_sample(S, ws[0], ws[1], sz)) << 1;
		diamond |= (uint32_t)(!shadow_sample(S, ws[0], ws[1] - 1u, sz));
	}
	uint32_t out[8];
	for (int vert = 0; vert < 4; vert++) {
		const uint32_t px = (ws[0] + c_quad_offset[i][vert][0]) & 0xFFFFu;
		const uint32_t py = (ws[1] + c_quad_offset[i][vert][1]) & 0xFFFFu;
		const uint32_t pz = (ws[2] + c_quad_offset[i][vert][2]) & 0xFFFFu;
		const uint32_t word = (colour | (va[vert] << 6) | ((uint32_t)(i + 3 * normal) << 8) |
				       ((uint32_t)vert << 11) | (shadow << 13) | (diamond << 14)) & 0xFFFFu;
		out[2 * vert] = px | (py << 16);
		out[2 * vert + 1] = pz | (word << 16);
	}
	uint4 *vd = (uint4 *)(vbo + (size_t)ordinal * 16);
	vd[0] = make_uint4(out[0], out[1], out[2], out[3]);
	vd[1] = make_uint4(out[4], out[5], out[6], out[7]);
	const uint32_t vb = ordinal * 4u;
	const uint8_t *qi = c_quad_index + normal * 12 + rotate;
	uint2 *id = (uint2 *)(ibo + (size_t)ordinal * 6);
	id[0] = make_uint2(vb + qi[0], vb + qi[1]);
	id[1] = make_uint2(vb + qi[2], vb + qi[3]);
	id[2] = make_uint2(vb + qi[4], vb + qi[5]);
}

template <int RB>
__device__ void mesh_chunk(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m, const uint32_t cv[3],
			   ChunkOut *out, const Arena &avbo, const Arena &aibo)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR;
	__shared__ unsigned long long s_base[2];
	__shared__ uint32_t s_ok;
	for (int r = threadIdx.x; r < RR; r += blockDim.x) {
		const int y = r & (R - 1), z = r >> RB;
		const uint64_t o = m.occ[hidx<RB>(y, z)];
		const uint64_t fx = (o ^ ((o >> 1) | ((uint64_t)m.xhi[hidx<RB>(y, z)] << (R - 1)))) & G::MASK;
		const uint64_t fy = o ^ m.occ[hidx<RB>(y + 1, z)];
		const uint64_t fz = o ^ m.occ[hidx<RB>(y, z + 1)];
		m.rowoff[r] = __popcll(fx) + __popcll(fy) + __popcll(fz);
	}
	__syncthreads();
	const uint32_t faces = block_scan_array(m.rowoff, RR, m.tmp);
	if (threadIdx.x == 0) {
		const uint64_t uv = (uint64_t)faces * 2u;             /* 32 B per face */
		const uint64_t ui = ((uint64_t)faces * 24u + 15u) / 16u;
		unsigned long long bv = atomicAdd(avbo.cursor, (unsigned long long)uv);
		unsigned long long bi = atomicAdd(aibo.cursor, (unsigned long long)ui);
		uint32_t ok = (bv + uv <= avbo.cap_units) && (bi + ui <= aibo.cap_units);
		s_base[0] = bv;
		s_base[1] = bi;
		s_ok = ok;
		out->vbo_off = bv * 8u;
		out->ibo_off = bi * 4u;
		out->vbo_items = faces * 16u;
		out->ibo_items = faces * 6u;
		out->svl_total = 0;
		for (int l = 0; l < kMaxLevels; l++) out->svl_items[l] = 0;
		out->svl_off = 0;
		out->status = ok ? 0u : kStatusOverflow;
	}
	__syncthreads();
	if (!s_ok || faces == 0) return;
	int16_t *vbo = (int16_t *)avbo.base + s_base[0] * 8u;
	uint32_t *ibo = (uint32_t *)aibo.base + s_base[1] * 4u;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int r = warp; r < RR; r += nw) {
		const int y = r & (R - 1), z = r >> RB;
		const uint64_t o = m.occ[hidx<RB>(y, z)];
		const uint64_t fx = (o ^ ((o >> 1) | ((uint64_t)m.xhi[hidx<RB>(y, z)] << (R - 1)))) & G::MASK;
		const uint64_t fy = o ^ m.occ[hidx<RB>(y + 1, z)];
		const uint64_t fz = o ^ m.occ[hidx<RB>(y, z + 1)];
		uint32_t base = m.rowoff[r];
		for (int h = 0; h < (R + 31) / 32; h++) {
			const int x = 32 * h + lane;
			uint32_t b0 = 0, b1 = 0, b2 = 0;
			if (x < R) {
				b0 = (uint32_t)((fx >> x) & 1ull);
				b1 = (uint32_t)((fy >> x) & 1ull);
				b2 = (uint32_t)((fz >> x) & 1ull);
			}
			const uint32_t n = b0 + b1 + b2;
			const uint32_t inc = warp_incl_add(n);
			uint32_t ord = base + inc - n;
			if (b0) emit_face<RB>(S, stream, m, cv, x, y, z, 0, ord++, vbo, ibo);
			if (b1) emit_face<RB>(S, stream, m, cv, x, y, z, 1, ord++, vbo, ibo);
			if (b2) emit_face<RB>(S, stream, m, cv, x, y, z, 2, ord++, vbo, ibo);
			base += __shfl_sync(kFull, inc, 31);
		}
	}
}

template <int RB>
__device__ void splat_chunk(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m, const uint32_t cv[3],
			    int lod_max, ChunkOut *out, const Arena &asvl)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR, S1 = G::S;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	__shared__ uint32_t s_cnt[kMaxLevels];
	__shared__ unsigned long long s_base;
	__shared__ uint32_t s_ok;
	int lvoff[kMaxLevels];
	{
		int t = 0;
		for (int l = 1; l < kMaxLevels; l++) {
			lvoff[l] = t;
			t += ((R >> l) + 1) * ((R >> l) + 1);
		}
		lvoff[0] = 0;
	}
	if (threadIdx.x < kMaxLevels) s_cnt[threadIdx.x] = 0;
	/* L0 exposure rows (src/chunkset/mesher.c:421-446 restated per bit):
	 * a solid voxel is in the mask when any +axis neighbour (the +chunk at
	 * coordinate R) is air, or a -axis neighbour inside the chunk is air. */
	for (int r = threadIdx.x; r < RR; r += blockDim.x) {
		const int y = r & (R - 1), z = r >> RB;
		const uint64_t o = m.occ[hidx<RB>(y, z)];
		const uint64_t xp = (o >> 1) | ((uint64_t)m.xhi[hidx<RB>(y, z)] << (R - 1));
		const uint64_t xm = ((o << 1) | 1ull) & G::MASK;
		const uint64_t yp = m.occ[hidx<RB>(y + 1, z)];
		const uint64_t ym = y ? m.occ[hidx<RB>(y - 1, z)] : G::MASK;
		const uint64_t zp = m.occ[hidx<RB>(y, z + 1)];
		const uint64_t zm = z ? m.occ[hidx<RB>(y, z - 1)] : G::MASK;
		m.e0[r] = o & ~(xp & xm & yp & ym & zp & zm);
	}
	/* cells at coordinate R: the +neighbour's voxel is solid and ours air */
	for (int z = warp; z < R; z += nw) {
		uint64_t b = 0;
		for (int h = 0; h < (R + 31) / 32; h++) {
			const int y = 32 * h + lane;
			bool bit = false;
			if (y < R) bit = m.xhi[hidx<RB>(y, z)] && !((m.occ[hidx<RB>(y, z)] >> (R - 1)) & 1ull);
			b |= (uint64_t)__ballot_sync(kFull, bit) << (32 * h);
		}
		if (lane == 0) m.e0p[z] = b & G::MASK;
	}
	for (int v = threadIdx.x; v < R; v += blockDim.x) {
		m.e0p[R + v] = m.occ[hidx<RB>(R, v)] & ~m.occ[hidx<RB>(R - 1, v)];
		m.e0p[2 * R + v] = m.occ[hidx<RB>(v, R)] & ~m.occ[hidx<RB>(v, R - 1)];
	}
	__syncthreads();
	/* level rows: pairwise OR of the child rows, compacted along x */
	for (int l = 1; l <= lod_max; l++) {
		const int n = (R >> l) + 1, np = (R >> (l - 1)) + 1;
		uint64_t *dst = m.lv + lvoff[l];
		for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
			const int y = i % n, z = i / n;
			uint64_t acc = 0;
			uint32_t accx = 0;
			for (int dz = 0; dz < 2; dz++)
				for (int dy = 0; dy < 2; dy++) {
					const int yy = 2 * y + dy, zz = 2 * z + dz;
					if (yy >= np || zz >= np) continue;
					if (l == 1) {
						uint32_t xr;
						acc |= e0_row<RB>(m, yy, zz, xr);
						accx |= xr;
					} else {
						acc |= m.lv[lvoff[l - 1] + zz * np + yy];
					}
				}
			uint64_t row = compress_pairs(acc);
			if (l == 1) row |= (uint64_t)accx << (R / 2);
			dst[i] = row;
		}
		__syncthreads();
	}
	/* counts per level */
	{
		uint32_t c0 = 0;
		for (int r = threadIdx.x; r < RR; r += blockDim.x) c0 += __popcll(m.e0[r]);
		for (int r = threadIdx.x; r < 3 * R; r += blockDim.x) c0 += __popcll(m.e0p[r]);
		for (int d = 16; d; d >>= 1) c0 += __shfl_xor_sync(kFull, c0, d);
		if (lane == 0 && c0) atomicAdd(&s_cnt[0], c0);
		for (int l = 1; l <= lod_max; l++) {
			const int n = (R >> l) + 1;
			uint32_t c = 0;
			for (int i = threadIdx.x; i < n * n; i += blockDim.x) c += __popcll(m.lv[lvoff[l] + i]);
			for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
			if (lane == 0 && c) atomicAdd(&s_cnt[l], c);
		}
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t total = 0;
		for (int l = 0; l <= lod_max; l++) total += s_cnt[l];
		const uint64_t units = ((uint64_t)total + 1u) / 2u; /* 8 B per splat */
		unsigned long long b = units ? atomicAdd(asvl.cursor, (unsigned long long)units) : 0ull;
		const uint32_t ok = (b + units <= asvl.cap_units);
		s_base = b;
		s_ok = ok;
		out->svl_off = b * 8u;
		out->svl_total = total * 4u;
		for (int l = 0; l < kMaxLevels; l++) out->svl_items[l] = l <= lod_max ? s_cnt[l] * 4u : 0u;
		out->vbo_off = out->ibo_off = 0;
		out->vbo_items = out->ibo_items = 0;
		out->status = ok ? 0u : kStatusOverflow;
	}
	__syncthreads();
	if (!s_ok) return;
	int16_t *dst = (int16_t *)asvl.base + s_base * 8u;
	uint32_t level_base = 0;
	for (int l = 0; l <= lod_max; l++) {
		const int n = l ? (R >> l) + 1 : S1;
		/* row counts and their scan */
		for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
			const int y = i % n, z = i / n;
			uint32_t c;
			if (l == 0) {
				uint32_t xr;
				c = __popcll(e0_row<RB>(m, y, z, xr)) + xr;
			} else {
				c = __popcll(m.lv[lvoff[l] + i]);
			}
			m.rowoff[i] = c;
		}
		__syncthreads();
		block_scan_array(m.rowoff, n * n, m.tmp);
		const uint32_t sh = l ? (1u << l) : 0u;
		for (int i = warp; i < n * n; i += nw) {
			const int y = i % n, z = i / n;
			uint64_t row;
			uint32_t xr = 0;
			if (l == 0)
				row = e0_row<RB>(m, y, z, xr);
			else
				row = m.lv[lvoff[l] + i];
			if (!row && !xr) continue;
			uint32_t base = level_base + m.rowoff[i];
			const int nbits = l ? n : R; /* x = R of level 0 handled after */
			for (int h = 0; h < (nbits + 31) / 32; h++) {
				const int x = 32 * h + lane;
				const bool bit = x < nbits && ((row >> x) & 1ull);
				const uint32_t bal = __ballot_sync(kFull, bit);
				if (bit) {
					const uint32_t k = base + __popc(bal & ((1u << lane) - 1u));
					int cx = x, cy = y, cz = z;
					for (int k2 = l; k2 >= 1; k2--) {
						const int np = (R >> (k2 - 1)) + 1;
						int best = 0;
						for (int d = 7; d >= 0; d--) {
							const int X = 2 * cx + (d & 1), Y = 2 * cy + ((d >> 1) & 1),
								  Z = 2 * cz + (d >> 2);
							if (X < np && Y < np && Z < np && level_bit<RB>(m, lvoff, k2 - 1, X, Y, Z)) {
								best = d;
								break;
							}
						}
						cx = 2 * cx + (best & 1);
						cy = 2 * cy + ((best >> 1) & 1);
						cz = 2 * cz + (best >> 2);
					}
					const uint32_t colour = mask_colour<RB>(stream, m, cx, cy, cz);
					const uint32_t wx = (cv[0] << RB) + ((uint32_t)x << l);
					const uint32_t wy = (cv[1] << RB) + ((uint32_t)y << l);
					const uint32_t wz = (cv[2] << RB) + ((uint32_t)z << l);
					const uint32_t sh_ = (uint32_t)shadow_sample(S, wx + sh, wy + sh, wz + sh);
					store_splat(dst + (size_t)k * 4, wx, wy, wz, colour | (sh_ << 6));
				}
				base += __popc(bal);
			}
			if (l == 0 && xr && lane == 0) {
				const uint32_t colour = mask_colour<RB>(stream, m, R, y, z);
				const uint32_t wx = (cv[0] << RB) + (uint32_t)R;
				const uint32_t wy = (cv[1] << RB) + (uint32_t)y;
				const uint32_t wz = (cv[2] << RB) + (uint32_t)z;
				const uint32_t sh_ = (uint32_t)shadow_sample(S, wx, wy, wz);
				store_splat(dst + (size_t)base * 4, wx, wy, wz, colour | (sh_ << 6));
			}
		}
		level_base += s_cnt[l];
		__syncthreads();
	}
}

template <int RB>
__global__ void __launch_bounds__(512) k_geometry(const SetDesc *__restrict__ sets, const WorkItem *__restrict__ items,
						  uint32_t nitems, unsigned int *queue, ChunkOut *outs, Arena asvl,
						  Arena avbo, Arena aibo, int lod_max)
{
	using G = Geo<RB>;
	constexpr int R = G::R;
	extern __shared__ __align__(16) uint8_t smem[];
	const Smem m = carve<RB>(smem);
	__shared__ uint32_t s_item;
	(void)sizeof(G);
	uint32_t next = blockIdx.x;
	for (;;) {
		if (threadIdx.x == 0) s_item = queue ? atomicAdd(queue, 1u) : next;
		__syncthreads();
		const uint32_t it = s_item;
		__syncthreads();
		if (it >= nitems) break;
		next = nitems;
		const WorkItem wi = items[it];
		const SetDesc S = sets[wi.set];
		ChunkOut *out = outs + it;
		uint32_t cv[3];
		chunk_coords(S, wi.chunk, cv);
		const uint32_t N = (uint32_t)R * R * R;
		const bool mesh = (wi.flags & kItemMesh) != 0;
		/* an all-air chunk whose +neighbours are all air has no geometry */
		bool empty = chunk_is_null(S, wi.chunk, N);
		for (int a = 0; a < 3 && empty; a++) {
			const int64_t nc = neighbour(S, cv, a == 0, a == 1, a == 2);
			if (nc >= 0 && !chunk_is_null(S, (uint32_t)nc, N)) empty = false;
		}
		if (empty) {
			if (threadIdx.x == 0) {
				out->svl_off = out->vbo_off = out->ibo_off = 0;
				for (int l = 0; l < kMaxLevels; l++) out->svl_items[l] = 0;
				out->svl_total = out->vbo_items = out->ibo_items = 0;
				out->status = 0;
			}
			continue;
		}
		const uint32_t *stream = S.pool + S.off[wi.chunk];
		decode_chunk<RB>(stream, S.len[wi.chunk] - 1u, m);
		load_halo<RB>(S, cv, m, mesh);
		if (mesh)
			mesh_chunk<RB>(S, stream, m, cv, out, avbo, aibo);
		else
			splat_chunk<RB>(S, stream, m, cv, lod_max, out, asvl);
		__syncthreads();
	}
}

/* ------------------------------------------------------------------ */
/* host launchers                                                      */
/* ------------------------------------------------------------------ */

template <int RB>
static cudaError_t launch_rb(const GeoLaunch &L, cudaStream_t st)
{
	using G = Geo<RB>;
	cudaError_t e;
	e = cudaFuncSetAttribute(k_shell<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::bytes);
	if (e != cudaSuccess) return e;
	e = cudaFuncSetAttribute(k_geometry<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::bytes);
	if (e != cudaSuccess) return e;
	if (L.run_shell && L.n_shell) {
		k_shell<RB><<<L.n_shell, L.threads, G::bytes, st>>>(L.sets, L.shell_items, L.n_shell);
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	if (L.n_items) {
		const uint32_t grid = L.queue ? L.ctas : L.n_items;
		k_geometry<RB><<<grid, L.threads, G::bytes, st>>>(L.sets, L.items, L.n_items, L.queue, L.outs, L.svl, L.vbo,
								 L.ibo, L.lod_max);
		e = cudaGetLastError();
	}
	return e;
}

size_t geometry_smem_bytes(int root_bitw)
{
	switch (root_bitw) {
	case 3: return Geo<3>::bytes;
	case 4: return Geo<4>::bytes;
	case 5: return Geo<5>::bytes;
	case 6: return Geo<6>::bytes;
	default: return 0;
	}
}

template <int RB>
static int ctas_per_sm(int threads)
{
	int n = 0;
	cudaFuncSetAttribute(k_geometry<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo<RB>::bytes);
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_geometry<RB>, threads, Geo<RB>::bytes) != cudaSuccess)
		return 1;
	return n;
}

int geometry_ctas_per_sm(int root_bitw, int threads)
{
	switch (root_bitw) {
	case 3: return ctas_per_sm<3>(threads);
	case 4: return ctas_per_sm<4>(threads);
	case 5: return ctas_per_sm<5>(threads);
	case 6: return ctas_per_sm<6>(threads);
	default: return 1;
	}
}

size_t shell_words_per_chunk(int root_bitw) { return 6u * (1u << root_bitw); }
size_t shell_cols_per_chunk(int root_bitw) { return 3u * (1u << root_bitw) * (1u << root_bitw); }

cudaError_t launch_geometry(int root_bitw, const GeoLaunch &L, cudaStream_t st)
{
	switch (root_bitw) {
	case 3: return launch_rb<3>(L, st);
	case 4: return launch_rb<4>(L, st);
	case 5: return launch_rb<5>(L, st);
	case 6: return launch_rb<6>(L, st);
	default: return cudaErrorInvalidValue;
	}
}

} // namespace vp
