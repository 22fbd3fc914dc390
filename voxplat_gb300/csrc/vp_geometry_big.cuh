/*
 * vp_geometry_big.cuh — the geometry pipeline for 128^3 chunks (root 128,
 * src/chunkset.h:9-118 allows roots up to 128).
 *
 * The steps are those of the <= 64^3 path (decode to bit rows, exposure,
 * LOD rows, counted emission), with two differences:
 *   - a row of x is 128 bits, two u64 words (x in [0, 64) and [64, 128));
 *     the L0 mask row has a third part, the x = 128 cell (xr), and so does
 *     the LOD-1 row (65 cells: a word plus the x = 64 cell);
 *   - the chunk's working set (occupancy with halo, run starts, run ranks,
 *     level rows: ~660 KB) does not fit in shared memory, so each CTA owns a
 *     slot of global scratch (L2 resident while the CTA works on it).
 * Included by vp_geometry_dev.cuh after the <= 64^3 path, whose helpers it uses.
 */
#pragma once

namespace vp {

constexpr int big_n_at(int l) { return (128 >> l) + 1; }

/* level rows: level 1 uses two words per row (64 cells + the x = 64 cell),
 * levels >= 2 one word */
constexpr size_t big_lv_off(int l)
{
	size_t t = 0;
	for (int k = 1; k < l; k++) t += (size_t)big_n_at(k) * big_n_at(k) * (k == 1 ? 2 : 1);
	return t;
}

constexpr int big_max_groups()
{
	int t = 0;
	for (int l = 0; l < kMaxLevels; l++) t += (big_n_at(l) * big_n_at(l) + 31) / 32;
	return t;
}

struct Big {
	static constexpr int RB = 7, R = 128, H = R + 2, RR = R * R, W = 2;
	/* scratch slot, offsets in u64 words */
	static constexpr size_t o_occ = 0;                            /* H*H rows x W */
	static constexpr size_t o_rs = o_occ + (size_t)H * H * W;     /* RR rows x W */
	static constexpr size_t o_rank = o_rs + (size_t)RR * W;       /* RR u32 */
	static constexpr size_t o_lv = o_rank + RR / 2;
	static constexpr size_t o_xrow = o_lv + big_lv_off(kMaxLevels);   /* [side][z+1] x W, bits over y */
	static constexpr size_t o_e0p = o_xrow + (size_t)2 * H * W;   /* [3][R] x W */
	static constexpr size_t o_sv = o_e0p + (size_t)3 * R * W;     /* [2][R] x W */
	static constexpr size_t o_grp = o_sv + (size_t)2 * R * W;     /* u32 group bases */
	static constexpr size_t o_xedge = o_grp + (big_max_groups() + 2) / 2 + 1; /* [4][H] bytes */
	static constexpr size_t words = o_xedge + (4 * H + 7) / 8 + 1;
	static constexpr size_t slot_bytes = (words * 8 + 255) & ~(size_t)255;
	static constexpr size_t shell_words = (size_t)6 * R * W;      /* u64 per chunk */
	static constexpr size_t shell_cols = (size_t)3 * RR;          /* bytes per chunk */
};

struct BigMem {
	uint64_t *occ, *rs, *lv, *xrow, *e0p, *sv;
	uint32_t *rank, *grp, *tmp;
	uint8_t *xedge;
	int32_t *nbr;
};

__device__ __forceinline__ BigMem big_carve(uint8_t *scratch, uint32_t slot, uint32_t *tmp, int32_t *nbr)
{
	uint64_t *b = (uint64_t *)(scratch + (size_t)slot * Big::slot_bytes);
	BigMem m;
	m.occ = b + Big::o_occ;
	m.rs = b + Big::o_rs;
	m.rank = (uint32_t *)(b + Big::o_rank);
	m.lv = b + Big::o_lv;
	m.xrow = b + Big::o_xrow;
	m.e0p = b + Big::o_e0p;
	m.sv = b + Big::o_sv;
	m.grp = (uint32_t *)(b + Big::o_grp);
	m.xedge = (uint8_t *)(b + Big::o_xedge);
	m.tmp = tmp;
	m.nbr = nbr;
	return m;
}

/* word index of halo row (y, z), y and z in [-1, R] */
__device__ __forceinline__ int bh(int y, int z) { return ((z + 1) * Big::H + (y + 1)) * Big::W; }

/* RLE stream -> occupancy rows, run-start rows and per-row run ranks, as
 * decode_chunk with 128-bit rows (four u32 words per row for the atomics). */
static __device__ void decode_big(const uint32_t *__restrict__ s, uint32_t nruns, const BigMem &m)
{
	constexpr int R = Big::R, RR = Big::RR;
	for (int r = threadIdx.x; r < RR; r += blockDim.x) {
		uint64_t *o = m.occ + bh(r & (R - 1), r >> 7);
		o[0] = 0;
		o[1] = 0;
		m.rs[2 * r] = 0;
		m.rs[2 * r + 1] = 0;
	}
	__syncthreads();
	uint32_t *rs32 = (uint32_t *)m.rs;
	uint32_t *occ32 = (uint32_t *)m.occ;
	constexpr int K = 8;
	uint32_t tile_start = 0;
	uint64_t covered = 0;
	for (uint32_t base = 0; base < nruns; base += (uint32_t)K * blockDim.x) {
		const uint32_t k0 = base + (uint32_t)K * threadIdx.x;
		uint32_t w[K];
#pragma unroll
		for (int j = 0; j < K; j++) w[j] = 0;
		if (k0 < nruns) {
			const uint4 q0 = __ldg((const uint4 *)(s + k0));
			const uint4 q1 = __ldg((const uint4 *)(s + k0 + 4));
			w[0] = q0.x; w[1] = q0.y; w[2] = q0.z; w[3] = q0.w;
			w[4] = q1.x; w[5] = q1.y; w[6] = q1.z; w[7] = q1.w;
#pragma unroll
			for (int j = 0; j < K; j++)
				if (k0 + j >= nruns) w[j] = 0;
		}
		uint32_t sum = 0;
#pragma unroll
		for (int j = 0; j < K; j++) sum += w[j] & 0xFFFFFFu;
		uint32_t tot;
		uint32_t pos = tile_start + block_excl_add(sum, m.tmp, &tot);
		if (k0 < nruns) {
			bool prev_solid = k0 > 0 ? ((__ldg(s + k0 - 1) >> 24) != 0) : false;
			uint32_t cur = 0xFFFFFFFFu, acc_r = 0, acc_t = 0;
#pragma unroll
			for (int j = 0; j < K; j++) {
				/* runs past R^3 voxels (a malformed stream) are dropped */
				if (k0 + j >= nruns || pos >= (uint32_t)(R * R * R)) break;
				const uint32_t p = pos;
				pos += w[j] & 0xFFFFFFu;
				const bool solid = (w[j] >> 24) != 0;
				const uint32_t key = p >> 5;
				if (key != cur) {
					if (cur != 0xFFFFFFFFu) {
						const uint32_t row = cur >> 2, q = cur & 3u;
						atomicOr(rs32 + 4 * row + q, acc_r);
						if (acc_t) atomicOr(occ32 + 2 * bh(row & (R - 1), row >> 7) + q, acc_t);
					}
					cur = key;
					acc_r = acc_t = 0;
				}
				const uint32_t bit = 1u << (p & 31u);
				acc_r |= bit;
				if (solid != prev_solid) acc_t |= bit;
				prev_solid = solid;
			}
			if (cur != 0xFFFFFFFFu) {
				const uint32_t row = cur >> 2, q = cur & 3u;
				atomicOr(rs32 + 4 * row + q, acc_r);
				if (acc_t) atomicOr(occ32 + 2 * bh(row & (R - 1), row >> 7) + q, acc_t);
			}
		}
		covered += tot;
		tile_start += tot;
		if (covered >= (uint64_t)R * R * R) break;
	}
	__syncthreads();
	/* prefix XOR of the toggles (carried across the row's two words) and
	 * run-start ranks; each warp owns a contiguous row segment */
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const int seg = (RR + nw - 1) / nw;
	const int lo = warp * seg, hi = min(RR, lo + seg);
	uint32_t par = 0, cnt = 0;
	for (int r = lo + lane; r < hi; r += 32) {
		const uint64_t *o = m.occ + bh(r & (R - 1), r >> 7);
		par ^= (uint32_t)(__popcll(o[0]) + __popcll(o[1])) & 1u;
		cnt += __popcll(m.rs[2 * r]) + __popcll(m.rs[2 * r + 1]);
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
	const uint32_t cv = m.tmp[32 + warp];
	uint32_t cpar = cv & 1u, ccnt = cv >> 1;
	for (int b = lo; b < hi; b += 32) {
		const int r = b + lane;
		uint64_t t0 = 0, t1 = 0, q0 = 0, q1 = 0;
		uint64_t *o = nullptr;
		if (r < hi) {
			o = m.occ + bh(r & (R - 1), r >> 7);
			t0 = o[0];
			t1 = o[1];
			q0 = m.rs[2 * r];
			q1 = m.rs[2 * r + 1];
		}
		const uint32_t p0 = (uint32_t)__popcll(t0) & 1u;
		const uint32_t p = (p0 + (uint32_t)__popcll(t1)) & 1u, n = __popcll(q0) + __popcll(q1);
		const uint32_t pi = warp_incl_xor(p), ni = warp_incl_add(n);
		if (r < hi) {
			const uint32_t before = cpar ^ pi ^ p; /* toggles before this row */
			uint64_t o0 = prefix_xor64(t0), o1 = prefix_xor64(t1);
			if (before) o0 = ~o0;
			if (before ^ p0) o1 = ~o1;
			o[0] = o0;
			o[1] = o1;
			m.rank[r] = ccnt + ni - n;
		}
		cpar ^= __shfl_sync(kFull, pi, 31);
		ccnt += __shfl_sync(kFull, ni, 31);
	}
	__syncthreads();
}

/* Colour of a solid voxel of the decoded chunk. */
__device__ __forceinline__ uint32_t colour_at_big(const uint32_t *__restrict__ s, const BigMem &m, int x, int y, int z)
{
	const int row = (z << 7) | y;
	const uint64_t a = m.rs[2 * row];
	uint32_t c;
	if (x < 64)
		c = __popcll(a & (~0ull >> (63 - x)));
	else
		c = __popcll(a) + __popcll(m.rs[2 * row + 1] & (~0ull >> (127 - x)));
	return __ldg(s + m.rank[row] + c - 1u) >> 24;
}

/* Shell of a decoded 128^3 chunk: planes x = 0 / R-1 (bits over y, per z),
 * y = 0 / R-1 (rows per z), z = 0 / R-1 (rows per y), two words each, and
 * the colours of the three low planes. */
static __device__ void shell_big(const uint32_t *__restrict__ stream, const BigMem &m, uint64_t *bits, uint8_t *cols)
{
	constexpr int R = Big::R, RR = Big::RR;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int z = warp; z < R; z += nw) {
		uint64_t b0[2] = {0, 0}, b1[2] = {0, 0};
#pragma unroll
		for (int h = 0; h < 4; h++) {
			const int y = 32 * h + lane;
			const uint64_t *o = m.occ + bh(y, z);
			const uint32_t lo = __ballot_sync(kFull, (o[0] & 1ull) != 0);
			const uint32_t hi = __ballot_sync(kFull, ((o[1] >> 63) & 1ull) != 0);
			b0[h >> 1] |= (uint64_t)lo << (32 * (h & 1));
			b1[h >> 1] |= (uint64_t)hi << (32 * (h & 1));
		}
		if (lane < 2) {
			bits[(kPX0 * R + z) * 2 + lane] = b0[lane];
			bits[(kPX1 * R + z) * 2 + lane] = b1[lane];
		}
	}
	for (int i = threadIdx.x; i < 2 * R; i += blockDim.x) {
		const int v = i >> 1, w = i & 1;
		bits[(kPY0 * R + v) * 2 + w] = m.occ[bh(0, v) + w];
		bits[(kPY1 * R + v) * 2 + w] = m.occ[bh(R - 1, v) + w];
		bits[(kPZ0 * R + v) * 2 + w] = m.occ[bh(v, 0) + w];
		bits[(kPZ1 * R + v) * 2 + w] = m.occ[bh(v, R - 1) + w];
	}
	for (int i = threadIdx.x; i < RR; i += blockDim.x) {
		const int a = i & (R - 1), b = i >> 7;
		uint32_t c0 = 0, c1 = 0, c2 = 0;
		if (m.occ[bh(a, b)] & 1ull) c0 = colour_at_big(stream, m, 0, a, b);
		if ((m.occ[bh(0, b) + (a >> 6)] >> (a & 63)) & 1ull) c1 = colour_at_big(stream, m, a, 0, b);
		if ((m.occ[bh(b, 0) + (a >> 6)] >> (a & 63)) & 1ull) c2 = colour_at_big(stream, m, a, b, 0);
		cols[i] = (uint8_t)c0;
		cols[RR + i] = (uint8_t)c1;
		cols[2 * RR + i] = (uint8_t)c2;
	}
}

/* Row (ly, lz) of the neighbour chunk nc, from one of its y or z planes. */
__device__ __forceinline__ void shell_row_big(const SetDesc &S, int32_t nc, int ly, int lz, uint64_t &w0, uint64_t &w1)
{
	constexpr int R = Big::R;
	w0 = w1 = 0;
	if (nc < 0) return;
	const uint64_t *b = S.shell_bits + (size_t)nc * Big::shell_words;
	int p, v;
	if (ly == 0) { p = kPY0; v = lz; }
	else if (ly == R - 1) { p = kPY1; v = lz; }
	else if (lz == 0) { p = kPZ0; v = ly; }
	else { p = kPZ1; v = ly; }
	w0 = b[(p * R + v) * 2];
	w1 = b[(p * R + v) * 2 + 1];
}

/* Row lz of the neighbour's x = 0 (lx == 0) or x = R-1 plane: bits over y. */
__device__ __forceinline__ void shell_xrow_big(const SetDesc &S, int32_t nc, int lx, int lz, uint64_t &w0, uint64_t &w1)
{
	constexpr int R = Big::R;
	w0 = w1 = 0;
	if (nc < 0) return;
	const uint64_t *b = S.shell_bits + (size_t)nc * Big::shell_words;
	const int p = lx == 0 ? kPX0 : kPX1;
	w0 = b[(p * R + lz) * 2];
	w1 = b[(p * R + lz) * 2 + 1];
}

static __device__ void load_halo_big(const SetDesc &S, const BigMem &m)
{
	constexpr int R = Big::R, H = Big::H;
	for (int i = threadIdx.x; i < 2 * H + 2 * R; i += blockDim.x) {
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
		uint64_t w0, w1;
		shell_row_big(S, m.nbr[nbr_slot(0, dy, dz)], y - dy * R, z - dz * R, w0, w1);
		m.occ[bh(y, z)] = w0;
		m.occ[bh(y, z) + 1] = w1;
	}
	for (int i = threadIdx.x; i < 2 * H; i += blockDim.x) {
		const int side = i / H, z = (i % H) - 1;
		const int dx = side ? 1 : -1;
		const int lx = side ? 0 : R - 1;
		const int dz = z < 0 ? -1 : (z >= R ? 1 : 0);
		const int lz = z - dz * R;
		uint64_t w0, w1, m0, m1, p0, p1;
		shell_xrow_big(S, m.nbr[nbr_slot(dx, 0, dz)], lx, lz, w0, w1);
		shell_xrow_big(S, m.nbr[nbr_slot(dx, -1, dz)], lx, lz, m0, m1);
		shell_xrow_big(S, m.nbr[nbr_slot(dx, 1, dz)], lx, lz, p0, p1);
		m.xrow[(side * H + z + 1) * 2] = w0;
		m.xrow[(side * H + z + 1) * 2 + 1] = w1;
		m.xedge[(side * 2 + 0) * H + z + 1] = (uint8_t)((m1 >> 63) & 1ull); /* y = R-1 of the y-1 chunk */
		m.xedge[(side * 2 + 1) * H + z + 1] = (uint8_t)(p0 & 1ull);         /* y = 0 of the y+1 chunk */
	}
	__syncthreads();
}

/* The x = R column bit at (y, z), y and z in [0, R). */
__device__ __forceinline__ uint64_t xhi_bit_big(const BigMem &m, int y, int z)
{
	return (m.xrow[(Big::H + z + 1) * 2 + (y >> 6)] >> (y & 63)) & 1ull;
}

__device__ __forceinline__ uint32_t occ_at_big(const BigMem &m, int x, int y, int z)
{
	constexpr int R = Big::R, H = Big::H;
	if (x < 0 || x >= R) {
		const int side = x >= R;
		if (y < 0) return m.xedge[(side * 2) * H + z + 1];
		if (y >= R) return m.xedge[(side * 2 + 1) * H + z + 1];
		return (uint32_t)((m.xrow[(side * H + z + 1) * 2 + (y >> 6)] >> (y & 63)) & 1ull);
	}
	return (uint32_t)((m.occ[bh(y, z) + (x >> 6)] >> (x & 63)) & 1ull);
}

/* Replace the occupancy rows by the L0 mask rows, as splat_prepare. */
static __device__ void splat_prepare_big(const BigMem &m)
{
	constexpr int R = Big::R;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int z = warp; z < R; z += nw) {
		uint64_t b[2] = {0, 0};
#pragma unroll
		for (int h = 0; h < 4; h++) {
			const int y = 32 * h + lane;
			const bool bit = xhi_bit_big(m, y, z) && !((m.occ[bh(y, z) + 1] >> 63) & 1ull);
			b[h >> 1] |= (uint64_t)__ballot_sync(kFull, bit) << (32 * (h & 1));
		}
		if (lane < 2) m.e0p[z * 2 + lane] = b[lane];
	}
	for (int i = threadIdx.x; i < 2 * R; i += blockDim.x) {
		const int v = i >> 1, w = i & 1;
		m.e0p[(R + v) * 2 + w] = m.occ[bh(R, v) + w] & ~m.occ[bh(R - 1, v) + w];
		m.e0p[(2 * R + v) * 2 + w] = m.occ[bh(v, R) + w] & ~m.occ[bh(v, R - 1) + w];
	}
	__syncthreads();
	const int P = min((int)blockDim.x / R, R); /* planes per slab */
	int cur = 0;
	for (int z0 = 0; z0 < R; z0 += P) {
		const int t = threadIdx.x;
		const bool act = t < P * R && z0 + t / R < R;
		const int y = t & (R - 1), z = z0 + t / R;
		uint64_t e0 = 0, e1 = 0, o0 = 0, o1 = 0;
		if (act) {
			const uint64_t *ro = m.occ + bh(y, z);
			o0 = ro[0];
			o1 = ro[1];
			const uint64_t xp0 = (o0 >> 1) | (o1 << 63), xp1 = (o1 >> 1) | (xhi_bit_big(m, y, z) << 63);
			const uint64_t xm0 = (o0 << 1) | 1ull, xm1 = (o1 << 1) | (o0 >> 63);
			const uint64_t *yp = m.occ + bh(y + 1, z), *zp = m.occ + bh(y, z + 1);
			uint64_t ym0 = ~0ull, ym1 = ~0ull, zm0 = ~0ull, zm1 = ~0ull;
			if (y) {
				ym0 = m.occ[bh(y - 1, z)];
				ym1 = m.occ[bh(y - 1, z) + 1];
			}
			if (z == z0 && z) {
				zm0 = m.sv[(cur * R + y) * 2];
				zm1 = m.sv[(cur * R + y) * 2 + 1];
			} else if (z) {
				zm0 = m.occ[bh(y, z - 1)];
				zm1 = m.occ[bh(y, z - 1) + 1];
			}
			e0 = o0 & ~(xp0 & xm0 & yp[0] & ym0 & zp[0] & zm0);
			e1 = o1 & ~(xp1 & xm1 & yp[1] & ym1 & zp[1] & zm1);
		}
		__syncthreads();
		if (act) {
			if (z == z0 + P - 1) {
				m.sv[((cur ^ 1) * R + y) * 2] = o0;
				m.sv[((cur ^ 1) * R + y) * 2 + 1] = o1;
			}
			m.occ[bh(y, z)] = e0;
			m.occ[bh(y, z) + 1] = e1;
		}
		__syncthreads();
		cur ^= 1;
	}
}

/* L0 mask row (y, z) in [0, R]^2 once splat_prepare_big has run: bits
 * x < 64 in a, 64 <= x < 128 in b, the x = R cell in xr. */
__device__ __forceinline__ void e0_row_big(const BigMem &m, int y, int z, uint64_t &a, uint64_t &b, uint32_t &xr)
{
	constexpr int R = Big::R;
	a = b = 0;
	xr = 0;
	if (y < R && z < R) {
		xr = (uint32_t)((m.e0p[z * 2 + (y >> 6)] >> (y & 63)) & 1ull);
		a = m.occ[bh(y, z)];
		b = m.occ[bh(y, z) + 1];
	} else if (y == R && z < R) {
		a = m.e0p[(R + z) * 2];
		b = m.e0p[(R + z) * 2 + 1];
	} else if (z == R && y < R) {
		a = m.e0p[(2 * R + y) * 2];
		b = m.e0p[(2 * R + y) * 2 + 1];
	}
}

/* Level-l mask row (y, z): cells x < 64 in a, 64 <= x < 128 in b (level 0
 * only), and xr = the cell at x = R >> l for levels 0 and 1 (R >> l >= 64);
 * for levels >= 2 every cell is in a. */
__device__ __forceinline__ void level_row_big(const BigMem &m, int l, int y, int z, uint64_t &a, uint64_t &b,
					      uint32_t &xr)
{
	if (l == 0) {
		e0_row_big(m, y, z, a, b, xr);
		return;
	}
	b = 0;
	const int n = big_n_at(l);
	if (l == 1) {
		const size_t i = (size_t)z * n + y;
		a = m.lv[2 * i];
		xr = (uint32_t)(m.lv[2 * i + 1] & 1ull);
		return;
	}
	xr = 0;
	/* levels >= 2 follow level 1's 65 x 65 two-word rows */
	a = m.lv[c_lv.off[7][l] + 65 * 65 + z * n + y];
}

__device__ __forceinline__ uint32_t mask_colour_big(const SetDesc &S, const uint32_t *__restrict__ s, const BigMem &m,
						   int x, int y, int z)
{
	constexpr int R = Big::R, RR = Big::RR;
	int a = -1, idx = 0;
	if (x == R) { a = 0; idx = (z << 7) | y; }
	else if (y == R) { a = 1; idx = (z << 7) | x; }
	else if (z == R) { a = 2; idx = (y << 7) | x; }
	if (a < 0) return colour_at_big(s, m, x, y, z);
	const int32_t nc = m.nbr[nbr_slot(a == 0, a == 1, a == 2)];
	if (nc < 0) return 0u;
	return S.shell_col[(size_t)nc * Big::shell_cols + (size_t)a * RR + idx];
}

/* One level-L splat, as emit_splat: walk down (compile-time levels),
 * colour, shadow (bounds-free when the chunk's sample window lies inside
 * the map), store. */
template <int L>
__device__ __forceinline__ void emit_splat_big(const SetDesc &S, const uint32_t *__restrict__ stream, const BigMem &m,
					       const uint32_t cv[3], int x, int y, int z, int16_t *dst, bool sh_in,
					       int colour_in = -1)
{
	constexpr int R = Big::R;
	int cx = x, cy = y, cz = z;
#pragma unroll
	for (int lc = L - 1; lc >= 0; lc--) {
		const int np = (R >> lc) + 1;
		const int X = 2 * cx;
		const int xpos = lc <= 1 ? (R >> lc) : (1 << 30);
		uint32_t pat = 0;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int Y = 2 * cy + (q & 1), Z = 2 * cz + (q >> 1);
			if (Y < np && Z < np) {
				uint64_t a, b;
				uint32_t xr;
				level_row_big(m, lc, Y, Z, a, b, xr);
				/* X is even: X and X + 1 lie in the same word */
				uint32_t b2;
				if (X == xpos) b2 = xr;
				else if (X < 64) b2 = (uint32_t)((a >> X) & 3ull);
				else b2 = (uint32_t)((b >> (X - 64)) & 3ull);
				pat |= b2 << (2 * q);
			}
		}
		const int best = pat ? 31 - __clz(pat) : 0;
		cx = X + (best & 1);
		cy = 2 * cy + ((best >> 1) & 1);
		cz = 2 * cz + (best >> 2);
	}
	const uint32_t colour = (L == 0 && colour_in >= 0) ? (uint32_t)colour_in : mask_colour_big(S, stream, m, cx, cy, cz);
	constexpr uint32_t sh = L ? (1u << L) : 0u;
	const uint32_t wx = (cv[0] << 7) + ((uint32_t)x << L);
	const uint32_t wy = (cv[1] << 7) + ((uint32_t)y << L);
	const uint32_t wz = (cv[2] << 7) + ((uint32_t)z << L);
	uint32_t shadow;
	if (sh_in) {
		const uint32_t lim = wy + sh + 1u;
		const uint16_t *p = S.shadow + (((uint64_t)((wx + sh) + (wy + sh)) + (uint64_t)S.shadow_w * (wz + sh)) -
						S.shadow_base);
		shadow = !((__ldg(p) < lim) & (__ldg(p + 1) < lim));
	} else {
		shadow = (uint32_t)shadow_sample(S, wx + sh, wy + sh, wz + sh);
	}
	store_splat(dst, wx, wy, wz, colour | (shadow << 6));
}

/* Level-L rows (L >= 1) of a 128^3 chunk, each 32-row group counted as a
 * warp writes it (the warp's 32 rows are one emission group). */
template <int L>
__device__ __forceinline__ void build_level_big(const BigMem &m)
{
	constexpr uint32_t n = (uint32_t)big_n_at(L), np = (uint32_t)big_n_at(L - 1);
	const uint32_t lane = threadIdx.x & 31u;
	for (uint32_t base = threadIdx.x & ~31u; base < n * n; base += blockDim.x) {
		const uint32_t i = base + lane;
		uint32_t c = 0;
		if (i < n * n) {
			const uint32_t z = i / n, y = i - z * n;
			uint64_t acc0 = 0, acc1 = 0;
			uint32_t accx = 0;
#pragma unroll
			for (uint32_t dz = 0; dz < 2; dz++)
#pragma unroll
				for (uint32_t dy = 0; dy < 2; dy++) {
					const uint32_t yy = 2 * y + dy, zz = 2 * z + dz;
					if (yy >= np || zz >= np) continue;
					uint64_t a, b;
					uint32_t xr;
					level_row_big(m, L - 1, (int)yy, (int)zz, a, b, xr);
					acc0 |= a;
					acc1 |= b;
					accx |= xr;
				}
			if (L == 1) {
				const uint64_t row = compress_pairs(acc0) | (compress_pairs(acc1) << 32);
				m.lv[2 * (size_t)i] = row;
				m.lv[2 * (size_t)i + 1] = accx;
				c = (uint32_t)__popcll(row) + accx;
			} else if (L == 2) {
				const uint64_t row = compress_pairs(acc0) | ((uint64_t)accx << 32);
				m.lv[big_lv_off(2) + i] = row;
				c = (uint32_t)__popcll(row);
			} else {
				const uint64_t row = compress_pairs(acc0);
				m.lv[c_lv.off[7][L] + 65 * 65 + i] = row;
				c = (uint32_t)__popcll(row);
			}
		}
		c = __reduce_add_sync(kFull, c);
		if (lane == 0) m.grp[c_lv.gstart[7][L] + base / 32u] = c;
	}
}

/* Pass 2 of one non-empty 32-row group of level L, as splat_group. */
template <int L>
__device__ __forceinline__ void splat_group_big(const SetDesc &S, const uint32_t *__restrict__ stream, const BigMem &m,
						const uint32_t cv[3], int g, int16_t *dst, bool sh_in)
{
	constexpr int R = Big::R;
	constexpr uint32_t n = (uint32_t)big_n_at(L);
	const int lane = threadIdx.x & 31;
	const uint32_t r = (uint32_t)(g - c_lv.gstart[7][L]) * 32u + (uint32_t)lane;
	uint64_t a = 0, b = 0;
	uint32_t xr = 0, yz = 0;
	/* level 0: the row's run starts and rank, read once per row (global
	 * scratch) and handed to the row's items by shuffles */
	uint64_t rsa = 0, rsb = 0;
	uint32_t rk = 0;
	if (r < n * n) {
		const uint32_t z = r / n, y = r - z * n;
		level_row_big(m, L, (int)y, (int)z, a, b, xr);
		yz = y | (z << 16);
		if (L == 0 && y < (uint32_t)R && z < (uint32_t)R) {
			const uint32_t row = (z << 7) | y;
			rsa = m.rs[2 * row];
			rsb = m.rs[2 * row + 1];
			rk = m.rank[row];
		}
	}
	const uint32_t c = (uint32_t)__popcll(a) + (L == 0 ? (uint32_t)__popcll(b) : 0u) + xr;
	const uint32_t inc = warp_incl_add(c);
	const uint32_t excl = inc - c;
	const uint32_t T = __shfl_sync(kFull, inc, 31);
	const uint32_t base = m.grp[g];
	for (uint32_t k = 0; k < T; k += 32) {
		const uint32_t j0 = k + (uint32_t)lane;
		const int s0 = search_lane(excl, j0);
		const uint32_t e0 = __shfl_sync(kFull, excl, s0), q0 = __shfl_sync(kFull, yz, s0);
		const uint64_t wa = shfl64(a, s0);
		const uint64_t wb = L == 0 ? shfl64(b, s0) : 0ull;
		const uint64_t ra = L == 0 ? shfl64(rsa, s0) : 0ull, rb = L == 0 ? shfl64(rsb, s0) : 0ull;
		const uint32_t rk0 = L == 0 ? __shfl_sync(kFull, rk, s0) : 0u;
		if (j0 < T) {
			int kk = (int)(j0 - e0);
			int x;
			const int ca = __popcll(wa);
			if (kk < ca) {
				x = select_bit(wa, kk);
			} else if (L == 0) {
				kk -= ca;
				x = kk < __popcll(wb) ? 64 + select_bit(wb, kk) : R;
			} else {
				x = R >> L; /* level 1: the x = 64 cell (levels >= 2 hold it in a) */
			}
			const int y = (int)(q0 & 0xFFFFu), z = (int)(q0 >> 16);
			int col = -1;
			if (L == 0 && x < R && y < R && z < R) {
				const uint32_t cnt = x < 64 ? (uint32_t)__popcll(ra & (~0ull >> (63 - x)))
							    : (uint32_t)(__popcll(ra) + __popcll(rb & (~0ull >> (127 - x))));
				col = (int)(__ldg(stream + (rk0 + cnt - 1u)) >> 24);
			}
			emit_splat_big<L>(S, stream, m, cv, x, y, z, dst + (size_t)(base + j0) * 4, sh_in, col);
		}
	}
}

static __device__ void splat_chunk_big(const SetDesc &S, const uint32_t *__restrict__ stream, const BigMem &m,
				const uint32_t cv[3], int lod_max, ChunkOut *out, const Arena &asvl)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	__shared__ unsigned long long s_base;
	__shared__ uint32_t s_ok, s_next;
	__shared__ uint16_t s_glist[big_max_groups()];
	const int *gstart = c_lv.gstart[7];
	splat_prepare_big(m);
	/* level rows: pairwise OR of the child rows, compacted along x; their
	 * groups are counted as they are written */
	for (int l = 1; l <= lod_max; l++) {
		switch (l) {
		case 1: build_level_big<1>(m); break;
		case 2: build_level_big<2>(m); break;
		case 3: build_level_big<3>(m); break;
		case 4: build_level_big<4>(m); break;
		case 5: build_level_big<5>(m); break;
		case 6: build_level_big<6>(m); break;
		default: build_level_big<7>(m); break;
		}
		__syncthreads();
	}
	/* pass 1: level 0's groups */
	const int ngroups = gstart[lod_max + 1];
	for (int g = warp; g < gstart[1]; g += nw) {
		const int r = g * 32 + lane;
		uint32_t c = 0;
		if (r < 129 * 129) {
			const int z = r / 129, y = r - z * 129;
			uint64_t a, b;
			uint32_t xr;
			e0_row_big(m, y, z, a, b, xr);
			c = (uint32_t)(__popcll(a) + __popcll(b)) + xr;
		}
		c = __reduce_add_sync(kFull, c);
		if (lane == 0) m.grp[g] = c;
	}
	__syncthreads();
	const uint32_t total = scan_groups(m.grp, ngroups, m.tmp, s_glist);
	const uint32_t listed = m.tmp[1];
	if (threadIdx.x == 0) {
		const uint64_t units = ((uint64_t)total + 1u) / 2u; /* 8 B per splat */
		unsigned long long b = units ? atomicAdd(asvl.cursor, (unsigned long long)units) : 0ull;
		const uint32_t ok = (b + units <= asvl.cap_units);
		s_base = b;
		s_ok = ok;
		s_next = 0;
		out->svl_off = b * 8u;
		out->svl_total = total * 4u;
		for (int l = 0; l < kMaxLevels; l++) {
			uint32_t c = 0;
			if (l <= lod_max) {
				const uint32_t b0 = m.grp[gstart[l]];
				const uint32_t b1 = gstart[l + 1] < ngroups ? m.grp[gstart[l + 1]] : total;
				c = b1 - b0;
			}
			out->svl_items[l] = c * 4u;
		}
		out->vbo_off = out->ibo_off = 0;
		out->vbo_items = out->ibo_items = 0;
		out->status = ok ? 0u : kStatusOverflow;
	}
	__syncthreads();
	if (!s_ok) return;
	int16_t *dst = (int16_t *)asvl.base + s_base * 8u;
	const bool sh_in = shadow_window_inside<7>(S, cv, lod_max);
	/* pass 2: warps take the non-empty groups from a shared counter */
	for (;;) {
		uint32_t k = 0;
		if (lane == 0) k = atomicAdd(&s_next, 1u);
		k = __shfl_sync(kFull, k, 0);
		if (k >= listed) break;
		const int g = s_glist[k];
		switch (group_level<7>(g)) {
		case 0: splat_group_big<0>(S, stream, m, cv, g, dst, sh_in); break;
		case 1: splat_group_big<1>(S, stream, m, cv, g, dst, sh_in); break;
		case 2: splat_group_big<2>(S, stream, m, cv, g, dst, sh_in); break;
		case 3: splat_group_big<3>(S, stream, m, cv, g, dst, sh_in); break;
		case 4: splat_group_big<4>(S, stream, m, cv, g, dst, sh_in); break;
		case 5: splat_group_big<5>(S, stream, m, cv, g, dst, sh_in); break;
		case 6: splat_group_big<6>(S, stream, m, cv, g, dst, sh_in); break;
		default: splat_group_big<7>(S, stream, m, cv, g, dst, sh_in); break;
		}
	}
}

struct BigAcc {
	const SetDesc &S;
	const uint32_t *__restrict__ stream;
	const BigMem &m;
	__device__ __forceinline__ uint32_t occ(int x, int y, int z) const { return occ_at_big(m, x, y, z); }
	__device__ __forceinline__ uint32_t mcolour(int x, int y, int z) const
	{
		return mask_colour_big(S, stream, m, x, y, z);
	}
};

/* Face bits of row (y, z) in two halves (x < 64: *0, x >= 64: *1). */
__device__ __forceinline__ void face_bits_big(const BigMem &m, int y, int z, uint64_t f[6])
{
	const uint64_t *ro = m.occ + bh(y, z);
	const uint64_t o0 = ro[0], o1 = ro[1];
	const uint64_t *yp = m.occ + bh(y + 1, z), *zp = m.occ + bh(y, z + 1);
	f[0] = o0 ^ ((o0 >> 1) | (o1 << 63));
	f[1] = o1 ^ ((o1 >> 1) | (xhi_bit_big(m, y, z) << 63));
	f[2] = o0 ^ yp[0];
	f[3] = o1 ^ yp[1];
	f[4] = o0 ^ zp[0];
	f[5] = o1 ^ zp[1];
}

static __device__ void mesh_chunk_big(const SetDesc &S, const uint32_t *__restrict__ stream, const BigMem &m,
			       const uint32_t cv[3], ChunkOut *out, const Arena &avbo, const Arena &aibo)
{
	constexpr int R = Big::R, RR = Big::RR, NG = RR / 32;
	__shared__ unsigned long long s_base[2];
	__shared__ uint32_t s_ok, s_next;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int g = warp; g < NG; g += nw) {
		const int r = g * 32 + lane;
		uint64_t f[6];
		face_bits_big(m, r & (R - 1), r >> 7, f);
		uint32_t c = 0;
#pragma unroll
		for (int k = 0; k < 6; k++) c += __popcll(f[k]);
#pragma unroll
		for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
		if (lane == 0) m.grp[g] = c;
	}
	__syncthreads();
	const uint32_t faces = scan_groups(m.grp, NG, m.tmp);
	if (threadIdx.x == 0) {
		const uint64_t uv = (uint64_t)faces * 2u;
		const uint64_t ui = ((uint64_t)faces * 24u + 15u) / 16u;
		unsigned long long bv = uv ? atomicAdd(avbo.cursor, (unsigned long long)uv) : 0ull;
		unsigned long long bi = ui ? atomicAdd(aibo.cursor, (unsigned long long)ui) : 0ull;
		uint32_t ok = (bv + uv <= avbo.cap_units) && (bi + ui <= aibo.cap_units);
		s_base[0] = bv;
		s_base[1] = bi;
		s_ok = ok;
		s_next = 0;
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
	const BigAcc acc{S, stream, m};
	for (;;) {
		uint32_t g = 0;
		if (lane == 0) g = atomicAdd(&s_next, 1u);
		g = __shfl_sync(kFull, g, 0);
		if (g >= (uint32_t)NG) break;
		const int r = (int)g * 32 + lane;
		uint64_t f[6];
		face_bits_big(m, r & (R - 1), r >> 7, f);
		const uint32_t clo = __popcll(f[0]) + __popcll(f[2]) + __popcll(f[4]);
		const uint32_t c = clo + __popcll(f[1]) + __popcll(f[3]) + __popcll(f[5]);
		const uint32_t inc = warp_incl_add(c);
		const uint32_t excl = inc - c;
		const uint32_t T = __shfl_sync(kFull, inc, 31);
		const uint32_t base = m.grp[g];
		for (uint32_t k = 0; k < T; k += 32) {
			const uint32_t j = k + lane;
			const int s = search_lane(excl, j);
			const uint32_t e = __shfl_sync(kFull, excl, s), lo = __shfl_sync(kFull, clo, s);
			uint64_t w[6];
#pragma unroll
			for (int q = 0; q < 6; q++) w[q] = shfl64(f[q], s);
			if (j < T) {
				uint32_t kk = j - e;
				int x, i;
				if (kk < lo) {
					select_face<6>(w[0], w[2], w[4], kk, x, i);
				} else {
					select_face<6>(w[1], w[3], w[5], kk - lo, x, i);
					x += 64;
				}
				const int rr = (int)g * 32 + s;
				emit_face<7>(acc, S, cv, x, rr & (R - 1), rr >> 7, i, base + j, vbo, ibo);
			}
		}
	}
}

/* The dense L0 mask of chunk_make_mask for a 128^3 chunk. */
static __device__ void mask_dense_big(const SetDesc &S, const uint32_t *__restrict__ stream, const BigMem &m, uint8_t *dst)
{
	constexpr int R = Big::R, S1 = R + 1;
	splat_prepare_big(m);
	for (int i = threadIdx.x; i < S1 * S1; i += blockDim.x) {
		const int y = i % S1, z = i / S1;
		uint64_t a, b;
		uint32_t xr;
		e0_row_big(m, y, z, a, b, xr);
		uint8_t *line = dst + ((size_t)z * S1 + y) * S1;
		for (uint64_t v = a; v; v &= v - 1ull) {
			const int x = __ffsll((long long)v) - 1;
			line[x] = (uint8_t)mask_colour_big(S, stream, m, x, y, z);
		}
		for (uint64_t v = b; v; v &= v - 1ull) {
			const int x = 64 + __ffsll((long long)v) - 1;
			line[x] = (uint8_t)mask_colour_big(S, stream, m, x, y, z);
		}
		if (xr) line[R] = (uint8_t)mask_colour_big(S, stream, m, R, y, z);
	}
}

/* One 128^3 work item: decode, halo, then mask / mesh / splats. */
static __device__ void geometry_item_big(const SetDesc &S, const WorkItem &wi, ChunkOut *out, const BigMem &m,
				  const Arena &asvl, const Arena &avbo, const Arena &aibo, int lod_max)
{
	constexpr int R = Big::R;
	uint32_t cv[3], wc[3];
	chunk_coords(S, wi.chunk, cv);
	for (int k = 0; k < 3; k++) wc[k] = (uint32_t)(S.origin[k] + (int32_t)cv[k]);
	const uint32_t N = (uint32_t)R * R * R;
	load_neighbours(S, cv, m.nbr, N);
	const bool empty = m.nbr[nbr_slot(0, 0, 0)] < 0 && m.nbr[nbr_slot(1, 0, 0)] < 0 &&
			   m.nbr[nbr_slot(0, 1, 0)] < 0 && m.nbr[nbr_slot(0, 0, 1)] < 0;
	if (empty && !(wi.flags & kItemMaskDense)) {
		if (threadIdx.x == 0) {
			out->svl_off = out->vbo_off = out->ibo_off = 0;
			for (int l = 0; l < kMaxLevels; l++) out->svl_items[l] = 0;
			out->svl_total = out->vbo_items = out->ibo_items = 0;
			out->status = 0;
		}
		return;
	}
	const uint32_t *stream = S.pool + S.off[wi.chunk];
	decode_big(stream, S.len[wi.chunk] - 1u, m);
	load_halo_big(S, m);
	if (wi.flags & kItemMaskDense)
		mask_dense_big(S, stream, m, (uint8_t *)asvl.base + (size_t)wi.slot * (R + 1) * (R + 1) * (R + 1));
	else if (wi.flags & kItemMesh)
		mesh_chunk_big(S, stream, m, wc, out, avbo, aibo);
	else
		splat_chunk_big(S, stream, m, wc, lod_max, out, asvl);
}

} // namespace vp
