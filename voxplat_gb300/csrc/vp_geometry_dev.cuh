/*
 * vp_geometry_dev.cuh — device code of the per-chunk geometry pipeline on
 * sm_103a, shared by the translation units that instantiate its kernels
 * (vp_geometry_r{3,4,5,6,7}.cu, vp_geometry_mixed{1,2}.cu; one root size or
 * one mixed variant each, so they compile in parallel).
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
#pragma once
#include <algorithm>

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
	/* shared memory carve, byte offsets (every region 16-byte aligned):
	 * 64^3 chunks need ~98 KB, so two CTAs share an SM */
	static constexpr size_t o_occ = 0;
	static constexpr size_t o_rs = a16(o_occ + sizeof(uint64_t) * H * H);
	static constexpr size_t o_rank = a16(o_rs + sizeof(uint64_t) * RR);
	static constexpr size_t o_lv = a16(o_rank + sizeof(uint32_t) * RR);
	static constexpr size_t o_xrow = a16(o_lv + sizeof(uint64_t) * lv_words());
	static constexpr size_t o_xedge = a16(o_xrow + sizeof(uint64_t) * 2 * H);
	static constexpr size_t o_tmp = a16(o_xedge + 4 * H);
	static constexpr int groups_of(int rows) { return (rows + 31) / 32; }
	static constexpr int max_groups()
	{
		int t = 0;
		for (int l = 0; l < kMaxLevels; l++) t += groups_of(n_at(l) * n_at(l));
		return t > groups_of(RR) ? t : groups_of(RR);
	}
	static constexpr size_t o_grp = a16(o_tmp + sizeof(uint32_t) * 64);
	static constexpr size_t o_glist = a16(o_grp + sizeof(uint32_t) * (max_groups() + 1));
	static constexpr size_t o_e0p = a16(o_glist + sizeof(uint16_t) * max_groups());
	static constexpr size_t o_sv = a16(o_e0p + sizeof(uint64_t) * 3 * R);
	static constexpr size_t o_nbr = a16(o_sv + sizeof(uint64_t) * 2 * R);
	static constexpr size_t bytes = a16(o_nbr + sizeof(int32_t) * 28);
	/* a decoded chunk handed from the shell pass to the geometry pass:
	 * occupancy rows and run-start rows (u64, row r = z R + y), then ranks */
	static constexpr size_t dec_occ = (size_t)R * H * 8;  /* z planes 0..R-1, halo rows included */
	static constexpr size_t dec_bytes = dec_occ + (size_t)RR * (8 + 4);
	static constexpr size_t shell_words = 6 * R;   /* u64 per chunk */
	static constexpr size_t shell_cols = 3 * RR;   /* bytes per chunk */
};

struct Smem {
	uint64_t *occ, *rs, *lv;
	uint32_t *rank, *tmp;
	uint32_t *grp;   /* emission base of every emission group (32 or 64 rows) */
	uint16_t *glist; /* the groups with any output, in order */
	uint64_t *e0p;   /* splat mode: L0 mask rows of the x = R, y = R, z = R planes */
	uint64_t *sv;    /* splat mode: two saved occupancy planes */
	uint64_t *xrow;  /* [side][z+1]: x = -1 (side 0) / x = R (side 1), bits over y */
	uint8_t *xedge;  /* [side*2 + (y == R)][z+1]: the y = -1 / y = R corners */
	int32_t *nbr;    /* 27 neighbour chunk indices, -1 = air (outside or null) */
};

template <int RB>
__device__ __forceinline__ Smem carve(uint8_t *base)
{
	using G = Geo<RB>;
	Smem s;
	s.occ = (uint64_t *)(base + G::o_occ);
	s.rs = (uint64_t *)(base + G::o_rs);
	s.rank = (uint32_t *)(base + G::o_rank);
	s.lv = (uint64_t *)(base + G::o_lv);
	s.xrow = (uint64_t *)(base + G::o_xrow);
	s.xedge = base + G::o_xedge;
	s.tmp = (uint32_t *)(base + G::o_tmp);
	s.grp = (uint32_t *)(base + G::o_grp);
	s.glist = (uint16_t *)(base + G::o_glist);
	s.e0p = (uint64_t *)(base + G::o_e0p);
	s.sv = (uint64_t *)(base + G::o_sv);
	s.nbr = (int32_t *)(base + G::o_nbr);
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
	(void)lane;
	uint32_t *rs32 = (uint32_t *)m.rs;
	uint32_t *occ32 = (uint32_t *)m.occ;
	/* each thread owns 8 consecutive runs per tile; bits falling in the same
	 * 32-bit word are combined in registers before one shared atomic */
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
				const uint32_t key = p >> KB;
				if (key != cur) {
					if (cur != 0xFFFFFFFFu) {
						const uint32_t row = (cur << KB) >> RB, half = ((cur << KB) & (R - 1)) >> 5;
						atomicOr(rs32 + 2 * row + half, acc_r);
						if (acc_t) atomicOr(occ32 + 2 * hidx<RB>(row & (R - 1), row >> RB) + half, acc_t);
					}
					cur = key;
					acc_r = acc_t = 0;
				}
				const uint32_t bit = 1u << (p & ((1u << KB) - 1u));
				acc_r |= bit;
				if (solid != prev_solid) acc_t |= bit;
				prev_solid = solid;
			}
			if (cur != 0xFFFFFFFFu) {
				const uint32_t row = (cur << KB) >> RB, half = ((cur << KB) & (R - 1)) >> 5;
				atomicOr(rs32 + 2 * row + half, acc_r);
				if (acc_t) atomicOr(occ32 + 2 * hidx<RB>(row & (R - 1), row >> RB) + half, acc_t);
			}
		}
		covered += tot;
		tile_start += tot;
		if (covered >= (uint64_t)R * R * R) break; /* the chunk is covered */
	}
	__syncthreads();
	/* prefix XOR of the toggle stream and run-start ranks, rows in scan
	 * order; each warp owns a contiguous row segment. */
	const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const int seg = (RR + nw - 1) / nw;
	const int lo = warp * seg, hi = min(RR, lo + seg);
	/* per row: run starts n (<= 64) and toggle parity p, packed as
	 * n << 13 | p so that one add-reduction gives both (the low bit of the
	 * summed parities is their XOR; at most 4096 rows, so the parity sum
	 * stays below 2^13 and the packed sum below 2^32) */
	uint32_t acc = 0;
	for (int r = lo + lane; r < hi; r += 32)
		acc += ((uint32_t)__popcll(m.rs[r]) << 13) | ((uint32_t)__popcll(m.occ[hidx<RB>(r & (R - 1), r >> RB)]) & 1u);
#pragma unroll
	for (int d = 16; d; d >>= 1) acc += __shfl_xor_sync(kFull, acc, d);
	const uint32_t par = acc & 1u, cnt = acc >> 13;
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
		/* one scan of n << 6 | p: the low 6 bits sum the 32 parities */
		const uint32_t p = __popcll(t) & 1u, n = __popcll(q);
		const uint32_t inc = warp_incl_add((n << 6) | p);
		const uint32_t pi = inc & 1u, ni = inc >> 6;
		if (r < hi) {
			uint64_t o = prefix_xor64(t);
			if (cpar ^ pi ^ p) o = ~o;
			m.occ[hi_] = o & G::MASK;
			m.rank[r] = ccnt + ni - n;
		}
		const uint32_t last = __shfl_sync(kFull, inc, 31);
		cpar ^= last & 1u;
		ccnt += last >> 6;
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

/* The decoded chunk handed from the shell pass to the geometry pass of the
 * same rebuild: the occupancy planes z = 0..R-1 as they lie in shared
 * memory (R+2 rows each, halo rows included; the geometry pass rewrites
 * those in load_halo), the run-start rows and the ranks. Both directions
 * are 1-D bulk copies (cp.async.bulk): three per chunk, issued by one
 * thread; every block starts on a 16-byte boundary and is a multiple of 16
 * bytes long. */
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <int RB>
__device__ __forceinline__ void store_decoded(const Smem &m, uint8_t *dst)
{
	using G = Geo<RB>;
	static_assert(G::dec_occ % 16 == 0 && (G::RR * 8) % 16 == 0 && (G::RR * 4) % 16 == 0, "bulk copy sizes");
	static_assert((G::o_occ + G::H * 8) % 16 == 0 && G::o_rs % 16 == 0 && G::o_rank % 16 == 0, "bulk copy bases");
	__syncthreads(); /* the decode's shared-memory writes, then the async proxy reads them */
	if (threadIdx.x == 0) {
		asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
		asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst),
			     "r"(smem_u32(m.occ + G::H)), "r"((uint32_t)G::dec_occ)
			     : "memory");
		asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst + G::dec_occ),
			     "r"(smem_u32(m.rs)), "r"((uint32_t)(G::RR * 8))
			     : "memory");
		asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(
				     dst + G::dec_occ + G::RR * 8),
			     "r"(smem_u32(m.rank)), "r"((uint32_t)(G::RR * 4))
			     : "memory");
		asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
	}
}

/* The bulk stores must have read shared memory before the next decode
 * overwrites it, and be complete before the kernel ends (no user spin: the
 * hardware wait instruction). */
__device__ __forceinline__ void store_decoded_wait()
{
	if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
}

/* Bounded wait on the mbarrier's phase; false when it ran out. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase)
{
	for (uint32_t tries = 0; tries < (1u << 16); tries++) {
		uint32_t ok;
		asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
			     " selp.u32 %0, 1, 0, p;\n}\n"
			     : "=r"(ok)
			     : "r"(smem_u32(bar)), "r"(phase)
			     : "memory");
		if (ok) return true;
	}
	return false;
}

/* Loads a decoded chunk with three bulk copies completing on `bar` (phase
 * `phase`). Returns false on every thread when they did not arrive within
 * the bounded wait (the flag is set). */
template <int RB>
__device__ bool load_decoded(const uint8_t *src, const Smem &m, uint64_t *bar, uint32_t phase, uint32_t *flag)
{
	using G = Geo<RB>;
	if (threadIdx.x == 0) {
		/* earlier generic accesses to these bytes come before the copies */
		asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
			     "r"((uint32_t)G::dec_bytes)
			     : "memory");
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
				     smem_u32(m.occ + G::H)),
			     "l"(src), "r"((uint32_t)G::dec_occ), "r"(smem_u32(bar))
			     : "memory");
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
				     smem_u32(m.rs)),
			     "l"(src + G::dec_occ), "r"((uint32_t)(G::RR * 8)), "r"(smem_u32(bar))
			     : "memory");
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
				     smem_u32(m.rank)),
			     "l"(src + G::dec_occ + G::RR * 8), "r"((uint32_t)(G::RR * 4)), "r"(smem_u32(bar))
			     : "memory");
	}
	const bool ok = mbar_wait(bar, phase);
	if (!ok) atomicOr(flag, 1u);
	__syncthreads();
	const bool all = *flag == 0u;
	__syncthreads();
	return all;
}

/* ------------------------------------------------------------------ */
/* Shell pass                                                          */
/* The shell of a single-run chunk (one run of R^3 voxels and the
 * terminator), without decoding, by one warp: an all-air chunk has none
 * (its neighbours see air); a solid one has every boundary bit set and its
 * run's colour on the three low planes, as the decode path writes them. An
 * item flagged kItemEmpty (all air, with all-air or no +x, +y and +z
 * neighbours) gets no geometry pass: its result record is zeroed here, as
 * the geometry pass would write it. */
template <int RB>
__device__ __forceinline__ void shell_uniform_item(const SetDesc *__restrict__ sets, const WorkItem &wi, ChunkOut *outs)
{
	using G = Geo<RB>;
	constexpr uint32_t N = (uint32_t)G::R * G::R * G::R;
	const int lane = threadIdx.x & 31;
	if (wi.flags & kItemEmpty) {
		static_assert(sizeof(ChunkOut) % 4 == 0, "result records are whole words");
		uint32_t *o = (uint32_t *)(outs + wi.slot);
		for (int i = lane; i < (int)(sizeof(ChunkOut) / 4); i += 32) o[i] = 0u;
		return;
	}
	const SetDesc *S = sets + wi.set;
	if (S->len[wi.chunk] != 2u) return;
	const uint32_t w0 = S->pool[S->off[wi.chunk]];
	if (w0 == N) return;
	uint64_t *bits = S->shell_bits + (size_t)wi.chunk * G::shell_words;
	for (int i = lane; i < (int)G::shell_words; i += 32) bits[i] = G::MASK;
	uint32_t *cols = (uint32_t *)(S->shell_col + (size_t)wi.chunk * G::shell_cols);
	const uint32_t c4 = (w0 >> 24) * 0x01010101u;
	for (int i = lane; i < (int)(G::shell_cols / 4); i += 32) cols[i] = c4;
}

/* ------------------------------------------------------------------ */

template <int RB>
__global__ void __launch_bounds__(512, 2) k_shell(const SetDesc *__restrict__ sets, const WorkItem *__restrict__ items,
					       uint32_t nitems, uint8_t *decoded, const uint32_t *__restrict__ dec_slot,
					       const WorkItem *__restrict__ uni_items, uint32_t n_uni, ChunkOut *outs)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR;
	extern __shared__ __align__(16) uint8_t smem[];
	const Smem m = carve<RB>(smem);
	/* the geometry pass may start launching once the last wave is on */
	grid_release();
	const uint32_t it = blockIdx.x;
	if (it >= nitems) {
		/* the CTAs past the decoded chunks: a single-run chunk per warp
		 * (they run in the launch's last wave) */
		const uint32_t u = (it - nitems) * (blockDim.x >> 5) + (threadIdx.x >> 5);
		if (u < n_uni) shell_uniform_item<RB>(sets, uni_items[u], outs);
		return;
	}
	const WorkItem wi = items[it];
	const SetDesc S = sets[wi.set];
	const uint32_t N = (uint32_t)R * R * R;
	if (chunk_is_null(S, wi.chunk, N)) return;
	const uint32_t *stream = S.pool + S.off[wi.chunk];
	decode_chunk<RB>(stream, S.len[wi.chunk] - 1u, m);
	const uint32_t ds = decoded ? dec_slot[wi.chunk] : kNoSlot;
	if (ds != kNoSlot) store_decoded<RB>(m, decoded + (size_t)ds * G::dec_bytes);
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
	/* branch-free: the three lookups of two cells are in flight together
	 * (an air cell reads a valid word and keeps 0) */
#pragma unroll 2
	for (int i = threadIdx.x; i < RR; i += blockDim.x) {
		const int a = i & (R - 1), b = i >> RB;
		const int r0 = (b << RB) | a, r1 = (b << RB);
		const uint64_t o0 = m.occ[hidx<RB>(a, b)], o1 = m.occ[hidx<RB>(0, b)], o2 = m.occ[hidx<RB>(b, 0)];
		const bool s0 = (o0 & 1ull) != 0, s1 = ((o1 >> a) & 1ull) != 0, s2 = ((o2 >> a) & 1ull) != 0;
		/* (0, a, b): row (a, b), x = 0; (a, 0, b): row (0, b), x = a;
		 * (a, b, 0): row (b, 0), x = a */
		const int ra = r0, rb = r1, rc = b;
		const uint32_t k0 = m.rank[ra] + (uint32_t)(m.rs[ra] & 1ull) - 1u;
		const uint32_t k1 = m.rank[rb] + (uint32_t)__popcll(m.rs[rb] & (~0ull >> (63 - a))) - 1u;
		const uint32_t k2 = m.rank[rc] + (uint32_t)__popcll(m.rs[rc] & (~0ull >> (63 - a))) - 1u;
		const uint32_t w0 = __ldg(stream + (s0 ? k0 : 0u)), w1 = __ldg(stream + (s1 ? k1 : 0u));
		const uint32_t w2 = __ldg(stream + (s2 ? k2 : 0u));
		cols[i] = s0 ? (uint8_t)(w0 >> 24) : (uint8_t)0;
		cols[RR + i] = s1 ? (uint8_t)(w1 >> 24) : (uint8_t)0;
		cols[2 * RR + i] = s2 ? (uint8_t)(w2 >> 24) : (uint8_t)0;
	}
	if (ds != kNoSlot) store_decoded_wait();
}

/* ------------------------------------------------------------------ */
/* Geometry pass                                                       */
/* ------------------------------------------------------------------ */

__device__ __forceinline__ int nbr_slot(int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); }

/* Fill the 27-entry neighbour table: chunk index, or -1 where the neighbour
 * is outside the world or all air (its shell was not written). */
__device__ __forceinline__ void load_neighbours(const SetDesc &S, const uint32_t cv[3], int32_t *nbr, uint32_t N)
{
	if (threadIdx.x < 27) {
		const int t = threadIdx.x;
		const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
		int64_t nc = neighbour(S, cv, dx, dy, dz);
		if (nc >= 0 && chunk_is_null(S, (uint32_t)nc, N)) nc = -1;
		nbr[t] = (int32_t)nc;
	}
	__syncthreads();
}

/* Occupancy row (bits over x) of neighbour-local row (ly, lz), from the
 * neighbour's shell; the row lies on one of its y or z boundary planes. */
template <int RB>
__device__ __forceinline__ uint64_t shell_row(const SetDesc &S, int32_t nc, int ly, int lz)
{
	constexpr int R = Geo<RB>::R;
	if (nc < 0) return 0ull;
	const uint64_t *b = S.shell_bits + (size_t)nc * Geo<RB>::shell_words;
	if (ly == 0) return b[kPY0 * R + lz];
	if (ly == R - 1) return b[kPY1 * R + lz];
	if (lz == 0) return b[kPZ0 * R + ly];
	return b[kPZ1 * R + ly];
}

/* Row lz of the neighbour's x = 0 (lx == 0) or x = R-1 plane: bits over y. */
template <int RB>
__device__ __forceinline__ uint64_t shell_xrow(const SetDesc &S, int32_t nc, int lx, int lz)
{
	constexpr int R = Geo<RB>::R;
	if (nc < 0) return 0ull;
	const uint64_t *b = S.shell_bits + (size_t)nc * Geo<RB>::shell_words;
	return (lx == 0) ? b[kPX0 * R + lz] : b[kPX1 * R + lz];
}

template <int RB>
__device__ void load_halo(const SetDesc &S, const Smem &m)
{
	using G = Geo<RB>;
	constexpr int R = G::R, H = G::H;
	/* halo rows: y in {-1, R} for z in [-1, R], and z in {-1, R} for y in [0, R) */
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
		m.occ[hidx<RB>(y, z)] = shell_row<RB>(S, m.nbr[nbr_slot(0, dy, dz)], y - dy * R, z - dz * R);
	}
	/* x = -1 / x = R columns: one word over y per z, plus the y = -1 and
	 * y = R corners from the diagonal neighbours */
	for (int i = threadIdx.x; i < 2 * H; i += blockDim.x) {
		const int side = i / H, z = (i % H) - 1;
		const int dx = side ? 1 : -1;
		const int lx = side ? 0 : R - 1;
		const int dz = z < 0 ? -1 : (z >= R ? 1 : 0);
		const int lz = z - dz * R;
		m.xrow[side * H + z + 1] = shell_xrow<RB>(S, m.nbr[nbr_slot(dx, 0, dz)], lx, lz);
		const uint64_t ym = shell_xrow<RB>(S, m.nbr[nbr_slot(dx, -1, dz)], lx, lz);
		const uint64_t yp = shell_xrow<RB>(S, m.nbr[nbr_slot(dx, 1, dz)], lx, lz);
		m.xedge[(side * 2 + 0) * H + z + 1] = (uint8_t)((ym >> (R - 1)) & 1ull);
		m.xedge[(side * 2 + 1) * H + z + 1] = (uint8_t)(yp & 1ull);
	}
	__syncthreads();
}

/* The x = R column bit at (y, z), y and z in [0, R). */
template <int RB>
__device__ __forceinline__ uint64_t xhi_bit(const Smem &m, int y, int z)
{
	return (m.xrow[Geo<RB>::H + z + 1] >> y) & 1ull;
}

template <int RB>
__device__ __forceinline__ uint32_t occ_at(const Smem &m, int x, int y, int z)
{
	constexpr int R = Geo<RB>::R, H = Geo<RB>::H;
	if (x < 0 || x >= R) {
		const int side = x >= R;
		if (y < 0) return m.xedge[(side * 2) * H + z + 1];
		if (y >= R) return m.xedge[(side * 2 + 1) * H + z + 1];
		return (uint32_t)((m.xrow[side * H + z + 1] >> y) & 1ull);
	}
	return (uint32_t)((m.occ[hidx<RB>(y, z)] >> x) & 1ull);
}

/* L0 mask row (y, z) in [0, R]^2 once splat_prepare has run: bits x in
 * [0, R); *xr = the x = R cell. */
template <int RB>
__device__ __forceinline__ uint64_t e0_row(const Smem &m, int y, int z, uint32_t &xr)
{
	constexpr int R = Geo<RB>::R;
	xr = 0;
	if (y < R && z < R) {
		xr = (uint32_t)((m.e0p[z] >> y) & 1ull);
		return m.occ[hidx<RB>(y, z)];
	}
	if (y == R && z < R) return m.e0p[R + z];
	if (z == R && y < R) return m.e0p[2 * R + y];
	return 0ull;
}

/* Replace the occupancy rows by the L0 mask rows (src/chunkset/mesher.c:
 * 421-446 restated per bit): a solid voxel is in the mask when any +axis
 * neighbour (the +chunk's voxel at coordinate R) is air, or a -axis
 * neighbour inside the chunk is air; a cell at coordinate R is in the mask
 * when the +chunk's voxel there is solid and ours air. Rows are rewritten in
 * z-slabs; the last original plane of each slab is kept for the next. */
template <int RB>
__device__ void splat_prepare(const Smem &m)
{
	using G = Geo<RB>;
	constexpr int R = G::R;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int z = warp; z < R; z += nw) {
		uint64_t b = 0;
		for (int h = 0; h < (R + 31) / 32; h++) {
			const int y = 32 * h + lane;
			bool bit = false;
			if (y < R) bit = xhi_bit<RB>(m, y, z) && !((m.occ[hidx<RB>(y, z)] >> (R - 1)) & 1ull);
			b |= (uint64_t)__ballot_sync(kFull, bit) << (32 * h);
		}
		if (lane == 0) m.e0p[z] = b & G::MASK;
	}
	for (int v = threadIdx.x; v < R; v += blockDim.x) {
		m.e0p[R + v] = m.occ[hidx<RB>(R, v)] & ~m.occ[hidx<RB>(R - 1, v)];
		m.e0p[2 * R + v] = m.occ[hidx<RB>(v, R)] & ~m.occ[hidx<RB>(v, R - 1)];
	}
	__syncthreads();
	const int P = min((int)blockDim.x / R, R); /* planes per slab */
	int cur = 0;
	for (int z0 = 0; z0 < R; z0 += P) {
		const int t = threadIdx.x;
		const bool act = t < P * R && z0 + t / R < R;
		const int y = t & (R - 1), z = z0 + t / R;
		uint64_t e = 0, o = 0;
		if (act) {
			o = m.occ[hidx<RB>(y, z)];
			const uint64_t xp = (o >> 1) | (xhi_bit<RB>(m, y, z) << (R - 1));
			const uint64_t xm = ((o << 1) | 1ull) & G::MASK;
			const uint64_t yp = m.occ[hidx<RB>(y + 1, z)];
			const uint64_t ym = y ? m.occ[hidx<RB>(y - 1, z)] : G::MASK;
			const uint64_t zp = m.occ[hidx<RB>(y, z + 1)];
			const uint64_t zm = z == 0 ? G::MASK : (z == z0 ? m.sv[cur * R + y] : m.occ[hidx<RB>(y, z - 1)]);
			e = o & ~(xp & xm & yp & ym & zp & zm);
		}
		__syncthreads();
		if (act) {
			if (z == z0 + P - 1) m.sv[(cur ^ 1) * R + y] = o;
			m.occ[hidx<RB>(y, z)] = e;
		}
		__syncthreads();
		cur ^= 1;
	}
}

/* Per chunk size 2^RB and LOD level l: the word offset of the level's rows
 * in the level-row area, its first emission group, and the
 * multiply-shift constant that divides a row index by n = (R >> l) + 1
 * (q = umulhi(r, magic) equals r / n for every r < 2^17 and n <= 129). */
constexpr int kMaxGroupsTab = 768; /* emission groups of a 128^3 chunk: 705 */

struct LevelTab {
	int off[8][kMaxLevels];
	int gstart[8][kMaxLevels + 1];
	uint32_t magic[8][kMaxLevels];
	uint8_t glevel[8][kMaxGroupsTab]; /* level of each emission group */
};

/* Rows per emission group of level l: 32, one per lane, except level 0 of
 * chunks up to 64^3, whose groups are 96 rows, three consecutive rows per
 * lane (a third of the groups to set up, and fewer partly filled steps). */
constexpr int group_rows(int rb, int l) { return (l == 0 && rb <= 6) ? 96 : 32; }

constexpr LevelTab make_level_tab()
{
	LevelTab t{};
	for (int rb = 0; rb < 8; rb++) {
		const int R = 1 << rb;
		int off = 0, g = 0;
		for (int l = 0; l < kMaxLevels; l++) {
			const int n = (R >> l) + 1;
			t.off[rb][l] = l == 0 ? 0 : off;
			if (l >= 1) off += n * n;
			t.gstart[rb][l] = g;
			g += (n * n + group_rows(rb, l) - 1) / group_rows(rb, l);
			t.magic[rb][l] = n == 1 ? 0u : (uint32_t)(0xFFFFFFFFu / (uint32_t)n + 1u);
		}
		t.gstart[rb][kMaxLevels] = g;
		for (int l = 0; l < kMaxLevels; l++)
			for (int k = t.gstart[rb][l]; k < t.gstart[rb][l + 1] && k < kMaxGroupsTab; k++)
				t.glevel[rb][k] = (uint8_t)l;
	}
	return t;
}

static __constant__ LevelTab c_lv = make_level_tab();
static_assert(make_level_tab().gstart[7][kMaxLevels] <= kMaxGroupsTab, "group level table too short");

/* (y, z) of row r of a level with n rows per z and division constant mg */
__device__ __forceinline__ void row_yz(uint32_t r, uint32_t n, uint32_t mg, int &y, int &z)
{
	const uint32_t q = __umulhi(r, mg);
	z = (int)q;
	y = (int)(r - q * n);
}

/* Level-l mask row (y, z); level 0 includes the x = R cell in *xr. */
template <int RB>
__device__ __forceinline__ uint64_t level_row(const Smem &m, int l, int y, int z, uint32_t &xr)
{
	constexpr int R = Geo<RB>::R;
	if (l == 0) return e0_row<RB>(m, y, z, xr);
	xr = 0;
	const int n = (R >> l) + 1;
	return m.lv[c_lv.off[RB][l] + z * n + y];
}

/* Colour of the L0 mask cell (x, y, z) in [0, R]^3: our own voxel, or the
 * +neighbour's voxel for cells at coordinate R (read from its shell). */
template <int RB>
__device__ __forceinline__ uint32_t mask_colour(const SetDesc &S, const uint32_t *__restrict__ s, const Smem &m,
						int x, int y, int z)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR;
	int a = -1, idx = 0;
	if (x == R) { a = 0; idx = (z << RB) | y; }
	else if (y == R) { a = 1; idx = (z << RB) | x; }
	else if (z == R) { a = 2; idx = (y << RB) | x; }
	if (a < 0) return colour_at<RB>(s, m, x, y, z);
	const int32_t nc = m.nbr[nbr_slot(a == 0, a == 1, a == 2)];
	if (nc < 0) return 0u;
	return S.shell_col[(size_t)nc * G::shell_cols + (size_t)a * RR + idx];
}

/* mask_colour with the colour in the top byte of the word returned, so a
 * stream word can be consumed (>> 24) after the next step's loads issue. */
template <int RB>
__device__ __forceinline__ uint32_t mask_colour_word(const SetDesc &S, const uint32_t *__restrict__ s, const Smem &m,
						     int x, int y, int z)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR;
	int a = -1, idx = 0;
	if (x == R) { a = 0; idx = (z << RB) | y; }
	else if (y == R) { a = 1; idx = (z << RB) | x; }
	else if (z == R) { a = 2; idx = (y << RB) | x; }
	if (a < 0) {
		const int row = (z << RB) | y;
		const uint64_t bits = m.rs[row] & (~0ull >> (63 - x));
		return __ldg(s + (m.rank[row] + __popcll(bits) - 1u));
	}
	const int32_t nc = m.nbr[nbr_slot(a == 0, a == 1, a == 2)];
	if (nc < 0) return 0u;
	return (uint32_t)S.shell_col[(size_t)nc * G::shell_cols + (size_t)a * RR + idx] << 24;
}

static __device__ __forceinline__ void store_splat(int16_t *dst, uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
	uint2 v;
	v.x = (x & 0xFFFFu) | ((y & 0xFFFFu) << 16);
	v.y = (z & 0xFFFFu) | ((w & 0xFFFFu) << 16);
	*(uint2 *)dst = v;
}

/* Position of the k-th (0-based) set bit of v. */
__device__ __forceinline__ int select_bit(uint64_t v, int k)
{
	int pos = 0;
	uint32_t w = (uint32_t)v;
	int c = __popc(w);
	if (k >= c) {
		k -= c;
		w = (uint32_t)(v >> 32);
		pos = 32;
	}
	c = __popc(w & 0xFFFFu);
	if (k >= c) { k -= c; w >>= 16; pos += 16; }
	c = __popc(w & 0xFFu);
	if (k >= c) { k -= c; w >>= 8; pos += 8; }
	c = __popc(w & 0xFu);
	if (k >= c) { k -= c; w >>= 4; pos += 4; }
	c = __popc(w & 0x3u);
	if (k >= c) { k -= c; w >>= 2; pos += 2; }
	c = (int)(w & 1u);
	if (k >= c) pos += 1;
	return pos;
}

/* For item j of a warp's group, the lane s (largest with excl[s] <= j) whose
 * row holds it. All lanes must call it. */
__device__ __forceinline__ int search_lane(uint32_t excl, uint32_t j)
{
	int s = 0;
#pragma unroll
	for (int step = 16; step; step >>= 1) {
		const uint32_t o = __shfl_sync(kFull, excl, s + step);
		if (o <= j) s += step;
	}
	return s;
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src)
{
	const uint32_t lo = __shfl_sync(kFull, (uint32_t)v, src);
	const uint32_t hi = __shfl_sync(kFull, (uint32_t)(v >> 32), src);
	return ((uint64_t)hi << 32) | lo;
}

/* Quad vertex offsets per visible face axis (lutv, src/chunkset/mesher.c:
 * 19-33) packed three bits (x, y, z) per vertex, four vertices per axis:
 *   axis 0: (1,0,0) (1,0,1) (1,1,1) (1,1,0)
 *   axis 1: (0,1,0) (1,1,0) (1,1,1) (0,1,1)
 *   axis 2: (1,0,1) (0,0,1) (0,1,1) (1,1,1)
 * and the index pattern (luti, src/chunkset/mesher.c:53-66) packed two bits
 * per index, one six-index sequence per (normal, rotate):
 *   0,3,1,2,1,3 | 3,2,0,1,0,2 | 1,3,0,3,1,2 | 0,2,3,2,0,1
 * Held in registers, so lanes with different axes never serialise on a
 * constant-memory lookup. */
__device__ __forceinline__ uint32_t quad_offsets(int i)
{
	constexpr uint32_t a0 = 1u | (5u << 3) | (7u << 6) | (3u << 9);
	constexpr uint32_t a1 = 2u | (3u << 3) | (7u << 6) | (6u << 9);
	constexpr uint32_t a2 = 5u | (4u << 3) | (6u << 6) | (7u << 9);
	return i == 0 ? a0 : (i == 1 ? a1 : a2);
}

__device__ __forceinline__ uint32_t quad_indices(int normal, int rotate)
{
	constexpr uint32_t q0 = 0u | (3u << 2) | (1u << 4) | (2u << 6) | (1u << 8) | (3u << 10);
	constexpr uint32_t q1 = 3u | (2u << 2) | (0u << 4) | (1u << 6) | (0u << 8) | (2u << 10);
	constexpr uint32_t q2 = 1u | (3u << 2) | (0u << 4) | (3u << 6) | (1u << 8) | (2u << 10);
	constexpr uint32_t q3 = 0u | (2u << 2) | (3u << 4) | (2u << 6) | (0u << 8) | (1u << 10);
	return normal ? (rotate ? q3 : q2) : (rotate ? q1 : q0);
}

/* Voxel access of one decoded chunk for the mesher: occupancy anywhere in
 * [-1, R]^3, the colour of a solid voxel of the chunk, and the colour of an
 * L0 mask cell (own voxel, or the +neighbour's at coordinate R). */
template <int RB>
struct SmallAcc {
	const SetDesc &S;
	const uint32_t *__restrict__ stream;
	const Smem &m;
	__device__ __forceinline__ uint32_t occ(int x, int y, int z) const { return occ_at<RB>(m, x, y, z); }
	__device__ __forceinline__ uint32_t mcolour(int x, int y, int z) const
	{
		return mask_colour<RB>(S, stream, m, x, y, z);
	}
};

/* One face: AO from the 8 samples around the air voxel, shadow / diamond
 * from the shadow map, 4 vertices and 6 indices (src/chunkset/mesher.c:
 * 236-349). Voxel A = (x, y, z), B = A + e_i; AIR is the air one, BLK the
 * solid one. */
template <int RB, class Acc>
__device__ __forceinline__ void emit_face(const Acc &A, const SetDesc &S, const uint32_t cv[3], int x, int y, int z,
					  int i, uint32_t ordinal, int16_t *vbo, uint32_t *ibo)
{
	const int nx = x + (i == 0), ny = y + (i == 1), nz = z + (i == 2);
	const uint32_t a_solid = A.occ(x, y, z);
	/* the solid voxel's colour: A's (inside the chunk), or B's (possibly
	 * on a + boundary plane, from the neighbour's shell): one lookup path */
	const uint32_t colour = a_solid ? A.mcolour(x, y, z) : A.mcolour(nx, ny, nz);
	const int normal = a_solid ? 0 : 1;
	const int ax = a_solid ? nx : x, ay = a_solid ? ny : y, az = a_solid ? nz : z;
	const int bx = a_solid ? x : nx, by = a_solid ? y : ny, bz = a_solid ? z : nz;
	/* the two axes other than i: u = y for i = 0 else x; v = y for i = 2
	 * else z */
	const int ux = i != 0, uy = i == 0, vy = i == 2, vz = i != 2;
#define OCC3(dU, dV) A.occ(ax + (dU) * ux, ay + (dU) * uy + (dV) * vy, az + (dV) * vz)
	const uint32_t an0 = OCC3(-1, 0), an2 = OCC3(1, 0), an1 = OCC3(0, -1), an3 = OCC3(0, 1);
	const uint32_t ac0 = OCC3(-1, -1), ac1 = OCC3(1, -1), ac2 = OCC3(1, 1), ac3 = OCC3(-1, 1);
#undef OCC3
	const uint32_t e0 = (an0 + an1) | ac0, e1 = (an1 + an2) | ac1;
	const uint32_t e2 = (an2 + an3) | ac2, e3 = (an3 + an0) | ac3;
	uint32_t va0, va1, va2, va3;
	if (i == 0) {
		va0 = e0; va3 = e1; va2 = e2; va1 = e3;
	} else if (i == 1) {
		va0 = e0; va1 = e1; va2 = e2; va3 = e3;
	} else {
		va1 = e0; va0 = e1; va3 = e2; va2 = e3;
	}
	const int rotate = (va0 + va2 < va1 + va3) ? 1 : 0;
	uint32_t wsx = (cv[0] << RB) + (uint32_t)bx;
	uint32_t wsy = (cv[1] << RB) + (uint32_t)by;
	uint32_t wsz = (cv[2] << RB) + (uint32_t)bz;
	/* The shadow samples, one path for every lane (uint32 index arithmetic
	 * as shadow_sample / shadow_sample_normal, src/chunkset/shadow.h:45-75):
	 * the three map entries around b are read, then combined per case.
	 *   i = 0, B air:   shadow_sample_normal(ws): b, b - 1, lim = wsy + 1
	 *   i = 1, A air:   shadow_sample(ws):        b, b + 1, lim = wsy + 1
	 *   i = 2 (diamond, z = wsz - normal + 1 when B is air):
	 *                   !shadow_sample(wsx, wsy, z):     b, b + 1, lim = wsy + 1
	 *                   !shadow_sample(wsx, wsy - 1, z): b - 1, b, lim = wsy
	 * A lim of 0 reads as shadowed, as the reference's early return. */
	const uint32_t zq = i == 2 ? wsz - (uint32_t)normal + (a_solid ? 1u : 0u) : wsz;
	const uint32_t b = (wsx + wsy) + S.shadow_w * zq;
	const uint32_t vm = shadow_at(S, b - 1u), v0 = shadow_at(S, b), vp = shadow_at(S, b + 1u);
	const uint32_t lim = wsy + 1u;
	uint32_t shadow = 0, diamond = 3;
	if (i == 0 && normal) shadow = !((v0 < lim) & (vm < lim));
	if (i == 1 && !normal) shadow = !((v0 < lim) & (vp < lim));
	if (i == 2) diamond = ((uint32_t)((v0 < lim) & (vp < lim)) << 1) | (uint32_t)((vm < wsy) & (v0 < wsy));
	if (i == 0) wsx -= (uint32_t)normal;
	else if (i == 1) wsy -= (uint32_t)normal;
	else wsz -= (uint32_t)normal;
	const uint32_t qo = quad_offsets(i);
	const uint32_t word0 = colour | ((uint32_t)(i + 3 * normal) << 8) | (shadow << 13) | (diamond << 14);
	uint32_t out[8];
	const uint32_t va[4] = {va0, va1, va2, va3};
#pragma unroll
	for (int vert = 0; vert < 4; vert++) {
		const uint32_t o = qo >> (3 * vert);
		const uint32_t px = (wsx + (o & 1u)) & 0xFFFFu;
		const uint32_t py = (wsy + ((o >> 1) & 1u)) & 0xFFFFu;
		const uint32_t pz = (wsz + ((o >> 2) & 1u)) & 0xFFFFu;
		const uint32_t word = (word0 | (va[vert] << 6) | ((uint32_t)vert << 11)) & 0xFFFFu;
		out[2 * vert] = px | (py << 16);
		out[2 * vert + 1] = pz | (word << 16);
	}
	uint4 *vd = (uint4 *)(vbo + (size_t)ordinal * 16);
	vd[0] = make_uint4(out[0], out[1], out[2], out[3]);
	vd[1] = make_uint4(out[4], out[5], out[6], out[7]);
	const uint32_t vb = ordinal * 4u;
	const uint32_t qi = quad_indices(normal, rotate);
	uint2 *id = (uint2 *)(ibo + (size_t)ordinal * 6);
	id[0] = make_uint2(vb + (qi & 3u), vb + ((qi >> 2) & 3u));
	id[1] = make_uint2(vb + ((qi >> 4) & 3u), vb + ((qi >> 6) & 3u));
	id[2] = make_uint2(vb + ((qi >> 8) & 3u), vb + ((qi >> 10) & 3u));
}

/* Face bits of row (y, z): bit x of f[i] = face between (x,y,z) and its
 * +axis-i neighbour (exactly one of them solid). */
template <int RB>
__device__ __forceinline__ void face_bits(const Smem &m, int y, int z, uint64_t &fx, uint64_t &fy, uint64_t &fz)
{
	using G = Geo<RB>;
	constexpr int R = G::R;
	const uint64_t o = m.occ[hidx<RB>(y, z)];
	fx = (o ^ ((o >> 1) | (xhi_bit<RB>(m, y, z) << (R - 1)))) & G::MASK;
	fy = o ^ m.occ[hidx<RB>(y + 1, z)];
	fz = o ^ m.occ[hidx<RB>(y, z + 1)];
}

/* (x, axis) of the k-th face of a row, faces ordered by x then axis. The
 * count of faces at each x, fx + fy + fz, is held as two bit planes (its
 * low bit and whether it is >= 2), so a prefix count is two popcounts; the
 * search takes the 32-bit half first, then halves within it. */
template <int RB>
__device__ __forceinline__ void select_face(uint64_t fx, uint64_t fy, uint64_t fz, uint32_t k, int &x, int &i)
{
	const uint64_t fxy = fx ^ fy;
	const uint64_t lo = fxy ^ fz, hi = (fx & fy) | (fz & fxy);
	uint32_t l32 = (uint32_t)lo, h32 = (uint32_t)hi;
	int pos = 0;
	const uint32_t c32 = __popc(l32) + 2u * __popc(h32);
	if (c32 <= k) {
		k -= c32;
		pos = 32;
		l32 = (uint32_t)(lo >> 32);
		h32 = (uint32_t)(hi >> 32);
	}
#pragma unroll
	for (int step = 16; step; step >>= 1) {
		const uint32_t below = (1u << step) - 1u;
		const uint32_t c = __popc(l32 & below) + 2u * __popc(h32 & below);
		if (c <= k) {
			k -= c;
			pos += step;
			l32 >>= step;
			h32 >>= step;
		}
	}
	const uint32_t b0 = (uint32_t)((fx >> pos) & 1ull), b1 = (uint32_t)((fy >> pos) & 1ull);
	x = pos;
	if (b0) {
		if (k == 0) { i = 0; return; }
		k--;
	}
	if (b1) {
		if (k == 0) { i = 1; return; }
	}
	i = 2;
}

/* Exclusive scan, in place, of n <= 32*8 group counts by warp 0; returns
 * the total to all threads. */
/* Exclusive scan of the n group counts in place; returns the total. With a
 * list, also writes the indices of the non-empty groups there, in order,
 * and their number to tmp[1]. */
__device__ __forceinline__ uint32_t scan_groups(uint32_t *g, int n, uint32_t *tmp, uint16_t *list = nullptr)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (warp == 0) {
		uint32_t carry = 0, listed = 0;
		for (int b = 0; b < n; b += 32) {
			const int i = b + lane;
			const uint32_t v = i < n ? g[i] : 0u;
			const uint32_t inc = warp_incl_add(v);
			if (i < n) g[i] = carry + inc - v;
			carry += __shfl_sync(kFull, inc, 31);
			if (list) {
				const uint32_t ne = __ballot_sync(kFull, v != 0u);
				if (v) list[listed + __popc(ne & ((1u << lane) - 1u))] = (uint16_t)i;
				listed += __popc(ne);
			}
		}
		if (lane == 0) {
			tmp[0] = carry;
			tmp[1] = listed;
		}
	}
	__syncthreads();
	const uint32_t t = tmp[0];
	__syncthreads();
	return t;
}

template <int RB>
__device__ void mesh_chunk(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m, const uint32_t cv[3],
			   ChunkOut *out, const Arena &avbo, const Arena &aibo)
{
	using G = Geo<RB>;
	constexpr int R = G::R, RR = G::RR, NG = (RR + 63) / 64; /* 64-row groups, two rows a lane */
	__shared__ unsigned long long s_base[2];
	__shared__ uint32_t s_ok, s_next;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	/* pass 1: faces per 64-row group */
	for (int g = warp; g < NG; g += nw) {
		uint32_t c = 0;
#pragma unroll
		for (int h = 0; h < 2; h++) {
			const int r = g * 64 + 2 * lane + h;
			if (r < RR) {
				uint64_t fx, fy, fz;
				face_bits<RB>(m, r & (R - 1), r >> RB, fx, fy, fz);
				c += __popcll(fx) + __popcll(fy) + __popcll(fz);
			}
		}
		c = __reduce_add_sync(kFull, c);
		if (lane == 0) m.grp[g] = c;
	}
	__syncthreads();
	const uint32_t faces = scan_groups(m.grp, NG, m.tmp, m.glist);
	const uint32_t listed = m.tmp[1];
	if (threadIdx.x == 0) {
		const uint64_t uv = (uint64_t)faces * 2u;             /* 32 B per face */
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
	const SmallAcc<RB> acc{S, stream, m};
	/* pass 2: warps take the non-empty groups from a shared counter; lane s
	 * holds the face counts of rows 2s and 2s + 1, and the lane that emits
	 * a face recomputes its row's three face words (cheaper than shuffling
	 * six words a step); one face per lane per step (a second face per
	 * step, with both searches first, measured slower) */
	for (;;) {
		uint32_t t = 0;
		if (lane == 0) t = atomicAdd(&s_next, 1u);
		t = __shfl_sync(kFull, t, 0);
		if (t >= listed) break;
		const uint32_t g = m.glist[t];
		const int r0 = (int)g * 64 + 2 * lane;
		uint32_t ca = 0, cb = 0;
		if (r0 < RR) {
			uint64_t fx, fy, fz;
			face_bits<RB>(m, r0 & (R - 1), r0 >> RB, fx, fy, fz);
			ca = __popcll(fx) + __popcll(fy) + __popcll(fz);
		}
		if (r0 + 1 < RR) {
			uint64_t fx, fy, fz;
			face_bits<RB>(m, (r0 + 1) & (R - 1), (r0 + 1) >> RB, fx, fy, fz);
			cb = __popcll(fx) + __popcll(fy) + __popcll(fz);
		}
		const uint32_t c = ca + cb;
		const uint32_t inc = warp_incl_add(c);
		const uint32_t excl = inc - c;
		const uint32_t T = __shfl_sync(kFull, inc, 31);
		const uint32_t base = m.grp[g];
		for (uint32_t k = 0; k < T; k += 32) {
			const uint32_t j0 = k + lane;
			const int s0 = search_lane(excl, j0);
			const uint32_t e0 = __shfl_sync(kFull, excl, s0), a0 = __shfl_sync(kFull, ca, s0);
			if (j0 < T) {
				uint32_t kk = j0 - e0;
				const bool second = kk >= a0;
				kk -= second ? a0 : 0u;
				const int rr = (int)g * 64 + 2 * s0 + (second ? 1 : 0);
				uint64_t ax, ay, az;
				face_bits<RB>(m, rr & (R - 1), rr >> RB, ax, ay, az);
				int x, i;
				select_face<RB>(ax, ay, az, kk, x, i);
				emit_face<RB>(acc, S, cv, x, rr & (R - 1), rr >> RB, i, base + j0, vbo, ibo);
			}
		}
	}
}

/* One level-l splat: walk down to the L0 cell whose colour the reference's
 * last-writer-wins downsample keeps (the nonzero child with the largest
 * (z, y, x) at every level, src/chunkset/mesher.c:474-489), then emit
 * {x, y, z, colour | shadow << 6} (src/chunkset/mesher.c:521-531). At each
 * level the eight child bits form a pattern indexed dx + 2 dy + 4 dz, and
 * the chosen child is its highest set bit. */
template <int RB, int L>
__device__ __forceinline__ void emit_splat(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m,
					   const uint32_t cv[3], int x, int y, int z, int16_t *dst, bool sh_in)
{
	constexpr int R = Geo<RB>::R;
	int cx = x, cy = y, cz = z;
#pragma unroll
	for (int lc = L - 1; lc >= 0; lc--) {
		const int np = (R >> lc) + 1;
		const int X = 2 * cx;
		uint32_t pat = 0;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int Y = 2 * cy + (q & 1), Z = 2 * cz + (q >> 1);
			if (Y < np && Z < np) {
				uint32_t xr;
				const uint64_t row = level_row<RB>(m, lc, Y, Z, xr);
				/* X is even and R even: X + 1 never equals R */
				const uint32_t b2 = (lc == 0 && X == R) ? xr : (uint32_t)((row >> X) & 3ull);
				pat |= b2 << (2 * q);
			}
		}
		const int best = pat ? 31 - __clz(pat) : 0;
		cx = X + (best & 1);
		cy = 2 * cy + ((best >> 1) & 1);
		cz = 2 * cz + (best >> 2);
	}
	const uint32_t colour = mask_colour<RB>(S, stream, m, cx, cy, cz);
	constexpr uint32_t sh = L ? (1u << L) : 0u;
	const uint32_t wx = (cv[0] << RB) + ((uint32_t)x << L);
	const uint32_t wy = (cv[1] << RB) + ((uint32_t)y << L);
	const uint32_t wz = (cv[2] << RB) + ((uint32_t)z << L);
	uint32_t shadow;
	if (sh_in) {
		/* the chunk's whole sample window lies inside the map: no bounds
		 * checks (shadow_sample, src/chunkset/shadow.h:45-63) */
		const uint32_t lim = wy + sh + 1u;
		const uint16_t *p = S.shadow + (((uint64_t)((wx + sh) + (wy + sh)) + (uint64_t)S.shadow_w * (wz + sh)) -
						S.shadow_base);
		shadow = !((__ldg(p) < lim) & (__ldg(p + 1) < lim));
	} else {
		shadow = (uint32_t)shadow_sample(S, wx + sh, wy + sh, wz + sh);
	}
	store_splat(dst, wx, wy, wz, colour | (shadow << 6));
}

/* emit_splat in two halves for the pipelined level-0 loop: splat_issue
 * walks down, issues the colour and shadow loads and stores the splat's x
 * and y; splat_finish, one step later, stores z and colour | shadow << 6
 * from the loaded values. */
struct SplatPend {
	uint32_t vz, c, a, b, lim;
};

template <int RB, int L>
__device__ __forceinline__ void splat_issue(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m,
					    const uint32_t cv[3], int x, int y, int z, bool sh_in, int16_t *dst, SplatPend &p)
{
	constexpr int R = Geo<RB>::R;
	int cx = x, cy = y, cz = z;
#pragma unroll
	for (int lc = L - 1; lc >= 0; lc--) {
		const int np = (R >> lc) + 1;
		const int X = 2 * cx;
		uint32_t pat = 0;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int Y = 2 * cy + (q & 1), Z = 2 * cz + (q >> 1);
			if (Y < np && Z < np) {
				uint32_t xr;
				const uint64_t row = level_row<RB>(m, lc, Y, Z, xr);
				const uint32_t b2 = (lc == 0 && X == R) ? xr : (uint32_t)((row >> X) & 3ull);
				pat |= b2 << (2 * q);
			}
		}
		const int best = pat ? 31 - __clz(pat) : 0;
		cx = X + (best & 1);
		cy = 2 * cy + ((best >> 1) & 1);
		cz = 2 * cz + (best >> 2);
	}
	p.c = mask_colour_word<RB>(S, stream, m, cx, cy, cz);
	constexpr uint32_t sh = L ? (1u << L) : 0u;
	const uint32_t wx = (cv[0] << RB) + ((uint32_t)x << L);
	const uint32_t wy = (cv[1] << RB) + ((uint32_t)y << L);
	const uint32_t wz = (cv[2] << RB) + ((uint32_t)z << L);
	*(uint32_t *)dst = (wx & 0xFFFFu) | ((wy & 0xFFFFu) << 16); /* x, y now; z and w in splat_finish */
	p.vz = wz & 0xFFFFu;
	p.lim = wy + sh + 1u; /* 0 after a wrap: nothing is < 0, the splat is shadowed */
	if (sh_in) {
		const uint16_t *q = S.shadow + (((uint64_t)((wx + sh) + (wy + sh)) + (uint64_t)S.shadow_w * (wz + sh)) -
						S.shadow_base);
		p.a = __ldg(q);
		p.b = __ldg(q + 1);
	} else {
		const uint32_t idx = ((wx + sh) + (wy + sh)) + S.shadow_w * (wz + sh);
		p.a = shadow_at(S, idx);
		p.b = shadow_at(S, idx + 1u);
	}
}

__device__ __forceinline__ void splat_finish(int16_t *dst, const SplatPend &p)
{
	const uint32_t shadow = !((p.a < p.lim) & (p.b < p.lim));
	((uint32_t *)dst)[1] = p.vz | (((p.c >> 24) | (shadow << 6)) << 16);
}

/* Whether every shadow sample of a chunk's splats (world coordinates up to
 * its far corner plus 2^lod_max, and the entry after) falls inside the map
 * and needs no uint32 wrap. */
template <int RB>
__device__ __forceinline__ bool shadow_window_inside(const SetDesc &S, const uint32_t cv[3], int lod_max)
{
	const uint64_t ext = (1u << RB) + (1u << lod_max);
	const uint64_t x0 = (uint64_t)cv[0] << RB, y0 = (uint64_t)cv[1] << RB, z0 = (uint64_t)cv[2] << RB;
	const uint64_t lo = x0 + y0 + (uint64_t)S.shadow_w * z0;
	const uint64_t hi = (x0 + ext) + (y0 + ext) + (uint64_t)S.shadow_w * (z0 + ext) + 1u;
	return hi < (1ull << 32) && lo >= S.shadow_base && hi - S.shadow_base < S.shadow_len;
}

static_assert(kMaxLevels == 8, "the level switches have one case per level");

/* Level of emission group g (one table read; warp-uniform g). */
template <int RB>
__device__ __forceinline__ int group_level(int g)
{
	return c_lv.glevel[RB][g];
}

/* Level-L rows (L >= 1): the pairwise OR of the four child rows of level
 * L - 1, compacted along x (src/chunkset/mesher.c:460-493 as occupancy). */
template <int RB, int L>
__device__ __forceinline__ void build_level(const Smem &m)
{
	constexpr int R = Geo<RB>::R;
	constexpr uint32_t n = (uint32_t)(R >> L) + 1u, np = (uint32_t)(R >> (L - 1)) + 1u;
	uint64_t *dst = m.lv + c_lv.off[RB][L];
	const uint32_t lane = threadIdx.x & 31u;
	/* warp-aligned: the 32 rows a warp writes are one emission group, whose
	 * item count it records on the way (no separate count pass) */
	for (uint32_t base = threadIdx.x & ~31u; base < n * n; base += blockDim.x) {
		const uint32_t i = base + lane;
		uint64_t row = 0;
		if (i < n * n) {
			const uint32_t z = i / n, y = i - z * n;
			uint64_t acc = 0;
			uint32_t accx = 0;
#pragma unroll
			for (uint32_t dz = 0; dz < 2; dz++)
#pragma unroll
				for (uint32_t dy = 0; dy < 2; dy++) {
					const uint32_t yy = 2 * y + dy, zz = 2 * z + dz;
					if (yy >= np || zz >= np) continue;
					uint32_t xr;
					acc |= level_row<RB>(m, L - 1, (int)yy, (int)zz, xr);
					accx |= xr;
				}
			row = compress_pairs(acc);
			if (L == 1) row |= (uint64_t)accx << (R / 2);
			dst[i] = row;
		}
		const uint32_t c = __reduce_add_sync(kFull, (uint32_t)__popcll(row));
		if (lane == 0) m.grp[c_lv.gstart[RB][L] + base / 32u] = c;
	}
}

/* Cells of group g of level L (all lanes call; every lane gets it). Used
 * for level 0, whose rows come from several sources; build_level counts
 * the groups of the levels above as it writes their rows. */
template <int RB, int L>
__device__ __forceinline__ uint32_t count_group(const Smem &m, int g)
{
	constexpr int R = Geo<RB>::R;
	constexpr uint32_t n = (uint32_t)(R >> L) + 1u;
	constexpr uint32_t rows = (uint32_t)group_rows(RB, L), per_lane = rows / 32u;
	const uint32_t r0 = (uint32_t)(g - c_lv.gstart[RB][L]) * rows + (threadIdx.x & 31u) * per_lane;
	uint32_t c = 0;
#pragma unroll
	for (uint32_t i = 0; i < per_lane; i++) {
		const uint32_t r = r0 + i;
		if (r < n * n) {
			const uint32_t z = r / n, y = r - z * n;
			uint32_t xr;
			c += __popcll(level_row<RB>(m, L, (int)y, (int)z, xr)) + xr;
		}
	}
	return __reduce_add_sync(kFull, c);
}

/* Pass 2 of one non-empty 32-row group of level L >= 1: lane s holds row s
 * and its exclusive item offset; items go one per lane per step (two per
 * step, both searches first, measured 4 % slower: more registers live
 * across the loads). Specialised per level, so the row division, the walk
 * down and the shifts are compile-time. */
template <int RB, int L>
__device__ __forceinline__ void splat_group(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m,
					    const uint32_t cv[3], int g, int16_t *dst, bool sh_in)
{
	static_assert(L >= 1, "level 0 has splat_group_l0");
	constexpr int R = Geo<RB>::R;
	constexpr uint32_t n = (uint32_t)(R >> L) + 1u;
	const int lane = threadIdx.x & 31;
	const uint32_t r = (uint32_t)(g - c_lv.gstart[RB][L]) * 32u + (uint32_t)lane;
	uint64_t row = 0;
	uint32_t xr = 0, yz = 0;
	if (r < n * n) {
		const uint32_t z = r / n, y = r - z * n;
		row = level_row<RB>(m, L, (int)y, (int)z, xr);
		yz = y | (z << 16);
	}
	const uint32_t c = __popcll(row) + xr;
	const uint32_t inc = warp_incl_add(c);
	const uint32_t excl = inc - c;
	const uint32_t T = __shfl_sync(kFull, inc, 31);
	const uint32_t base = m.grp[g];
	for (uint32_t k = 0; k < T; k += 32) {
		const uint32_t j0 = k + lane;
		const int s0 = search_lane(excl, j0);
		const uint32_t e0 = __shfl_sync(kFull, excl, s0), q0 = __shfl_sync(kFull, yz, s0);
		const uint64_t w0 = shfl64(row, s0);
		if (j0 < T) {
			const int kk = (int)(j0 - e0);
			const int x = kk < __popcll(w0) ? select_bit(w0, kk) : R;
			emit_splat<RB, L>(S, stream, m, cv, x, (int)(q0 & 0xFFFFu), (int)(q0 >> 16),
					  dst + (size_t)(base + j0) * 4, sh_in);
		}
	}
}

/* Pass 2 of one non-empty 96-row level-0 group (three quarters of the
 * splats): lane s holds rows 3s .. 3s + 2, consecutive in the item order,
 * and their exclusive item offset. An item's row follows from the first two
 * rows' counts, its (y, z) from the row index. The loop is
 * software-pipelined: a step's colour and shadow loads are issued, and
 * consumed one step later, after the next step's search and select. */
template <int RB>
__device__ __forceinline__ void splat_group_l0(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m,
					       const uint32_t cv[3], int g, int16_t *dst, bool sh_in)
{
	constexpr int R = Geo<RB>::R;
	constexpr uint32_t n = (uint32_t)R + 1u;
	const int lane = threadIdx.x & 31;
	static_assert(group_rows(RB, 0) == 96, "level-0 groups of three rows a lane");
	const uint32_t rbase = (uint32_t)(g - c_lv.gstart[RB][0]) * 96u;
	const uint32_t r0 = rbase + 3u * (uint32_t)lane;
	uint64_t ra = 0, rb = 0, rc = 0;
	uint32_t ca = 0, cb = 0, cc = 0;
	if (r0 < n * n) {
		const uint32_t z = r0 / n, y = r0 - z * n;
		uint32_t xr;
		ra = e0_row<RB>(m, (int)y, (int)z, xr);
		ca = __popcll(ra) + xr;
	}
	if (r0 + 1u < n * n) {
		const uint32_t z = (r0 + 1u) / n, y = (r0 + 1u) - z * n;
		uint32_t xr;
		rb = e0_row<RB>(m, (int)y, (int)z, xr);
		cb = __popcll(rb) + xr;
	}
	if (r0 + 2u < n * n) {
		const uint32_t z = (r0 + 2u) / n, y = (r0 + 2u) - z * n;
		uint32_t xr;
		rc = e0_row<RB>(m, (int)y, (int)z, xr);
		cc = __popcll(rc) + xr;
	}
	const uint32_t c = ca + cb + cc;
	const uint32_t inc = warp_incl_add(c);
	const uint32_t excl = inc - c;
	const uint32_t T = __shfl_sync(kFull, inc, 31);
	const uint32_t base = m.grp[g];
	const uint32_t cab = ca | (cb << 8); /* row counts are at most R + 1 */
	SplatPend pend;
	bool pv = false;
	uint32_t pj = 0;
	for (uint32_t k = 0; k < T; k += 32) {
		const uint32_t j0 = k + lane;
		const int s0 = search_lane(excl, j0);
		const uint32_t e0 = __shfl_sync(kFull, excl, s0), p0 = __shfl_sync(kFull, cab, s0);
		const uint64_t wa = shfl64(ra, s0), wb = shfl64(rb, s0), wc = shfl64(rc, s0);
		const bool v = j0 < T;
		int x = 0, y = 0, z = 0;
		if (v) {
			int kk = (int)(j0 - e0);
			const int a0 = (int)(p0 & 0xFFu), b0 = (int)(p0 >> 8);
			uint32_t i = 0;
			uint64_t w = wa;
			if (kk >= a0) {
				kk -= a0;
				i = 1;
				w = wb;
				if (kk >= b0) {
					kk -= b0;
					i = 2;
					w = wc;
				}
			}
			/* the x = R cell is its row's last item */
			x = kk < __popcll(w) ? select_bit(w, kk) : R;
			const uint32_t r = rbase + 3u * (uint32_t)s0 + i;
			z = (int)(r / n);
			y = (int)(r - (uint32_t)z * n);
		}
		/* the previous step's loads had the search and select to land */
		if (pv) splat_finish(dst + (size_t)(base + pj) * 4, pend);
		if (v) splat_issue<RB, 0>(S, stream, m, cv, x, y, z, sh_in, dst + (size_t)(base + j0) * 4, pend);
		pv = v;
		pj = j0;
	}
	if (pv) splat_finish(dst + (size_t)(base + pj) * 4, pend);
}

template <int RB>
__device__ void splat_chunk(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m, const uint32_t cv[3],
			    int lod_max, ChunkOut *out, const Arena &asvl)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	__shared__ unsigned long long s_base;
	__shared__ uint32_t s_ok, s_next;
	const int *gstart = c_lv.gstart[RB];
	splat_prepare<RB>(m);
	/* level rows: pairwise OR of the child rows, compacted along x */
	for (int l = 1; l <= lod_max; l++) {
		switch (l) {
		case 1: build_level<RB, 1>(m); break;
		case 2: build_level<RB, 2>(m); break;
		case 3: build_level<RB, 3>(m); break;
		case 4: build_level<RB, 4>(m); break;
		case 5: build_level<RB, 5>(m); break;
		case 6: build_level<RB, 6>(m); break;
		default: build_level<RB, 7>(m); break;
		}
		__syncthreads();
	}
	/* pass 1: splats per group; the level rows' groups were counted
	 * as they were built, level 0's are counted here */
	const int ngroups = gstart[lod_max + 1];
	for (int g = warp; g < gstart[1]; g += nw) {
		const uint32_t c = count_group<RB, 0>(m, g);
		if (lane == 0) m.grp[g] = c;
	}
	__syncthreads();
	const uint32_t total = scan_groups(m.grp, ngroups, m.tmp, m.glist);
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
	const bool sh_in = shadow_window_inside<RB>(S, cv, lod_max);
	/* pass 2: warps take the non-empty groups from a shared counter */
	for (;;) {
		uint32_t k = 0;
		if (lane == 0) k = atomicAdd(&s_next, 1u);
		k = __shfl_sync(kFull, k, 0);
		if (k >= listed) break;
		const int g = m.glist[k];
		switch (group_level<RB>(g)) {
		case 0: splat_group_l0<RB>(S, stream, m, cv, g, dst, sh_in); break;
		case 1: splat_group<RB, 1>(S, stream, m, cv, g, dst, sh_in); break;
		case 2: splat_group<RB, 2>(S, stream, m, cv, g, dst, sh_in); break;
		case 3: splat_group<RB, 3>(S, stream, m, cv, g, dst, sh_in); break;
		case 4: splat_group<RB, 4>(S, stream, m, cv, g, dst, sh_in); break;
		case 5: splat_group<RB, 5>(S, stream, m, cv, g, dst, sh_in); break;
		case 6: splat_group<RB, 6>(S, stream, m, cv, g, dst, sh_in); break;
		default: splat_group<RB, 7>(S, stream, m, cv, g, dst, sh_in); break;
		}
	}
}

/* The L0 mask of chunk_make_mask (src/chunkset/mesher.c:377-456) as a dense
 * (R+1)^3 byte array: every mask cell gets its colour; other cells keep
 * what `dst` held (the reference's caller zeroes it). */
template <int RB>
__device__ void mask_dense(const SetDesc &S, const uint32_t *__restrict__ stream, const Smem &m, uint8_t *dst)
{
	using G = Geo<RB>;
	constexpr int R = G::R, S1 = G::S;
	splat_prepare<RB>(m);
	for (int i = threadIdx.x; i < S1 * S1; i += blockDim.x) {
		const int y = i % S1, z = i / S1;
		uint32_t xr;
		const uint64_t row = e0_row<RB>(m, y, z, xr);
		uint8_t *line = dst + ((size_t)z * S1 + y) * S1;
		for (uint64_t b = row; b; b &= b - 1ull) {
			const int x = __ffsll((long long)b) - 1;
			line[x] = (uint8_t)mask_colour<RB>(S, stream, m, x, y, z);
		}
		if (xr) line[R] = (uint8_t)mask_colour<RB>(S, stream, m, R, y, z);
	}
}

/* One work item of a <= 64^3 chunk: neighbours, decode, halo, then mask /
 * mesh / splats. Returns with the block synchronised. */
template <int RB>
__device__ __forceinline__ void geometry_item(const SetDesc &S, const WorkItem &wi, ChunkOut *out, const Smem &m,
					      const Arena &asvl, const Arena &avbo, const Arena &aibo, int lod_max,
					      const uint8_t *decoded = nullptr, const uint32_t *dec_slot = nullptr,
					      uint64_t *bar = nullptr, uint32_t *phase = nullptr, uint32_t *flag = nullptr)
{
	using G = Geo<RB>;
	constexpr int R = G::R;
	uint32_t cv[3], wc[3];
	chunk_coords(S, wi.chunk, cv);
	for (int k = 0; k < 3; k++) wc[k] = (uint32_t)(S.origin[k] + (int32_t)cv[k]);
	const uint32_t N = (uint32_t)R * R * R;
	const bool mesh = (wi.flags & kItemMesh) != 0;
	load_neighbours(S, cv, m.nbr, N);
	/* an all-air chunk whose +neighbours are all air has no geometry */
	const bool empty = m.nbr[nbr_slot(0, 0, 0)] < 0 && m.nbr[nbr_slot(1, 0, 0)] < 0 &&
			   m.nbr[nbr_slot(0, 1, 0)] < 0 && m.nbr[nbr_slot(0, 0, 1)] < 0;
	if (empty && !(wi.flags & kItemMaskDense)) {
		if (threadIdx.x == 0) {
			out->svl_off = out->vbo_off = out->ibo_off = 0;
			for (int l = 0; l < kMaxLevels; l++) out->svl_items[l] = 0;
			out->svl_total = out->vbo_items = out->ibo_items = 0;
			out->status = 0;
		}
		__syncthreads();
		return;
	}
	const uint32_t *stream = S.pool + S.off[wi.chunk];
	/* the shell pass of this rebuild stored every chunk but the all-air ones */
	const uint32_t ds = decoded && !chunk_is_null(S, wi.chunk, N) ? dec_slot[wi.chunk] : kNoSlot;
	if (ds != kNoSlot) {
		if (!load_decoded<RB>(decoded + (size_t)ds * G::dec_bytes, m, bar, *phase, flag)) {
			/* the copies did not arrive: one more bounded wait for them,
			 * then report the chunk; the CTA stops */
			mbar_wait(bar, *phase);
			if (threadIdx.x == 0) out->status = kStatusTimeout;
			__syncthreads();
			return;
		}
		*phase ^= 1u;
	} else {
		decode_chunk<RB>(stream, S.len[wi.chunk] - 1u, m);
	}
	load_halo<RB>(S, m);
	if (wi.flags & kItemMaskDense)
		mask_dense<RB>(S, stream, m, (uint8_t *)asvl.base + (size_t)wi.slot * G::S * G::S * G::S);
	else if (mesh)
		mesh_chunk<RB>(S, stream, m, wc, out, avbo, aibo);
	else
		splat_chunk<RB>(S, stream, m, wc, lod_max, out, asvl);
	__syncthreads();
}

template <int RB>
__global__ void __launch_bounds__(512, 2) k_geometry(const SetDesc *__restrict__ sets, const WorkItem *__restrict__ items,
						     uint32_t nitems, unsigned int *queue, ChunkOut *outs, Arena asvl,
						     Arena avbo, Arena aibo, int lod_max, const uint8_t *decoded,
						     const uint32_t *__restrict__ dec_slot)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const Smem m = carve<RB>(smem);
	__shared__ uint32_t s_item;
	grid_wait(); /* the shell pass's shells and handed-over chunks */
	grid_release();
	__shared__ __align__(8) uint64_t s_bar; /* completion of the decoded-chunk bulk copies */
	__shared__ uint32_t s_flag;             /* a bounded wait ran out */
	uint32_t phase = 0;
	if (threadIdx.x == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_bar)) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		s_flag = 0u;
	}
	__syncthreads();
	uint32_t next = blockIdx.x;
	for (;;) {
		if (threadIdx.x == 0) s_item = queue ? atomicAdd(queue, 1u) : next;
		__syncthreads();
		const uint32_t it = s_item;
		if (it >= nitems || s_flag) {
			/* a CTA stopped by a timed-out wait reports the item it had
			 * just dequeued, which it does not build */
			if (s_flag && threadIdx.x == 0 && it < nitems) outs[items[it].slot].status = kStatusTimeout;
			break;
		}
		next = nitems;
		const WorkItem wi = items[it];
		const SetDesc S = sets[wi.set];
		geometry_item<RB>(S, wi, outs + wi.slot, m, asvl, avbo, aibo, lod_max, decoded, dec_slot, &s_bar, &phase,
				  &s_flag);
	}
}

} // namespace vp

#include "vp_geometry_big.cuh"

namespace vp {


/* Work items of any root size 8..128 in one persistent launch: each item
 * takes the path of its set's root size (the shared-memory carve of its size,
 * or this CTA's scratch slot for 128^3). Shared memory is sized for 64^3. */
template <int MINB>
__global__ void __launch_bounds__(512, MINB) k_geometry_mixed(const SetDesc *__restrict__ sets,
							      const WorkItem *__restrict__ items, uint32_t nitems,
							      unsigned int *queue, ChunkOut *outs, Arena asvl,
							      Arena avbo, Arena aibo, int lod_max, uint8_t *scratch,
							      uint32_t grain)
{
	extern __shared__ __align__(16) uint8_t smem[];
	__shared__ uint32_t s_item;
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
			ChunkOut *out = outs + wi.slot;
			switch (S.root_bitw) {
			case 3: geometry_item<3>(S, wi, out, carve<3>(smem), asvl, avbo, aibo, lod_max); break;
			case 4: geometry_item<4>(S, wi, out, carve<4>(smem), asvl, avbo, aibo, lod_max); break;
			case 5: geometry_item<5>(S, wi, out, carve<5>(smem), asvl, avbo, aibo, lod_max); break;
			case 6: geometry_item<6>(S, wi, out, carve<6>(smem), asvl, avbo, aibo, lod_max); break;
			default: {
				const Smem m6 = carve<6>(smem);
				const BigMem bm = big_carve(scratch, blockIdx.x, m6.tmp, m6.nbr);
				geometry_item_big(S, wi, out, bm, asvl, avbo, aibo, lod_max);
				__syncthreads();
			}
			}
		}
	}
}

/* host-side launch of the <= 64^3 kernels of root 2^RB */
template <int RB>
static cudaError_t launch_rb(const GeoLaunch &L, cudaStream_t st)
{
	using G = Geo<RB>;
	cudaError_t e;
	e = cudaFuncSetAttribute(k_shell<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::bytes);
	if (e != cudaSuccess) return e;
	e = cudaFuncSetAttribute(k_geometry<RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::bytes);
	if (e != cudaSuccess) return e;
	if (L.run_shell && (L.n_shell || L.n_uni)) {
		/* the decoded chunks, then the single-run ones a warp each */
		const uint32_t warps = (uint32_t)L.threads / 32u;
		const uint32_t grid = L.n_shell + (L.n_uni + warps - 1u) / warps;
		k_shell<RB><<<grid, L.threads, G::bytes, st>>>(L.sets, L.shell_items, L.n_shell, L.decoded, L.dec_slot,
							       L.uni_items, L.n_uni, L.outs);
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	if (L.n_items) {
		const uint32_t grid = L.queue ? L.ctas : L.n_items;
		e = launch_dependent(k_geometry<RB>, dim3(grid), dim3(L.threads), G::bytes, st, L.sets, L.items,
				     L.n_items, L.queue, L.outs, L.svl, L.vbo, L.ibo, L.lod_max, L.decoded, L.dec_slot);
		if (e != cudaSuccess) return e;
		e = cudaGetLastError();
	}
	return e;
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

} // namespace vp
