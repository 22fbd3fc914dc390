/*
 * vp_io.cu — the RLE world file / wire format (host code).
 *
 * The reference keeps its world only in memory (per-chunk u32 streams,
 * src/chunkset/rle.c:14-22, in ChunkMD.rle). A file holds exactly that:
 *
 *   offset  size          field
 *   0       4             magic 0x31575056 ("VPW1", little endian)
 *   4       4             version (1)
 *   8       4             root_bitw
 *   12      12            max_bitw[3]
 *   24      4             nchunks = 2^(max_bitw sum)
 *   28      4             shadow_w (world X + Y)
 *   32      8             pool_words
 *   40      8             shadow_len (elements, padded rows included)
 *   48      4             pad_rows
 *   52      12            reserved (0)
 *   64      8 * nchunks   off[c]   word offset of chunk c's stream in the pool
 *   ..      4 * nchunks   len[c]   words incl. the 0 terminator
 *   ..      4 * pool_words         the streams, each on a 16-byte boundary
 *   ..      2 * shadow_len         the u16 shadow map
 *
 * Everything is little endian. Streams are written packed (in chunk order,
 * each padded to 4 words), so a file is also the upload layout.
 */
#include "voxgpu.h"
#include "vp_internal.h"

#include <cstdio>
#include <cstring>
#include <vector>

namespace {

struct FileHeader {
	uint32_t magic, version;
	int32_t root_bitw, max_bitw[3];
	uint32_t nchunks, shadow_w;
	uint64_t pool_words, shadow_len;
	uint32_t pad_rows, reserved[3];
};
static_assert(sizeof(FileHeader) == 64, "file header layout");

constexpr uint32_t kMagic = 0x31575056u;

struct File {
	FILE *f = nullptr;
	~File()
	{
		if (f) fclose(f);
	}
};

} // namespace

extern "C" {

VP_API int vp_world_save(vp_world *w, const char *path)
{
	if (!w || !path || !w->uploaded) return VP_EINVAL;
	CK(cudaSetDevice(w->ctx->device));
	cudaStream_t st = w->ctx->stream;
	const uint32_t n = w->nchunks;
	std::vector<uint64_t> off(n);
	std::vector<uint32_t> len(n);
	std::vector<uint32_t> pool(w->pool_tail);
	std::vector<uint16_t> shadow(w->shadow_len);
	CK(cudaMemcpyAsync(off.data(), w->d_off, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(len.data(), w->d_len, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	if (w->pool_tail)
		CK(cudaMemcpyAsync(pool.data(), w->d_pool, w->pool_tail * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	if (w->shadow_len)
		CK(cudaMemcpyAsync(shadow.data(), w->d_shadow, w->shadow_len * sizeof(uint16_t), cudaMemcpyDeviceToHost,
				   st));
	CK(cudaStreamSynchronize(st));
	/* packed streams in chunk order (edits leave stale streams in the pool) */
	std::vector<uint64_t> noff(n);
	uint64_t total = 0;
	for (uint32_t c = 0; c < n; c++) {
		if (off[c] + len[c] > pool.size()) return VP_EINVAL;
		noff[c] = total;
		total += (len[c] + 3u) & ~3u;
	}
	std::vector<uint32_t> packed(total, 0u);
	for (uint32_t c = 0; c < n; c++) memcpy(&packed[noff[c]], &pool[off[c]], (size_t)len[c] * sizeof(uint32_t));
	FileHeader h;
	memset(&h, 0, sizeof(h));
	h.magic = kMagic;
	h.version = 1;
	h.root_bitw = w->root_bitw;
	for (int i = 0; i < 3; i++) h.max_bitw[i] = w->max_bitw[i];
	h.nchunks = n;
	h.shadow_w = w->shadow_w;
	h.pool_words = total;
	h.shadow_len = w->shadow_len;
	const uint64_t z = (uint64_t)(1u << w->max_bitw[2]) << w->root_bitw;
	h.pad_rows = (w->shadow_w && w->shadow_len / w->shadow_w > z) ? (uint32_t)(w->shadow_len / w->shadow_w - z) : 0u;
	File f;
	f.f = fopen(path, "wb");
	if (!f.f) return VP_EINVAL;
	bool ok = fwrite(&h, sizeof(h), 1, f.f) == 1 && fwrite(noff.data(), 8, n, f.f) == n &&
		  fwrite(len.data(), 4, n, f.f) == n && fwrite(packed.data(), 4, total, f.f) == total &&
		  fwrite(shadow.data(), 2, w->shadow_len, f.f) == w->shadow_len;
	ok = (fflush(f.f) == 0) && ok;
	return ok ? VP_OK : VP_EINVAL;
}

VP_API int vp_world_open(vp_ctx *ctx, const char *path, vp_world **out)
{
	if (!ctx || !path || !out) return VP_EINVAL;
	*out = nullptr;
	File f;
	f.f = fopen(path, "rb");
	if (!f.f) return VP_EINVAL;
	FileHeader h;
	if (fread(&h, sizeof(h), 1, f.f) != 1 || h.magic != kMagic || h.version != 1) return VP_EINVAL;
	if (h.max_bitw[0] < 0 || h.max_bitw[1] < 0 || h.max_bitw[2] < 0 ||
	    h.max_bitw[0] + h.max_bitw[1] + h.max_bitw[2] > 24 ||
	    h.nchunks != (1u << (h.max_bitw[0] + h.max_bitw[1] + h.max_bitw[2])))
		return VP_EINVAL;
	if (h.pool_words > (1ull << 40) || h.shadow_len > (1ull << 40)) return VP_EINVAL;
	const uint32_t n = h.nchunks;
	std::vector<uint64_t> off(n);
	std::vector<uint32_t> len(n);
	std::vector<uint32_t> pool(h.pool_words);
	std::vector<uint16_t> shadow(h.shadow_len);
	if (fread(off.data(), 8, n, f.f) != n || fread(len.data(), 4, n, f.f) != n ||
	    fread(pool.data(), 4, h.pool_words, f.f) != h.pool_words ||
	    fread(shadow.data(), 2, h.shadow_len, f.f) != h.shadow_len)
		return VP_EINVAL;
	vp_world *w = nullptr;
	int rc = vp_world_create(ctx, h.root_bitw, h.max_bitw, &w);
	if (rc) return rc;
	/* vp_world_upload validates every stream on the device */
	rc = vp_world_upload(w, pool.data(), h.pool_words, off.data(), len.data(), shadow.data(), h.shadow_len,
			     h.shadow_w);
	if (rc) {
		vp_world_destroy(w);
		return rc;
	}
	*out = w;
	return VP_OK;
}

} // extern "C"
