"""vp_rebuild_noalloc, the geometry rebuild for callers that cannot allocate
device memory when they need geometry (a render thread that must not stall
on cudaMalloc's implicit synchronisation, an engine whose allocator owns all
device memory). Every buffer here is allocated by the test (torch); the
entry point itself only uses its fixed device scratch array.

Its output must equal the regular world rebuild's and the oracle's bit for
bit, on two calls in a row (the scratch array keeps the previous call's
contents, so the second call checks that everything that must start at zero
is cleared), for the largest set of each chunk size the 4 MiB array holds;
the second call must leave the device's free memory unchanged; malformed
streams must come back flagged and be built as air.

This file is collected last so that a run stopping at the first failure has
run every other test before it."""
import ctypes

import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from voxplat_gb300 import gpu

pytestmark = pytest.mark.gpu
V, I, U32, U64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64
STATUS_BAD_STREAM = 2
LOD = 4


def _bind(lib):
    f = lib.vp_rebuild_noalloc
    f.restype = I
    f.argtypes = [I, V, I, V, V, U64, V, V, V, U64, U32, V, I, V, U64, V, U64, V, U64, V]
    return f


class _Call:
    """Device copies of a world's inputs and output buffers for the entry point."""

    def __init__(self, torch, w, pool=None, off=None, lens=None, cap=64 << 20):
        dev = torch.device("cuda:0")
        pool = w.pool if pool is None else pool
        self.pool_words = len(pool) + 8
        self.pool = torch.from_numpy(np.concatenate([pool, np.zeros(8, np.uint32)]).view(np.int32)).to(dev)
        self.off = torch.from_numpy(np.ascontiguousarray(w.off if off is None else off, np.uint64).view(np.int64)).to(dev)
        self.lens = torch.from_numpy(np.ascontiguousarray(w.len if lens is None else lens, np.uint32).view(np.int32)).to(dev)
        self.shadow = torch.from_numpy(w.shadow.view(np.int16)).to(dev)
        self.cap = cap
        self.svl = torch.zeros(cap, dtype=torch.uint8, device=dev)
        self.vbo = torch.zeros(cap, dtype=torch.uint8, device=dev)
        self.ibo = torch.zeros(cap, dtype=torch.uint8, device=dev)
        self.results = torch.zeros(w.nchunks * gpu.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.mb = (ctypes.c_int * 3)(*w.max_bitw)
        self.w = w
        self.torch = torch

    def set_modes(self, modes):
        self.mm = self.torch.from_numpy(np.ascontiguousarray(modes, np.uint8)).to("cuda:0")
        self.torch.cuda.synchronize()

    def run(self, rebuild, modes=None):
        torch = self.torch
        if modes is not None:
            self.set_modes(modes)
        mm = self.mm
        stream = torch.cuda.current_stream(0).cuda_stream
        rc = rebuild(0, stream, self.w.root_bitw, self.mb, self.pool.data_ptr(), self.pool_words, self.off.data_ptr(),
                     self.lens.data_ptr(), self.shadow.data_ptr(), len(self.w.shadow), self.w.shadow_w, mm.data_ptr(),
                     LOD, self.svl.data_ptr(), self.cap, self.vbo.data_ptr(), self.cap, self.ibo.data_ptr(), self.cap,
                     self.results.data_ptr())
        torch.cuda.synchronize()
        return rc

    def outputs(self):
        return (self.svl.cpu().numpy().view(np.int16), self.vbo.cpu().numpy().view(np.int16),
                self.ibo.cpu().numpy().view(np.uint32), self.results.cpu().numpy().view(gpu.RESULT_DTYPE))


def _same_as_world_rebuild(dw, modes, got, s16, v16, i32):
    dw.set_modes(modes)
    dw.rebuild(lod_max=LOD)
    dw.finish()
    want = dw.results()
    for c in range(dw.nchunks):
        if modes[c]:
            wv, wi = dw.chunk_mesh(want, c)
            gv = v16[got[c]["vbo_off"]:got[c]["vbo_off"] + got[c]["vbo_items"]]
            gi = i32[got[c]["ibo_off"]:got[c]["ibo_off"] + got[c]["ibo_items"]]
            if not (np.array_equal(gv, wv) and np.array_equal(gi, wi)):
                return c
        else:
            ws, witems = dw.chunk_splats(want, c)
            gs = s16[got[c]["svl_off"]:got[c]["svl_off"] + got[c]["svl_total"]]
            if not (np.array_equal(got[c]["svl_items"], witems) and np.array_equal(gs, ws)):
                return c
    return None


# the largest set of each chunk size that the 4 MiB scratch array holds
@pytest.mark.parametrize("root_bitw,max_bitw", [(3, (4, 4, 4)), (4, (4, 3, 4)), (5, (3, 3, 3)), (6, (3, 2, 3))])
def test_noalloc_rebuild_matches_world_rebuild_and_oracle(root_bitw, max_bitw):
    torch = pytest.importorskip("torch")
    rebuild = _bind(gpu.load())
    ctx = gpu.Context(0)
    w = worlds.cave_world(root_bitw, max_bitw, seed=61 + root_bitw)
    n = w.nchunks
    dw = gpu.DeviceWorld(ctx, w)
    o = OracleWorld(w)
    call = _Call(torch, w)
    for k, modes in enumerate([(np.arange(n) % 3 == 0), (np.arange(n) % 2 == 1)]):
        modes = modes.astype(np.uint8)
        # the regular rebuild first: it may allocate; the second call's
        # allocation-free claim is checked around the entry point alone
        dw.set_modes(modes)
        dw.rebuild(lod_max=LOD)
        dw.finish()
        call.set_modes(modes)
        free0 = torch.cuda.mem_get_info(0)[0]
        assert call.run(rebuild) == 0
        free1 = torch.cuda.mem_get_info(0)[0]
        if k == 1:
            assert free1 == free0, "the entry point changed the device's free memory"
        s16, v16, i32, got = call.outputs()
        assert (got["status"] == 0).all(), (k, np.nonzero(got["status"])[0][:8])
        assert _same_as_world_rebuild(dw, modes, got, s16, v16, i32) is None, k
        bad, nbad = o.check(np.arange(n), modes, LOD, s16, v16, i32, got)
        assert nbad == 0, (k, bad)
    dw.close()
    ctx.close()


def test_noalloc_flags_malformed_streams_and_builds_them_as_air():
    """Malformed streams (all of them inside the pool, so a decoder that
    skipped the check would still read in bounds) come back with
    VP_STATUS_BAD_STREAM, and every chunk equals the oracle's with those
    chunks replaced by air."""
    torch = pytest.importorskip("torch")
    rebuild = _bind(gpu.load())
    w = worlds.cave_world(5, (2, 1, 2), seed=71)
    n = w.nchunks
    N = 32 ** 3
    extra = (len(w.pool) + 3) // 4 * 4  # 16-byte aligned words at the pool's tail
    pool = np.concatenate([w.pool, np.zeros(extra - len(w.pool) + 64, np.uint32)]).astype(np.uint32)
    off = w.off.astype(np.uint64).copy()
    lens = w.len.astype(np.uint32).copy()
    # chunk 1: a zero count in the middle; chunk 4: counts one voxel short;
    # chunk 6: no terminator; chunk 9: a length of 1
    pool[extra:extra + 4] = [5, 0, N - 5, 0]
    off[1], lens[1] = extra, 4
    pool[extra + 8:extra + 11] = [N - 1 | (7 << 24), 0, 0]
    off[4], lens[4] = extra + 8, 2
    pool[extra + 16:extra + 18] = [N | (9 << 24), 3]
    off[6], lens[6] = extra + 16, 2
    lens[9] = 1
    flagged = [1, 4, 6, 9]
    call = _Call(torch, w, pool=pool, off=off, lens=lens)
    modes = (np.arange(n) % 2).astype(np.uint8)
    for _ in range(2):
        assert call.run(rebuild, modes) == 0
        s16, v16, i32, got = call.outputs()
        assert sorted(np.nonzero(got["status"])[0].tolist()) == flagged
        assert (got["status"][flagged] == STATUS_BAD_STREAM).all()
        # the oracle with the flagged chunks as air: every chunk, the flagged
        # ones included (an air chunk still has the faces of its solid
        # +neighbours), once their status is set aside
        air = worlds.world_from_voxels(5, w.max_bitw, [None if c in flagged else w.chunk_voxels(c) for c in range(n)])
        air.shadow[:] = w.shadow
        o = OracleWorld(air)
        rec = got.copy()
        rec["status"][flagged] = 0
        bad, nbad = o.check(np.arange(n), modes, LOD, s16, v16, i32, rec)
        assert nbad == 0, bad


def test_noalloc_rejects_sets_beyond_its_scratch():
    rebuild = _bind(gpu.load())
    for rb, mb in ((6, (4, 4, 1)), (5, (4, 3, 3)), (4, (4, 4, 4)), (3, (5, 4, 4))):
        m = (ctypes.c_int * 3)(*mb)
        rc = rebuild(0, None, rb, m, 16, 1 << 20, 16, 16, 16, 0, 0, None, 4, 16, 0, 16, 0, 16, 0, 16)
        assert rc == -4, (rb, mb, rc)  # VP_EOVERFLOW
    # more than 2^24 chunks: refused before any size arithmetic
    m = (ctypes.c_int * 3)(12, 12, 8)
    assert rebuild(0, None, 6, m, 16, 1 << 20, 16, 16, 16, 0, 0, None, 4, 16, 0, 16, 0, 16, 0, 16) == -6
    # a pool that is not 4-byte aligned
    m = (ctypes.c_int * 3)(1, 1, 1)
    assert rebuild(0, None, 6, m, 18, 1 << 20, 16, 16, 16, 0, 0, None, 4, 16, 0, 16, 0, 16, 0, 16) == -1
