"""vp_rebuild_noalloc, the geometry rebuild for callers that cannot allocate
device memory when they need geometry (a render thread that must not stall
on cudaMalloc's implicit synchronisation, an engine whose allocator owns all
device memory). Every buffer here is allocated by the test (torch); the
entry point itself only uses its fixed device scratch array. Its output must
equal the regular world rebuild's bit for bit, on two calls in a row (the
scratch array keeps the previous call's contents, so the second call checks
that everything that must start at zero is cleared)."""
import ctypes

import numpy as np
import pytest

from tests import worlds
from voxplat_gb300 import gpu

pytestmark = pytest.mark.gpu
V, I, U32, U64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64


def _bind(lib):
    f = lib.vp_rebuild_noalloc
    f.restype = I
    f.argtypes = [I, V, I, V, V, V, V, V, U64, U32, V, I, V, U64, V, U64, V, U64, V]
    return f


def test_noalloc_rebuild_matches_world_rebuild():
    torch = pytest.importorskip("torch")
    lib = gpu.load()
    rebuild = _bind(lib)
    ctx = gpu.Context(0)
    w = worlds.cave_world(5, (1, 2, 1), seed=61)  # 16 chunks of 32^3
    n = w.nchunks
    dw = gpu.DeviceWorld(ctx, w)
    dev = torch.device("cuda:0")
    pool = torch.from_numpy(np.concatenate([w.pool, np.zeros(8, np.uint32)]).view(np.int32)).to(dev)
    off = torch.from_numpy(w.off.view(np.int64)).to(dev)
    lens = torch.from_numpy(w.len.view(np.int32)).to(dev)
    shadow = torch.from_numpy(w.shadow.view(np.int16)).to(dev)
    cap = 64 << 20
    svl = torch.zeros(cap, dtype=torch.uint8, device=dev)
    vbo = torch.zeros(cap, dtype=torch.uint8, device=dev)
    ibo = torch.zeros(cap, dtype=torch.uint8, device=dev)
    results = torch.zeros(n * gpu.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    mb = (ctypes.c_int * 3)(*w.max_bitw)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call, modes in enumerate([(np.arange(n) % 3 == 0), (np.arange(n) % 2 == 1)]):
        modes = modes.astype(np.uint8)
        dw.set_modes(modes)
        dw.rebuild(lod_max=4)
        dw.finish()
        want = dw.results()
        mm = torch.from_numpy(modes).to(dev)
        rc = rebuild(0, stream, w.root_bitw, mb, pool.data_ptr(), off.data_ptr(), lens.data_ptr(),
                     shadow.data_ptr(), len(w.shadow), w.shadow_w, mm.data_ptr(), 4, svl.data_ptr(), cap,
                     vbo.data_ptr(), cap, ibo.data_ptr(), cap, results.data_ptr())
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = results.cpu().numpy().view(gpu.RESULT_DTYPE)
        s16 = svl.cpu().numpy().view(np.int16)
        v16 = vbo.cpu().numpy().view(np.int16)
        i32 = ibo.cpu().numpy().view(np.uint32)
        for c in range(n):
            assert got[c]["status"] == 0, (call, c)
            if modes[c]:
                wv, wi = dw.chunk_mesh(want, c)
                gv = v16[got[c]["vbo_off"]:got[c]["vbo_off"] + got[c]["vbo_items"]]
                gi = i32[got[c]["ibo_off"]:got[c]["ibo_off"] + got[c]["ibo_items"]]
                assert np.array_equal(gv, wv) and np.array_equal(gi, wi), (call, c)
            else:
                ws, witems = dw.chunk_splats(want, c)
                gs = s16[got[c]["svl_off"]:got[c]["svl_off"] + got[c]["svl_total"]]
                assert np.array_equal(got[c]["svl_items"], witems), (call, c)
                assert np.array_equal(gs, ws), (call, c)


def test_noalloc_rejects_sets_beyond_its_scratch():
    rebuild = _bind(gpu.load())
    mb = (ctypes.c_int * 3)(4, 4, 1)  # 512 chunks of 64^3 need more than 4 MiB of shells
    rc = rebuild(0, None, 6, mb, 16, 16, 16, 16, 0, 0, None, 4, 16, 0, 16, 0, 16, 0, 16)
    assert rc == -4  # VP_EOVERFLOW
