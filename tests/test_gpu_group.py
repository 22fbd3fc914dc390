"""LOD/octree grouping on the device against the oracle's restatement of
gfx_update_svl (src/gfx/vsplat.c:209-331), and the plain per-chunk launch
path against the batched one."""
import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from voxplat_gb300 import gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


@pytest.mark.parametrize("root_bitw,max_bitw,lod_max", [(4, (2, 3, 2), 4), (4, (3, 1, 2), 5), (5, (1, 2, 1), 3)])
def test_group_matches_oracle(ctx, root_bitw, max_bitw, lod_max):
    w = worlds.cave_world(root_bitw, max_bitw, seed=31)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    modes = (np.arange(w.nchunks) % 5 == 0).astype(np.uint8)  # meshed chunks contribute nothing
    dw.set_modes(modes)
    dw.rebuild(lod_max=lod_max, group=True)
    dw.finish()
    svl, items = [], []
    for c in range(w.nchunks):
        if modes[c]:
            svl.append(np.zeros(0, np.int16))
            items.append(np.zeros(8, np.uint32))
        else:
            g, it = o.splats(c, lod_max)
            svl.append(g)
            items.append(np.concatenate([it, np.zeros(8 - len(it), np.uint32)]))
    for lod in range(lod_max + 1):
        ob = [b - min(lod, b) for b in max_bitw]
        off, nit = dw.group_nodes(lod)
        for nz in range(1 << ob[2]):
            for ny in range(1 << ob[1]):
                for nx in range(1 << ob[0]):
                    idx = ((nz << ob[1] | ny) << ob[0]) | nx
                    want = o.group_node(lod, (nx, ny, nz), svl, items)
                    got = dw.read_group(lod, off[idx], nit[idx])
                    assert np.array_equal(got, want), (lod, nx, ny, nz)


@pytest.mark.parametrize("concurrent", [False, True])
def test_plain_path_matches_batched(ctx, concurrent):
    w = worlds.cave_world(5, (1, 2, 1), seed=77)
    dw = gpu.DeviceWorld(ctx, w)
    modes = (np.arange(w.nchunks) % 2).astype(np.uint8)
    dw.set_modes(modes)
    dw.rebuild(lod_max=4)
    dw.finish()
    a = dw.results()
    ref = {c: (dw.chunk_mesh(a, c) if modes[c] else dw.chunk_splats(a, c)[0]) for c in range(w.nchunks)}
    dw.rebuild(lod_max=4, persistent=False, plain=not concurrent, concurrent=concurrent)
    dw.finish()
    b = dw.results()
    for c in range(w.nchunks):
        got = dw.chunk_mesh(b, c) if modes[c] else dw.chunk_splats(b, c)[0]
        if modes[c]:
            assert np.array_equal(got[0], ref[c][0]) and np.array_equal(got[1], ref[c][1])
        else:
            assert np.array_equal(got, ref[c])


def test_overflowing_arenas_grow_and_rerun(ctx):
    """Arenas of 16 bytes overflow on the first pass: finish() grows them and
    reruns the rebuild and the grouping, with the same results as a rebuild
    that fit at once."""
    w = worlds.cave_world(4, (2, 3, 2), seed=31)
    modes = (np.arange(w.nchunks) % 5 == 0).astype(np.uint8)
    got = []
    for tiny in (False, True):
        dw = gpu.DeviceWorld(ctx, w)
        dw.set_modes(modes)
        if tiny:
            dw.reserve(16, 16, 16)
        dw.rebuild(lod_max=4, group=True)
        dw.finish()
        res = dw.results()
        assert (res["status"] == 0).all()
        geo = [dw.chunk_mesh(res, c) if modes[c] else dw.chunk_splats(res, c)[0] for c in range(w.nchunks)]
        groups = []
        for lod in range(5):
            off, nit = dw.group_nodes(lod)
            nodes = 1 << sum(b - min(lod, b) for b in (2, 3, 2))
            groups.append([dw.read_group(lod, off[i], nit[i]) for i in range(nodes)])
        got.append((geo, groups))
        dw.close()
    (ga, gra), (gb, grb) = got
    for c in range(w.nchunks):
        if modes[c]:
            assert all(np.array_equal(x, y) for x, y in zip(ga[c], gb[c])), c
        else:
            assert np.array_equal(ga[c], gb[c]), c
    for lod in range(5):
        assert all(np.array_equal(x, y) for x, y in zip(gra[lod], grb[lod])), lod
