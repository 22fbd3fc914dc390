"""Sphere edits on the device (chunkset_edit_sphere, src/chunkset/edit.c:
179-244) against the reference's own edit results and the oracle; batching
equivalence (an edit's result is the same alone and in a batch); and the
serving loop."""
import os

import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


def decode(words, n):
    s = words[:-1]
    return np.repeat((s >> 24).astype(np.uint8), (s & 0xFFFFFF).astype(np.int64))[:n]


def geometry(dw, modes, c, res):
    return dw.chunk_mesh(res, c) if modes[c] else dw.chunk_splats(res, c)


def same_geometry(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_edits_match_reference_fixture(ctx):
    w, d = worlds.load_fixture(os.path.join(GOLDEN, "edits_r16.npz"))
    dw = gpu.DeviceWorld(ctx, w)
    dw.set_modes(None)
    dw.rebuild(lod_max=4)
    dw.finish()
    for k, e in enumerate(d["edits"]):
        dw.edit(gpu.make_edits([e]))
        assert set(dw.dirty().tolist()) == set(np.nonzero(d["dirty%d" % k])[0].tolist()), k
    N = w.R ** 3
    for c in range(w.nchunks):
        assert np.array_equal(decode(dw.chunk_rle(c), N), d["voxels"][c]), c
    assert np.array_equal(dw.shadow(len(d["shadow_after"])), d["shadow_after"])
    dw.rebuild(lod_max=4)
    dw.finish()
    res = dw.results()
    pieces = worlds.split(d["post_svl4"], d["post_svl4_items"].sum(axis=1))
    for c in range(w.nchunks):
        g, _ = dw.chunk_splats(res, c)
        assert np.array_equal(g, pieces[c]), c


def random_edits(rng, n, extent, rmax):
    rows = []
    for _ in range(n):
        r = int(rng.integers(1, rmax + 1))
        v = 0 if rng.random() < 0.5 else int(rng.integers(1, 256))
        rows.append((int(rng.integers(-4, extent[0] + 4)), int(rng.integers(0, extent[1])),
                     int(rng.integers(-4, extent[2] + 4)), r, v))
    return rows


@pytest.mark.parametrize("root_bitw,max_bitw", [(4, (2, 3, 2)), (5, (1, 2, 1))])
def test_random_edits_match_oracle(ctx, root_bitw, max_bitw):
    w = worlds.cave_world(root_bitw, max_bitw, seed=90 + root_bitw)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    modes = (np.arange(w.nchunks) % 4 == 0).astype(np.uint8)
    dw.set_modes(modes)
    dw.rebuild(lod_max=4)
    dw.finish()
    rng = np.random.default_rng(root_bitw)
    extent = [w.R * (1 << b) for b in max_bitw]
    for step in range(6):
        batch = random_edits(rng, 1 + step % 3, extent, 12)
        for e in batch:
            o.edit_sphere(e[:3], e[3], e[4])
        dw.edit(gpu.make_edits(batch))
        res = dw.results()
        for c in dw.dirty():
            want = o.mesh(c) if modes[c] else o.splats(c, 4)[0]
            got = geometry(dw, modes, c, res)
            if modes[c]:
                assert same_geometry(got, want), (step, c)
            else:
                assert np.array_equal(got[0], want), (step, c)
    N = w.R ** 3
    for c in range(w.nchunks):
        assert np.array_equal(decode(dw.chunk_rle(c), N), o.voxels(c)), c
    assert np.array_equal(dw.shadow(len(w.shadow)), o.shadow_map())


def test_batch_equals_one_by_one(ctx):
    w = worlds.cave_world(4, (2, 3, 2), seed=123)
    rng = np.random.default_rng(9)
    edits = random_edits(rng, 10, [64, 128, 64], 10)
    worlds_ = []
    for batched in (False, True):
        dw = gpu.DeviceWorld(ctx, w)
        dw.set_modes(None)
        dw.rebuild(lod_max=4)
        dw.finish()
        if batched:
            dw.edit(gpu.make_edits(edits))
        else:
            for e in edits:
                dw.edit(gpu.make_edits([e]))
        dw.rebuild(lod_max=4)
        dw.finish()
        res = dw.results()
        worlds_.append(([dw.chunk_rle(c) for c in range(w.nchunks)], dw.shadow(len(w.shadow)),
                        [dw.chunk_splats(res, c)[0] for c in range(w.nchunks)]))
    a, b = worlds_
    for c in range(w.nchunks):
        assert np.array_equal(a[0][c], b[0][c]) and np.array_equal(a[2][c], b[2][c]), c
    assert np.array_equal(a[1], b[1])


def test_serve_loop_applies_every_edit_in_order(ctx):
    w = worlds.cave_world(5, (2, 2, 2), seed=7)
    rng = np.random.default_rng(4)
    rows = random_edits(rng, 60, [128, 128, 128], 16)
    arrival = np.cumsum(rng.exponential(1 / 2000.0, len(rows)))
    served = gpu.DeviceWorld(ctx, w)
    served.set_modes(None)
    served.rebuild(lod_max=4)
    served.finish()
    lat, st = served.serve(gpu.make_edits(rows, arrival), max_batch=8)
    assert st.edits == len(rows) and st.batches >= 1 and (lat > 0).all()
    serial = gpu.DeviceWorld(ctx, w)
    serial.set_modes(None)
    serial.rebuild(lod_max=4)
    serial.finish()
    for r in rows:
        serial.edit(gpu.make_edits([r]))
    for c in range(w.nchunks):
        assert np.array_equal(served.chunk_rle(c), serial.chunk_rle(c)), c
    assert np.array_equal(served.shadow(len(w.shadow)), serial.shadow(len(w.shadow)))
