"""Picking rays on the device (vp_world_raycast) against the oracle's
restatement of chunkset_edit_raycast_until_solid (src/chunkset/edit.c:
248-314), before and after edits; the VPW1 world file between the C ABI
(vp_world_save / vp_world_open) and the NumPy reader/writer."""
import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from tests.test_oracle_raycast import rays  # noqa: E402
from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


def check_rays(dw, o, extent, seed, n=400):
    rs = rays(np.random.default_rng(seed), extent, n)
    org = np.array([r[0] for r in rs], np.float32)
    vec = np.array([r[1] for r in rs], np.float32)
    vox, coords, normals = dw.raycast(org, vec)
    hits = 0
    for k in range(n):
        v, c, nm = o.raycast(org[k], vec[k])
        assert vox[k] == v and np.array_equal(coords[k], c) and np.array_equal(normals[k], nm), (k, org[k], vec[k])
        hits += v > 0
    return hits


@pytest.mark.parametrize("root_bitw,max_bitw", [(4, (2, 3, 2)), (5, (1, 2, 1)), (6, (1, 1, 1))])
def test_raycast_matches_oracle(ctx, root_bitw, max_bitw):
    w = worlds.cave_world(root_bitw, max_bitw, seed=13)
    dw = gpu.DeviceWorld(ctx, w)
    extent = [w.R << b for b in max_bitw]
    assert check_rays(dw, OracleWorld(w), extent, root_bitw) > 50


def test_raycast_after_edits(ctx):
    w = worlds.cave_world(4, (2, 3, 2), seed=13)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    dw.set_modes(None)
    dw.rebuild(lod_max=4)
    dw.finish()
    check_rays(dw, o, [64, 128, 64], 1, 100)
    edits = [(20, 60, 20, 9, 0), (40, 30, 40, 6, 99), (10, 80, 50, 12, 7)]
    for e in edits:
        o.edit_sphere(e[:3], e[3], e[4])
    dw.edit(gpu.make_edits(edits))
    check_rays(dw, o, [64, 128, 64], 2, 300)


def test_world_file_between_c_and_numpy(ctx, tmp_path):
    w = worlds.cave_world(5, (1, 2, 1), seed=4)
    p1 = tmp_path / "a.vpw"
    w.save(p1)
    dw = gpu.DeviceWorld.open(ctx, str(p1))
    assert worlds.compare_world(dw, OracleWorld(w), None, 4) == []
    # edits, then save from the device and read back with NumPy
    dw.edit(gpu.make_edits([(30, 50, 30, 8, 0), (10, 20, 40, 5, 200)]))
    p2 = tmp_path / "b.vpw"
    dw.save(str(p2))
    v = wg.World.load(p2)
    for c in range(w.nchunks):
        assert np.array_equal(v.chunk_rle(c), dw.chunk_rle(c))
    assert np.array_equal(v.shadow[:len(w.shadow)], dw.shadow(len(w.shadow)))
    assert v.pad_rows == w.pad_rows and v.shadow_z == w.shadow_z


def test_generated_world_file_round_trip(ctx, tmp_path):
    dw = gpu.DeviceWorld.generated(ctx, wg.TERRAIN_CAVES, 6, (2, 1, 2), 7)
    p = tmp_path / "g.vpw"
    dw.save(str(p))
    host = wg.terrain(wg.TERRAIN_CAVES, 6, (2, 1, 2), seed=7)
    v = wg.World.load(p)
    for c in range(host.nchunks):
        assert np.array_equal(v.chunk_rle(c), host.chunk_rle(c))
    assert np.array_equal(v.shadow, host.shadow)
