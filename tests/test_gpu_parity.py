"""GPU parity: the CUDA pipeline against the C restatement of the reference,
bit-exact, through the C ABI (include/voxgpu.h)."""
import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


@pytest.mark.parametrize("lod_max", [3, 4])
def test_config1_chunk_splats(ctx, lod_max):
    w = worlds.config1_chunk()
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, OracleWorld(w), None, lod_max) == []


def test_config1_chunk_mesh(ctx):
    w = worlds.config1_chunk()
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, OracleWorld(w), np.ones(1, np.uint8), 4) == []


@pytest.mark.parametrize("root_bitw,max_bitw", [(5, (1, 3, 1)), (6, (1, 2, 1)), (4, (2, 4, 2)), (3, (2, 5, 2))])
def test_cave_world_mixed_modes(ctx, root_bitw, max_bitw):
    w = worlds.cave_world(root_bitw, max_bitw, seed=11 + root_bitw)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    modes = (np.arange(w.nchunks) % 3 == 0).astype(np.uint8)
    assert worlds.compare_world(dw, o, modes, 4) == []
    assert worlds.compare_world(dw, o, 1 - modes, 4) == []


@pytest.mark.parametrize("k", range(12))
def test_uneven_chunks(ctx, k):
    w = wg.uneven_chunk(5, k)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, o, None, 4) == []
    assert worlds.compare_world(dw, o, np.ones(1, np.uint8), 4) == []


@pytest.mark.parametrize("max_bitw", [(1, 0, 1), (0, 1, 0)])
def test_big_chunk_worlds(ctx, max_bitw):
    """128^3 chunks (two-word rows, working set in global scratch) with
    neighbours across x and z, or across y."""
    w = worlds.cave_world(7, max_bitw, seed=21)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    modes = (np.arange(w.nchunks) % 2).astype(np.uint8)
    assert worlds.compare_world(dw, o, modes, 4) == []
    assert worlds.compare_world(dw, o, 1 - modes, 5) == []


@pytest.mark.parametrize("lod_max", [0, 1, 5, 7])
def test_big_chunk_lod_levels(ctx, lod_max):
    w = wg.uneven_chunk(5, 8)
    assert w.root_bitw == 7
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, OracleWorld(w), None, lod_max) == []


@pytest.mark.parametrize("lod_max", [0, 1, 5, 7])
def test_lod_levels(ctx, lod_max):
    w = worlds.cave_world(5, (1, 2, 1), seed=3)
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, OracleWorld(w), None, lod_max) == []


def _edge_worlds():
    R = 16
    rng = np.random.default_rng(9)
    air = np.zeros(R ** 3, np.uint8)
    solid = np.full(R ** 3, 200, np.uint8)
    one = air.copy()
    one[5 + R * (6 + R * 7)] = 77
    corner = air.copy()
    corner[0] = 3
    corner[R ** 3 - 1] = 250
    checker = np.fromfunction(lambda i: ((i % R + (i // R) % R + i // (R * R)) % 2) * 99 + 1, (R ** 3,),
                              dtype=np.int64).astype(np.uint8) * ((np.arange(R ** 3) % 2).astype(np.uint8))
    noise = rng.integers(0, 256, R ** 3).astype(np.uint8)
    noise[rng.random(R ** 3) < 0.5] = 0
    return {
        "all_air": [air] * 8,
        "all_solid": [solid] * 8,
        "single_voxel": [one, None, None, None, None, None, None, one],
        "corners": [corner] * 8,
        "checker": [checker] * 8,
        "noise": [noise, noise[::-1].copy(), None, noise, None, noise, noise, None],
    }


@pytest.mark.parametrize("name", list(_edge_worlds()))
def test_edge_cases(ctx, name):
    vox = _edge_worlds()[name]
    rng = np.random.default_rng(4)
    w = worlds.world_from_voxels(4, (1, 1, 1), vox)
    w.shadow[:w.shadow_w * w.shadow_z] = rng.integers(0, 40, w.shadow_w * w.shadow_z)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    for modes in (None, np.ones(8, np.uint8), (np.arange(8) % 2).astype(np.uint8)):
        assert worlds.compare_world(dw, o, modes, 4) == [], modes


def test_rejects_malformed_streams(ctx):
    w = worlds.cave_world(4, (0, 0, 0), seed=1)
    bad = w.pool.copy()
    bad[w.off[0]] = bad[w.off[0]] & 0xFF000000  # a zero-length run
    broken = wg.World(w.root_bitw, w.max_bitw, bad, w.off, w.len, w.shadow, w.shadow_w, w.shadow_z)
    with pytest.raises(gpu.VoxGpuError):
        gpu.DeviceWorld(ctx, broken)


def test_upload_validates_on_device_and_repacks_unaligned_streams(ctx):
    """Streams are checked on the device (sum of counts, zero counts, the
    terminator); streams off 16-byte boundaries are repacked; a rejected
    upload leaves nothing to rebuild, and the next valid upload works."""
    w = worlds.cave_world(4, (1, 1, 1), seed=8)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, o, None, 4) == []
    cases = []
    short = w.pool.copy()
    short[w.off[3]] -= 1                       # counts sum to N - 1
    cases.append((short, w.len))
    noterm = w.pool.copy()
    noterm[w.off[5] + w.len[5] - 1] = 7       # no terminator
    cases.append((noterm, w.len))
    lens = w.len.copy()
    lens[2] = 1                               # a stream of one word
    cases.append((w.pool, lens))
    for pool, ln in cases:
        with pytest.raises(gpu.VoxGpuError):
            dw.upload_arrays(pool, w.off, ln, w.shadow, w.shadow_w)
        with pytest.raises(gpu.VoxGpuError):
            dw.rebuild(lod_max=4)
    # the same streams shifted by one word: offsets off 16-byte boundaries
    shifted = np.concatenate([np.zeros(1, np.uint32), w.pool])
    dw.upload_arrays(shifted, w.off + 1, w.len, w.shadow, w.shadow_w)
    assert worlds.compare_world(dw, o, np.ones(w.nchunks, np.uint8), 4) == []
    assert worlds.compare_world(dw, o, None, 4) == []


def test_read_outputs_returns_the_arena_layout(ctx):
    w = worlds.cave_world(5, (1, 1, 1), seed=12)
    dw = gpu.DeviceWorld(ctx, w)
    modes = (np.arange(w.nchunks) % 2).astype(np.uint8)
    dw.set_modes(modes)
    dw.rebuild(lod_max=4)
    dw.finish()
    res = dw.results()
    svl = np.zeros(1 << 22, np.int16)
    vbo = np.zeros(1 << 23, np.int16)
    ibo = np.zeros(1 << 22, np.uint32)
    used = dw.read_outputs(svl, vbo, ibo)
    for c in range(w.nchunks):
        r = res[c]
        if modes[c]:
            v, i = dw.chunk_mesh(res, c)
            assert np.array_equal(vbo[r["vbo_off"]:r["vbo_off"] + r["vbo_items"]], v)
            assert np.array_equal(ibo[r["ibo_off"]:r["ibo_off"] + r["ibo_items"]], i)
        else:
            g, _ = dw.chunk_splats(res, c)
            assert np.array_equal(svl[r["svl_off"]:r["svl_off"] + r["svl_total"]], g)
    assert used[0] >= int(np.max(res["svl_off"] + res["svl_total"])) * 2
    with pytest.raises(gpu.VoxGpuError):
        dw.read_outputs(svl[:16], vbo, ibo)
