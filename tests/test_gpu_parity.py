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
def test_terrain_chunk64_splats(ctx, lod_max):
    w = worlds.terrain_chunk64()
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, OracleWorld(w), None, lod_max) == []


def test_terrain_chunk64_mesh(ctx):
    w = worlds.terrain_chunk64()
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


def test_single_run_chunk_shells(ctx):
    """All-air and one-colour chunks (one run each) next to chunks of many
    runs: the shell pass writes the one-colour chunks' shells without
    decoding and skips the air ones, and an air chunk with only air beyond
    its +x, +y and +z faces gets a zeroed result record without a geometry
    pass. Then edits turn two air chunks (one of them that one) and a
    one-colour chunk into many-run chunks (the work orders follow the new
    lengths) before a full rebuild."""
    R = 16
    rng = np.random.default_rng(12)
    air = np.zeros(R ** 3, np.uint8)
    noise = rng.integers(1, 256, R ** 3).astype(np.uint8)
    noise[rng.random(R ** 3) < 0.6] = 0
    # chunk 7 (the +x +y +z corner) is air with nothing beyond it: no geometry
    vox = [air, np.full(R ** 3, 200, np.uint8), noise, np.full(R ** 3, 13, np.uint8),
           noise[::-1].copy(), air, np.full(R ** 3, 200, np.uint8), air]
    w = worlds.world_from_voxels(4, (1, 1, 1), vox)
    w.shadow[:w.shadow_w * w.shadow_z] = rng.integers(0, 40, w.shadow_w * w.shadow_z)
    o = OracleWorld(w)
    dw = gpu.DeviceWorld(ctx, w)
    for modes in (None, np.ones(8, np.uint8), (np.arange(8) % 2).astype(np.uint8)):
        assert worlds.compare_world(dw, o, modes, 4) == [], modes
    # a sphere into the air chunk 0 and into the chunk without geometry,
    # a hole in the one-colour chunk 1
    batch = [(8, 8, 8, 5, 90), (24, 24, 24, 5, 77), (24, 8, 8, 4, 0)]
    for e in batch:
        o.edit_sphere(e[:3], e[3], e[4])
    dw.edit(gpu.make_edits(batch))
    for modes in (None, (np.arange(8) % 2).astype(np.uint8)):
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


@pytest.mark.parametrize("slabs", [1, 3, 8])
def test_streamed_rebuild_matches_the_plain_sequence(ctx, slabs):
    """vp_world_rebuild_to_host: the same records and output bytes as
    rebuild + finish + results + read_outputs, also when the arenas start
    too small (the streamed pass falls back and grows them)."""
    w = worlds.cave_world(5, (2, 1, 2), seed=23)
    modes = (np.arange(w.nchunks) % 3 == 0).astype(np.uint8)
    ref = gpu.DeviceWorld(ctx, w)
    ref.set_modes(modes)
    ref.rebuild(lod_max=4, group=True)
    ref.finish()
    res_a = ref.results()
    bufs_a = [np.zeros(1 << 23, np.int16), np.zeros(1 << 23, np.int16), np.zeros(1 << 22, np.uint32)]
    used_a = ref.read_outputs(*bufs_a)
    for tiny in (False, True):
        dw = gpu.DeviceWorld(ctx, w)
        dw.set_modes(modes)
        if tiny:
            dw.reserve(16, 16, 16)
        res_b = np.zeros(w.nchunks, gpu.RESULT_DTYPE)
        bufs_b = [np.zeros(1 << 23, np.int16), np.zeros(1 << 23, np.int16), np.zeros(1 << 22, np.uint32)]
        used_b = dw.rebuild_to_host(4, *bufs_b, res_b, group=True, slabs=slabs)
        # offsets differ (the slabs allocate in another order): compare per chunk
        assert (res_b["status"] == 0).all()
        for c in range(w.nchunks):
            ra, rb = res_a[c], res_b[c]
            assert np.array_equal(ra["svl_items"], rb["svl_items"]) and ra["vbo_items"] == rb["vbo_items"]
            for arr_a, arr_b, ko, kn in ((bufs_a[0], bufs_b[0], "svl_off", "svl_total"),
                                         (bufs_a[1], bufs_b[1], "vbo_off", "vbo_items"),
                                         (bufs_a[2], bufs_b[2], "ibo_off", "ibo_items")):
                n = int(ra[kn])
                assert np.array_equal(arr_a[int(ra[ko]):int(ra[ko]) + n], arr_b[int(rb[ko]):int(rb[ko]) + n]), (c, kn)
        assert sum(used_b) >= sum(int(res_b[k].astype(np.int64).sum()) for k in ("svl_total",)) * 2
        off, items = dw.group_nodes(0)
        offr, itemsr = ref.group_nodes(0)
        assert np.array_equal(items, itemsr)


def _same_outputs(res_a, bufs_a, res_b, bufs_b):
    """Per-chunk comparison of two rebuilds' records and output bytes (the
    allocation order, and so the offsets, may differ)."""
    for c in range(len(res_a)):
        ra, rb = res_a[c], res_b[c]
        if not (np.array_equal(ra["svl_items"], rb["svl_items"]) and ra["vbo_items"] == rb["vbo_items"]
                and ra["ibo_items"] == rb["ibo_items"] and rb["status"] == 0):
            return c
        for arr_a, arr_b, ko, kn in ((bufs_a[0], bufs_b[0], "svl_off", "svl_total"),
                                     (bufs_a[1], bufs_b[1], "vbo_off", "vbo_items"),
                                     (bufs_a[2], bufs_b[2], "ibo_off", "ibo_items")):
            n = int(ra[kn])
            if not np.array_equal(arr_a[int(ra[ko]):int(ra[ko]) + n], arr_b[int(rb[ko]):int(rb[ko]) + n]):
                return c
    return None


@pytest.mark.parametrize("tiny", [False, True])
def test_pipelined_rebuilds_match_the_synchronous_one(ctx, tiny):
    """vp_world_rebuild_to_host_async over alternating host buffer sets:
    every call's outputs equal a synchronous rebuild's at the same LOD, the
    records of call k final once call k+1 (or outputs_wait) returned; with
    arenas that start too small the first call grows them and reruns."""
    w = worlds.cave_world(5, (2, 1, 2), seed=29)
    modes = (np.arange(w.nchunks) % 4 == 1).astype(np.uint8)
    lods = [4, 2, 3, 4, 1, 3]
    ref = gpu.DeviceWorld(ctx, w)
    ref.set_modes(modes)
    want = {}
    for lod in set(lods):
        res = np.zeros(w.nchunks, gpu.RESULT_DTYPE)
        bufs = [np.zeros(1 << 22, np.int16), np.zeros(1 << 22, np.int16), np.zeros(1 << 21, np.uint32)]
        ref.rebuild_to_host(lod, *bufs, res, slabs=3)
        want[lod] = (res, bufs)
    dw = gpu.DeviceWorld(ctx, w)
    dw.set_modes(modes)
    if tiny:
        dw.reserve(16, 16, 16)
    sets = [([np.zeros(1 << 22, np.int16), np.zeros(1 << 22, np.int16), np.zeros(1 << 21, np.uint32)],
             np.zeros(w.nchunks, gpu.RESULT_DTYPE)) for _ in range(2)]
    for k, lod in enumerate(lods):
        bufs, res = sets[k % 2]
        for b in bufs:
            b.fill(0)
        res.fill(0)
        used = dw.rebuild_to_host_async(lod, *bufs, res, slabs=4)
        assert all(u <= b.nbytes for u, b in zip(used, bufs))
        if k >= 1:
            pbufs, pres = sets[(k - 1) % 2]  # call k-1's outputs are final now
            assert _same_outputs(want[lods[k - 1]][0], want[lods[k - 1]][1], pres, pbufs) is None, k - 1
    dw.outputs_wait()
    k = len(lods) - 1
    bufs, res = sets[k % 2]
    assert _same_outputs(want[lods[k]][0], want[lods[k]][1], res, bufs) is None, k
    # a synchronous rebuild after pipelined ones sees the whole arenas again
    res = np.zeros(w.nchunks, gpu.RESULT_DTYPE)
    bufs = [np.zeros(1 << 22, np.int16), np.zeros(1 << 22, np.int16), np.zeros(1 << 21, np.uint32)]
    dw.rebuild_to_host(3, *bufs, res, slabs=2)
    assert _same_outputs(want[3][0], want[3][1], res, bufs) is None


def test_full_rebuilds_never_see_a_stale_decoded_handoff(ctx):
    """Full rebuilds hand each decoded chunk from the shell pass to the
    geometry pass. Uploading another world of the same size, edits between
    full rebuilds, and switching between synchronous, streamed and pipelined
    rebuilds must each leave every chunk bit-exact to the oracle."""
    a = worlds.cave_world(5, (2, 1, 2), seed=31)
    b = worlds.cave_world(5, (2, 1, 2), seed=32)
    oa, ob = OracleWorld(a), OracleWorld(b)
    modes = (np.arange(a.nchunks) % 3 == 0).astype(np.uint8)
    dw = gpu.DeviceWorld(ctx, a)
    assert worlds.compare_world(dw, oa, modes, 4) == []
    dw.upload_arrays(b.pool, b.off, b.len, b.shadow, b.shadow_w)
    assert worlds.compare_world(dw, ob, modes, 4) == []
    dw.upload_arrays(a.pool, a.off, a.len, a.shadow, a.shadow_w)
    assert worlds.compare_world(dw, oa, None, 3) == []
    # edits (remeshed without the handoff), then full rebuilds of the edited world
    edits = [(40, 30, 50, 9, 0), (70, 20, 90, 6, 77), (10, 5, 120, 12, 0)]
    for e in edits:
        oa.edit_sphere(e[:3], e[3], e[4])
    dw.set_modes(modes)
    dw.edit(gpu.make_edits(edits))
    assert worlds.compare_world(dw, oa, modes, 4) == []
    res = np.zeros(a.nchunks, gpu.RESULT_DTYPE)
    bufs = [np.zeros(1 << 22, np.int16), np.zeros(1 << 22, np.int16), np.zeros(1 << 21, np.uint32)]
    dw.rebuild_to_host_async(4, *bufs, res, slabs=3)
    dw.outputs_wait()
    for c in range(a.nchunks):
        if modes[c]:
            continue
        n0 = int(res[c]["svl_off"])
        got = bufs[0][n0:n0 + int(res[c]["svl_total"])]
        assert np.array_equal(got, oa.splats(c, 4)[0]), c
    assert worlds.compare_world(dw, oa, modes, 2) == []


def test_pipelined_rebuilds_reusing_one_buffer_set(ctx):
    """A caller that does not alternate buffer sets still gets each call's
    outputs: the previous call is finished before its records are reused."""
    w = worlds.cave_world(5, (2, 1, 2), seed=33)
    modes = (np.arange(w.nchunks) % 5 == 2).astype(np.uint8)
    ref = gpu.DeviceWorld(ctx, w)
    ref.set_modes(modes)
    want = {}
    for lod in (2, 4):
        res = np.zeros(w.nchunks, gpu.RESULT_DTYPE)
        bufs = [np.zeros(1 << 22, np.int16), np.zeros(1 << 22, np.int16), np.zeros(1 << 21, np.uint32)]
        ref.rebuild_to_host(lod, *bufs, res, slabs=2)
        want[lod] = (res, bufs)
    dw = gpu.DeviceWorld(ctx, w)
    dw.set_modes(modes)
    res = np.zeros(w.nchunks, gpu.RESULT_DTYPE)
    bufs = [np.zeros(1 << 22, np.int16), np.zeros(1 << 22, np.int16), np.zeros(1 << 21, np.uint32)]
    for lod in (4, 2, 4, 2):
        dw.rebuild_to_host_async(lod, *bufs, res, slabs=3)
    dw.outputs_wait()
    assert _same_outputs(want[2][0], want[2][1], res, bufs) is None


def test_handoff_wait_gives_up_and_device_stays_usable(ctx):
    """The decoded-chunk handoff's bounded wait, armed for bytes that no
    copy brings, gives up and reports VP_STATUS_TIMEOUT; the context then
    rebuilds a world bit-exact."""
    assert gpu.selftest_handoff_wait(0) == gpu.VP_STATUS_TIMEOUT
    w = worlds.cave_world(4, (1, 1, 1), seed=2)
    dw = gpu.DeviceWorld(ctx, w)
    assert worlds.compare_world(dw, OracleWorld(w), None, 4) == []
