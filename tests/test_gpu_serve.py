"""The edit server (vp_server_*): continuous batching with several
independent batches on the GPU at once. Its results must equal serial
application of the same edits in submission order (the reference applies
edits one after the other, src/chunkset/edit.c:179-244, and remeshes the
dirty chunks on the next mesher tick, src/chunkset.c:246-309), each edit's
result must be the same alone and in the mix, and admission must refuse
what does not fit instead of waiting for ever."""
import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from voxplat_gb300 import gpu

pytestmark = pytest.mark.gpu
LOD = 4
VP_ENOMEM = -2


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


def edit_rows(rng, n, extent, rmax, fills=True):
    rows = np.zeros((n, 5), np.int64)
    for i in range(n):
        rows[i, :3] = [rng.integers(0, e) for e in extent]
        rows[i, 3] = rng.integers(1, rmax + 1)
        rows[i, 4] = rng.integers(1, 256) if (fills and rng.random() < 0.5) else 0
    return rows


def fresh(ctx, w, modes):
    dw = gpu.DeviceWorld(ctx, w)
    dw.set_modes(modes)
    dw.rebuild(lod_max=LOD)
    dw.finish()
    return dw


def outputs(dw):
    res = dw.results()
    n_svl = int((res["svl_off"] + res["svl_total"]).max()) + 8
    n_vbo = int((res["vbo_off"] + res["vbo_items"]).max()) + 8
    n_ibo = int((res["ibo_off"] + res["ibo_items"]).max()) + 4
    svl, vbo, ibo = np.zeros(n_svl, np.int16), np.zeros(n_vbo, np.int16), np.zeros(n_ibo, np.uint32)
    dw.read_outputs(svl, vbo, ibo)
    return svl, vbo, ibo, res


def chunk_geometry(dw, res, modes, c):
    return dw.chunk_mesh(res, c) if modes[c] else (dw.chunk_splats(res, c)[0],)


def test_overlapping_batches_equal_serial_application(ctx):
    """Many small batches submitted at once: independent ones run together
    on the GPU; the world (streams, shadow map, geometry of every chunk)
    equals edits applied one by one, and the oracle's."""
    w = worlds.cave_world(5, (3, 2, 3), seed=91)  # 256 x 128 x 256 voxels, 32^3 chunks
    n = w.nchunks
    modes = (np.arange(n) % 4 == 0).astype(np.uint8)
    rng = np.random.default_rng(17)
    rows = edit_rows(rng, 48, [256, 128, 256], 10)
    served = fresh(ctx, w, modes)
    srv = gpu.EditServer(served, slots=4, max_batch=2, slot_chunks=64)
    first = srv.submit(gpu.make_edits(rows))
    srv.drain()
    done = srv.poll(cap=256)
    st, nslots = srv.stats()
    srv.close()
    assert first == 0 and sorted(done["ticket"].tolist()) == list(range(len(rows)))
    assert (done["status"] == 0).all()
    assert st.edits == len(rows) and st.max_inflight >= 2, (st.max_inflight, nslots)
    serial = fresh(ctx, w, modes)
    o = OracleWorld(w)
    for r in rows:
        serial.edit(gpu.make_edits([r]))
        o.edit_sphere(r[:3], int(r[3]), int(r[4]))
    for c in range(n):
        assert np.array_equal(served.chunk_rle(c), serial.chunk_rle(c)), c
    assert np.array_equal(served.shadow(len(w.shadow)), serial.shadow(len(w.shadow)))
    assert np.array_equal(served.shadow(len(w.shadow)), o.shadow_map())
    # the geometry the served world holds now (only dirty chunks were
    # remeshed, the rest is from the first rebuild) against serial's
    ra, rb = served.results(), serial.results()
    for c in range(n):
        ga, gb = chunk_geometry(served, ra, modes, c), chunk_geometry(serial, rb, modes, c)
        assert all(np.array_equal(x, y) for x, y in zip(ga, gb)), c
    # and a full rebuild of the served world against the oracle after the edits
    served.rebuild(lod_max=LOD)
    served.finish()
    svl, vbo, ibo, res = outputs(served)
    bad, nbad = o.check(np.arange(n), modes, LOD, svl, vbo, ibo, res)
    assert nbad == 0, bad


def test_each_edit_same_alone_and_in_the_mix(ctx):
    """Carves spread over the world (so no two touch the same chunks, and
    carves leave the shadow map alone): the streams and geometry of each
    edit's dirty chunks are the same when it runs alone as when it runs in
    the mix, with batches overlapping on the GPU."""
    w = worlds.cave_world(5, (3, 1, 3), seed=93)  # 256 x 64 x 256
    n = w.nchunks
    modes = (np.arange(n) % 3 == 0).astype(np.uint8)
    rows = []
    for gx in range(4):
        for gz in range(4):
            rows.append([gx * 64 + 20, 40, gz * 64 + 20, 6 + (gx + gz) % 5, 0])
    rows = np.array(rows, np.int64)
    mix = fresh(ctx, w, modes)
    srv = gpu.EditServer(mix, slots=4, max_batch=1, slot_chunks=64)
    srv.submit(gpu.make_edits(rows))
    srv.drain()
    st, _ = srv.stats()
    srv.close()
    assert st.max_inflight >= 2
    rm = mix.results()
    for k, r in enumerate(rows):
        alone = fresh(ctx, w, modes)
        alone.edit(gpu.make_edits([r]))
        dirty = alone.dirty()
        ra = alone.results()
        for c in dirty.tolist():
            assert np.array_equal(alone.chunk_rle(c), mix.chunk_rle(c)), (k, c)
            ga, gm = chunk_geometry(alone, ra, modes, c), chunk_geometry(mix, rm, modes, c)
            assert all(np.array_equal(x, y) for x, y in zip(ga, gm)), (k, c)
        alone.close()


def test_server_refuses_an_edit_larger_than_a_slot(ctx):
    w = worlds.cave_world(5, (2, 2, 2), seed=95)
    dw = fresh(ctx, w, None)
    before = [dw.chunk_rle(c) for c in range(w.nchunks)]
    srv = gpu.EditServer(dw, slots=2, max_batch=4, slot_chunks=4)
    big = [60, 60, 60, 40, 7]      # its AABB covers 64 chunks of 32^3
    small = [10, 20, 10, 3, 0]     # one chunk
    srv.submit(gpu.make_edits([big, small]))
    srv.drain()
    done = srv.poll()
    srv.close()
    status = {int(t): int(s) for t, s in zip(done["ticket"], done["status"])}
    assert status == {0: VP_ENOMEM, 1: 0}
    serial = fresh(ctx, w, None)
    serial.edit(gpu.make_edits([small]))
    for c in range(w.nchunks):
        assert np.array_equal(dw.chunk_rle(c), serial.chunk_rle(c)), c
    assert any(not np.array_equal(dw.chunk_rle(c), before[c]) for c in range(w.nchunks))


def test_admission_without_memory_fails_instead_of_waiting(ctx):
    """A reserve larger than the device: no slot fits, so creating the
    server (and replaying a trace) returns VP_ENOMEM at once."""
    w = worlds.cave_world(4, (1, 1, 1), seed=97)
    dw = fresh(ctx, w, None)
    with pytest.raises(gpu.VoxGpuError, match="vp_server_create"):
        gpu.EditServer(dw, slots=2, max_batch=4, slot_chunks=64, hbm_reserve=1 << 60)
    e = gpu.make_edits([[10, 20, 10, 4, 3]], np.array([0.0]))
    with pytest.raises(gpu.VoxGpuError, match="vp_world_serve"):
        dw.serve(e, max_batch=4, hbm_reserve=1 << 60)
    # the world still works
    dw.edit(e)
    assert len(dw.dirty()) > 0
