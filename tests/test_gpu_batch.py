"""Batches of standalone chunks of mixed root sizes (32/64/128) through
vp_batch_*: every strategy (one mixed persistent launch, one launch per root
size, CUDA graph replay, plain per-chunk launches) bit-exact against the
oracle's per-chunk results (each chunk a 1x1x1 ChunkSet, src/chunkset.c:
233-507 with the air null chunk as every neighbour)."""
import numpy as np
import pytest

from oracle.bindings import OracleWorld
from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu
SEED = 5
N = 24
LOD = 4


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


@pytest.fixture(scope="module")
def chunks():
    ws = [wg.uneven_chunk(SEED, k) for k in range(N)]
    assert {w.root_bitw for w in ws} == {5, 6, 7}
    return ws


@pytest.fixture(scope="module")
def expected(chunks):
    modes = (np.arange(N) % 3 == 0).astype(np.uint8)
    out = []
    for k, w in enumerate(chunks):
        o = OracleWorld(w)
        out.append(o.mesh(0) if modes[k] else o.splats(0, LOD))
    return modes, out


def check_batch(b, modes, want):
    res = b.results()
    assert (res["status"] == 0).all()
    for k in range(b.n):
        if modes[k]:
            v, i = b.chunk_mesh(res, k)
            assert np.array_equal(v, want[k][0]) and np.array_equal(i, want[k][1]), k
        else:
            g, items = b.chunk_splats(res, k)
            assert np.array_equal(items[:LOD + 1], want[k][1]), k
            assert np.array_equal(g, want[k][0]), k


# (strategy, min_blocks, order, threads per chunk, chunks per dequeue, CTAs)
@pytest.mark.parametrize("cfg", [("mixed", 2, 0, 512, 1, 0), ("mixed", 1, 0, 512, 1, 0), ("mixed", 2, 1, 512, 1, 0),
                                 ("split", 2, 1, 512, 1, 0), ("mixed", 2, 0, 256, 4, 0), ("mixed", 2, 0, 512, 2, 152),
                                 ("split", 2, 1, 256, 2, 0)])
@pytest.mark.parametrize("mode", ["direct", "graph"])
def test_batch_strategies_match_oracle(ctx, chunks, expected, cfg, mode):
    modes, want = expected
    b = gpu.DeviceBatch(ctx, chunks)
    b.set_modes(modes)
    b.set_tune(cfg[0], min_blocks=cfg[1], order=cfg[2], threads=cfg[3], grain=cfg[4], ctas=cfg[5])
    b.rebuild(LOD, mode=mode)
    b.finish()
    check_batch(b, modes, want)
    if mode == "graph":
        # replays of the captured graph give the same results
        b.rebuild(LOD, mode="graph")
        b.rebuild(LOD, mode="graph")
        b.finish()
        check_batch(b, modes, want)


@pytest.mark.parametrize("mode", ["plain", "concurrent"])
def test_batch_plain_matches_oracle(ctx, chunks, expected, mode):
    modes, want = expected
    b = gpu.DeviceBatch(ctx, chunks)
    b.set_modes(modes)
    b.rebuild(LOD, mode=mode)
    b.finish()
    check_batch(b, modes, want)


def test_batch_autotune_picks_a_timed_config(ctx, chunks, expected):
    modes, want = expected
    b = gpu.DeviceBatch(ctx, chunks)
    b.set_modes(modes)
    best, tried = b.autotune(LOD)
    assert len(tried) >= 8 and all(t["ms"] > 0 for t in tried)
    assert {t["threads"] for t in tried} == {256, 512} and {t["grain"] for t in tried} >= {1, 2, 4}
    assert best["ms"] == min(t["ms"] for t in tried)
    b.rebuild(LOD, mode="graph")
    b.finish()
    check_batch(b, modes, want)
    # a mode change is read by the captured graph from device memory
    flipped = 1 - modes
    b.set_modes(flipped)
    b.rebuild(LOD, mode="graph")
    b.finish()
    res = b.results()
    w = chunks[1]
    assert flipped[1] == 1
    v, i = b.chunk_mesh(res, 1)
    ov, oi = OracleWorld(w).mesh(0)
    assert np.array_equal(v, ov) and np.array_equal(i, oi)


def test_batch_rejects_bad_tunes(ctx, chunks):
    b = gpu.DeviceBatch(ctx, chunks[:4])
    with pytest.raises(gpu.VoxGpuError):
        b.set_tune("split", order=0)
    with pytest.raises(gpu.VoxGpuError):
        b.set_tune("mixed", min_blocks=3)
    with pytest.raises(gpu.VoxGpuError):
        b.set_tune("mixed", threads=384)
    with pytest.raises(gpu.VoxGpuError):
        b.set_tune("mixed", grain=65)
