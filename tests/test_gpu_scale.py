"""GPU parity at the benchmark's own sizes, bit-exact against the oracle:

- the 2048x256x2048 world (32x4x32 = 4096 chunks of 64^3, terrain + caves,
  seed 2024) that bench.py times, every chunk, with its near/far modes,
  LOD 0..4 and grouping (the sequence of src/chunkset.c:337-459 for every
  chunk, and src/gfx/vsplat.c:264-312 for every octree node);
- all 4096 standalone chunks of the uneven batch (roots 32/64/128 in ratio
  1:6:1, seed 3) through the autotuned configuration's CUDA graph;
- a random sample of chunks of the 16384x512x16384 world (524,288 chunks,
  generated on the device) at LOD 0..5.
"""
import ctypes
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import bench
from oracle.bindings import OracleWorld, vpo_lib
from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


def _read_all(dw, res):
    """Every output of the last rebuild, in the arena layout the results index."""
    n_svl = int((res["svl_off"] + res["svl_total"]).max())
    n_vbo = int((res["vbo_off"] + res["vbo_items"]).max())
    n_ibo = int((res["ibo_off"] + res["ibo_items"]).max())
    svl = np.zeros(n_svl + 8, np.int16)
    vbo = np.zeros(n_vbo + 8, np.int16)
    ibo = np.zeros(n_ibo + 4, np.uint32)
    dw.read_outputs(svl, vbo, ibo)
    return svl, vbo, ibo


def _group_nodes_match(dw, res, svl, max_bitw, lod_max, modes):
    """Grouping (gfx_update_svl, src/gfx/vsplat.c:209-331) of the whole world
    against the oracle's restatement over the checked per-chunk outputs."""
    lib = vpo_lib()
    n = len(res)
    empty = np.zeros(1, np.int16)
    ptrs = (ctypes.c_void_p * n)(*[svl.ctypes.data + 2 * int(res[c]["svl_off"]) if not modes[c] else empty.ctypes.data
                                   for c in range(n)])
    items = np.ascontiguousarray(np.where(modes[:, None] != 0, 0, res["svl_items"]), np.uint32)
    iptrs = (ctypes.c_void_p * n)(*[items.ctypes.data + 32 * c for c in range(n)])
    o = OracleWorld.partial(6, max_bitw, wg.DEFAULT_PAD_ROWS, {}, np.zeros(1, np.uint16))
    bad = []
    for lod in range(lod_max + 1):
        ob_ = [b - min(lod, b) for b in max_bitw]
        off, nit = dw.group_nodes(lod)
        want = np.zeros(max(int(items[:, lod].astype(np.int64).sum()), 1), np.int16)
        for idx in range(1 << sum(ob_)):
            node = np.array([idx & ((1 << ob_[0]) - 1), (idx >> ob_[0]) & ((1 << ob_[1]) - 1),
                             idx >> (ob_[0] + ob_[1])], np.uint32)
            m = lib.vpo_group_node(o.h, lod, node.ctypes.data, ctypes.cast(ptrs, ctypes.c_void_p),
                                   ctypes.cast(iptrs, ctypes.c_void_p), want.ctypes.data)
            got = dw.read_group(lod, off[idx], nit[idx])
            if not np.array_equal(got, want[:m]):
                bad.append((lod, idx))
    return bad


def test_bench_world_every_chunk(ctx):
    """Every chunk of the benchmark world, as bench.py rebuilds it."""
    w = bench.make_world()
    modes = bench.mesh_modes(w)
    assert w.nchunks == 4096 and 0 < modes.sum() < w.nchunks
    dw = gpu.DeviceWorld(ctx, w)
    dw.set_modes(modes)
    dw.rebuild(bench.LOD_MAX, group=True)
    dw.finish()
    res = dw.results()
    assert (res["status"] == 0).all()
    svl, vbo, ibo = _read_all(dw, res)
    o = OracleWorld(w)
    bad, nbad = o.check(np.arange(w.nchunks), modes, bench.LOD_MAX, svl, vbo, ibo, res, nthreads=THREADS)
    assert nbad == 0, bad
    # a second rebuild into the same arenas gives the same bytes
    dw.rebuild(bench.LOD_MAX, group=True)
    dw.finish()
    res2 = dw.results()
    svl2, vbo2, ibo2 = _read_all(dw, res2)
    bad, nbad = o.check(np.arange(w.nchunks), modes, bench.LOD_MAX, svl2, vbo2, ibo2, res2, nthreads=THREADS)
    assert nbad == 0, bad
    assert _group_nodes_match(dw, res2, svl2, w.max_bitw, bench.LOD_MAX, modes) == []
    dw.close()


def test_uneven_batch_every_chunk(ctx):
    """All 4096 chunks of the uneven batch (roots 32/64/128, occupancy
    log-uniform 0.1 %..100 %) through the autotuned CUDA-graph replay."""
    with ThreadPoolExecutor(THREADS) as ex:
        ws = list(ex.map(lambda k: wg.uneven_chunk(3, k), range(4096)))
    roots = np.array([w.root_bitw for w in ws])
    assert set(roots.tolist()) == {5, 6, 7}
    b = gpu.DeviceBatch(ctx, ws)
    b.set_modes(None)
    b.autotune(bench.LOD_MAX)
    b.rebuild(bench.LOD_MAX, mode="graph")
    b.finish()
    b.rebuild(bench.LOD_MAX, mode="graph")  # a replay into arenas that hold the last outputs
    b.finish()
    res = b.results()
    assert (res["status"] == 0).all()

    def one(k):
        g, items = b.chunk_splats(res, k)
        og, oitems = OracleWorld(ws[k]).splats(0, bench.LOD_MAX)
        return k if not (np.array_equal(items[:bench.LOD_MAX + 1], oitems) and np.array_equal(g, og)) else None

    # the densest chunks first, so the long oracle runs overlap the rest
    order = np.argsort([-int(w.len[0]) for w in ws])
    with ThreadPoolExecutor(THREADS) as ex:
        bad = [k for k in ex.map(one, order) if k is not None]
    assert bad == []
    # meshes of a sample of the same batch, 128^3 chunks included
    rng = np.random.default_rng(11)
    mesh = np.zeros(len(ws), np.uint8)
    pick = np.concatenate([rng.choice(np.nonzero(roots == r)[0], 24, replace=False) for r in (5, 6, 7)])
    mesh[pick] = 1
    b.set_modes(mesh)
    b.rebuild(bench.LOD_MAX, mode="graph")
    b.finish()
    res = b.results()

    def one_mesh(k):
        v, i = b.chunk_mesh(res, k)
        ov, oi = OracleWorld(ws[k]).mesh(0)
        return k if not (np.array_equal(v, ov) and np.array_equal(i, oi)) else None

    with ThreadPoolExecutor(THREADS) as ex:
        bad = [k for k in ex.map(one_mesh, pick) if k is not None]
    assert bad == []
    b.close()


def test_full_scale_world_sample(ctx):
    """A random sample of the 524,288 chunks of the 16384x512x16384 world
    (generated on the device, LOD 0..5, the benchmark's near/far modes),
    every meshed chunk of the sample included. The oracle gets the sampled
    chunks' 3x3x3 neighbourhoods and the whole shadow map."""
    max_bitw = (8, 3, 8)
    dw = gpu.DeviceWorld.generated(ctx, wg.TERRAIN_CAVES, 6, max_bitw, seed=99, hshift=2)
    n = dw.nchunks
    c = np.arange(n)
    xs, ys, zs = (c & 255) * 64 + 32, ((c >> 8) & 7) * 64 + 32, (c >> 11) * 64 + 32
    modes = (np.sqrt((xs - 8192.0) ** 2 + (ys - 160.0) ** 2 + (zs - 8192.0) ** 2) < bench.MESH_RADIUS)
    modes = modes.astype(np.uint8)
    dw.set_modes(modes)
    dw.rebuild(5, group=True)
    dw.finish()
    res = dw.results()
    assert (res["status"] == 0).all()
    rng = np.random.default_rng(2026)
    sample = np.unique(np.concatenate([rng.choice(n, 2000, replace=False),
                                       rng.choice(np.nonzero(modes)[0], 200, replace=False)])).astype(np.uint32)
    # neighbourhoods of the sample
    need = set()
    for ch in sample.tolist():
        x, y, z = ch & 255, (ch >> 8) & 7, ch >> 11
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if 0 <= x + dx < 256 and 0 <= y + dy < 8 and 0 <= z + dz < 256:
                        need.add(((z + dz) << 11) | ((y + dy) << 8) | (x + dx))
    streams = {k: dw.chunk_rle(k) for k in sorted(need)}
    W, Z = (256 + 8) * 64, 256 * 64
    shadow = dw.shadow(W * (Z + wg.DEFAULT_PAD_ROWS))
    o = OracleWorld.partial(6, max_bitw, wg.DEFAULT_PAD_ROWS, streams, shadow)
    # the sampled chunks' outputs, packed, with offsets rebased to the packs
    sub = res.copy()
    svl, vbo, ibo = [], [], []
    so = vo = io = 0
    for ch in sample.tolist():
        r = res[ch]
        if modes[ch]:
            v, i = dw.chunk_mesh(res, ch)
            sub[ch]["vbo_off"], sub[ch]["ibo_off"] = vo, io
            vbo.append(v)
            ibo.append(i)
            vo += len(v)
            io += len(i)
        else:
            g, _ = dw.chunk_splats(res, ch)
            sub[ch]["svl_off"] = so
            svl.append(g)
            so += len(g)
        assert r["status"] == 0
    svl = np.concatenate(svl) if svl else np.zeros(0, np.int16)
    vbo = np.concatenate(vbo) if vbo else np.zeros(0, np.int16)
    ibo = np.concatenate(ibo) if ibo else np.zeros(0, np.uint32)
    bad, nbad = o.check(sample, modes, 5, svl, vbo, ibo, sub, nthreads=THREADS)
    assert nbad == 0, bad
    assert int(modes[sample].sum()) >= 200
    dw.close()
