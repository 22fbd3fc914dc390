"""The drop-in entry points (include/voxgpu_dropin.h), called the way the
reference's chunkset.c calls its own mesher, against the oracle: per-chunk
mask/downsample/splat chains and meshes for chunks held as RLE or as
decoded voxels, the batched chunkset_manage with its published fields, and
the rle_compress / rle_decompress pair."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle.bindings import OracleWorld
from tests import worlds
from voxplat_gb300 import build

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
V = ctypes.c_void_p


@pytest.fixture(scope="module")
def harness():
    lib = build.build_cuda()
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libdropin_harness.so")
    subprocess.check_call(["gcc", "-O1", "-shared", "-fPIC", "-o", so, os.path.join(HERE, "dropin_harness.c"),
                           "-I", os.path.join(ROOT, "include"), lib, "-Wl,-rpath," + os.path.dirname(lib),
                           "-lpthread"])
    h = ctypes.CDLL(so)
    h.harness_new.restype = V
    h.harness_new.argtypes = [ctypes.c_int, V, V, V, V, V, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                              ctypes.c_int]
    h.harness_splats.restype = ctypes.c_long
    h.harness_splats.argtypes = [V, ctypes.c_uint32, ctypes.c_int, V, V]
    h.harness_mesh.restype = ctypes.c_long
    h.harness_mesh.argtypes = [V, ctypes.c_uint32, V, V, V, V]
    h.harness_manage.argtypes = [V, V]
    h.harness_published.argtypes = [V, ctypes.c_uint32, V, V, V, V]
    h.harness_copy_published.argtypes = [V, ctypes.c_uint32, V, V, V]
    h.harness_rle.restype = ctypes.c_uint32
    h.harness_rle.argtypes = [V, ctypes.c_uint32, V, V]
    return h


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def make(h, w, decoded):
    mb = np.array(w.max_bitw, np.int32)
    return h.harness_new(w.root_bitw, _p(mb), _p(w.pool), _p(w.off), _p(w.len), _p(w.shadow),
                         w.shadow_w * w.shadow_z, w.shadow_w, w.shadow_z, 1 if decoded else 0)


@pytest.mark.parametrize("decoded", [False, True])
def test_per_chunk_dropins_match_oracle(harness, decoded):
    w = worlds.cave_world(4, (1, 2, 1), seed=44)
    o = OracleWorld(w)
    hs = make(harness, w, decoded)
    R = w.R
    for c in range(w.nchunks):
        geom = np.zeros(4 * 2 * (R + 1) ** 3, np.int16)
        items = np.zeros(8, np.uint32)
        n = harness.harness_splats(hs, c, 4, _p(geom), _p(items))
        assert n >= 0
        og, oitems = o.splats(c, 4)
        assert np.array_equal(items[:5], oitems), c
        assert np.array_equal(geom[:n], og), c
        vbo = np.zeros(3 * R ** 3 * 16, np.int16)
        ibo = np.zeros(3 * R ** 3 * 6, np.uint32)
        nv = np.zeros(1, np.uint32)
        ni = np.zeros(1, np.uint32)
        assert harness.harness_mesh(hs, c, _p(vbo), _p(nv), _p(ibo), _p(ni)) >= 0
        ov, oi = o.mesh(c)
        assert np.array_equal(vbo[:nv[0]], ov), c
        assert np.array_equal(ibo[:ni[0]], oi), c


def test_chunkset_manage_publishes_reference_results(harness):
    w = worlds.cave_world(4, (2, 2, 1), seed=45)
    o = OracleWorld(w)
    hs = make(harness, w, True)
    modes = (np.arange(w.nchunks) % 3 == 1).astype(np.uint8)
    assert harness.harness_manage(hs, _p(modes)) == 0
    for c in range(w.nchunks):
        items = np.zeros(5, np.uint32)
        nv, ni, fl = (np.zeros(1, np.uint32) for _ in range(3))
        harness.harness_published(hs, c, _p(items), _p(nv), _p(ni), _p(fl))
        flags = int(fl[0])
        assert flags & 8 == 0 and flags & 16 == 0  # dirty and changing cleared
        if modes[c]:
            ov, oi = o.mesh(c)
            assert flags & 2  # mesh_dirty
            assert nv[0] == len(ov) and ni[0] == len(oi)
            vbo = np.zeros(max(len(ov), 1), np.int16)
            ibo = np.zeros(max(len(oi), 1), np.uint32)
            harness.harness_copy_published(hs, c, None, _p(vbo), _p(ibo))
            assert np.array_equal(vbo[:len(ov)], ov) and np.array_equal(ibo[:len(oi)], oi)
        else:
            og, oitems = o.splats(c, 4)
            assert flags & 1  # svl_dirty
            assert np.array_equal(items, oitems)
            assert bool(flags & 4) == (len(og) == 0)
            svl = np.zeros(max(len(og), 1), np.int16)
            harness.harness_copy_published(hs, c, _p(svl), None, None)
            assert np.array_equal(svl[:len(og)], og)


def test_rle_dropins(harness):
    rng = np.random.default_rng(3)
    for n in (1, 100, 4096, 262144):
        v = np.repeat(rng.integers(0, 4, n).astype(np.uint8), rng.integers(1, 9, n))[:n]
        out = np.zeros(n + 2, np.uint32)
        back = np.zeros(n, np.uint8)
        k = harness.harness_rle(_p(v), n, _p(out), _p(back))
        from oracle.bindings import vpo_rle_encode
        assert np.array_equal(out[:k], vpo_rle_encode(v))
        assert np.array_equal(back, v)
