"""The CUDA pipeline against the reference's own outputs (golden fixtures
made by tests/golden/make_golden.py from the compiled reference sources)."""
import glob
import os

import numpy as np
import pytest

from tests import worlds
from voxplat_gb300 import gpu

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GEOM = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
              if not os.path.basename(p).startswith(("rle_", "edits_")))


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


@pytest.mark.parametrize("path", GEOM, ids=[os.path.basename(p)[:-4] for p in GEOM])
def test_gpu_matches_reference_outputs(ctx, path):
    w, d = worlds.load_fixture(path)
    dw = gpu.DeviceWorld(ctx, w)
    n = w.nchunks
    for key in d:
        if not (key.startswith("svl") and key.endswith("_items")):
            continue
        lod = int(key[3:-6])
        items = d[key]
        pieces = worlds.split(d["svl%d" % lod], items.sum(axis=1))
        dw.set_modes(None)
        dw.rebuild(lod_max=lod)
        dw.finish()
        res = dw.results()
        for c in range(n):
            g, it = dw.chunk_splats(res, c)
            assert np.array_equal(it[:lod + 1], items[c]), (c, lod)
            assert np.array_equal(g, pieces[c]), (c, lod)
    if "vbo" in d:
        dw.set_modes(np.ones(n, np.uint8))
        dw.rebuild(lod_max=4)
        dw.finish()
        res = dw.results()
        vb = worlds.split(d["vbo"], d["vbo_items"])
        ib = worlds.split(d["ibo"], d["ibo_items"])
        for c in range(n):
            v, i = dw.chunk_mesh(res, c)
            assert np.array_equal(v, vb[c]), c
            assert np.array_equal(i, ib[c]), c
