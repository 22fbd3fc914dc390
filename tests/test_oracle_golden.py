"""The oracle (C restatement, oracle/vpo.c) against golden fixtures produced
by the reference's own hot-path sources (tests/golden/make_golden.py):
bit-exact splat lists per LOD, quad meshes, RLE codec and sphere edits."""
import glob
import os

import numpy as np
import pytest

from oracle import bindings as ob
from tests import worlds

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GEOM = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
              if not os.path.basename(p).startswith(("rle_", "edits_")))


def test_fixtures_present():
    assert len(GEOM) >= 5


@pytest.mark.parametrize("path", GEOM, ids=[os.path.basename(p)[:-4] for p in GEOM])
def test_oracle_geometry_matches_reference(path):
    w, d = worlds.load_fixture(path)
    o = ob.OracleWorld(w)
    n = w.nchunks
    for key in d:
        if not (key.startswith("svl") and key.endswith("_items")):
            continue
        lod = int(key[3:-6])
        items = d[key]
        pieces = worlds.split(d["svl%d" % lod], items.sum(axis=1))
        for c in range(n):
            g, it = o.splats(c, lod)
            assert np.array_equal(it, items[c]), (c, lod)
            assert np.array_equal(g, pieces[c]), (c, lod)
    if "vbo" in d:
        vb = worlds.split(d["vbo"], d["vbo_items"])
        ib = worlds.split(d["ibo"], d["ibo_items"])
        for c in range(n):
            v, i = o.mesh(c)
            assert np.array_equal(v, vb[c]), c
            assert np.array_equal(i, ib[c]), c


def test_oracle_rle_matches_reference():
    d = dict(np.load(os.path.join(GOLDEN, "rle_codec.npz")))
    names = [k[3:] for k in d if k.startswith("in_")]
    assert names
    for nm in names:
        v = d["in_" + nm]
        enc = ob.vpo_rle_encode(v)
        assert np.array_equal(enc, d["out_" + nm]), nm
        assert np.array_equal(ob.vpo_rle_decode(enc, len(v)), v), nm


def test_oracle_sphere_edits_match_reference():
    w, d = worlds.load_fixture(os.path.join(GOLDEN, "edits_r16.npz"))
    o = ob.OracleWorld(w)
    for e, (x, y, z, r, v) in enumerate(d["edits"]):
        dirty = o.edit_sphere((x, y, z), int(r), int(v))
        assert np.array_equal(dirty, d["dirty%d" % e]), e
    for c in range(w.nchunks):
        assert np.array_equal(o.voxels(c), d["voxels"][c]), c
    assert np.array_equal(o.shadow_map(), d["shadow_after"])
    post = worlds.world_from_voxels(w.root_bitw, w.max_bitw, list(d["voxels"]), shadow=d["shadow_after"],
                                    pad_rows=w.pad_rows)
    op = ob.OracleWorld(post)
    pieces = worlds.split(d["post_svl4"], d["post_svl4_items"].sum(axis=1))
    for c in range(post.nchunks):
        g, it = op.splats(c, 4)
        assert np.array_equal(g, pieces[c]), c
