"""Where the reference tree is present, pin the oracle against the compiled
reference sources on more seeds than the committed fixtures hold."""
import numpy as np
import pytest

from oracle import bindings as ob
from tests import worlds
from voxplat_gb300 import worldgen as wg

ref = pytest.mark.skipif(ob.ref_lib() is None, reason="reference sources not present")


@ref
@pytest.mark.parametrize("seed", [101, 202, 303])
def test_oracle_vs_reference_caves(seed):
    w = worlds.cave_world(4, (1, 3, 2), seed=seed)
    o, r = ob.OracleWorld(w), ob.RefWorld(w)
    for c in range(w.nchunks):
        g1, i1 = o.splats(c, 5)
        g2, i2 = r.splats(c, 5)
        assert np.array_equal(i1, i2) and np.array_equal(g1, g2), c
        v1, b1 = o.mesh(c)
        v2, b2 = r.mesh(c)
        assert np.array_equal(v1, v2) and np.array_equal(b1, b2), c


@ref
@pytest.mark.parametrize("k", [1, 4, 9, 13])
def test_oracle_vs_reference_uneven(k):
    if wg.uneven_root_bitw(8, k) > 6:
        pytest.skip("large chunk")
    w = wg.uneven_chunk(8, k)
    o, r = ob.OracleWorld(w), ob.RefWorld(w)
    g1, i1 = o.splats(0, 4)
    g2, i2 = r.splats(0, 4)
    assert np.array_equal(g1, g2)
    v1, b1 = o.mesh(0)
    v2, b2 = r.mesh(0)
    assert np.array_equal(v1, v2) and np.array_equal(b1, b2)


@ref
def test_oracle_vs_reference_random_edits():
    w = worlds.cave_world(4, (2, 2, 2), seed=17)
    o, r = ob.OracleWorld(w), ob.RefWorld(w)
    rng = np.random.default_rng(5)
    for _ in range(12):
        c = rng.integers(0, 64, 3)
        rad = int(rng.integers(1, 14))
        v = int(rng.integers(0, 256)) if rng.random() < 0.5 else 0
        assert np.array_equal(o.edit_sphere(c, rad, v), r.edit_sphere(c, rad, v))
    for ch in range(w.nchunks):
        assert np.array_equal(o.voxels(ch), r.voxels(ch)), ch
    assert np.array_equal(o.shadow_map(), r.shadow())


@ref
def test_oracle_vs_reference_rle():
    rng = np.random.default_rng(2)
    for n in (1, 2, 64, 4096, 32768):
        v = rng.integers(0, 3, n).astype(np.uint8)
        assert np.array_equal(ob.vpo_rle_encode(v), ob.ref_rle_compress(v))
