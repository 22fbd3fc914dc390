"""Picking rays (chunkset_edit_raycast_until_solid, src/chunkset/edit.c:
248-314): the oracle's restatement bit-exact against the compiled reference
on a cave world, including rays along axes (zero components), rays that
leave the world and rays starting outside it."""
import numpy as np
import pytest

from oracle import bindings as ob
from tests import worlds


def rays(rng, extent, n):
    out = []
    for k in range(n):
        o = rng.uniform([-20, 0, -20], [extent[0] + 20, extent[1] + 40, extent[2] + 20]).astype(np.float32)
        v = rng.normal(size=3).astype(np.float32)
        if k % 5 == 0:
            v[rng.integers(0, 3)] = 0.0       # in a coordinate plane
        if k % 11 == 0:
            v = np.zeros(3, np.float32)
            v[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])   # along an axis
        if k % 7 == 0:
            v[1] = -abs(v[1]) - 0.5            # downwards, into the terrain
        out.append((o, v))
    return out


@pytest.mark.parametrize("root_bitw,max_bitw", [(4, (2, 3, 2)), (5, (1, 2, 1))])
def test_oracle_raycast_matches_reference(root_bitw, max_bitw):
    if ob.ref_lib() is None:
        pytest.skip("reference tree not present")
    w = worlds.cave_world(root_bitw, max_bitw, seed=13)
    o, r = ob.OracleWorld(w), ob.RefWorld(w)
    extent = [w.R << b for b in max_bitw]
    hits = 0
    for k, (org, vec) in enumerate(rays(np.random.default_rng(root_bitw), extent, 300)):
        a, b = o.raycast(org, vec), r.raycast(org, vec)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), (k, org, vec, a, b)
        hits += a[0] > 0
    assert hits > 50
