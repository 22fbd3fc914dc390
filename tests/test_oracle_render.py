"""The oracle's software rasteriser on its own (CPU): a cave world's meshes
and grouped splats from a few cameras draw depth-tested, fogged pixels, and
the result does not depend on draw order."""
import numpy as np

from oracle import bindings as ob
from tests import worlds
from voxplat_gb300.camera import camera


def test_oracle_frame_is_order_independent_and_shaded():
    w = worlds.cave_world(4, (2, 2, 2), seed=5)
    o = ob.OracleWorld(w)
    cam = camera((90, 80, -40), (32, 20, 32), 160, 100, fov_deg=70, far=2048.0)
    meshes = [o.mesh(c) for c in range(w.nchunks)]
    splats = [o.splats(c, 2) for c in range(w.nchunks)]
    a, b = ob.Frame(cam), ob.Frame(cam)
    for c in range(w.nchunks):
        a.mesh(*meshes[c])
    for c in reversed(range(w.nchunks)):
        b.mesh(*meshes[c])
    assert np.array_equal(a.words, b.words)
    assert (a.depth < 1.0).sum() > 1000
    for c in range(w.nchunks):
        g, items = splats[c]
        a.splats(g[:items[0]], 0)
    assert (a.depth < 1.0).sum() > 1000
    px = a.rgba[a.depth < 1.0]
    assert len(np.unique(px)) > 10
