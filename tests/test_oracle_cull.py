"""Draw culling and LOD selection in the oracle: the frustum functions
bit-exact against the reference's own src/gfx/fcull.c (compiled into the
reference library), and properties of the octree walk (src/game.c:
319-395)."""
import numpy as np
import pytest

from oracle import bindings as ob


def random_view_proj(rng):
    eye = rng.uniform([-500, 0, -500], [2500, 600, 2500])
    target = eye + rng.normal(size=3) * 100
    return ob.perspective_view(eye, target, fov_deg=float(rng.uniform(30, 110)),
                               aspect=float(rng.uniform(0.5, 2.5)))


def test_planes_and_visibility_match_the_reference():
    if ob.ref_lib() is None:
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(3)
    for _ in range(200):
        m = random_view_proj(rng)
        if rng.random() < 0.3:
            m = (m + rng.normal(size=16) * 0.1).astype(np.float32)
        p = ob.fcull_extract_planes(m)
        assert np.array_equal(p.view(np.uint32), ob.ref_fcull_extract_planes(m).view(np.uint32))
        for _ in range(20):
            loc = rng.uniform(-3000, 5000, 3).astype(np.float32)
            r = float(rng.choice([54.4, 108.8, 217.6, 435.2, 870.4]))
            assert ob.fcull_visible(p, loc, r) == ob.ref_fcull_visible(p, loc, r)


def _walk(origin, view_proj, mb=(5, 2, 5), rb=6, items=None, mesh=None):
    n = 1 << sum(mb)
    if mesh is None:
        mesh = np.zeros(n, np.uint8)
    if items is None:
        items = [np.ones(n, np.uint32) for _ in range(5)]
    return ob.octree_cull(rb, mb, ob.fcull_extract_planes(view_proj), origin, mesh, items)


def test_walk_covers_each_chunk_at_most_once_and_picks_lods_by_distance():
    rng = np.random.default_rng(5)
    mb = (5, 2, 5)
    for _ in range(20):
        eye = rng.uniform([0, 50, 0], [2048, 300, 2048]).astype(np.float32)
        vp = ob.perspective_view(eye, eye + rng.normal(size=3) * 50)
        mq, sq, visits = _walk(eye, vp, mb)
        assert len(mq) == 0 and visits > 0
        covered = np.zeros((1 << mb[2], 1 << mb[1], 1 << mb[0]), np.int32)
        for e in sq:
            lod, node = int(e) >> 24, int(e) & 0xFFFFFF
            ob_ = [b - min(lod, b) for b in mb]
            x = node & ((1 << ob_[0]) - 1)
            y = (node >> ob_[0]) & ((1 << ob_[1]) - 1)
            z = node >> (ob_[0] + ob_[1])
            covered[z << lod:(z + 1) << lod, y << lod:(y + 1) << lod, x << lod:(x + 1) << lod] += 1
            ws = 64 << lod
            centre = np.array([x * ws + ws // 2, y * ws + ws // 2, z * ws + ws // 2], np.float32)
            d = np.float32(np.sqrt(np.float32(((centre - eye) ** 2).sum())))
            assert lod == 0 or d > lod * 1024
        assert covered.max() <= 1


def test_camera_far_away_draws_top_level_nodes_only():
    eye = np.array([1024, 20000, 1024], np.float32)
    vp = ob.perspective_view(eye, [1024, 0, 1024.5], fov_deg=90, far=100000)
    mq, sq, _ = _walk(eye, vp)
    assert len(sq) > 0 and all((int(e) >> 24) == 4 for e in sq)


def test_mesh_queue_and_missing_splats():
    mb = (5, 2, 5)
    n = 1 << sum(mb)
    eye = np.array([1000, 150, 1000], np.float32)
    vp = ob.perspective_view(eye, [1400, 100, 1400])
    flags = ob.mesh_flags(6, mb, eye)
    assert 0 < flags.sum() < n
    items = [np.ones(n, np.uint32) for _ in range(5)]
    items[0][:] = 0  # no chunk-level splats: near chunks without a mesh draw nothing
    mq, sq, _ = _walk(eye, vp, mb, items=items, mesh=flags)
    assert len(mq) > 0 and all(flags[int(c)] for c in mq)
    assert all((int(e) >> 24) > 0 for e in sq)
