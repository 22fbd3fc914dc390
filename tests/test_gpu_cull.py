"""Draw culling and LOD selection on the device (vp_world_cull,
vp_world_camera_modes) against the oracle's octree walk (src/game.c:
319-395, 517-524, 612-625) on the 2048x256x2048 world: same queues, same
order, for many cameras."""
import numpy as np
import pytest

from oracle import bindings as ob
from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu
MB = (5, 2, 5)


@pytest.fixture(scope="module")
def world():
    ctx = gpu.Context(0)
    dw = gpu.DeviceWorld.generated(ctx, wg.TERRAIN_CAVES, 6, MB, 2024, 0)
    return ctx, dw


def cameras():
    rng = np.random.default_rng(17)
    cams = []
    for _ in range(24):
        eye = rng.uniform([-300, 20, -300], [2400, 700, 2400]).astype(np.float32)
        target = eye + rng.normal(size=3) * 100
        cams.append((eye, ob.perspective_view(eye, target, fov_deg=float(rng.uniform(40, 100)))))
    eye = np.array([1024, 5000, 1024], np.float32)
    cams.append((eye, ob.perspective_view(eye, [1024, 0, 1024.5], fov_deg=90, far=100000)))  # everything
    eye = np.array([1024, 160, 1024], np.float32)
    cams.append((eye, ob.perspective_view(eye, [1024, 1000, 1024.5])))                         # sky only
    return cams


def test_camera_modes_match_oracle(world):
    ctx, dw = world
    for eye, _ in cameras()[:6]:
        assert np.array_equal(dw.camera_modes(eye), ob.mesh_flags(6, MB, eye))


def test_cull_queues_match_oracle(world):
    ctx, dw = world
    n = dw.nchunks
    for k, (eye, vp) in enumerate(cameras()):
        modes = dw.camera_modes(eye)
        dw.rebuild(lod_max=4, group=True)
        dw.finish()
        res = dw.results()
        has_mesh = (res["vbo_items"] > 0).astype(np.uint8)
        items = [dw.group_nodes(l)[1] for l in range(5)]
        want_m, want_s, _ = ob.octree_cull(6, MB, ob.fcull_extract_planes(vp), eye, has_mesh, items)
        got_m, got_s = dw.cull(vp, eye)
        assert np.array_equal(got_m, want_m), k
        assert np.array_equal(got_s, want_s), k
        assert modes.sum() >= len(got_m)


def test_cull_needs_grouped_lists(world):
    ctx, dw = world
    dw.rebuild(lod_max=4)
    dw.finish()
    eye = np.array([1000, 150, 1000], np.float32)
    with pytest.raises(gpu.VoxGpuError):
        dw.cull(ob.perspective_view(eye, [0, 0, 0]), eye)
