"""The CUDA rasteriser (vp_world_render) against the oracle's software
rasteriser of the same shaders (resources/splat.*.glsl, resources/mesh.*.glsl):
identical frames (RGBA8 and depth bits) for the draw queues of several
cameras, meshes near the camera and splats of several LODs farther away."""
import numpy as np
import pytest

from oracle import bindings as ob
from tests import worlds
from voxplat_gb300 import gpu
from voxplat_gb300.camera import camera

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


def oracle_frame(dw, cam, mq, sq, res):
    f = ob.Frame(cam)
    for c in mq:
        v, i = dw.chunk_mesh(res, int(c))
        f.mesh(v, i)
    offs = {}
    for e in sq:
        lod, node = int(e) >> 24, int(e) & 0xFFFFFF
        if lod not in offs:
            offs[lod] = dw.group_nodes(lod)
        off, items = offs[lod]
        f.splats(dw.read_group(lod, off[node], items[node]), lod)
    return f


CAMS = [
    ((100, 90, -60), (64, 30, 64), 70),     # near: meshes
    ((64, 700, 64), (64, 0, 64.5), 60),     # above, farther than 512: lod-0 splats
    ((-900, 900, -900), (64, 30, 64), 12),  # far: coarser splat levels
    ((70, 40, 70), (0, 20, 120), 100),      # inside the world, wide angle
]


@pytest.mark.parametrize("k", range(len(CAMS)))
def test_frames_match_oracle(ctx, k):
    w = worlds.cave_world(5, (2, 1, 2), seed=19)
    dw = gpu.DeviceWorld(ctx, w)
    eye, target, fov = CAMS[k]
    eye = np.array(eye, np.float32)
    dw.camera_modes(eye)
    dw.rebuild(lod_max=4, group=True)
    dw.finish()
    res = dw.results()
    cam = camera(eye, target, 320, 200, fov_deg=fov, far=4096.0)
    mq, sq = dw.cull(cam["view_projection"], eye)
    assert len(mq) + len(sq) > 0
    rgba, depth, stats = dw.render(cam, mq, sq)
    f = oracle_frame(dw, cam, mq, sq, res)
    drawn = int((f.depth < 1.0).sum())
    assert drawn > 500, drawn
    assert np.array_equal(rgba, f.rgba), int((rgba != f.rgba).sum())
    assert np.array_equal(depth.view(np.uint32), f.depth.view(np.uint32))


def test_frame_into_caller_arrays(ctx):
    """render(out=...) writes the same frame into the caller's arrays (here
    page-locked, reused for a second frame) and rejects mismatched ones."""
    import torch
    w = worlds.cave_world(5, (2, 1, 2), seed=19)
    dw = gpu.DeviceWorld(ctx, w)
    eye, target, fov = CAMS[0]
    eye = np.array(eye, np.float32)
    dw.camera_modes(eye)
    dw.rebuild(lod_max=4, group=True)
    dw.finish()
    cam = camera(eye, target, 320, 200, fov_deg=fov, far=4096.0)
    mq, sq = dw.cull(cam["view_projection"], eye)
    want_rgba, want_depth, want_stats = dw.render(cam, mq, sq)
    host_rgba = torch.empty((200, 320), dtype=torch.int32).pin_memory()
    host_depth = torch.empty((200, 320), dtype=torch.float32).pin_memory()
    out = (host_rgba.numpy().view(np.uint32), host_depth.numpy())
    for _ in range(2):
        rgba, depth, stats = dw.render(cam, mq, sq, out=out)
        assert rgba is out[0] and depth is out[1]
        assert np.array_equal(rgba, want_rgba)
        assert np.array_equal(depth.view(np.uint32), want_depth.view(np.uint32))
        assert np.array_equal(stats, want_stats)
    with pytest.raises(ValueError):
        dw.render(cam, mq, sq, out=(np.zeros((200, 321), np.uint32), np.zeros((200, 320), np.float32)))
    dw.close()
