"""The device world generator produces exactly the host generator's worlds:
every chunk's RLE stream and the whole padded shadow map."""
import numpy as np
import pytest

from voxplat_gb300 import gpu
from voxplat_gb300 import worldgen as wg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


@pytest.mark.parametrize("kind,rb,mb,seed,hshift", [
    (wg.TERRAIN_SMALL, 6, (1, 0, 1), 1, 0),
    (wg.TERRAIN_SMALL, 5, (2, 2, 1), 3, 1),
    (wg.TERRAIN_CAVES, 5, (1, 3, 1), 7, 0),
    (wg.TERRAIN_CAVES, 6, (2, 2, 2), 2024, 0),
    (wg.TERRAIN_CAVES, 4, (2, 4, 2), 11, 2),
])
def test_device_world_equals_host_world(ctx, kind, rb, mb, seed, hshift):
    host = wg.terrain(kind, rb, mb, seed=seed, hshift=hshift)
    dev = gpu.DeviceWorld.generated(ctx, kind, rb, mb, seed, hshift)
    for c in range(host.nchunks):
        assert np.array_equal(dev.chunk_rle(c), host.chunk_rle(c)), c
    assert np.array_equal(dev.shadow(len(host.shadow)), host.shadow)
    assert dev.rle_bytes() == int(host.len.astype(np.int64).sum()) * 4
