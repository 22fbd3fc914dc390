"""The VPW1 world file: round trip through the NumPy reader/writer (CPU)."""
import numpy as np

from tests import worlds
from voxplat_gb300 import worldgen as wg


def test_world_file_round_trip(tmp_path):
    w = worlds.cave_world(4, (2, 3, 2), seed=3)
    p = tmp_path / "w.vpw"
    w.save(p)
    v = wg.World.load(p)
    assert (v.root_bitw, v.max_bitw, v.shadow_w, v.shadow_z, v.pad_rows) == \
        (w.root_bitw, w.max_bitw, w.shadow_w, w.shadow_z, w.pad_rows)
    assert np.array_equal(v.shadow, w.shadow)
    for c in range(w.nchunks):
        assert np.array_equal(v.chunk_rle(c), w.chunk_rle(c))
        assert int(v.off[c]) % 4 == 0
    raw = p.read_bytes()
    assert raw[:4] == b"VPW1"
    assert len(raw) == 64 + 12 * w.nchunks + 4 * len(v.pool) + 2 * len(w.shadow)


def test_world_file_rejects_other_files(tmp_path):
    p = tmp_path / "x.bin"
    p.write_bytes(b"\\0" * 128)
    try:
        wg.World.load(p)
    except ValueError:
        return
    raise AssertionError("accepted a file without the magic")
