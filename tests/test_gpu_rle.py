"""RLE codec kernels against the reference encodings (golden fixture) and
the oracle, including edge cases the reference format has: single voxels,
lengths that are not multiples of 16, one uniform run, alternating runs,
all 256 colours."""
import os

import numpy as np
import pytest

from oracle import bindings as ob
from voxplat_gb300 import gpu

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rle_codec.npz")


@pytest.fixture(scope="module")
def ctx():
    return gpu.Context(0)


def test_encode_matches_reference(ctx):
    d = np.load(GOLDEN)
    for k in d.files:
        if k.startswith("in_"):
            enc = ctx.rle_encode(d[k])
            assert np.array_equal(enc, d["out_" + k[3:]]), k
            assert np.array_equal(ctx.rle_decode(enc), d[k]), k


@pytest.mark.parametrize("n", [1, 2, 15, 16, 17, 31, 4095, 4096, 8193, 262144, 2097152])
def test_roundtrip_sizes(ctx, n):
    rng = np.random.default_rng(n)
    for kind in ("random", "runs", "uniform", "alternating"):
        if kind == "random":
            v = rng.integers(0, 256, n).astype(np.uint8)
        elif kind == "runs":
            v = np.repeat(rng.integers(0, 5, n).astype(np.uint8), rng.integers(1, 40, n))[:n]
        elif kind == "uniform":
            v = np.full(n, 9, np.uint8)
        else:
            v = (np.arange(n) % 2 * 255).astype(np.uint8)
        enc = ctx.rle_encode(v)
        assert np.array_equal(enc, ob.vpo_rle_encode(v)), (n, kind)
        assert np.array_equal(ctx.rle_decode(enc), v), (n, kind)


def test_decode_stops_at_first_zero_word(ctx):
    words = np.array([3 | (5 << 24), 2 | (7 << 24), 0, 9 | (1 << 24), 0], np.uint32)
    assert np.array_equal(ctx.rle_decode(words), np.array([5, 5, 5, 7, 7], np.uint8))
