"""The device edit kernel tests d0^2 + d1^2 + d2^2 < r^2 in integers; the
reference tests sqrtf(d0^2 + d1^2 + d2^2) < (float)r in float
(src/chunkset/edit.c:216-221). For every radius the edit API accepts (<= 250)
and every integer squared distance an AABB voxel can have, the two agree:
the squares and their sum are exact in float and sqrtf rounds correctly."""
import numpy as np


def test_float_sqrt_compare_equals_integer_compare():
    for r in range(0, 251):
        smax = 3 * (r + 1) ** 2
        s = np.arange(smax + 1, dtype=np.int64)
        f = np.sqrt(s.astype(np.float32)) < np.float32(r)
        assert np.array_equal(f, s < r * r), r
        assert (s.astype(np.float32).astype(np.int64) == s).all()
