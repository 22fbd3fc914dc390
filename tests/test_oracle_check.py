"""The oracle's bulk parity checker (vpo_check_chunks), which the GPU tests
use to compare whole worlds at the benchmark sizes: it must accept outputs
that equal the reference's and flag every planted mistake. Mistakes are
planted in the candidate arrays on the CPU."""
import numpy as np
import pytest

from oracle import bindings as ob
from tests import worlds
from voxplat_gb300 import gpu

LOD = 4


def _assemble(src, n, modes, order):
    """Candidate outputs built from `src` (OracleWorld or RefWorld), chunks
    laid out in `order` so offsets are not monotonic in the chunk index."""
    res = np.zeros(n, gpu.RESULT_DTYPE)
    svl, vbo, ibo = [], [], []
    so = vo = io = 0
    for c in order:
        if modes[c]:
            v, i = src.mesh(c)
            res[c]["vbo_off"], res[c]["vbo_items"] = vo, len(v)
            res[c]["ibo_off"], res[c]["ibo_items"] = io, len(i)
            vbo.append(v)
            ibo.append(i)
            vo += len(v)
            io += len(i)
        else:
            g, it = src.splats(c, LOD)
            res[c]["svl_off"], res[c]["svl_total"] = so, len(g)
            res[c]["svl_items"][:LOD + 1] = it
            svl.append(g)
            so += len(g)
    cat = lambda parts, dt: np.concatenate(parts).astype(dt) if parts else np.zeros(0, dt)
    return cat(svl, np.int16), cat(vbo, np.int16), cat(ibo, np.uint32), res


@pytest.fixture(scope="module")
def world():
    return worlds.cave_world(4, (2, 2, 2), seed=5)


def test_checker_accepts_reference_outputs(world):
    """Outputs of the compiled reference (or, without its tree, of the
    restatement the other CPU tests pin to the committed reference
    fixtures) pass the checker."""
    n = world.nchunks
    modes = (np.arange(n) % 3 == 0).astype(np.uint8)
    src = ob.RefWorld(world) if ob.ref_lib() is not None else ob.OracleWorld(world)
    order = np.random.default_rng(1).permutation(n)
    svl, vbo, ibo, res = _assemble(src, n, modes, order)
    o = ob.OracleWorld(world)
    bad, nbad = o.check(np.arange(n), modes, LOD, svl, vbo, ibo, res, nthreads=4)
    assert nbad == 0 and bad == []


def test_checker_flags_planted_mistakes(world):
    n = world.nchunks
    modes = (np.arange(n) % 3 == 0).astype(np.uint8)
    o = ob.OracleWorld(world)
    svl, vbo, ibo, res = _assemble(o, n, modes, np.arange(n))
    splat_chunks = [c for c in range(n) if not modes[c] and res[c]["svl_total"] > 8]
    mesh_chunks = [c for c in range(n) if modes[c] and res[c]["ibo_items"] > 0]
    a, b, c_, d = splat_chunks[:4]
    m1, m2 = mesh_chunks[:2]
    svl[res[a]["svl_off"] + 5] ^= 1           # one splat coordinate
    res[b]["svl_items"][2] += 4               # a level count
    res[c_]["status"] = 1                     # an overflowed chunk
    res[d]["svl_off"] = len(svl)              # a range past the array
    vbo[res[m1]["vbo_off"] + res[m1]["vbo_items"] - 1] ^= 0x40  # last vertex word
    ibo[res[m2]["ibo_off"]] += 1              # first index
    bad, nbad = o.check(np.arange(n), modes, LOD, svl, vbo, ibo, res, nthreads=4)
    assert nbad == 6 and bad == sorted([a, b, c_, d, m1, m2])
    # only the listed chunks are checked
    bad, nbad = o.check(np.array([m1]), modes, LOD, svl, vbo, ibo, res, nthreads=2)
    assert bad == [m1] and nbad == 1
