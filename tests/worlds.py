"""Seeded test worlds and oracle comparison helpers shared by the tests."""
import numpy as np

from voxplat_gb300 import worldgen as wg


def terrain_chunk64(seed=1):
    """One 64^3 terrain chunk (heights 8..56, colour 1 + h/4 + jitter)."""
    return wg.terrain(wg.TERRAIN_SMALL, 6, (0, 0, 0), seed=seed)


def cave_world(root_bitw=5, max_bitw=(1, 3, 1), seed=7):
    return wg.terrain(wg.TERRAIN_CAVES, root_bitw, max_bitw, seed=seed)


def world_from_voxels(root_bitw, max_bitw, chunks_vox, shadow=None, pad_rows=wg.DEFAULT_PAD_ROWS):
    """Build a World from a list of per-chunk voxel arrays (None = air)."""
    R = 1 << root_bitw
    mx = [1 << b for b in max_bitw]
    n = mx[0] * mx[1] * mx[2]
    pool, off, lens = [], [], []
    o = 0
    for c in range(n):
        v = chunks_vox[c] if c < len(chunks_vox) else None
        if v is None:
            v = np.zeros(R ** 3, np.uint8)
        s = wg.encode(v)
        pad = (-len(s)) % 4
        pool.append(s)
        pool.append(np.zeros(pad, np.uint32))
        off.append(o)
        lens.append(len(s))
        o += len(s) + pad
    W = (mx[0] + mx[1]) * R
    Z = mx[2] * R
    sh = np.zeros(W * (Z + pad_rows), np.uint16)
    if shadow is not None:
        sh[:len(shadow)] = shadow
    return wg.World(root_bitw, max_bitw, np.concatenate(pool), np.array(off, np.uint64),
                    np.array(lens, np.uint32), sh, W, Z, pad_rows)


def compare_world(gpu_world, oracle, make_mesh, lod_max, chunks=None):
    """Rebuild on the GPU and compare every chunk with the oracle.
    Returns a list of mismatch descriptions (empty = bit-exact)."""
    gpu_world.set_modes(make_mesh)
    gpu_world.rebuild(lod_max=lod_max)
    gpu_world.finish()
    res = gpu_world.results()
    bad = []
    idx = range(gpu_world.nchunks) if chunks is None else chunks
    for c in idx:
        if res[c]["status"] != 0:
            bad.append("chunk %d status %d" % (c, res[c]["status"]))
            continue
        if make_mesh is not None and make_mesh[c]:
            v, i = gpu_world.chunk_mesh(res, c)
            ov, oi = oracle.mesh(c)
            if len(v) != len(ov) or not np.array_equal(v, ov):
                bad.append("chunk %d vbo %d vs %d" % (c, len(v), len(ov)))
            if len(i) != len(oi) or not np.array_equal(i, oi):
                bad.append("chunk %d ibo %d vs %d" % (c, len(i), len(oi)))
        else:
            g, items = gpu_world.chunk_splats(res, c)
            og, oitems = oracle.splats(c, lod_max)
            if not np.array_equal(items[:lod_max + 1], oitems):
                bad.append("chunk %d items %s vs %s" % (c, list(items[:lod_max + 1]), list(oitems)))
            elif not np.array_equal(g, og):
                k = int(np.nonzero(g != og)[0][0])
                bad.append("chunk %d svl differs at %d: %s vs %s" % (c, k, g[k - k % 4:k - k % 4 + 4],
                                                                     og[k - k % 4:k - k % 4 + 4]))
    return bad


def load_fixture(path):
    """(World, dict of arrays) from a golden .npz written by make_golden.py."""
    d = dict(np.load(path))
    w = wg.World(int(d["root_bitw"]), tuple(int(b) for b in d["max_bitw"]), d["pool"], d["off"], d["len"],
                 d["shadow"], int(d["shadow_w"]), int(d["shadow_z"]), int(d["pad_rows"]))
    return w, d


def split(flat, counts):
    """Split a concatenation back into per-chunk pieces."""
    out, o = [], 0
    for c in counts:
        out.append(flat[o:o + int(c)])
        o += int(c)
    return out
