"""Generate the golden fixtures in this directory from the reference itself.

Runs the unmodified reference hot-path sources, compiled by
oracle/build_ref.sh into oracle/_ref/libvpref.so, on small seeded worlds
and records inputs (RLE streams + shadow map) and outputs (splat lists per
LOD, quad meshes, RLE encodings, sphere-edit results). Needs the reference
tree (VP_REFERENCE, else the default of oracle/build_ref.sh); run from the
repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import bindings as ob  # noqa: E402
from tests import worlds  # noqa: E402
from voxplat_gb300 import worldgen as wg  # noqa: E402


def world_arrays(w):
    return dict(root_bitw=w.root_bitw, max_bitw=np.array(w.max_bitw), pool=w.pool, off=w.off, len=w.len,
                shadow=w.shadow, shadow_w=w.shadow_w, shadow_z=w.shadow_z, pad_rows=w.pad_rows)


def geometry(ref, n, lod_levels, mesh=True):
    out = {}
    for lod in lod_levels:
        svl, items = [], []
        for c in range(n):
            g, it = ref.splats(c, lod)
            svl.append(g)
            items.append(it)
        out["svl%d" % lod] = np.concatenate(svl) if svl else np.zeros(0, np.int16)
        out["svl%d_items" % lod] = np.stack(items)
    if mesh:
        vbo, ibo, nv, ni = [], [], [], []
        for c in range(n):
            v, i = ref.mesh(c)
            vbo.append(v)
            ibo.append(i)
            nv.append(len(v))
            ni.append(len(i))
        out["vbo"] = np.concatenate(vbo)
        out["ibo"] = np.concatenate(ibo)
        out["vbo_items"] = np.array(nv, np.uint32)
        out["ibo_items"] = np.array(ni, np.uint32)
    return out


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("%-24s %8.1f KB" % (name, os.path.getsize(path) / 1024))


def main():
    if ob.ref_lib() is None:
        sys.exit("reference tree not found; set VP_REFERENCE")
    # one 64^3 terrain chunk (heights 8..56, colour 1 + h/4 + jitter)
    w = worlds.terrain_chunk64(seed=1)
    save("terrain_chunk64", **world_arrays(w), **geometry(ob.RefWorld(w), w.nchunks, (3, 4)))
    # multi-chunk cave worlds: halo and shadow-map handling across chunks
    w = worlds.cave_world(5, (1, 3, 1), seed=7)
    save("caves_r32", **world_arrays(w), **geometry(ob.RefWorld(w), w.nchunks, (4,)))
    w = worlds.cave_world(4, (2, 3, 2), seed=5)
    save("caves_r16", **world_arrays(w), **geometry(ob.RefWorld(w), w.nchunks, (4, 5)))
    # standalone uneven chunks: colours up to 255 (colour/shadow bit overlap)
    picked = []
    for k in range(64):
        rb = wg.uneven_root_bitw(3, k)
        ppm = wg.uneven_occupancy_ppm(3, k)
        if rb <= 6 and ppm < 250000 and len(picked) < 4 and (rb == 5 or ppm < 60000):
            picked.append(k)
    for k in picked:
        w = wg.uneven_chunk(3, k)
        save("uneven_k%d" % k, **world_arrays(w), **geometry(ob.RefWorld(w), 1, (4,)))
    # one sparse standalone 128^3 chunk (the large-chunk path)
    for k in range(64):
        if wg.uneven_root_bitw(3, k) == 7 and wg.uneven_occupancy_ppm(3, k) < 3000:
            w = wg.uneven_chunk(3, k)
            save("uneven128_k%d" % k, **world_arrays(w), **geometry(ob.RefWorld(w), 1, (4,)))
            break
    # RLE codec on edge-case voxel arrays
    rng = np.random.default_rng(11)
    cases = {
        "zeros": np.zeros(4096, np.uint8),
        "full": np.full(32768, 7, np.uint8),
        "alternating": (np.arange(4096) % 2 * 200).astype(np.uint8),
        "random": rng.integers(0, 256, 32768).astype(np.uint8),
        "runs": np.repeat(rng.integers(0, 4, 600).astype(np.uint8), rng.integers(1, 300, 600))[:65536],
    }
    rle = {}
    for nm, v in cases.items():
        rle["in_" + nm] = v
        rle["out_" + nm] = ob.ref_rle_compress(v)
    save("rle_codec", **rle)
    # sphere edits: voxels, dirty flags and shadow map after each edit
    w = worlds.cave_world(4, (2, 3, 2), seed=9)
    ref = ob.RefWorld(w)
    edits = np.array([[20, 50, 20, 6, 0], [33, 40, 31, 9, 77], [5, 60, 60, 4, 200],
                      [48, 30, 10, 12, 0], [16, 16, 48, 3, 31], [63, 80, 63, 10, 5]], np.int32)
    after = {}
    for e, (x, y, z, r, v) in enumerate(edits):
        dirty = ref.edit_sphere((x, y, z), int(r), int(v))
        after["dirty%d" % e] = dirty
    vox = np.stack([ref.voxels(c) for c in range(w.nchunks)])
    after["voxels"] = vox
    after["shadow_after"] = ref.shadow()
    after["edits"] = edits
    post = worlds.world_from_voxels(w.root_bitw, w.max_bitw, list(vox), shadow=after["shadow_after"],
                                    pad_rows=w.pad_rows)
    after.update({"post_" + k: v for k, v in geometry(ob.RefWorld(post), post.nchunks, (4,)).items()})
    save("edits_r16", **world_arrays(w), **after)


if __name__ == "__main__":
    main()
