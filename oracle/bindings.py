"""ctypes bindings of the oracle libraries (TEST INFRASTRUCTURE ONLY).

`OracleWorld` wraps the C restatement (libvpo.so); `RefWorld` wraps the
reference's own sources compiled by build_ref.sh (libvpref.so, present only
where the reference tree is). Both load a `voxplat_gb300.worldgen.World`.
"""
import ctypes

import numpy as np

from . import build

c_u32p = ctypes.POINTER(ctypes.c_uint32)
_vpo = None
_ref = None


def _vp(a):
    return ctypes.c_void_p(a.ctypes.data)


def vpo_lib():
    global _vpo
    if _vpo is None:
        lib = ctypes.CDLL(build.build_oracle())
        V = ctypes.c_void_p
        lib.vpo_world_new.restype = V
        lib.vpo_world_new.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_uint32]
        lib.vpo_world_free.argtypes = [V]
        lib.vpo_world_set_rle.argtypes = [V, ctypes.c_uint32, V, ctypes.c_uint32]
        lib.vpo_world_set_shadow.argtypes = [V, V, ctypes.c_uint64]
        lib.vpo_world_voxels.restype = ctypes.POINTER(ctypes.c_uint8)
        lib.vpo_world_voxels.argtypes = [V, ctypes.c_uint32]
        lib.vpo_chunk_splats.restype = ctypes.c_uint32
        lib.vpo_chunk_splats.argtypes = [V, ctypes.c_uint32, ctypes.c_int, V, V, V, V]
        lib.vpo_make_mesh.argtypes = [V, ctypes.c_uint32, V, V, V, V]
        lib.vpo_make_mask.argtypes = [V, ctypes.c_uint32, V]
        lib.vpo_rle_encode.restype = ctypes.c_uint32
        lib.vpo_rle_encode.argtypes = [V, ctypes.c_uint32, V]
        lib.vpo_rle_decode.restype = ctypes.c_uint32
        lib.vpo_rle_decode.argtypes = [V, V, ctypes.c_uint32]
        lib.vpo_edit_sphere.restype = ctypes.c_uint32
        lib.vpo_edit_sphere.argtypes = [V, V, ctypes.c_uint32, ctypes.c_uint8, V]
        lib.vpo_world_drop_voxels.argtypes = [V]
        lib.vpo_rebuild.restype = ctypes.c_uint64
        lib.vpo_rebuild.argtypes = [V, V, ctypes.c_uint32, V, ctypes.c_int, ctypes.c_int]
        lib.vpo_group_node.restype = ctypes.c_uint64
        lib.vpo_group_node.argtypes = [V, ctypes.c_int, V, V, V, V]
        lib.vpo_fcull_extract_planes.argtypes = [V, V]
        lib.vpo_fcull_visible.restype = ctypes.c_int
        lib.vpo_fcull_visible.argtypes = [V, V, ctypes.c_float]
        lib.vpo_octree_cull.restype = ctypes.c_uint64
        lib.vpo_octree_cull.argtypes = [ctypes.c_int, V, V, V, ctypes.c_int, V, V, V, V, V, V]
        lib.vpo_mesh_flags.argtypes = [ctypes.c_int, V, V, V]
        lib.vpo_world_set_pool.argtypes = [V, V, V, V]
        lib.vpo_check_chunks.restype = ctypes.c_uint32
        lib.vpo_check_chunks.argtypes = [V, V, ctypes.c_uint32, V, ctypes.c_int, ctypes.c_int,
                                         V, ctypes.c_uint64, V, ctypes.c_uint64, V, ctypes.c_uint64,
                                         V, V, V, V, V, V, V, V, ctypes.c_uint32]
        _vpo = lib
    return _vpo


def ref_lib():
    """The compiled reference, or None where the reference tree is absent."""
    global _ref
    if _ref is None:
        path = build.build_ref()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        V = ctypes.c_void_p
        lib.vpref_world_new.restype = V
        lib.vpref_world_new.argtypes = [ctypes.c_int] * 4 + [ctypes.c_uint32]
        lib.vpref_set_shadow.argtypes = [V, V, ctypes.c_uint64]
        lib.vpref_get_shadow.argtypes = [V, V, ctypes.c_uint64]
        lib.vpref_set_chunk_rle.argtypes = [V, ctypes.c_uint32, V, ctypes.c_uint32]
        lib.vpref_chunk_splats.restype = ctypes.c_uint32
        lib.vpref_chunk_splats.argtypes = [V, ctypes.c_uint32, ctypes.c_int, V, V, V, V]
        lib.vpref_chunk_mesh.argtypes = [V, ctypes.c_uint32, V, V, V, V]
        lib.vpref_edit_sphere.argtypes = [V] + [ctypes.c_int32] * 3 + [ctypes.c_uint32, ctypes.c_uint8]
        lib.vpref_chunk_voxels.argtypes = [V, ctypes.c_uint32, V]
        lib.vpref_chunk_dirty.argtypes = [V, ctypes.c_uint32]
        lib.vpref_clear_dirty.argtypes = [V]
        lib.vpref_rle_compress.restype = ctypes.c_uint32
        lib.vpref_rle_compress.argtypes = [V, ctypes.c_uint32, V]
        lib.vpref_rle_decompress.restype = ctypes.c_uint32
        lib.vpref_rle_decompress.argtypes = [V, V, ctypes.c_uint32]
        lib.vpref_rebuild.restype = ctypes.c_uint64
        lib.vpref_rebuild.argtypes = [V, V, ctypes.c_uint32, V, ctypes.c_int, ctypes.c_int]
        _ref = lib
    return _ref


def _splat_cap(R, lod_max):
    return 4 * sum(((R >> l) + 1) ** 3 for l in range(lod_max + 1)) + 16


def _mesh_cap(R):
    return 3 * R ** 3 + 16  # faces


class _Base:
    def splats(self, c, lod_max=4):
        """(int16 svl array, per-level int16 item counts) of chunk c."""
        R = self.R
        S3 = (R + 1) ** 3
        geom = np.zeros(_splat_cap(R, lod_max), np.int16)
        items = np.zeros(max(lod_max + 1, 8), np.uint32)
        mask = np.zeros(S3, np.uint8)
        work = np.zeros(S3, np.uint8)
        n = self._splats(c, lod_max, geom, items, mask, work)
        return geom[:n].copy(), items[:lod_max + 1].copy()

    def mesh(self, c):
        """(int16 vbo, uint32 ibo) of chunk c."""
        F = _mesh_cap(self.R)
        vbo = np.zeros(16 * F, np.int16)
        ibo = np.zeros(6 * F, np.uint32)
        nv = np.zeros(1, np.uint32)
        ni = np.zeros(1, np.uint32)
        self._mesh(c, vbo, nv, ibo, ni)
        return vbo[:int(nv[0])].copy(), ibo[:int(ni[0])].copy()


class _VpoWorldHead(ctypes.Structure):
    """Leading fields of struct vpo_world (oracle/vpo.h)."""
    _fields_ = [("root_bitw", ctypes.c_int), ("R", ctypes.c_int), ("max_bitw", ctypes.c_int * 3),
                ("max", ctypes.c_int * 3), ("nchunks", ctypes.c_uint32),
                ("rle", ctypes.c_void_p), ("rle_len", ctypes.c_void_p), ("vox", ctypes.c_void_p),
                ("shadow", ctypes.POINTER(ctypes.c_uint16)), ("shadow_len", ctypes.c_uint64),
                ("shadow_w", ctypes.c_uint32), ("shadow_z", ctypes.c_uint32)]


class OracleWorld(_Base):
    def __init__(self, world):
        lib = vpo_lib()
        self.lib = lib
        self.R = world.R
        mb = (ctypes.c_int * 3)(*world.max_bitw)
        self.h = lib.vpo_world_new(world.root_bitw, mb, world.pad_rows)
        self.nchunks = world.nchunks
        pool = np.ascontiguousarray(world.pool, np.uint32)
        off = np.ascontiguousarray(world.off, np.uint64)
        lens = np.ascontiguousarray(world.len, np.uint32)
        lib.vpo_world_set_pool(self.h, _vp(pool), _vp(off), _vp(lens))
        sh = np.ascontiguousarray(world.shadow, np.uint16)
        lib.vpo_world_set_shadow(self.h, _vp(sh), len(sh))

    @classmethod
    def partial(cls, root_bitw, max_bitw, pad_rows, streams, shadow):
        """A world of which only some chunks are known: `streams` maps chunk
        index -> RLE stream, every other chunk is air. Enough to check the
        chunks whose neighbourhoods (26 neighbours) are all in `streams`."""
        self = cls.__new__(cls)
        lib = vpo_lib()
        self.lib = lib
        self.R = 1 << root_bitw
        mb = (ctypes.c_int * 3)(*max_bitw)
        self.h = lib.vpo_world_new(root_bitw, mb, pad_rows)
        self.nchunks = 1 << sum(max_bitw)
        for c, st in streams.items():
            st = np.ascontiguousarray(st, np.uint32)
            lib.vpo_world_set_rle(self.h, int(c), _vp(st), len(st))
        sh = np.ascontiguousarray(shadow, np.uint16)
        lib.vpo_world_set_shadow(self.h, _vp(sh), len(sh))
        return self

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.vpo_world_free(self.h)
            self.h = None

    def _splats(self, c, lod_max, geom, items, mask, work):
        return self.lib.vpo_chunk_splats(self.h, c, lod_max, _vp(geom), _vp(items), _vp(mask), _vp(work))

    def _mesh(self, c, vbo, nv, ibo, ni):
        self.lib.vpo_make_mesh(self.h, c, _vp(vbo), _vp(nv), _vp(ibo), _vp(ni))

    def raycast(self, origin, vector):
        """(voxel, coord[3], normal[3]) of chunkset_edit_raycast_until_solid."""
        o = np.ascontiguousarray(origin, np.float32)
        v = np.ascontiguousarray(vector, np.float32)
        coord = np.zeros(3, np.uint32)
        normal = np.zeros(3, np.int8)
        f = self.lib.vpo_raycast
        f.restype = ctypes.c_uint8
        f.argtypes = [ctypes.c_void_p] * 5
        hit = f(self.h, _vp(o), _vp(v), _vp(coord), _vp(normal))
        return int(hit), coord, normal

    def rebuild(self, chunks, make_mesh, lod_max, nthreads, cold=True):
        """Timed CPU baseline: reference per-chunk work over `chunks`."""
        chunks = np.ascontiguousarray(chunks, np.uint32)
        mm = None if make_mesh is None else np.ascontiguousarray(make_mesh, np.uint8)
        if cold:
            self.lib.vpo_world_drop_voxels(self.h)
        return self.lib.vpo_rebuild(self.h, _vp(chunks), len(chunks), _vp(mm) if mm is not None else None,
                                    lod_max, nthreads)

    def check(self, chunks, make_mesh, lod_max, svl, vbo, ibo, results, nthreads=None, bad_cap=64):
        """Parity check of a candidate rebuild: `results` is a structured
        array indexed by chunk (fields svl_off, svl_items[8], vbo_off,
        vbo_items, ibo_off, ibo_items, status; offsets in elements of the
        int16 svl / int16 vbo / uint32 ibo arrays). Every chunk in `chunks`
        is recomputed (OpenMP) and compared byte for byte. Returns the list
        of mismatching chunks (at most bad_cap of them) and their count."""
        import os
        nthreads = nthreads or os.cpu_count() or 1
        chunks = np.ascontiguousarray(chunks, np.uint32)
        mm = None if make_mesh is None else np.ascontiguousarray(make_mesh, np.uint8)
        svl = np.ascontiguousarray(svl, np.int16)
        vbo = np.ascontiguousarray(vbo, np.int16)
        ibo = np.ascontiguousarray(ibo, np.uint32)
        f = {k: np.ascontiguousarray(results[k]) for k in ("svl_off", "vbo_off", "ibo_off")}
        f["svl_items"] = np.ascontiguousarray(results["svl_items"], np.uint32).reshape(-1)
        assert f["svl_items"].size == 8 * len(results)
        for k in ("vbo_items", "ibo_items", "status"):
            f[k] = np.ascontiguousarray(results[k], np.uint32)
        for k in ("svl_off", "vbo_off", "ibo_off"):
            f[k] = f[k].astype(np.uint64)
        bad = np.zeros(bad_cap, np.uint32)
        nbad = self.lib.vpo_check_chunks(
            self.h, _vp(chunks), len(chunks), _vp(mm) if mm is not None else None, lod_max, nthreads,
            _vp(svl), len(svl), _vp(vbo), len(vbo), _vp(ibo), len(ibo), _vp(f["svl_off"]), _vp(f["svl_items"]),
            _vp(f["vbo_off"]), _vp(f["vbo_items"]), _vp(f["ibo_off"]), _vp(f["ibo_items"]), _vp(f["status"]),
            _vp(bad), bad_cap)
        return sorted(int(b) for b in bad[:min(nbad, bad_cap)]), int(nbad)

    def drop_voxels(self):
        """Free every decoded chunk (they are decoded again on demand)."""
        self.lib.vpo_world_drop_voxels(self.h)

    def group_node(self, lod, node, svl_lists, svl_items):
        """gfx_update_svl's concatenation for one node (oracle/vpo.c)."""
        n = self.nchunks
        keep = [np.ascontiguousarray(a, np.int16) for a in svl_lists]
        its = [np.ascontiguousarray(a, np.uint32) for a in svl_items]
        P16 = (ctypes.c_void_p * n)(*[a.ctypes.data if len(a) else 0 for a in keep])
        P32 = (ctypes.c_void_p * n)(*[a.ctypes.data for a in its])
        total = sum(int(a[lod]) for a in its)
        out = np.zeros(max(total, 1), np.int16)
        nd = np.asarray(node, np.uint32)
        m = self.lib.vpo_group_node(self.h, lod, _vp(nd), ctypes.cast(P16, ctypes.c_void_p),
                                    ctypes.cast(P32, ctypes.c_void_p), _vp(out))
        return out[:m].copy()

    def mask(self, c):
        m = np.zeros((self.R + 1) ** 3, np.uint8)
        self.lib.vpo_make_mask(self.h, c, _vp(m))
        return m

    def voxels(self, c):
        p = self.lib.vpo_world_voxels(self.h, c)
        return np.ctypeslib.as_array(p, shape=(self.R ** 3,)).copy()

    def edit_sphere(self, ws, r, v):
        ws = np.asarray(ws, np.int32)
        dirty = np.zeros(self.nchunks, np.uint8)
        self.lib.vpo_edit_sphere(self.h, _vp(ws), r, v, _vp(dirty))
        return dirty

    def shadow_map(self):
        """The (padded) shadow map, e.g. after edits."""
        w = ctypes.cast(self.h, ctypes.POINTER(_VpoWorldHead)).contents
        return np.ctypeslib.as_array(w.shadow, shape=(w.shadow_len,)).copy()


class RefWorld(_Base):
    def __init__(self, world):
        lib = ref_lib()
        if lib is None:
            raise RuntimeError("reference tree not present")
        self.lib = lib
        self.R = world.R
        self.nchunks = world.nchunks
        bx, by, bz = world.max_bitw
        self.h = lib.vpref_world_new(world.root_bitw, bx, by, bz, world.pad_rows)
        for c in range(world.nchunks):
            s = np.ascontiguousarray(world.chunk_rle(c))
            lib.vpref_set_chunk_rle(self.h, c, _vp(s), len(s))
        lib.vpref_set_shadow(self.h, _vp(world.shadow), len(world.shadow))
        self.shadow_len = len(world.shadow)

    def _splats(self, c, lod_max, geom, items, mask, work):
        return self.lib.vpref_chunk_splats(self.h, c, lod_max, _vp(geom), _vp(items), _vp(mask), _vp(work))

    def rebuild(self, chunks, make_mesh, lod_max, nthreads):
        """Timed CPU baseline on the reference's own code (cold decode)."""
        chunks = np.ascontiguousarray(chunks, np.uint32)
        mm = None if make_mesh is None else np.ascontiguousarray(make_mesh, np.uint8)
        return self.lib.vpref_rebuild(self.h, _vp(chunks), len(chunks), _vp(mm) if mm is not None else None,
                                      lod_max, nthreads)

    def _mesh(self, c, vbo, nv, ibo, ni):
        self.lib.vpref_chunk_mesh(self.h, c, _vp(vbo), _vp(nv), _vp(ibo), _vp(ni))

    def raycast(self, origin, vector):
        o = np.ascontiguousarray(origin, np.float32)
        v = np.ascontiguousarray(vector, np.float32)
        coord = np.zeros(3, np.uint32)
        normal = np.zeros(3, np.int8)
        f = self.lib.vpref_raycast
        f.restype = ctypes.c_uint8
        f.argtypes = [ctypes.c_void_p] * 5
        hit = f(self.h, _vp(o), _vp(v), _vp(coord), _vp(normal))
        return int(hit), coord, normal

    def voxels(self, c):
        out = np.zeros(self.R ** 3, np.uint8)
        self.lib.vpref_chunk_voxels(self.h, c, _vp(out))
        return out

    def edit_sphere(self, ws, r, v):
        self.lib.vpref_clear_dirty(self.h)
        self.lib.vpref_edit_sphere(self.h, int(ws[0]), int(ws[1]), int(ws[2]), r, v)
        return np.array([self.lib.vpref_chunk_dirty(self.h, c) for c in range(self.nchunks)], np.uint8)

    def shadow(self):
        out = np.zeros(self.shadow_len, np.uint16)
        self.lib.vpref_get_shadow(self.h, _vp(out), self.shadow_len)
        return out


def ref_rle_compress(vox):
    lib = ref_lib()
    vox = np.ascontiguousarray(vox, np.uint8)
    out = np.zeros(len(vox) + 2, np.uint32)
    n = lib.vpref_rle_compress(_vp(vox), len(vox), _vp(out))
    return out[:n].copy()


def vpo_rle_encode(vox):
    vox = np.ascontiguousarray(vox, np.uint8)
    out = np.zeros(len(vox) + 2, np.uint32)
    n = vpo_lib().vpo_rle_encode(_vp(vox), len(vox), _vp(out))
    return out[:n].copy()


def vpo_rle_decode(words, n):
    words = np.ascontiguousarray(words, np.uint32)
    out = np.zeros(n, np.uint8)
    vpo_lib().vpo_rle_decode(_vp(words), _vp(out), n)
    return out


# ---------------------------------------------------------------------------
# draw culling and LOD selection (src/gfx/fcull.c, src/game.c:319-395, 612-625)

def fcull_extract_planes(m):
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    out = np.zeros(24, np.float32)
    vpo_lib().vpo_fcull_extract_planes(_vp(m), _vp(out))
    return out


def fcull_visible(planes, loc, radius):
    planes = np.ascontiguousarray(planes, np.float32)
    loc = np.ascontiguousarray(loc, np.float32)
    return vpo_lib().vpo_fcull_visible(_vp(planes), _vp(loc), float(np.float32(radius)))


def ref_fcull_extract_planes(m):
    """The reference's own gfx_fcull_extract_planes (None without the tree)."""
    lib = ref_lib()
    if lib is None:
        return None
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    out = np.zeros(24, np.float32)
    f = lib.gfx_fcull_extract_planes
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    f(_vp(m), _vp(out))
    return out


def ref_fcull_visible(planes, loc, radius):
    lib = ref_lib()
    if lib is None:
        return None
    f = lib.gfx_fcull_visible
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float]
    planes = np.ascontiguousarray(planes, np.float32)
    loc = np.ascontiguousarray(loc, np.float32)
    return f(_vp(planes), _vp(loc), float(np.float32(radius)))


def octree_cull(root_bitw, max_bitw, planes, origin, has_mesh, svl_items, top=4):
    """Draw queues of the octree walk: (mesh chunk indices, svl entries
    lod << 24 | node, nodes visited). svl_items[lod] = items per node."""
    mb = np.array(max_bitw, np.int32)
    planes = np.ascontiguousarray(planes, np.float32)
    origin = np.ascontiguousarray(origin, np.float32)
    has_mesh = np.ascontiguousarray(has_mesh, np.uint8)
    n = 1 << int(mb.sum())
    rows = [np.ascontiguousarray(svl_items[l], np.uint32) for l in range(top + 1)]
    ptrs = (ctypes.c_void_p * len(rows))(*[r.ctypes.data for r in rows])
    mesh_out = np.zeros(n, np.uint32)
    svl_out = np.zeros(2 * n + 64, np.uint32)
    nm = np.zeros(1, np.uint32)
    ns = np.zeros(1, np.uint32)
    visits = vpo_lib().vpo_octree_cull(int(root_bitw), _vp(mb), _vp(planes), _vp(origin), top, _vp(has_mesh),
                                       ctypes.cast(ptrs, ctypes.c_void_p), _vp(mesh_out), _vp(nm), _vp(svl_out),
                                       _vp(ns))
    return mesh_out[:int(nm[0])].copy(), svl_out[:int(ns[0])].copy(), int(visits)


def mesh_flags(root_bitw, max_bitw, origin):
    mb = np.array(max_bitw, np.int32)
    origin = np.ascontiguousarray(origin, np.float32)
    out = np.zeros(1 << int(mb.sum()), np.uint8)
    vpo_lib().vpo_mesh_flags(int(root_bitw), _vp(mb), _vp(origin), _vp(out))
    return out


def perspective_view(*args, **kw):
    """A column-major view-projection matrix (voxplat_gb300.camera)."""
    from voxplat_gb300.camera import perspective_view as pv
    return pv(*args, **kw)


# ---------------------------------------------------------------------------
# software rasteriser (resources/splat.*.glsl, resources/mesh.*.glsl)

class _VpoCamera(ctypes.Structure):
    _fields_ = [("projection", ctypes.c_float * 16), ("view_rotation", ctypes.c_float * 16),
                ("view_translation", ctypes.c_float * 16), ("view_projection", ctypes.c_float * 16),
                ("inv_proj_view_rot", ctypes.c_float * 16), ("proj_view_rot", ctypes.c_float * 16),
                ("far_plane", ctypes.c_float), ("width", ctypes.c_int), ("height", ctypes.c_int)]


class Frame:
    """A frame drawn by the oracle's rasteriser: packed (depth << 32 | RGBA8)."""

    def __init__(self, cam):
        self.cam = _VpoCamera()
        for k in ("projection", "view_rotation", "view_translation", "view_projection", "inv_proj_view_rot",
                  "proj_view_rot"):
            getattr(self.cam, k)[:] = [float(x) for x in np.asarray(cam[k], np.float32)]
        self.cam.far_plane, self.cam.width, self.cam.height = cam["far_plane"], cam["width"], cam["height"]
        self.w, self.h = cam["width"], cam["height"]
        self.words = np.zeros(self.w * self.h, np.uint64)
        lib = vpo_lib()
        lib.vpo_frame_clear.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.vpo_draw_splats.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.c_void_p]
        lib.vpo_draw_mesh.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                      ctypes.c_void_p]
        self.lib = lib
        lib.vpo_frame_clear(_vp(self.words), self.w, self.h)

    def splats(self, svl, lod):
        svl = np.ascontiguousarray(svl, np.int16)
        self.lib.vpo_draw_splats(ctypes.byref(self.cam), _vp(svl), len(svl) // 4, int(lod), _vp(self.words))

    def mesh(self, vbo, ibo):
        vbo = np.ascontiguousarray(vbo, np.int16)
        ibo = np.ascontiguousarray(ibo, np.uint32)
        self.lib.vpo_draw_mesh(ctypes.byref(self.cam), _vp(vbo), _vp(ibo), len(ibo) // 6, _vp(self.words))

    @property
    def rgba(self):
        return (self.words & 0xFFFFFFFF).astype(np.uint32).reshape(self.h, self.w)

    @property
    def depth(self):
        return (self.words >> 32).astype(np.uint32).view(np.float32).reshape(self.h, self.w)
