"""ctypes binding of libvoxgpu.so (include/voxgpu.h).

`Context` and `DeviceWorld` mirror the C ABI one to one; `rebuild_world`
is the convenience path used by tests and the benchmark.
"""
import atexit as _atexit
import ctypes
import os
import weakref as _weakref

import numpy as np

from . import build as _build

VP_OK = 0
VP_MAX_LEVELS = 8
VP_REBUILD_PERSISTENT = 1
VP_REBUILD_PLAIN = 2
VP_REBUILD_GROUP = 4
VP_REBUILD_GRAPH = 8
VP_REBUILD_CONCURRENT = 16
VP_BATCH_MIXED = 0
VP_BATCH_SPLIT = 1


class VoxGpuError(RuntimeError):
    pass


class ChunkResult(ctypes.Structure):
    _fields_ = [
        ("svl_off", ctypes.c_uint64),
        ("vbo_off", ctypes.c_uint64),
        ("ibo_off", ctypes.c_uint64),
        ("svl_items", ctypes.c_uint32 * VP_MAX_LEVELS),
        ("svl_total", ctypes.c_uint32),
        ("vbo_items", ctypes.c_uint32),
        ("ibo_items", ctypes.c_uint32),
        ("status", ctypes.c_uint32),
    ]


RESULT_DTYPE = np.dtype([
    ("svl_off", np.uint64), ("vbo_off", np.uint64), ("ibo_off", np.uint64),
    ("svl_items", np.uint32, (VP_MAX_LEVELS,)), ("svl_total", np.uint32),
    ("vbo_items", np.uint32), ("ibo_items", np.uint32), ("status", np.uint32)])
assert RESULT_DTYPE.itemsize == ctypes.sizeof(ChunkResult)

EDIT_DTYPE = np.dtype([("x", np.int32), ("y", np.int32), ("z", np.int32), ("radius", np.uint32),
                       ("voxel", np.uint8), ("pad", np.uint8, (7,)), ("arrival_s", np.float64)])
assert EDIT_DTYPE.itemsize == 32


class BatchTune(ctypes.Structure):
    _fields_ = [("strategy", ctypes.c_int), ("min_blocks", ctypes.c_int), ("order", ctypes.c_int),
                ("ctas", ctypes.c_uint32), ("ms", ctypes.c_float), ("threads", ctypes.c_uint32),
                ("grain", ctypes.c_uint32)]

    def as_dict(self):
        return {"strategy": "mixed" if self.strategy == VP_BATCH_MIXED else "split", "min_blocks": self.min_blocks,
                "order": "longest_first" if self.order == 0 else "by_root_then_longest", "ctas": self.ctas,
                "threads": self.threads, "grain": self.grain, "ms": round(float(self.ms), 4)}


class Camera(ctypes.Structure):
    _fields_ = [("projection", ctypes.c_float * 16), ("view_rotation", ctypes.c_float * 16),
                ("view_translation", ctypes.c_float * 16), ("view_projection", ctypes.c_float * 16),
                ("inv_proj_view_rot", ctypes.c_float * 16), ("proj_view_rot", ctypes.c_float * 16),
                ("far_plane", ctypes.c_float), ("width", ctypes.c_int32), ("height", ctypes.c_int32)]

    @classmethod
    def from_dict(cls, d):
        c = cls()
        for k in ("projection", "view_rotation", "view_translation", "view_projection", "inv_proj_view_rot",
                  "proj_view_rot"):
            getattr(c, k)[:] = [float(x) for x in np.asarray(d[k], np.float32)]
        c.far_plane, c.width, c.height = d["far_plane"], d["width"], d["height"]
        return c


class ServeStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_uint32), ("edits", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("deferred", ctypes.c_uint32), ("chunks_remeshed", ctypes.c_uint64), ("busy_s", ctypes.c_double),
                ("wall_s", ctypes.c_double), ("max_inflight", ctypes.c_uint32), ("rejected", ctypes.c_uint32),
                ("inflight_s", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32), ("slot_chunks", ctypes.c_uint32),
                ("hbm_reserve", ctypes.c_uint64)]


EDIT_DONE_DTYPE = np.dtype([("ticket", np.uint64), ("status", np.int32), ("batch", np.uint32),
                            ("submit_s", np.float64), ("start_s", np.float64), ("done_s", np.float64)])


def make_edits(rows, arrival=None):
    """vp_edit array from (x, y, z, radius, voxel) rows."""
    rows = np.asarray(rows)
    e = np.zeros(len(rows), EDIT_DTYPE)
    if len(rows):
        e["x"], e["y"], e["z"] = rows[:, 0], rows[:, 1], rows[:, 2]
        e["radius"], e["voxel"] = rows[:, 3], rows[:, 4]
    if arrival is not None:
        e["arrival_s"] = arrival
    return e

_lib = None

# Live handles, so that the interpreter's exit closes servers, worlds and
# batches before the contexts they use (finalisation would otherwise call
# the destructors in any order).
_live = {k: _weakref.WeakSet() for k in ("server", "world", "batch", "ctx")}


@_atexit.register
def _close_all():
    for kind in ("server", "world", "batch", "ctx"):
        for obj in list(_live[kind]):
            try:
                obj.close()
            except Exception:
                pass


def lib_path():
    return _build.LIBGPU


def load(build_if_missing=True):
    """Load libvoxgpu.so; raises VoxGpuError if it is missing or broken."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIBGPU
    if build_if_missing and not os.path.exists(path):
        _build.build_cuda()
    if not os.path.exists(path):
        raise VoxGpuError("libvoxgpu.so not built (run __graft_entry__.build())")
    try:
        lib = ctypes.CDLL(path)
    except OSError as e:
        raise VoxGpuError("cannot load %s: %s" % (path, e))
    V, I, U32, U64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64
    PV = ctypes.POINTER(V)
    sig = {
        "vp_strerror": (ctypes.c_char_p, [I]),
        "vp_last_cuda_error": (ctypes.c_char_p, []),
        "vp_ctx_create": (I, [I, PV]),
        "vp_ctx_destroy": (None, [V]),
        "vp_ctx_stream": (V, [V]),
        "vp_ctx_sync": (I, [V]),
        "vp_ctx_set_timing": (I, [V, I]),
        "vp_world_create": (I, [V, I, V, PV]),
        "vp_world_destroy": (None, [V]),
        "vp_world_upload": (I, [V, V, U64, V, V, V, U64, U32]),
        "vp_world_set_modes": (I, [V, V]),
        "vp_world_set_handoff": (I, [V, I]),
        "vp_world_handoff_bytes": (I, [V, ctypes.POINTER(U64)]),
        "vp_world_rebuild": (I, [V, I, ctypes.c_uint]),
        "vp_world_finish": (I, [V]),
        "vp_world_reserve": (I, [V, V]),
        "vp_world_results": (I, [V, V, U32]),
        "vp_world_read_outputs": (I, [V, V, U64, V, U64, V, U64, V]),
        "vp_world_rebuild_to_host": (I, [V, I, ctypes.c_uint, I, V, U64, V, U64, V, U64, V, V]),
        "vp_world_rebuild_to_host_async": (I, [V, I, ctypes.c_uint, I, V, U64, V, U64, V, U64, V, V]),
        "vp_world_outputs_wait": (I, [V]),
        "vp_world_cull": (I, [V, V, V, I, V, U32, ctypes.POINTER(U32), V, U32, ctypes.POINTER(U32)]),
        "vp_world_camera_modes": (I, [V, V, V]),
        "vp_world_raycast": (I, [V, U32, V, V, V, V, V]),
        "vp_world_save": (I, [V, ctypes.c_char_p]),
        "vp_world_render": (I, [V, V, V, U32, V, U32, V, V, V]),
        "vp_world_open": (I, [V, ctypes.c_char_p, PV]),
        "vp_world_read_svl": (I, [V, U64, U64, V]),
        "vp_world_read_vbo": (I, [V, U64, U64, V]),
        "vp_world_read_ibo": (I, [V, U64, U64, V]),
        "vp_world_group_nodes": (I, [V, I, V, V, U32]),
        "vp_world_read_group": (I, [V, I, U64, U64, V]),
        "vp_world_generate": (I, [V, I, U64, I, U32]),
        "vp_world_edit": (I, [V, V, U32]),
        "vp_world_dirty": (I, [V, V, U32, ctypes.POINTER(U32)]),
        "vp_world_serve": (I, [V, V, U32, U32, U32, U64, V, V]),
        "vp_server_create": (I, [V, V, PV]),
        "vp_server_destroy": (None, [V]),
        "vp_edit_submit": (I, [V, V, U32, ctypes.POINTER(U64)]),
        "vp_poll_results": (I, [V, V, U32, ctypes.POINTER(U32), U32]),
        "vp_server_drain": (I, [V]),
        "vp_server_stats": (I, [V, V, ctypes.POINTER(U32)]),
        "vp_world_chunk_rle": (I, [V, U32, V, U32, ctypes.POINTER(U32)]),
        "vp_world_read_shadow": (I, [V, V, U64]),
        "vp_world_rle_words": (I, [V, ctypes.POINTER(U64)]),
        "vp_rle_encode": (I, [V, V, U32, V, U32, ctypes.POINTER(U32)]),
        "vp_rle_decode": (I, [V, V, U32, V, U32, ctypes.POINTER(U32)]),
        "vp_world_kernel_ms": (I, [V, V, I, ctypes.POINTER(U32)]),
        "vp_batch_create": (I, [V, U32, V, PV]),
        "vp_batch_destroy": (None, [V]),
        "vp_batch_upload": (I, [V, V, U64, V, V, V, V, V]),
        "vp_batch_set_modes": (I, [V, V]),
        "vp_batch_rebuild": (I, [V, I, ctypes.c_uint]),
        "vp_batch_finish": (I, [V]),
        "vp_batch_autotune": (I, [V, I, V, V, ctypes.POINTER(I)]),
        "vp_batch_set_tune": (I, [V, V]),
        "vp_batch_get_tune": (I, [V, V]),
        "vp_batch_results": (I, [V, V, U32]),
        "vp_batch_read_svl": (I, [V, U64, U64, V]),
        "vp_batch_read_vbo": (I, [V, U64, U64, V]),
        "vp_batch_read_ibo": (I, [V, U64, U64, V]),
        "vp_batch_kernel_ms": (I, [V, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(U32)]),
        "vp_selftest_handoff_wait": (I, [I, ctypes.POINTER(U32)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc, what=""):
    if rc != VP_OK:
        lib = load()
        raise VoxGpuError("%s failed: %s (%d) %s" % (
            what, lib.vp_strerror(rc).decode(), rc, lib.vp_last_cuda_error().decode()))


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Context:
    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.vp_ctx_create(device, ctypes.byref(h)), "vp_ctx_create")
        self.h = h
        _live["ctx"].add(self)

    def close(self):
        if self.h:
            self.lib.vp_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self.lib.vp_ctx_stream(self.h)

    def sync(self):
        check(self.lib.vp_ctx_sync(self.h), "vp_ctx_sync")

    def rle_encode(self, vox):
        """rle_compress on the device: the stream incl. its 0 terminator."""
        vox = np.ascontiguousarray(vox, dtype=np.uint8)
        out = np.zeros(len(vox) + 2, np.uint32)
        n = ctypes.c_uint32()
        check(self.lib.vp_rle_encode(self.h, _p(vox), len(vox), _p(out), len(out), ctypes.byref(n)), "vp_rle_encode")
        return out[:n.value].copy()

    def rle_decode(self, words, cap=None):
        """rle_decompress on the device."""
        words = np.ascontiguousarray(words, dtype=np.uint32)
        if cap is None:
            cap = int((words & 0xFFFFFF).astype(np.int64).sum())
        out = np.zeros(max(cap, 1), np.uint8)
        n = ctypes.c_uint32()
        check(self.lib.vp_rle_decode(self.h, _p(words), len(words), _p(out), len(out), ctypes.byref(n)),
              "vp_rle_decode")
        return out[:n.value].copy()

    def set_timing(self, on):
        check(self.lib.vp_ctx_set_timing(self.h, 1 if on else 0), "vp_ctx_set_timing")


class DeviceWorld:
    """A device-resident world (one reference ChunkSet)."""

    def __init__(self, ctx, world=None, root_bitw=None, max_bitw=None):
        self.ctx = ctx
        self.lib = ctx.lib
        self.world = world
        if world is not None:
            root_bitw, max_bitw = world.root_bitw, world.max_bitw
        self.root_bitw = root_bitw
        self.max_bitw = tuple(max_bitw)
        self.nchunks = 1 << sum(self.max_bitw)
        h = ctypes.c_void_p()
        mb = (ctypes.c_int * 3)(*self.max_bitw)
        check(self.lib.vp_world_create(ctx.h, root_bitw, mb, ctypes.byref(h)), "vp_world_create")
        self.h = h
        _live["world"].add(self)
        if world is not None:
            self.upload(world)

    @classmethod
    def generated(cls, ctx, kind, root_bitw, max_bitw, seed, hshift=0, pad_rows=66):
        """A world generated on the device (same bits as worldgen.terrain)."""
        dw = cls(ctx, None, root_bitw, max_bitw)
        check(dw.lib.vp_world_generate(dw.h, kind, seed, hshift, pad_rows), "vp_world_generate")
        return dw

    @classmethod
    def open(cls, ctx, path):
        """A world read from a VPW1 file (vp_world_open)."""
        h = ctypes.c_void_p()
        check(ctx.lib.vp_world_open(ctx.h, os.fsencode(path), ctypes.byref(h)), "vp_world_open")
        with open(path, "rb") as f:
            hdr = np.frombuffer(f.read(24), np.int32)
        dw = cls.__new__(cls)
        dw.ctx, dw.lib, dw.world, dw.h = ctx, ctx.lib, None, h
        _live["world"].add(dw)
        dw.root_bitw, dw.max_bitw = int(hdr[2]), tuple(int(b) for b in hdr[3:6])
        dw.nchunks = 1 << sum(dw.max_bitw)
        return dw

    def upload(self, world):
        self.upload_arrays(world.pool, world.off, world.len, world.shadow, world.shadow_w)

    def upload_arrays(self, pool, off, lens, shadow, shadow_w):
        """vp_world_upload from host arrays (pinned ones copy fastest)."""
        check(self.lib.vp_world_upload(self.h, _p(pool), len(pool), _p(off), _p(lens), _p(shadow), len(shadow),
                                       shadow_w), "vp_world_upload")

    def close(self):
        if self.h:
            self.lib.vp_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_handoff(self, on):
        """Decoded-chunk handoff between the passes of a full rebuild."""
        check(self.lib.vp_world_set_handoff(self.h, 1 if on else 0), "vp_world_set_handoff")

    def handoff_bytes(self):
        n = ctypes.c_uint64()
        check(self.lib.vp_world_handoff_bytes(self.h, ctypes.byref(n)), "vp_world_handoff_bytes")
        return n.value

    def set_modes(self, make_mesh):
        if make_mesh is None:
            check(self.lib.vp_world_set_modes(self.h, None), "vp_world_set_modes")
        else:
            m = np.ascontiguousarray(make_mesh, dtype=np.uint8)
            assert len(m) == self.nchunks
            check(self.lib.vp_world_set_modes(self.h, _p(m)), "vp_world_set_modes")

    def rebuild(self, lod_max=4, persistent=True, plain=False, group=False, concurrent=False):
        """plain: one launch per chunk and pass on the context stream;
        concurrent: the same launches spread over 16 streams."""
        flags = (VP_REBUILD_PERSISTENT if persistent else 0) | (VP_REBUILD_PLAIN if plain else 0) \
            | (VP_REBUILD_GROUP if group else 0) | (VP_REBUILD_CONCURRENT if concurrent else 0)
        check(self.lib.vp_world_rebuild(self.h, lod_max, flags), "vp_world_rebuild")

    def group_nodes(self, lod):
        """(offsets, items) of every octree node of LOD `lod` (int16 units)."""
        off = np.zeros(self.nchunks, np.uint64)
        items = np.zeros(self.nchunks, np.uint32)
        check(self.lib.vp_world_group_nodes(self.h, lod, _p(off), _p(items), self.nchunks), "vp_world_group_nodes")
        return off, items

    def read_group(self, lod, off, n):
        """n int16 items of a LOD-`lod` node list at `off` (group_nodes)."""
        out = np.zeros(int(n), np.int16)
        check(self.lib.vp_world_read_group(self.h, int(lod), int(off), int(n), _p(out)), "vp_world_read_group")
        return out

    def reserve(self, svl_bytes, vbo_bytes, ibo_bytes):
        b = (ctypes.c_uint64 * 3)(svl_bytes, vbo_bytes, ibo_bytes)
        check(self.lib.vp_world_reserve(self.h, b), "vp_world_reserve")

    def finish(self):
        check(self.lib.vp_world_finish(self.h), "vp_world_finish")

    def results(self):
        out = np.zeros(self.nchunks, RESULT_DTYPE)
        check(self.lib.vp_world_results(self.h, _p(out), self.nchunks), "vp_world_results")
        return out

    def rebuild_to_host(self, lod_max, svl, vbo, ibo, results, group=False, slabs=4):
        """A full rebuild streaming its outputs into the given host arrays
        (pinned copies fastest) and the result records into `results`
        (RESULT_DTYPE array); returns the used bytes of each output."""
        used = np.zeros(3, np.uint64)
        flags = VP_REBUILD_PERSISTENT | (VP_REBUILD_GROUP if group else 0)
        check(self.lib.vp_world_rebuild_to_host(self.h, lod_max, flags, slabs, _p(svl), svl.nbytes, _p(vbo),
                                                vbo.nbytes, _p(ibo), ibo.nbytes, _p(results), _p(used)),
              "vp_world_rebuild_to_host")
        return [int(u) for u in used]

    def rebuild_to_host_async(self, lod_max, svl, vbo, ibo, results, group=False, slabs=4):
        """rebuild_to_host pipelined with the next call: returns once the
        copies are issued. The arrays stay in use until outputs_wait() (or
        any other call on this world) returns; successive calls must
        alternate between two sets of arrays."""
        used = np.zeros(3, np.uint64)
        flags = VP_REBUILD_PERSISTENT | (VP_REBUILD_GROUP if group else 0)
        check(self.lib.vp_world_rebuild_to_host_async(self.h, lod_max, flags, slabs, _p(svl), svl.nbytes,
                                                      _p(vbo), vbo.nbytes, _p(ibo), ibo.nbytes, _p(results),
                                                      _p(used)),
              "vp_world_rebuild_to_host_async")
        return [int(u) for u in used]

    def outputs_wait(self):
        check(self.lib.vp_world_outputs_wait(self.h), "vp_world_outputs_wait")

    def read_outputs(self, svl, vbo, ibo):
        """Copy the used part of the three output arenas into the given
        arrays (pinned ones copy fastest); returns the used bytes of each."""
        used = np.zeros(3, np.uint64)
        check(self.lib.vp_world_read_outputs(self.h, _p(svl), svl.nbytes, _p(vbo), vbo.nbytes, _p(ibo), ibo.nbytes,
                                             _p(used)), "vp_world_read_outputs")
        return [int(u) for u in used]

    def cull(self, view_proj, lod_origin, top_lod=4):
        """Draw queues of the octree walk: (mesh chunk indices, splat nodes
        lod << 24 | node)."""
        vp = np.ascontiguousarray(view_proj, np.float32).reshape(16)
        org = np.ascontiguousarray(lod_origin, np.float32)
        mq = np.zeros(self.nchunks, np.uint32)
        sq = np.zeros(self.nchunks, np.uint32)
        nm, ns = ctypes.c_uint32(), ctypes.c_uint32()
        check(self.lib.vp_world_cull(self.h, _p(vp), _p(org), top_lod, _p(mq), len(mq), ctypes.byref(nm), _p(sq),
                                     len(sq), ctypes.byref(ns)), "vp_world_cull")
        return mq[:nm.value].copy(), sq[:ns.value].copy()

    def render(self, cam, mesh_queue, svl_queue, out=None):
        """(rgba[h, w] uint32, depth[h, w] float32, stats[4]) of the drawn
        queues; cam is a voxplat_gb300.camera.camera() dict. `out` = (rgba,
        depth) arrays of those shapes and types to write the frame into
        (page-locked ones make the copy back a direct one)."""
        c = Camera.from_dict(cam)
        mq = np.ascontiguousarray(mesh_queue, np.uint32)
        sq = np.ascontiguousarray(svl_queue, np.uint32)
        shape = (cam["height"], cam["width"])
        if out is None:
            rgba = np.zeros(shape, np.uint32)
            depth = np.zeros(shape, np.float32)
        else:
            rgba, depth = out
            if (rgba.shape != shape or rgba.dtype != np.uint32 or not rgba.flags.c_contiguous or
                    depth.shape != shape or depth.dtype != np.float32 or not depth.flags.c_contiguous):
                raise ValueError("render: out must be C-contiguous uint32 and float32 arrays of shape %r" % (shape,))
        stats = np.zeros(4, np.uint64)
        check(self.lib.vp_world_render(self.h, ctypes.byref(c), _p(mq), len(mq), _p(sq), len(sq), _p(rgba),
                                       _p(depth), _p(stats)), "vp_world_render")
        return rgba, depth, stats

    def save(self, path):
        """Write the world (streams + shadow map) in the VPW1 file format."""
        check(self.lib.vp_world_save(self.h, os.fsencode(path)), "vp_world_save")

    def raycast(self, origins, vectors):
        """(voxels[n], coords[n, 3], normals[n, 3]) of n picking rays."""
        o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(vectors, np.float32).reshape(-1, 3)
        n = len(o)
        vox = np.zeros(n, np.uint8)
        coords = np.zeros((n, 3), np.uint32)
        normals = np.zeros((n, 3), np.int8)
        check(self.lib.vp_world_raycast(self.h, n, _p(o), _p(v), _p(vox), _p(coords), _p(normals)),
              "vp_world_raycast")
        return vox, coords, normals

    def camera_modes(self, lod_origin):
        org = np.ascontiguousarray(lod_origin, np.float32)
        out = np.zeros(self.nchunks, np.uint8)
        check(self.lib.vp_world_camera_modes(self.h, _p(org), _p(out)), "vp_world_camera_modes")
        return out

    def read_svl(self, off, n):
        out = np.zeros(int(n), np.int16)
        check(self.lib.vp_world_read_svl(self.h, int(off), int(n), _p(out)), "vp_world_read_svl")
        return out

    def read_vbo(self, off, n):
        out = np.zeros(int(n), np.int16)
        check(self.lib.vp_world_read_vbo(self.h, int(off), int(n), _p(out)), "vp_world_read_vbo")
        return out

    def read_ibo(self, off, n):
        out = np.zeros(int(n), np.uint32)
        check(self.lib.vp_world_read_ibo(self.h, int(off), int(n), _p(out)), "vp_world_read_ibo")
        return out

    def kernel_ms(self):
        """(shell ms, geometry ms, grouping ms, launches) since the last call."""
        ms = np.zeros(3, np.float64)
        n = ctypes.c_uint32()
        check(self.lib.vp_world_kernel_ms(self.h, _p(ms), 3, ctypes.byref(n)), "vp_world_kernel_ms")
        return float(ms[0]), float(ms[1]), float(ms[2]), n.value

    def edit(self, edits):
        """Apply a batch of edits (EDIT_DTYPE array) and rebuild the dirty chunks."""
        edits = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        check(self.lib.vp_world_edit(self.h, _p(edits), len(edits)), "vp_world_edit")

    def dirty(self):
        n = ctypes.c_uint32()
        check(self.lib.vp_world_dirty(self.h, None, 0, ctypes.byref(n)), "vp_world_dirty")
        out = np.zeros(n.value, np.uint32)
        check(self.lib.vp_world_dirty(self.h, _p(out), len(out), ctypes.byref(n)), "vp_world_dirty")
        return out

    def serve(self, edits, max_batch=64, hbm_reserve=1 << 30, slots=4):
        """Replay a timed trace through an edit server with `slots` batches
        in flight at most; returns (latency_ms array, ServeStats)."""
        edits = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        lat = np.zeros(len(edits), np.float64)
        st = ServeStats()
        check(self.lib.vp_world_serve(self.h, _p(edits), len(edits), max_batch, slots, hbm_reserve, _p(lat),
                                      ctypes.byref(st)), "vp_world_serve")
        return lat, st

    def chunk_rle(self, c):
        n = ctypes.c_uint32()
        self.lib.vp_world_chunk_rle(self.h, c, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, np.uint32)
        check(self.lib.vp_world_chunk_rle(self.h, c, _p(out), len(out), ctypes.byref(n)), "vp_world_chunk_rle")
        return out

    def rle_bytes(self):
        n = ctypes.c_uint64()
        check(self.lib.vp_world_rle_words(self.h, ctypes.byref(n)), "vp_world_rle_words")
        return n.value * 4

    def shadow(self, n):
        out = np.zeros(int(n), np.uint16)
        check(self.lib.vp_world_read_shadow(self.h, _p(out), int(n)), "vp_world_read_shadow")
        return out

    def chunk_splats(self, res, c):
        r = res[c]
        return self.read_svl(r["svl_off"], r["svl_total"]), r["svl_items"].copy()

    def chunk_mesh(self, res, c):
        r = res[c]
        return self.read_vbo(r["vbo_off"], r["vbo_items"]), self.read_ibo(r["ibo_off"], r["ibo_items"])


class EditServer:
    """Continuous batching of edits on a device world (vp_server_*): submit
    edits as they arrive, poll for the finished ones."""

    def __init__(self, world, slots=4, max_batch=16, slot_chunks=512, hbm_reserve=1 << 30):
        self.world = world
        self.lib = world.lib
        cfg = ServerConfig(slots, max_batch, slot_chunks, hbm_reserve)
        h = ctypes.c_void_p()
        check(self.lib.vp_server_create(world.h, ctypes.byref(cfg), ctypes.byref(h)), "vp_server_create")
        self.h = h
        _live["server"].add(self)

    def close(self):
        if self.h:
            self.lib.vp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, edits):
        """Queue edits (EDIT_DTYPE rows); returns the first ticket."""
        edits = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        t = ctypes.c_uint64()
        check(self.lib.vp_edit_submit(self.h, _p(edits), len(edits), ctypes.byref(t)), "vp_edit_submit")
        return t.value

    def poll(self, cap=1024, wait_us=0):
        """Finished edits (EDIT_DONE_DTYPE array, completion order)."""
        out = np.zeros(cap, EDIT_DONE_DTYPE)
        n = ctypes.c_uint32()
        check(self.lib.vp_poll_results(self.h, _p(out), cap, ctypes.byref(n), wait_us), "vp_poll_results")
        return out[:n.value].copy()

    def drain(self):
        check(self.lib.vp_server_drain(self.h), "vp_server_drain")

    def stats(self):
        st = ServeStats()
        n = ctypes.c_uint32()
        check(self.lib.vp_server_stats(self.h, ctypes.byref(st), ctypes.byref(n)), "vp_server_stats")
        return st, n.value


class DeviceBatch:
    """A batch of standalone chunks (each a 1x1x1 World, any root 8..128)
    resident on the device (include/voxgpu.h, vp_batch_*)."""

    def __init__(self, ctx, chunk_worlds):
        self.ctx = ctx
        self.lib = ctx.lib
        self.h = None
        self.n = len(chunk_worlds)
        rb = np.array([w.root_bitw for w in chunk_worlds], np.int32)
        for w in chunk_worlds:
            assert w.nchunks == 1, "batch members are 1x1x1 sets"
        self.root_bitw = rb
        h = ctypes.c_void_p()
        check(self.lib.vp_batch_create(ctx.h, self.n, _p(rb), ctypes.byref(h)), "vp_batch_create")
        self.h = h
        _live["batch"].add(self)
        lens = np.array([int(w.len[0]) for w in chunk_worlds], np.uint32)
        offs = np.zeros(self.n, np.uint64)
        pieces, o = [], 0
        for k, w in enumerate(chunk_worlds):
            s = w.pool[int(w.off[0]):int(w.off[0]) + int(w.len[0])]
            pad = (-len(s)) % 4
            pieces.append(s)
            if pad:
                pieces.append(np.zeros(pad, np.uint32))
            offs[k] = o
            o += len(s) + pad
        pool = np.ascontiguousarray(np.concatenate(pieces), np.uint32)
        sh_len = np.array([len(w.shadow) for w in chunk_worlds], np.uint64)
        sh_off = np.zeros(self.n, np.uint64)
        sh_off[1:] = np.cumsum(sh_len)[:-1]
        shadow = np.ascontiguousarray(np.concatenate([w.shadow for w in chunk_worlds]), np.uint16)
        check(self.lib.vp_batch_upload(self.h, _p(pool), len(pool), _p(offs), _p(lens), _p(shadow), _p(sh_off),
                                       _p(sh_len)), "vp_batch_upload")
        self.rle_bytes = int(lens.astype(np.int64).sum()) * 4
        self.voxels = int(sum(1 << (3 * int(r)) for r in rb))

    def close(self):
        if self.h:
            self.lib.vp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_modes(self, make_mesh):
        if make_mesh is None:
            check(self.lib.vp_batch_set_modes(self.h, None), "vp_batch_set_modes")
        else:
            m = np.ascontiguousarray(make_mesh, dtype=np.uint8)
            assert len(m) == self.n
            check(self.lib.vp_batch_set_modes(self.h, _p(m)), "vp_batch_set_modes")

    def rebuild(self, lod_max=4, mode="graph"):
        """mode: "graph" (replay the tuned configuration's CUDA graph),
        "direct" (the tuned configuration launched directly), "plain" (one
        launch per chunk) or "concurrent" (one launch per chunk over 16
        streams)."""
        flags = {"graph": VP_REBUILD_GRAPH, "direct": VP_REBUILD_PERSISTENT, "plain": VP_REBUILD_PLAIN,
                 "concurrent": VP_REBUILD_CONCURRENT}[mode]
        check(self.lib.vp_batch_rebuild(self.h, lod_max, flags), "vp_batch_rebuild")

    def finish(self):
        check(self.lib.vp_batch_finish(self.h), "vp_batch_finish")

    def autotune(self, lod_max=4):
        best = BatchTune()
        tried = (BatchTune * 32)()
        n = ctypes.c_int(32)
        check(self.lib.vp_batch_autotune(self.h, lod_max, ctypes.byref(best), tried, ctypes.byref(n)),
              "vp_batch_autotune")
        return best.as_dict(), [tried[i].as_dict() for i in range(n.value)]

    def set_tune(self, strategy, min_blocks=2, order=None, ctas=0, threads=512, grain=1):
        t = BatchTune()
        t.strategy = VP_BATCH_MIXED if strategy == "mixed" else VP_BATCH_SPLIT
        t.min_blocks = min_blocks
        t.order = (0 if t.strategy == VP_BATCH_MIXED else 1) if order is None else order
        t.ctas = ctas
        t.threads = threads
        t.grain = grain
        check(self.lib.vp_batch_set_tune(self.h, ctypes.byref(t)), "vp_batch_set_tune")

    def results(self):
        out = np.zeros(self.n, RESULT_DTYPE)
        check(self.lib.vp_batch_results(self.h, _p(out), self.n), "vp_batch_results")
        return out

    def chunk_splats(self, res, k):
        r = res[k]
        out = np.zeros(int(r["svl_total"]), np.int16)
        check(self.lib.vp_batch_read_svl(self.h, int(r["svl_off"]), len(out), _p(out)), "vp_batch_read_svl")
        return out, r["svl_items"].copy()

    def chunk_mesh(self, res, k):
        r = res[k]
        v = np.zeros(int(r["vbo_items"]), np.int16)
        i = np.zeros(int(r["ibo_items"]), np.uint32)
        check(self.lib.vp_batch_read_vbo(self.h, int(r["vbo_off"]), len(v), _p(v)), "vp_batch_read_vbo")
        check(self.lib.vp_batch_read_ibo(self.h, int(r["ibo_off"]), len(i), _p(i)), "vp_batch_read_ibo")
        return v, i

    def kernel_ms(self):
        """(summed rebuild ms, launches) since the last call."""
        ms = ctypes.c_double()
        n = ctypes.c_uint32()
        check(self.lib.vp_batch_kernel_ms(self.h, ctypes.byref(ms), ctypes.byref(n)), "vp_batch_kernel_ms")
        return ms.value, n.value


VP_STATUS_TIMEOUT = 4  # a bounded device wait for a chunk's data ran out


def selftest_handoff_wait(device=0):
    """Run the self-test of the decoded-chunk handoff's bounded wait on a
    barrier armed for bytes that never come; returns the status it recorded
    (VP_STATUS_TIMEOUT when the wait gave up and the kernel returned)."""
    lib = load()
    st = ctypes.c_uint32(0)
    check(lib.vp_selftest_handoff_wait(device, ctypes.byref(st)), "vp_selftest_handoff_wait")
    return st.value
