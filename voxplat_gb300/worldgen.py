"""Seeded synthetic worlds (host C generator in csrc/vp_worldgen.c).

A `World` holds what the GPU pipeline keeps resident: every chunk's RLE
stream in one 16-byte aligned word pool (`pool`, `off`, `len`), and the
zero-padded u16 shadow map. Generation is integer-only, so worlds are
bit-identical on every host.
"""
import ctypes
import os

import numpy as np

from . import build as _build

TERRAIN_SMALL = 1
TERRAIN_CAVES = 2
UNEVEN = 3
DEFAULT_PAD_ROWS = 66


class _VpgWorld(ctypes.Structure):
    _fields_ = [
        ("root_bitw", ctypes.c_int),
        ("max_bitw", ctypes.c_int * 3),
        ("max", ctypes.c_int * 3),
        ("nchunks", ctypes.c_uint32),
        ("pool", ctypes.POINTER(ctypes.c_uint32)),
        ("pool_words", ctypes.c_uint64),
        ("pool_cap", ctypes.c_uint64),
        ("off", ctypes.POINTER(ctypes.c_uint64)),
        ("len", ctypes.POINTER(ctypes.c_uint32)),
        ("shadow", ctypes.POINTER(ctypes.c_uint16)),
        ("shadow_len", ctypes.c_uint64),
        ("shadow_w", ctypes.c_uint32),
        ("shadow_z", ctypes.c_uint32),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build_worldgen()
        lib = ctypes.CDLL(path)
        P = ctypes.POINTER(_VpgWorld)
        lib.vpg_world_alloc.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_uint32]
        lib.vpg_world_free.argtypes = [P]
        lib.vpg_gen_terrain.argtypes = [P, ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
        lib.vpg_uneven_root_bitw.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
        lib.vpg_uneven_occupancy_ppm.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
        lib.vpg_uneven_occupancy_ppm.restype = ctypes.c_uint32
        lib.vpg_gen_uneven.argtypes = [P, ctypes.c_uint64, ctypes.c_uint32]
        lib.vpg_rle_encode.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        lib.vpg_rle_encode.restype = ctypes.c_uint32
        _lib = lib
    return _lib


class World:
    """A resident-format world: RLE pool + offsets + lengths + shadow map."""

    def __init__(self, root_bitw, max_bitw, pool, off, lens, shadow, shadow_w, shadow_z,
                 pad_rows=DEFAULT_PAD_ROWS):
        self.root_bitw = int(root_bitw)
        self.max_bitw = tuple(int(b) for b in max_bitw)
        self.pool = np.ascontiguousarray(pool, dtype=np.uint32)
        self.off = np.ascontiguousarray(off, dtype=np.uint64)
        self.len = np.ascontiguousarray(lens, dtype=np.uint32)
        self.shadow = np.ascontiguousarray(shadow, dtype=np.uint16)
        self.shadow_w = int(shadow_w)
        self.shadow_z = int(shadow_z)
        self.pad_rows = int(pad_rows)

    @property
    def R(self):
        return 1 << self.root_bitw

    @property
    def max(self):
        return tuple(1 << b for b in self.max_bitw)

    @property
    def nchunks(self):
        m = self.max
        return m[0] * m[1] * m[2]

    def chunk_rle(self, c):
        o = int(self.off[c])
        return self.pool[o:o + int(self.len[c])]

    FILE_MAGIC = 0x31575056  # "VPW1"

    def save(self, path):
        """Write the VPW1 world file (layout in csrc/vp_io.cu): header, offset
        and length tables, the streams packed on 16-byte boundaries, the
        shadow map; little endian."""
        n = self.nchunks
        noff = np.zeros(n, np.uint64)
        pieces, o = [], 0
        for c in range(n):
            s_ = self.chunk_rle(c)
            pad = (-len(s_)) % 4
            noff[c] = o
            pieces.append(s_)
            if pad:
                pieces.append(np.zeros(pad, np.uint32))
            o += len(s_) + pad
        pool = np.concatenate(pieces).astype("<u4") if pieces else np.zeros(0, "<u4")
        hdr = np.zeros(16, "<u4")
        hdr[0], hdr[1], hdr[2] = self.FILE_MAGIC, 1, self.root_bitw
        hdr[3:6] = self.max_bitw
        hdr[6], hdr[7] = n, self.shadow_w
        hdr[8:10] = np.array([len(pool)], "<u8").view("<u4")
        hdr[10:12] = np.array([len(self.shadow)], "<u8").view("<u4")
        hdr[12] = self.pad_rows
        with open(path, "wb") as f:
            f.write(hdr.tobytes())
            f.write(noff.astype("<u8").tobytes())
            f.write(self.len.astype("<u4").tobytes())
            f.write(pool.tobytes())
            f.write(self.shadow.astype("<u2").tobytes())

    @classmethod
    def load(cls, path):
        """Read a VPW1 world file."""
        with open(path, "rb") as f:
            hdr = np.frombuffer(f.read(64), "<u4")
            if int(hdr[0]) != cls.FILE_MAGIC or int(hdr[1]) != 1:
                raise ValueError("not a VPW1 world file")
            rb, mb, n, sw = int(hdr[2]), tuple(int(b) for b in hdr[3:6]), int(hdr[6]), int(hdr[7])
            pool_words = int(hdr[8:10].view("<u8")[0])
            shadow_len = int(hdr[10:12].view("<u8")[0])
            pad = int(hdr[12])
            off = np.frombuffer(f.read(8 * n), "<u8").astype(np.uint64)
            lens = np.frombuffer(f.read(4 * n), "<u4").astype(np.uint32)
            pool = np.frombuffer(f.read(4 * pool_words), "<u4").astype(np.uint32)
            shadow = np.frombuffer(f.read(2 * shadow_len), "<u2").astype(np.uint16)
        z = (1 << mb[2]) << rb
        return cls(rb, mb, pool, off, lens, shadow, sw, z, pad)

    def chunk_coords(self, c):
        bx, by, _ = self.max_bitw
        return (c & ((1 << bx) - 1), (c >> bx) & ((1 << by) - 1), c >> (bx + by))

    def chunk_index(self, x, y, z):
        bx, by, _ = self.max_bitw
        return ((z << by | y) << bx) | x

    def chunk_voxels(self, c):
        s = self.chunk_rle(c)[:-1]
        counts = (s & 0xFFFFFF).astype(np.int64)
        cols = (s >> 24).astype(np.uint8)
        return np.repeat(cols, counts)

    def set_chunk_voxels(self, c, vox):
        """Re-encode chunk c from a voxel array (appends to the pool)."""
        words = encode(vox)
        o = len(self.pool)
        pad = (-len(words)) % 4
        self.pool = np.concatenate([self.pool, words, np.zeros(pad, np.uint32)])
        self.off[c] = o
        self.len[c] = len(words)

    def rle_bytes(self):
        return int(self.len.astype(np.int64).sum()) * 4


def _from_c(w, pad_rows):
    n = w.nchunks
    pool = np.ctypeslib.as_array(w.pool, shape=(w.pool_words,)).copy()
    off = np.ctypeslib.as_array(w.off, shape=(n,)).copy()
    lens = np.ctypeslib.as_array(w.len, shape=(n,)).copy()
    shadow = np.ctypeslib.as_array(w.shadow, shape=(w.shadow_len,)).copy()
    return World(w.root_bitw, tuple(w.max_bitw), pool, off, lens, shadow, w.shadow_w, w.shadow_z,
                 pad_rows)


def terrain(kind, root_bitw, max_bitw, seed, hshift=0, nthreads=0, pad_rows=DEFAULT_PAD_ROWS):
    """Generate a terrain world (TERRAIN_SMALL or TERRAIN_CAVES)."""
    lib = _load()
    w = _VpgWorld()
    mb = (ctypes.c_int * 3)(*max_bitw)
    if lib.vpg_world_alloc(ctypes.byref(w), root_bitw, mb, pad_rows) != 0:
        raise MemoryError("world allocation failed")
    try:
        if lib.vpg_gen_terrain(ctypes.byref(w), kind, seed, hshift, nthreads) != 0:
            raise MemoryError("world generation failed")
        return _from_c(w, pad_rows)
    finally:
        lib.vpg_world_free(ctypes.byref(w))


def uneven_root_bitw(seed, k):
    return _load().vpg_uneven_root_bitw(seed, k)


def uneven_occupancy_ppm(seed, k):
    return _load().vpg_uneven_occupancy_ppm(seed, k)


def uneven_chunk(seed, k, pad_rows=DEFAULT_PAD_ROWS):
    """Standalone chunk k of the uneven batch, as a 1x1x1 world."""
    lib = _load()
    rb = lib.vpg_uneven_root_bitw(seed, k)
    w = _VpgWorld()
    mb = (ctypes.c_int * 3)(0, 0, 0)
    if lib.vpg_world_alloc(ctypes.byref(w), rb, mb, pad_rows) != 0:
        raise MemoryError("world allocation failed")
    try:
        if lib.vpg_gen_uneven(ctypes.byref(w), seed, k) != 0:
            raise MemoryError("world generation failed")
        return _from_c(w, pad_rows)
    finally:
        lib.vpg_world_free(ctypes.byref(w))


def encode(vox):
    """RLE-encode a voxel array (reference format, 0-terminated)."""
    vox = np.ascontiguousarray(vox, dtype=np.uint8)
    out = np.empty(len(vox) + 2, np.uint32)
    n = _load().vpg_rle_encode(vox.ctypes.data, len(vox), out.ctypes.data)
    return out[:n].copy()
