"""The C-ABI library builds, loads without a GPU and exports every entry
point its public headers declare."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

from voxplat_gb300 import build

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(INCLUDE, "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = "\n".join(ln for ln in text.splitlines() if not ln.lstrip().startswith("#"))
        for m in re.finditer(r"VP_API\s+[^;{]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            names.add(m.group(1))
    return names


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "vp_world_rebuild" in names and "vp_ctx_create" in names


def test_library_exports_all_declared_symbols():
    path = build.build_cuda()
    lib = ctypes.CDLL(path)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings_without_gpu():
    lib = ctypes.CDLL(build.build_cuda())
    lib.vp_strerror.restype = ctypes.c_char_p
    assert lib.vp_strerror(0) == b"ok"
    assert lib.vp_strerror(-4) == b"output overflow"


def _probe(tmp_path, name, extra):
    exe = str(tmp_path / name)
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "abi", "layout_probe.c")
    subprocess.check_call(["gcc", "-O0", "-o", exe, src] + extra)
    return subprocess.check_output([exe]).decode()


def test_chunkset_layout_matches_reference(tmp_path):
    from oracle.build import reference_root
    ref = reference_root()
    if not os.path.exists(os.path.join(ref, "src", "chunkset.h")):
        pytest.skip("reference sources not present")
    ours = _probe(tmp_path, "ours", ["-I", INCLUDE])
    theirs = _probe(tmp_path, "theirs", ["-DUSE_REFERENCE", "-I", os.path.join(ref, "src")])
    assert ours == theirs


def test_dropin_harness_compiles(tmp_path):
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dropin_harness.c")
    subprocess.check_call(["gcc", "-O1", "-fsyntax-only", "-I", INCLUDE, src])
