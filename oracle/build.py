"""Build recipes for the parity oracle (TEST INFRASTRUCTURE ONLY).

`build_oracle()` compiles the C restatement (oracle/vpo.c) into
oracle/_build/libvpo.so; `build_ref()` compiles the reference's own hot-path
sources into oracle/_ref/libvpref.so when the reference tree is present.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIBVPO = os.path.join(HERE, "_build", "libvpo.so")
LIBREF = os.path.join(HERE, "_ref", "libvpref.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "vpo.c"), os.path.join(HERE, "vpo.h")]
    if force or _stale(LIBVPO, srcs):
        os.makedirs(os.path.dirname(LIBVPO), exist_ok=True)
        tmp = LIBVPO + ".tmp.%d" % os.getpid()
        subprocess.check_call(
            ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
             "-ffp-contract=off", "-o", tmp, srcs[0], "-lm"])
        os.replace(tmp, LIBVPO)
    return LIBVPO


def reference_root():
    """Where the reference tree is looked for: VP_REFERENCE, else the
    default of the build recipe (build_ref.sh, the one place that names it)."""
    if os.environ.get("VP_REFERENCE"):
        return os.environ["VP_REFERENCE"]
    out = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), "--root"], capture_output=True, text=True)
    return out.stdout.strip()


def build_ref(force=False):
    """Returns the path of libvpref.so, or None without the reference tree."""
    script = os.path.join(HERE, "build_ref.sh")
    ref = reference_root()
    if not os.path.exists(os.path.join(ref, "src", "chunkset", "mesher.c")):
        return None
    srcs = [script, os.path.join(HERE, "ref_harness.c"),
            os.path.join(HERE, "refshim", "ref_stubs.c")]
    srcs.append(os.path.join(ref, "src", "gfx", "fcull.c"))
    if force or _stale(LIBREF, srcs):
        subprocess.check_call(["sh", script], stdout=subprocess.DEVNULL)
    return LIBREF
