"""Build recipes for the package's native libraries.

libvoxgpu.so  — the CUDA pipeline and its C ABI (include/voxgpu.h),
                compiled for sm_103a only.
libvpgen.so   — the host-side synthetic world generator.
Both are built in-tree under voxplat_gb300/_lib/.
"""
import glob
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIBGPU = os.path.join(LIBDIR, "libvoxgpu.so")
LIBGEN = os.path.join(LIBDIR, "libvpgen.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _atomic_build(target, cmd_for):
    os.makedirs(os.path.dirname(target), exist_ok=True)
    tmp = "%s.tmp.%d" % (target, os.getpid())
    subprocess.check_call(cmd_for(tmp))
    os.replace(tmp, target)


def build_worldgen(force=False):
    srcs = [os.path.join(CSRC, f) for f in ("vp_worldgen.c", "vp_worldgen.h", "vp_noise.h")]
    if force or _stale(LIBGEN, srcs):
        _atomic_build(LIBGEN, lambda out: [
            "gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-o", out, srcs[0]])
    return LIBGEN


def cuda_sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def build_cuda(force=False, jobs=None):
    """Compile every .cu in csrc/ (in parallel) and link libvoxgpu.so."""
    cus = cuda_sources()
    deps = cus + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) \
        + [os.path.join(ROOT, "include", "voxgpu.h")]
    if not (force or _stale(LIBGPU, deps)):
        return LIBGPU
    objdir = os.path.join(PKG, "_build")
    os.makedirs(objdir, exist_ok=True)
    flags = ["nvcc", ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
             "-I", CSRC, "--expt-relaxed-constexpr"]
    procs, objs = [], []
    for cu in cus:
        obj = os.path.join(objdir, os.path.basename(cu) + ".o")
        objs.append(obj)
        procs.append(subprocess.Popen(flags + ["-c", cu, "-o", obj]))
    bad = [p for p in procs if p.wait() != 0]
    if bad:
        raise RuntimeError("nvcc failed for %d translation unit(s)" % len(bad))
    _atomic_build(LIBGPU, lambda out: ["nvcc", ARCH, "-shared", "-o", out] + objs + ["-lcudart"])
    return LIBGPU
