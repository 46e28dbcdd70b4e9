"""In-tree build of the GB300 library (nvcc, sm_103a only).

``build()`` compiles every translation unit under ``fv3d_gb300/csrc`` in
parallel with ``nvcc -gencode arch=compute_103a,code=sm_103a`` and links
``fv3d_gb300/_lib/libfv3d_gb300.so`` (C ABI of include/fv3d_gb300.h) and the
``fv3d_gb300/_lib/fv3d`` driver executable.  Objects go to
``fv3d_gb300/_build``.  Rebuilds only what changed.

The FP64 translation units (FP64_EXACT_SOURCES) are compiled with
``-fmad=false``: the compiler may not contract a*b+c into one fused
operation, so every FP64 operation rounds exactly as in the reference's FP64
CPU build and the plain path reproduces it bit for bit.  Fused operations in
those files are written out explicitly (fma()) only where they are exact by
construction.  ``variant="fmad"`` lets the compiler contract them too (faster,
no longer bit-exact), for comparison.  Host code is compiled with
``-ffp-contract=off`` everywhere: the host computes constants the kernels use
(the B02 conductivity table, the CFL constants) with the reference's rounding
on both x86-64 and aarch64 hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["fv_stage2d.cu", "fv_stage3d.cu", "fv_stage3d32.cu", "fv_batch64.cu", "fv_batch32.cu", "fv_aux.cu", "fv_api.cpp", "fv_ini.cpp",
               "fv_batch.cpp", "fv_noalloc.cu", "fv_probe.cu", "fv_init.cu", "fv_h5.cpp"]
DRIVER_SOURCES = ["fv3d_main.cpp"]
FP64_EXACT_SOURCES = {"fv_stage2d.cu", "fv_stage3d.cu", "fv_batch64.cu", "fv_aux.cu", "fv_init.cu"}
# the FP32-mixed kernels: approximate FP32 division/sqrt, FMA contraction
FAST_MATH_SOURCES = {"fv_batch32.cu", "fv_stage3d32.cu"}


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_dir(variant="default"):
    return os.path.join(PKG, "_lib" if variant == "default" else "_lib_" + variant)


def lib_path(variant="default"):
    return os.path.join(lib_dir(variant), "libfv3d_gb300.so")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, obj, fmad):
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj + ".tmp"]
    if not fmad:
        cmd.insert(1, "-fmad=false")
    if os.path.basename(src) in FAST_MATH_SOURCES:
        cmd.insert(1, "-use_fast_math")
    if src.endswith(".cpp"):
        cmd[cmd.index("-c"):cmd.index("-c")] = ["-x", "cu"]
    subprocess.check_call(cmd)
    os.replace(obj + ".tmp", obj)
    return obj


def build(variant="default", jobs=None, verbose=False):
    """Compile and link; returns the path of the shared library."""
    objdir = os.path.join(PKG, "_build", variant)
    os.makedirs(objdir, exist_ok=True)
    os.makedirs(lib_dir(variant), exist_ok=True)
    headers = _headers()
    todo, objs = [], {}
    for src in LIB_SOURCES + DRIVER_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        objs[src] = o
        if _stale(o, [s, __file__] + headers):
            fmad = variant == "fmad" or src not in FP64_EXACT_SOURCES
            todo.append((s, o, fmad))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            list(ex.map(lambda a: _compile(*a), todo))
    lib = lib_path(variant)
    lib_objs = [objs[s] for s in LIB_SOURCES if s in objs]
    if _stale(lib, lib_objs):
        subprocess.check_call([_nvcc(), *ARCH, "-shared", "-o", lib + ".tmp", *lib_objs])
        os.replace(lib + ".tmp", lib)
    drv_objs = [objs[s] for s in DRIVER_SOURCES if s in objs]
    if drv_objs:
        exe = os.path.join(lib_dir(variant), "fv3d")
        if _stale(exe, drv_objs + [lib]):
            subprocess.check_call([_nvcc(), *ARCH, "-o", exe + ".tmp", *drv_objs,
                                   "-L", lib_dir(variant), "-lfv3d_gb300",
                                   "-Xlinker", "-rpath=$ORIGIN"])
            os.replace(exe + ".tmp", exe)
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    import sys
    build(sys.argv[1] if len(sys.argv) > 1 else "default", verbose=True)
