"""Build recipe for the oracle libraries -- TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/libfv3d_oracle.so``: the plain-C restatement
  (fv3d_oracle.c: the step; fv3d_ini.c: readInifile), gcc -O3 -fopenmp
  -ffp-contract=off.  Built on every machine.
* ``oracle/_ref/libfv3d_ref.so``: the reference's own hot-path headers,
  unmodified, compiled from the reference tree with g++ against the
  Kokkos/INIReader shims in oracle/shim/ (ref_harness.cpp).  Built only where
  the reference sources are present: the directory named by
  ``FV3D_REFERENCE_DIR``, else a checkout named ``reference`` beside this
  repository.

-ffp-contract=off keeps both free of fused multiply-adds, so they give the
same bits on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE_DIR = os.environ.get("FV3D_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")

ORACLE_SO = os.path.join(HERE, "_build", "libfv3d_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfv3d_ref.so")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "fv3d_oracle.c"), os.path.join(HERE, "fv3d_ini.c")]
    deps = srcs + [os.path.join(HERE, "fv3d_oracle.h"), os.path.join(ROOT, "include", "fv3d_gb300.h")]
    if not force and _newer(ORACLE_SO, deps):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    cmd = ["gcc", "-std=c11", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include")] + srcs + ["-o", ORACLE_SO + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def reference_available():
    return os.path.exists(os.path.join(REFERENCE_DIR, "Update.h"))


def build_ref(force=False):
    """Compile the reference headers; returns the .so path or None when the
    reference tree is absent."""
    if not reference_available():
        return None
    src = os.path.join(HERE, "ref_harness.cpp")
    shim = os.path.join(HERE, "shim")
    deps = [src, os.path.join(ROOT, "include", "fv3d_gb300.h")] + [
        os.path.join(shim, f) for f in os.listdir(shim)]
    if not force and _newer(REF_SO, deps):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-I", shim, "-I", REFERENCE_DIR, "-I", os.path.join(ROOT, "include"), src,
           "-o", REF_SO + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(REF_SO + ".tmp", REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
