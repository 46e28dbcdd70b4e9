"""The C-ABI library: builds, loads on a machine without a GPU, exports every
entry point include/fv3d_gb300.h declares, and agrees with the ctypes mirror
of struct fv_params field by field."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import build
from fv3d_gb300._abi import FvParams

HEADER = os.path.join(build.INCLUDE, "fv3d_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:fv|fvgpu)_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = fv.load_library()
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_c():
    fields = [f for f, _ in FvParams._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "fv3d_gb300.h"', "int main(void){",
           'printf("%zu\\n", sizeof(fv_params));']
    src += ['printf("%%zu\\n", offsetof(fv_params, %s));' % f for f in fields]
    src.append("return 0;}")
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "l.c"), "w") as f:
        f.write("\n".join(src))
    subprocess.check_call(["gcc", "-I", build.INCLUDE, os.path.join(d, "l.c"), "-o", os.path.join(d, "l")])
    out = [int(x) for x in subprocess.check_output([os.path.join(d, "l")]).split()]
    assert out[0] == C.sizeof(FvParams)
    for name, off in zip(fields, out[1:]):
        assert getattr(FvParams, name).offset == off, name


def test_status_strings():
    lib = fv.load_library()
    assert lib.fv_status_string(0) == b"FV_OK"
    assert lib.fv_status_string(2) == b"FV_ERR_UNSUPPORTED"
    assert lib.fv_status_string(99) == b"FV_ERR_UNKNOWN"


def test_null_arguments_rejected_without_gpu():
    lib = fv.load_library()
    assert lib.fv_parse_ini(None, None) == 1
    assert lib.fvgpu_create(None, None) == 1
    assert lib.fvgpu_destroy(None) == 0


def test_no_cpu_fallback_in_product():
    """The product package never reaches the oracle."""
    pkg = os.path.dirname(fv.__file__)
    banned = re.compile(r"(from\s+oracle|import\s+oracle|fvora_|fvref_|fv3d_oracle|libfv3d_ref)")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cpp", ".cu", ".h", ".cuh")):
                text = open(os.path.join(root, f), errors="ignore").read()
                assert not banned.search(text), f


@pytest.mark.skipif(not os.path.exists(os.path.join(build.lib_dir(), "fv3d")), reason="driver not built")
def test_driver_binary_prints_usage():
    exe = os.path.join(build.lib_dir(), "fv3d")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2
    assert "usage" in (r.stdout + r.stderr).lower()
