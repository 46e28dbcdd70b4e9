"""Shared helpers of the test suite."""
import json
import os

import numpy as np

from fv3d_gb300._abi import FvParams

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Per-step parity bound of the plain FP64 path against the reference's FP64
# CPU arithmetic: relative L1 per field.
REL_L1_STEP = 1e-12

# Bounds of the FP32-mixed form against the bit-exact FP64 form: relative L1
# <= 1e-5 on density (the stated target) and pressure; on the velocities a
# mean absolute difference <= 1e-5 of the largest signal speed |u| + c of the
# FP64 state.  Velocity components can start at zero and stay tiny (the
# x-velocity of a Rayleigh-Taylor run, the viscosity-driven third
# component), where a relative L1 would measure FP32 rounding against an
# almost empty norm; the signal speed is the scale of the rounding of the
# momentum fluxes.
MIXED_L1 = 1e-5
MIXED_VEL = 1e-5
FIELD_NAMES = ("rho", "u", "v", "w", "p")


def assert_mixed(got, want, gamma, ctx=""):
    """The mixed-form state got (rho, u, v, w, p) against the FP64 state
    want, within MIXED_L1 / MIXED_VEL; the message states every field."""
    errs = rel_l1_fields(got, want)
    c = np.sqrt(gamma * np.asarray(want[4]) / np.asarray(want[0]))
    speed = float((np.sqrt(want[1] ** 2 + want[2] ** 2 + want[3] ** 2) + c).max())
    dv = [float(np.abs(np.asarray(got[k]) - np.asarray(want[k])).mean()) / speed for k in (1, 2, 3)]
    msg = (ctx, dict(zip(FIELD_NAMES, errs)), {"du": dv[0], "dv": dv[1], "dw": dv[2]})
    assert errs[0] <= MIXED_L1 and errs[4] <= MIXED_L1, msg
    assert max(dv) <= MIXED_VEL, msg


def golden_cases():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        return json.load(f)


def load_case(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    params = json.loads(str(d["params"]))
    return {
        "ini": str(d["ini"]),
        "params": params,
        "qin": d["qin"],
        "q0": d["q0"],
        "q1": d["q1"],
        "qN": d["qN"],
        "dts": d["dts"],
    }


def params_from_dict(dct):
    p = FvParams()
    for name, _ in FvParams._fields_:
        v = dct.get(name, 0)  # fields added after a fixture was made default to 0
        setattr(p, name, v.encode() if isinstance(v, str) else v)
    return p


def rel_l1(a, b):
    """sum|a-b| / sum|b|; 0 when both vanish identically."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    num = float(np.abs(a - b).sum())
    den = float(np.abs(b).sum())
    if den == 0.0:
        return 0.0 if num == 0.0 else float("inf")
    return num / den


def rel_l1_fields(A, B):
    return [rel_l1(a, b) for a, b in zip(A, B)]


# Generator fixtures (tests/golden/generators.npz, InitFunctor::init of the
# reference): per case, the fields computed through cos / pow (compared to
# within a few units in the last place: libm and CUDA round those
# differently) and the random ones (the fixture holds the test shim's draws,
# not the reference's: checked by their range only).
GEN_LIBM = {"rt_xz": (3,), "rt_3d": (3,), "h84_3d": (0, 4), "c91_3d": (0,)}
GEN_RANDOM = {"h84_3d": (3,), "c91_3d": (4,)}
GEN_MAX_ULP = 4


def generator_cases():
    with np.load(os.path.join(GOLDEN, "generators.npz")) as g:
        return sorted(k for k in g.files if not k.endswith("__ini"))


def load_generator(name):
    """(ini text, q) of a generator fixture; q has shape (5, Nz, Ny, Nx)."""
    with np.load(os.path.join(GOLDEN, "generators.npz")) as g:
        return str(g[name + "__ini"]), g[name]


def assert_generated(got, want, name):
    """got (5 fields) against the fixture `want` of generator case `name`:
    bit for bit, cos / pow fields within GEN_MAX_ULP, random fields skipped."""
    for v in range(5):
        if v in GEN_RANDOM.get(name, ()):
            continue
        if v in GEN_LIBM.get(name, ()):
            np.testing.assert_array_max_ulp(np.asarray(got[v]), want[v], maxulp=GEN_MAX_ULP)
        else:
            np.testing.assert_array_equal(np.asarray(got[v]), want[v], err_msg="%s field %d" % (name, v))
