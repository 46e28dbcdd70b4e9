"""The .ini surface: fv_parse_ini / fv_read_ini against readInifile.

Every golden case stores the Params the reference's own readInifile produced
from its .ini text; the product's parser must give the same fields.  Edge
cases of the INIReader semantics (comments, case, continuation lines,
unknown enum strings, single-precision floats, defaults) are checked against
values written here, and -- where the reference sources are present --
against the reference's readInifile as well.
"""
import os
import tempfile

import numpy as np
import pytest

import fv3d_gb300 as fv
from _helpers import golden_cases, load_case
from oracle import pyoracle

F32 = lambda x: float(np.float32(x))  # noqa: E731


@pytest.mark.parametrize("name", [c["name"] for c in golden_cases()])
def test_parse_matches_reference_params(name):
    case = load_case(name)
    got = fv.parse_ini(case["ini"]).as_dict()
    want = case["params"]
    for k, v in want.items():
        if k.startswith("b02_"):
            continue  # never set by readInifile
        assert got[k] == v, (k, got[k], v)


@pytest.mark.parametrize("name", [c["name"] for c in golden_cases()])
def test_oracle_parse_matches_reference_params(name):
    """The oracle's own readInifile restatement (what the CPU reference arm of
    the benchmark parses with) gives the reference's Params too."""
    case = load_case(name)
    got = pyoracle.parse_ini(case["ini"]).as_dict()
    for k, v in case["params"].items():
        if k.startswith("b02_"):
            continue
        assert got[k] == v, (k, got[k], v)


EDGE = {
    "defaults": ("", dict(Nx=32, Ny=32, Nz=32, Ng=2, CFL=F32(0.8), gamma0=F32(5.0 / 3.0), tend=1.0,
                          boundary_x=fv._abi.FV_BC_REFLECTING, reconstruction=fv._abi.FV_PCM,
                          riemann_solver=fv._abi.FV_HLLC, time_stepping=fv._abi.FV_TS_EULER,
                          epsilon=F32(1e-6), seed=12345, log_frequency=10, problem="blast",
                          filename_out="run", kappa=0.0, mu=0.0, save_freq=F32(0.1))),
    "float_precision": ("[physics]\ngamma0=1.4\ng=-0.1\n[solvers]\nCFL=0.8\n",
                        dict(gamma0=F32(1.4), g=F32(-0.1), CFL=F32(0.8))),
    "case_insensitive_keys": ("[MESH]\nNX=17\nnY = 9\n[Solvers]\nRiemann_Solver=hll\n",
                              dict(Nx=17, Ny=9, riemann_solver=fv._abi.FV_HLL)),
    "case_sensitive_values": ("[solvers]\ntime_stepping=rk2\nriemann_solver=HLL\n",
                              dict(time_stepping=fv._abi.FV_TS_EULER, riemann_solver=fv._abi.FV_HLL)),
    "unknown_enum_is_zero": ("[run]\nboundaries_x=open\nboundaries_y=periodic\n[solvers]\nreconstruction=weno\n",
                             dict(boundary_x=fv._abi.FV_BC_ABSORBING, boundary_y=fv._abi.FV_BC_PERIODIC,
                                  reconstruction=fv._abi.FV_PCM)),
    "comments": ("; comment\n# another\n[mesh]\nNx=12 ; inline\nNy=13;not a comment start\n",
                 dict(Nx=12, Ny=13)),
    "colon_separator": ("[mesh]\nNx : 21\n", dict(Nx=21)),
    "hex_and_bad_int": ("[mesh]\nNx=0x10\nNy=abc\n", dict(Nx=16, Ny=32)),
    "booleans": ("[physics]\ngravity=Yes\n[viscosity]\nactive=ON\n[thermal_conduction]\nactive=maybe\n",
                 dict(gravity=1, viscosity_active=1, thermal_conductivity_active=0)),
    "continuation": ("[physics]\nproblem=sod_x\n  extra\n", dict(problem="sod_x\nextra")),
    "duplicate_key_joins": ("[run]\nboundaries_x=periodic\nboundaries_x=periodic\n",
                            dict(boundary_x=fv._abi.FV_BC_ABSORBING)),
    "derived_mesh": ("[mesh]\nNx=50\nNy=150\nNz=1\nxmin=-0.25\nxmax= 0.25\nymin=-0.75\nymax= 0.75\n",
                     dict(dx=0.5 / 50, dy=1.5 / 150, dz=1.0, Ntot=None)),
}


@pytest.mark.parametrize("case", sorted(EDGE))
def test_ini_edge_cases(case):
    text, want = EDGE[case]
    got = fv.parse_ini(text).as_dict()
    for k, v in want.items():
        if v is None:
            continue
        assert got[k] == v, (k, got[k], v)


@pytest.mark.parametrize("case", sorted(EDGE))
def test_oracle_ini_edge_cases(case):
    text, want = EDGE[case]
    got = pyoracle.parse_ini(text).as_dict()
    prod = fv.parse_ini(text).as_dict()
    for k, v in want.items():
        if v is not None:
            assert got[k] == v, (k, got[k], v)
    assert got == prod


@pytest.mark.skipif(not pyoracle.reference_available(), reason="reference sources absent")
@pytest.mark.parametrize("case", sorted(EDGE))
def test_ini_edge_cases_against_reference(case):
    text, _ = EDGE[case]
    path = os.path.join(tempfile.mkdtemp(), "e.ini")
    with open(path, "w") as f:
        f.write(text)
    ref = pyoracle.ref_read_ini(path).as_dict()
    got = fv.read_ini(path).as_dict()
    ora = pyoracle.parse_ini(text).as_dict()
    for k, v in ref.items():
        if k.startswith("b02_") or k == "precision":
            continue
        assert got[k] == v, (k, got[k], v)
        assert ora[k] == v, (k, ora[k], v)


def test_reference_settings_files_parse():
    """The reference's example settings parse like readInifile would."""
    blast = "[mesh]\nNx=64\nNy=64\nNz=64\n[run]\ntend=0.2\nboundaries_x=periodic\n[solvers]\nCFL=0.1\n"
    p = fv.parse_ini(blast)
    assert (p.Nx, p.Ny, p.Nz) == (64, 64, 64)
    assert p.tend == F32(0.2) and p.CFL == F32(0.1)
    assert p.boundary_x == fv._abi.FV_BC_PERIODIC and p.boundary_y == fv._abi.FV_BC_REFLECTING


def test_missing_file_gives_defaults():
    p = fv.read_ini("/nonexistent/settings.ini")
    assert (p.Nx, p.Ny, p.Nz) == (32, 32, 32)
