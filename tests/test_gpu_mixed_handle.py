"""The FP32-mixed form through the single-problem calls (fvgpu_create with
precision = FV_PREC_FP32_MIXED, `[gpu] precision = fp32_mixed` in a settings
file): the problem runs as a batch of one.  Results are compared with the
bit-exact FP64 handle by relative L1 per field (1e-5 on density and
pressure, velocities within 1e-5 of the signal speed), on a 2-D and a 3-D
problem, through every call the driver uses.
"""
import os
import re
import subprocess

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import build, problems
from _helpers import assert_mixed
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _mixed(p):
    q = p.copy()
    q.precision = fv._abi.FV_PREC_FP32_MIXED
    return q


def _cases():
    rt = problems.rayleigh_taylor(64, 192)
    r3 = problems.random_problem(
        "r3", problems._mesh(24, 20, 28),
        {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "absorbing", "boundaries_z": "reflecting"},
        {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.4},
        {"gamma0": 1.4}, seed=701, wmag=0.5, vmag=0.8,
        extra={"viscosity": {"active": True, "mu": 0.01}})
    return {"rt_2d": rt, "random_3d": r3}


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_handle_steps_like_fp64(name):
    pr = CASES[name]
    a = fv.Simulation(pr.params)
    m = fv.Simulation(_mixed(pr.params))
    for s in (a, m):
        s.set_prim(*pr.prim)
    dt64 = a.compute_dt()
    dtm = m.compute_dt()
    assert abs(dtm - dt64) <= 1e-5 * dt64
    a.step(dt64)
    m.step(dt64)  # the same given dt
    assert_mixed(m.get_prim(), a.get_prim(), pr.params.gamma0)
    a.enqueue_steps(10)
    m.enqueue_steps(10)
    assert_mixed(m.get_prim(), a.get_prim(), pr.params.gamma0)
    ta, na = a.advance(0.02)
    tm, nm = m.advance(0.02)
    assert abs(na - nm) <= 1 and abs(ta - tm) <= 1e-4 * ta
    ca, cm = a.conserved_totals(), m.conserved_totals()
    assert abs(cm[0] - ca[0]) <= 1e-6 * abs(ca[0])
    assert abs(cm[4] - ca[4]) <= 1e-6 * abs(ca[4])


def test_mixed_handle_step_host_and_refusals():
    pr = CASES["rt_2d"]
    m = fv.Simulation(_mixed(pr.params))
    out, dt = m.step_host([np.ascontiguousarray(x) for x in pr.prim])
    a = fv.Simulation(pr.params)
    a.set_prim(*pr.prim)
    a.step(dt)
    assert_mixed(out, a.get_prim(), pr.params.gamma0)
    with pytest.raises(fv.FvError) as e:
        m.set_cons(*a.get_cons())
    assert e.value.status == 2


SOD_MIXED = """[mesh]
Nx=64
Ny=16
Nz=16
[run]
tend=0.02
save_freq=0.01
boundaries_x=reflecting
boundaries_y=reflecting
boundaries_z=reflecting
[solvers]
riemann_solver=hllc
reconstruction=pcm
CFL=0.1
[physics]
gamma0=1.666666667
problem=sod_x
[gpu]
precision=fp32_mixed
"""


def test_driver_runs_the_mixed_form(tmp_path):
    exe = os.path.join(build.lib_dir(), "fv3d")
    ini = tmp_path / "run.ini"
    ini.write_text(SOD_MIXED)
    prefix = str(tmp_path / "snap")
    ic = str(tmp_path / "ic.bin")
    r = subprocess.run([exe, str(ini), "--out", prefix, "--write-ic", ic, "--device-loop", "--format", "raw"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"done: (\d+) steps, t = (\S+)", r.stdout)
    steps = int(m.group(1))
    p = fv.parse_ini(SOD_MIXED)
    assert p.precision == fv._abi.FV_PREC_FP32_MIXED
    shape = (p.Nz, p.Ny, p.Nx)
    q0 = np.fromfile(ic, dtype=np.float64).reshape(5, *shape)
    ora = pyoracle.Oracle(p)
    ora.set_prim(*q0)
    _, n_o = ora.advance(p.tend)
    assert abs(steps - n_o) <= 1
    snaps = sorted(f for f in os.listdir(tmp_path) if re.fullmatch(r"snap_\d{4}\.bin", f))
    got = np.fromfile(str(tmp_path / snaps[-1]), dtype=np.float64).reshape(5, *shape)
    assert_mixed(list(got), ora.get_prim(), p.gamma0)
