"""Several RK2 steps per launch for small FP32-mixed problems.

Grids of a few hundred thousand cells are bound by launch latency: each RK2
step is three launches of short kernels.  Such batches (one group of 2-D
problems) run their steps in one cooperative launch whose CTAs decide every
problem's dt themselves and meet at bounded grid barriers between the
stages.  Its work items run the per-stage kernel's body, so the state, the
times and the step counts are bit-identical to the per-stage launches
(FV3D_MULTISTEP=0), whatever the rows per work item (FV3D_MULTI_ROWS).
"""
import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems

pytestmark = pytest.mark.gpu


def mixed(params):
    q = params.copy()
    q.precision = fv._abi.FV_PREC_FP32_MIXED
    return q


def run_batch(probs, nsteps, monkeypatch, multi, rows=None):
    monkeypatch.setenv("FV3D_MULTISTEP", "1" if multi else "0")
    if rows is None:
        monkeypatch.delenv("FV3D_MULTI_ROWS", raising=False)
    else:
        monkeypatch.setenv("FV3D_MULTI_ROWS", str(rows))
    b = fv.Batch([mixed(p.params) for p in probs])
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(nsteps)
    out = [b.get_prim(i) for i in range(len(probs))], b.times(), b.launch_count()
    b.close()
    return out


SETS = {
    "sedov256": lambda: [problems.sedov(256)],
    "uneven_xy": lambda: [problems.sod(100, "x", gamma=1.3, nx_other=37), problems.sedov(90, gamma=1.5, tend=1e30),
                          problems.sod(61, "y", gamma=1.62, nx_other=45), problems.sedov(64, gamma=1.2, tend=1e30)],
    "rt_xz_tc_visc": lambda: [problems.rayleigh_taylor(60, 150, kappa=1e-3, mu=1e-3, tend=1e30),
                              problems.rayleigh_taylor(64, 192, g=-0.15, ratio=2.5, kappa=1e-3, mu=1e-3,
                                                       tend=1e30)],
    "thermal_xy_visc": lambda: [problems.thermal_pulse(96)],
}


@pytest.mark.parametrize("rows", [None, 4, 13])
@pytest.mark.parametrize("name", sorted(SETS))
def test_multistep_bitwise_equals_per_stage(name, rows, monkeypatch):
    probs = SETS[name]()
    nsteps = 17
    ref, t_ref, launches_ref = run_batch(probs, nsteps, monkeypatch, multi=False)
    got, t_got, launches = run_batch(probs, nsteps, monkeypatch, multi=True, rows=rows)
    np.testing.assert_array_equal(t_got, t_ref)
    for i in range(len(probs)):
        for k in range(5):
            np.testing.assert_array_equal(got[i][k], ref[i][k], err_msg="problem %d field %d" % (i, k))
    # one launch for all the steps instead of three per step (the same set-up)
    assert launches_ref - launches == 3 * nsteps - 1


def test_multistep_advance_to_tend(monkeypatch):
    """The main.cpp loop of the mixed handle (time bound, own dt each step)
    takes the same steps to the same time and state either way."""
    pr = problems.sedov(128, tend=0.02)
    res = []
    for multi in (False, True):
        monkeypatch.setenv("FV3D_MULTISTEP", "1" if multi else "0")
        sim = fv.Simulation(mixed(pr.params))
        sim.set_prim(*pr.prim)
        t, n = sim.advance(pr.params.tend)
        res.append((t, n, sim.get_prim()))
        sim.close()
    assert res[0][0] == res[1][0] and res[0][1] == res[1][1] and res[0][1] > 8
    for k in range(5):
        np.testing.assert_array_equal(res[1][2][k], res[0][2][k])


def test_multistep_nonfinite_reported(monkeypatch):
    monkeypatch.setenv("FV3D_MULTISTEP", "1")
    pr = problems.sedov(64, tend=1e30)
    prim = [a.copy() for a in pr.prim]
    prim[4][0, 5, 7] = -1.0  # negative pressure -> NaN sound speed
    b = fv.Batch([mixed(pr.params)])
    b.set_prim(0, *prim)
    with pytest.raises(fv.FvError) as e:
        b.run(3)
        b.times()
    assert e.value.status == 4


def test_grid_barrier_wait_gives_up_and_reports(monkeypatch):
    """The grid barrier's wait is bounded: with a CTA that never arrives it
    returns FV_ERR_TIMEOUT after its polls (no hang, the context stays
    usable); when every CTA arrives it passes."""
    assert fv.probe_grid_wait(True, 100000) == 0
    assert fv.probe_grid_wait(False, 1000) == 7  # FV_ERR_TIMEOUT
    assert fv.probe_grid_wait(True, 100000) == 0
    probs = SETS["uneven_xy"]()
    ref, t_ref, _ = run_batch(probs, 3, monkeypatch, multi=False)
    got, t_got, _ = run_batch(probs, 3, monkeypatch, multi=True)
    np.testing.assert_array_equal(t_got, t_ref)
