"""3-D problems in batches (fvgpu_batch_*): FP64 and FP32-mixed.

A 3-D problem advanced in a batch runs the same body as the one-problem 3-D
kernel, so the FP64 form equals fvgpu_create / fvgpu_enqueue_steps bit for
bit, problem by problem, whatever else shares the batch (2-D problems, other
solvers).  The FP32-mixed 3-D form is checked against that FP64 result by
relative L1 per field (bound 1e-5 on density and pressure), including the
z-boundary physics (C91 ghosts, conduction boundaries) and viscosity.
"""
import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import assert_mixed

pytestmark = pytest.mark.gpu

M = problems._mesh


def _rand3d(name, mesh, bcs, solver, seed, physics=None, extra=None, ts="RK2", wmag=0.5):
    run = {"tend": 1.0, "boundaries_x": bcs[0], "boundaries_y": bcs[1], "boundaries_z": bcs[2]}
    solvers = {"riemann_solver": solver, "reconstruction": "plm", "time_stepping": ts, "CFL": 0.4}
    return problems.random_problem(name, mesh, run, solvers, dict({"gamma0": 1.4}, **(physics or {})), seed=seed,
                                   extra=extra, wmag=wmag, vmag=0.8)


def _problems():
    tcv = {"thermal_conduction": {"active": True, "kappa": 0.02}, "viscosity": {"active": True, "mu": 0.01}}
    c91 = {"polytrope": {"theta1": 1.0},
           "thermal_conduction": {"active": True, "kappa": 0.02, "bc_zmin": "fixed_temperature",
                                  "bc_zmax": "fixed_gradient", "bc_zmin_value": 1.0, "bc_zmax_value": 2.0}}
    return [
        _rand3d("a", M(34, 20, 40), ("periodic", "reflecting", "absorbing"), "hllc", 601, extra=tcv),
        _rand3d("b", M(24, 30, 18), ("absorbing", "periodic", "periodic"), "hll", 602),
        _rand3d("c", M(20, 18, 24), ("periodic", "periodic", "C91"), "hllc", 603,
                physics={"gravity": True, "g": -1.0}, extra=c91, wmag=0.2),
        problems.sedov(48),  # a 2-D problem in the same batch
    ]


def _fp64_alone(pr, nsteps):
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    sim.enqueue_steps(nsteps)
    return sim.get_prim()


def _mixed(p):
    q = p.copy()
    q.precision = fv._abi.FV_PREC_FP32_MIXED
    return q


def test_batch3d_fp64_equals_one_problem():
    probs = _problems()
    b = fv.Batch([p.params for p in probs])
    for i, p in enumerate(probs):
        b.set_prim(i, *p.prim)
    b.run(6)
    for i, p in enumerate(probs):
        want = _fp64_alone(p, 6)
        got = b.get_prim(i)
        for a, w in zip(got, want):
            np.testing.assert_array_equal(a, w)


@pytest.mark.parametrize("layers", [8, 32, 64])
def test_batch3d_z_chunks_fp64_equal_one_problem(layers, monkeypatch):
    """Every z-chunk length the autotuner may pick (layers per work item,
    forced through FV3D_TILE) gives the bits of each problem advanced alone,
    and the schedule reports it."""
    monkeypatch.setenv("FV3D_TILE", "16x%d" % layers)
    probs = _problems()[:3]
    b = fv.Batch([p.params for p in probs])
    for i, p in enumerate(probs):
        b.set_prim(i, *p.prim)
    sched = b.schedule()
    assert all((s["tx"], s["rows"], s["block_rows"]) == (16, layers, 0) for s in sched), sched
    b.run(4)
    for i, p in enumerate(probs):
        for a, w in zip(b.get_prim(i), _fp64_alone(p, 4)):
            np.testing.assert_array_equal(a, w)


def test_batch3d_euler_fp64_equals_one_problem():
    pr = problems.blast(24, nz=20)  # Euler stepping (ping-pong buffers)
    b = fv.Batch([pr.params])
    b.set_prim(0, *pr.prim)
    b.run(5)
    for a, w in zip(b.get_prim(0), _fp64_alone(pr, 5)):
        np.testing.assert_array_equal(a, w)


@pytest.mark.parametrize("nsteps", [1, 20])
def test_batch3d_mixed_close_to_fp64(nsteps):
    probs = _problems()
    b = fv.Batch([_mixed(p.params) for p in probs])
    for i, p in enumerate(probs):
        b.set_prim(i, *p.prim)
    b.run(nsteps)
    for i, p in enumerate(probs):
        got = b.get_prim(i)
        assert all(np.isfinite(a).all() for a in got)
        want = _fp64_alone(p, nsteps)
        assert_mixed(got, want, p.params.gamma0, i)


def test_batch3d_rejects_what_it_does_not_run():
    # corrected physics runs in batches (tests/test_gpu_corrected.py); a
    # reflecting one-cell axis and B02 conductivity do not
    pr = _rand3d("y", M(1, 8, 8), ("reflecting", "periodic", "periodic"), "hllc", 605)
    with pytest.raises(fv.FvError) as e:
        fv.Batch([pr.params])
    assert e.value.status == 2
    # B02 conductivity (a per-layer kappa table) runs with the FP64 handle only
    b02 = _rand3d("z", M(8, 8, 12), ("periodic", "periodic", "reflecting"), "hllc", 606,
                  extra={"thermal_conduction": {"active": True, "kappa": 0.02, "conductivity_mode": "B02"}})
    b02.params.b02_zmid, b02.params.b02_kappa1, b02.params.b02_kappa2, b02.params.b02_thickness = 0.5, 1.0, 3.0, 0.1
    for params in (b02.params, _mixed(b02.params)):
        with pytest.raises(fv.FvError) as e:
            fv.Batch([params])
        assert e.value.status == 2
    with pytest.raises(fv.FvError) as e:
        fv.Simulation(_mixed(b02.params))
    assert e.value.status == 2


def test_mixed_refuses_fields_of_2_32_cells_or_more():
    """The FP32-mixed kernels address fields with 32-bit offsets; a grid
    whose field reaches 2^32 cells is refused before anything is
    allocated (the FP64 kernels use 64-bit offsets)."""
    ini = ("[mesh]\nNx=1640\nNy=1640\nNz=1640\n[run]\nboundaries_x=periodic\nboundaries_y=periodic\n"
           "boundaries_z=periodic\n[gpu]\nprecision=fp32_mixed\n")
    p = fv.parse_ini(ini)
    with pytest.raises(fv.FvError) as e:
        fv.Batch([p])
    assert e.value.status == 2
    assert "2^32" in str(e.value)
