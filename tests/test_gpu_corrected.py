"""The physically corrected mode ([gpu] physics = corrected, fv_physics).

No reference counterpart: the viscous flux differences are divided by the
cell size, the viscous z branch mirrors the x and y branches, and HLLC's
energy takes all three velocities.  Parity is against the oracle's
restatement of the same corrected formulas (bit for bit, per step); the
physics is checked on the viscous decay of a shear wave, whose amplitude
falls as exp(-mu k^2 t / rho) in the corrected mode and hardly at all in the
reference's (its viscous term lacks the 1/dy).
"""
import math

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import REL_L1_STEP, rel_l1_fields
from oracle import pyoracle

pytestmark = pytest.mark.gpu

M = problems._mesh
GPU = {"gpu": {"physics": "corrected"}}


def _case(name, mesh, bcs, solver, extra, seed, wmag=0.6):
    run = {"tend": 1.0, "boundaries_x": bcs[0], "boundaries_y": bcs[1], "boundaries_z": bcs[2]}
    solvers = {"riemann_solver": solver, "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.4}
    ex = dict(extra)
    ex.update(GPU)
    return problems.random_problem(name, mesh, run, solvers, {"gamma0": 1.4}, seed=seed, extra=ex, wmag=wmag,
                                   vmag=1.0)


VISC = {"viscosity": {"active": True, "mu": 0.02}, "thermal_conduction": {"active": True, "kappa": 0.01}}
CASES = {
    "3d_hllc_visc": lambda: _case("a", M(18, 14, 12), ("periodic", "reflecting", "absorbing"), "hllc", VISC, 501),
    "3d_hll_visc": lambda: _case("b", M(12, 16, 10), ("absorbing", "periodic", "periodic"), "hll", VISC, 502),
    "xy_plane_visc": lambda: _case("c", M(30, 26, 1), ("periodic", "periodic", "periodic"), "hllc", VISC, 503),
    "xz_plane_hllc": lambda: _case("d", M(24, 1, 20), ("periodic", "periodic", "reflecting"), "hllc", {}, 504),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_corrected_step_parity(name):
    pr = CASES[name]()
    assert pr.params.physics == fv._abi.FV_PHYS_CORRECTED
    ora = pyoracle.Oracle(pr.params)
    ora.set_prim(*pr.prim)
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    for k in range(2):
        if k:
            sim.set_cons(*ora.get_cons())
        dt = ora.compute_dt()
        assert sim.compute_dt() == dt
        ora.step(dt)
        sim.step(dt)
        a, b = sim.get_prim(), ora.get_prim()
        assert max(rel_l1_fields(a, b)) <= REL_L1_STEP
        np.testing.assert_array_equal(np.stack(a), np.stack(b))


def test_corrected_differs_from_reference_mode():
    pr = CASES["3d_hllc_visc"]()
    ref = pr.params.copy()
    ref.physics = fv._abi.FV_PHYS_REFERENCE
    out = []
    for p in (pr.params, ref):
        sim = fv.Simulation(p)
        sim.set_prim(*pr.prim)
        sim.step(1.0e-3)
        out.append(sim.get_prim())
    assert max(rel_l1_fields(out[0], out[1])) > 1e-6


def _shear_wave(physics, n=64, mu=0.01, amp=0.01, tend=0.5):
    ini = problems.ini_text({
        "mesh": M(8, n, 1),
        "run": {"tend": tend, "boundaries_x": "periodic", "boundaries_y": "periodic", "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.8},
        "physics": {"gamma0": 1.4},
        "viscosity": {"active": True, "mu": mu},
        "gpu": {"physics": physics},
    })
    p = fv.parse_ini(ini)
    X, Y, _ = problems._centres(p)
    rho = np.ones_like(X)
    u = amp * np.sin(2 * np.pi * Y)
    z = np.zeros_like(X)
    sim = fv.Simulation(p)
    sim.set_prim(rho, u, z, z, np.full_like(X, 100.0))
    t, _ = sim.advance(tend)
    got = sim.get_prim()[1]
    # amplitude of the sin(2 pi y) mode
    a = 2.0 * float(np.mean(got * np.sin(2 * np.pi * Y)))
    return a / amp, t, float(p.mu)


def test_shear_wave_decays_at_the_viscous_rate():
    ratio, t, mu = _shear_wave("corrected")
    expect = math.exp(-mu * (2 * math.pi) ** 2 * t)
    assert abs(ratio - expect) < 0.02, (ratio, expect)
    ratio_ref, _, _ = _shear_wave("reference")
    assert ratio_ref > 0.97, ratio_ref  # the reference's viscous term is 1/dy = 64x too weak


def test_corrected_in_batches():
    """Batches run the corrected mode on the 3-D batch kernels (FP64 and
    FP32-mixed), side by side with reference-mode problems: an FP64 batch
    member equals the same problem on its own handle bit for bit; the mixed
    batch stays within the mixed tolerances of the FP64 batch."""
    from _helpers import assert_mixed
    prs = [CASES[n]() for n in sorted(CASES)]
    plain = CASES["3d_hllc_visc"]()
    plain.params.physics = fv._abi.FV_PHYS_REFERENCE
    prs.append(plain)
    b = fv.Batch([pr.params for pr in prs])
    for i, pr in enumerate(prs):
        b.set_prim(i, *pr.prim)
    b.run(3)
    singles = []
    for i, pr in enumerate(prs):
        sim = fv.Simulation(pr.params)
        sim.set_prim(*pr.prim)
        assert sim.advance(1.0e30, max_steps=3)[1] == 3
        singles.append(sim.get_prim())
        np.testing.assert_array_equal(np.stack(b.get_prim(i)), np.stack(singles[-1]))
    mixed = []
    for pr in prs:
        q = pr.params.copy()
        q.precision = fv._abi.FV_PREC_FP32_MIXED
        mixed.append(q)
    m = fv.Batch(mixed)
    for i, pr in enumerate(prs):
        m.set_prim(i, *pr.prim)
    m.run(3)
    for i, pr in enumerate(prs):
        assert_mixed(m.get_prim(i), singles[i], pr.params.gamma0, "corrected batch %d" % i)
