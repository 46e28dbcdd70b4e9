"""The FP32-mixed form at high Mach: a density perturbation advected by a
uniform flow at Mach 10, 30 and 100 (periodic, HLL and HLLC, PLM, RK2).

In exact arithmetic pressure and velocity stay uniform (for HLL and HLLC the
momentum and energy fluxes of such states are u F_rho + p and
u^2 F_rho / 2 + const); the bit-exact FP64 form keeps p uniform to ~1e-12.
The mixed form recovers p = (gamma-1)(E - |m|^2/(2 rho)) (States.h:42-43) in
double-float arithmetic from the (hi, lo) pairs of U^n and from the internal
energy kept in U*; what remains is the FP32 rounding of the fluxes, whose
effect on p grows like 2^-24 gamma (gamma-1) M^2 / 2 per step.  Measured
after 50 steps: relative L1 of p against FP64 = 4.0-4.6e-8 x
gamma (gamma-1) M^2 / 2 (1.3e-6 at Mach 10, 1.1e-4 at Mach 100); an FP32
kinetic energy in the recovery gave 7.5-8.9e-8 x the same factor.  The bound
below, 6e-8 x gamma (gamma-1) M^2 / 2, separates the two.
"""
import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import rel_l1

pytestmark = pytest.mark.gpu

NSTEPS = 50


def contact(mach, riemann, n=256, gamma=1.4, amp=1e-3, seed=99):
    ini = problems.ini_text({
        "mesh": problems._mesh(n, n, 1),
        "run": {"tend": 1e30, "boundaries_x": "periodic", "boundaries_y": "periodic", "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": riemann, "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.8},
        "physics": {"gamma0": gamma, "problem": "contact"}})
    p = fv.parse_ini(ini)
    X, Y, _ = problems._centres(p)
    noise = problems.uniform(seed, 1, X.size).reshape(X.shape) - 0.5
    rho = 1.0 + amp * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y) + 0.1 * amp * noise
    c = np.sqrt(p.gamma0)  # p = 1, rho ~ 1
    u = np.full_like(X, 0.8 * mach * c)
    v = np.full_like(X, 0.6 * mach * c)
    return p, [rho, u, v, np.zeros_like(X), np.ones_like(X)]


def run(params, prim, precision):
    q = params.copy()
    q.precision = precision
    b = fv.Batch([q])
    b.set_prim(0, *prim)
    b.run(NSTEPS)
    return b.get_prim(0)


@pytest.mark.parametrize("riemann", ["hll", "hllc"])
@pytest.mark.parametrize("mach", [10, 30, 100])
def test_mixed_pressure_at_high_mach(mach, riemann):
    params, prim = contact(mach, riemann)
    ref = run(params, prim, fv._abi.FV_PREC_FP64)
    got = run(params, prim, fv._abi.FV_PREC_FP32_MIXED)
    g = params.gamma0
    factor = g * (g - 1.0) * mach * mach / 2.0
    assert np.abs(ref[4] - 1.0).max() <= 1e-14 * factor  # FP64 keeps p uniform
    err_p = rel_l1(got[4], ref[4])
    assert err_p <= 6e-8 * factor, (mach, riemann, err_p, err_p / factor)
    assert rel_l1(got[0], ref[0]) <= 1e-6
    for k in (1, 2):  # the uniform velocities
        assert rel_l1(got[k], ref[k]) <= 1e-6
