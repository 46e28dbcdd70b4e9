"""Parity of the 3-D FP64 kernel (through the C ABI) with the oracle.

The 3-D kernel runs true 3-D grids and every 2-D setting the plane kernels do
not take: gravity in the x-y plane, the C91 z boundary, well-balanced z
fluxes, fixed-temperature / fixed-gradient conduction boundaries and B02
conductivity.  Each case steps the GPU and the oracle from the same state
with the same dt and requires the fields to agree to a relative L1 of 1e-12
per step (in practice they agree bit for bit); grids are ragged and large
enough to cross tile and z-chunk boundaries.
"""
import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import REL_L1_STEP, rel_l1_fields
from oracle import pyoracle

pytestmark = pytest.mark.gpu

M = problems._mesh


def _case(name, mesh, bcs, solver, recon, ts, physics=None, extra=None, seed=0, wmag=0.6, vmag=1.0,
          cfl=0.4, b02=None):
    run = {"tend": 1.0, "boundaries_x": bcs[0], "boundaries_y": bcs[1], "boundaries_z": bcs[2]}
    solvers = {"riemann_solver": solver, "reconstruction": recon, "time_stepping": ts, "CFL": cfl}
    pr = problems.random_problem(name, mesh, run, solvers, dict({"gamma0": 1.4}, **(physics or {})),
                                 seed=seed, extra=extra, wmag=wmag, vmag=vmag)
    if b02 is not None:
        (pr.params.b02_zmid, pr.params.b02_kappa1, pr.params.b02_kappa2, pr.params.b02_thickness) = b02
    return pr


TC = {"thermal_conduction": {"active": True, "kappa": 0.02}}
TCV = {"thermal_conduction": {"active": True, "kappa": 0.02}, "viscosity": {"active": True, "mu": 0.01}}
C91 = {"polytrope": {"theta1": 2.0},
       "thermal_conduction": {"active": True, "kappa": 0.02, "bc_zmin": "fixed_temperature",
                              "bc_zmax": "fixed_gradient", "bc_zmin_value": 1.0, "bc_zmax_value": 2.0},
       "viscosity": {"active": True, "mu": 0.01}}

CASES = {
    "hllc_plm_rk2_mixed_bc": lambda: _case("a", M(21, 18, 13), ("periodic", "reflecting", "absorbing"),
                                           "hllc", "plm", "RK2", seed=301),
    "hll_pcm_euler": lambda: _case("b", M(17, 12, 10), ("absorbing", "periodic", "reflecting"),
                                   "hll", "pcm", "euler", seed=302),
    "pcm_wb_gravity": lambda: _case("c", M(12, 10, 16), ("periodic", "periodic", "reflecting"), "hllc",
                                    "pcm_wb", "RK2", physics={"gravity": True, "g": -0.5}, seed=303),
    "tc_visc_periodic": lambda: _case("d", M(14, 13, 12), ("periodic",) * 3, "hll", "plm", "RK2", extra=TCV,
                                      seed=304),
    "c91_bctc_visc": lambda: _case("e", M(16, 12, 14), ("periodic", "reflecting", "C91"), "hllc", "plm",
                                   "RK2", physics={"gravity": True, "g": -1.5, "gamma0": 1.6666667},
                                   extra=C91, seed=305, wmag=0.4, vmag=0.4, cfl=0.3),
    "wb_flux_b02": lambda: _case("f", M(10, 12, 16), ("absorbing", "periodic", "reflecting"), "hll", "plm",
                                 "RK2", physics={"gravity": True, "g": -0.8, "well_balanced_flux_at_z_bc": True},
                                 extra={"thermal_conduction": {"active": True, "kappa": 0.05,
                                                               "conductivity_mode": "B02"}},
                                 seed=306, b02=(0.5, 1.0, 3.0, 0.1)),
    "wb_flux_c91_euler": lambda: _case("g", M(9, 11, 12), ("reflecting", "absorbing", "C91"), "hllc", "plm",
                                       "euler", physics={"gravity": True, "g": -1.0,
                                                         "well_balanced_flux_at_z_bc": True},
                                       extra={"polytrope": {"theta1": 1.0}}, seed=307, wmag=0.3, vmag=0.3),
    "xy_plane_gravity": lambda: _case("h", M(40, 33, 1), ("periodic", "absorbing", "periodic"), "hllc",
                                      "plm", "RK2", physics={"gravity": True, "g": -0.4}, seed=308),
    "xz_plane_c91": lambda: _case("i", M(37, 1, 30), ("periodic", "periodic", "C91"), "hllc", "plm", "RK2",
                                  physics={"gravity": True, "g": -1.0}, extra={"polytrope": {"theta1": 1.5}},
                                  seed=309, vmag=0.5),
    "yz_plane": lambda: _case("j", M(1, 26, 19), ("periodic", "reflecting", "absorbing"), "hll", "plm",
                              "RK2", extra=TC, seed=310),
    "z_chunks": lambda: _case("k", M(40, 36, 70), ("periodic", "absorbing", "periodic"), "hllc", "plm",
                              "RK2", extra=TCV, seed=311),
    "x_reflecting_one_cell_zero_u": lambda: _zero_u(_case("l", M(1, 18, 15), ("reflecting", "periodic",
                                                                               "periodic"),
                                                          "hllc", "plm", "RK2", seed=312)),
}


def _zero_u(pr):
    pr.prim[1] = np.zeros_like(pr.prim[1])
    return pr


def _per_step(pr, nsteps=2):
    ora = pyoracle.Oracle(pr.params)
    ora.set_prim(*pr.prim)
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    np.testing.assert_array_equal(np.stack(sim.get_prim()), np.stack(ora.get_prim()))
    for k in range(nsteps):
        if k:
            sim.set_cons(*ora.get_cons())
        dt_o = ora.compute_dt()
        dt_g = sim.compute_dt()
        assert dt_g == dt_o, (k, dt_g, dt_o)
        ora.step(dt_o)
        sim.step(dt_o)
        a, b = sim.get_prim(), ora.get_prim()
        errs = rel_l1_fields(a, b)
        assert max(errs) <= REL_L1_STEP, (k, errs)
        np.testing.assert_array_equal(np.stack(a), np.stack(b))
    sim.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_step_parity_3d_kernel(name):
    _per_step(CASES[name]())


def test_tile_layers_cover_grid():
    """The z-chunk size splits Nz into CTAs that cover every layer."""
    pr = CASES["z_chunks"]()
    assert pr.params.Nz == 70
    _per_step(pr, nsteps=1)


def test_advance_matches_oracle_loop_3d():
    pr = CASES["tc_visc_periodic"]()
    ora = pyoracle.Oracle(pr.params)
    ora.set_prim(*pr.prim)
    t_o, n_o = ora.advance(0.05, max_steps=12)
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    t_g, n_g = sim.advance(0.05, max_steps=12)
    assert n_g == n_o and t_g == t_o, (n_g, n_o, t_g, t_o)
    np.testing.assert_array_equal(np.stack(sim.get_prim()), np.stack(ora.get_prim()))


def test_blast_3d_conservation_symmetry_trajectory():
    """The reference's blast problem (periodic, 48^3, PCM, Euler): mass and
    energy are conserved to round-off; after one step the x, y and z axes are
    exactly interchangeable (later steps break the symmetry at round-off level
    and HLLC's star-region switch amplifies it -- the reference does the
    same); 20 free-running steps equal the oracle's bit for bit."""
    pr = problems.blast(48)
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    ora = pyoracle.Oracle(pr.params)
    ora.set_prim(*pr.prim)
    tot0 = sim.conserved_totals()
    sim.enqueue_steps(1)
    r, u, v, w, p = sim.get_prim()
    np.testing.assert_array_equal(r, np.transpose(r, (0, 2, 1)))
    np.testing.assert_array_equal(r, np.transpose(r, (2, 1, 0)))
    np.testing.assert_array_equal(u, np.transpose(v, (0, 2, 1)))
    np.testing.assert_array_equal(u, np.transpose(w, (2, 1, 0)))
    sim.enqueue_steps(19)
    tot1 = sim.conserved_totals()
    assert abs(tot1[0] - tot0[0]) <= 1e-12 * abs(tot0[0])
    assert abs(tot1[4] - tot0[4]) <= 1e-12 * abs(tot0[4])
    for _ in range(20):
        ora.step(ora.compute_dt())
    np.testing.assert_array_equal(np.stack(sim.get_prim()), np.stack(ora.get_prim()))


def test_nonzero_velocity_on_reflecting_one_cell_axis_rejected():
    pr = _case("m", M(1, 12, 10), ("reflecting", "periodic", "periodic"), "hllc", "plm", "RK2", seed=313)
    sim = fv.Simulation(pr.params)
    with pytest.raises(fv.FvError) as e:
        sim.set_prim(*pr.prim)
    assert e.value.status == 2


def test_c91_needs_two_layers():
    p = fv.parse_ini("[mesh]\nNx=8\nNy=8\nNz=1\n[run]\nboundaries_z=C91\n")
    with pytest.raises(fv.FvError) as e:
        fv.Simulation(p)
    assert e.value.status == 2
