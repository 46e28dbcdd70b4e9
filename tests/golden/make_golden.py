"""Generates the golden fixtures in this directory from the reference itself.

Runs the reference's own FP64 hot-path headers (compiled unmodified against
the Kokkos/INIReader shims into oracle/_ref/ by oracle/build.py) on small
seeded problems and records, per case:
  ini       the .ini text (parsed by the reference's readInifile)
  params    every Params field readInifile produced (JSON)
  qin       the primitive input state, shape (5, Nz, Ny, Nx)
  q0        consToPrim(primToCons(qin)) as the reference stores it
  dts       the dt of each step (ComputeDtFunctor::computeDt)
  q1        primitive state after one step
  qN        primitive state after all steps
and Riemann-solver known answers (hll / hllc) on seeded state pairs that
cover every wave-speed branch, and (generators.npz) the state each problem
generator of Init.h writes (InitFunctor::init) on small grids shaped like the
reference's settings files: key <case> is the primitive state (5, Nz, Ny,
Nx), <case>__ini its .ini text.  The random pool of the shim is not Kokkos':
the H84 w and C91 p fields of those two cases hold the shim's draws and are
not compared.

Needs the reference sources (only present where the fixtures are made):
    python tests/golden/make_golden.py [case names]
"""
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fv3d_gb300 import problems  # noqa: E402
from oracle import pyoracle  # noqa: E402


random_problem = problems.random_problem


def cases():
    out = []
    s = problems.sedov(64)
    s.name = "sedov_64"
    out.append((s, 4))
    r = problems.rayleigh_taylor(32, 96)
    r.name = "rt_32x96"
    out.append((r, 4))
    r = problems.rayleigh_taylor(24, 40, riemann="hllc", kappa=1e-3, mu=1e-3)
    r.name = "rt_hllc_tc_visc"
    out.append((r, 3))
    t = problems.thermal_pulse(40)
    t.name = "thermal_40"
    out.append((t, 3))
    sh = problems.shear_layer(36)
    sh.name = "shear_36"
    out.append((sh, 3))
    out.append((problems.sod(48, "x", nx_other=8), 4))
    out.append((problems.sod(48, "y", nx_other=8), 4))
    mesh = problems._mesh(37, 23, 1)
    out.append((random_problem("random_hll_absorbing", mesh,
                               {"tend": 1.0, "boundaries_x": "absorbing", "boundaries_y": "reflecting",
                                "boundaries_z": "periodic"},
                               {"riemann_solver": "hll", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4}, seed=101, wmag=0.7), 3))
    out.append((random_problem("random_hllc_periodic_w", mesh,
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "periodic",
                                "boundaries_z": "absorbing"},
                               {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.6}, {"gamma0": 1.6666667}, seed=102, wmag=0.9), 3))
    out.append((random_problem("random_euler_pcm", problems._mesh(33, 17, 1),
                               {"tend": 1.0, "boundaries_x": "reflecting", "boundaries_y": "absorbing",
                                "boundaries_z": "periodic"},
                               {"riemann_solver": "hllc", "reconstruction": "pcm", "time_stepping": "euler",
                                "CFL": 0.4}, {"gamma0": 1.4}, seed=103), 3))
    out.append((random_problem("random_xz_pcm_wb_gravity", problems._mesh(20, 1, 28),
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "periodic",
                                "boundaries_z": "reflecting"},
                               {"riemann_solver": "hllc", "reconstruction": "pcm_wb", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4, "gravity": True, "g": -0.7}, seed=104), 3))
    out.append((random_problem("random_xy_tc_visc", problems._mesh(26, 30, 1),
                               {"tend": 1.0, "boundaries_x": "absorbing", "boundaries_y": "periodic",
                                "boundaries_z": "periodic"},
                               {"riemann_solver": "hll", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4}, seed=105,
                               extra={"thermal_conduction": {"active": True, "kappa": 0.02},
                                      "viscosity": {"active": True, "mu": 0.01}}), 3))
    out.append((random_problem("random_xz_visc_hll", problems._mesh(22, 1, 18),
                               {"tend": 1.0, "boundaries_x": "reflecting", "boundaries_y": "periodic",
                                "boundaries_z": "absorbing"},
                               {"riemann_solver": "hll", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4, "gravity": True, "g": -0.3}, seed=106,
                               extra={"thermal_conduction": {"active": True, "kappa": 0.01},
                                      "viscosity": {"active": True, "mu": 0.02}}), 3))
    out.append((random_problem("random_3d_oracle_only", problems._mesh(9, 7, 6),
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "reflecting",
                                "boundaries_z": "absorbing"},
                               {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4}, seed=107, wmag=1.0,
                               extra={"thermal_conduction": {"active": True, "kappa": 0.01},
                                      "viscosity": {"active": True, "mu": 0.01}}), 2))
    out += cases_z_physics()
    return out


def cases_z_physics():
    """3-D grids and the z-boundary physics (C91 ghosts, well-balanced z
    fluxes, fixed-temperature / gradient conduction boundaries, B02
    conductivity), plus 2-D grids that need the 3-D kernel."""
    out = []
    b = problems.blast(16)
    b.name = "blast_3d_pcm"
    out.append((b, 3))
    out.append((random_problem("c91_3d_tc_visc", problems._mesh(12, 10, 14),
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "reflecting",
                                "boundaries_z": "C91"},
                               {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.3}, {"gamma0": 1.6666667, "gravity": True, "g": -1.5}, seed=201,
                               wmag=0.5, vmag=0.5,
                               extra={"polytrope": {"theta1": 2.0},
                                      "thermal_conduction": {"active": True, "kappa": 0.02,
                                                             "bc_zmin": "fixed_temperature",
                                                             "bc_zmax": "fixed_gradient",
                                                             "bc_zmin_value": 1.0, "bc_zmax_value": 2.0},
                                      "viscosity": {"active": True, "mu": 0.01}}), 3))
    wb = random_problem("wb_b02_3d", problems._mesh(10, 12, 16),
                        {"tend": 1.0, "boundaries_x": "absorbing", "boundaries_y": "periodic",
                         "boundaries_z": "reflecting"},
                        {"riemann_solver": "hll", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.4},
                        {"gamma0": 1.4, "gravity": True, "g": -0.8, "well_balanced_flux_at_z_bc": True},
                        seed=202, wmag=0.6,
                        extra={"thermal_conduction": {"active": True, "kappa": 0.05,
                                                      "conductivity_mode": "B02"}})
    wb.b02 = (0.5, 1.0, 3.0, 0.1)
    out.append((wb, 3))
    out.append((random_problem("euler_3d_pcm_wb", problems._mesh(11, 9, 13),
                               {"tend": 1.0, "boundaries_x": "reflecting", "boundaries_y": "absorbing",
                                "boundaries_z": "absorbing"},
                               {"riemann_solver": "hllc", "reconstruction": "pcm_wb", "time_stepping": "euler",
                                "CFL": 0.5}, {"gamma0": 1.4, "gravity": True, "g": -0.5}, seed=203, wmag=0.8), 3))
    out.append((random_problem("xy_gravity_rk2", problems._mesh(20, 16, 1),
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "absorbing",
                                "boundaries_z": "periodic"},
                               {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4, "gravity": True, "g": -0.4}, seed=204), 3))
    out.append((random_problem("xz_c91_bctc", problems._mesh(18, 1, 20),
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "periodic",
                                "boundaries_z": "C91"},
                               {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.4}, {"gamma0": 1.4, "gravity": True, "g": -1.0}, seed=205,
                               vmag=0.5,
                               extra={"polytrope": {"theta1": 1.5},
                                      "thermal_conduction": {"active": True, "kappa": 0.02,
                                                             "bc_zmin": "fixed_gradient",
                                                             "bc_zmax": "fixed_temperature",
                                                             "bc_zmin_value": 0.5, "bc_zmax_value": 1.2}}), 3))
    out.append((random_problem("yz_plane_hll", problems._mesh(1, 20, 18),
                               {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "reflecting",
                                "boundaries_z": "absorbing"},
                               {"riemann_solver": "hll", "reconstruction": "plm", "time_stepping": "RK2",
                                "CFL": 0.5}, {"gamma0": 1.4}, seed=206, wmag=0.7), 3))
    return out


def _gen_ini(problem, mesh, bcs=("periodic", "periodic", "periodic"), physics=None, extra=None):
    sec = {"mesh": dict(mesh),
           "run": {"tend": 0.1, "boundaries_x": bcs[0], "boundaries_y": bcs[1], "boundaries_z": bcs[2]},
           "solvers": {"riemann_solver": "hllc", "reconstruction": "plm", "CFL": 0.1},
           "physics": dict({"gamma0": 1.4, "problem": problem}, **(physics or {}))}
    sec.update(extra or {})
    return problems.ini_text(sec)


def generator_cases():
    """(name, ini text): every generator of Init.h, on 2-D planes and 3-D
    grids, with the parameter ranges of the reference's settings files."""
    unit3 = {"xmin": 0.0, "xmax": 1.0, "ymin": 0.0, "ymax": 1.0, "zmin": 0.0, "zmax": 1.0}
    refl = ("reflecting",) * 3
    out = [
        ("sod_x_3d", _gen_ini("sod_x", dict(unit3, Nx=32, Ny=4, Nz=4), refl, {"gamma0": 1.666666667})),
        ("sod_y_xy", _gen_ini("sod_y", dict(unit3, Nx=8, Ny=32, Nz=1), refl, {"gamma0": 1.666666667})),
        ("sod_z_xz", _gen_ini("sod_z", dict(unit3, Nx=8, Ny=1, Nz=33), refl)),
        ("blast_3d", _gen_ini("blast", dict(unit3, Nx=16, Ny=16, Nz=16))),
        ("blast_xy", _gen_ini("blast", dict(unit3, Nx=40, Ny=24, Nz=1))),
        ("diffusion_xy", _gen_ini("diffusion", dict(unit3, Nx=32, Ny=32, Nz=1),
                                  extra={"viscosity": {"active": True, "mu": 0.01}})),
        ("diffusion_3d", _gen_ini("diffusion", dict(unit3, Nx=12, Ny=10, Nz=14))),
        ("rt_xz", _gen_ini("rayleigh-taylor", {"Nx": 16, "Ny": 1, "Nz": 48, "xmin": -0.25, "xmax": 0.25,
                                               "zmin": -0.75, "zmax": 0.75}, refl,
                           {"gravity": True, "g": -0.1})),
        ("rt_3d", _gen_ini("rayleigh-taylor", {"Nx": 10, "Ny": 6, "Nz": 30, "xmin": -0.25, "xmax": 0.25,
                                               "ymin": -0.25, "ymax": 0.25, "zmin": -0.75, "zmax": 0.75},
                           ("periodic", "periodic", "reflecting"), {"gravity": True, "g": -0.1})),
        ("h84_3d", _gen_ini("H84", {"Nx": 16, "Ny": 8, "xmin": 0.0, "xmax": 4.0, "ymin": 2.0, "ymax": 3.0},
                            ("periodic", "reflecting", "periodic"), {"gamma0": 1.66666667, "gravity": True, "g": 2.0},
                            {"H84": {"perturbation": 1.0e-4}, "polytrope": {"m1": 1.5}})),
        ("c91_3d", _gen_ini("C91", {"Nx": 16, "Ny": 16, "Nz": 8, "xmin": 0.0, "xmax": 4.0, "ymin": 0.0, "ymax": 4.0,
                                    "zmin": 0.0, "zmax": 1.0}, ("periodic", "periodic", "C91"),
                            {"gamma0": 1.66666667, "gravity": True, "g": 40.0},
                            {"C91": {"perturbation": 1.0e-3}, "polytrope": {"theta1": 20.0, "m1": 1.0}})),
    ]
    return out


def generators():
    tmp = tempfile.mkdtemp()
    out = {}
    for name, ini in generator_cases():
        path = os.path.join(tmp, name + ".ini")
        with open(path, "w") as f:
            f.write(ini)
        ref = pyoracle.RefOracle(path)
        out[name] = np.stack(ref.generate())
        out[name + "__ini"] = np.array(ini)
        print(name, out[name].shape)
    return out


def riemann_kats(seed=2024, n=600):
    """State pairs over every branch: subsonic, supersonic left/right moving,
    strong contrasts, and exact ties."""
    u = lambda s: problems.uniform(seed, s, n)  # noqa: E731
    qL = np.stack([0.1 + 3 * u(1), 6 * (2 * u(2) - 1), 2 * (2 * u(3) - 1), 2 * (2 * u(4) - 1), 0.05 + 5 * u(5)], 1)
    qR = np.stack([0.1 + 3 * u(6), 6 * (2 * u(7) - 1), 2 * (2 * u(8) - 1), 2 * (2 * u(9) - 1), 0.05 + 5 * u(10)], 1)
    qR[: n // 10] = qL[: n // 10]  # identical states
    out = {"qL": qL, "qR": qR}
    for solver, name in ((0, "hll"), (1, "hllc")):
        for g in (1.4, 5.0 / 3.0):
            f, po = pyoracle.riemann(solver, g, qL, qR, use_ref=True)
            out["%s_%g_flux" % (name, g)] = f
            out["%s_%g_pout" % (name, g)] = po
    return out


def main(only=None):
    """Writes every fixture, or with `only` (names) just those, keeping the
    index complete."""
    pyoracle.load_ref()
    tmp = tempfile.mkdtemp()
    index = []
    for pr, nsteps in cases():
        if only and pr.name not in only:
            index.append({"name": pr.name, "steps": nsteps, "shape": list(pr.shape)})
            continue
        path = os.path.join(tmp, pr.name + ".ini")
        with open(path, "w") as f:
            f.write(pr.ini)
        ref = pyoracle.RefOracle(path, b02=getattr(pr, "b02", None))
        ref.set_prim(*pr.prim)
        q0 = np.stack(ref.get_prim())
        dts, q1 = [], None
        for k in range(nsteps):
            dt = ref.compute_dt()
            ref.step(dt)
            dts.append(dt)
            if k == 0:
                q1 = np.stack(ref.get_prim())
        qN = np.stack(ref.get_prim())
        params = ref.params.as_dict()
        np.savez_compressed(os.path.join(HERE, pr.name + ".npz"), qin=np.stack(pr.prim), q0=q0, q1=q1, qN=qN,
                            dts=np.array(dts),
                            ini=np.array(pr.ini), params=np.array(json.dumps(params)))
        index.append({"name": pr.name, "steps": nsteps, "shape": list(q0.shape[1:])})
        print(pr.name, q0.shape, dts[:2])
    if not only:
        np.savez_compressed(os.path.join(HERE, "riemann_kats.npz"), **riemann_kats())
    if not only or "generators" in only:
        np.savez_compressed(os.path.join(HERE, "generators.npz"), **generators())
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
