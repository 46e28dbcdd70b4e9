"""Seeded synthetic problems (initial conditions + .ini settings).

The reference publishes no benchmark inputs; every workload here is generated
from a seed with a repo-defined counter-based splitmix64 stream (uniform
[0,1) from the top 53 bits, Gaussians by Box-Muller).  The master seed
defaults to 12345, the reference's [misc] seed default (SimInfo.h:293).

Each builder returns a :class:`Problem`: the .ini text a reference user would
write (so every float setting is parsed with single precision, as the
reference's INIReader does) and primitive fields of shape (Nz, Ny, Nx)
computed in float64 from the parsed parameters and cell centres
``xmin + (i + 0.5) * dx`` (getPos, SimInfo.h:162-167).

Configurations (2-D means Nz = 1 with a periodic z axis, dz = 1; gravity runs
use the x-z plane, Ny = 1, because the reference applies gravity along z
only, Update.h:148):
  sedov            256^2 point blast, HLLC, absorbing, RK2, CFL 0.8, t = 0.1
  rayleigh_taylor  512 x 1536 (x-z), HLL, g = -0.1, periodic x, reflecting z, t = 5
  thermal_pulse    1024^2 Gaussian temperature pulse, kappa = 0.01, mu = 0.005
  shear_layer      4096^2 periodic shear layer, gamma 5/3, kappa = mu = 1e-4, t = 1
  batch_sod_sedov  512 instances, sides in {64..256}, Sod tubes and blasts
  batch_rt         64 Rayleigh-Taylor instances, 256x768 ... 1024x3072
  blast            the reference's 3-D blast (settings/blast.ini), n^3, PCM
  stratified       the reference's H84 / C91 polytropes from an .ini
  random_problem   seeded random states for parity tests
"""
import math
from dataclasses import dataclass, field

import numpy as np

MASTER_SEED = 12345
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed, stream, n):
    """n uniforms in [0,1) from (seed, stream): splitmix64 of a counter."""
    with np.errstate(over="ignore"):
        key = _mix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + _GOLDEN * np.uint64(stream + 1))
        ctr = np.arange(1, n + 1, dtype=np.uint64)
        x = _mix64(key + _GOLDEN * ctr)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed, stream, n):
    u1 = uniform(seed, 2 * stream, n)
    u2 = uniform(seed, 2 * stream + 1, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


@dataclass
class Problem:
    name: str
    ini: str
    prim: list = field(default_factory=list)   # rho, u, v, w, p, each (Nz, Ny, Nx)
    nsteps: int = 0                              # fixed-step runs (0: run to tend)
    params: object = None

    @property
    def shape(self):
        return self.prim[0].shape

    @property
    def cells(self):
        return int(np.prod(self.prim[0].shape))


def ini_text(sections):
    out = []
    for sec, kv in sections.items():
        out.append("[%s]" % sec)
        for k, v in kv.items():
            if isinstance(v, bool):
                v = "true" if v else "false"
            out.append("%s=%s" % (k, v))
        out.append("")
    return "\n".join(out)


def _parse(ini, parse=None):
    """Params of the .ini text: the library's readInifile by default, or
    the callable `parse` (text -> FvParams) a caller supplies."""
    if parse is not None:
        return parse(ini)
    from fv3d_gb300 import parse_ini
    return parse_ini(ini)


def _centres(p):
    x = p.xmin + (np.arange(p.Nx) + 0.5) * p.dx
    y = p.ymin + (np.arange(p.Ny) + 0.5) * p.dy
    z = p.zmin + (np.arange(p.Nz) + 0.5) * p.dz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return X, Y, Z


def _mesh(nx, ny, nz, xr=(0.0, 1.0), yr=(0.0, 1.0), zr=(0.0, 1.0)):
    return {"Nx": nx, "Ny": ny, "Nz": nz, "xmin": xr[0], "xmax": xr[1], "ymin": yr[0], "ymax": yr[1],
            "zmin": zr[0], "zmax": zr[1]}


def sedov(n=256, gamma=1.4, tend=0.1, cfl=0.8, riemann="hllc", extra=None, name="sedov"):
    """Point blast: rho = 1, u = 0, p = 1e-5, p = (gamma-1)/(pi r0^2) for
    cell centres within r0 = 0.02 of (0.5, 0.5)."""
    sec = {
        "mesh": _mesh(n, n, 1),
        "run": {"tend": tend, "boundaries_x": "absorbing", "boundaries_y": "absorbing",
                "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": riemann, "reconstruction": "plm", "time_stepping": "RK2", "CFL": cfl},
        "physics": {"gamma0": repr(float(gamma)), "problem": name},
    }
    for k, v in (extra or {}).items():
        sec.setdefault(k, {}).update(v)
    ini = ini_text(sec)
    p = _parse(ini)
    X, Y, _ = _centres(p)
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
    rho = np.ones_like(X)
    prs = np.full_like(X, 1e-5)
    prs[r < 0.02] = (p.gamma0 - 1.0) / (math.pi * 0.02 ** 2)
    z = np.zeros_like(X)
    return Problem(name, ini, [rho, z.copy(), z.copy(), z.copy(), prs], params=p)


def rayleigh_taylor(nx=512, nz=1536, g=-0.1, ratio=2.0, tend=5.0, kappa=0.0, mu=0.0, seed=MASTER_SEED,
                    riemann="hll", name="rayleigh_taylor", parse=None):
    """Two layers in the x-z plane: rho = ratio above z = 0.75, 1 below,
    hydrostatic p = 2.5 + g rho (z - 0.75), w perturbed by
    0.01 (1 + cos 4 pi x)(1 + cos(3 pi z / 1.5))/4 plus uniform noise 1e-4.
    `parse` (optional): the .ini parser to use (see _parse)."""
    sec = {
        "mesh": _mesh(nx, 1, nz, xr=(0.0, 0.5), zr=(0.0, 1.5)),
        "run": {"tend": tend, "boundaries_x": "periodic", "boundaries_y": "periodic",
                "boundaries_z": "reflecting"},
        "solvers": {"riemann_solver": riemann, "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.8},
        "physics": {"gamma0": 1.4, "gravity": True, "g": repr(float(g)), "problem": name},
    }
    if kappa:
        sec["thermal_conduction"] = {"active": True, "kappa": repr(float(kappa))}
    if mu:
        sec["viscosity"] = {"active": True, "mu": repr(float(mu))}
    ini = ini_text(sec)
    p = _parse(ini, parse)
    X, _, Z = _centres(p)
    rho = np.where(Z > 0.75, ratio, 1.0)
    prs = 2.5 + p.g * rho * (Z - 0.75)
    noise = uniform(seed, 7, X.size).reshape(X.shape)
    w = 0.01 * (1.0 + np.cos(4 * np.pi * X)) * (1.0 + np.cos(3 * np.pi * Z / 1.5)) / 4.0 + 1e-4 * (2 * noise - 1)
    z = np.zeros_like(X)
    return Problem(name, ini, [rho, z.copy(), z.copy(), w, prs], params=p)


def thermal_pulse(n=1024, nsteps=200, kappa=0.01, mu=0.005, name="thermal_pulse"):
    """rho = 1 at rest, T = 1 + exp(-r^2 / (2 * 0.05^2)), p = rho T (R = 1);
    constant conduction and viscosity, periodic, HLLC, a fixed step count."""
    sec = {
        "mesh": _mesh(n, n, 1),
        "run": {"tend": 1.0e30, "boundaries_x": "periodic", "boundaries_y": "periodic",
                "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.8},
        "physics": {"gamma0": 1.4, "problem": name},
        "thermal_conduction": {"active": True, "kappa": repr(float(kappa))},
        "viscosity": {"active": True, "mu": repr(float(mu))},
    }
    ini = ini_text(sec)
    p = _parse(ini)
    X, Y, _ = _centres(p)
    r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2
    T = 1.0 + np.exp(-r2 / (2 * 0.05 ** 2))
    rho = np.ones_like(X)
    z = np.zeros_like(X)
    return Problem(name, ini, [rho, z.copy(), z.copy(), z.copy(), rho * T], nsteps=nsteps, params=p)


def shear_layer(n=4096, tend=1.0, kappa=1e-4, mu=1e-4, seed=MASTER_SEED, name="shear_layer"):
    """Periodic shear layer: rho = 2, u = +0.5 for |y - 0.5| < 0.25, else
    rho = 1, u = -0.5; p = 2.5; v = 1e-2 sin(4 pi x) + N(0, 1e-3); gamma 5/3."""
    sec = {
        "mesh": _mesh(n, n, 1),
        "run": {"tend": tend, "boundaries_x": "periodic", "boundaries_y": "periodic",
                "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.8},
        "physics": {"gamma0": repr(5.0 / 3.0), "problem": name},
        "thermal_conduction": {"active": bool(kappa), "kappa": repr(float(kappa))},
        "viscosity": {"active": bool(mu), "mu": repr(float(mu))},
    }
    ini = ini_text(sec)
    p = _parse(ini)
    X, Y, _ = _centres(p)
    inner = np.abs(Y - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    u = np.where(inner, 0.5, -0.5)
    v = 1e-2 * np.sin(4 * np.pi * X) + 1e-3 * normal(seed, 3, X.size).reshape(X.shape)
    z = np.zeros_like(X)
    return Problem(name, ini, [rho, u, v, z, np.full_like(X, 2.5)], params=p)


def sod(n=128, axis="x", gamma=1.4, nx_other=None, tend=0.2, name="sod"):
    """Sod tube along x or y: (rho, p) = (1, 1) for position <= 0.5, else
    (0.125, 0.1); reflecting walls (settings/sod_x.ini:16-18)."""
    other = nx_other or n
    nx, ny = (n, other) if axis == "x" else (other, n)
    sec = {
        "mesh": _mesh(nx, ny, 1),
        "run": {"tend": tend, "boundaries_x": "reflecting", "boundaries_y": "reflecting",
                "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.8},
        "physics": {"gamma0": repr(float(gamma)), "problem": "sod_" + axis},
    }
    ini = ini_text(sec)
    p = _parse(ini)
    X, Y, _ = _centres(p)
    pos = X if axis == "x" else Y
    left = pos <= 0.5
    rho = np.where(left, 1.0, 0.125)
    prs = np.where(left, 1.0, 0.1)
    z = np.zeros_like(X)
    return Problem(name + "_" + axis, ini, [rho, z.copy(), z.copy(), z.copy(), prs], params=p)


def blast(n=64, nz=None, tend=0.2, cfl=0.1, riemann="hllc", recon="pcm", name="blast"):
    """The reference's blast problem (Init.h:72-100) on an n x n x nz grid
    (settings/blast.ini: 64^3, PCM, HLLC, periodic, CFL 0.1): rho = 1,
    p = 10 within r < 0.2 of the centre, rho = 1.2, p = 0.1 outside."""
    nz = n if nz is None else nz
    sec = {
        "mesh": _mesh(n, n, nz),
        "run": {"tend": tend, "boundaries_x": "periodic", "boundaries_y": "periodic",
                "boundaries_z": "periodic"},
        "solvers": {"riemann_solver": riemann, "reconstruction": recon, "CFL": cfl},
        "physics": {"gamma0": 1.4, "problem": "blast"},
    }
    ini = ini_text(sec)
    p = _parse(ini)
    X, Y, Z = _centres(p)
    xr = 0.5 * (p.xmin + p.xmax) - X
    yr = 0.5 * (p.ymin + p.ymax) - Y
    zr = 0.5 * (p.zmin + p.zmax) - Z
    r = np.sqrt(xr * xr + yr * yr + zr * zr)
    inside = r < 0.2
    rho = np.where(inside, 1.0, 1.2)
    prs = np.where(inside, 10.0, 0.1)
    z = np.zeros_like(X)
    return Problem(name, ini, [rho, z.copy(), z.copy(), z.copy(), prs], params=p)


def stratified(ini, seed=None):
    """The reference's H84 / C91 generators (Init.h:104-148) for the .ini
    text `ini` (problem = H84 or C91): polytropic rho, p from cell centres,
    the perturbation drawn per cell from stream 31 (H84) / 32 (C91) of
    [misc] seed -- the same numbers as the fv3d driver draws (the reference
    draws them from Kokkos' XorShift64 pool instead)."""
    p = _parse(ini)
    name = p.problem.decode()
    X, Y, Z = _centres(p)
    n = X.size
    s = p.seed if seed is None else seed
    z = np.zeros_like(X)
    if name == "H84":
        rho = np.power(Z, p.m1)
        prs = np.power(Z, p.m1 + 1.0)
        w = p.h84_pert * (uniform(s, 31, n).reshape(X.shape) - 0.5)
        return Problem(name, ini, [rho, z.copy(), z.copy(), w, prs], params=p)
    if name == "C91":
        T = 1.0 + p.theta1 * Z
        rho = np.power(T, p.m1)
        prs = np.power(T, p.m1 + 1.0)
        prs = prs * (1.0 + p.c91_pert * (uniform(s, 32, n).reshape(X.shape) - 0.5))
        return Problem(name, ini, [rho, z.copy(), z.copy(), z.copy(), prs], params=p)
    raise ValueError("not a stratified problem: %s" % name)


def random_state(shape, seed, wmag=0.0, vmag=1.5):
    """Seeded random primitive fields: rho, p in [0.5, 2), u, v in
    (-vmag, vmag), w in (-wmag, wmag)."""
    n = int(np.prod(shape))
    u = lambda s: uniform(seed, s, n).reshape(shape)  # noqa: E731
    rho = 0.5 + 1.5 * u(1)
    prs = 0.5 + 1.5 * u(2)
    vx = vmag * (2 * u(3) - 1)
    vy = vmag * (2 * u(4) - 1)
    vz = wmag * (2 * u(5) - 1)
    return [rho, vx, vy, vz, prs]


def random_problem(name, mesh, run, solvers, physics, seed, extra=None, wmag=0.0, vmag=1.5):
    """A random state on the grid of `mesh` with the given .ini sections."""
    sec = {"mesh": mesh, "run": run, "solvers": solvers, "physics": physics}
    sec.update(extra or {})
    ini = ini_text(sec)
    p = _parse(ini)
    return Problem(name, ini, random_state((p.Nz, p.Ny, p.Nx), seed, wmag=wmag, vmag=vmag), params=p)


def batch_sod_sedov(n_inst=512, nsteps=200, seed=MASTER_SEED, sides=(64, 96, 128, 192, 256)):
    """Independent instances: side from `sides`, gamma ~ U[1.1, 1.67];
    even ids Sod tubes (x or y by a coin flip), odd ids point blasts."""
    us = uniform(seed, 11, n_inst)
    ug = uniform(seed, 12, n_inst)
    ua = uniform(seed, 13, n_inst)
    out = []
    for i in range(n_inst):
        n = sides[min(int(us[i] * len(sides)), len(sides) - 1)]
        gamma = 1.1 + 0.57 * ug[i]
        if i % 2 == 0:
            pr = sod(n, "x" if ua[i] < 0.5 else "y", gamma=gamma)
        else:
            pr = sedov(n, gamma=gamma, tend=1.0e30)
        pr.nsteps = nsteps
        out.append(pr)
    return out


def batch_rt(n_inst=64, nsteps=500, seed=MASTER_SEED, kappa=1e-4, mu=1e-4):
    """Rayleigh-Taylor instances with Nx a multiple of 64 in [256, 1024],
    Nz = 3 Nx, g ~ -U[0.05, 0.2], density ratio ~ U[1.5, 3]."""
    un = uniform(seed, 21, n_inst)
    ugr = uniform(seed, 22, n_inst)
    urt = uniform(seed, 23, n_inst)
    out = []
    for i in range(n_inst):
        nx = 64 * (4 + min(int(un[i] * 13), 12))
        g = -(0.05 + 0.15 * ugr[i])
        ratio = 1.5 + 1.5 * urt[i]
        pr = rayleigh_taylor(nx, 3 * nx, g=g, ratio=ratio, tend=1.0e30, kappa=kappa, mu=mu, seed=seed + i)
        pr.nsteps = nsteps
        out.append(pr)
    return out


BUILDERS = {
    "sedov": sedov,
    "rayleigh_taylor": rayleigh_taylor,
    "thermal_pulse": thermal_pulse,
    "shear_layer": shear_layer,
    "sod": sod,
    "blast": blast,
}
