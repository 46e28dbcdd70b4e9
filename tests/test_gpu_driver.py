"""The fv3d driver binary: the main.cpp:51-74 loop on the GPU, from a .ini.

Runs fv3d_gb300/_lib/fv3d on a Sod tube settings file (the reference's own
`sod_x` generator, Init.h:19-31, run on the GPU by fvgpu_init_problem) and
checks the final snapshot against the oracle's loop over the same settings
from the oracle's own generator: same number of saves, bit-identical final
primitive state.  Both the host loop (one compute_dt/step round trip
per step, like main.cpp) and --device-loop are run.  Two 3-D settings files
shaped like the reference's settings/sod_x.ini (64 x 16 x 16, reflecting,
PCM, Euler) and settings/blast.ini (periodic cube, PCM, HLLC, CFL 0.1),
with shorter end times, run the same check on the 3-D kernel.
"""
import os
import re
import subprocess

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import build, problems
from oracle import pyoracle

pytestmark = pytest.mark.gpu

INI = """[mesh]
Nx=64
Ny=8
Nz=1
[run]
tend=0.05
save_freq=0.02
boundaries_x=reflecting
boundaries_y=reflecting
boundaries_z=periodic
[solvers]
riemann_solver=hllc
reconstruction=plm
time_stepping=RK2
CFL=0.8
[physics]
gamma0=1.4
problem=sod_x
[misc]
log_frequency=5
"""


def _check_xdmf(tmp_path, shape, nsnaps):
    """The XDMF index lists every snapshot in order, and each data item
    (file, byte offset, dimensions) reads back the snapshot's field."""
    import xml.etree.ElementTree as ET
    root = ET.parse(str(tmp_path / "snap.xdmf")).getroot()
    coll = root.find("Domain/Grid")
    assert coll.get("CollectionType") == "Temporal"
    nz, ny, nx = shape
    geo = coll.findall("Geometry/DataItem")
    assert len(geo) == 3
    xs = np.fromfile(str(tmp_path / geo[0].text), dtype=np.float64, count=(nz + 1) * (ny + 1) * (nx + 1),
                     offset=int(geo[0].get("Seek")))
    assert xs[1] > xs[0] == 0.0
    grids = coll.findall("Grid")
    assert len(grids) == nsnaps
    times = [float(g.find("Time").get("Value")) for g in grids]
    assert times == sorted(times) and times[0] == 0.0
    for g in grids:
        items = g.findall(".//Attribute/DataItem") + g.findall(".//Attribute/DataItem/DataItem")
        items = [d for d in items if d.get("Format") == "Binary"]
        assert len(items) == 5
        for d in items:
            dims = tuple(int(v) for v in d.get("Dimensions").split())
            assert dims == shape
            a = np.fromfile(str(tmp_path / d.text), dtype=np.float64, count=nz * ny * nx, offset=int(d.get("Seek")))
            raw = np.fromfile(str(tmp_path / d.text), dtype=np.float64).reshape(5, nz * ny * nx)
            k = int(d.get("Seek")) // (8 * nz * ny * nx)
            np.testing.assert_array_equal(a, raw[k])
    # the same run through the h5py-like reader the reference's tools can use
    from fv3d_gb300 import snapshots
    f = snapshots.File(str(tmp_path / "snap"))
    assert len(f.keys()) == 3 + nsnaps and f.attrs["Nx"] == nx
    for n, g in enumerate(grids):
        assert f["ite_%d" % n].attrs["time"] == times[n]
        name = g.find(".//Attribute/DataItem").text
        raw = np.fromfile(str(tmp_path / name), dtype=np.float64).reshape(5, nz, ny, nx)
        for v, field in enumerate(("rho", "u", "v", "w", "prs")):
            np.testing.assert_array_equal(f["ite_%d/%s" % (n, field)], raw[v])


@pytest.mark.parametrize("mode", ["host", "device"])
def test_driver_matches_oracle(tmp_path, mode):
    exe = os.path.join(build.lib_dir(), "fv3d")
    assert os.path.exists(exe)
    ini = tmp_path / "sod.ini"
    ini.write_text(INI)
    prefix = str(tmp_path / "snap")
    args = [exe, str(ini), "--out", prefix, "--format", "raw"] + (["--device-loop"] if mode == "device" else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Computing dts at (t=0)" in r.stdout
    m = re.search(r"done: (\d+) steps, t = (\S+)", r.stdout)
    steps, t_end = int(m.group(1)), float(m.group(2))
    snaps = sorted(f for f in os.listdir(tmp_path) if re.fullmatch(r"snap_\d{4}\.bin", f))
    assert len(snaps) == r.stdout.count("Saving at time") + 1

    p = fv.parse_ini(INI)
    ora = pyoracle.Oracle(p)
    q0 = ora.generate()
    np.testing.assert_array_equal(np.stack(q0), np.stack(problems.sod(64, "x", nx_other=8).prim))
    t_o, n_o = ora.advance(p.tend)
    assert (steps, t_end) == (n_o, t_o)
    got = np.fromfile(str(tmp_path / snaps[-1]), dtype=np.float64).reshape(5, 1, 8, 64)
    np.testing.assert_array_equal(got, np.stack(ora.get_prim()))
    _check_xdmf(tmp_path, (1, 8, 64), len(snaps))


SOD_3D = """[mesh]
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
"""

BLAST_3D = """[mesh]
Nx=32
Ny=32
Nz=32
[run]
tend=0.01
save_freq=0.004
boundaries_x=periodic
boundaries_y=periodic
boundaries_z=periodic
[solvers]
riemann_solver=hllc
reconstruction=pcm
CFL=0.1
[physics]
gamma0=1.4
problem=blast
"""


def _ic_3d(p, problem):
    if problem == "blast":
        return problems.blast(p.Nx, nz=p.Nz).prim
    X = p.xmin + (np.arange(p.Nx) + 0.5) * p.dx
    left = np.broadcast_to(X <= 0.5, (p.Nz, p.Ny, p.Nx))
    z = np.zeros((p.Nz, p.Ny, p.Nx))
    return [np.where(left, 1.0, 0.125), z, z, z, np.where(left, 1.0, 0.1)]


@pytest.mark.parametrize("problem", ["sod_x", "blast"])
def test_driver_3d_matches_oracle(tmp_path, problem):
    text = SOD_3D if problem == "sod_x" else BLAST_3D
    exe = os.path.join(build.lib_dir(), "fv3d")
    ini = tmp_path / "run.ini"
    ini.write_text(text)
    prefix = str(tmp_path / "snap")
    r = subprocess.run([exe, str(ini), "--out", prefix, "--device-loop", "--format", "raw"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"done: (\d+) steps, t = (\S+)", r.stdout)
    steps, t_end = int(m.group(1)), float(m.group(2))
    snaps = sorted(f for f in os.listdir(tmp_path) if re.fullmatch(r"snap_\d{4}\.bin", f))
    p = fv.parse_ini(text)
    ora = pyoracle.Oracle(p)
    np.testing.assert_array_equal(np.stack(ora.generate()), np.stack(_ic_3d(p, problem)))
    t_o, n_o = ora.advance(p.tend)
    assert (steps, t_end) == (n_o, t_o)
    got = np.fromfile(str(tmp_path / snaps[-1]), dtype=np.float64).reshape(5, p.Nz, p.Ny, p.Nx)
    np.testing.assert_array_equal(got, np.stack(ora.get_prim()))


# settings/C91.ini with a smaller grid and end time: 3-D, C91 z boundary,
# fixed-temperature / fixed-gradient conduction boundaries, viscosity, gravity.
# With these settings the reference's own run turns non-finite after a few
# steps (its C91 ghost fill scales the hydrostatic term by the boolean
# params.gravity instead of g = 40, BoundaryConditions.h:104); the end time
# keeps the run to the first two steps, before that.
C91_3D = """[mesh]
Nx=16
Ny=16
Nz=8
xmin=0.0
xmax=4.0
ymin=0.0
ymax=4.0
zmin=0.0
zmax=1.0
[run]
tend=0.002
save_freq=0.001
boundaries_x=periodic
boundaries_y=periodic
boundaries_z=C91
[solvers]
riemann_solver=hllc
reconstruction=plm
CFL=0.1
[physics]
gamma0=1.66666667
problem=C91
gravity=true
g=40.0
[C91]
perturbation=1.0e-3
[polytrope]
theta1=20.0
m1=1.0
[thermal_conduction]
active=true
kappa=0.07
bc_zmin=fixed_temperature
bc_zmax=fixed_gradient
bc_zmin_value=1.0
bc_zmax_value=20.0
[viscosity]
active=true
mu=0.0028
"""

# settings/H84_chi1.5.ini with a smaller grid and end time; Nz is left unset,
# so it takes readInifile's default of 32 (a 3-D run, as in the reference)
H84_3D = """[mesh]
Nx=16
Ny=8
xmin=0.0
xmax=4.0
ymin=2.0
ymax=3.0
[run]
tend=0.01
save_freq=0.005
boundaries_x=periodic
boundaries_y=reflecting
[solvers]
time_stepping=euler
riemann_solver=hllc
reconstruction=plm
CFL=0.1
[physics]
gamma0=1.66666667
problem=H84
gravity=true
g=2.0
[H84]
perturbation=1.0e-4
[thermal_conduction]
active=true
kappa=0.0071
[viscosity]
active=true
mu=0.0028
"""


@pytest.mark.parametrize("problem", ["C91", "H84"])
def test_driver_random_generators_match_oracle(tmp_path, problem):
    """The perturbed stratified problems (Init.h:104-148) run end to end
    from the reference's settings: the driver's generated state (--write-ic)
    advanced by the oracle equals the driver's final snapshot bit for bit."""
    text = C91_3D if problem == "C91" else H84_3D
    exe = os.path.join(build.lib_dir(), "fv3d")
    ini = tmp_path / "run.ini"
    ini.write_text(text)
    prefix = str(tmp_path / "snap")
    ic = str(tmp_path / "ic.bin")
    r = subprocess.run([exe, str(ini), "--out", prefix, "--write-ic", ic, "--device-loop", "--format", "raw"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"done: (\d+) steps, t = (\S+)", r.stdout)
    steps, t_end = int(m.group(1)), float(m.group(2))
    p = fv.parse_ini(text)
    if problem == "H84":
        assert p.Nz == 32
    shape = (p.Nz, p.Ny, p.Nx)
    q0 = np.fromfile(ic, dtype=np.float64).reshape(5, *shape)
    assert np.all(np.isfinite(q0))
    pert = q0[3] if problem == "H84" else q0[4]
    assert np.std(pert) > 0  # the perturbation is present
    ora = pyoracle.Oracle(p)
    ora.set_prim(*q0)
    t_o, n_o = ora.advance(p.tend)
    assert (steps, t_end) == (n_o, t_o)
    snaps = sorted(f for f in os.listdir(tmp_path) if re.fullmatch(r"snap_\d{4}\.bin", f))
    got = np.fromfile(str(tmp_path / snaps[-1]), dtype=np.float64).reshape(5, *shape)
    np.testing.assert_array_equal(got, np.stack(ora.get_prim()))


def test_driver_rejects_unknown_problem(tmp_path):
    exe = os.path.join(build.lib_dir(), "fv3d")
    ini = tmp_path / "x.ini"
    ini.write_text(INI.replace("sod_x", "kelvin_helmholtz"))
    r = subprocess.run([exe, str(ini)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "unknown problem" in r.stderr


@pytest.mark.parametrize("fmt", ["raw", "h5"])
@pytest.mark.parametrize("mode", ["host", "device"])
def test_driver_restart_continues_bit_for_bit(tmp_path, mode, fmt):
    """A run stopped at tend/2 and resumed with --restart ends in the same
    state, bit for bit, as the uninterrupted run (the checkpoint holds the
    conserved state), and the XDMF index (raw) or the HDF5 file keeps every
    snapshot."""
    exe = os.path.join(build.lib_dir(), "fv3d")
    extra = (["--device-loop"] if mode == "device" else []) + ["--format", fmt]
    full = tmp_path / "full"
    part = tmp_path / "part"
    full.mkdir()
    part.mkdir()
    (full / "run.ini").write_text(INI)
    r = subprocess.run([exe, str(full / "run.ini"), "--out", str(full / "snap")] + extra, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    n_full = int(re.search(r"done: (\d+) steps", r.stdout).group(1))
    (part / "half.ini").write_text(INI.replace("tend=0.05", "tend=0.025"))
    (part / "run.ini").write_text(INI)
    r = subprocess.run([exe, str(part / "half.ini"), "--out", str(part / "snap")] + extra, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    n_half = int(re.search(r"done: (\d+) steps", r.stdout).group(1))
    r = subprocess.run([exe, str(part / "run.ini"), "--out", str(part / "snap"), "--restart"] + extra,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"done: (\d+) steps, t = (\S+)", r.stdout)
    assert int(m.group(1)) == n_full > n_half
    if fmt == "h5":
        # the final saves hold the same state; the resumed file keeps every
        # save of both legs (the first leg's final save included), in order
        from fv3d_gb300 import snapshots
        a, b = snapshots.File(str(full / "snap.h5")), snapshots.File(str(part / "snap.h5"))
        ka = sorted((k for k in a.keys() if k.startswith("ite_")), key=lambda k: int(k[4:]))
        kb = sorted((k for k in b.keys() if k.startswith("ite_")), key=lambda k: int(k[4:]))
        assert kb == ["ite_%d" % i for i in range(len(kb))] and len(kb) == len(ka) + 1
        assert a[ka[-1]].attrs["time"] == b[kb[-1]].attrs["time"]
        for field in ("rho", "u", "v", "w", "prs"):
            np.testing.assert_array_equal(a[ka[-1] + "/" + field], b[kb[-1] + "/" + field])
        times = [b[k].attrs["time"] for k in kb]
        assert times == sorted(times)
        return
    last = lambda d: sorted(f for f in os.listdir(d) if re.fullmatch(r"snap_\d{4}\.bin", f))[-1]
    a = np.fromfile(str(full / last(full)), dtype=np.float64)
    b = np.fromfile(str(part / last(part)), dtype=np.float64)
    np.testing.assert_array_equal(a, b)
    nsnaps = len([f for f in os.listdir(part) if re.fullmatch(r"snap_\d{4}\.bin", f)])
    _check_xdmf(part, (1, 8, 64), nsnaps)


def test_driver_hdf5_snapshots_equal_raw(tmp_path):
    """The default output, <out>.h5 in the reference's layout (root
    attributes, x / y / z, ite_<n>/{rho,u,v,w,prs} with a time attribute)
    with an XDMF index naming its datasets, holds what --format raw writes."""
    exe = os.path.join(build.lib_dir(), "fv3d")
    ini = tmp_path / "sod.ini"
    ini.write_text(INI)
    for fmt, d in (("raw", "raw"), ("h5", "h5")):
        (tmp_path / d).mkdir()
        r = subprocess.run([exe, str(ini), "--out", str(tmp_path / d / "snap")] + (["--format", fmt] if fmt == "raw"
                                                                                   else []),
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
    assert not any(re.fullmatch(r"snap_\d{4}\.bin", f) for f in os.listdir(tmp_path / "h5"))
    from fv3d_gb300 import snapshots
    h5 = snapshots.File(str(tmp_path / "h5" / "snap"))
    raw = snapshots.File(str(tmp_path / "raw" / "snap"))
    assert isinstance(raw, snapshots.File) and not isinstance(h5, snapshots.File)
    assert sorted(h5.keys()) == sorted(raw.keys())
    p = fv.parse_ini(INI)
    for k in ("Nx", "Ny", "Nz", "Ntx", "Nty", "Ntz", "ibeg", "iend", "jbeg", "jend", "kbeg", "kend"):
        assert h5.attrs[k] == raw.attrs[k]
    assert h5.attrs["problem"] == b"sod_x" and p.Nx == h5.attrs["Nx"]
    for k in ("x", "y", "z"):
        np.testing.assert_array_equal(h5[k], raw[k])
    for k in raw.keys():
        if k.startswith("ite_"):
            assert h5[k].attrs["time"] == raw[k].attrs["time"]
            for field in ("rho", "u", "v", "w", "prs"):
                np.testing.assert_array_equal(h5[k + "/" + field], raw[k + "/" + field])
    import xml.etree.ElementTree as ET
    items = [d.text for d in ET.parse(str(tmp_path / "h5" / "snap.xdmf")).getroot().iter("DataItem")
             if d.get("Format") == "HDF"]
    assert items[:3] == ["snap.h5:/x", "snap.h5:/y", "snap.h5:/z"] and "snap.h5:/ite_0/rho" in items


def test_driver_restart_needs_a_checkpoint(tmp_path):
    exe = os.path.join(build.lib_dir(), "fv3d")
    (tmp_path / "run.ini").write_text(INI)
    r = subprocess.run([exe, str(tmp_path / "run.ini"), "--out", str(tmp_path / "none"), "--restart"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "checkpoint" in r.stderr
