"""Batches: many independent problems in one persistent launch per stage.

FP64 batches must reproduce, bit for bit, each problem advanced alone (which
itself reproduces the reference bit for bit), whatever tile shape the
autotuner picks.  The FP32-mixed form must stay within the mixed-form
bounds of the FP64 result on every field (assert_mixed: relative L1 1e-5 on
density and pressure, velocities within 1e-5 of the signal speed).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import assert_mixed, rel_l1_fields

pytestmark = pytest.mark.gpu


def mixed_set():
    """Uneven sizes (some not powers of two), several gammas, both planes,
    conduction/viscosity in one x-z problem (a second group)."""
    return [
        problems.sod(64, "x", gamma=1.3, nx_other=48),
        problems.sedov(96, gamma=1.5, tend=1.0e30),
        problems.sod(48, "y", gamma=1.62, nx_other=40),
        problems.rayleigh_taylor(32, 96, kappa=1e-3, mu=1e-3, tend=1.0e30),
        problems.sedov(64, gamma=1.2, tend=1.0e30),
        problems.rayleigh_taylor(48, 144, riemann="hllc", tend=1.0e30),
    ]


def run_singles(probs, nsteps):
    out, times = [], []
    for pr in probs:
        s = fv.Simulation(pr.params)
        s.set_prim(*pr.prim)
        t, n = s.advance(1.0e30, max_steps=nsteps)
        assert n == nsteps
        out.append(s.get_prim())
        times.append(t)
        s.close()
    return out, times


def test_fp64_strip_march_equals_tiles():
    """The single-problem FP64 kernel marches strips of rows (several blocks
    per CTA, segments that cross strip ends, viscous fluxes computed once per
    face); the batch kernel computes independent tiles with the per-cell
    viscous formula.  On grids large enough for multi-block strips the two
    agree bit for bit (x-z viscosity with gravity, x-y conduction + viscosity,
    Euler ping-pong)."""
    probs = [problems.rayleigh_taylor(128, 1536, kappa=1e-3, mu=1e-3, tend=1.0e30),
             problems.thermal_pulse(512),
             problems.shear_layer(320, kappa=0.0, mu=2e-3),
             problems.random_problem("euler_pcm", problems._mesh(90, 2600, 1),
                                     {"tend": 1.0, "boundaries_x": "absorbing", "boundaries_y": "reflecting",
                                      "boundaries_z": "periodic"},
                                     {"riemann_solver": "hllc", "reconstruction": "pcm", "time_stepping": "euler",
                                      "CFL": 0.5}, {"gamma0": 1.4}, seed=77)]
    for pr in probs:
        b = fv.Batch([pr.params])
        b.set_prim(0, *pr.prim)
        b.run(3)
        ref, ref_t = run_singles([pr], 3)
        assert b.times()[0] == ref_t[0], pr.name
        for k, (x, y) in enumerate(zip(b.get_prim(0), ref[0])):
            np.testing.assert_array_equal(x, y, err_msg="%s field %d" % (pr.name, k))


@pytest.mark.parametrize("nsteps", [3, 11])
def test_fp64_batch_bitwise_equals_single(nsteps):
    probs = mixed_set()
    b = fv.Batch([p.params for p in probs])
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(nsteps)
    t = b.times()
    ref, ref_t = run_singles(probs, nsteps)
    for i in range(len(probs)):
        assert t[i] == ref_t[i], (i, t[i], ref_t[i])
        for k, (x, y) in enumerate(zip(b.get_prim(i), ref[i])):
            np.testing.assert_array_equal(x, y, err_msg="problem %d field %d" % (i, k))
    assert len(set(t.tolist())) == len(probs)  # every problem has its own dt
    assert b.launch_count() > 0
    assert len(b.tiling()) == 3  # x-y; x-z with conduction/viscosity; x-z without


def test_fp64_batch_state_replaced_after_steps():
    """A problem whose state is set again after some steps restarts from that
    state (the primitive copy an RK2 stage 2 kept of its old state is not
    reused) while the other problems carry on."""
    probs = mixed_set()
    b = fv.Batch([p.params for p in probs])
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(3)
    replaced = 1  # the 96^2 Sedov problem
    pr = probs[replaced]
    other = [None if a is None else a.copy() for a in pr.prim]
    other[0] = other[0] * 1.25
    other[4] = other[4] * 0.8
    b.set_prim(replaced, *other)
    b.run(4)
    ref, _ = run_singles([problems.Problem(pr.name, pr.ini, other, params=pr.params)], 4)
    for k, (x, y) in enumerate(zip(b.get_prim(replaced), ref[0])):
        np.testing.assert_array_equal(x, y, err_msg="field %d" % k)
    kept, _ = run_singles([probs[0]], 7)
    for k, (x, y) in enumerate(zip(b.get_prim(0), kept[0])):
        np.testing.assert_array_equal(x, y, err_msg="kept problem field %d" % k)


def _run_forced_tile(tile, nsteps):
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
        "import fv3d_gb300 as fv\n"
        "from test_gpu_batch import mixed_set\n"
        "probs = mixed_set()\n"
        "b = fv.Batch([p.params for p in probs])\n"
        "[b.set_prim(i, *pr.prim) for i, pr in enumerate(probs)]\n"
        "b.run(%d)\n"
        "np.save(sys.argv[1], np.concatenate([np.stack(b.get_prim(i)).ravel() for i in range(len(probs))]))\n"
        "print(b.tiling())\n"
    ) % (os.path.dirname(os.path.dirname(os.path.abspath(__file__))), os.path.dirname(os.path.abspath(__file__)),
         nsteps)
    return code


@pytest.mark.parametrize("tile", ["32x16", "32x32", "64x32", "32x64", "32x21", "64x13"])
def test_fp64_batch_independent_of_tile_shape(tile, tmp_path):
    """Forcing another work-item shape (FV3D_TILE: strip width x rows, rows
    not a whole number of marching blocks included) gives the same bits."""
    nsteps = 5
    probs = mixed_set()
    ref, _ = run_singles(probs, nsteps)
    want = np.concatenate([np.stack(r).ravel() for r in ref])
    out = str(tmp_path / "x.npy")
    env = dict(os.environ, FV3D_TILE=tile)
    r = subprocess.run([sys.executable, "-c", _run_forced_tile(tile, nsteps), out], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "(%s, %s)" % tuple(tile.split("x")) in r.stdout
    np.testing.assert_array_equal(np.load(out), want)


def test_fp64_batch_fresh_autotune_keeps_state(tmp_path):
    """With an empty tile cache the autotuner times whole RK2 steps on the
    problems' own state (stage 2 overwrites U^n) and puts U^n back: the run
    that follows gives the same bits as each problem advanced alone."""
    nsteps = 5
    probs = mixed_set()
    ref, _ = run_singles(probs, nsteps)
    want = np.concatenate([np.stack(r).ravel() for r in ref])
    out = str(tmp_path / "x.npy")
    env = dict(os.environ, FV3D_TILE_CACHE=str(tmp_path / "tiles.txt"), FV3D_TILE_LOG="1")
    env.pop("FV3D_TILE", None)
    r = subprocess.run([sys.executable, "-c", _run_forced_tile(None, nsteps), out], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "fv3d tile candidate" in r.stderr  # the tuning ran
    np.testing.assert_array_equal(np.load(out), want)


def test_fp64_batch_euler_pingpong():
    probs = [problems.sod(64, "x"), problems.sedov(48, tend=1.0e30), problems.sod(40, "y")]
    for pr in probs:
        pr.params.time_stepping = fv._abi.FV_TS_EULER
    b = fv.Batch([p.params for p in probs])
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(5)    # odd: the state ends in the second buffer
    b.run(9)    # starts with one step to realign, then one graph replay
    ref, ref_t = run_singles(probs, 14)
    t = b.times()
    for i in range(len(probs)):
        assert t[i] == ref_t[i]
        for x, y in zip(b.get_prim(i), ref[i]):
            np.testing.assert_array_equal(x, y)


def test_mixed_batch_l1_against_fp64():
    """FP32-mixed vs FP64 after 200 steps: every field within the mixed-form
    bounds (assert_mixed)."""
    probs = [problems.sod(128, "x", nx_other=32), problems.sedov(96, tend=1.0e30),
             problems.sod(64, "y", gamma=1.6, nx_other=48), problems.sedov(128, gamma=1.3, tend=1.0e30)]
    nsteps = 200
    ref, ref_t = run_singles(probs, nsteps)
    params = []
    for pr in probs:
        q = pr.params.copy()
        q.precision = fv._abi.FV_PREC_FP32_MIXED
        params.append(q)
    b = fv.Batch(params)
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(nsteps)
    t = b.times()
    for i in range(len(probs)):
        assert_mixed(b.get_prim(i), ref[i], probs[i].params.gamma0, i)
        assert abs(t[i] - ref_t[i]) <= 1e-4 * ref_t[i], (i, t[i], ref_t[i])


def test_mixed_batch_rt_with_diffusion():
    probs = [problems.rayleigh_taylor(64, 192, kappa=1e-4, mu=1e-4, tend=1.0e30),
             problems.rayleigh_taylor(32, 96, g=-0.15, ratio=2.5, kappa=1e-4, mu=1e-4, tend=1.0e30)]
    nsteps = 100
    ref, _ = run_singles(probs, nsteps)
    params = []
    for pr in probs:
        q = pr.params.copy()
        q.precision = fv._abi.FV_PREC_FP32_MIXED
        params.append(q)
    b = fv.Batch(params)
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(nsteps)
    for i in range(len(probs)):
        assert_mixed(b.get_prim(i), ref[i], probs[i].params.gamma0, i)


def test_batch_nonfinite_reported():
    probs = [problems.sedov(64, tend=1.0e30), problems.sod(64, "x")]
    prim = [a.copy() for a in probs[1].prim]
    prim[4][0, 3, 5] = -1.0
    b = fv.Batch([p.params for p in probs])
    b.set_prim(0, *probs[0].prim)
    b.set_prim(1, *prim)
    b.run(2)
    with pytest.raises(fv.FvError) as e:
        b.times()
    assert e.value.status == 4


def test_batch_rejects_mixed_settings():
    a = problems.sod(32, "x").params
    c = problems.sod(32, "x").params
    c.time_stepping = fv._abi.FV_TS_EULER
    with pytest.raises(fv.FvError) as e:
        fv.Batch([a, c])
    assert e.value.status == 2


def _schedule_set():
    """Both planes, with and without viscosity (three groups)."""
    return [problems.rayleigh_taylor(48, 144, kappa=1e-3, mu=1e-3, tend=1.0e30),
            problems.thermal_pulse(80),
            problems.sod(70, "x", gamma=1.3, nx_other=45)]


def _run_forced(probs, tile, nsteps, monkeypatch):
    monkeypatch.setenv("FV3D_TILE", tile)
    params = []
    for pr in probs:
        q = pr.params.copy()
        q.precision = fv._abi.FV_PREC_FP32_MIXED
        params.append(q)
    b = fv.Batch(params)
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    sched = b.schedule()
    b.run(nsteps)
    out = [b.get_prim(i) for i in range(len(probs))], b.times()
    b.close()
    return sched, out


@pytest.mark.parametrize("tile,block,split", [("32x16/8", 8, 0), ("64x24/8", 8, 0), ("32x40/16", 16, 0),
                                              ("32x16v", 16, 1), ("64x20v", 16, 1)])
def test_mixed_schedules(tile, block, split, monkeypatch):
    """Every mixed schedule -- blocks of 8 or 16 rows (one to four cells per
    thread in the update), viscous fluxes fused per cell or computed once per
    face -- is reported by fvgpu_batch_schedule and gives the same flow:
    bit for bit across block sizes of one viscous form, to FP32 rounding
    across the two forms (relative L1 <= 1e-6 on density and pressure,
    velocities within 1e-6 of the signal speed)."""
    probs = _schedule_set()
    nsteps = 12
    sched, (got, t) = _run_forced(probs, tile, nsteps, monkeypatch)
    tx, rows = (int(x) for x in tile.rstrip("v").split("/")[0].split("x"))
    assert len(sched) == 3
    for s in sched:
        assert (s["tx"], s["rows"], s["block_rows"], s["split_viscous"]) == (tx, rows, block, split)
    base_sched, (ref, t_ref) = _run_forced(probs, "32x16", nsteps, monkeypatch)
    assert all(s["block_rows"] == 16 and s["split_viscous"] == 0 for s in base_sched)
    for i, pr in enumerate(probs):
        if split == 0 or not pr.params.viscosity_active:
            np.testing.assert_array_equal(t[i], t_ref[i])
            for k in range(5):
                np.testing.assert_array_equal(got[i][k], ref[i][k], err_msg="%s %d" % (pr.name, k))
        else:
            errs = rel_l1_fields(got[i], ref[i])
            assert errs[0] <= 1e-6 and errs[4] <= 1e-6, (pr.name, errs)
            c = np.sqrt(pr.params.gamma0 * ref[i][4] / ref[i][0])
            speed = float((np.sqrt(ref[i][1] ** 2 + ref[i][2] ** 2 + ref[i][3] ** 2) + c).max())
            for k in (1, 2, 3):
                assert float(np.abs(got[i][k] - ref[i][k]).mean()) <= 1e-6 * speed, (pr.name, k)


def test_autotuned_schedule_is_cached(tmp_path, monkeypatch):
    """A fresh tuning records width, rows, block rows and viscous form per
    group in the tile cache, and a new batch of the same problems takes the
    recorded schedule."""
    cache = tmp_path / "tiles.txt"
    monkeypatch.delenv("FV3D_TILE", raising=False)
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import fv3d_gb300 as fv\n"
            "from test_gpu_batch import _schedule_set\n"
            "probs = _schedule_set()\n"
            "ps = []\n"
            "for p in probs:\n"
            "    q = p.params.copy(); q.precision = 1; ps.append(q)\n"
            "b = fv.Batch(ps)\n"
            "[b.set_prim(i, *p.prim) for i, p in enumerate(probs)]\n"
            "print([tuple(s.values()) for s in b.schedule()])\n") % (
        os.path.dirname(os.path.dirname(os.path.abspath(__file__))), os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FV3D_TILE_CACHE=str(cache))
    env.pop("FV3D_TILE", None)
    first = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert first.returncode == 0, first.stderr[-2000:]
    lines = [l.split() for l in cache.read_text().splitlines() if l.strip()]
    assert len(lines) == 3 and all(len(l) == 5 for l in lines)
    recorded = sorted(tuple(int(x) for x in l[1:]) for l in lines)
    again = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert again.returncode == 0, again.stderr[-2000:]
    assert again.stdout == first.stdout
    assert sorted(eval(first.stdout.strip().splitlines()[-1])) == recorded
    assert len(cache.read_text().splitlines()) == 3  # nothing tuned the second time
