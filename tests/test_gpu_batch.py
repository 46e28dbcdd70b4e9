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
from _helpers import assert_mixed

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
