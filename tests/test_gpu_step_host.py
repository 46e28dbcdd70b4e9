"""fvgpu_step_host: one step from and to caller arrays the GPU addresses
directly (pinned host memory, ordinary host memory where the device reads
pageable memory, device memory).

It must equal set_prim + compute_dt + step + get_prim bit for bit (the same
primToCons / consToPrim round trip and CFL dt as the reference's set-up),
for the 2-D plane kernels and the 3-D kernel, with a given dt and with the
CFL dt.
"""
import ctypes as C

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def _cases():
    out = {
        "rt_xz_no_v": problems.rayleigh_taylor(64, 192),
        "thermal_xy_visc": problems.thermal_pulse(96),
        "blast_3d_euler": problems.blast(24, nz=20),
        "random_3d_c91": problems.random_problem(
            "c91", problems._mesh(20, 18, 16),
            {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "reflecting", "boundaries_z": "C91"},
            {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.3},
            {"gamma0": 1.4, "gravity": True, "g": -1.0}, seed=401, wmag=0.3, vmag=0.3,
            extra={"polytrope": {"theta1": 1.5}}),
    }
    out["rt_xz_no_v"].prim[2] = None  # v: identically zero in the x-z plane, not passed
    return out


CASES = _cases()


def _reference_path(pr, dt=None):
    sim = fv.Simulation(pr.params)
    sim.set_prim(*[np.zeros(pr.shape) if a is None else a for a in pr.prim])
    d = sim.compute_dt() if dt is None else dt
    sim.step(d)
    return sim.get_prim(), d


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("given_dt", [False, True])
def test_step_host_pinned_equals_set_step_get(name, given_dt):
    torch = pytest.importorskip("torch")
    pr = CASES[name]
    want, dt_want = _reference_path(pr, dt=1.0e-4 if given_dt else None)
    pin_in = [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
              for a in pr.prim]
    pin_out = [torch.empty(pr.shape, dtype=torch.float64).pin_memory().numpy() for _ in range(5)]
    sim = fv.Simulation(pr.params)
    for _ in range(2):  # a second call starts again from prim_in
        got, dt_used = sim.step_host(pin_in, dt=1.0e-4 if given_dt else 0.0, out=pin_out)
        assert dt_used == dt_want
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)
    # the handle keeps the result
    for a, b in zip(sim.get_prim(), want):
        np.testing.assert_array_equal(a, b)


def test_step_host_pageable_or_refused():
    pr = CASES["thermal_xy_visc"]
    want, dt_want = _reference_path(pr)
    sim = fv.Simulation(pr.params)
    try:
        got, dt_used = sim.step_host([np.ascontiguousarray(a) for a in pr.prim])
    except fv.FvError as e:  # a device that cannot read pageable memory
        assert e.status == 1
        return
    assert dt_used == dt_want
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_step_host_device_arrays():
    torch = pytest.importorskip("torch")
    pr = CASES["random_3d_c91"]
    want, dt_want = _reference_path(pr)
    dev_in = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in pr.prim]
    dev_out = [torch.empty(pr.shape, dtype=torch.float64, device="cuda") for _ in range(5)]
    sim = fv.Simulation(pr.params)
    ins = (_dp * 5)(*[C.cast(C.c_void_p(t.data_ptr()), _dp) for t in dev_in])
    outs = (_dp * 5)(*[C.cast(C.c_void_p(t.data_ptr()), _dp) for t in dev_out])
    used = C.c_double(0.0)
    torch.cuda.synchronize()
    rc = sim.lib.fvgpu_step_host(sim.handle, ins, 0.0, outs, C.byref(used))
    assert rc == 0, sim.last_error()
    assert used.value == dt_want
    for t, b in zip(dev_out, want):
        np.testing.assert_array_equal(t.cpu().numpy(), b)


def test_step_host_rejects_wrong_layout():
    pr = CASES["thermal_xy_visc"]
    sim = fv.Simulation(pr.params)
    with pytest.raises(ValueError):
        sim.step_host([a.astype(np.float32) for a in pr.prim])


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("given_dt", [False, True])
def test_step_host_then_advance(name, given_dt):
    """Steps run after fvgpu_step_host (which leaves the primitive copy of
    its input and of its result for the next RK2 stage) equal the same steps
    after set_prim + step, bit for bit."""
    pr = CASES[name]
    prim = [np.zeros(pr.shape) if a is None else a for a in pr.prim]
    a = fv.Simulation(pr.params)
    _, dt_a = a.step_host(prim, dt=1.0e-4 if given_dt else 0.0)
    b = fv.Simulation(pr.params)
    b.set_prim(*prim)
    b.step(1.0e-4 if given_dt else b.compute_dt())
    t_a, n_a = a.advance(1.0e30, max_steps=3)
    t_b, n_b = b.advance(1.0e30, max_steps=3)
    assert n_a == n_b == 3 and t_a == t_b
    for x, y in zip(a.get_prim(), b.get_prim()):
        np.testing.assert_array_equal(x, y)
