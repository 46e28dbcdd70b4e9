"""fvgpu_step_noalloc: the time step for callers that cannot allocate.

Host codes whose device memory belongs to another allocator (a pool or arena
that already reserved the GPU), or whose time loop cannot take the device
synchronisation of cudaMalloc/cudaFree, keep their conserved state in their
own device arrays and call fvgpu_step_noalloc, which allocates nothing: its
stage scratch is a fixed 32 MiB array in device memory.  These tests drive it
through the C ABI on device arrays with a padded row pitch and check, over
two calls in a row, that it produces the same state as the regular handle
(fvgpu_create / fvgpu_step) within the per-step tolerance of the parity
tests -- in fact bit for bit -- and that the next dt it reports equals
fvgpu_compute_dt's.  Kept in a file pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import REL_L1_STEP, rel_l1_fields

pytestmark = pytest.mark.gpu


def _device_state(torch, cons, pitch, skip):
    """Copies (rho, mx, my, mz, E) into padded device rows; field `skip`
    (the momentum along the one-cell axis) is passed as NULL."""
    nz, ny, nx = cons[0].shape
    rows = nz * ny
    arrs, ptrs = [], (C.c_void_p * 5)()
    for k, a in enumerate(cons):
        if k == skip:
            arrs.append(None)
            ptrs[k] = None
            continue
        t = torch.full((rows, pitch), float("nan"), dtype=torch.float64, device="cuda")
        t[:, :nx] = torch.from_numpy(np.ascontiguousarray(a).reshape(rows, nx)).cuda()
        arrs.append(t)
        ptrs[k] = t.data_ptr()
    return arrs, ptrs


def _to_host(arrs, shape):
    nz, ny, nx = shape
    return [np.zeros(shape) if t is None else t[:, :nx].cpu().numpy().reshape(shape) for t in arrs]


def _sod_euler_null_w():
    pr = problems.sod(96, "y", nx_other=40)
    text = pr.ini.replace("time_stepping=RK2", "time_stepping=euler")
    pr.params = fv.parse_ini(text)
    return pr


def _random_3d_rk2():
    return problems.random_problem(
        "r3", problems._mesh(20, 18, 16),
        {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "absorbing", "boundaries_z": "reflecting"},
        {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2", "CFL": 0.5},
        {"gamma0": 1.4}, seed=4242, wmag=0.7,
        extra={"thermal_conduction": {"active": True, "kappa": 1e-3}, "viscosity": {"active": True, "mu": 1e-3}})


@pytest.mark.parametrize("case", ["rt_xz_null_v", "thermal_xy_visc", "blast_3d_euler", "sod_xy_euler_null_w",
                                  "random_3d_rk2"])
def test_noalloc_matches_handle_two_calls(case):
    torch = pytest.importorskip("torch")
    if case == "rt_xz_null_v":
        pr = problems.rayleigh_taylor(64, 192)
        skip = 2          # rho*v: zero in the x-z plane without viscosity
    elif case == "blast_3d_euler":
        pr = problems.blast(24, nz=20)  # 3-D kernel, Euler stepping (copies U* back)
        skip = -1
    elif case == "sod_xy_euler_null_w":
        pr = _sod_euler_null_w()        # 2-D Euler: copy-back without the third momentum
        skip = 3
    elif case == "random_3d_rk2":
        pr = _random_3d_rk2()           # 3-D RK2: stage 2 writes into the caller's arrays
        skip = -1
    else:
        pr = problems.thermal_pulse(96)
        skip = -1         # viscosity drives rho*w: pass it
    lib = fv.load_library()
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    shape = sim.shape
    pitch = shape[2] + 24  # padded rows
    arrs, ptrs = _device_state(torch, sim.get_cons(), pitch, skip)
    params = pr.params.copy()
    err = C.create_string_buffer(512)
    next_dt = C.c_double()
    dt = sim.compute_dt()
    for call in range(2):
        sim.step(dt)
        torch.cuda.synchronize()
        rc = lib.fvgpu_step_noalloc(C.byref(params), ptrs, pitch, dt, C.byref(next_dt), None, err, 512)
        assert rc == 0, (rc, err.value)
        got = _to_host(arrs, shape)
        want = sim.get_cons()
        errs = rel_l1_fields(got, [w if k != skip else np.zeros(shape) for k, w in enumerate(want)])
        assert max(errs) <= REL_L1_STEP, (call, errs)
        for k in range(5):
            if k != skip:
                np.testing.assert_array_equal(got[k], want[k])
        dt_handle = sim.compute_dt()
        assert next_dt.value == dt_handle, (call, next_dt.value, dt_handle)
        dt = dt_handle
    # the padding columns were never written
    for t in arrs:
        if t is not None:
            assert torch.isnan(t[:, shape[2]:]).all()


def test_noalloc_rejects_problems_beyond_its_scratch():
    """A 2048^2 run needs 160 MiB of stage scratch, more than the fixed 32 MiB:
    the call refuses with a message before touching the GPU."""
    lib = fv.load_library()
    params = fv.parse_ini("[mesh]\nNx=2048\nNy=2048\nNz=1\n[run]\nboundaries_z=periodic\n"
                          "[solvers]\ntime_stepping=RK2\nreconstruction=plm\n")
    ptrs = (C.c_void_p * 5)(1, 1, 1, None, 1)  # never dereferenced: rejected first
    err = C.create_string_buffer(512)
    rc = lib.fvgpu_step_noalloc(C.byref(params), ptrs, 2048, 1e-3, None, None, err, 512)
    assert rc == 1
    assert b"scratch" in err.value and b"fvgpu_create" in err.value


def test_noalloc_refuses_bad_dt_and_huge_pitch():
    """dt must be positive and finite (no CFL fallback here), and a pitch
    whose product with the row count would overflow is refused before any
    size arithmetic."""
    lib = fv.load_library()
    params = fv.parse_ini("[mesh]\nNx=64\nNy=64\nNz=1\n[run]\nboundaries_z=periodic\n"
                          "[solvers]\ntime_stepping=RK2\nreconstruction=plm\n")
    ptrs = (C.c_void_p * 5)(1, 1, 1, None, 1)  # never dereferenced: rejected first
    err = C.create_string_buffer(512)
    for dt in (0.0, -1e-3, float("nan"), float("inf")):
        assert lib.fvgpu_step_noalloc(C.byref(params), ptrs, 64, dt, None, None, err, 512) == 1
        assert b"dt" in err.value
    for pitch in (1 << 40, (1 << 31) + 5, 200000):
        assert lib.fvgpu_step_noalloc(C.byref(params), ptrs, pitch, 1e-3, None, None, err, 512) == 1
        assert b"pitch" in err.value


def test_noalloc_error_flag_is_sticky_until_read():
    """A non-finite state met by a call without next_dt is reported by the
    next call that passes next_dt, which clears the flag: a clean call after
    it reports FV_OK and matches the handle bit for bit."""
    torch = pytest.importorskip("torch")
    lib = fv.load_library()
    pr = problems.sedov(48)
    sim = fv.Simulation(pr.params)
    sim.set_prim(*pr.prim)
    dt = sim.compute_dt()
    good = sim.get_cons()
    shape = sim.shape
    params = pr.params.copy()
    err = C.create_string_buffer(512)
    next_dt = C.c_double()
    bad = [a.copy() for a in good]
    bad[4][0, 5, 7] = -1.0  # negative energy, so negative pressure: NaN sound speed
    arrs1, ptrs1 = _device_state(torch, bad, shape[2], 3)
    rc = lib.fvgpu_step_noalloc(C.byref(params), ptrs1, shape[2], dt, None, None, err, 512)
    assert rc == 0, err.value           # asynchronous: nothing checked yet
    torch.cuda.synchronize()
    arrs2, ptrs2 = _device_state(torch, good, shape[2], 3)
    rc = lib.fvgpu_step_noalloc(C.byref(params), ptrs2, shape[2], dt, C.byref(next_dt), None, err, 512)
    assert rc == 4, (rc, err.value)     # the earlier call's non-finite state
    arrs3, ptrs3 = _device_state(torch, good, shape[2], 3)
    rc = lib.fvgpu_step_noalloc(C.byref(params), ptrs3, shape[2], dt, C.byref(next_dt), None, err, 512)
    assert rc == 0, (rc, err.value)     # cleared once reported
    sim.step(dt)
    want = sim.get_cons()
    got = _to_host(arrs3, shape)
    for k in (0, 1, 2, 4):
        np.testing.assert_array_equal(got[k], want[k])
    sim.close()
