"""fv3d_gb300 -- GB300-native (sm_103a) finite-volume hydro step of fv3d.

Python access to the C ABI declared in include/fv3d_gb300.h, for tests,
benchmarks and scripting.  The compute path is the in-tree CUDA library
``fv3d_gb300/_lib/libfv3d_gb300.so``; there is no CPU fallback: importing the
bindings without the built library raises.

The classes mirror the reference's hot-path interface (fv3d::readInifile,
ComputeDtFunctor::computeDt, UpdateFunctor::update and the main.cpp loop) on
device-resident state:

    params = read_ini("run.ini")
    sim = Simulation(params)
    sim.set_prim(rho, u, v, w, p)          # arrays of shape (Nz, Ny, Nx)
    dt = sim.compute_dt()
    sim.step(dt)                           # one UpdateFunctor::update
    t, n = sim.advance(tend)               # the main.cpp:51-74 loop
    rho, u, v, w, p = sim.get_prim()
"""
import ctypes as C
import os

import numpy as np

from ._abi import FvParams, STATUS_NAMES  # noqa: F401
from . import _abi  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))
_dp = C.POINTER(C.c_double)
_lib = None
_lib_variant = None


class FvError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status, message):
        self.status = status
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))


def library_path(variant=None):
    from . import build as _b
    return _b.lib_path(variant or os.environ.get("FV3D_LIB_VARIANT", "default"))


def load_library(variant=None, build_if_missing=True):
    """Load (building first if needed) the in-tree CUDA library."""
    global _lib, _lib_variant
    variant = variant or os.environ.get("FV3D_LIB_VARIANT", "default")
    if _lib is not None and _lib_variant == variant:
        return _lib
    path = library_path(variant)
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("fv3d_gb300 CUDA library not built: %s" % path)
        from . import build as _b
        _b.build(variant)
    lib = C.CDLL(path)
    _declare(lib)
    _lib, _lib_variant = lib, variant
    return lib


def _declare(lib):
    P = C.POINTER(FvParams)
    vp = C.c_void_p
    sig = {
        "fv_status_string": (C.c_char_p, [C.c_int]),
        "fv_read_ini": (C.c_int, [C.c_char_p, P]),
        "fv_parse_ini": (C.c_int, [C.c_char_p, P]),
        "fvgpu_create": (C.c_int, [P, C.POINTER(vp)]),
        "fvgpu_destroy": (C.c_int, [vp]),
        "fvgpu_last_error": (C.c_char_p, [vp]),
        "fvgpu_set_prim": (C.c_int, [vp] + [_dp] * 5),
        "fvgpu_get_prim": (C.c_int, [vp] + [_dp] * 5),
        "fvgpu_set_cons": (C.c_int, [vp] + [_dp] * 5),
        "fvgpu_get_cons": (C.c_int, [vp] + [_dp] * 5),
        "fvgpu_init_problem": (C.c_int, [vp]),
        "fvgpu_generate": (C.c_int, [P] + [_dp] * 5),
        "fv_h5_save": (C.c_int, [P, C.c_char_p, C.c_int, C.c_double] + [_dp] * 5),
        "fvgpu_compute_dt": (C.c_int, [vp, _dp, _dp]),
        "fvgpu_step": (C.c_int, [vp, C.c_double]),
        "fvgpu_advance": (C.c_int, [vp, C.c_double, C.c_long, _dp, C.POINTER(C.c_long)]),
        "fvgpu_enqueue_steps": (C.c_int, [vp, C.c_long]),
        "fvgpu_step_noalloc": (C.c_int, [P, C.POINTER(C.c_void_p), C.c_long, C.c_double, _dp, vp,
                                         C.c_char_p, C.c_size_t]),
        "fvgpu_conserved_totals": (C.c_int, [vp, _dp]),
        "fvgpu_set_stream": (C.c_int, [vp, vp]),
        "fvgpu_synchronize": (C.c_int, [vp]),
        "fvgpu_launch_count": (C.c_int, [vp, C.POINTER(C.c_long)]),
        "fvgpu_profile_enable": (C.c_int, [vp, C.c_int]),
        "fvgpu_kernel_times": (C.c_int, [vp, C.POINTER(C.c_long), _dp]),
        "fvgpu_batch_create": (C.c_int, [P, C.c_int, C.POINTER(vp)]),
        "fvgpu_batch_destroy": (C.c_int, [vp]),
        "fvgpu_batch_last_error": (C.c_char_p, [vp]),
        "fvgpu_batch_set_prim": (C.c_int, [vp, C.c_int] + [_dp] * 5),
        "fvgpu_batch_get_prim": (C.c_int, [vp, C.c_int] + [_dp] * 5),
        "fvgpu_batch_init_problem": (C.c_int, [vp, C.c_int]),
        "fvgpu_batch_run": (C.c_int, [vp, C.c_long]),
        "fvgpu_batch_times": (C.c_int, [vp, _dp]),
        "fvgpu_batch_set_stream": (C.c_int, [vp, vp]),
        "fvgpu_batch_synchronize": (C.c_int, [vp]),
        "fvgpu_batch_launch_count": (C.c_int, [vp, C.POINTER(C.c_long)]),
        "fvgpu_probe_fp64_rate": (C.c_int, [_dp]),
        "fvgpu_probe_wait": (C.c_int, [C.c_int, C.c_int]),
        "fvgpu_probe_grid_wait": (C.c_int, [C.c_int, C.c_int]),
        "fvgpu_step_host": (C.c_int, [vp, C.POINTER(_dp), C.c_double, C.POINTER(_dp), _dp]),
        "fvgpu_batch_tiling": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]),
        "fvgpu_batch_schedule": (C.c_int, [vp, C.POINTER(C.c_int)] + [C.POINTER(C.c_int)] * 4 + [C.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def probe_fp64_rate():
    """Measured FP64 FMA lane operations per second of the current GPU."""
    r = C.c_double(0.0)
    rc = load_library().fvgpu_probe_fp64_rate(C.byref(r))
    if rc:
        raise FvError(rc, "fvgpu_probe_fp64_rate")
    return r.value


def probe_wait(arrive, max_polls):
    """Status of the bounded mbarrier wait run on its own (fvgpu_probe_wait):
    0 when it completed, FV_ERR_TIMEOUT when it gave up."""
    return load_library().fvgpu_probe_wait(1 if arrive else 0, int(max_polls))


def probe_grid_wait(arrive_all, max_polls):
    """Status of the multi-step kernel's bounded grid-barrier wait run on its
    own (fvgpu_probe_grid_wait): 0 when it completed, FV_ERR_TIMEOUT when it
    gave up because a CTA never arrived."""
    return load_library().fvgpu_probe_grid_wait(1 if arrive_all else 0, int(max_polls))


def generate(params):
    """The reference's generator for params.problem (Init.h:18-209) run on the
    GPU (fvgpu_generate): the primitives (rho, u, v, w, p), each [Nz][Ny][Nx]."""
    shape = (params.Nz, params.Ny, params.Nx)
    arrs = [np.empty(shape, np.float64) for _ in range(5)]
    rc = load_library().fvgpu_generate(C.byref(params), *[_ptr(a) for a in arrs])
    if rc:
        raise FvError(rc, "fvgpu_generate(%r)" % params.problem)
    return arrs


def save_solution(params, path, iteration, t, prim):
    """IOManager::saveSolution (IOManager.h:88-192) through fv_h5_save: the
    primitives (rho, u, v, w, p; each [Nz][Ny][Nx]) as group ite_<iteration>
    of the HDF5 file `path` (iteration 0 creates it)."""
    shape = (params.Nz, params.Ny, params.Nx)
    arrs = [_as_field(a, shape) for a in prim]
    rc = load_library().fv_h5_save(C.byref(params), os.fspath(path).encode(), int(iteration), float(t),
                                   *[_ptr(a) for a in arrs])
    if rc:
        raise FvError(rc, "fv_h5_save(%s)" % os.fspath(path))


def parse_ini(text):
    """readInifile semantics on INI text (SimInfo.h:169-306)."""
    p = FvParams()
    rc = load_library().fv_parse_ini(text.encode(), C.byref(p))
    if rc:
        raise FvError(rc, "fv_parse_ini")
    return p


def read_ini(path):
    """readInifile semantics on an .ini file (SimInfo.h:169-306)."""
    p = FvParams()
    rc = load_library().fv_read_ini(os.fspath(path).encode(), C.byref(p))
    if rc:
        raise FvError(rc, "fv_read_ini")
    return p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _checked(a, shape):
    """An array passed by address: must already be float64, C-contiguous and
    of the grid's shape (no copy is made, so results land in the caller's
    memory)."""
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous and a.shape == shape):
        raise ValueError("expected a C-contiguous float64 array of shape %s" % (shape,))
    return a


def _as_field(a, shape):
    if a is None:
        return None
    return np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), shape))


class Simulation:
    """One problem on the GPU (fvgpu_* handle)."""

    def __init__(self, params):
        self.lib = load_library()
        self.params = params.copy()
        h = C.c_void_p()
        rc = self.lib.fvgpu_create(C.byref(self.params), C.byref(h))
        self._h = h
        if rc:
            msg = self.last_error()
            self.close()
            raise FvError(rc, msg)

    @property
    def shape(self):
        return (self.params.Nz, self.params.Ny, self.params.Nx)

    @property
    def handle(self):
        return self._h

    def last_error(self):
        return (self.lib.fvgpu_last_error(self._h) or b"").decode()

    def _check(self, rc, what):
        if rc:
            raise FvError(rc, "%s: %s" % (what, self.last_error()))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.fvgpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_prim(self, rho, u=None, v=None, w=None, p=None):
        arrs = [_as_field(a, self.shape) for a in (rho, u, v, w, p)]
        self._check(self.lib.fvgpu_set_prim(self._h, *[_ptr(a) for a in arrs]), "set_prim")

    def init_problem(self):
        """InitFunctor::init + primToCons on the GPU (fvgpu_init_problem): the
        generator named by params.problem sets the state."""
        self._check(self.lib.fvgpu_init_problem(self._h), "init_problem")

    def set_cons(self, rho, mx=None, my=None, mz=None, E=None):
        arrs = [_as_field(a, self.shape) for a in (rho, mx, my, mz, E)]
        self._check(self.lib.fvgpu_set_cons(self._h, *[_ptr(a) for a in arrs]), "set_cons")

    def get_prim(self, out=None):
        arrs = out if out is not None else [np.empty(self.shape, np.float64) for _ in range(5)]
        self._check(self.lib.fvgpu_get_prim(self._h, *[_ptr(a) for a in arrs]), "get_prim")
        return arrs

    def get_cons(self, out=None):
        arrs = out if out is not None else [np.empty(self.shape, np.float64) for _ in range(5)]
        self._check(self.lib.fvgpu_get_cons(self._h, *[_ptr(a) for a in arrs]), "get_cons")
        return arrs

    def compute_dt(self, with_inv=False):
        dt = C.c_double()
        inv = (C.c_double * 3)()
        self._check(self.lib.fvgpu_compute_dt(self._h, C.byref(dt), C.cast(inv, _dp)), "compute_dt")
        return (dt.value, list(inv)) if with_inv else dt.value

    def step(self, dt):
        self._check(self.lib.fvgpu_step(self._h, float(dt)), "step")

    def advance(self, tend, max_steps=0, t=0.0):
        tt = C.c_double(t)
        n = C.c_long(0)
        self._check(self.lib.fvgpu_advance(self._h, float(tend), int(max_steps), C.byref(tt), C.byref(n)),
                    "advance")
        return tt.value, n.value

    def step_host(self, prim_in, dt=0.0, out=None):
        """One step from and to primitive arrays the GPU reads and writes
        directly (fvgpu_step_host); dt <= 0 takes the CFL dt.  Arrays must be
        C-contiguous float64 of the grid's shape (pinned host memory for full
        speed).  Returns (out, dt_used)."""
        ins = (_dp * 5)(*[None if a is None else _ptr(_checked(a, self.shape)) for a in prim_in])
        if out is None:
            out = [np.empty(self.shape, np.float64) for _ in range(5)]
        outs = (_dp * 5)(*[None if a is None else _ptr(_checked(a, self.shape)) for a in out])
        used = C.c_double(0.0)
        self._check(self.lib.fvgpu_step_host(self._h, ins, float(dt), outs, C.byref(used)), "step_host")
        return out, used.value

    def enqueue_steps(self, nsteps):
        """Queue nsteps CFL steps on the GPU and return without waiting."""
        self._check(self.lib.fvgpu_enqueue_steps(self._h, int(nsteps)), "enqueue_steps")

    def conserved_totals(self):
        out = (C.c_double * 5)()
        self._check(self.lib.fvgpu_conserved_totals(self._h, C.cast(out, _dp)), "conserved_totals")
        return list(out)

    def set_stream(self, stream_ptr):
        self._check(self.lib.fvgpu_set_stream(self._h, C.c_void_p(stream_ptr)), "set_stream")

    def synchronize(self):
        self._check(self.lib.fvgpu_synchronize(self._h), "synchronize")

    def launch_count(self):
        c = C.c_long()
        self._check(self.lib.fvgpu_launch_count(self._h, C.byref(c)), "launch_count")
        return c.value

    def profile(self, enable=True):
        self._check(self.lib.fvgpu_profile_enable(self._h, int(bool(enable))), "profile_enable")

    def kernel_times(self):
        counts = (C.c_long * 3)()
        ms = (C.c_double * 3)()
        self._check(self.lib.fvgpu_kernel_times(self._h, counts, C.cast(ms, _dp)), "kernel_times")
        names = ("stage", "dt", "conversion")
        return {n: (counts[i], ms[i]) for i, n in enumerate(names)}


class Batch:
    """Many independent problems advanced together (fvgpu_batch_* handle).

    Every problem keeps its own grid, parameters and dt; problems sharing the
    plane and layout are advanced by one persistent kernel launch per stage.
    All problems must share the precision (FV_PREC_FP64 or
    FV_PREC_FP32_MIXED) and the time-stepping scheme.
    """

    def __init__(self, params_list):
        self.lib = load_library()
        self.params = [p.copy() for p in params_list]
        arr = (FvParams * len(self.params))(*self.params)
        h = C.c_void_p()
        rc = self.lib.fvgpu_batch_create(arr, len(self.params), C.byref(h))
        self._h = h
        if rc:
            msg = self.last_error()
            self.close()
            raise FvError(rc, msg)

    def __len__(self):
        return len(self.params)

    def shape(self, i):
        p = self.params[i]
        return (p.Nz, p.Ny, p.Nx)

    def last_error(self):
        return (self.lib.fvgpu_batch_last_error(self._h) or b"").decode()

    def _check(self, rc, what):
        if rc:
            raise FvError(rc, "%s: %s" % (what, self.last_error()))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.fvgpu_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_prim(self, i, rho, u=None, v=None, w=None, p=None):
        arrs = [_as_field(a, self.shape(i)) for a in (rho, u, v, w, p)]
        self._check(self.lib.fvgpu_batch_set_prim(self._h, int(i), *[_ptr(a) for a in arrs]), "batch_set_prim")

    def init_problem(self, i):
        """The generator of problem i's params.problem on the GPU."""
        self._check(self.lib.fvgpu_batch_init_problem(self._h, int(i)), "batch_init_problem")

    def get_prim(self, i):
        arrs = [np.empty(self.shape(i), np.float64) for _ in range(5)]
        self._check(self.lib.fvgpu_batch_get_prim(self._h, int(i), *[_ptr(a) for a in arrs]), "batch_get_prim")
        return arrs

    def run(self, nsteps):
        self._check(self.lib.fvgpu_batch_run(self._h, int(nsteps)), "batch_run")

    def times(self):
        t = np.empty(len(self), np.float64)
        self._check(self.lib.fvgpu_batch_times(self._h, _ptr(t)), "batch_times")
        return t

    def set_stream(self, stream_ptr):
        self._check(self.lib.fvgpu_batch_set_stream(self._h, C.c_void_p(stream_ptr)), "batch_set_stream")

    def synchronize(self):
        self._check(self.lib.fvgpu_batch_synchronize(self._h), "batch_synchronize")

    def launch_count(self):
        c = C.c_long()
        self._check(self.lib.fvgpu_batch_launch_count(self._h, C.byref(c)), "batch_launch_count")
        return c.value

    def schedule(self):
        """[{tx, rows, block_rows, split_viscous}] the autotuner chose per group."""
        ng = C.c_int()
        arrs = [(C.c_int * 8)() for _ in range(4)]
        self._check(self.lib.fvgpu_batch_schedule(self._h, C.byref(ng), *arrs, 8), "batch_schedule")
        keys = ("tx", "rows", "block_rows", "split_viscous")
        return [{k: a[g] for k, a in zip(keys, arrs)} for g in range(ng.value)]

    def tiling(self):
        """[(tx, ty)] tile shape chosen per group."""
        ng = C.c_int()
        tx = (C.c_int * 8)()
        ty = (C.c_int * 8)()
        self._check(self.lib.fvgpu_batch_tiling(self._h, C.byref(ng), tx, ty, 8), "batch_tiling")
        return [(tx[g], ty[g]) for g in range(ng.value)]
