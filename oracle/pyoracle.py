"""Python access to the oracle libraries -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, always for results to compare with.  Two back ends share one interface:

* :class:`Oracle` -- the C restatement (oracle/fv3d_oracle.c), fed an
  ``FvParams``; available everywhere.
* :class:`RefOracle` -- the reference's own headers compiled against the
  shim (oracle/ref_harness.cpp), fed an .ini file the reference's own
  ``readInifile`` parses; available only where the reference tree is.

Field arrays are numpy float64 of shape (Nz, Ny, Nx) (interior cells).
"""
import ctypes as C
import os

import numpy as np

from fv3d_gb300._abi import FvParams
from oracle import build as _build

_dp = C.POINTER(C.c_double)
_lib_oracle = None
_lib_ref = None


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def load_oracle():
    global _lib_oracle
    if _lib_oracle is None:
        path = _build.build_oracle()
        lib = C.CDLL(path)
        lib.fvora_create.restype = C.c_void_p
        lib.fvora_create.argtypes = [C.POINTER(FvParams)]
        lib.fvora_destroy.argtypes = [C.c_void_p]
        for n in ("fvora_set_prim", "fvora_set_cons", "fvora_get_prim", "fvora_get_cons", "fvora_generate"):
            getattr(lib, n).argtypes = [C.c_void_p] + [_dp] * 5
            getattr(lib, n).restype = C.c_int
        lib.fvora_compute_dt.restype = C.c_double
        lib.fvora_compute_dt.argtypes = [C.c_void_p, _dp]
        lib.fvora_step.argtypes = [C.c_void_p, C.c_double]
        lib.fvora_advance.argtypes = [C.c_void_p, C.c_double, C.c_long, _dp, C.POINTER(C.c_long)]
        lib.fvora_riemann.argtypes = [C.c_int, C.c_double, C.c_long, _dp, _dp, _dp, _dp]
        lib.fvora_set_threads.argtypes = [C.c_int]
        lib.fvora_set_threads.restype = C.c_int
        lib.fvora_parse_ini.argtypes = [C.c_char_p, C.POINTER(FvParams)]
        lib.fvora_parse_ini.restype = C.c_int
        _lib_oracle = lib
    return _lib_oracle


def reference_available():
    return _build.reference_available() or os.path.exists(_build.REF_SO)


def load_ref():
    global _lib_ref
    if _lib_ref is None:
        path = _build.build_ref()
        if path is None:
            if not os.path.exists(_build.REF_SO):
                raise RuntimeError("reference sources absent; oracle/_ref not built")
            path = _build.REF_SO
        lib = C.CDLL(path)
        lib.fvref_read_ini.argtypes = [C.c_char_p, C.POINTER(FvParams)]
        lib.fvref_create.restype = C.c_void_p
        lib.fvref_create.argtypes = [C.c_char_p]
        lib.fvref_create_b02.restype = C.c_void_p
        lib.fvref_create_b02.argtypes = [C.c_char_p] + [C.c_double] * 4
        lib.fvref_destroy.argtypes = [C.c_void_p]
        for n in ("fvref_set_prim", "fvref_get_prim", "fvref_get_cons", "fvref_generate"):
            getattr(lib, n).argtypes = [C.c_void_p] + [_dp] * 5
        lib.fvref_compute_dt.restype = C.c_double
        lib.fvref_compute_dt.argtypes = [C.c_void_p]
        lib.fvref_step.argtypes = [C.c_void_p, C.c_double]
        lib.fvref_advance.argtypes = [C.c_void_p, C.c_double, C.c_long, _dp, C.POINTER(C.c_long)]
        lib.fvref_riemann.argtypes = [C.c_int, C.c_double, C.c_long, _dp, _dp, _dp, _dp]
        _lib_ref = lib
    return _lib_ref


def set_threads(n):
    return load_oracle().fvora_set_threads(int(n))


def _shape(p):
    return (p.Nz, p.Ny, p.Nx)


def _fields_in(shape, fields):
    out = []
    for f in fields:
        if f is None:
            out.append(None)
        else:
            a = np.ascontiguousarray(np.broadcast_to(np.asarray(f, dtype=np.float64), shape))
            out.append(a)
    return out


class _Base:
    params: FvParams

    def _get(self, fn):
        shape = _shape(self.params)
        arrs = [np.empty(shape, np.float64) for _ in range(5)]
        fn(self._h, *[_ptr(a) for a in arrs])
        return arrs


class Oracle(_Base):
    """The C restatement of the reference step."""

    def __init__(self, params):
        self.lib = load_oracle()
        self.params = params.copy()
        self._h = self.lib.fvora_create(C.byref(self.params))
        if not self._h:
            raise ValueError("oracle rejected the parameters")

    def close(self):
        if self._h:
            self.lib.fvora_destroy(self._h)
            self._h = None

    __del__ = close

    def set_prim(self, rho, u, v, w, p):
        arrs = _fields_in(_shape(self.params), (rho, u, v, w, p))
        self.lib.fvora_set_prim(self._h, *[_ptr(a) for a in arrs])

    def set_cons(self, rho, mx, my, mz, E):
        arrs = _fields_in(_shape(self.params), (rho, mx, my, mz, E))
        self.lib.fvora_set_cons(self._h, *[_ptr(a) for a in arrs])

    def get_prim(self):
        return self._get(self.lib.fvora_get_prim)

    def generate(self):
        """The generator named by params.problem (Init.h:18-209): sets the
        state and returns the generated primitives (rho, u, v, w, p)."""
        shape = _shape(self.params)
        arrs = [np.empty(shape, np.float64) for _ in range(5)]
        if self.lib.fvora_generate(self._h, *[_ptr(a) for a in arrs]) != 0:
            raise ValueError("unknown problem %r" % self.params.problem)
        return arrs

    def get_cons(self):
        return self._get(self.lib.fvora_get_cons)

    def compute_dt(self, with_inv=False):
        inv = (C.c_double * 3)()
        dt = self.lib.fvora_compute_dt(self._h, C.cast(inv, _dp))
        return (dt, list(inv)) if with_inv else dt

    def step(self, dt):
        self.lib.fvora_step(self._h, float(dt))

    def advance(self, tend, max_steps=0, t=0.0):
        tt = C.c_double(t)
        n = C.c_long(0)
        self.lib.fvora_advance(self._h, float(tend), int(max_steps), C.byref(tt), C.byref(n))
        return tt.value, n.value


class RefOracle(_Base):
    """The reference's own headers, compiled against the shim."""

    def __init__(self, ini_path, b02=None):
        """b02 = (zmid, kappa1, kappa2, thickness) sets the B02 profile,
        which the reference's readInifile leaves unset."""
        self.lib = load_ref()
        self.params = ref_read_ini(ini_path)
        if b02 is None:
            self._h = self.lib.fvref_create(ini_path.encode())
        else:
            self._h = self.lib.fvref_create_b02(ini_path.encode(), *[float(x) for x in b02])
            (self.params.b02_zmid, self.params.b02_kappa1, self.params.b02_kappa2,
             self.params.b02_thickness) = [float(x) for x in b02]

    def close(self):
        if self._h:
            self.lib.fvref_destroy(self._h)
            self._h = None

    __del__ = close

    def set_prim(self, rho, u, v, w, p):
        arrs = _fields_in(_shape(self.params), (rho, u, v, w, p))
        self.lib.fvref_set_prim(self._h, *[_ptr(a) for a in arrs])

    def get_prim(self):
        return self._get(self.lib.fvref_get_prim)

    def generate(self):
        """The reference's InitFunctor::init (its random pool replaced by
        the shim's: H84 / C91 perturbations are not the reference's)."""
        return self._get(self.lib.fvref_generate)

    def get_cons(self):
        return self._get(self.lib.fvref_get_cons)

    def compute_dt(self):
        return self.lib.fvref_compute_dt(self._h)

    def step(self, dt):
        self.lib.fvref_step(self._h, float(dt))

    def advance(self, tend, max_steps=0, t=0.0):
        tt = C.c_double(t)
        n = C.c_long(0)
        self.lib.fvref_advance(self._h, float(tend), int(max_steps), C.byref(tt), C.byref(n))
        return tt.value, n.value


def parse_ini(text):
    """readInifile (SimInfo.h:169-306) on .ini text, by the oracle's own
    restatement (fv3d_ini.c): Params without the GPU library."""
    p = FvParams()
    rc = load_oracle().fvora_parse_ini(text.encode(), C.byref(p))
    if rc:
        raise ValueError("fvora_parse_ini failed: %d" % rc)
    return p


def ref_read_ini(path):
    p = FvParams()
    load_ref().fvref_read_ini(path.encode(), C.byref(p))
    return p


def riemann(solver, gamma0, qL, qR, use_ref=False):
    """Flux and pout of hll (solver 0) / hllc (solver 1) for (n,5) state pairs."""
    qL = np.ascontiguousarray(qL, np.float64)
    qR = np.ascontiguousarray(qR, np.float64)
    n = qL.shape[0]
    flux = np.empty((n, 5), np.float64)
    pout = np.empty(n, np.float64)
    lib = load_ref() if use_ref else load_oracle()
    fn = lib.fvref_riemann if use_ref else lib.fvora_riemann
    fn(int(solver), float(gamma0), n, _ptr(qL), _ptr(qR), _ptr(flux), _ptr(pout))
    return flux, pout
