"""ctypes mirror of include/fv3d_gb300.h (types and enums only).

The field order of :class:`FvParams` must match ``struct fv_params`` exactly;
``tests/test_abi.py`` checks the size against the C compiler's.
"""
import ctypes as C

FV_BC_ABSORBING, FV_BC_REFLECTING, FV_BC_PERIODIC, FV_BC_C91 = 0, 1, 2, 3
FV_HLL, FV_HLLC = 0, 1
FV_TS_EULER, FV_TS_RK2 = 0, 1
FV_PCM, FV_PCM_WB, FV_PLM = 0, 1, 2
FV_TCM_CONSTANT, FV_TCM_B02 = 0, 1
FV_BCTC_NONE, FV_BCTC_FIXED_TEMPERATURE, FV_BCTC_FIXED_GRADIENT = 0, 1, 2
FV_VSC_CONSTANT = 0
FV_PREC_FP64, FV_PREC_FP32_MIXED = 0, 1
FV_PHYS_REFERENCE, FV_PHYS_CORRECTED = 0, 1

FV_OK, FV_ERR_PARAM, FV_ERR_UNSUPPORTED, FV_ERR_CUDA, FV_ERR_NONFINITE = 0, 1, 2, 3, 4
FV_ERR_NOMEM, FV_ERR_IO, FV_ERR_TIMEOUT, FV_ERR_STATE = 5, 6, 7, 8

STATUS_NAMES = {
    0: "FV_OK",
    1: "FV_ERR_PARAM",
    2: "FV_ERR_UNSUPPORTED",
    3: "FV_ERR_CUDA",
    4: "FV_ERR_NONFINITE",
    5: "FV_ERR_NOMEM",
    6: "FV_ERR_IO",
    7: "FV_ERR_TIMEOUT",
    8: "FV_ERR_STATE",
}


class FvParams(C.Structure):
    """``struct fv_params`` (mirror of fv3d::Params, SimInfo.h:72-159)."""

    _fields_ = [
        ("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("Ng", C.c_int),
        ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
        ("ymax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("save_freq", C.c_double), ("tend", C.c_double),
        ("boundary_x", C.c_int), ("boundary_y", C.c_int), ("boundary_z", C.c_int),
        ("reconstruction", C.c_int), ("riemann_solver", C.c_int), ("time_stepping", C.c_int),
        ("CFL", C.c_double),
        ("epsilon", C.c_double), ("gamma0", C.c_double),
        ("gravity", C.c_int), ("well_balanced_flux_at_z_bc", C.c_int),
        ("g", C.c_double),
        ("well_balanced", C.c_int), ("thermal_conductivity_active", C.c_int),
        ("thermal_conductivity_mode", C.c_int), ("bctc_zmin", C.c_int),
        ("kappa", C.c_double),
        ("bctc_zmax", C.c_int), ("viscosity_active", C.c_int),
        ("bctc_zmin_value", C.c_double), ("bctc_zmax_value", C.c_double),
        ("viscosity_mode", C.c_int), ("seed", C.c_int),
        ("mu", C.c_double),
        ("m1", C.c_double), ("theta1", C.c_double), ("m2", C.c_double), ("theta2", C.c_double),
        ("h84_pert", C.c_double), ("c91_pert", C.c_double),
        ("b02_zmid", C.c_double), ("b02_kappa1", C.c_double), ("b02_kappa2", C.c_double),
        ("b02_thickness", C.c_double),
        ("log_frequency", C.c_int), ("precision", C.c_int),
        ("problem", C.c_char * 64),
        ("filename_out", C.c_char * 256),
        ("physics", C.c_int),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = v.decode() if isinstance(v, bytes) else v
        return out

    def copy(self):
        c = FvParams()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(FvParams))
        return c
