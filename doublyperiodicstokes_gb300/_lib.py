"""ctypes binding of libdpstokes_gb300.so (include/dpstokes_gb300.h).

The library is the only implementation: if it is missing this module raises
instead of falling back to anything else.  Build it with
`python -m doublyperiodicstokes_gb300.build` (or __graft_entry__.build())."""
import ctypes
import os

from . import build as _build

DPST_OK = 0
ERRORS = {1: "invalid argument", 2: "not ready", 3: "out of domain", 4: "CUDA error",
          5: "unsupported", 6: "allocation failed"}
MODE = {"nowall": 0, "bottom": 1, "slit": 2, "periodic": 3}
PREC = {"fp64": 0, "mixed": 1}
SOLVE = {"default": 0, "fp64": 1, "df64": 2}
F64, F32 = 0, 1


class DpstParams(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("nz", ctypes.c_int), ("Lx", ctypes.c_double), ("Ly", ctypes.c_double),
                ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
                ("viscosity", ctypes.c_double), ("w", ctypes.c_int), ("beta", ctypes.c_double),
                ("alpha", ctypes.c_double), ("has_torque", ctypes.c_int), ("w_d", ctypes.c_int),
                ("beta_d", ctypes.c_double), ("alpha_d", ctypes.c_double),
                ("precision", ctypes.c_int), ("torque_kernel", ctypes.c_int),
                ("solve_arith", ctypes.c_int)]


class DpstInfo(ctypes.Structure):
    _fields_ = [("nxh", ctypes.c_int), ("n_modes", ctypes.c_int), ("nzeff_m", ctypes.c_int),
                ("nzeff_d", ctypes.c_int), ("ghost_m", ctypes.c_int), ("ghost_d", ctypes.c_int),
                ("wz_max_m", ctypes.c_int), ("wz_max_d", ctypes.c_int),
                ("thr_m", ctypes.c_double), ("thr_d", ctypes.c_double),
                ("norm_m", ctypes.c_double), ("norm_d", ctypes.c_double),
                ("device_bytes", ctypes.c_int64), ("n_particles", ctypes.c_int64),
                ("kernels_per_mdot", ctypes.c_int), ("ghost_layers_in_use", ctypes.c_int),
                ("ztransform", ctypes.c_int), ("ztransform_ms", ctypes.c_float * 2),
                ("fused_particle_passes", ctypes.c_int), ("ztransform_inverse", ctypes.c_int),
                ("ztransform_inverse_ms", ctypes.c_float * 2), ("z_fused", ctypes.c_int),
                ("solve_arith", ctypes.c_int), ("solve_variant", ctypes.c_int),
                ("solve_ms", ctypes.c_float * 4), ("xy_transform", ctypes.c_int),
                ("xy_ms", ctypes.c_float * 2), ("spread_tiles", ctypes.c_int),
                ("ztransform_tma_ms", ctypes.c_float * 2), ("ztransform_tma_variant", ctypes.c_int * 2),
                ("ztransform_tma_variant_ms", ctypes.c_float * 6), ("xy_cluster_ms", ctypes.c_float)]


class DpstBatchInfo(ctypes.Structure):
    _fields_ = [("n_systems", ctypes.c_int), ("n_size_classes", ctypes.c_int),
                ("n_particles", ctypes.c_int64), ("n_modes", ctypes.c_int64),
                ("kernels_per_mdot", ctypes.c_int), ("fft_plans", ctypes.c_int),
                ("device_bytes", ctypes.c_int64), ("ztransform", ctypes.c_int),
                ("ztransform_inverse", ctypes.c_int), ("ztransform_ms", ctypes.c_float * 2),
                ("ztransform_inverse_ms", ctypes.c_float * 2), ("ztransform_tma_ms", ctypes.c_float * 2)]


# every entry point of include/dpstokes_gb300.h with its signature
SIGNATURES = {
    "dpst_create": (ctypes.c_int, [ctypes.POINTER(DpstParams), ctypes.c_int64, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_void_p)]),
    "dpst_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dpst_set_positions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p]),
    "dpst_mdot": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "dpst_mdot_multi": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "dpst_set_positions_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                               ctypes.c_void_p]),
    "dpst_mdot_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_void_p]),
    "dpst_spread_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "dpst_velocity_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dpst_mdot_timed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "dpst_mdot_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p]),
    "dpst_mdot_backward": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_void_p] * 7
                           + [ctypes.c_int, ctypes.c_void_p]),
    "dpst_forward_serial": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "dpst_mdot_backward_saved": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64] + [ctypes.c_void_p] * 7
                                 + [ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "dpst_batched_create": (ctypes.c_int, [ctypes.POINTER(DpstParams), ctypes.POINTER(ctypes.c_int64),
                                           ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "dpst_batched_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dpst_batched_set_positions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                  ctypes.c_void_p]),
    "dpst_batched_mdot": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_void_p] * 4
                          + [ctypes.c_int, ctypes.c_void_p]),
    "dpst_batched_get_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DpstBatchInfo)]),
    "dpst_get_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DpstInfo)]),
    "dpst_xy_transform": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p]),
    "dpst_last_error": (ctypes.c_char_p, []),
    "dpst_version": (ctypes.c_char_p, []),
}

_LIB = None


class DPStokesError(RuntimeError):
    """Error reported by the C ABI (code + message)."""

    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


def lib(build_if_missing=False):
    """The loaded library (cached).  Raises if it is not built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError("libdpstokes_gb300.so is not built (%s); run "
                              "`python -m doublyperiodicstokes_gb300.build`" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def check(code):
    if code != DPST_OK:
        msg = lib().dpst_last_error()
        raise DPStokesError(code, msg.decode() if msg else "")
