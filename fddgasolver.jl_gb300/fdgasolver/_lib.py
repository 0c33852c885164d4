"""ctypes binding of libfdga (include/fdga.h).  The library is loaded from this package's _lib/
directory; importing never falls back to a CPU path: a missing or unloadable library raises."""
import ctypes
import os

from . import build as _build


class FdgaError(RuntimeError):
    """A nonzero libfdga status, with the library's message."""

    def __init__(self, code, msg):
        super().__init__(f"libfdga error {code}: {msg}")
        self.code = code


class fdga_config(ctypes.Structure):
    _fields_ = [
        ("nG", ctypes.c_int32), ("nK1", ctypes.c_int32), ("nK2", ctypes.c_int32 * 2), ("nK3", ctypes.c_int32 * 2),
        ("L", ctypes.c_int32), ("LG", ctypes.c_int32), ("mPi_factor", ctypes.c_int32), ("local", ctypes.c_int32),
        ("T", ctypes.c_double), ("U", ctypes.c_double), ("nR", ctypes.c_int32 * 2), ("precision", ctypes.c_int32),
        ("f0_vertex", ctypes.c_int32), ("nF0K1", ctypes.c_int32), ("nF0K2", ctypes.c_int32 * 2),
        ("nF0K3", ctypes.c_int32 * 2),
    ]


EXPORTS = {
    "fdga_create": (ctypes.c_int, [ctypes.POINTER(fdga_config), ctypes.POINTER(ctypes.c_void_p)]),
    "fdga_destroy": (None, [ctypes.c_void_p]),
    "fdga_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "fdga_create_error": (ctypes.c_char_p, []),
    "fdga_set_input": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_finalize": (ctypes.c_int, [ctypes.c_void_p]),
    "fdga_init_sym_grp": (ctypes.c_int, [ctypes.c_void_p]),
    "fdga_group_map": (ctypes.c_int, [ctypes.POINTER(fdga_config), ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_int)]),
    "fdga_state_len": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "fdga_flatten": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_unflatten": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_iterate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "fdga_set_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdga_set_option": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "fdga_residual": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                  ctypes.c_void_p]),
    "fdga_solve_mixed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_void_p, ctypes.c_void_p]),
    "fdga_solve_newton": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "fdga_jvp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_mfrg_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_size_t]),
    "fdga_residual_mfrg": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_double)]),
    "fdga_solve_mfrg": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "fdga_frule": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_rrule": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_set_U": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "fdga_dyson_bubbles": (ctypes.c_int, [ctypes.c_void_p]),
    "fdga_interpolate_solver": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdga_dchi_dU": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t,
                                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
    "fdga_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "fdga_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "fdga_batch_destroy": (None, [ctypes.c_void_p]),
    "fdga_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "fdga_batch_iterate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "fdga_batch_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "fdga_batch_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)]),
    "fdga_get_named": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_named_len": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]),
    "fdga_occupation": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "fdga_susceptibility": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_event_record": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdga_event_elapsed_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "fdga_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "fdga_stage_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "fdga_tangent_stage_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "fdga_map_repeat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "fdga_tangent_repeat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "fdga_adjoint_repeat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "fdga_flush_l2": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t]),
    "fdga_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "fdga_host_free": (ctypes.c_int, [ctypes.c_void_p]),
    "fdga_bubble_noalloc": (ctypes.c_int, [ctypes.POINTER(fdga_config), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "fdga_query": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]),
    "fdga_launches_per_iteration": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
}

FDGA_FDPA, FDGA_SCPA, FDGA_FDPA_NEW, FDGA_SCPA_NEW, FDGA_FDPA_1LOOP = 0, 1, 2, 3, 4
FDGA_FP64, FDGA_MIXED = 0, 1
IN_GBARE, IN_G0, IN_SIGMA0, IN_FP_P, IN_FP_X, IN_FT_P, IN_FT_X, IN_F0_VERTEX = range(8)

_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libfdga (building it first if it is missing and nvcc is available)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale()):
        _build.build()
    if not os.path.exists(path):
        raise FdgaError(-1, f"libfdga not built: {path} is missing")
    lib = ctypes.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc: int, h=None) -> None:
    if rc != 0:
        lib = load()
        msg = lib.fdga_last_error(h) if h else lib.fdga_create_error()
        raise FdgaError(rc, (msg or b"").decode(errors="replace"))
