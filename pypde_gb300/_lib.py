"""ctypes binding of libpypde_gb300.so (the C ABI of include/pypde_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded,
every call raises.  There is no CPU fallback.
"""
import ctypes
import os
import threading
from ctypes import (POINTER, Structure, c_bool, c_char_p, c_double, c_int,
                    c_longlong, c_ulonglong, c_void_p)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpypde_gb300.so")

PYPDE_OK = 0
PYPDE_ERR_ARG = 1
PYPDE_ERR_CUDA = 2
PYPDE_ERR_UNSUPPORTED = 3
PYPDE_NAN_FOUND = 4
PYPDE_ERR_COMPILE = 5


class Options(Structure):
    _fields_ = [("max_steps", c_longlong), ("newton_tol", c_double),
                ("device", c_int), ("steps_per_graph", c_int), ("profile_stages", c_int),
                ("warm_start", c_void_p), ("mixed_precision", c_int), ("strips", c_int)]

STAGES = ("boundaries", "weno", "cfl", "predictor", "faces", "centers", "gather", "other")


class Stats(Structure):
    _fields_ = [("steps", c_longlong), ("t_final", c_double),
                ("pred_iters", c_ulonglong), ("pred_max_iters", c_int),
                ("pred_fail", c_int), ("nan_found", c_int),
                ("device_seconds", c_double), ("kernel_launches", c_longlong),
                ("stage_seconds", c_double * 8), ("pred_fallbacks", c_ulonglong),
                ("pred_iters32", c_ulonglong)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "stage_seconds"}
        d["stage_seconds"] = dict(zip(STAGES, list(self.stage_seconds)))
        return d


dp = POINTER(c_double)
ip = POINTER(c_int)
fp = POINTER(ctypes.c_float)


class BatchProblem(Structure):
    _fields_ = [("u", dp), ("tf", c_double), ("nX", c_int * 3), ("dX", c_double * 3),
                ("boundaryTypes", c_int * 3), ("N", c_int), ("cfl", c_double)]


class BatchOptions(Structure):
    _fields_ = [("max_steps", c_longlong), ("newton_tol", c_double), ("device", c_int),
                ("steps_per_graph", c_int), ("autotune", c_int), ("per_pop", c_int),
                ("mixed_precision", c_int), ("warm_start", c_void_p * 4)]


BATCH_STAGES = ("boundaries", "weno0", "weno1", "weno2", "cfl", "predictor", "faces",
                "centers", "gather", "guess")


class BatchStats(Structure):
    _fields_ = [("steps", c_longlong), ("max_problem_steps", c_longlong),
                ("device_seconds", c_double), ("kernel_launches", c_longlong),
                ("pred_iters", c_ulonglong), ("nan_found", c_int), ("per_pop", c_int * 10),
                ("tune_seconds", c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "per_pop"}
        d["per_pop"] = dict(zip(BATCH_STAGES, list(self.per_pop)))
        return d

# name -> (restype, argtypes)
SIGNATURES = {
    "pypde_system_builtin": (c_int, [c_char_p, c_int, POINTER(c_void_p)]),
    "pypde_system_compile": (c_int, [c_char_p, c_char_p, c_int, c_int, c_int, c_int, c_int,
                                     c_int, POINTER(c_void_p)]),
    "pypde_system_info": (c_int, [c_void_p, ip, ip, ip, ip, ip, ip]),
    "pypde_system_free": (None, [c_void_p]),
    "pde_solver": (c_int, [c_void_p, c_void_p, c_void_p, c_bool, c_bool, c_bool, dp, c_double,
                           ip, c_int, dp, c_double, ip, c_bool, c_int, c_int, c_int, c_int,
                           c_bool, dp, c_int]),
    "pde_solver_ex": (c_int, [c_void_p, c_bool, c_bool, c_bool, dp, c_double, ip, c_int, dp,
                              c_double, ip, c_bool, c_int, c_int, c_int, dp, POINTER(Options),
                              POINTER(Stats)]),
    "weno_solver": (c_int, [dp, dp, ip, c_int, c_int, c_int]),
    "weno_solver_noalloc": (c_int, [c_void_p, c_void_p, ip, c_int, c_int, c_int, c_void_p]),
    "pypde_boundaries": (c_int, [dp, ip, c_int, ip, c_int, c_int, dp]),
    "pypde_timestep": (c_int, [c_void_p, dp, c_longlong, dp, c_int, c_int, c_double, c_double,
                               c_double, c_longlong, dp]),
    "pypde_predictor": (c_int, [c_void_p, dp, c_longlong, dp, c_int, c_int, c_bool, c_double,
                                c_double, dp, POINTER(Stats)]),
    "pypde_fv": (c_int, [c_void_p, dp, dp, ip, dp, c_int, c_int, c_int, c_double]),
    "pypde_tables": (c_int, [c_int, dp]),
    "pypde_measure_fp64_peak": (c_int, [c_int, dp]),
    "pypde_measure_dmma_peak": (c_int, [c_int, dp]),
    "pde_solver_batch": (c_int, [c_void_p, c_bool, c_int, c_int, POINTER(BatchProblem),
                                 POINTER(BatchOptions), POINTER(BatchStats),
                                 POINTER(c_longlong), dp]),
    "pypde_warm_start_shape": (c_int, [c_void_p, c_int, ip, ip, ip]),
    "pypde_warm_start_create": (c_int, [c_void_p, c_int, c_int] + [fp] * 10 +
                                [c_int, POINTER(c_void_p)]),
    "pypde_warm_start_free": (c_int, [c_void_p]),
    "pypde_predictor_guess": (c_int, [c_void_p, dp, c_longlong, dp, c_int, c_int, c_double,
                                      c_double, dp, c_void_p, dp, POINTER(Stats)]),
    "pypde_harvest": (c_int, [c_void_p, dp, c_double, ip, c_int, dp, c_double, ip, c_bool,
                              c_int, c_int, c_longlong, c_longlong, dp, dp, dp,
                              POINTER(Options), POINTER(Stats)]),
    "pypde_mlp_gemm": (c_int, [c_void_p, c_longlong, c_longlong, c_void_p, c_longlong,
                               c_longlong, c_void_p, c_int, c_int, c_int, c_int, c_void_p,
                               c_void_p, c_void_p, c_void_p]),
    "pypde_mlp_silu_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_longlong, c_void_p]),
    "pypde_mlp_colsum": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p]),
    "pypde_last_error": (c_char_p, []),
}

_lib = None
_lock = threading.Lock()


class PyPDEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pypde_gb300 error {code}: {msg}")
        self.code = code


def lib():
    """Load libpypde_gb300.so once; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is not built; run `python -m pypde_gb300.build` "
                    "(there is no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(code):
    if code not in (PYPDE_OK, PYPDE_NAN_FOUND):
        raise PyPDEError(code, lib().pypde_last_error().decode())
    return code


def c_ptr(arr):
    """Pointer to a contiguous float64 or int32 array (pypde/utils.py:25-34)."""
    if arr.dtype == "int32":
        return arr.ctypes.data_as(ip)
    if arr.dtype == "float64":
        return arr.ctypes.data_as(dp)
    print("invalid array type")
    raise TypeError("arrays passed to the solver must be float64 or int32")
