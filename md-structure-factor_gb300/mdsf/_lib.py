"""ctypes binding of ``libmsf.so`` (C ABI in ``include/msf.h``).

The library is the product path: if it is missing or cannot be loaded this
module raises, it never substitutes a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_int = C.c_int32
c_i64 = C.c_int64
c_p = C.c_void_p
c_d = C.c_double
c_size = C.c_size_t

MSF_WRAP = 1
MSF_CONTINUE = 2
ERRORS = {
    0: "MSF_OK", -1: "MSF_E_INVALID", -2: "MSF_E_UNSUPPORTED", -3: "MSF_E_WORKSPACE",
    -4: "MSF_E_CUDA", -5: "MSF_E_RANGE", -6: "MSF_E_NOT_BOUND", -7: "MSF_E_TIMEOUT",
    -8: "MSF_E_TYPE",
}


class MsfError(RuntimeError):
    """A libmsf entry point returned a negative status."""

    def __init__(self, status, where):
        self.status = status
        msg = _lib.msf_strerror(status).decode() if _lib is not None else ERRORS.get(status, "?")
        super().__init__(f"{where}: {ERRORS.get(status, status)} ({msg})")


class PlanDesc(C.Structure):
    _fields_ = [("n0", c_int), ("n1", c_int), ("n2", c_int), ("batch", c_int),
                ("box", c_d * 3), ("variant", c_int), ("tile_w", c_int),
                ("rows_per_block", c_int), ("deposit_block", c_int), ("max_atoms", c_i64),
                ("options", c_int)]


class BatchSystem(C.Structure):
    _fields_ = [("pos_w", c_p), ("scale", c_p), ("sf", c_p), ("n_atoms", c_i64), ("n_frames", c_i64),
                ("box", c_d * 3), ("n0", c_int), ("n1", c_int), ("n2", c_int), ("flags", c_int),
                ("batch", c_int), ("variant", c_int), ("tile_w", c_int)]


# name -> (restype, argtypes); every symbol declared in include/msf.h
SIGNATURES = {
    "msf_strerror": (C.c_char_p, [c_int]),
    "msf_version": (c_int, []),
    "msf_plan_create": (c_int, [C.POINTER(c_p), C.POINTER(PlanDesc)]),
    "msf_plan_destroy": (c_int, [c_p]),
    "msf_plan_workspace_bytes": (c_size, [c_p]),
    "msf_plan_bind": (c_int, [c_p, c_p, c_size, c_p]),
    "msf_plan_status": (c_int, [c_p, c_p]),
    "msf_plan_query": (c_int, [c_p, C.POINTER(c_int)]),
    "msf_hist_grid_f32": (c_int, [c_p, c_p, c_i64, c_p, c_int, c_p, c_p]),
    "msf_hist_grid_f32xyz": (c_int, [c_p, c_p, c_p, c_i64, c_p, c_int, c_p, c_p]),
    "msf_hist_grid_f64": (c_int, [c_p, c_p, c_p, c_i64, c_p, c_int, c_p, c_p]),
    "msf_power_accum_i32": (c_int, [c_p, c_p, c_int, c_p, c_p]),
    "msf_power_accum_f32": (c_int, [c_p, c_p, c_int, c_p, c_p]),
    "msf_power_accum_f64": (c_int, [c_p, c_p, c_int, c_p, c_p]),
    "msf_hist_sf_f32": (c_int, [c_p, c_p, c_i64, c_i64, c_p, c_int, c_p, c_p]),
    "msf_hist_sf_f32xyz": (c_int, [c_p, c_p, c_p, c_i64, c_i64, c_p, c_int, c_p, c_p]),
    "msf_hist_sf_f64": (c_int, [c_p, c_p, c_p, c_i64, c_i64, c_p, c_int, c_p, c_p]),
    "msf_hist_bucket_grid": (c_int, [c_p, c_int, c_p, c_p, c_i64, c_p, c_int, c_p, c_p]),
    "msf_hist_batch_stages": (c_int, [c_p, c_int, c_int, c_p, c_p, c_i64, c_int, c_p, c_int, c_p, c_p]),
    "msf_gauss_grid_f64": (c_int, [c_p, c_p, c_p, c_i64, c_p, c_int, c_p, c_p, c_p]),
    "msf_sfplt": (c_int, [c_p, c_int, c_int, c_int, c_p, c_p]),
    "msf_ewald": (c_int, [c_p, c_int, c_int, c_int, c_p, c_p, c_p, c_d, c_p, c_p, c_p, c_p]),
    "msf_cyl_average": (c_int, [c_p, c_int, c_int, c_int, c_p, c_p, c_p, c_p, c_p, c_p, c_int, c_p, c_int,
                                c_p, c_p]),
    "msf_rz_hist": (c_int, [c_p, c_int, c_int, c_int, c_p, c_p, c_p, c_p, c_int, c_p, c_int, c_p, c_int, c_p, c_p,
                            c_p]),
    "msf_nearest_sheared": (c_int, [c_p, c_int, c_int, c_int, c_p, c_p, c_p, c_p, c_p, c_i64, c_p, c_p, c_p]),
    "msf_radial_range": (c_int, [c_p, c_i64, c_p, c_p]),
    "msf_radial_bin_points": (c_int, [c_p, c_i64, c_p, c_int, c_p, c_p, c_p, c_p]),
    "msf_radial_bin_grid": (c_int, [c_p, c_int, c_int, c_int, c_p, c_p, c_p, c_p, c_int, c_p, c_p, c_p, c_p]),
    "msf_direct_fwd": (c_int, [c_p, c_i64, c_p, c_i64, c_int, c_int, c_p, c_p, c_p]),
    "msf_direct_bwd": (c_int, [c_p, c_i64, c_p, c_i64, c_int, c_int, c_p, c_p, c_p, c_p]),
    "msf_batch_create": (c_int, [C.POINTER(c_p), C.POINTER(BatchSystem), c_int, c_int]),
    "msf_batch_workspace_bytes": (c_size, [c_p]),
    "msf_batch_bind": (c_int, [c_p, c_p, c_size, c_p]),
    "msf_batch_run": (c_int, [c_p, c_p]),
    "msf_batch_query": (c_int, [c_p, c_int, C.POINTER(c_int)]),
    "msf_batch_destroy": (c_int, [c_p]),
    "msf_hist_sf_f32_noalloc": (c_int, [c_p, c_i64, c_i64, c_p, c_int, c_int, c_int, c_int, c_p, c_p]),
    "msf_noalloc_scratch_bytes": (c_size, []),
    "msf_noalloc_init": (c_int, [c_int, c_int, c_int, c_p, c_p]),
    "msf_noalloc_status": (c_int, [c_p]),
    "msf_gro_scan": (c_int, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "msf_gro_read": (c_int, [C.c_char_p, C.c_int64, C.c_int64, c_p, c_p, c_p, c_int]),
    "msf_trr_scan": (c_int, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "msf_trr_read": (c_int, [C.c_char_p, C.c_int64, C.c_int64, c_p, c_p, c_int]),
}


def lib_path():
    return os.environ.get("MSF_LIB", _build.LIB)


def load(build_if_missing=True):
    """Load (building first when stale and nvcc is present) and type the library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if build_if_missing and "MSF_LIB" not in os.environ:
            try:
                _build.build()
            except RuntimeError:
                if not os.path.exists(path):
                    raise
        if not os.path.exists(path):
            raise OSError(f"libmsf.so not found at {path}; run mdsf.build.build() (needs nvcc)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status, where):
    if status != 0:
        raise MsfError(status, where)
    return status


def call(name, *args):
    lib = load()
    return check(getattr(lib, name)(*args), name)
