"""ctypes binding of libpluto_gb300.so (the C ABI in include/pluto_gb300.h).

There is no fallback: if the shared library is missing or fails to load,
``lib()`` raises.  ``build()`` compiles it in-tree with nvcc.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

LIB_PATH = _build.LIB

PG_OK = 0
PG_LINEAR, PG_PARABOLIC = 0, 1
PG_FLAT_LIM, PG_MINMOD_LIM, PG_VANLEER_LIM, PG_MC_LIM, PG_DEFAULT_LIM = 0, 1, 2, 3, 4
PG_HLL, PG_HLLD, PG_ROE = 0, 1, 2
PG_RK2, PG_RK3, PG_HANCOCK, PG_CHAR_TRACING, PG_HANCOCK_CONS = 2, 3, 4, 5, 6
PG_DIVB_NONE, PG_CONSTRAINED_TRANSPORT = 0, 1
PG_ARITHMETIC, PG_UCT0, PG_UCT_CONTACT, PG_UCT_HLL = 1, 2, 3, 4
PG_PERIODIC, PG_OUTFLOW, PG_REFLECTIVE, PG_EQTSYMMETRIC, PG_USERDEF = 0, 1, 2, 3, 4
PG_EULER = 1
PG_FP64, PG_MIXED, PG_MIXED_DW, PG_FP64_TANGENT, PG_FP64_DD = 0, 1, 2, 3, 4
PG_LAYOUT_INTERIOR, PG_LAYOUT_PLUTO = 0, 1

PG_ERR_INVALID, PG_ERR_CUDA, PG_ERR_NOMEM, PG_ERR_NAN = 1, 2, 3, 4
PG_ERR_DT_TOO_SMALL, PG_ERR_TIMEOUT, PG_ERR_TOO_LARGE = 5, 6, 7
ERRORS = {1: "PG_ERR_INVALID", 2: "PG_ERR_CUDA", 3: "PG_ERR_NOMEM", 4: "PG_ERR_NAN",
          5: "PG_ERR_DT_TOO_SMALL", 6: "PG_ERR_TIMEOUT", 7: "PG_ERR_TOO_LARGE"}

# Every symbol declared in include/pluto_gb300.h (checked by the CPU tests).
EXPORTS = ["pg_create", "pg_destroy", "pg_upload", "pg_download", "pg_advance", "pg_run",
           "pg_run_async", "pg_sync", "pg_run_timed", "pg_profile_kernels", "pg_get_stream",
           "pg_get_info", "pg_kernel_launches_per_step", "pg_last_error", "pg_abi_version",
           "pg_tube_step_static", "pg_batch_create", "pg_batch_destroy", "pg_batch_upload",
           "pg_batch_download", "pg_batch_run", "pg_batch_get", "pg_batch_autotune",
           "pg_batch_set_schedule", "pg_tangent_upload", "pg_tangent_download", "pg_tangent_kink", "pg_adjoint_set",
           "pg_adjoint_step", "pg_adjoint_get", "pg_adjoint_slots", "pg_adjoint_forward",
           "pg_adjoint_reverse", "pg_checkpoint_save", "pg_checkpoint_load", "pg_selftest_conversions", "pg_set_userdef", "pg_set_internal_boundary",
           "pg_write_output", "pg_output_wait", "pg_read_output", "pg_download_async", "pg_download_wait"]
PG_ABI_VERSION = 3  # the pg_config layout these bindings describe
# pg_userdef_fn: (user, side 0..5, vpos 0 cells / 1..3 faces, stage)
USERDEF_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_int)
PG_STATIC_MAX_ZONES = 32768
PG_MAX_CHECKPOINTS = 256


class PgConfig(C.Structure):
    _fields_ = [("dims", C.c_int), ("components", C.c_int), ("nx", C.c_int * 3),
                ("dx", C.c_double * 3), ("gamma", C.c_double),
                ("reconstruction", C.c_int), ("limiter", C.c_int), ("riemann", C.c_int),
                ("time_stepping", C.c_int), ("divb", C.c_int), ("emf_average", C.c_int),
                ("bc", C.c_int * 3), ("precision", C.c_int), ("compute_mach", C.c_int),
                ("small_density", C.c_double), ("small_pressure", C.c_double),
                ("bc_hi", C.c_int * 3), ("bc_sides", C.c_int), ("char_limiting", C.c_int)]


PG_OUT_DBL, PG_OUT_FLT, PG_OUT_VTK = 0, 1, 2
PG_OUT_MAX_VARS = 16
PG_OUT_VECTOR = 5


class PgOutput(C.Structure):
    _fields_ = [("format", C.c_int), ("single_file", C.c_int), ("nfile", C.c_int), ("nvar", C.c_int),
                ("var", C.c_int * PG_OUT_MAX_VARS), ("dump", C.c_int * PG_OUT_MAX_VARS),
                ("name", C.c_char_p * PG_OUT_MAX_VARS), ("unit", C.c_double * PG_OUT_MAX_VARS),
                ("dir", C.c_char_p), ("xnode", C.POINTER(C.c_double) * 3),
                ("time", C.c_double), ("dt", C.c_double), ("step", C.c_long), ("write_record", C.c_int)]


class PgStepInfo(C.Structure):
    _fields_ = [("inv_dt_hyp", C.c_double), ("max_mach", C.c_double), ("nfail", C.c_int64)]


class PgError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def build(force: bool = False) -> Path:
    return _build.build(force=force)


def load(path: Path | str | None = None):
    """Load the library without building (raises OSError when absent)."""
    return C.CDLL(str(path or LIB_PATH))


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise OSError(f"{LIB_PATH} is missing: run pluto_gb300.build.build() (nvcc) first")
    L = C.CDLL(str(LIB_PATH))
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    L.pg_create.argtypes = [C.POINTER(PgConfig), C.POINTER(vp)]
    L.pg_destroy.argtypes = [vp]
    L.pg_upload.argtypes = [vp, C.POINTER(dp), C.POINTER(dp), ip]
    L.pg_download.argtypes = [vp, C.POINTER(dp), C.POINTER(dp), ip]
    L.pg_advance.argtypes = [vp, C.c_double, C.POINTER(PgStepInfo)]
    L.pg_run.argtypes = [vp, ip, C.c_double, C.c_double, C.c_double, dp, dp]
    L.pg_run_async.argtypes = [vp, ip, C.c_double, C.c_double, C.c_double]
    L.pg_sync.argtypes = [vp]
    L.pg_run_timed.argtypes = [vp, ip, C.c_double, C.c_double, C.c_double, dp]
    L.pg_profile_kernels.argtypes = [vp, ip, C.c_double, C.c_double, C.c_double, C.c_char_p, ip, dp,
                                     C.POINTER(C.c_int), ip, C.POINTER(C.c_int)]
    L.pg_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.pg_get_info.argtypes = [vp, C.POINTER(PgStepInfo), dp, dp]
    L.pg_kernel_launches_per_step.argtypes = [vp]
    L.pg_tube_step_static.argtypes = [C.POINTER(PgConfig), vp, vp, C.c_double, vp, C.POINTER(PgStepInfo)]
    IP = C.POINTER(C.c_int)
    L.pg_batch_create.argtypes = [C.POINTER(PgConfig), ip, IP, dp, C.POINTER(vp)]
    L.pg_batch_destroy.argtypes = [vp]
    L.pg_batch_upload.argtypes = [vp, dp]
    L.pg_batch_download.argtypes = [vp, dp]
    L.pg_batch_run.argtypes = [vp, ip, C.c_double, C.c_double, C.c_double, dp]
    L.pg_batch_get.argtypes = [vp, dp, dp, C.POINTER(C.c_int64)]
    L.pg_batch_autotune.argtypes = [vp, ip, C.c_double, C.c_double, C.c_double, IP, IP, IP, dp]
    L.pg_batch_set_schedule.argtypes = [vp, ip, ip, ip]
    for fn in ("pg_tangent_upload", "pg_tangent_download", "pg_adjoint_set", "pg_adjoint_get"):
        getattr(L, fn).argtypes = [vp, C.POINTER(dp), C.POINTER(dp), ip]
    L.pg_adjoint_step.argtypes = [vp, C.c_double]
    L.pg_adjoint_slots.argtypes = [vp, ip]
    L.pg_adjoint_forward.argtypes = [vp, C.c_double, ip]
    L.pg_adjoint_reverse.argtypes = [vp, C.c_double, ip]
    L.pg_tangent_kink.argtypes = [vp, ip, dp]
    L.pg_checkpoint_save.argtypes = [vp, ip]
    L.pg_checkpoint_load.argtypes = [vp, ip]
    L.pg_selftest_conversions.argtypes = [C.POINTER(C.c_ulonglong)]
    L.pg_set_userdef.argtypes = [vp, USERDEF_FN, vp, C.POINTER(dp), C.POINTER(dp)]
    L.pg_set_internal_boundary.argtypes = [vp, C.POINTER(C.c_ubyte)]
    L.pg_write_output.argtypes = [vp, C.POINTER(PgOutput)]
    L.pg_output_wait.argtypes = [vp]
    L.pg_read_output.argtypes = [vp, C.POINTER(PgOutput)]
    L.pg_download_async.argtypes = [vp, C.POINTER(dp), C.POINTER(dp)]
    L.pg_download_wait.argtypes = [vp]
    L.pg_last_error.restype = C.c_char_p
    for fn in ("pg_create", "pg_destroy", "pg_upload", "pg_download", "pg_advance", "pg_run",
               "pg_run_async", "pg_sync", "pg_run_timed", "pg_profile_kernels", "pg_get_stream",
               "pg_get_info", "pg_kernel_launches_per_step", "pg_abi_version", "pg_tube_step_static",
               "pg_batch_create", "pg_batch_destroy", "pg_batch_upload", "pg_batch_download",
               "pg_batch_run", "pg_batch_get", "pg_batch_autotune", "pg_batch_set_schedule",
               "pg_tangent_upload", "pg_tangent_download", "pg_tangent_kink", "pg_adjoint_set", "pg_adjoint_step",
               "pg_adjoint_get", "pg_adjoint_slots", "pg_adjoint_forward", "pg_adjoint_reverse",
               "pg_checkpoint_save", "pg_checkpoint_load", "pg_selftest_conversions",
               "pg_set_userdef", "pg_set_internal_boundary", "pg_write_output", "pg_output_wait",
               "pg_read_output", "pg_download_async", "pg_download_wait"):
        getattr(L, fn).restype = C.c_int
    if L.pg_abi_version() != PG_ABI_VERSION:
        raise OSError(f"libpluto_gb300 has ABI version {L.pg_abi_version()}, these bindings expect "
                      f"{PG_ABI_VERSION}: rebuild the library")
    _lib = L
    return L


def check(rc: int, where: str):
    if rc != PG_OK:
        raise PgError(rc, where, lib().pg_last_error().decode())
