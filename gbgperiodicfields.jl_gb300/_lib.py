"""ctypes binding of libgbg_gb300.so (the C ABI declared in include/gbg_transfer.h).

This is the product path: there is no CPU fallback.  ``load()`` raises if the shared
library has not been built or cannot be loaded, and every transfer refuses host arrays.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libgbg_gb300.so"
HEADER = PKG.parent / "include" / "gbg_transfer.h"

GBG_OK = 0
GBG_EARG = 1
GBG_EDIM = 2
GBG_ENOMEM = 3
GBG_ECUDA = 4
GBG_ENONFINITE = 5
GBG_ETIMEOUT = 6
GBG_EUNSUPPORTED = 7
GBG_EBUSY = 8
GBG_ETRAVERSAL = 9

GBG_F32 = 1
GBG_F64 = 2

GBG_DEV_NONFINITE = 1
GBG_DEV_TRAVERSAL = 2
GBG_DEV_TIMEOUT = 4

GBG_MAX_NODES = 16
GBG_MAX_POWERS = 32


class ArgumentError(ValueError):
    """The reference's ArgumentError."""


class DimensionMismatch(ValueError):
    """The reference's DimensionMismatch."""


class InexactError(ArithmeticError):
    """A non-finite or out-of-range position reached floor(Int, ...) (the reference's
    InexactError from _locate)."""


class MethodError(TypeError):
    """The reference's MethodError: no method for this combination of argument types
    (a spectral transfer scheme with a physical field, or the other way round)."""


class GBGError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class GridC(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64 * 3), ("domain", ctypes.c_double * 3),
                ("spacing", ctypes.c_double * 3), ("origin", ctypes.c_double * 3)]


class SchemeC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("stencil_width", ctypes.c_int32),
                ("smoothness", ctypes.c_int32), ("num_powers", ctypes.c_int32),
                ("coefficients", ctypes.c_double * (GBG_MAX_NODES * GBG_MAX_POWERS))]


class BatchItemC(ctypes.Structure):
    _fields_ = [("field", ctypes.c_void_p), ("bins", ctypes.c_void_p), ("scheme", SchemeC),
                ("out", ctypes.c_void_p), ("dest", ctypes.c_void_p), ("q", ctypes.c_void_p),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double)]


class ServerConfigC(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int32), ("max_batch", ctypes.c_int32), ("brick", ctypes.c_int32 * 3),
                ("reserved", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_size_t),
                ("timeout_seconds", ctypes.c_double)]


class RequestC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("pos_dtype", ctypes.c_int32), ("field", ctypes.c_void_p),
                ("scheme", SchemeC), ("positions", ctypes.c_void_p), ("npoints", ctypes.c_int64),
                ("out", ctypes.c_void_p), ("q", ctypes.c_void_p), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("ready_event", ctypes.c_void_p)]


class ServerCountersC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "failed", "queued", "in_flight", "runs",
                                               "points")] + \
               [(n, ctypes.c_double) for n in ("p50_ms", "p99_ms", "mean_ms", "max_ms", "first_submit_s",
                                                "last_done_s")] + \
               [(n, ctypes.c_size_t) for n in ("hbm_in_use", "hbm_peak", "hbm_budget")]


GBG_REQ_INTERPOLATE = 1
GBG_REQ_ANTERPOLATE = 2
GBG_FAULT_ALLOC = 1
GBG_FAULT_DEADLINE = 2

_lib = None

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_GP = ctypes.POINTER(GridC)
_SP = ctypes.POINTER(SchemeC)

# name -> (restype, argtypes).  Every function the header declares is listed here and
# checked against the header by the tests.
SIGNATURES = {
    "gbg_abi_version": (_I32, []),
    "gbg_status_string": (ctypes.c_char_p, [_I32]),
    "gbg_last_error": (ctypes.c_char_p, []),
    "gbg_kernel_launches": (ctypes.c_uint64, []),
    "gbg_set_kernel_timing_events": (_I32, [_P, _P]),
    "gbg_scheme_lalescu": (_I32, [_I32, _I32, _SP]),
    "gbg_scheme_lagrange": (_I32, [_I32, _SP]),
    "gbg_scheme_custom": (_I32, [_I32, _I32, ctypes.POINTER(_D), _SP]),
    "gbg_axis_weights": (_I32, [_SP, _D, ctypes.POINTER(_D)]),
    "gbg_interpolate": (_I32, [_GP, _I32, _I32, _P, _P, _I64, _P, _SP, _P, _P, _P]),
    "gbg_anterpolate": (_I32, [_GP, _I32, _I32, _P, _P, _I64, _P, _P, _SP, _D, _D, _P, _SZ, _P, _P]),
    "gbg_anterpolate_workspace_size": (_I32, [_GP, _I32, _I32, _I64, _SP, ctypes.POINTER(_SZ)]),
    "gbg_point_traversal_order": (_I32, [_GP, _I32, _P, _I64, _I64, _P, _P, _SZ, _P]),
    "gbg_point_traversal_order_workspace_size": (_I32, [_GP, _I64, _I64, ctypes.POINTER(_SZ)]),
    "gbg_validate_traversal": (_I32, [_P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                      ctypes.POINTER(_I64), _P]),
    "gbg_anterpolate_noalloc": (_I32, [_GP, _I32, _I32, _P, _P, _I64, _P, _SP, _D, _D, _P, _P]),
    "gbg_field_create": (_I32, [_GP, _I32, _I32, _I32, ctypes.POINTER(_P)]),
    "gbg_field_destroy": (_I32, [_P]),
    "gbg_field_import": (_I32, [_P, _I32, _P, _P]),
    "gbg_field_export": (_I32, [_P, _I32, _P, _P]),
    "gbg_field_bytes": (_I32, [_P, ctypes.POINTER(_SZ)]),
    "gbg_bins_create": (_I32, [_GP, _I64, ctypes.POINTER(_I32), ctypes.POINTER(_P)]),
    "gbg_bins_destroy": (_I32, [_P]),
    "gbg_bins_set_launch": (_I32, [_P, _I32, _I32]),
    "gbg_bins_set_compensated": (_I32, [_P, _I32]),
    "gbg_bins_set_sparse_regions": (_I32, [_P, _I32]),
    "gbg_bins_set_wait_limit": (_I32, [_P, ctypes.c_uint32]),
    "gbg_points_displace": (_I32, [_GP, _I32, _P, _P, _I64, _I32, ctypes.POINTER(_D), ctypes.POINTER(_P), _P]),
    "gbg_bins_build_displaced": (_I32, [_P, _I32, _P, _P, _I64, _I32, ctypes.POINTER(_D), ctypes.POINTER(_P),
                                        _I32, _P, _P]),
    "gbg_bins_permute": (_I32, [_P, _I32, _I32, _P, _P, _P]),
    "gbg_bins_build": (_I32, [_P, _I32, _P, _I64, _P, _P]),
    "gbg_bins_build_batch": (_I32, [_P, _P, _P, _P, _I32, _P, _P]),
    "gbg_bins_order": (_I32, [_P, _P, _P]),
    "gbg_interpolate_binned": (_I32, [_P, _P, _SP, _I32, _P, _P, _P]),
    "gbg_anterpolate_binned": (_I32, [_P, _P, _SP, _I32, _P, _D, _D, _P, _P]),
    "gbg_batch_create": (_I32, [ctypes.POINTER(BatchItemC), _I32, ctypes.POINTER(_P)]),
    "gbg_batch_run": (_I32, [_P, _P, _P]),
    "gbg_batch_destroy": (_I32, [_P]),
    "gbg_server_create": (_I32, [ctypes.POINTER(ServerConfigC), ctypes.POINTER(_P)]),
    "gbg_server_submit": (_I32, [_P, ctypes.POINTER(RequestC), ctypes.POINTER(_I64)]),
    "gbg_server_wait": (_I32, [_P, _I64, _D, ctypes.POINTER(_I32)]),
    "gbg_server_drain": (_I32, [_P, _D]),
    "gbg_server_stats": (_I32, [_P, _I32, ctypes.POINTER(ServerCountersC)]),
    "gbg_server_inject": (_I32, [_P, _I32, _I32]),
    "gbg_server_destroy": (_I32, [_P]),
    "gbg_server_plan": (_I32, [ctypes.POINTER(_I32), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(_SZ), _I32,
                               _SZ, _I32, ctypes.POINTER(_I32)]),
    "gbg_nufft_deconvolution_axis": (_I32, [_I64, _I32, _I32, _I32, _D, _I32, ctypes.POINTER(_D)]),
    "gbg_nufft_interp_workspace_size": (_I32, [_GP, _I32, _I32, _I64, _I32, ctypes.POINTER(_SZ)]),
    "gbg_nufft_interp": (_I32, [_GP, _I32, _I32, _P, _P, _I64, _P, _I32, _D, _P, _P, _SZ, _P, _P]),
    "gbg_nufft_spread_workspace_size": (_I32, [_GP, _I32, _I32, _I64, _I32, ctypes.POINTER(_SZ)]),
    "gbg_nufft_spread": (_I32, [_GP, _I32, _I32, _P, _P, _I64, _P, _P, _I32, _D, _P, _SZ, _P, _P]),
}


def header_functions() -> list[str]:
    """Names of the functions declared in include/*.h (for the export test)."""
    names = []
    for h in sorted(HEADER.parent.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(gbg_\w+)\s*\(", text)
    return sorted(set(names))


def load():
    """Load the extension (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        from . import builder
        builder.build()
    if not LIB_PATH.exists():
        raise RuntimeError(f"the CUDA extension {LIB_PATH} is missing; run build() first")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().gbg_last_error().decode()


def check(status: int, what: str = ""):
    """Map a status code to the reference's exception types."""
    if status == GBG_OK:
        return
    msg = last_error() or load().gbg_status_string(status).decode()
    if what:
        msg = f"{what}: {msg}"
    if status in (GBG_EARG, GBG_ETRAVERSAL):
        raise ArgumentError(msg)
    if status == GBG_EDIM:
        raise DimensionMismatch(msg)
    if status == GBG_ENONFINITE:
        raise InexactError(msg)
    raise GBGError(status, msg)
