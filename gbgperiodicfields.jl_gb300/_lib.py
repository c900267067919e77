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

GBG_MAX_NODES = 16
GBG_MAX_POWERS = 32


class ArgumentError(ValueError):
    """The reference's ArgumentError."""


class DimensionMismatch(ValueError):
    """The reference's DimensionMismatch."""


class InexactError(ArithmeticError):
    """A non-finite or out-of-range position reached floor(Int, ...) (the reference's
    InexactError from _locate)."""


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
    "gbg_bins_build": (_I32, [_P, _I32, _P, _I64, _P, _P]),
    "gbg_bins_order": (_I32, [_P, _P, _P]),
    "gbg_interpolate_binned": (_I32, [_P, _P, _SP, _I32, _P, _P]),
    "gbg_anterpolate_binned": (_I32, [_P, _P, _SP, _I32, _P, _D, _D, _P]),
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
