"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the reference's spline transfer
(GBGPeriodicFields.jl src/Interpolation.jl, src/Points.jl); see gbg_oracle.h for
the per-function citations.  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it, and only as the checker or the timed CPU
baseline -- never as a product code path.

Array conventions are the reference's column-major ones, held here as numpy
arrays in Fortran order:
  field       (Nx, Ny, Nz, ncomp)
  positions   (M, 3)
  values      (M, ncomp)
  coefficients (N2, M2)  [node, power]
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "libgbg_oracle.so"
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_ip = ctypes.POINTER(ctypes.c_int)


class OracleError(RuntimeError):
    pass


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    src = _HERE / "gbg_oracle.c"
    if force or not _LIB_PATH.exists() or _LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-C", str(_HERE), "-s"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(_LIB_PATH))
        L.gbgo_fornberg.argtypes = [ctypes.c_double, _dp, ctypes.c_int, ctypes.c_int, _dp]
        L.gbgo_lalescu.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _ip, _ip]
        L.gbgo_lagrange.argtypes = [ctypes.c_int, _dp, _ip, _ip]
        L.gbgo_axis_weights_f64.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp]
        L.gbgo_axis_weights_f64.restype = None
        L.gbgo_axis_weights_f32.argtypes = [_fp, ctypes.c_int, ctypes.c_int, ctypes.c_float, _fp]
        L.gbgo_axis_weights_f32.restype = None
        L.gbgo_tile_index_f64.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int64]
        L.gbgo_tile_index_f64.restype = ctypes.c_int64
        L.gbgo_tile_index_f32.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int64]
        L.gbgo_tile_index_f32.restype = ctypes.c_int64
        L.gbgo_wrap_coordinate_f64.argtypes = [ctypes.c_double] * 3
        L.gbgo_wrap_coordinate_f64.restype = ctypes.c_double
        L.gbgo_wrap_coordinate_f32.argtypes = [ctypes.c_float] * 3
        L.gbgo_wrap_coordinate_f32.restype = ctypes.c_float
        for suf, vp in (("f64", _dp), ("f32", _fp)):
            fn = getattr(L, f"gbgo_displace_{suf}")
            fn.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int32, _dp, ctypes.POINTER(vp), ctypes.c_int32, _dp, _dp]
            fn.restype = None
        L.gbgo_walk.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, _i64p]
        L.gbgo_walk.restype = None
        for suf, vp in (("f64", _dp), ("f32", _fp)):
            g = [_i64p, _dp, _dp, ctypes.c_int, vp, vp, ctypes.c_int64, _i32p, _dp,
                 ctypes.c_int, ctypes.c_int, vp]
            getattr(L, f"gbgo_gather_{suf}").argtypes = g
            getattr(L, f"gbgo_gather_{suf}_mt").argtypes = g + [ctypes.c_int]
            s = [_i64p, _dp, _dp, ctypes.c_int, vp, vp, ctypes.c_int64, vp, _i32p, _dp,
                 ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
            getattr(L, f"gbgo_scatter_{suf}").argtypes = s
            getattr(L, f"gbgo_scatter_{suf}_mt").argtypes = s + [ctypes.c_int]
            getattr(L, f"gbgo_traversal_order_{suf}").argtypes = [
                _i64p, _dp, _dp, vp, ctypes.c_int64, ctypes.c_int64, _i32p, _i64p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _check(status: int, what: str):
    if status == 1:
        raise ValueError(f"oracle {what}: invalid argument")
    if status == 2:
        raise OracleError(f"oracle {what}: non-finite position")
    if status != 0:
        raise OracleError(f"oracle {what}: status {status}")


# ----------------------------------------------------------------- schemes

def fornberg(x0: float, nodes, max_order: int) -> np.ndarray:
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    w = np.zeros((len(nodes), max_order + 1), dtype=np.float64, order="F")
    _check(lib().gbgo_fornberg(x0, _ptr(nodes, ctypes.c_double), len(nodes), max_order,
                               _ptr(w, ctypes.c_double)), "fornberg")
    return w


def lalescu(stencil_width: int, smoothness: int | None = None) -> np.ndarray:
    if smoothness is None:
        smoothness = stencil_width // 2 - 1
    buf = np.zeros(32 * 64, dtype=np.float64)
    n2, m2 = ctypes.c_int(), ctypes.c_int()
    _check(lib().gbgo_lalescu(stencil_width, smoothness, _ptr(buf, ctypes.c_double),
                              ctypes.byref(n2), ctypes.byref(m2)), "lalescu")
    return buf[: n2.value * m2.value].reshape((n2.value, m2.value), order="F").copy(order="F")


def lagrange(stencil_width: int) -> np.ndarray:
    buf = np.zeros(32 * 64, dtype=np.float64)
    n2, m2 = ctypes.c_int(), ctypes.c_int()
    _check(lib().gbgo_lagrange(stencil_width, _ptr(buf, ctypes.c_double),
                               ctypes.byref(n2), ctypes.byref(m2)), "lagrange")
    return buf[: n2.value * m2.value].reshape((n2.value, m2.value), order="F").copy(order="F")


def axis_weights(coeffs: np.ndarray, t, dtype=np.float64) -> np.ndarray:
    n2, m2 = coeffs.shape
    w = np.zeros(n2, dtype=dtype)
    if dtype == np.float64:
        c = np.asfortranarray(coeffs, dtype=np.float64)
        lib().gbgo_axis_weights_f64(_ptr(c, ctypes.c_double), n2, m2, float(t),
                                    _ptr(w, ctypes.c_double))
    else:
        c = np.asfortranarray(coeffs.astype(np.float32))
        lib().gbgo_axis_weights_f32(_ptr(c, ctypes.c_float), n2, m2, float(np.float32(t)),
                                    _ptr(w, ctypes.c_float))
    return w


# ------------------------------------------------------------- transfers

def _grid_arrays(grid):
    n = np.ascontiguousarray(grid["n"], dtype=np.int64)
    origin = np.ascontiguousarray(grid["origin"], dtype=np.float64)
    spacing = np.ascontiguousarray(grid["spacing"], dtype=np.float64)
    domain = np.ascontiguousarray(grid["domain"], dtype=np.float64)
    return n, origin, spacing, domain


def _suffix(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.float64:
        return "f64", ctypes.c_double
    if dtype == np.float32:
        return "f32", ctypes.c_float
    raise TypeError(dtype)


def _trav_ptr(traversal):
    if traversal is None:
        return None, None
    t = np.ascontiguousarray(traversal, dtype=np.int32)
    return t, _ptr(t, ctypes.c_int32)


def gather(grid, field: np.ndarray, positions: np.ndarray, coeffs: np.ndarray,
           traversal=None, nthreads: int = 1) -> np.ndarray:
    """Interpolation.jl:1181-1198 (interpolate!) through the oracle."""
    suf, ct = _suffix(field.dtype)
    n, origin, spacing, _ = _grid_arrays(grid)
    ncomp = int(np.prod(field.shape[3:])) if field.ndim > 3 else 1
    f = np.asfortranarray(field)
    pos = np.asfortranarray(positions, dtype=field.dtype)
    m = pos.shape[0]
    out = np.zeros((m, ncomp), dtype=field.dtype, order="F")
    c = np.asfortranarray(coeffs, dtype=np.float64)
    keep, tp = _trav_ptr(traversal)
    fn = getattr(lib(), f"gbgo_gather_{suf}" + ("_mt" if nthreads != 1 else ""))
    args = [_ptr(n, ctypes.c_int64), _ptr(origin, ctypes.c_double), _ptr(spacing, ctypes.c_double),
            ncomp, _ptr(f, ct), _ptr(pos, ct), m, tp, _ptr(c, ctypes.c_double),
            c.shape[0], c.shape[1], _ptr(out, ct)]
    if nthreads != 1:
        args.append(nthreads)
    _check(fn(*args), "gather")
    return out


def scatter(grid, field: np.ndarray, positions: np.ndarray, quantities: np.ndarray,
            coeffs: np.ndarray, alpha: float = 1.0, beta: float = 0.0, traversal=None,
            nthreads: int = 1) -> np.ndarray:
    """Interpolation.jl:1299-1323 (anterpolate!) through the oracle; field is updated
    in place (it must be Fortran-ordered) and returned."""
    suf, ct = _suffix(field.dtype)
    n, origin, spacing, _ = _grid_arrays(grid)
    ncomp = int(np.prod(field.shape[3:])) if field.ndim > 3 else 1
    if not field.flags.f_contiguous:
        raise ValueError("field must be Fortran-contiguous")
    pos = np.asfortranarray(positions, dtype=field.dtype)
    q = np.asfortranarray(quantities, dtype=field.dtype).reshape((pos.shape[0], ncomp), order="F")
    c = np.asfortranarray(coeffs, dtype=np.float64)
    keep, tp = _trav_ptr(traversal)
    fn = getattr(lib(), f"gbgo_scatter_{suf}" + ("_mt" if nthreads != 1 else ""))
    args = [_ptr(n, ctypes.c_int64), _ptr(origin, ctypes.c_double), _ptr(spacing, ctypes.c_double),
            ncomp, _ptr(field, ct), _ptr(pos, ct), pos.shape[0], _ptr(q, ct), tp,
            _ptr(c, ctypes.c_double), c.shape[0], c.shape[1], float(alpha), float(beta)]
    if nthreads != 1:
        args.append(nthreads)
    _check(fn(*args), "scatter")
    return field


def traversal_order(grid, positions: np.ndarray, tile_size: int = 4, return_keys=False):
    """Interpolation.jl:816-833 (point_traversal_order), stable within a tile."""
    suf, ct = _suffix(positions.dtype)
    n, origin, _, domain = _grid_arrays(grid)
    pos = np.asfortranarray(positions)
    m = pos.shape[0]
    order = np.zeros(m, dtype=np.int32)
    keys = np.zeros(m, dtype=np.int64)
    _check(getattr(lib(), f"gbgo_traversal_order_{suf}")(
        _ptr(n, ctypes.c_int64), _ptr(domain, ctypes.c_double), _ptr(origin, ctypes.c_double),
        _ptr(pos, ct), m, tile_size, _ptr(order, ctypes.c_int32), _ptr(keys, ctypes.c_int64)),
        "traversal_order")
    return (order, keys) if return_keys else order


def tile_index(coordinate, origin, inverse_tile, tiles, dtype=np.float64) -> int:
    if np.dtype(dtype) == np.float64:
        return lib().gbgo_tile_index_f64(coordinate, origin, inverse_tile, tiles)
    return lib().gbgo_tile_index_f32(coordinate, origin, inverse_tile, tiles)


def wrap_coordinate(coordinate, extent, origin, dtype=np.float64):
    if np.dtype(dtype) == np.float64:
        return lib().gbgo_wrap_coordinate_f64(coordinate, extent, origin)
    return lib().gbgo_wrap_coordinate_f32(coordinate, extent, origin)


def displace(src, terms, grid=None):
    """Points.jl displace!: src (M,3) plus sum_j c_j * v_j in order, wrapped when a grid dict
    (with 'domain' and 'origin') is given.  Returns a new (M,3) column-major array."""
    src = np.asfortranarray(src)
    dt = src.dtype
    m = src.shape[0]
    dst = np.zeros_like(src, order="F")
    secs = [np.asfortranarray(v, dtype=dt) for _, v in terms]
    coefs = np.array([float(c) for c, _ in terms] or [0.0], dtype=np.float64)
    ctype = ctypes.c_double if dt == np.float64 else ctypes.c_float
    arr = (ctypes.POINTER(ctype) * max(1, len(secs)))(*[_ptr(v, ctype) for v in secs])
    ext = np.array(grid["domain"] if grid else (1.0, 1.0, 1.0), dtype=np.float64)
    org = np.array(grid["origin"] if grid else (0.0, 0.0, 0.0), dtype=np.float64)
    fn = lib().gbgo_displace_f64 if dt == np.float64 else lib().gbgo_displace_f32
    fn(_ptr(dst, ctype), _ptr(src, ctype), m, len(secs), _ptr(coefs, ctypes.c_double), arr,
       1 if grid else 0, _ptr(ext, ctypes.c_double), _ptr(org, ctypes.c_double))
    return dst


def walk(base: int, neighbourhood: int, extent: int, width: int) -> np.ndarray:
    idx = np.zeros(width, dtype=np.int64)
    lib().gbgo_walk(base, neighbourhood, extent, width, _ptr(idx, ctypes.c_int64))
    return idx


def grid_dict(n, domain=(2 * np.pi,) * 3, origin=(0.0, 0.0, 0.0), dtype=np.float64):
    """A grid record as the reference's Grid3D{T} stores it (Fields.jl:165-200): the
    spacing is domain ./ T.(n) computed in the grid's element type T."""
    dt = np.dtype(dtype).type
    n = tuple(int(v) for v in n)
    dom = tuple(dt(v) for v in domain)
    org = tuple(dt(v) for v in origin)
    spacing = tuple(dt(d / dt(k)) for d, k in zip(dom, n))
    return {"n": n, "domain": tuple(float(v) for v in dom), "origin": tuple(float(v) for v in org),
            "spacing": tuple(float(v) for v in spacing), "dtype": np.dtype(dtype)}
