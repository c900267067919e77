"""Resident precision form over the C ABI: GB300-owned field storage (FP32, ghost-padded,
components adjacent) and device cell-binned point sets, with the staged gather and the
deterministic scatter.  Positions may be Float64: they keep FP64 only for the periodic
wrap and the cell/fraction split."""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .api import Grid3D, _DTYPE_CODE, colmajor, empty_colmajor


def _stream():
    return torch.cuda.current_stream().cuda_stream


class ResidentField:
    """A field of ncomp components held on the device in the library's own layout
    (gbg_field_create)."""

    def __init__(self, grid: Grid3D, ncomp: int, max_stencil_width: int = 6):
        self.grid = grid
        self.ncomp = int(ncomp)
        self.max_stencil_width = int(max_stencil_width)
        h = ctypes.c_void_p()
        _lib.check(_lib.load().gbg_field_create(grid.c(), self.ncomp, _lib.GBG_F32, self.max_stencil_width,
                                                ctypes.byref(h)), "gbg_field_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().gbg_field_destroy(h)
            except Exception:
                pass
            self.handle = None

    @property
    def nbytes(self) -> int:
        n = ctypes.c_size_t()
        _lib.check(_lib.load().gbg_field_bytes(self.handle, ctypes.byref(n)))
        return int(n.value)

    def load(self, data: torch.Tensor):
        """Import a reference-layout (Nx, Ny, Nz, ncomp) array (Float32 or Float64); a host
        array is copied to the device first (the import kernel reads device memory)."""
        data = colmajor(data if data.is_cuda else data.cuda())
        if tuple(data.shape[:3]) != self.grid.grid_size or data.numel() != self.grid.npoints * self.ncomp:
            raise _lib.ArgumentError("field data does not match the resident field's shape")
        _lib.check(_lib.load().gbg_field_import(self.handle, _DTYPE_CODE[data.dtype], data.data_ptr(), _stream()),
                   "gbg_field_import")
        return self

    def read(self, dtype=torch.float64, device="cuda") -> torch.Tensor:
        """The field in the reference layout (Nx, Ny, Nz, ncomp), column-major, on `device`.
        The export kernel always writes device memory; a host result is copied from it
        after the kernel (a host pointer handed to the kernel would be written
        asynchronously where the GPU can address host memory, and read too early)."""
        dev = torch.device(device)
        out = empty_colmajor(self.grid.grid_size + (self.ncomp,), dtype, dev if dev.type == "cuda" else "cuda")
        _lib.check(_lib.load().gbg_field_export(self.handle, _DTYPE_CODE[dtype], out.data_ptr(), _stream()),
                   "gbg_field_export")
        return out if dev.type == "cuda" else out.to(dev)


class PointBins:
    """A device cell-binned sort of a point set (gbg_bins_create / gbg_bins_build)."""

    def __init__(self, grid: Grid3D, max_points: int, brick=None):
        self.grid = grid
        self.max_points = int(max_points)
        h = ctypes.c_void_p()
        br = (ctypes.c_int32 * 3)(*brick) if brick is not None else None
        _lib.check(_lib.load().gbg_bins_create(grid.c(), self.max_points, br, ctypes.byref(h)), "gbg_bins_create")
        self.handle = h
        self.npoints = 0
        self.status = None
        # the configuration a checkpoint records (the binned order itself is derived data)
        self.brick = tuple(int(v) for v in brick) if brick is not None else None
        self.gather_threads = self.scatter_threads = 0
        self.compensated = True

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().gbg_bins_destroy(h)
            except Exception:
                pass
            self.handle = None

    def build(self, positions: torch.Tensor, status: torch.Tensor | None = None):
        if not positions.is_cuda:
            raise _lib.ArgumentError("positions must be a CUDA tensor")
        positions = colmajor(positions)
        self.npoints = int(positions.shape[0])
        self.status = status
        _lib.check(_lib.load().gbg_bins_build(self.handle, _DTYPE_CODE[positions.dtype], positions.data_ptr(),
                                              self.npoints, status.data_ptr() if status is not None else None,
                                              _stream()), "gbg_bins_build")
        return self

    def nbricks_count(self) -> int:
        """Bricks covering the grid (the brick is the one given, or the library's default)."""
        import math
        brick = self.brick or (11, 8, 8)
        return math.prod(-(-n // b) for n, b in zip(self.grid.grid_size, brick))

    def set_launch(self, gather_threads: int = 0, scatter_threads: int = 0):
        """Threads per CTA of the binned gather and scatter (0 = default)."""
        _lib.check(_lib.load().gbg_bins_set_launch(self.handle, int(gather_threads), int(scatter_threads)),
                   "gbg_bins_set_launch")
        self.gather_threads, self.scatter_threads = int(gather_threads), int(scatter_threads)
        return self

    def build_displaced(self, dst: torch.Tensor, src: torch.Tensor, terms=(), wrap: bool = True,
                        status: torch.Tensor | None = None):
        """Move the points (dst = src + sum c_j v_j, wrapped onto the grid's box when wrap)
        and bin the moved points in the same pass (gbg_bins_build_displaced).  dst may be
        src; terms are (coefficient, (M, 3) tensor) pairs of the positions' dtype."""
        import ctypes
        src = colmajor(src)
        if not dst.is_cuda or dst.dtype != src.dtype or tuple(dst.shape) != tuple(src.shape):
            raise _lib.ArgumentError("dst must be a CUDA tensor shaped and typed like src")
        secs = [colmajor(v) for _, v in terms]
        if any(v.dtype != src.dtype or tuple(v.shape) != tuple(src.shape) for v in secs):
            raise _lib.ArgumentError("displacement sections must be (M, 3) tensors of the positions' dtype")
        carr = (ctypes.c_double * max(1, len(secs)))(*[float(c) for c, _ in terms])
        parr = (ctypes.c_void_p * max(1, len(secs)))(*[v.data_ptr() for v in secs])
        self.npoints = int(src.shape[0])
        self.status = status
        self._keep = secs
        _lib.check(_lib.load().gbg_bins_build_displaced(
            self.handle, _DTYPE_CODE[src.dtype], dst.data_ptr(), src.data_ptr(), self.npoints, len(secs), carr, parr,
            int(bool(wrap)), status.data_ptr() if status is not None else None, _stream()), "gbg_bins_build_displaced")
        return self

    def permute(self, src: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """An (M, ncols) array copied into the bins' sorted order (gbg_bins_permute)."""
        if not src.is_cuda or (out is not None and not out.is_cuda):
            raise _lib.ArgumentError("src and out must be CUDA tensors")
        src = colmajor(src)
        two = src if src.dim() == 2 else src.reshape(src.shape[0], -1)
        if out is None:
            out = empty_colmajor(tuple(src.shape), src.dtype, src.device)
        _lib.check(_lib.load().gbg_bins_permute(self.handle, _DTYPE_CODE[src.dtype], int(two.shape[1]), src.data_ptr(),
                                                out.data_ptr(), _stream()), "gbg_bins_permute")
        return out

    def set_compensated(self, on: bool = True):
        """Compensated summation of chunk partial sums in the binned scatter (the default) or
        one plain FP32 running sum per node (gbg_bins_set_compensated)."""
        _lib.check(_lib.load().gbg_bins_set_compensated(self.handle, int(bool(on))), "gbg_bins_set_compensated")
        self.compensated = bool(on)
        return self

    def set_sparse_regions(self, allow: bool = True):
        """Whether the binned scatter may take a sparse set's regions from the neighbouring
        bricks' point lists (the default) or always builds per-cell region tables; the
        results are the same bits (gbg_bins_set_sparse_regions)."""
        _lib.check(_lib.load().gbg_bins_set_sparse_regions(self.handle, int(bool(allow))), "gbg_bins_set_sparse_regions")
        return self

    def set_wait_limit(self, polls: int = 0):
        """Polls of a staged tile's barrier before the binned gather gives up on it (0 = the
        default; gbg_bins_set_wait_limit)."""
        _lib.check(_lib.load().gbg_bins_set_wait_limit(self.handle, int(polls)), "gbg_bins_set_wait_limit")
        return self

    def order(self) -> torch.Tensor:
        o = torch.empty(self.npoints, dtype=torch.int32, device="cuda")
        _lib.check(_lib.load().gbg_bins_order(self.handle, o.data_ptr(), _stream()), "gbg_bins_order")
        return o


def build_bins(pairs, status: torch.Tensor | None = None):
    """Builds many PointBins at once, each from its own positions: [(bins, positions), ...]
    (gbg_bins_build_batch).  Independent bins build concurrently on the library's side
    streams; the result is what bins.build(positions) gives for each."""
    pairs = [(b, colmajor(p)) for b, p in pairs]
    n = len(pairs)
    if n == 0:
        return []
    handles = (ctypes.c_void_p * n)(*[b.handle.value for b, _ in pairs])
    dtypes = (ctypes.c_int32 * n)(*[_DTYPE_CODE[p.dtype] for _, p in pairs])
    ptrs = (ctypes.c_void_p * n)(*[p.data_ptr() for _, p in pairs])
    counts = (ctypes.c_int64 * n)(*[int(p.shape[0]) for _, p in pairs])
    for b, p in pairs:
        b.npoints = int(p.shape[0])
        b.status = status
    _lib.check(_lib.load().gbg_bins_build_batch(handles, dtypes, ptrs, counts, n,
                                                status.data_ptr() if status is not None else None, _stream()),
               "gbg_bins_build_batch")
    return [b for b, _ in pairs]


def interpolate_binned(field: ResidentField, bins: PointBins, scheme, out: torch.Tensor | None = None,
                       dtype=torch.float32, status: torch.Tensor | None = None) -> torch.Tensor:
    if out is None:
        out = empty_colmajor((bins.npoints, field.ncomp), dtype, "cuda")
    _lib.check(_lib.load().gbg_interpolate_binned(field.handle, bins.handle, scheme.c(), _DTYPE_CODE[out.dtype],
                                                  out.data_ptr(), status.data_ptr() if status is not None else None,
                                                  _stream()), "gbg_interpolate_binned")
    return out


def anterpolate_binned(field: ResidentField, bins: PointBins, scheme, q: torch.Tensor, alpha=1.0, beta=0.0,
                       status: torch.Tensor | None = None):
    q = colmajor(q)
    _lib.check(_lib.load().gbg_anterpolate_binned(field.handle, bins.handle, scheme.c(), _DTYPE_CODE[q.dtype],
                                                  q.data_ptr(), float(alpha), float(beta),
                                                  status.data_ptr() if status is not None else None, _stream()),
               "gbg_anterpolate_binned")
    return field


class Batch:
    """Many independent instances in one persistent gather launch and one persistent scatter
    launch (gbg_batch_create / gbg_batch_run).  Each instance is a dict with keys field,
    bins, scheme and optionally out (FP32 (M, ncomp)), dest (ResidentField), q (FP32
    (M, ncomp)), alpha, beta.  The batch records each instance's point count and device
    arrays at creation; rebuilding the bins with the same point count keeps it valid."""

    def __init__(self, instances):
        items = (_lib.BatchItemC * len(instances))()
        self._keep = []
        for i, inst in enumerate(instances):
            it = items[i]
            it.field = inst["field"].handle
            it.bins = inst["bins"].handle
            it.scheme = inst["scheme"].c()
            out = inst.get("out")
            it.out = out.data_ptr() if out is not None else None
            dest = inst.get("dest")
            it.dest = dest.handle if dest is not None else None
            q = inst.get("q")
            if q is not None:
                q = colmajor(q)
                self._keep.append(q)
            it.q = q.data_ptr() if q is not None else None
            it.alpha = float(inst.get("alpha", 1.0))
            it.beta = float(inst.get("beta", 0.0))
        self.instances = instances
        h = ctypes.c_void_p()
        _lib.check(_lib.load().gbg_batch_create(items, len(instances), ctypes.byref(h)), "gbg_batch_create")
        self.handle = h

    def run(self, status: torch.Tensor | None = None):
        _lib.check(_lib.load().gbg_batch_run(self.handle, status.data_ptr() if status is not None else None,
                                             _stream()), "gbg_batch_run")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().gbg_batch_destroy(h)
            except Exception:
                pass
            self.handle = None
