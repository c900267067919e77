"""Host-side mirror of the reference's transfer API, over the C ABI.

Names, argument meanings and error behaviour follow GBGPeriodicFields.jl:
  Grid3D                         src/Fields.jl:165-200
  Scalar/Vector/TensorFieldPhysical   src/Fields.jl:469-503, 623-660, 786-829
  PointSet, Scalar/Vector/TensorPointValues   src/Points.jl:124-240
  LalescuSpline, LagrangeSpline, CatmullRom   src/Interpolation.jl:227-424
  interpolate!, interpolate, field(x)         src/Interpolation.jl:1181-1235
  anterpolate!, anterpolate                   src/Interpolation.jl:1299-1350
  point_traversal_order(!), PointTraversalOrder(Scratch)   src/Interpolation.jl:519-980

Julia's bang functions are spelled with a trailing underscore (``interpolate_`` is
``interpolate!``).  Arrays are torch tensors on a CUDA device, held column-major like
the reference's (a (M, 3) PointSet has strides (1, M)).  The transfers are synchronous,
as the reference's are: each call synchronizes the current stream before it returns.
There is no CPU path: host tensors are refused.
"""
from __future__ import annotations

import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import ArgumentError, DimensionMismatch, InexactError

_DTYPE_CODE = {torch.float32: _lib.GBG_F32, torch.float64: _lib.GBG_F64}
_NP = {torch.float32: np.float32, torch.float64: np.float64}


def colmajor(t: torch.Tensor) -> torch.Tensor:
    """The tensor with column-major (Fortran) strides, copying only if needed."""
    if t.dim() <= 1:
        return t.contiguous()
    rev = tuple(range(t.dim() - 1, -1, -1))
    if t.permute(rev).is_contiguous():
        return t
    return t.permute(rev).contiguous().permute(rev)


def empty_colmajor(shape: Sequence[int], dtype, device) -> torch.Tensor:
    rev = tuple(range(len(shape) - 1, -1, -1))
    return torch.empty(tuple(reversed(tuple(shape))), dtype=dtype, device=device).permute(rev)


def zeros_colmajor(shape, dtype, device) -> torch.Tensor:
    t = empty_colmajor(shape, dtype, device)
    t.zero_()
    return t


# -------------------------------------------------------------------- grid


class Grid3D:
    """A periodic box of grid_size nodes (Fields.jl:165-200).  grid_spacing is stored and
    equals domain_size ./ T.(grid_size), computed in the element type T."""

    def __init__(self, grid_size, domain_size, origin=(0.0, 0.0, 0.0), dtype=torch.float64,
                 grid_spacing=None):
        if dtype not in _NP:
            raise ArgumentError(f"Grid3D element type must be float32 or float64, got {dtype}")
        T = _NP[dtype]
        gs = tuple(int(v) for v in grid_size)
        if len(gs) != 3 or any(v <= 0 for v in gs):
            raise ArgumentError(f"grid_size must be positive along every axis, got {tuple(grid_size)}")
        dom = tuple(T(v) for v in domain_size)
        if len(dom) != 3 or not all(np.isfinite(d) and d > 0 for d in dom):
            raise ArgumentError(f"domain_size must be finite and positive along every axis, got {tuple(domain_size)}")
        org = tuple(T(v) for v in origin)
        if len(org) != 3 or not all(np.isfinite(o) for o in org):
            raise ArgumentError(f"origin must be finite along every axis, got {tuple(origin)}")
        implied = tuple(T(d / T(n)) for d, n in zip(dom, gs))
        if grid_spacing is not None:
            sp = tuple(T(v) for v in grid_spacing)
            tol = math.sqrt(np.finfo(T).eps)
            if not all(abs(a - b) <= tol * max(abs(a), abs(b)) for a, b in zip(sp, implied)):
                raise ArgumentError(f"grid_spacing {sp} contradicts domain_size ./ grid_size = {implied}")
        else:
            sp = implied
        self.grid_size = gs
        self.domain_size = tuple(float(v) for v in dom)
        self.origin = tuple(float(v) for v in org)
        self.grid_spacing = tuple(float(v) for v in sp)
        self.dtype = dtype

    def __eq__(self, other):
        return (isinstance(other, Grid3D) and self.grid_size == other.grid_size
                and self.domain_size == other.domain_size and self.origin == other.origin
                and self.grid_spacing == other.grid_spacing and self.dtype == other.dtype)

    def __hash__(self):
        return hash((self.grid_size, self.domain_size, self.origin, self.dtype))

    def __repr__(self):
        return f"Grid3D({self.grid_size}, {self.domain_size}, origin={self.origin}, dtype={self.dtype})"

    @property
    def npoints(self) -> int:
        return self.grid_size[0] * self.grid_size[1] * self.grid_size[2]

    def c(self) -> _lib.GridC:
        g = _lib.GridC()
        for d in range(3):
            g.n[d] = self.grid_size[d]
            g.domain[d] = self.domain_size[d]
            g.spacing[d] = self.grid_spacing[d]
            g.origin[d] = self.origin[d]
        return g

    def node_coordinates(self, device="cpu"):
        """Per-axis node coordinates x0 + (i-1)*dx in the grid's element type
        (Fields.jl:484-503)."""
        T = _NP[self.dtype]
        return [torch.from_numpy(T(self.origin[d]) + np.arange(self.grid_size[d], dtype=T) * T(self.grid_spacing[d])).to(device)
                for d in range(3)]


# ----------------------------------------------------------------- schemes


class AbstractTransferScheme:
    """The supertype of the transfer schemes (the reference exports `AbstractTransferScheme`):
    the local splines, the NUFFT plan and the DirectDFT record are its subtypes."""


class _SplineScheme(AbstractTransferScheme):
    kind_name = "spline"

    def __init__(self, c: _lib.SchemeC):
        self._c = c
        self.stencil_width = int(c.stencil_width)

    @property
    def coefficients(self) -> np.ndarray:
        n2, m2 = self._c.stencil_width, self._c.num_powers
        flat = np.frombuffer(self._c.coefficients, dtype=np.float64)[: n2 * m2]
        return flat.reshape((n2, m2), order="F").copy()

    def axis_weights(self, t: float) -> np.ndarray:
        w = (ctypes_double_array(self.stencil_width))
        _lib.check(_lib.load().gbg_axis_weights(self._c, float(t), w), "axis weights")
        return np.array(w[:])

    def c(self):
        return self._c

    def __eq__(self, other):
        return type(self) is type(other) and np.array_equal(self.coefficients, other.coefficients)

    def __hash__(self):
        return hash((type(self).__name__, self.stencil_width))


def ctypes_double_array(n):
    import ctypes
    return (ctypes.c_double * n)()


class LalescuSpline(_SplineScheme):
    """Smooth C^m local spline (Interpolation.jl:244-258)."""

    def __init__(self, stencil_width: int, smoothness: Optional[int] = None):
        if smoothness is None:
            smoothness = int(stencil_width) // 2 - 1
        c = _lib.SchemeC()
        _lib.check(_lib.load().gbg_scheme_lalescu(int(stencil_width), int(smoothness), c), "LalescuSpline")
        super().__init__(c)
        self.smoothness = int(c.smoothness)

    def __repr__(self):
        return f"LalescuSpline({self.stencil_width}; smoothness={self.smoothness})"


class LagrangeSpline(_SplineScheme):
    """C^0 Lagrange interpolation over the stencil (Interpolation.jl:293-306)."""

    def __init__(self, stencil_width: int):
        c = _lib.SchemeC()
        _lib.check(_lib.load().gbg_scheme_lagrange(int(stencil_width), c), "LagrangeSpline")
        super().__init__(c)

    def __repr__(self):
        return f"LagrangeSpline({self.stencil_width})"


_CATMULL_ROM = None


def _catmull_rom():
    global _CATMULL_ROM
    if _CATMULL_ROM is None:
        _CATMULL_ROM = LalescuSpline(4)
    return _CATMULL_ROM


# ----------------------------------------------------------------- points


def Point(x, y, z, dtype=torch.float64) -> torch.Tensor:
    """One position as a 3-vector (Points.jl:107, `Point{T} = SVector{3, T}`), of the
    positions' real type; the callable field(x) and point sets take it."""
    if dtype not in (torch.float32, torch.float64):
        raise ArgumentError("Point: the coordinates are Float32 or Float64")
    return torch.tensor([float(x), float(y), float(z)], dtype=dtype)


def fiber_shape(R: int) -> tuple:
    """The per-point (or per-node) shape of a tensor of order R: (3,) * R
    (FiberSections.jl:1100-1108)."""
    R = int(R)
    if R < 0:
        raise ArgumentError("fiber_shape: the tensor order is a non-negative integer")
    return (3,) * R


class PointSet:
    """M positions, stored (M, 3) column-major (Points.jl:124-133)."""

    def __init__(self, positions: torch.Tensor):
        if not isinstance(positions, torch.Tensor) or positions.dim() != 2 or positions.shape[1] != 3:
            raise ArgumentError("a PointSet holds an (M, 3) array of positions")
        if positions.dtype not in _NP:
            raise ArgumentError(f"positions must be float32 or float64, got {positions.dtype}")
        self.positions = colmajor(positions)

    @property
    def npoints(self) -> int:
        return int(self.positions.shape[0])

    @property
    def dtype(self):
        return self.positions.dtype

    @property
    def device(self):
        return self.positions.device


class AbstractPointValues:
    tensor_order = 0

    def __init__(self, data: torch.Tensor, tensor_order: int):
        if data.dim() != 1 + tensor_order or any(s != 3 for s in data.shape[1:]):
            raise ArgumentError(f"point values of tensor order {tensor_order} are (M{', 3' * tensor_order}), got {tuple(data.shape)}")
        self.data = colmajor(data)
        self.tensor_order = tensor_order

    @property
    def npoints(self) -> int:
        return int(self.data.shape[0])

    @property
    def values(self) -> torch.Tensor:
        return self.data


def ScalarPointValues(data):
    return AbstractPointValues(data, 0)


def VectorPointValues(data):
    return AbstractPointValues(data, 1)


def TensorPointValues(data, R: int = 2):
    return AbstractPointValues(data, R)


def point_value_tensor_order(v: AbstractPointValues) -> int:
    """The tensor order R of point values (Points.jl:268-273)."""
    return int(v.tensor_order)


def similar_point_values(reference: AbstractPointValues, data_or_order=None) -> AbstractPointValues:
    """Point values shaped like `reference` (Points.jl:341-365): given an array, that array
    wrapped with the reference's tensor order; otherwise fresh (uninitialized) storage of
    (M, fiber_shape(R)...) -- R the order given, by default the reference's -- with the
    reference's element type and device."""
    if isinstance(data_or_order, torch.Tensor):
        return AbstractPointValues(data_or_order, reference.tensor_order)
    R = reference.tensor_order if data_or_order is None else int(data_or_order)
    data = empty_colmajor((npoints(reference),) + fiber_shape(R), reference.data.dtype, reference.data.device)
    return AbstractPointValues(data, R)


def point_values(v: AbstractPointValues) -> torch.Tensor:
    return v.data


def point_positions(p: PointSet) -> torch.Tensor:
    return p.positions


def npoints(x) -> int:
    return x.npoints


# ----------------------------------------------------------------- fields


class AbstractFieldPhysical:
    """A field in physical representation on a Grid3D: (Nx, Ny, Nz, 3^R...) column-major
    (Fields.jl:469-503, 623-660, 786-829)."""

    def __init__(self, data: torch.Tensor, grid: Grid3D, tensor_order: int):
        want = tuple(grid.grid_size) + (3,) * tensor_order
        if tuple(data.shape) != want:
            raise ArgumentError(f"field data of shape {tuple(data.shape)} does not match {want}")
        if data.dtype != grid.dtype:
            raise ArgumentError(f"field data is {data.dtype} but the grid is {grid.dtype}")
        self.data = colmajor(data)
        self.grid = grid
        self.tensor_order = tensor_order

    @property
    def ncomp(self) -> int:
        return 3 ** self.tensor_order

    def __call__(self, x, scheme=None):
        """The callable field(x): a one-point gather (Interpolation.jl:1229-1235)."""
        scheme = scheme or _catmull_rom()
        coords = empty_colmajor((1, 3), self.data.dtype, self.data.device)
        coords[0] = torch.tensor([float(v) for v in x[:3]], dtype=self.data.dtype)
        vals = interpolate(self, PointSet(coords), scheme)
        arr = vals.data.cpu().numpy()
        if self.tensor_order == 0:
            return arr[0].item()
        return arr[0]


def ScalarFieldPhysical(data, grid):
    return AbstractFieldPhysical(data, grid, 0)


def VectorFieldPhysical(data, grid):
    return AbstractFieldPhysical(data, grid, 1)


def TensorFieldPhysical(data, grid, R: int = 2):
    return AbstractFieldPhysical(data, grid, R)


def field_tensor_order(f) -> int:
    """The tensor order R of a field, physical or spectral (Fields.jl:349-350)."""
    return int(f.tensor_order)


def field_scalar_type(f) -> torch.dtype:
    """The real scalar type T of a field, physical or spectral (Fields.jl:341-342)."""
    return {torch.complex64: torch.float32, torch.complex128: torch.float64}.get(f.data.dtype, f.data.dtype)


def field_physical_shape(grid: Grid3D, R: int) -> tuple:
    """The storage shape of a field of tensor order R in physical space on `grid`:
    (grid_size..., fiber_shape(R)...) (Fields.jl:365-369)."""
    return tuple(grid.grid_size) + fiber_shape(R)


def similar_field(reference, data_or_order=None):
    """A field like `reference` (Fields.jl:1013-1070): given an array, that array wrapped as a
    field of the reference's kind (physical or spectral, with its grid and Fourier layout) and
    tensor order; otherwise fresh (uninitialized) storage of order R -- by default the
    reference's -- with the reference's element type and device."""
    from .nufft import AbstractFieldSpectral, field_spectral_shape
    spectral = isinstance(reference, AbstractFieldSpectral)
    if isinstance(data_or_order, torch.Tensor):
        if spectral:
            return AbstractFieldSpectral(data_or_order, reference.grid, reference.tensor_order, reference.layout)
        return AbstractFieldPhysical(data_or_order, reference.grid, reference.tensor_order)
    R = reference.tensor_order if data_or_order is None else int(data_or_order)
    dev, dt = reference.data.device, reference.data.dtype
    if spectral:
        data = empty_colmajor(field_spectral_shape(reference.grid, reference.layout, R), dt, dev)
        return AbstractFieldSpectral(data, reference.grid, R, reference.layout)
    return AbstractFieldPhysical(empty_colmajor(field_physical_shape(reference.grid, R), dt, dev), reference.grid, R)


def field_data(f: AbstractFieldPhysical) -> torch.Tensor:
    return f.data


def field_grid(f: AbstractFieldPhysical) -> Grid3D:
    return f.grid


def sample_field(fn, grid: Grid3D, tensor_order: int = 0, device="cuda"):
    """A field from a function sampled at the nodes x0 + (i-1)*dx (Fields.jl:484-503)."""
    xs, ys, zs = grid.node_coordinates("cpu")
    X, Y, Z = torch.meshgrid(xs, ys, zs, indexing="ij")
    vals = fn(X, Y, Z)
    if tensor_order == 0:
        data = torch.as_tensor(vals, dtype=grid.dtype)
    else:
        data = torch.stack([torch.as_tensor(v, dtype=grid.dtype) for v in vals], dim=-1)
        data = data.reshape(tuple(grid.grid_size) + (3,) * tensor_order)
    return AbstractFieldPhysical(colmajor(data).to(device), grid, tensor_order)


# --------------------------------------------------------- traversal order


class PointTraversalOrder:
    """A validated permutation of 1:M saying which point each unit of work handles
    (Interpolation.jl:519-531); the constructor refuses anything else."""

    def __init__(self, indices, _validated: bool = False):
        if isinstance(indices, range):
            indices = torch.tensor(list(indices), dtype=torch.int32)
        if not isinstance(indices, torch.Tensor):
            indices = torch.as_tensor(np.asarray(indices))
        if indices.dtype.is_floating_point or indices.dtype == torch.bool:
            raise ArgumentError(f"a point traversal order must hold integer indices, got {indices.dtype}")
        indices = indices.reshape(-1).to(torch.int32).contiguous()
        if not _validated:
            _validate_traversal(indices)
        self.indices = indices

    def __len__(self):
        return int(self.indices.numel())


def _validate_traversal(indices: torch.Tensor):
    """Interpolation.jl:560-589."""
    m = int(indices.numel())
    if m == 0:
        return
    if indices.is_cuda:
        import ctypes
        lo, hi, vis = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        with torch.cuda.device(indices.device):
            st = _lib.load().gbg_validate_traversal(
                indices.data_ptr(), m, ctypes.byref(lo), ctypes.byref(hi), ctypes.byref(vis),
                torch.cuda.current_stream().cuda_stream)
        _lib.check(st, "PointTraversalOrder")
        return
    a = indices.numpy().astype(np.int64)
    lo, hi = int(a.min()), int(a.max())
    if lo < 1 or hi > m:
        raise ArgumentError(f"a point traversal order must name points in 1:{m}, but it spans {lo}:{hi}")
    visited = np.unique(a).size
    if visited != m:
        raise ArgumentError(f"a point traversal order must name every point exactly once, but it names {visited} of {m}")


def _traversal_tiles(grid: Grid3D, tile_size: int):
    if tile_size < 1:
        raise ArgumentError(f"tile_size must be at least 1, got {tile_size}")
    return tuple(max(-(-n // tile_size), 1) for n in grid.grid_size)


def _check_order_precision(points: PointSet, grid: Grid3D):
    if points.dtype != grid.dtype:
        raise ArgumentError(f"the points hold {points.dtype} coordinates but the grid is {grid.dtype}; "
                            "a point traversal order is built for one precision and does not convert")


class PointTraversalOrderScratch:
    """Storage for point_traversal_order! so a rebuild allocates nothing that grows with
    the point count (Interpolation.jl:870-893)."""

    def __init__(self, grid: Grid3D, points: PointSet, tile_size: int = 4):
        _check_order_precision(points, grid)
        self.tiles = _traversal_tiles(grid, int(tile_size))
        self.tile_size = int(tile_size)
        self.grid = grid
        self.npoints = points.npoints
        import ctypes
        nbytes = ctypes.c_size_t()
        _lib.check(_lib.load().gbg_point_traversal_order_workspace_size(
            grid.c(), points.npoints, self.tile_size, ctypes.byref(nbytes)), "PointTraversalOrderScratch")
        self.workspace = torch.empty(max(int(nbytes.value), 1), dtype=torch.uint8, device=points.device)


def _build_order(indices: torch.Tensor, grid: Grid3D, points: PointSet, tile_size: int, workspace):
    _require_cuda(points.positions, "point_traversal_order")
    with torch.cuda.device(points.device):
        st = _lib.load().gbg_point_traversal_order(
            grid.c(), _DTYPE_CODE[points.dtype], points.positions.data_ptr(), points.npoints,
            int(tile_size), indices.data_ptr(),
            workspace.data_ptr() if workspace is not None else None,
            workspace.numel() if workspace is not None else 0,
            torch.cuda.current_stream().cuda_stream)
        _lib.check(st, "point_traversal_order")
        torch.cuda.current_stream().synchronize()


def point_traversal_order(grid: Grid3D, points: PointSet, tile_size: int = 4) -> PointTraversalOrder:
    """Interpolation.jl:816-833."""
    _check_order_precision(points, grid)
    _traversal_tiles(grid, int(tile_size))
    m = points.npoints
    indices = torch.empty(m, dtype=torch.int32, device=points.device)
    if m == 0:
        return PointTraversalOrder(indices, _validated=True)
    _build_order(indices, grid, points, tile_size, None)
    return PointTraversalOrder(indices)


def point_traversal_order_(traversal: PointTraversalOrder, grid: Grid3D, points: PointSet,
                           scratch: PointTraversalOrderScratch) -> PointTraversalOrder:
    """point_traversal_order! -- rebuild in place (Interpolation.jl:953-980)."""
    _check_order_precision(points, grid)
    m = points.npoints
    if len(traversal) != m:
        raise ArgumentError(f"the traversal names {len(traversal)} points but the set holds {m}; "
                            "a traversal is rebuilt for the set it was sized for")
    if scratch.npoints != m:
        raise ArgumentError(f"the scratch is sized for {scratch.npoints} points but the set holds {m}")
    if scratch.grid != grid:
        raise ArgumentError("the scratch was built for a different grid than this rebuild is using; a "
                            f"scratch fixes the block layout (tile_size {scratch.tile_size}, {scratch.tiles} blocks)")
    if m == 0:
        return traversal
    _build_order(traversal.indices, grid, points, scratch.tile_size, scratch.workspace)
    _validate_traversal(traversal.indices)
    return traversal


# -------------------------------------------------------------- transfers


def _require_cuda(t: torch.Tensor, what: str):
    if not t.is_cuda:
        raise ArgumentError(f"{what}: this implementation runs on a CUDA device only; got a host array "
                            "(there is no CPU path)")


def _check_colocation(field: AbstractFieldPhysical, points: PointSet, values: AbstractPointValues):
    """Interpolation.jl:1125-1138."""
    T = field.data.dtype
    if points.dtype != T:
        raise ArgumentError(f"point coordinates are {points.dtype} but the field is {T}; "
                            "a transfer does not convert between precisions")
    if values.data.dtype != T:
        raise ArgumentError(f"point values are {values.data.dtype} but the field is {T}")
    devs = {field.data.device, points.device, values.data.device}
    if len(devs) != 1:
        raise ArgumentError("a transfer launches one kernel, so its field, points and values must live in "
                            f"the same array family; got {sorted(str(d) for d in devs)}")
    _require_cuda(field.data, "transfer")


def _check_npoints_match(a, b):
    """Points.jl:301-305."""
    if a.npoints != b.npoints:
        raise DimensionMismatch(f"point counts differ: {a.npoints} and {b.npoints}")


def _check_traversal(traversal, m: int, device):
    """Interpolation.jl:596-615."""
    if traversal is None:
        return None
    if not isinstance(traversal, PointTraversalOrder):
        raise ArgumentError("a point traversal order must be a `PointTraversalOrder`, got "
                            f"{type(traversal).__name__}. Build one with `point_traversal_order(grid, points)`")
    if len(traversal) != m:
        raise ArgumentError(f"the point traversal order has {len(traversal)} entries but there are {m} points; "
                            "it must name every point exactly once")
    if traversal.indices.device != device:
        raise ArgumentError("the point traversal order is on a different array family than the field; build "
                            "it from the same point set with `point_traversal_order`, or move it")
    return traversal.indices


def _status_buffer(device):
    return torch.zeros(1, dtype=torch.int32, device=device)


def _raise_device_status(status: torch.Tensor):
    v = int(status.item())
    if v & _lib.GBG_DEV_NONFINITE:
        raise InexactError("a non-finite or out-of-range position reached the locate step "
                           "(floor(Int, x) of a non-finite coordinate)")
    if v & _lib.GBG_DEV_TRAVERSAL:
        raise ArgumentError("a traversal entry outside 1:M reached the device")


def interpolate_(out: AbstractPointValues, field: AbstractFieldPhysical, points: PointSet, scheme,
                 traversal: Optional[PointTraversalOrder] = None) -> AbstractPointValues:
    """interpolate! (Interpolation.jl:1181-1198): out = field sampled at points.  A
    field in spectral representation with a NUFFT scheme goes to the NUFFT path."""
    from . import nufft as _nufft
    if isinstance(scheme, (_nufft.NUFFT, _nufft.DirectDFT)) or isinstance(field, _nufft.AbstractFieldSpectral):
        return _nufft.dispatch_interpolate_(out, field, points, scheme, traversal)
    if out.tensor_order != field.tensor_order:
        raise ArgumentError(f"output tensor order {out.tensor_order} must equal field tensor order {field.tensor_order}")
    _check_npoints_match(out, points)
    _check_colocation(field, points, out)
    m = points.npoints
    trav = _check_traversal(traversal, m, field.data.device)
    if m == 0:
        return out
    status = _status_buffer(field.data.device)
    with torch.cuda.device(field.data.device):
        stream = torch.cuda.current_stream()
        st = _lib.load().gbg_interpolate(
            field.grid.c(), _DTYPE_CODE[field.data.dtype], field.ncomp, field.data.data_ptr(),
            points.positions.data_ptr(), m, trav.data_ptr() if trav is not None else None,
            scheme.c(), out.data.data_ptr(), status.data_ptr(), stream.cuda_stream)
        _lib.check(st, "interpolate!")
        stream.synchronize()
    _raise_device_status(status)
    return out


def interpolate(field: AbstractFieldPhysical, points: PointSet, scheme,
                traversal: Optional[PointTraversalOrder] = None) -> AbstractPointValues:
    """Allocating form of interpolate! (Interpolation.jl:1212-1217)."""
    from . import nufft as _nufft
    if isinstance(scheme, (_nufft.NUFFT, _nufft.DirectDFT)) or isinstance(field, _nufft.AbstractFieldSpectral):
        return _nufft.dispatch_interpolate(field, points, scheme, traversal)
    data = empty_colmajor((points.npoints,) + (3,) * field.tensor_order, field.data.dtype, points.device)
    return interpolate_(AbstractPointValues(data, field.tensor_order), field, points, scheme, traversal)


def anterpolate_(field: AbstractFieldPhysical, points: PointSet, quantities: AbstractPointValues, scheme,
                 alpha=None, beta=None, traversal: Optional[PointTraversalOrder] = None):
    """anterpolate! (Interpolation.jl:1299-1329): field = alpha*W^T q + beta*field, with
    beta == 0 overwriting.  alpha and beta come as a pair or not at all (1, 0)."""
    if (alpha is None) != (beta is None):
        raise ArgumentError("alpha and beta come as a pair or not at all")
    if alpha is None:
        alpha, beta = 1.0, 0.0
    from . import nufft as _nufft
    if isinstance(scheme, (_nufft.NUFFT, _nufft.DirectDFT)) or isinstance(field, _nufft.AbstractFieldSpectral):
        return _nufft.dispatch_anterpolate_(field, points, quantities, scheme, alpha, beta, traversal)
    if field.tensor_order != quantities.tensor_order:
        raise ArgumentError(f"field tensor order {field.tensor_order} must equal quantities tensor order {quantities.tensor_order}")
    _check_npoints_match(points, quantities)
    _check_colocation(field, points, quantities)
    m = points.npoints
    trav = _check_traversal(traversal, m, field.data.device)
    status = _status_buffer(field.data.device)
    import ctypes
    nbytes = ctypes.c_size_t()
    lib = _lib.load()
    _lib.check(lib.gbg_anterpolate_workspace_size(field.grid.c(), _DTYPE_CODE[field.data.dtype], field.ncomp,
                                                  m, scheme.c(), ctypes.byref(nbytes)), "anterpolate!")
    # scratch from torch's caching allocator, so repeated calls do not re-allocate
    ws = torch.empty(max(int(nbytes.value), 1), dtype=torch.uint8, device=field.data.device)
    with torch.cuda.device(field.data.device):
        stream = torch.cuda.current_stream()
        st = lib.gbg_anterpolate(
            field.grid.c(), _DTYPE_CODE[field.data.dtype], field.ncomp, field.data.data_ptr(),
            points.positions.data_ptr() if m else None, m,
            quantities.data.data_ptr() if m else None, trav.data_ptr() if trav is not None else None,
            scheme.c(), float(alpha), float(beta), ws.data_ptr(), ws.numel(), status.data_ptr(),
            stream.cuda_stream)
        _lib.check(st, "anterpolate!")
        stream.synchronize()
    _raise_device_status(status)
    return field


def anterpolate(grid: Grid3D, points: PointSet, quantities: AbstractPointValues, scheme,
                traversal: Optional[PointTraversalOrder] = None, layout=None) -> AbstractFieldPhysical:
    """Allocating form (Interpolation.jl:1344-1350): a fresh field in the quantities'
    array family (in spectral representation, in `layout` or the plan's, for a NUFFT)."""
    from . import nufft as _nufft
    if isinstance(scheme, _nufft.NUFFT):
        return _nufft.anterpolate_nufft(grid, points, quantities, scheme, layout=layout, traversal=traversal)
    R = quantities.tensor_order
    data = empty_colmajor(tuple(grid.grid_size) + (3,) * R, grid.dtype, quantities.data.device)
    return anterpolate_(AbstractFieldPhysical(data, grid, R), points, quantities, scheme, traversal=traversal)


# ------------------------------------------------------------ displacement


def _displace_terms(destination: PointSet, terms):
    """Points.jl:1286-1307: every section matches the point set's count, precision and
    array family; coefficients are real."""
    secs, coefs = [], []
    for term in terms:
        if not (isinstance(term, tuple) and len(term) == 2 and isinstance(term[1], AbstractPointValues)
                and term[1].tensor_order == 1):
            raise ArgumentError("a displacement term is a (coefficient, VectorPointValues) tuple")
        c, v = term
        if isinstance(c, complex) or not isinstance(c, (int, float)) or isinstance(c, bool):
            raise ArgumentError(f"a displacement coefficient must be real, got {type(c).__name__}")
        _check_npoints_match(destination, v)
        if v.data.dtype != destination.dtype:
            raise ArgumentError(f"a displacement section's scalar type {v.data.dtype} does not match the point "
                                f"set's {destination.dtype}; displacement does not convert between precisions")
        if v.data.device != destination.device:
            raise ArgumentError("a displacement section must live in the point set's array family")
        secs.append(v.data)
        coefs.append(float(c))
    return secs, coefs


def displace_(destination: PointSet, *args) -> PointSet:
    """displace! (Points.jl:1382-1440).  Forms, as in the reference:

        displace_(destination, source, (c1, v1), (c2, v2), ...)
        displace_(destination, source, grid, (c1, v1), ...)
        displace_(points, (c1, v1), ...)
        displace_(points, grid, (c1, v1), ...)

    Each coordinate becomes source + c1*v1 + c2*v2 + ... (products and sums rounded in the
    positions' type, left to right); with a grid the result is wrapped into
    [origin, origin + domain).  Returns destination."""
    args = list(args)
    source = destination
    if args and isinstance(args[0], PointSet):
        source = args.pop(0)
    grid = None
    if args and isinstance(args[0], Grid3D):
        grid = args.pop(0)
    _check_npoints_match(destination, source)
    if source.dtype != destination.dtype:
        raise ArgumentError(f"point-set scalar types differ: {destination.dtype} and {source.dtype}; "
                            "displacement does not convert between precisions")
    if source.device != destination.device:
        raise ArgumentError("point sets must live in the same array family")
    if grid is not None and grid.dtype != destination.dtype:
        raise ArgumentError(f"the domain's element type {grid.dtype} does not match the point set's "
                            f"{destination.dtype}; displacement does not convert between precisions")
    secs, coefs = _displace_terms(destination, args)
    _require_cuda(destination.positions, "displace!")
    m = destination.npoints
    if m == 0:
        return destination
    lib = _lib.load()
    import ctypes
    carr = (ctypes.c_double * max(1, len(coefs)))(*coefs)
    parr = (ctypes.c_void_p * max(1, len(secs)))(*[v.data_ptr() for v in secs])
    with torch.cuda.device(destination.device):
        stream = torch.cuda.current_stream()
        _lib.check(lib.gbg_points_displace(grid.c() if grid is not None else None, _DTYPE_CODE[destination.dtype],
                                           destination.positions.data_ptr(), source.positions.data_ptr(), m,
                                           len(secs), carr, parr, stream.cuda_stream), "displace!")
        stream.synchronize()
    return destination


def wrap_(points: PointSet, grid: Grid3D) -> PointSet:
    """wrap! (Points.jl:1481-1490): every coordinate reduced to [origin, origin + domain)."""
    return displace_(points, grid)
