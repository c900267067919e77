"""Spectral fields and the NUFFT transfer scheme over the C ABI.

Mirrors of the reference:
  RealFourierLayout, field_spectral_shape        src/Fields.jl:204-239, 388
  Scalar/Vector/TensorFieldSpectral              src/Fields.jl:420-441 (spectral storage)
  FieldTransformPlans, to_spectral, to_physical  the unnormalized forward real FFT and its
                                                 1/N inverse (the convention DirectDFT states,
                                                 src/Interpolation.jl:1386-1404)
  NUFFT (plan, width and shape rules)            src/Interpolation.jl:1652-1860
  interpolate!/anterpolate! with a NUFFT         src/Interpolation.jl:1984-2062

A NUFFT transfer is spread/gather on an oversampled (sigma*N) grid with the exponential-of-
semicircle window (the device kernels gbg_nufft_spread / gbg_nufft_interp), the real FFT of
that grid (cuFFT, through torch.fft), the exchange of the modes the two grids share, and
the division by the window's transform.  Type 2 (interpolate): deconvolve, embed the
reference modes (times sigma^3) into the zero oversampled spectrum, inverse FFT, gather.
Type 1 (anterpolate): spread, forward FFT, take the shared modes (over sigma^3),
deconvolve, times sigma^3.  An even axis's Nyquist mode is projected out (its deconvolution
factor is 0), which makes the two exact adjoints on the resolved band.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._lib import ArgumentError, DimensionMismatch, MethodError
from .api import (AbstractPointValues, AbstractTransferScheme, Grid3D, PointSet, PointTraversalOrder, _DTYPE_CODE, _check_npoints_match,
                  _check_traversal, _raise_device_status, _require_cuda, _status_buffer, colmajor, empty_colmajor)

_COMPLEX = {torch.float32: torch.complex64, torch.float64: torch.complex128}
_REAL = {torch.complex64: torch.float32, torch.complex128: torch.float64}
MAX_WINDOW_WIDTH = 16


# ------------------------------------------------------------------ layout


class RealFourierLayout:
    """The real-FFT layout (Fields.jl:204-224): fft_dims is a permutation of (1, 2, 3)
    (1-based, as in the reference); axis fft_dims[1] is stored halved, N//2 + 1 long."""

    def __init__(self, fft_dims=(1, 2, 3)):
        d = tuple(int(v) for v in fft_dims)
        if len(d) != 3 or sorted(d) != [1, 2, 3]:
            raise ArgumentError(f"fft_dims must be a permutation of (1, 2, 3), got {tuple(fft_dims)}")
        self.fft_dims = d

    @property
    def half_axis(self) -> int:
        """The halved axis, 0-based."""
        return self.fft_dims[0] - 1

    def __eq__(self, other):
        return isinstance(other, RealFourierLayout) and self.fft_dims == other.fft_dims

    def __hash__(self):
        return hash(self.fft_dims)

    def __repr__(self):
        return f"RealFourierLayout({self.fft_dims})"


def rfft_shape(grid_size, layout: RealFourierLayout):
    """Fields.jl:239 -- _rfft_shape."""
    h = layout.half_axis
    return tuple(n // 2 + 1 if d == h else n for d, n in enumerate(grid_size))


def field_spectral_shape(grid: Grid3D, layout: RealFourierLayout, tensor_order: int):
    """Fields.jl:388."""
    return rfft_shape(grid.grid_size, layout) + (3,) * tensor_order


# ------------------------------------------------------------- spectral fields


class AbstractFieldSpectral:
    """A field in spectral representation: the stored rfft half-spectrum, complex,
    (stored spatial shape..., 3^R...) column-major."""

    def __init__(self, data: torch.Tensor, grid: Grid3D, tensor_order: int, layout: Optional[RealFourierLayout] = None):
        layout = layout or RealFourierLayout()
        want = field_spectral_shape(grid, layout, tensor_order)
        if tuple(data.shape) != want:
            raise ArgumentError(f"spectral field data of shape {tuple(data.shape)} does not match {want}")
        if data.dtype != _COMPLEX[grid.dtype]:
            raise ArgumentError(f"spectral field data is {data.dtype} but the grid wants {_COMPLEX[grid.dtype]}")
        self.data = colmajor(data)
        self.grid = grid
        self.tensor_order = tensor_order
        self.layout = layout

    @property
    def ncomp(self) -> int:
        return 3 ** self.tensor_order


def ScalarFieldSpectral(data, grid, layout=None):
    return AbstractFieldSpectral(data, grid, 0, layout)


def VectorFieldSpectral(data, grid, layout=None):
    return AbstractFieldSpectral(data, grid, 1, layout)


def TensorFieldSpectral(data, grid, R: int = 2, layout=None):
    return AbstractFieldSpectral(data, grid, R, layout)


def field_layout(f: AbstractFieldSpectral) -> RealFourierLayout:
    return f.layout


def zeros_spectral(grid: Grid3D, tensor_order: int = 0, layout: Optional[RealFourierLayout] = None, device="cuda"):
    layout = layout or RealFourierLayout()
    t = empty_colmajor(field_spectral_shape(grid, layout, tensor_order), _COMPLEX[grid.dtype], device)
    t.zero_()
    return AbstractFieldSpectral(t, grid, tensor_order, layout)


# ------------------------------------------------------------- transforms


def _fft_dims(layout: RealFourierLayout):
    """torch's real FFT halves the last dimension it is given: the half axis goes last."""
    h = layout.half_axis
    return tuple(d for d in range(3) if d != h) + (h,)


class FieldTransformPlans:
    """The pair of transforms between a physical field and its spectral representation.
    cuFFT keeps its own plan cache, so this holds only the context it was made for."""

    def __init__(self, physical, spectral: AbstractFieldSpectral):
        if physical.grid != spectral.grid or physical.tensor_order != spectral.tensor_order:
            raise ArgumentError("transform plans need a physical and a spectral field of one grid and tensor order")
        self.grid = spectral.grid
        self.layout = spectral.layout
        self.tensor_order = spectral.tensor_order


def _fft_forward(data: torch.Tensor, layout: RealFourierLayout) -> torch.Tensor:
    return colmajor(torch.fft.rfftn(data, dim=_fft_dims(layout)))


def _fft_inverse(data: torch.Tensor, grid_size, layout: RealFourierLayout) -> torch.Tensor:
    dims = _fft_dims(layout)
    return colmajor(torch.fft.irfftn(data, s=tuple(grid_size[d] for d in dims), dim=dims))


def to_spectral(physical, plans: Optional[FieldTransformPlans] = None, layout: Optional[RealFourierLayout] = None):
    """The unnormalized forward transform: f_hat(k) = sum_x f(x) exp(-i k.(x - o))."""
    layout = plans.layout if plans is not None else (layout or RealFourierLayout())
    return AbstractFieldSpectral(_fft_forward(physical.data, layout), physical.grid, physical.tensor_order, layout)


def to_physical(spectral: AbstractFieldSpectral, plans: Optional[FieldTransformPlans] = None):
    """The inverse, f(x) = (1/N) sum_k f_hat(k) exp(i k.(x - o)); the real transform keeps
    the Hermitian part of the self-conjugate modes."""
    from .api import AbstractFieldPhysical
    data = _fft_inverse(spectral.data, spectral.grid.grid_size, spectral.layout)
    return AbstractFieldPhysical(data, spectral.grid, spectral.tensor_order)


def _check_matches_plans(field, plans: FieldTransformPlans):
    """_check_field_matches_context (Fields.jl:1295-1305): the field was made for the plans'
    grid (and, spectral, Fourier layout), with their tensor order."""
    if field.grid != plans.grid:
        raise ArgumentError("field grid must be equal to FieldTransformPlans grid")
    if isinstance(field, AbstractFieldSpectral) and field.layout != plans.layout:
        raise ArgumentError("field Fourier layout must be equal to FieldTransformPlans Fourier layout")
    if field.tensor_order != plans.tensor_order:
        raise ArgumentError("field tensor order must be equal to FieldTransformPlans tensor order")


def _check_pair_precision(physical, spectral):
    want = {torch.float32: torch.complex64, torch.float64: torch.complex128}.get(physical.data.dtype)
    if spectral.data.dtype != want:
        raise ArgumentError("the physical and spectral fields must have one scalar type")


def to_physical_(physical, spectral: AbstractFieldSpectral, plans: FieldTransformPlans,
                 spectral_scratch: Optional[AbstractFieldSpectral] = None):
    """to_physical! (Fields.jl:1546-1620): the inverse transform written into `physical`.  With
    `spectral_scratch` the coefficients are copied there first and `spectral` is left as it
    was (the scratch may not share `spectral`'s storage); without it the source may serve as
    the transform's scratch (here it is left unchanged as well)."""
    _check_matches_plans(physical, plans)
    _check_matches_plans(spectral, plans)
    _check_pair_precision(physical, spectral)
    src = spectral.data
    if spectral_scratch is not None:
        _check_matches_plans(spectral_scratch, plans)
        if spectral_scratch.data.data_ptr() == spectral.data.data_ptr():
            raise ArgumentError("spectral_scratch must not alias spectral: a shared array would let the "
                                "transform consume the source this argument exists to preserve")
        spectral_scratch.data.copy_(spectral.data)
        src = spectral_scratch.data
    physical.data.copy_(_fft_inverse(src, spectral.grid.grid_size, spectral.layout))
    return physical


def to_spectral_(spectral: AbstractFieldSpectral, physical, plans: FieldTransformPlans):
    """to_spectral! (Fields.jl:1623-1657): the forward transform written into `spectral`."""
    _check_matches_plans(spectral, plans)
    _check_matches_plans(physical, plans)
    _check_pair_precision(physical, spectral)
    spectral.data.copy_(_fft_forward(physical.data, spectral.layout))
    return spectral


def _shared_axis(n_coarse: int, n_fine: int, folded: bool, device):
    """One axis of the modes a coarse and a fine grid over one box share (Fields.jl:3157-3185):
    the coarse stored indices kept and the fine stored indices of the same frequencies.  A full
    axis stores frequencies 0, 1, ..., then the negative ones (fftfreq order); the folded axis
    stores 0 .. N//2.  The coarse Nyquist mode of an even axis is left out: the fine grid holds
    +N/2 and -N/2 apart where the coarse grid holds one sampled wave."""
    stored = n_coarse // 2 + 1 if folded else n_coarse
    coarse, fine = [], []
    for i in range(stored):
        if n_coarse % 2 == 0 and i == n_coarse // 2:
            continue
        if folded:
            coarse.append(i)
            fine.append(i)
            continue
        freq = i if i < (n_coarse + 1) // 2 else i - n_coarse
        coarse.append(i)
        fine.append(freq if freq >= 0 else n_fine + freq)
    return (torch.tensor(coarse, dtype=torch.long, device=device), torch.tensor(fine, dtype=torch.long, device=device))


def _check_shared_modes(coarse: AbstractFieldSpectral, fine: AbstractFieldSpectral):
    """_check_shared_mode_compatibility (Fields.jl:3287-3310): one scalar type, tensor order,
    device, box and Fourier layout; the coarse grid no larger on any axis and not equal."""
    if coarse.data.dtype != fine.data.dtype:
        raise ArgumentError("field scalar types must be equal")
    if coarse.tensor_order != fine.tensor_order:
        raise ArgumentError("field tensor orders must be equal")
    if coarse.data.device != fine.data.device:
        raise ArgumentError(f"fields must live on one device; got {coarse.data.device} and {fine.data.device}")
    cg, fg = coarse.grid, fine.grid
    if tuple(cg.domain_size) != tuple(fg.domain_size) or tuple(cg.origin) != tuple(fg.origin):
        raise ArgumentError(f"fields must cover the same box; got domain size {cg.domain_size} at origin "
                            f"{cg.origin} and {fg.domain_size} at {fg.origin}")
    if coarse.layout != fine.layout:
        raise ArgumentError("field Fourier layouts must be equal")
    if any(c > f for c, f in zip(cg.grid_size, fg.grid_size)):
        raise ArgumentError(f"the coarse grid {cg.grid_size} must be no larger than the fine grid {fg.grid_size} on any axis")
    if tuple(cg.grid_size) == tuple(fg.grid_size):
        raise ArgumentError(f"the two grids are equal ({cg.grid_size}); moving between grid resolutions needs "
                            "a coarser and a finer field, and two fields on one grid combine by addition")


def _shared_modes(destination: AbstractFieldSpectral, source: AbstractFieldSpectral, to_fine: bool, alpha, beta):
    """The body both resolution verbs share (Fields.jl:3329-3355): destination = alpha' * source
    on the shared modes (beta == 0), else beta * destination + alpha' * source, where alpha'
    is alpha times the ratio of the destination's to the source's point count in the fields'
    real type (stored coefficients are point count x physical amplitude); no other mode is
    read or written."""
    coarse, fine = (source, destination) if to_fine else (destination, source)
    _check_shared_modes(coarse, fine)
    real = torch.float32 if destination.data.dtype == torch.complex64 else torch.float64
    ratio = math.prod(destination.grid.grid_size) / math.prod(source.grid.grid_size)
    scale = float(torch.tensor(float(alpha), dtype=real) * torch.tensor(ratio, dtype=real))
    b = float(torch.tensor(float(beta), dtype=real))
    h = coarse.layout.half_axis
    dev = destination.data.device
    axes = [_shared_axis(coarse.grid.grid_size[d], fine.grid.grid_size[d], d == h, dev) for d in range(3)]
    ci = [ax[0] for ax in axes]
    fi = [ax[1] for ax in axes]
    grid = lambda idx: (idx[0][:, None, None], idx[1][None, :, None], idx[2][None, None, :])
    di, si = (grid(fi), grid(ci)) if to_fine else (grid(ci), grid(fi))
    src = source.data[si]
    if b == 0.0:
        destination.data[di] = scale * src
    else:
        destination.data[di] = b * destination.data[di] + scale * src
    return destination


def embed_modes_(destination: AbstractFieldSpectral, source: AbstractFieldSpectral, alpha=1, beta=0):
    """embed_modes! (Fields.jl:3360-3405): a coarser field's modes written into a finer one over
    the same box (added when beta is nonzero), physical amplitudes kept; the fine field's other
    modes, and the coarse grid's even-axis Nyquist modes, are left alone."""
    return _shared_modes(destination, source, True, alpha, beta)


def extract_modes_(destination: AbstractFieldSpectral, source: AbstractFieldSpectral, alpha=1, beta=0):
    """extract_modes! (Fields.jl:3408-3446): a finer field's modes the coarser destination can
    hold read into it, physical amplitudes kept; the destination's other modes (its even-axis
    Nyquist modes among them) are left as they were."""
    return _shared_modes(destination, source, False, alpha, beta)


# ------------------------------------------------------------------ NUFFT


def nufft_width(tolerance) -> int:
    """Interpolation.jl:1670-1676 -- _nufft_width: max(4, ceil(-log10(tol)) + 2).  This
    build's kernels take at most 16 nodes, the width the rule gives at tolerance 1e-14,
    where Float64's own resolution is reached; a derived width is capped there."""
    tol = float(tolerance)
    if not (math.isfinite(tol) and tol > 0):
        raise ArgumentError(f"NUFFT tolerance must be finite and positive; got {tolerance}")
    return min(MAX_WINDOW_WIDTH, max(4, math.ceil(-math.log10(tol)) + 2))


def nufft_beta(width: int, dtype) -> float:
    """Interpolation.jl:1677 -- _nufft_beta: T(23)/10 * width, in T."""
    T = np.float32 if dtype == torch.float32 else np.float64
    return float(T(T(23) / T(10) * T(width)))


def _shared_slices(n: int, nf: int, is_half: bool):
    """The modes the reference axis (n) shares with the oversampled one (nf): pairs of
    (reference slice, oversampled slice); an even axis's Nyquist mode is not shared."""
    if is_half:
        k = (n + 1) // 2
        return [(slice(0, k), slice(0, k))]
    pos = (n + 1) // 2
    neg = n - n // 2 - 1
    pairs = [(slice(0, pos), slice(0, pos))]
    if neg > 0:
        pairs.append((slice(n - neg, n), slice(nf - neg, nf)))
    return pairs


class NUFFT(AbstractTransferScheme):
    """The fast spectral transfer scheme (Interpolation.jl:1718-1860).

    NUFFT(reference_spectral_field; tolerance=1e-10, oversampling=2, window_width=None,
    window_shape=None), or NUFFT.for_grid(grid, tensor_order, device=..., layout=...,
    ...) when no field is at hand.  The plan holds the window (width W, shape beta), the
    oversampled grid (sigma*N, same box and origin) and the deconvolution on the
    reference grid's stored modes."""

    def __init__(self, reference: AbstractFieldSpectral, tolerance=1e-10, oversampling=2, window_width=None,
                 window_shape=None):
        if not isinstance(reference, AbstractFieldSpectral):
            raise MethodError("NUFFT(reference) takes a field in spectral representation")
        self._build(reference.grid, reference.layout, reference.tensor_order, reference.data.device, tolerance,
                    oversampling, window_width, window_shape)

    @classmethod
    def for_grid(cls, grid: Grid3D, tensor_order: int, device="cuda", layout: Optional[RealFourierLayout] = None,
                 tolerance=1e-10, oversampling=2, window_width=None, window_shape=None):
        self = cls.__new__(cls)
        self._build(grid, layout or RealFourierLayout(), int(tensor_order), torch.device(device), tolerance,
                    oversampling, window_width, window_shape)
        return self

    def _build(self, grid, layout, R, device, tolerance, oversampling, window_width, window_shape):
        # the width default is evaluated first, so a bad tolerance is refused there too
        if window_width is None:
            window_width = nufft_width(tolerance)
        if window_shape is None:
            window_shape = nufft_beta(int(window_width), grid.dtype)
        tol = float(tolerance)
        if not (math.isfinite(tol) and tol > 0):
            raise ArgumentError(f"NUFFT tolerance must be finite and positive; got {tolerance}")
        sigma = int(oversampling)
        if sigma < 2:
            raise ArgumentError(f"NUFFT oversampling must be at least 2 (got {sigma}): with no oversampling the work "
                                "grid has no spectral guard band")
        if int(window_width) <= 0:
            raise ArgumentError(f"NUFFT window_width must be a positive number of nodes; got {window_width}")
        ws = float(window_shape)
        if not (math.isfinite(ws) and ws > 0):
            raise ArgumentError(f"NUFFT window_shape must be finite and positive; got {window_shape}")
        if int(window_width) > MAX_WINDOW_WIDTH:
            raise _lib.GBGError(_lib.GBG_EUNSUPPORTED, f"NUFFT window_width {window_width}: this build's window "
                                f"kernels take at most {MAX_WINDOW_WIDTH} nodes")
        T = np.float32 if grid.dtype == torch.float32 else np.float64
        self.width = int(window_width)
        self.beta = float(T(ws))
        self.oversampling = sigma
        self.reference_grid = grid
        self.reference_layout = layout
        self.tensor_order = R
        self.dtype = grid.dtype
        self.device = device
        self.oversampled_grid = Grid3D(tuple(sigma * n for n in grid.grid_size), grid.domain_size, origin=grid.origin,
                                       dtype=grid.dtype)
        self.total_oversampling = float(T(np.prod(self.oversampled_grid.grid_size) / np.prod(grid.grid_size)))
        # the deconvolution on the reference grid's stored modes (outer product of the axes)
        lib = _lib.load()
        axes = []
        for d in range(3):
            n = grid.grid_size[d]
            is_half = d == layout.half_axis
            buf = (ctypes.c_double * (n // 2 + 1 if is_half else n))()
            _lib.check(lib.gbg_nufft_deconvolution_axis(n, int(is_half), sigma, self.width, self.beta,
                                                        _DTYPE_CODE[grid.dtype], buf), "NUFFT")
            axes.append(np.asarray(buf, dtype=T))
        dec = axes[0][:, None, None] * axes[1][None, :, None] * axes[2][None, None, :]
        self.deconvolution = colmajor(torch.from_numpy(np.ascontiguousarray(dec.astype(T))).to(device))

    def __repr__(self):
        return (f"NUFFT(width={self.width}, beta={self.beta}, oversampling={self.oversampling}, "
                f"grid={self.reference_grid}, layout={self.reference_layout})")

    # the modes the two grids share, per axis
    def _pairs(self):
        h = self.reference_layout.half_axis
        return [_shared_slices(self.reference_grid.grid_size[d], self.oversampled_grid.grid_size[d], d == h)
                for d in range(3)]

    def _dec(self, R):
        return self.deconvolution.reshape(self.deconvolution.shape + (1,) * R)


def _check_nufft_compatibility(scheme: NUFFT, field: AbstractFieldSpectral):
    """Interpolation.jl:1971-1985."""
    if scheme.reference_grid != field.grid or scheme.reference_layout != field.layout:
        raise ArgumentError("this NUFFT plan was built for another grid or Fourier layout than the field's")
    if scheme.dtype != field.grid.dtype:
        raise ArgumentError(f"this NUFFT plan was built for scalar type {scheme.dtype}, but the field carries "
                            f"{field.grid.dtype}")
    if torch.device(scheme.device) != field.data.device:
        raise ArgumentError("this NUFFT plan holds work buffers in a different array family than the field")
    if scheme.tensor_order != field.tensor_order:
        raise ArgumentError(f"this NUFFT plan was built at tensor order {scheme.tensor_order}; it cannot transfer a "
                            f"field of order {field.tensor_order}")


def _check_colocation_spectral(field: AbstractFieldSpectral, points: PointSet, values: AbstractPointValues):
    """Interpolation.jl:1125-1138 for a spectral field (its scalar type is the grid's)."""
    T = field.grid.dtype
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


def interpolate_nufft_(out: AbstractPointValues, field: AbstractFieldSpectral, points: PointSet, scheme: NUFFT,
                       traversal: Optional[PointTraversalOrder] = None) -> AbstractPointValues:
    """interpolate! with a NUFFT (Interpolation.jl:1984-2010), type 2."""
    trav = _check_traversal(traversal, out.npoints, field.data.device)
    _check_nufft_compatibility(scheme, field)
    if out.tensor_order != field.tensor_order:
        raise ArgumentError(f"output tensor order {out.tensor_order} must equal field tensor order {field.tensor_order}")
    _check_npoints_match(out, points)
    _check_colocation_spectral(field, points, out)
    R, m = field.tensor_order, points.npoints
    fine = scheme.oversampled_grid
    layout = scheme.reference_layout
    coarse = field.data * scheme._dec(R)
    spec = torch.zeros(field_spectral_shape(fine, layout, R), dtype=field.data.dtype, device=field.data.device)
    px, py, pz = scheme._pairs()
    for cx, fx in px:
        for cy, fy in py:
            for cz, fz in pz:
                spec[fx, fy, fz] = coarse[cx, cy, cz] * scheme.total_oversampling
    phys = _fft_inverse(spec, fine.grid_size, layout)
    if m == 0:
        return out
    status = _status_buffer(field.data.device)
    lib = _lib.load()
    nbytes = ctypes.c_size_t()
    _lib.check(lib.gbg_nufft_interp_workspace_size(fine.c(), _DTYPE_CODE[fine.dtype], field.ncomp, m, scheme.width,
                                                   ctypes.byref(nbytes)), "interpolate!")
    ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=field.data.device)
    with torch.cuda.device(field.data.device):
        stream = torch.cuda.current_stream()
        st = lib.gbg_nufft_interp(fine.c(), _DTYPE_CODE[fine.dtype], field.ncomp, phys.data_ptr(),
                                  points.positions.data_ptr(), m,
                                  trav.data_ptr() if trav is not None else None, scheme.width, scheme.beta,
                                  out.data.data_ptr(), ws.data_ptr(), ws.numel(), status.data_ptr(),
                                  stream.cuda_stream)
        _lib.check(st, "interpolate!")
        stream.synchronize()
    _raise_device_status(status)
    return out


def anterpolate_nufft_(field: AbstractFieldSpectral, points: PointSet, quantities: AbstractPointValues,
                       scheme: NUFFT, alpha=1.0, beta=0.0, traversal: Optional[PointTraversalOrder] = None):
    """anterpolate! with a NUFFT (Interpolation.jl:2021-2062), type 1: field = alpha *
    (W^T q) + beta * field, beta == 0 overwriting."""
    trav = _check_traversal(traversal, quantities.npoints, field.data.device)
    _check_nufft_compatibility(scheme, field)
    if field.tensor_order != quantities.tensor_order:
        raise ArgumentError(f"field tensor order {field.tensor_order} must equal quantities tensor order "
                            f"{quantities.tensor_order}")
    _check_npoints_match(points, quantities)
    _check_colocation_spectral(field, points, quantities)
    R, m = field.tensor_order, points.npoints
    fine = scheme.oversampled_grid
    layout = scheme.reference_layout
    dev = field.data.device
    phys = empty_colmajor(tuple(fine.grid_size) + (3,) * R, fine.dtype, dev)
    lib = _lib.load()
    nbytes = ctypes.c_size_t()
    _lib.check(lib.gbg_nufft_spread_workspace_size(fine.c(), _DTYPE_CODE[fine.dtype], field.ncomp, m, scheme.width,
                                                   ctypes.byref(nbytes)), "anterpolate!")
    ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=dev)
    status = _status_buffer(dev)
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream()
        st = lib.gbg_nufft_spread(fine.c(), _DTYPE_CODE[fine.dtype], field.ncomp, phys.data_ptr(),
                                  points.positions.data_ptr() if m else None, m,
                                  quantities.data.data_ptr() if m else None,
                                  trav.data_ptr() if trav is not None else None, scheme.width, scheme.beta,
                                  ws.data_ptr(), ws.numel(), status.data_ptr(), stream.cuda_stream)
        _lib.check(st, "anterpolate!")
    _raise_device_status(status)
    spec = _fft_forward(phys, layout)
    coarse = torch.zeros(field_spectral_shape(scheme.reference_grid, layout, R), dtype=field.data.dtype, device=dev)
    px, py, pz = scheme._pairs()
    for cx, fx in px:
        for cy, fy in py:
            for cz, fz in pz:
                coarse[cx, cy, cz] = spec[fx, fy, fz] / scheme.total_oversampling
    T = np.float32 if scheme.dtype == torch.float32 else np.float64
    dep = coarse * float(T(alpha)) * scheme.total_oversampling * scheme._dec(R)
    if float(beta) == 0.0:
        field.data.copy_(dep)
    else:
        field.data.copy_(dep + float(T(beta)) * field.data)
    torch.cuda.current_stream(dev).synchronize()
    return field


def interpolate_nufft(field: AbstractFieldSpectral, points: PointSet, scheme: NUFFT,
                      traversal: Optional[PointTraversalOrder] = None) -> AbstractPointValues:
    data = empty_colmajor((points.npoints,) + (3,) * field.tensor_order, field.grid.dtype, points.device)
    return interpolate_nufft_(AbstractPointValues(data, field.tensor_order), field, points, scheme, traversal)


def anterpolate_nufft(grid: Grid3D, points: PointSet, quantities: AbstractPointValues, scheme: NUFFT,
                      layout: Optional[RealFourierLayout] = None,
                      traversal: Optional[PointTraversalOrder] = None) -> AbstractFieldSpectral:
    """The allocating form (Interpolation.jl:2066-2072); the layout defaults to the plan's."""
    layout = layout or scheme.reference_layout
    R = quantities.tensor_order
    data = empty_colmajor(field_spectral_shape(grid, layout, R), _COMPLEX[grid.dtype], quantities.data.device)
    return anterpolate_nufft_(AbstractFieldSpectral(data, grid, R, layout), points, quantities, scheme,
                              traversal=traversal)


# ------------------------------------------------ the exact spectral scheme, as a record


class DirectDFT(AbstractTransferScheme):
    """The reference's exact spectral transfer scheme (src/Interpolation.jl:1382-1433), a
    parameterless singleton.  This package carries it as a scheme record -- it round-trips
    through write_scheme/read_scheme, so checkpoints that name it stay readable -- but the
    exact O(N*M) Fourier transfer itself is outside the accelerated path: a transfer with
    it raises MethodError (NUFFT is the fast transfer for spectral fields)."""
    _instance = None

    def __new__(cls):
        if cls._instance is None:
            cls._instance = super().__new__(cls)
        return cls._instance

    def __eq__(self, other):
        return isinstance(other, DirectDFT)

    def __hash__(self):
        return hash("DirectDFT")

    def __repr__(self):
        return "DirectDFT()"


def _refuse_direct_dft(scheme):
    if isinstance(scheme, DirectDFT):
        raise MethodError("DirectDFT, the exact O(N*M) Fourier transfer, is not provided by this package; "
                          "use a NUFFT scheme for a field in spectral representation")


# ------------------------------------------------ dispatch from the generic entry points


def _refuse_mixed():
    raise MethodError("a NUFFT transfers a field in spectral representation, and a spline scheme a field in "
                      "physical representation; there is no method for this combination")


def dispatch_interpolate_(out, field, points, scheme, traversal):
    _refuse_direct_dft(scheme)
    if not (isinstance(field, AbstractFieldSpectral) and isinstance(scheme, NUFFT)):
        _refuse_mixed()
    return interpolate_nufft_(out, field, points, scheme, traversal)


def dispatch_interpolate(field, points, scheme, traversal):
    _refuse_direct_dft(scheme)
    if not (isinstance(field, AbstractFieldSpectral) and isinstance(scheme, NUFFT)):
        _refuse_mixed()
    return interpolate_nufft(field, points, scheme, traversal)


def dispatch_anterpolate_(field, points, quantities, scheme, alpha, beta, traversal):
    _refuse_direct_dft(scheme)
    if not (isinstance(field, AbstractFieldSpectral) and isinstance(scheme, NUFFT)):
        _refuse_mixed()
    return anterpolate_nufft_(field, points, quantities, scheme, alpha, beta, traversal)
