"""Checkpoint and restore through HDF5: the reference's persistence verbs for fields,
point sets, point values and transfer schemes (ext/GBGPeriodicFieldsHDF5Ext.jl), and a
checkpoint of the resident serving state built on them.

Each object maps to a self-describing HDF5 group, with the reference's schema:

* a field: dataset ``data`` (the real array, or the complex half-spectrum of a field in
  spectral representation) and attributes ``type``, ``version`` (1), ``representation``,
  ``eltype``, ``tensor_order``, ``grid_size``, ``domain_size``, ``origin``,
  ``grid_spacing`` and ``fft_dims`` (write_field, ext/...HDF5Ext.jl:73-99);
* a point set or point values: ``data`` and ``type``, ``version``, ``eltype``,
  ``npoints`` (+ ``tensor_order`` for values) (write_points, :262-280);
* a transfer scheme: attributes only, its parameters rather than its derived weights
  (``type``, ``version`` 2, ``eltype``, ``stencil_width``, ``smoothness``); a NUFFT is
  refused (write_scheme, :336-386).

Reading checks the schema the way the reference does (:120-217, :282-306, :388-419): an
absent or mistyped object, a missing tag, data or geometry attribute, a schema version
from the future, and self-describing attributes that contradict the tag or the data are
refused with ArgumentError, and read_field_ checks every stored property against its
destination before it writes anything.  The files are written by ``h5.py`` (superblock
2, version 2 object headers): files written here read in HDF5.jl with the reference's own
read_field/read_points/read_scheme, and files the reference wrote read here.

Resident state.  A ResidentField of 1, 3 or 9 components is written as a reference
Scalar/Vector/TensorFieldPhysical group of Float32 data (the storage precision; the
export is exact), plus a ``max_stencil_width`` attribute, so the reference can read it;
other component counts (the 12-component velocity + gradient field) use the tag
``GBGPeriodicFields_GB300.ResidentField`` with data (Nx, Ny, Nz, ncomp).  PointBins are
derived data, like the reference's plans: a checkpoint records their configuration
(brick, launch shape, compensation) and the positions they were built from, and
restoring rebuilds them, which reproduces the binned order -- and so every binned
result -- bitwise."""
from __future__ import annotations

import numpy as np
import torch

from . import h5
from ._lib import ArgumentError
from .api import (AbstractFieldPhysical, AbstractPointValues, Grid3D, LagrangeSpline, LalescuSpline, PointSet,
                  colmajor)
from .nufft import NUFFT, AbstractFieldSpectral, DirectDFT, RealFourierLayout

SCHEMA_VERSION = 1
# Version 2 names the splines' parameters stencil_width and smoothness; version 1 stored
# the half-width `neighbours` (width = 2 * neighbours + 2) and is still read.
SCHEME_SCHEMA_VERSION = 2
_PKG = "GBGPeriodicFields."
RESIDENT_TAG = "GBGPeriodicFields_GB300.ResidentField"
BINS_TAG = "GBGPeriodicFields_GB300.PointBins"

_JULIA_NAME = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32"}
_TORCH_REAL = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32}
# the element types a stored scheme may name: a closed table, never an evaluated string
_SCHEME_ELTYPES = ("Float32", "Float64")


def _real(dt) -> np.dtype:
    dt = np.dtype(dt)
    return np.dtype(np.float64) if dt == np.complex128 else np.dtype(np.float32) if dt == np.complex64 else dt


def _julia_eltype(dt) -> str:
    dt = np.dtype(dt)
    if dt in _JULIA_NAME:
        return _JULIA_NAME[dt]
    return {np.dtype(np.complex128): "ComplexF64", np.dtype(np.complex64): "ComplexF32"}.get(dt, str(dt))


def _np_real(grid: Grid3D) -> np.dtype:
    return np.dtype(np.float64) if grid.dtype == torch.float64 else np.dtype(np.float32)


def _host(t: torch.Tensor) -> np.ndarray:
    """The tensor's elements as a Fortran-ordered host array (a view for a CPU tensor)."""
    return colmajor(t).detach().cpu().numpy()


def _family(order: int) -> str:
    return "Scalar" if order == 0 else "Vector" if order == 1 else "Tensor"


def _field_tag(field) -> str:
    rep = "Spectral" if isinstance(field, AbstractFieldSpectral) else "Physical"
    return f"{_PKG}{_family(field.tensor_order)}Field{rep}"


def _layout_of(field) -> RealFourierLayout:
    return getattr(field, "layout", None) or RealFourierLayout()


def _short(tag: str) -> str:
    return tag.replace(_PKG, "")


# ----------------------------------------------------------------------------- fields


def write_field(parent: h5.Group, name: str, field) -> h5.Group:
    """write_field (ext/GBGPeriodicFieldsHDF5Ext.jl:73-99): the field as a group."""
    if not isinstance(field, (AbstractFieldPhysical, AbstractFieldSpectral)):
        raise ArgumentError(f"write_field: {type(field).__name__} is not a field")
    g = parent.create_group(name)
    g.create_dataset("data", _host(field.data))
    grid = field.grid
    T = _np_real(grid)
    a = g.attrs
    a["type"] = _field_tag(field)
    a["version"] = SCHEMA_VERSION
    a["representation"] = "spectral" if isinstance(field, AbstractFieldSpectral) else "physical"
    a["eltype"] = _JULIA_NAME[T]
    a["tensor_order"] = int(field.tensor_order)
    a["grid_size"] = np.array(grid.grid_size, np.int64)
    a["domain_size"] = np.array(grid.domain_size, T)
    a["origin"] = np.array(grid.origin, T)
    a["grid_spacing"] = np.array(grid.grid_spacing, T)
    a["fft_dims"] = np.array(_layout_of(field).fft_dims, np.int64)
    return g


def _open_group(parent, name, caller, what):
    if name not in parent:
        raise ArgumentError(f'{caller}: no object named "{name}" under the given parent')
    g = parent[name]
    if not isinstance(g, h5.Group):
        raise ArgumentError(f'{caller}: "{name}" is a dataset, not a {what} group')
    if "type" not in g.attrs:
        raise ArgumentError(f'{caller}: group "{name}" has no `type` attribute -- it was not written by '
                            f'{"write_field" if what == "field" else "write_points" if what == "point" else "write_scheme"}')
    return g, g.attrs["type"]


def _open_field_group(parent, name, caller):
    """The group-level checks both read verbs make (ext/...HDF5Ext.jl:120-137)."""
    g, tag = _open_group(parent, name, caller, "field")
    if "data" not in g or not isinstance(g["data"], h5.Dataset):
        raise ArgumentError(f'{caller}: field group "{name}" has no `data` dataset -- the group is incomplete')
    for attribute in ("grid_size", "domain_size", "origin", "fft_dims"):
        if attribute not in g.attrs:
            raise ArgumentError(f'{caller}: field group "{name}" is missing the `{attribute}` attribute -- '
                                "the group is incomplete")
    return g, tag


def _validate_schema_version(a, name, caller, understood=SCHEMA_VERSION):
    if "version" not in a:
        return
    version = int(a["version"])
    if version > understood:
        raise ArgumentError(f'{caller}: group "{name}" declares schema version {version}, but this package '
                            f"understands up to {understood} -- the file was written by a newer version")


def _validate_field_schema(g, name, tag, element_type, dimensions, caller):
    """Every self-describing attribute must agree with the tag and the data
    (ext/...HDF5Ext.jl:188-217)."""
    a = g.attrs
    _validate_schema_version(a, name, caller)
    if "representation" in a:
        declared = a["representation"]
        implied = "spectral" if "Spectral" in str(tag) else "physical"
        if declared != implied:
            raise ArgumentError(f'{caller}: group "{name}" declares representation "{declared}" but its type tag '
                                f'"{tag}" is {implied}')
    if "eltype" in a:
        declared = a["eltype"]
        if _julia_eltype(_real(element_type)) != declared:
            raise ArgumentError(f'{caller}: group "{name}" declares eltype "{declared}" but its data carries '
                                f"{_julia_eltype(_real(element_type))}")
    if "tensor_order" in a:
        declared = int(a["tensor_order"])
        if declared != dimensions - 3:
            raise ArgumentError(f'{caller}: group "{name}" declares tensor_order {declared} but its data has '
                                f"{dimensions} dimensions, implying order {dimensions - 3}")


def _reconstruct_grid(g, T: np.dtype) -> Grid3D:
    """The grid in the data's real element type; the stored spacing is used when present,
    so the round trip is exact (ext/...HDF5Ext.jl:222-229)."""
    a = g.attrs
    if T not in _TORCH_REAL:
        raise ArgumentError(f"a field's element type must be Float32 or Float64, got {T}")
    vec = lambda key, conv: tuple(conv(v) for v in np.atleast_1d(a[key]))
    grid_size = vec("grid_size", int)
    domain = vec("domain_size", T.type)
    origin = vec("origin", T.type)
    spacing = vec("grid_spacing", T.type) if "grid_spacing" in a else None
    return Grid3D(grid_size, domain, origin=origin, dtype=_TORCH_REAL[T], grid_spacing=spacing)


_FIELD_TAGS = {f"{_PKG}{fam}Field{rep}": (fam, rep) for fam in ("Scalar", "Vector", "Tensor")
               for rep in ("Physical", "Spectral")}


def _make_field(tag, name, caller, data: torch.Tensor, grid: Grid3D, layout: RealFourierLayout):
    if tag not in _FIELD_TAGS:
        raise ArgumentError(f'{caller}: unrecognized field type tag "{tag}" in group "{name}"')
    fam, rep = _FIELD_TAGS[tag]
    R = data.dim() - 3
    if (fam == "Scalar" and R != 0) or (fam == "Vector" and R != 1) or (fam == "Tensor" and R < 2):
        raise ArgumentError(f'{caller}: group "{name}" is tagged {_short(tag)} but its data has tensor order {R}')
    if rep == "Spectral":
        return AbstractFieldSpectral(data, grid, R, layout)
    f = AbstractFieldPhysical(data, grid, R)
    f.layout = layout
    return f


def read_field(parent: h5.Group, name: str, device="cpu"):
    """read_field (ext/...HDF5Ext.jl:140-163): the field the group holds, its data on
    `device` (the reference's host array by default)."""
    g, tag = _open_field_group(parent, name, "read_field")
    data = g["data"].read()
    if not isinstance(data, np.ndarray) or data.dtype.kind not in "fc":
        raise ArgumentError(f'read_field: the `data` of group "{name}" is not a real or complex array')
    _validate_field_schema(g, name, tag, data.dtype, data.ndim, "read_field")
    grid = _reconstruct_grid(g, _real(data.dtype))
    layout = RealFourierLayout(tuple(int(v) for v in np.atleast_1d(g.attrs["fft_dims"])))
    t = torch.from_numpy(np.asfortranarray(data)).to(device)
    return _make_field(tag, name, "read_field", t, grid, layout)


def read_field_(destination, parent: h5.Group, name: str):
    """read_field! (ext/...HDF5Ext.jl:167-196): fills an existing field, after checking
    the stored type, precision, grid, layout and tensor order against it; a refused read
    writes nothing.  A host destination is read into directly; a device one is staged
    through one host buffer."""
    g, tag = _open_field_group(parent, name, "read_field!")
    ds = g["data"]
    _validate_field_schema(g, name, tag, ds.dtype, ds.ndim, "read_field!")
    want = _field_tag(destination)
    if tag != want:
        raise ArgumentError(f'read_field!: group "{name}" holds a {_short(tag)}, but the destination is a '
                            f"{_short(want)}")
    storage = destination.data
    st_np = np.dtype(str(storage.dtype).replace("torch.", ""))
    if np.dtype(ds.dtype) != st_np:
        raise ArgumentError(f'read_field!: group "{name}" holds a {_julia_eltype(_real(ds.dtype))} field, but the '
                            f"destination is {_julia_eltype(_real(st_np))}; reading does not convert between "
                            "precisions")
    grid = _reconstruct_grid(g, _real(st_np))
    if grid != destination.grid:
        raise ArgumentError(f'read_field!: group "{name}" was written on {grid}, but the destination is on '
                            f"{destination.grid}")
    layout = RealFourierLayout(tuple(int(v) for v in np.atleast_1d(g.attrs["fft_dims"])))
    if layout != _layout_of(destination):
        raise ArgumentError(f'read_field!: group "{name}" was written with {layout}, but the destination has '
                            f"{_layout_of(destination)}")
    if tuple(ds.shape) != tuple(storage.shape):
        raise ArgumentError(f'read_field!: group "{name}" stores a field of tensor order {ds.ndim - 3}, but the '
                            f"destination's is {destination.tensor_order}")
    if storage.device.type == "cpu" and storage.numpy().flags.f_contiguous:
        ds.read_into(storage.numpy())  # straight into the field's own memory
    else:
        host = np.empty(tuple(storage.shape), dtype=st_np, order="F")
        ds.read_into(host)
        storage.copy_(torch.from_numpy(host))
    return destination


# ----------------------------------------------------------------------------- points


def _point_tag(points) -> str:
    if isinstance(points, PointSet):
        return _PKG + "PointSet"
    return f"{_PKG}{_family(points.tensor_order)}PointValues"


def write_points(parent: h5.Group, name: str, points) -> h5.Group:
    """write_points (ext/...HDF5Ext.jl:262-280): a point set's positions or point
    values' samples as a group; positions and values stay separate groups."""
    if isinstance(points, PointSet):
        array = points.positions
    elif isinstance(points, AbstractPointValues):
        array = points.data
    else:
        raise ArgumentError(f"write_points: {type(points).__name__} is neither a PointSet nor point values")
    g = parent.create_group(name)
    g.create_dataset("data", _host(array))
    a = g.attrs
    a["type"] = _point_tag(points)
    a["version"] = SCHEMA_VERSION
    a["eltype"] = _julia_eltype(np.dtype(str(array.dtype).replace("torch.", "")))
    a["npoints"] = int(points.npoints)
    if isinstance(points, AbstractPointValues):
        a["tensor_order"] = int(points.tensor_order)
    return g


def read_points(parent: h5.Group, name: str, device="cpu"):
    """read_points (ext/...HDF5Ext.jl:292-318)."""
    g, tag = _open_group(parent, name, "read_points", "point")
    _validate_schema_version(g.attrs, name, "read_points")
    if "data" not in g or not isinstance(g["data"], h5.Dataset):
        raise ArgumentError(f'read_points: point group "{name}" has no `data` dataset -- the group is incomplete')
    data = g["data"].read()
    if not isinstance(data, np.ndarray):
        raise ArgumentError(f'read_points: the `data` of group "{name}" is not an array')
    t = torch.from_numpy(np.asfortranarray(data)).to(device)
    if tag == _PKG + "PointSet":
        return PointSet(t)
    if tag == _PKG + "ScalarPointValues":
        return AbstractPointValues(t, 0)
    if tag == _PKG + "VectorPointValues":
        return AbstractPointValues(t, 1)
    if tag == _PKG + "TensorPointValues":
        if t.dim() < 3:
            raise ArgumentError(f'read_points: group "{name}" is tagged TensorPointValues but its data has '
                                f"tensor order {t.dim() - 1}")
        return AbstractPointValues(t, t.dim() - 1)  # the order follows the array's dimensionality
    raise ArgumentError(f'read_points: unrecognized point type tag "{tag}" in group "{name}"')


# ----------------------------------------------------------------------------- schemes


def write_scheme(parent: h5.Group, name: str, scheme) -> h5.Group:
    """write_scheme (ext/...HDF5Ext.jl:336-386): the scheme's parameters as attributes
    of a group with no data."""
    if isinstance(scheme, NUFFT):
        raise ArgumentError(
            "write_scheme: a NUFFT scheme is not persistable -- it owns oversampled FFT plans and a "
            "deconvolution window built against a reference field, which are derived objects rather than "
            "parameters. Rebuild it from the reference field you restore anyway, NUFFT(reference, tolerance), "
            "and record the tolerance in your own snapshot if it varies.")
    if not isinstance(scheme, (LalescuSpline, LagrangeSpline, DirectDFT)):
        raise ArgumentError(f"write_scheme: {type(scheme).__name__} is not a transfer scheme")
    g = parent.create_group(name)
    a = g.attrs
    a["type"] = _PKG + type(scheme).__name__
    a["version"] = SCHEME_SCHEMA_VERSION
    if isinstance(scheme, LalescuSpline):
        a["eltype"] = "Float64"  # the weights are kept in Float64 and converted at each launch
        a["stencil_width"] = int(scheme.stencil_width)
        a["smoothness"] = int(scheme.smoothness)
    elif isinstance(scheme, LagrangeSpline):
        a["eltype"] = "Float64"
        a["stencil_width"] = int(scheme.stencil_width)
    return g


def _scheme_parameter(a, name, key) -> int:
    if key not in a:
        raise ArgumentError(f'read_scheme: scheme group "{name}" has no `{key}` attribute -- the group is '
                            "incomplete")
    return int(a[key])


def _scheme_eltype(a, name):
    if "eltype" not in a:
        raise ArgumentError(f'read_scheme: scheme group "{name}" has no `eltype` attribute -- the group is '
                            "incomplete")
    declared = a["eltype"]
    if declared not in _SCHEME_ELTYPES:
        raise ArgumentError(f'read_scheme: scheme group "{name}" declares element type "{declared}", which this '
                            f"package does not build schemes in (expected one of {', '.join(_SCHEME_ELTYPES)})")


def read_scheme(parent: h5.Group, name: str):
    """read_scheme (ext/...HDF5Ext.jl:388-419): the scheme rebuilt from its parameters;
    the constructors revalidate them, so an impossible combination is refused."""
    g, tag = _open_group(parent, name, "read_scheme", "scheme")
    a = g.attrs
    _validate_schema_version(a, name, "read_scheme", understood=SCHEME_SCHEMA_VERSION)
    version = int(a["version"]) if "version" in a else 1

    def width():
        if version >= 2:
            return _scheme_parameter(a, name, "stencil_width")
        return 2 * _scheme_parameter(a, name, "neighbours") + 2

    if tag == _PKG + "LalescuSpline":
        _scheme_eltype(a, name)
        return LalescuSpline(width(), smoothness=_scheme_parameter(a, name, "smoothness"))
    if tag == _PKG + "LagrangeSpline":
        _scheme_eltype(a, name)
        return LagrangeSpline(width())
    if tag == _PKG + "DirectDFT":
        return DirectDFT()
    raise ArgumentError(f'read_scheme: unrecognized scheme type tag "{tag}" in group "{name}"')


def write_object(parent: h5.Group, name: str, value) -> bool:
    """The sugar parent[name] = value for fields, points and schemes; False for anything
    else (which h5 stores as a plain dataset)."""
    if isinstance(value, (AbstractFieldPhysical, AbstractFieldSpectral)):
        write_field(parent, name, value)
    elif isinstance(value, (PointSet, AbstractPointValues)):
        write_points(parent, name, value)
    elif isinstance(value, (LalescuSpline, LagrangeSpline, DirectDFT, NUFFT)):
        write_scheme(parent, name, value)
    else:
        return False
    return True


# ----------------------------------------------------------------------------- resident state


def _write_grid(a, grid: Grid3D, T: np.dtype):
    a["grid_size"] = np.array(grid.grid_size, np.int64)
    a["domain_size"] = np.array(grid.domain_size, T)
    a["origin"] = np.array(grid.origin, T)
    a["grid_spacing"] = np.array(grid.grid_spacing, T)


def write_resident_field(parent: h5.Group, name: str, field) -> h5.Group:
    """A ResidentField as a field group: its components exported in their storage
    precision (FP32, exact), tagged as the reference's physical field of that tensor
    order for 1, 3 or 9 components, else as a GBGPeriodicFields_GB300.ResidentField.  The
    geometry attributes keep the grid's own precision (``grid_eltype``), so a Float64
    grid is restored exactly; the reference's reader converts them to the data's
    Float32."""
    grid = field.grid
    host = field.read(dtype=torch.float32, device="cpu").numpy()  # (Nx, Ny, Nz, ncomp), Fortran
    order = {1: 0, 3: 1, 9: 2}.get(field.ncomp)
    g = parent.create_group(name)
    if order is None:
        data, tag = host, RESIDENT_TAG
    else:
        data = host.reshape(grid.grid_size + (3,) * order, order="F")
        tag = f"{_PKG}{_family(order)}FieldPhysical"
    g.create_dataset("data", data)
    a = g.attrs
    a["type"] = tag
    a["version"] = SCHEMA_VERSION
    a["representation"] = "physical"
    a["eltype"] = "Float32"
    if order is not None:
        a["tensor_order"] = order
    a["ncomp"] = int(field.ncomp)
    _write_grid(a, grid, _np_real(grid))
    a["grid_eltype"] = _JULIA_NAME[_np_real(grid)]
    a["fft_dims"] = np.array((1, 2, 3), np.int64)
    a["max_stencil_width"] = int(field.max_stencil_width)
    return g


def _grid_of(g, data_dtype) -> Grid3D:
    declared = g.attrs.get("grid_eltype")
    T = np.dtype(np.float64) if declared == "Float64" else np.dtype(np.float32) if declared == "Float32" else _real(
        data_dtype)
    return _reconstruct_grid(g, T)


def read_resident_field(parent: h5.Group, name: str, max_stencil_width: int | None = None):
    """A ResidentField restored from a group write_resident_field wrote (or from any
    physical field group of the reference's schema, converted to FP32 storage)."""
    from .resident import ResidentField
    g, tag = _open_field_group(parent, name, "read_resident_field")
    data = g["data"].read()
    if not isinstance(data, np.ndarray) or data.dtype.kind != "f":
        raise ArgumentError(f'read_resident_field: the `data` of group "{name}" is not a real array')
    if tag == RESIDENT_TAG:
        _validate_schema_version(g.attrs, name, "read_resident_field")
        if data.ndim != 4:
            raise ArgumentError(f'read_resident_field: group "{name}" has data of {data.ndim} dimensions, not 4')
    elif tag in _FIELD_TAGS and _FIELD_TAGS[tag][1] == "Physical":
        _validate_field_schema(g, name, tag, data.dtype, data.ndim, "read_resident_field")
    else:
        raise ArgumentError(f'read_resident_field: group "{name}" is not a physical field (tag "{tag}")')
    grid = _grid_of(g, data.dtype)
    ncomp = int(np.prod(data.shape[3:])) if data.ndim > 3 else 1
    width = int(max_stencil_width or g.attrs.get("max_stencil_width", 6))
    f = ResidentField(grid, ncomp, max_stencil_width=width)
    flat = np.asfortranarray(data).reshape(grid.grid_size + (ncomp,), order="F")
    f.load(torch.from_numpy(flat).cuda())
    return f


def write_bins(parent: h5.Group, name: str, bins, positions) -> h5.Group:
    """A PointBins record: its grid, the configuration it was built with and, as a point
    group, the positions it was built from (in the caller's order)."""
    g = parent.create_group(name)
    a = g.attrs
    a["type"] = BINS_TAG
    a["version"] = SCHEMA_VERSION
    _write_grid(a, bins.grid, _np_real(bins.grid))
    a["grid_eltype"] = _JULIA_NAME[_np_real(bins.grid)]
    a["max_points"] = int(bins.max_points)
    if bins.brick is not None:
        a["brick"] = np.array(bins.brick, np.int64)
    a["gather_threads"] = int(getattr(bins, "gather_threads", 0))
    a["scatter_threads"] = int(getattr(bins, "scatter_threads", 0))
    a["compensated"] = int(bool(getattr(bins, "compensated", True)))
    write_points(g, "positions", positions if isinstance(positions, PointSet) else PointSet(positions))
    return g


def read_bins(parent: h5.Group, name: str):
    """PointBins rebuilt from a write_bins record; returns (bins, positions on the
    device).  The rebuilt binned order equals the checkpointed one bitwise."""
    from .resident import PointBins
    g, tag = _open_group(parent, name, "read_bins", "bins")
    if tag != BINS_TAG:
        raise ArgumentError(f'read_bins: group "{name}" is not a PointBins record (tag "{tag}")')
    _validate_schema_version(g.attrs, name, "read_bins")
    a = g.attrs
    for key in ("grid_size", "domain_size", "origin", "max_points"):
        if key not in a:
            raise ArgumentError(f'read_bins: bins group "{name}" is missing the `{key}` attribute')
    grid = _grid_of(g, np.float64)
    pts = read_points(g, "positions", device="cuda")
    brick = tuple(int(v) for v in a["brick"]) if "brick" in a else None
    bins = PointBins(grid, int(a["max_points"]), brick=brick)
    bins.set_launch(int(a.get("gather_threads", 0)), int(a.get("scatter_threads", 0)))
    bins.set_compensated(bool(int(a.get("compensated", 1))))
    bins.build(pts.positions)
    return bins, pts.positions


def save_state(path, *, fields=None, resident=None, points=None, values=None, schemes=None, bins=None,
               attrs=None):
    """One checkpoint file of a serving state: `fields` (name -> field), `resident`
    (name -> ResidentField), `points` (name -> PointSet), `values` (name -> point
    values), `schemes` (name -> scheme) and `bins` (name -> (PointBins, positions)),
    each family in its own group, plus the caller's own attributes on the root."""
    with h5.File(path, "w") as f:
        for key, value in (attrs or {}).items():
            f.attrs[key] = value
        for family, items, writer in (("fields", fields, write_field), ("resident", resident, write_resident_field),
                                      ("points", points, write_points), ("values", values, write_points),
                                      ("schemes", schemes, write_scheme)):
            if items:
                grp = f.create_group(family)
                for name, obj in items.items():
                    writer(grp, name, obj)
        if bins:
            grp = f.create_group("bins")
            for name, (b, pos) in bins.items():
                write_bins(grp, name, b, pos)


def load_state(path, device="cuda"):
    """The state save_state wrote: a dict of the families present, each name -> object
    (bins as (PointBins, positions), rebuilt on their resident field's grid or on the
    grid recorded with them)."""
    out = {}
    with h5.File(path, "r") as f:
        out["attrs"] = dict(f.attrs)
        if "fields" in f:
            out["fields"] = {n: read_field(f["fields"], n, device=device) for n in f["fields"].keys()}
        if "resident" in f:
            out["resident"] = {n: read_resident_field(f["resident"], n) for n in f["resident"].keys()}
        if "points" in f:
            out["points"] = {n: read_points(f["points"], n, device=device) for n in f["points"].keys()}
        if "values" in f:
            out["values"] = {n: read_points(f["values"], n, device=device) for n in f["values"].keys()}
        if "schemes" in f:
            out["schemes"] = {n: read_scheme(f["schemes"], n) for n in f["schemes"].keys()}
        if "bins" in f:
            out["bins"] = {n: read_bins(f["bins"], n) for n in f["bins"].keys()}
    return out
