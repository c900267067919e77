"""GB300-native (sm_103a) particle gather/scatter for GBGPeriodicFields.jl's spline
transfer path: interpolate!/anterpolate! of periodic scalar, vector and tensor fields at
points, the traversal order, the resident precision/batched/served forms, and the NUFFT
spectral transfer built on the same window gather/scatter.

The compute runs in hand-written CUDA kernels in libgbg_gb300.so, reached through the C
ABI in include/gbg_transfer.h.  This package is the host-side mirror of the reference's
API over that ABI (the Julia facade binds the same ABI with ccall)."""
from . import _lib
from ._lib import ArgumentError, DimensionMismatch, GBGError, InexactError, MethodError
from .api import (AbstractFieldPhysical, AbstractPointValues, AbstractTransferScheme, Grid3D, LagrangeSpline,
                  LalescuSpline, Point, PointSet, PointTraversalOrder, PointTraversalOrderScratch,
                  ScalarFieldPhysical, ScalarPointValues, TensorFieldPhysical, TensorPointValues,
                  VectorFieldPhysical, VectorPointValues, anterpolate, anterpolate_, colmajor, displace_,
                  empty_colmajor, fiber_shape, field_data, field_grid, field_physical_shape, field_scalar_type,
                  field_tensor_order, interpolate, interpolate_, npoints, point_positions,
                  point_traversal_order, point_traversal_order_, point_value_tensor_order, point_values,
                  sample_field, similar_field, similar_point_values, wrap_, zeros_colmajor)
from .nufft import (NUFFT, AbstractFieldSpectral, DirectDFT, FieldTransformPlans, RealFourierLayout,
                    ScalarFieldSpectral, TensorFieldSpectral, VectorFieldSpectral, embed_modes_, extract_modes_,
                    field_layout, field_spectral_shape, to_physical, to_physical_, to_spectral, to_spectral_)
from .checkpoint import (read_field, read_field_, read_points, read_scheme, write_field, write_points,
                         write_scheme)
from .h5 import h5open


def __getattr__(name):
    if name == "CatmullRom":
        from .api import _catmull_rom
        return _catmull_rom()
    raise AttributeError(name)


def build(verbose: bool = False):
    from . import builder
    return builder.build(verbose)
