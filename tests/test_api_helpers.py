"""The reference's type queries and allocation helpers around the transfer API, on the CPU:
field_tensor_order / field_scalar_type / point_value_tensor_order, fiber_shape and
field_physical_shape, similar_field / similar_point_values (the data and the order forms),
Point, the AbstractTransferScheme supertype, and the in-place transforms to_physical! /
to_spectral! (Fields.jl:1546-1657) against the allocating ones."""
import math

import pytest
import torch

TWO_PI = 2 * math.pi


def test_type_queries_and_shapes(gbg):
    grid = gbg.Grid3D((6, 5, 4), (TWO_PI,) * 3)
    f = gbg.AbstractFieldPhysical(gbg.colmajor(torch.rand(6, 5, 4, 3, 3, dtype=torch.float64)), grid, 2)
    assert gbg.field_tensor_order(f) == 2 and gbg.field_scalar_type(f) == torch.float64
    assert gbg.fiber_shape(0) == () and gbg.fiber_shape(1) == (3,) and gbg.fiber_shape(2) == (3, 3)
    assert gbg.field_physical_shape(grid, 1) == (6, 5, 4, 3)
    fh = gbg.to_spectral(f)
    assert gbg.field_tensor_order(fh) == 2 and gbg.field_scalar_type(fh) == torch.float64
    v = gbg.VectorPointValues(gbg.colmajor(torch.rand(7, 3, dtype=torch.float32)))
    assert gbg.point_value_tensor_order(v) == 1
    with pytest.raises(gbg.ArgumentError):
        gbg.fiber_shape(-1)


def test_similar_point_values_and_fields(gbg):
    grid = gbg.Grid3D((6, 5, 4), (TWO_PI,) * 3, dtype=torch.float32)
    v = gbg.VectorPointValues(gbg.colmajor(torch.rand(9, 3, dtype=torch.float32)))
    same = gbg.similar_point_values(v)
    assert same.tensor_order == 1 and tuple(same.data.shape) == (9, 3) and same.data.dtype == torch.float32
    scal = gbg.similar_point_values(v, 0)
    assert scal.tensor_order == 0 and tuple(scal.data.shape) == (9,)
    wrapped = gbg.similar_point_values(v, gbg.colmajor(torch.ones(9, 3, dtype=torch.float32)))
    assert wrapped.tensor_order == 1 and bool((wrapped.data == 1).all())
    with pytest.raises(gbg.ArgumentError):
        gbg.similar_point_values(v, torch.ones(9, 2))
    f = gbg.AbstractFieldPhysical(gbg.colmajor(torch.rand(6, 5, 4, dtype=torch.float32)), grid, 0)
    g2 = gbg.similar_field(f, 2)
    assert g2.tensor_order == 2 and tuple(g2.data.shape) == (6, 5, 4, 3, 3) and g2.grid == grid
    assert g2.data.dtype == torch.float32 and g2.data.stride()[0] == 1
    fh = gbg.to_spectral(f, layout=gbg.RealFourierLayout((2, 1, 3)))
    sh = gbg.similar_field(fh, 1)
    assert isinstance(sh, gbg.AbstractFieldSpectral) and sh.layout == fh.layout and sh.tensor_order == 1
    assert tuple(sh.data.shape) == gbg.field_spectral_shape(grid, fh.layout, 1)
    w = gbg.similar_field(fh, fh.data.clone())
    assert torch.equal(w.data, fh.data) and w.layout == fh.layout


def test_point_and_scheme_supertype(gbg):
    p = gbg.Point(0.5, 1.0, 2.0)
    assert p.dtype == torch.float64 and p.tolist() == [0.5, 1.0, 2.0]
    assert gbg.Point(1, 2, 3, dtype=torch.float32).dtype == torch.float32
    with pytest.raises(gbg.ArgumentError):
        gbg.Point(1, 2, 3, dtype=torch.int64)
    for s in (gbg.CatmullRom, gbg.LalescuSpline(6), gbg.LagrangeSpline(4), gbg.DirectDFT()):
        assert isinstance(s, gbg.AbstractTransferScheme)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_in_place_transforms(gbg, dtype):
    grid = gbg.Grid3D((8, 6, 5), (TWO_PI, 3.0, 2.5), dtype=dtype)
    f = gbg.AbstractFieldPhysical(gbg.colmajor(torch.rand(8, 6, 5, 3, dtype=dtype)), grid, 1)
    fh = gbg.to_spectral(f)
    plans = gbg.FieldTransformPlans(f, fh)
    dest = gbg.similar_field(fh)
    assert gbg.to_spectral_(dest, f, plans) is dest
    assert torch.equal(dest.data, fh.data)
    back = gbg.similar_field(f)
    keep = fh.data.clone()
    scratch = gbg.similar_field(fh)
    assert gbg.to_physical_(back, fh, plans, scratch) is back
    assert torch.equal(back.data, gbg.to_physical(fh).data) and torch.equal(fh.data, keep)
    with pytest.raises(gbg.ArgumentError):
        gbg.to_physical_(back, fh, plans, fh)                       # the scratch may not alias the source
    other = gbg.Grid3D((8, 6, 4), (TWO_PI, 3.0, 2.5), dtype=dtype)
    g = gbg.AbstractFieldPhysical(gbg.colmajor(torch.rand(8, 6, 4, 3, dtype=dtype)), other, 1)
    with pytest.raises(gbg.ArgumentError):
        gbg.to_spectral_(dest, g, plans)                            # another grid than the plans'
    wrong_order = gbg.similar_field(f, 0)
    with pytest.raises(gbg.ArgumentError):
        gbg.to_physical_(wrong_order, fh, plans)                    # another tensor order
