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


# ------------------------------------------------------------ embed_modes! / extract_modes!

L = (TWO_PI, 3.0, 2.5)


def _wave(x, y, z):
    """A field band-limited below the coarse grids' Nyquist frequencies (kx <= 3, ky <= 2, kz <= 2)."""
    return (torch.cos(3 * TWO_PI * x / L[0] + 0.3) * torch.sin(2 * TWO_PI * y / L[1])
            + 0.5 * torch.cos(TWO_PI * x / L[0] - 2 * TWO_PI * z / L[2] + 1.1) + 0.25)


@pytest.mark.parametrize("fft_dims", [(1, 2, 3), (2, 1, 3), (3, 1, 2)])
def test_embed_and_extract_keep_the_field(gbg, fft_dims):
    """A band-limited field sampled on a coarse grid, embedded into a finer one's modes, transforms
    back to the same field sampled on the fine grid; extracted from the fine grid's modes, to the
    same field on the coarse grid (Fields.jl:3360-3446: physical amplitudes kept)."""
    lay = gbg.RealFourierLayout(fft_dims)
    coarse = gbg.Grid3D((8, 6, 5), L, origin=(0.2, -0.1, 0.4))
    fine = gbg.Grid3D((16, 12, 9), L, origin=(0.2, -0.1, 0.4))
    fc = gbg.sample_field(_wave, coarse, device="cpu")
    ff = gbg.sample_field(_wave, fine, device="cpu")
    ch = gbg.to_spectral(fc, layout=lay)
    fh = gbg.to_spectral(ff, layout=lay)
    up = gbg.similar_field(fh, torch.zeros_like(fh.data))
    assert gbg.embed_modes_(up, ch) is up
    assert torch.allclose(gbg.to_physical(up).data, ff.data, rtol=0, atol=1e-12)
    down = gbg.similar_field(ch, torch.zeros_like(ch.data))
    assert gbg.extract_modes_(down, fh) is down
    assert torch.allclose(gbg.to_physical(down).data, fc.data, rtol=0, atol=1e-12)
    # extract after embed gives the coarse modes back (up to the two scalings' rounding)
    back = gbg.similar_field(ch, torch.zeros_like(ch.data))
    gbg.extract_modes_(back, up)
    assert torch.allclose(back.data, ch.data, rtol=1e-14, atol=1e-12)


def test_shared_modes_leave_the_rest_alone_and_scale(gbg):
    """Only the shared modes are written: the fine field's other modes and the coarse grid's
    even-axis Nyquist modes keep their values; alpha and beta act as in mul!(C, A, B, a, b),
    with alpha carrying the ratio of the two grids' point counts."""
    coarse = gbg.Grid3D((8, 6, 5), L)
    fine = gbg.Grid3D((12, 10, 7), L)
    g = torch.Generator().manual_seed(3)
    c = gbg.ScalarFieldSpectral(gbg.colmajor(torch.randn(5, 6, 5, dtype=torch.complex128, generator=g)), coarse)
    sentinel = complex(7.0, -7.0)
    f = gbg.ScalarFieldSpectral(gbg.colmajor(torch.full((7, 10, 7), sentinel, dtype=torch.complex128)), fine)
    ratio = (12 * 10 * 7) / (8 * 6 * 5)
    pairs = []                               # (coarse index, fine index) of every shared mode
    for i in range(5):                       # folded x: 0..4, the coarse Nyquist (4) left out
        for j in range(6):                   # full y: 0, 1, 2, (3: Nyquist), -2, -1
            for k in range(5):               # full z, odd: 0, 1, 2, -2, -1
                if i == 4 or j == 3:
                    continue
                pairs.append(((i, j, k), (i, j if j < 3 else 10 + j - 6, k if k < 3 else 7 + k - 5)))
    shared = torch.zeros((7, 10, 7), dtype=torch.bool)
    for _, fi in pairs:
        shared[fi] = True
    gbg.embed_modes_(f, c)
    for ci, fi in pairs:
        assert torch.isclose(f.data[fi], ratio * c.data[ci], rtol=1e-15, atol=0)
    assert bool((f.data[~shared] == sentinel).all())
    before = f.data.clone()
    gbg.embed_modes_(f, c, 2.0, 0.5)
    for ci, fi in pairs:
        assert torch.isclose(f.data[fi], 0.5 * before[fi] + (2.0 * ratio) * c.data[ci], rtol=1e-15, atol=0)
    assert bool((f.data[~shared] == sentinel).all())
    # extract leaves the coarse destination's Nyquist modes as they were
    d = gbg.ScalarFieldSpectral(gbg.colmajor(torch.full((5, 6, 5), sentinel, dtype=torch.complex128)), coarse)
    gbg.extract_modes_(d, f)
    assert bool((d.data[4] == sentinel).all()) and bool((d.data[:, 3] == sentinel).all())
    for ci, fi in pairs:
        assert torch.isclose(d.data[ci], f.data[fi] / ratio, rtol=1e-15, atol=0)


def test_shared_modes_refusals(gbg):
    coarse = gbg.Grid3D((8, 6, 5), L)
    fine = gbg.Grid3D((12, 10, 7), L)
    spec = lambda grid, R=0, dtype=torch.complex128, lay=None: gbg.similar_field(
        gbg.to_spectral(gbg.AbstractFieldPhysical(
            gbg.colmajor(torch.zeros(tuple(grid.grid_size) + (3,) * R, dtype=torch.float64 if dtype == torch.complex128 else torch.float32)),
            grid, R), layout=lay))
    c, f = spec(coarse), spec(fine)
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(c, f)                                  # the destination of embed is the finer field
    with pytest.raises(gbg.ArgumentError):
        gbg.extract_modes_(f, c)                                # the destination of extract is the coarser one
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(coarse), c)                       # equal grids
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(gbg.Grid3D((12, 4, 7), L)), c)    # coarser on one axis, finer on another
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(gbg.Grid3D((12, 10, 7), (TWO_PI, 3.0, 2.0))), c)     # another box
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(gbg.Grid3D((12, 10, 7), L, origin=(0.1, 0, 0))), c)  # another origin
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(fine, lay=gbg.RealFourierLayout((2, 1, 3))), c)    # another Fourier layout
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(fine, R=1), c)                    # another tensor order
    with pytest.raises(gbg.ArgumentError):
        gbg.embed_modes_(spec(gbg.Grid3D((12, 10, 7), L, dtype=torch.float32), dtype=torch.complex64), c)
