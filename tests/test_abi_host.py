"""CPU tests of the C ABI (loads, exports every declared symbol, host-side checks that
return before any launch) and of the host-side mirror's error contract, which follows
the reference's ArgumentError / DimensionMismatch behaviour."""
import ctypes

import numpy as np
import pytest
import torch

TWO_PI = 2 * np.pi


def test_library_exports_every_declared_symbol(gbg):
    lib = gbg._lib.load()
    declared = gbg._lib.header_functions()
    assert declared, "no functions parsed from include/*.h"
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in declared if n not in gbg._lib.SIGNATURES]
    assert not unbound, unbound
    assert lib.gbg_abi_version() == 1


def test_status_strings(gbg):
    lib = gbg._lib.load()
    for code in range(0, 10):
        assert lib.gbg_status_string(code)


@pytest.mark.parametrize("w,m", [(2, 0), (4, 1), (4, 2), (6, 1), (6, 2), (8, 2), (8, 3), (10, 4)])
def test_lalescu_coefficients_match_oracle(gbg, oracle, w, m):
    got = gbg.LalescuSpline(w, m).coefficients
    want = oracle.lalescu(w, m)
    assert got.shape == want.shape
    assert np.abs(got - want).max() <= 1e-15


@pytest.mark.parametrize("w", [2, 4, 6, 8, 10])
def test_lagrange_coefficients_match_oracle(gbg, oracle, w):
    assert np.abs(gbg.LagrangeSpline(w).coefficients - oracle.lagrange(w)).max() <= 1e-15


def test_axis_weights_match_oracle(gbg, oracle):
    for scheme in (gbg.CatmullRom, gbg.LalescuSpline(6), gbg.LagrangeSpline(8)):
        for t in np.linspace(0, 1, 17):
            assert np.array_equal(scheme.axis_weights(t), oracle.axis_weights(scheme.coefficients, t))


def test_scheme_refusals(gbg):
    # interpolation_transfer.jl:63-67
    gbg.LalescuSpline(4, 2)
    for args in ((4, 3), (2, 1), (0,), (3,)):
        with pytest.raises(gbg.ArgumentError):
            gbg.LalescuSpline(*args)
    with pytest.raises(gbg.ArgumentError):
        gbg.LagrangeSpline(0)
    with pytest.raises(gbg.GBGError):
        gbg.LagrangeSpline(18)  # wider than this build's stencil limit


def test_grid_refusals(gbg):
    with pytest.raises(gbg.ArgumentError):
        gbg.Grid3D((0, 4, 4), (1.0, 1.0, 1.0))
    with pytest.raises(gbg.ArgumentError):
        gbg.Grid3D((4, 4, 4), (1.0, float("inf"), 1.0))
    with pytest.raises(gbg.ArgumentError):
        gbg.Grid3D((4, 4, 4), (1.0, 1.0, 1.0), origin=(float("nan"), 0, 0))
    with pytest.raises(gbg.ArgumentError):
        gbg.Grid3D((4, 4, 4), (1.0, 1.0, 1.0), grid_spacing=(0.3, 0.25, 0.25))
    g32 = gbg.Grid3D((16, 15, 14), (TWO_PI,) * 3, dtype=torch.float32)
    assert g32.grid_spacing[1] == float(np.float32(np.float32(TWO_PI) / np.float32(15)))


def test_transfer_argument_contract(gbg):
    grid = gbg.Grid3D((8, 7, 6), (TWO_PI,) * 3)
    field = gbg.VectorFieldPhysical(torch.rand((8, 7, 6, 3), dtype=torch.float64), grid)
    pts = gbg.PointSet(TWO_PI * torch.rand((5, 3), dtype=torch.float64))
    # tensor order mismatch -> ArgumentError
    with pytest.raises(gbg.ArgumentError):
        gbg.interpolate_(gbg.ScalarPointValues(torch.zeros(5, dtype=torch.float64)), field, pts, gbg.CatmullRom)
    # npoints mismatch -> DimensionMismatch (interpolation_transfer.jl:307-310)
    with pytest.raises(gbg.DimensionMismatch):
        gbg.interpolate_(gbg.VectorPointValues(torch.zeros((4, 3), dtype=torch.float64)), field, pts, gbg.CatmullRom)
    with pytest.raises(gbg.DimensionMismatch):
        gbg.anterpolate_(field, pts, gbg.VectorPointValues(torch.zeros((4, 3), dtype=torch.float64)), gbg.CatmullRom)
    # mixed precision -> ArgumentError (test/contracts.jl:145-149)
    with pytest.raises(gbg.ArgumentError):
        gbg.interpolate(field, gbg.PointSet(torch.rand((5, 3), dtype=torch.float32)), gbg.CatmullRom)
    # host arrays: there is no CPU path
    with pytest.raises(gbg.ArgumentError):
        gbg.interpolate(field, pts, gbg.CatmullRom)
    # alpha and beta come as a pair
    with pytest.raises(gbg.ArgumentError):
        gbg.anterpolate_(field, pts, gbg.VectorPointValues(torch.zeros((5, 3), dtype=torch.float64)),
                         gbg.CatmullRom, 1.0)
    # a traversal must be a PointTraversalOrder of the right length
    with pytest.raises(gbg.ArgumentError):
        gbg.api._check_traversal(torch.arange(1, 6), 5, field.data.device)
    with pytest.raises(gbg.ArgumentError):
        gbg.api._check_traversal(gbg.PointTraversalOrder(range(1, 5)), 5, field.data.device)


def test_traversal_order_validation_host(gbg):
    # Interpolation.jl:560-589
    gbg.PointTraversalOrder(range(5, 0, -1))
    with pytest.raises(gbg.ArgumentError):
        gbg.PointTraversalOrder([1, 1, 3])
    with pytest.raises(gbg.ArgumentError):
        gbg.PointTraversalOrder([2, 3, 4])
    with pytest.raises(gbg.ArgumentError):
        gbg.PointTraversalOrder(torch.tensor([1.0, 2.0]))
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    with pytest.raises(gbg.ArgumentError):
        gbg.point_traversal_order(grid, gbg.PointSet(torch.rand((10, 3), dtype=torch.float32)))
    with pytest.raises(gbg.ArgumentError):
        gbg.point_traversal_order(grid, gbg.PointSet(torch.rand((10, 3), dtype=torch.float64)), tile_size=0)


def test_c_abi_checks_before_launch(gbg):
    """Argument errors come back as status codes with no CUDA call (no GPU needed)."""
    lib = gbg._lib.load()
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3).c()
    scheme = gbg.CatmullRom.c()
    bad = gbg._lib.SchemeC()
    bad.stencil_width = 3
    bad.num_powers = 4
    assert lib.gbg_interpolate(grid, 2, 1, 1, 1, 10, None, bad, 1, None, None) == gbg._lib.GBG_EARG
    assert lib.gbg_interpolate(grid, 7, 1, 1, 1, 10, None, scheme, 1, None, None) == gbg._lib.GBG_EARG
    assert lib.gbg_interpolate(grid, 2, 0, 1, 1, 10, None, scheme, 1, None, None) == gbg._lib.GBG_EARG
    assert lib.gbg_interpolate(grid, 2, 1, 1, 1, -1, None, scheme, 1, None, None) == gbg._lib.GBG_EDIM
    assert lib.gbg_interpolate(grid, 2, 1, None, None, 0, None, scheme, None, None, None) == gbg._lib.GBG_OK
    badgrid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3).c()
    badgrid.n[1] = 0
    assert lib.gbg_interpolate(badgrid, 2, 1, 1, 1, 1, None, scheme, 1, None, None) == gbg._lib.GBG_EARG
    assert "grid_size" in gbg._lib.last_error()
    nbytes = ctypes.c_size_t()
    assert lib.gbg_anterpolate_workspace_size(grid, 2, 3, 1000, scheme, ctypes.byref(nbytes)) == 0
    # keys, sorted keys, permutation, a 32-byte record and 3 quantities per point, at least
    assert nbytes.value > 1000 * (3 * 4 + 32 + 3 * 8)
    assert lib.gbg_point_traversal_order_workspace_size(grid, 1000, 0, ctypes.byref(nbytes)) == gbg._lib.GBG_EARG


def test_autotune_heuristic_and_cache_keys(gbg, tmp_path, monkeypatch):
    from gbgperiodicfields_gb300 import autotune
    monkeypatch.setenv("GBG_TUNE_CACHE", str(tmp_path / "t.json"))
    big = autotune.heuristic((256, 256, 256), 3, gbg.CatmullRom, 10**6)
    assert big["brick"] == list(autotune.DEFAULT_BRICK) and big["source"] == "heuristic"
    small = autotune.heuristic((32, 32, 32), 3, gbg.CatmullRom, 10**6)
    nb = np.prod([-(-32 // e) for e in small["brick"]])
    assert nb >= 2 * 152 or small["brick"] == list(min(autotune.BRICKS, key=np.prod))
    k1 = autotune.key((64, 64, 64), 3, gbg.CatmullRom, 64 ** 3)
    k2 = autotune.key((64, 64, 64), 3, gbg.LalescuSpline(6), 64 ** 3)
    k3 = autotune.key((64, 64, 64), 3, gbg.CatmullRom, 8 * 64 ** 3)
    assert len({k1, k2, k3}) == 3
    assert autotune.choose((64, 64, 64), 3, gbg.CatmullRom, 64 ** 3)["source"] == "heuristic"


def test_displacement_refusals(gbg):
    """test/displacement.jl:149-157: mixed precision and mismatched counts are refused
    before any launch; the C ABI bounds the term count."""
    M = 7
    pts = gbg.PointSet(torch.rand((M, 3), dtype=torch.float64))
    with pytest.raises(gbg.ArgumentError):
        gbg.displace_(pts, (1.0, gbg.VectorPointValues(torch.rand((M, 3), dtype=torch.float32))))
    with pytest.raises(gbg.DimensionMismatch):
        gbg.displace_(pts, (1.0, gbg.VectorPointValues(torch.rand((M + 1, 3), dtype=torch.float64))))
    with pytest.raises(gbg.DimensionMismatch):
        gbg.displace_(pts, gbg.PointSet(torch.rand((M + 1, 3), dtype=torch.float64)))
    g32 = gbg.Grid3D((8, 12, 16), (TWO_PI, 2 * TWO_PI, 3 * TWO_PI), dtype=torch.float32)
    with pytest.raises(gbg.ArgumentError):
        gbg.wrap_(pts, g32)
    with pytest.raises(gbg.ArgumentError):
        gbg.displace_(pts, (1j, gbg.VectorPointValues(torch.rand((M, 3), dtype=torch.float64))))
    with pytest.raises(gbg.ArgumentError):  # host arrays: no CPU path
        gbg.displace_(pts, (1.0, gbg.VectorPointValues(torch.rand((M, 3), dtype=torch.float64))))
    lib = gbg._lib.load()
    coefs = (ctypes.c_double * 33)()
    secs = (ctypes.c_void_p * 33)(*([1] * 33))
    assert lib.gbg_points_displace(None, 2, 1, 1, 10, 33, coefs, secs, None) == gbg._lib.GBG_EUNSUPPORTED
    assert lib.gbg_points_displace(None, 2, 1, 1, 10, 1, coefs, None, None) == gbg._lib.GBG_EARG
    bad = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3).c()
    bad.domain[1] = -1.0
    assert lib.gbg_points_displace(bad, 2, 1, 1, 10, 0, None, None, None) == gbg._lib.GBG_EARG
    assert lib.gbg_points_displace(None, 2, 1, 1, 0, 0, None, None, None) == gbg._lib.GBG_OK
