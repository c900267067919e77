"""NUFFT on the GPU through the C ABI, against the CPU oracle.

Bars: the device path against the oracle's restatement of the reference's NUFFT with the
same window (FP64: 1e-12 relative to max|oracle|; FP32: 1e-5); against DirectDFT to the
NUFFT's own tolerance (FP64 tol 1e-10: 1e-8; FP32 tol 1e-4: 1e-3), as the reference's
test/transfer_spectral.jl does; the adjoint pair M<Wf,q> = N<f,W^T q>; alpha/beta
accumulation; the permuted rfft layout; odd widths; tensor order 2; and the spread's bitwise
reproducibility under any visiting order."""
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import nufft_oracle as no  # noqa: E402

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


@pytest.fixture(scope="module")
def pkg():
    import __graft_entry__ as ge
    return ge.load_package()


scalar = lambda x, y, z: np.cos(2 * x) + 0.5 * np.sin(y) * np.cos(3 * z) + 0.3  # noqa: E731
vector = lambda x, y, z: (np.sin(y) + np.cos(2 * z), np.sin(2 * x) + np.cos(z), np.sin(x) + np.cos(2 * y))  # noqa: E731


def sample(fn, n):
    xs = [np.arange(n[d]) * 2 * np.pi / n[d] for d in range(3)]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    v = fn(X, Y, Z)
    return np.stack(v, axis=-1) if isinstance(v, tuple) else v


def spectral(pkg, phys, grid, R, layout=None):
    layout = layout or pkg.RealFourierLayout()
    fh = no.to_spectral(phys, layout.half_axis)
    t = pkg.colmajor(torch.from_numpy(np.asfortranarray(fh)).to(DEV).to(torch.complex128 if grid.dtype == torch.float64 else torch.complex64))
    return pkg.AbstractFieldSpectral(t, grid, R, layout), fh


def points(pkg, P, dtype):
    return pkg.PointSet(pkg.colmajor(torch.from_numpy(np.asfortranarray(P)).to(DEV).to(dtype)))


def values(pkg, q, R, dtype):
    return pkg.AbstractPointValues(pkg.colmajor(torch.from_numpy(np.asfortranarray(q)).to(DEV).to(dtype)), R)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("R,fn", [(0, scalar), (1, vector)], ids=["scalar", "vector"])
def test_interpolate_matches_oracle_and_direct(pkg, dtype, R, fn):
    n = (16, 16, 16)
    grid = pkg.Grid3D(n, (2 * np.pi,) * 3, dtype=dtype)
    g = no.grid(n)
    P = np.random.default_rng(99).random((8, 3)) * 2 * np.pi
    fhd, fh = spectral(pkg, sample(fn, n), grid, R)
    tol = 1e-10 if dtype == torch.float64 else 1e-4
    plan = pkg.NUFFT(fhd, tolerance=tol)
    got = pkg.interpolate(fhd, points(pkg, P, dtype), plan).data.cpu().numpy().reshape(8, -1, order="F")
    npdt = np.float64 if dtype == torch.float64 else np.float32
    oracle = no.nufft_interpolate(fh, g, 0, P.astype(npdt), plan.width, npdt(plan.beta), dtype=npdt)
    assert rel(got, oracle) <= (1e-12 if dtype == torch.float64 else 1e-5)
    exact = no.direct_interpolate(fh, g, 0, P)
    atol = 1e-8 if dtype == torch.float64 else 1e-3
    assert np.allclose(got, exact, rtol=atol, atol=atol)
    if R == 0:
        assert np.allclose(got[:, 0], scalar(P[:, 0], P[:, 1], P[:, 2]), rtol=atol, atol=atol)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_anterpolate_matches_oracle_and_adjoint(pkg, dtype):
    n = (16, 16, 16)
    grid = pkg.Grid3D(n, (2 * np.pi,) * 3, dtype=dtype)
    g = no.grid(n)
    rng = np.random.default_rng(5)
    P = rng.random((8, 3)) * 2 * np.pi
    q = rng.standard_normal((8, 3))
    fhd, fh = spectral(pkg, sample(vector, n), grid, 1)
    tol = 1e-10 if dtype == torch.float64 else 1e-4
    plan = pkg.NUFFT(fhd, tolerance=tol)
    pts = points(pkg, P, dtype)
    qv = values(pkg, q, 1, dtype)
    dep = pkg.anterpolate(grid, pts, qv, plan)
    got = dep.data.cpu().numpy()
    npdt = np.float64 if dtype == torch.float64 else np.float32
    oracle = no.nufft_anterpolate(g, 0, P.astype(npdt), q.astype(npdt), plan.width, npdt(plan.beta), dtype=npdt)
    assert rel(got, oracle) <= (1e-12 if dtype == torch.float64 else 1e-5)
    gathered = pkg.interpolate(fhd, pts, plan).data.cpu().numpy()
    left = float(np.sum(gathered * q))
    right = float(np.prod(n)) * no.inner_spectral(fh, got, n, 0)
    atol = 1e-8 if dtype == torch.float64 else 1e-3
    assert abs(left - right) <= atol * max(1.0, abs(left))


def test_alpha_beta_accumulate_and_explicit_window(pkg):
    n = (16, 16, 16)
    grid = pkg.Grid3D(n, (2 * np.pi,) * 3)
    fhd, _ = spectral(pkg, sample(scalar, n), grid, 0)
    plan = pkg.NUFFT(fhd, window_width=8, window_shape=18)
    assert plan.width == 8 and plan.beta == 18.0
    rng = np.random.default_rng(11)
    pts = points(pkg, rng.random((8, 3)) * 2 * np.pi, torch.float64)
    q = values(pkg, rng.standard_normal(8), 0, torch.float64)
    once = pkg.anterpolate(grid, pts, q, plan)
    twice = pkg.ScalarFieldSpectral(once.data.clone(), grid)
    pkg.anterpolate_(twice, pts, q, plan, 1.0, 1.0)
    assert torch.allclose(twice.data, 2 * once.data, rtol=1e-12, atol=1e-12)
    half = pkg.ScalarFieldSpectral(once.data.clone(), grid)
    pkg.anterpolate_(half, pts, q, plan, 0.5, 0.0)  # beta = 0 overwrites
    assert torch.allclose(half.data, 0.5 * once.data, rtol=1e-12, atol=1e-12)


def test_permuted_layout_and_odd_width(pkg):
    n = (8, 6, 4)
    grid = pkg.Grid3D(n, (2 * np.pi,) * 3)
    g = no.grid(n)
    layout = pkg.RealFourierLayout((2, 1, 3))
    bl = lambda x, y, z: np.cos(x) + 0.5 * np.sin(2 * y) * np.cos(z) + 0.25  # noqa: E731
    fhd, fh = spectral(pkg, sample(bl, n), grid, 0, layout)
    assert tuple(fhd.data.shape) == (8, 4, 4)
    P = np.random.default_rng(3).random((6, 3)) * 2 * np.pi
    pts = points(pkg, P, torch.float64)
    plan = pkg.NUFFT(fhd, tolerance=1e-10)
    got = pkg.interpolate(fhd, pts, plan).data.cpu().numpy().reshape(6, -1, order="F")
    assert np.allclose(got, no.direct_interpolate(fh, g, 1, P), rtol=1e-8, atol=1e-8)
    # an odd width follows the nearer node on each axis
    odd = pkg.NUFFT(fhd, tolerance=1e-10, window_width=13)
    got13 = pkg.interpolate(fhd, pts, odd).data.cpu().numpy().reshape(6, -1, order="F")
    want13 = no.nufft_interpolate(fh, g, 1, P, 13, odd.beta)
    assert rel(got13, want13) <= 1e-12
    dep = pkg.anterpolate(grid, pts, values(pkg, np.ones(6), 0, torch.float64), odd).data.cpu().numpy()
    want_dep = no.nufft_anterpolate(g, 1, P, np.ones(6), 13, odd.beta)[..., 0]
    assert rel(dep, want_dep) <= 1e-12


def test_tensor_order_two_and_bitwise_spread(pkg):
    n = (12, 10, 8)
    grid = pkg.Grid3D(n, (2 * np.pi, 3.0, 4.0), origin=(0.5, -1.0, 2.0))
    g = no.grid(n, (2 * np.pi, 3.0, 4.0), (0.5, -1.0, 2.0))
    rng = np.random.default_rng(21)
    M = 300
    lo = np.array([0.5, -1.0, 2.0]); ext = np.array([2 * np.pi, 3.0, 4.0])
    P = lo + rng.random((M, 3)) * ext
    q = rng.standard_normal((M, 3, 3))
    plan = pkg.NUFFT.for_grid(grid, 2, device=DEV, tolerance=1e-8)
    pts = points(pkg, P, torch.float64)
    qv = values(pkg, q, 2, torch.float64)
    a = pkg.anterpolate(grid, pts, qv, plan).data.clone()
    trav = pkg.point_traversal_order(grid, pts)
    b = pkg.anterpolate(grid, pts, qv, plan, traversal=trav).data
    assert torch.equal(a, b)  # integer sums: the same bits whatever the visiting order
    oracle = no.nufft_anterpolate(g, 0, P, q, plan.width, plan.beta)
    assert rel(a.cpu().numpy().reshape(oracle.shape, order="F"), oracle) <= 1e-12
    # and the gather of a tensor field (the spectrum of a real one)
    fh = no.to_spectral(rng.standard_normal(n + (3, 3)), 0)
    fhd = pkg.TensorFieldSpectral(pkg.colmajor(torch.from_numpy(np.asfortranarray(fh)).to(DEV)), grid, 2)
    got = pkg.interpolate(fhd, pts, plan).data.cpu().numpy().reshape(M, -1, order="F")
    want = no.nufft_interpolate(fh, g, 0, P, plan.width, plan.beta)
    assert rel(got, want) <= 1e-12


def test_refusals(pkg):
    n = (8, 8, 8)
    grid = pkg.Grid3D(n, (2 * np.pi,) * 3)
    other = pkg.Grid3D(n, (3.0,) * 3)
    fhd, _ = spectral(pkg, sample(scalar, n), grid, 0)
    plan = pkg.NUFFT(fhd, tolerance=1e-6)
    pts = points(pkg, np.random.default_rng(0).random((4, 3)), torch.float64)
    foh, _ = spectral(pkg, sample(scalar, n), other, 0)
    with pytest.raises(pkg.ArgumentError):
        pkg.interpolate(foh, pts, plan)  # a plan for another domain
    vfh, _ = spectral(pkg, sample(vector, n), grid, 1)
    with pytest.raises(pkg.ArgumentError):
        pkg.interpolate(vfh, pts, plan)  # another tensor order
    phys = pkg.ScalarFieldPhysical(torch.zeros(n, dtype=torch.float64, device=DEV), grid)
    with pytest.raises(pkg.MethodError):
        pkg.interpolate(phys, pts, plan)
    with pytest.raises(pkg.MethodError):
        pkg.interpolate(fhd, pts, pkg.CatmullRom)
    with pytest.raises(pkg.DimensionMismatch):
        pkg.anterpolate(grid, pts, values(pkg, np.ones(5), 0, torch.float64), plan)
    bad = pkg.PointSet(pkg.colmajor(torch.tensor([[float("nan"), 0.0, 0.0]], dtype=torch.float64, device=DEV)))
    with pytest.raises(pkg.InexactError):
        pkg.interpolate(fhd, bad, plan)


def test_spread_edge_cases(pkg):
    """No points (a zero deposit, beta still applied); quantities of 1e-300 and 1e290 (the
    fixed-point scale follows max|q| over the whole range); a NaN quantity (NaN on every
    resolved mode, as the FFT of the reference's NaN-holding grid gives; the Nyquist shell,
    which no oversampled mode maps to, stays 0)."""
    n = (8, 8, 8)
    grid = pkg.Grid3D(n, (2 * np.pi,) * 3)
    g = no.grid(n)
    plan = pkg.NUFFT.for_grid(grid, 0, device=DEV, tolerance=1e-8)
    empty = pkg.PointSet(pkg.colmajor(torch.empty((0, 3), dtype=torch.float64, device=DEV)))
    dep = pkg.anterpolate(grid, empty, values(pkg, np.empty(0), 0, torch.float64), plan)
    assert torch.count_nonzero(dep.data) == 0
    fh = pkg.ScalarFieldSpectral(torch.ones_like(dep.data), grid)
    pkg.anterpolate_(fh, empty, values(pkg, np.empty(0), 0, torch.float64), plan, 1.0, 0.5)
    assert torch.allclose(fh.data, torch.full_like(fh.data, 0.5))
    rng = np.random.default_rng(4)
    P = rng.random((20, 3)) * 2 * np.pi
    q = rng.standard_normal(20)
    pts = points(pkg, P, torch.float64)
    want = no.nufft_anterpolate(g, 0, P, q, plan.width, plan.beta)[..., 0]
    for scale in (1e-300, 1e290):
        got = pkg.anterpolate(grid, pts, values(pkg, q * scale, 0, torch.float64), plan).data.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got / scale, want) <= 1e-12
    qn = q.copy()
    qn[3] = np.nan
    got = pkg.anterpolate(grid, pts, values(pkg, qn, 0, torch.float64), plan).data.cpu()
    band = torch.ones(got.shape, dtype=torch.bool)
    band[4, :, :] = False  # the even axes' Nyquist shell is not a shared mode: it stays 0
    band[:, 4, :] = False
    band[:, :, 4] = False
    assert torch.isnan(got[band]).all() and torch.count_nonzero(got[~band]) == 0
