"""The spectral-transfer oracle pinned to the reference's own tests (CPU only).

Follows test/transfer_spectral.jl: DirectDFT against the grid transforms at the nodes,
against analytic band-limited fields off the grid (the reference's five test points), the
node-sample deposit against to_spectral, and the adjoint relation M<Wf,q> = N<f,W^T q>;
then the NUFFT restatement against DirectDFT to the tolerance, its adjoint pair, and the
permuted rfft layout.  Also: the library's host-side window transform against the oracle's,
and the NUFFT plan's argument rules (no GPU needed for either)."""
import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import nufft_oracle as no  # noqa: E402

# the reference's off-grid test points (test/transfer_spectral.jl:31)
P5 = np.array([[0.37, 1.11, 2.93], [1.7, 0.2, 5.0], [4.4, 3.3, 2.2], [0.05, 6.0, 0.5], [2.0, 2.0, 2.0]])


def nodes(n, domain=(2 * np.pi,) * 3):
    xs = [np.arange(n[d]) * domain[d] / n[d] for d in range(3)]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    return np.stack([X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")], axis=1), (X, Y, Z)


def sample(fn, n):
    _, (X, Y, Z) = nodes(n)
    v = fn(X, Y, Z)
    if isinstance(v, tuple):
        return np.stack(v, axis=-1)
    return v


scalar = lambda x, y, z: np.cos(2 * x) + 0.5 * np.sin(y) * np.cos(3 * z) + 0.3  # noqa: E731
vector = lambda x, y, z: (np.sin(y) + np.cos(2 * z), np.sin(2 * x) + np.cos(z), np.sin(x) + np.cos(2 * y))  # noqa: E731


def test_direct_interpolate_equals_to_physical_at_nodes():
    n = (8, 8, 8)
    g = no.grid(n)
    pts, _ = nodes(n)
    for fn in (lambda x, y, z: np.cos(2 * x) + 0.3, lambda x, y, z: (np.sin(y), np.cos(z), np.sin(x))):
        phys = sample(fn, n)
        fh = no.to_spectral(phys, 0)
        got = no.direct_interpolate(fh, g, 0, pts)
        want = no.to_physical(fh, n, 0).reshape(len(pts), -1, order="F")
        assert np.allclose(got, want, rtol=1e-11, atol=1e-11)


def test_direct_reproduces_band_limited_fields_off_grid():
    n = (8, 8, 8)
    g = no.grid(n)
    fh = no.to_spectral(sample(scalar, n), 0)
    got = no.direct_interpolate(fh, g, 0, P5)[:, 0]
    want = scalar(P5[:, 0], P5[:, 1], P5[:, 2])
    assert np.allclose(got, want, rtol=1e-11, atol=1e-11)
    sol = lambda x, y, z: (np.sin(y) + np.cos(z), np.sin(z) + np.cos(2 * x), np.sin(2 * x) + np.cos(y))  # noqa: E731
    uh = no.to_spectral(sample(sol, n), 0)
    got_u = no.direct_interpolate(uh, g, 0, P5)
    want_u = np.stack(sol(P5[:, 0], P5[:, 1], P5[:, 2]), axis=1)
    assert np.allclose(got_u, want_u, rtol=1e-11, atol=1e-11)


def test_direct_anterpolate_equals_to_spectral_of_node_samples():
    n = (8, 8, 8)
    g = no.grid(n)
    pts, (X, Y, Z) = nodes(n)
    fn = lambda x, y, z: np.cos(x) + np.sin(2 * y)  # noqa: E731
    vals = fn(pts[:, 0], pts[:, 1], pts[:, 2])
    dep = no.direct_anterpolate(g, 0, pts, vals)[..., 0]
    assert np.allclose(dep, no.to_spectral(fn(X, Y, Z), 0), rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("R", [0, 1, 2])
def test_direct_adjointness(R):
    n = (8, 8, 8)
    g = no.grid(n)
    rng = np.random.default_rng(2024 + R)
    phys = rng.standard_normal(n + (3,) * R)
    fh = no.to_spectral(phys, 0)
    q = rng.standard_normal((5,) + (3,) * R)
    gathered = no.direct_interpolate(fh, g, 0, P5)
    dep = no.direct_anterpolate(g, 0, P5, q)
    left = float(np.sum(gathered * q.reshape(5, -1, order="F")))
    right = float(np.prod(n)) * no.inner_spectral(fh, dep, n, 0)
    assert abs(left - right) <= 1e-11 * max(1.0, abs(left))


@pytest.mark.parametrize("fn", [scalar, vector], ids=["scalar", "vector"])
def test_nufft_oracle_matches_direct_to_tolerance(fn):
    n = (16, 16, 16)
    g = no.grid(n)
    rng = np.random.default_rng(99)
    pts = rng.random((8, 3)) * 2 * np.pi
    fh = no.to_spectral(sample(fn, n), 0)
    W = no.nufft_width(1e-10)
    beta = no.nufft_beta(W)
    fast = no.nufft_interpolate(fh, g, 0, pts, W, beta)
    exact = no.direct_interpolate(fh, g, 0, pts)
    assert np.allclose(fast, exact, rtol=1e-8, atol=1e-8)
    if fn is scalar:
        assert np.allclose(fast[:, 0], scalar(pts[:, 0], pts[:, 1], pts[:, 2]), rtol=1e-8, atol=1e-8)


def test_nufft_oracle_adjoint_pair():
    n = (16, 16, 16)
    g = no.grid(n)
    rng = np.random.default_rng(7)
    pts = rng.random((8, 3)) * 2 * np.pi
    fh = no.to_spectral(sample(vector, n), 0)
    q = rng.standard_normal((8, 3))
    W = no.nufft_width(1e-10)
    beta = no.nufft_beta(W)
    gathered = no.nufft_interpolate(fh, g, 0, pts, W, beta)
    dep = no.nufft_anterpolate(g, 0, pts, q, W, beta)
    left = float(np.sum(gathered * q))
    right = float(np.prod(n)) * no.inner_spectral(fh, dep, n, 0)
    assert abs(left - right) <= 1e-8 * max(1.0, abs(left))
    # the deposit against the exact one, on the resolved band (Nyquist planes projected out)
    exact = no.direct_anterpolate(g, 0, pts, q)
    band = np.ones(exact.shape[:3], bool)
    band[8, :, :] = False
    band[:, 8, :] = False
    band[:, :, 8] = False
    assert np.allclose(dep[band], exact[band], rtol=1e-8, atol=1e-8 * np.abs(exact).max())


def test_permuted_layout():
    n = (8, 6, 4)
    g = no.grid(n)
    half = 1  # RealFourierLayout((2, 1, 3))
    rng = np.random.default_rng(3)
    phys = rng.random(n)
    fh = no.to_spectral(phys, half)
    assert fh.shape == (8, 4, 4)
    pts, _ = nodes(n)
    at_nodes = no.direct_interpolate(fh, g, half, pts)[:, 0]
    assert np.allclose(at_nodes, phys.ravel(order="F"), rtol=1e-11, atol=1e-11)
    # NUFFT against DirectDFT off-grid on a band-limited field under the permuted fold
    bl = lambda x, y, z: np.cos(x) + 0.5 * np.sin(2 * y) * np.cos(z) + 0.25  # noqa: E731
    fb = no.to_spectral(sample(bl, n), half)
    off = rng.random((6, 3)) * 2 * np.pi
    W = no.nufft_width(1e-10)
    fast = no.nufft_interpolate(fb, g, half, off, W, no.nufft_beta(W))
    assert np.allclose(fast, no.direct_interpolate(fb, g, half, off), rtol=1e-8, atol=1e-8)


def test_library_window_transform_matches_oracle():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    pkg = ge.load_package()
    lib = pkg._lib.load()
    for n, is_half, sigma, W, dt, code in [(16, 1, 2, 12, np.float64, pkg._lib.GBG_F64),
                                           (15, 0, 2, 7, np.float64, pkg._lib.GBG_F64),
                                           (16, 0, 3, 6, np.float32, pkg._lib.GBG_F32)]:
        beta = float(no.nufft_beta(W, dt))
        stored = n // 2 + 1 if is_half else n
        buf = (ctypes.c_double * stored)()
        pkg._lib.check(lib.gbg_nufft_deconvolution_axis(n, is_half, sigma, W, beta, code, buf))
        want = no.deconvolution_axis(n, bool(is_half), sigma, W, dt(beta), dt)
        rtol = 1e-13 if dt == np.float64 else 2e-6
        assert np.allclose(np.asarray(buf), want.astype(np.float64), rtol=rtol, atol=0)
        if n % 2 == 0:
            assert buf[stored - 1 if is_half else n // 2] == 0.0


def test_plan_argument_rules():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    pkg = ge.load_package()
    import torch
    grid = pkg.Grid3D((8, 8, 8), (2 * np.pi,) * 3)
    NU = pkg.NUFFT
    for bad in (0.0, -1e-6, float("inf"), float("nan")):
        with pytest.raises(pkg.ArgumentError):
            NU.for_grid(grid, 0, device="cpu", tolerance=bad)
    with pytest.raises(pkg.ArgumentError):
        NU.for_grid(grid, 0, device="cpu", oversampling=1)
    for w in (0, -2):
        with pytest.raises(pkg.ArgumentError):
            NU.for_grid(grid, 0, device="cpu", window_width=w)
    for s in (0.0, -1.0, float("inf")):
        with pytest.raises(pkg.ArgumentError):
            NU.for_grid(grid, 0, device="cpu", window_shape=s)
    derived = NU.for_grid(grid, 0, device="cpu", tolerance=1e-6)
    assert derived.width == 8 and derived.beta == pytest.approx(2.3 * 8)
    assert NU.for_grid(grid, 0, device="cpu", tolerance=1e-6, window_width=derived.width).width == derived.width
    assert NU.for_grid(grid, 0, device="cpu", tolerance=1e-6, window_shape=derived.beta).beta == derived.beta
    assert NU.for_grid(grid, 0, device="cpu", tolerance=1e-10).width == 12
    # the plan's deconvolution is the oracle's
    plan = NU.for_grid(grid, 1, device="cpu", tolerance=1e-8)
    want = no.deconvolution(grid.grid_size, 0, 2, plan.width, plan.beta)
    assert np.allclose(plan.deconvolution.numpy(), want, rtol=1e-13, atol=0)
    with pytest.raises(pkg.ArgumentError):
        pkg.RealFourierLayout((1, 1, 2))
    # a spectral field's shape follows the layout's half axis
    assert pkg.field_spectral_shape(grid, pkg.RealFourierLayout((2, 1, 3)), 1) == (8, 5, 8, 3)
    assert torch.is_tensor(plan.deconvolution)
