"""GPU parity of the drop-in transfers (gbg_interpolate / gbg_anterpolate /
gbg_point_traversal_order) against the CPU oracle, through the C ABI.

Tolerances (relative to max|oracle|): Float64 1e-13 (the stated bar for the plain
FP64 path), Float32 2e-5.  Integer work (the traversal order) is compared bitwise.
The cases follow the reference's transfer tests (test/interpolation_transfer.jl,
test/point_traversal_order.jl, test/gpu/suite.jl:553-642).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi
TOL = {np.float64: 1e-13, np.float32: 2e-5}


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def to_dev(a, dev):
    return torch.from_numpy(np.asfortranarray(a)).to(dev)


def relerr(got, want):
    scale = max(np.abs(want).max(), 1e-300)
    return np.abs(np.asarray(got, dtype=np.float64) - want).max() / scale


def make(gbg, oracle, n=(16, 15, 14), domain=(TWO_PI,) * 3, origin=(0.0, 0.0, 0.0), dtype=np.float64):
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    grid = gbg.Grid3D(n, domain, origin=origin, dtype=tdt)
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin, dtype=dtype)
    return grid, g


def scheme_list(gbg):
    return [gbg.CatmullRom, gbg.LalescuSpline(6, 1), gbg.LagrangeSpline(6), gbg.LalescuSpline(2, 0),
            gbg.LalescuSpline(6), gbg.LalescuSpline(8, 2), gbg.LagrangeSpline(10)]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("R", [0, 1, 2, 3])
def test_gather_matches_oracle(gbg, oracle, dev, dtype, R):
    grid, g = make(gbg, oracle, origin=(0.3, -1.1, 2.0), dtype=dtype)
    rng = np.random.default_rng(100 + R)
    M, C = 257, 3 ** R
    pos = (np.array(grid.origin) + TWO_PI * (rng.random((M, 3)) * 1.4 - 0.2)).astype(dtype)
    f = rng.standard_normal(grid.grid_size + (C,)).astype(dtype)
    field = gbg.AbstractFieldPhysical(to_dev(f.reshape(grid.grid_size + (3,) * R, order="F"), dev), grid, R)
    points = gbg.PointSet(to_dev(pos, dev))
    for scheme in scheme_list(gbg):
        # column-major fibres: component (a, b) is fibre a + 3b
        got = gbg.interpolate(field, points, scheme).data.cpu().numpy().reshape((M, C), order="F")
        want = oracle.gather(g, f, pos, scheme.coefficients)
        assert relerr(got, want) <= TOL[dtype], (scheme, relerr(got, want))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gather_bitwise_invariant_under_traversal(gbg, oracle, dev, dtype):
    # test/point_traversal_order.jl:60-117 -- the gather is == under any order.
    grid, g = make(gbg, oracle, n=(14, 16, 12), domain=(TWO_PI, TWO_PI, 2 * TWO_PI),
                   origin=(0.25, -2, 0), dtype=dtype)
    rng = np.random.default_rng(4242)
    M = 600
    pos = np.stack([0.25 + TWO_PI * rng.random(M), -2 + TWO_PI * rng.random(M),
                    2 * TWO_PI * rng.random(M)], 1).astype(dtype)
    f = rng.random((14, 16, 12, 3)).astype(dtype)
    field = gbg.VectorFieldPhysical(to_dev(f, dev), grid)
    points = gbg.PointSet(to_dev(pos, dev))
    order = gbg.point_traversal_order(grid, points)
    rev = gbg.PointTraversalOrder(torch.flip(order.indices, [0]))
    for scheme in (gbg.CatmullRom, gbg.LalescuSpline(6, 1), gbg.LagrangeSpline(4)):
        a = gbg.interpolate(field, points, scheme).data
        b = gbg.interpolate(field, points, scheme, traversal=order).data
        c = gbg.interpolate(field, points, scheme, traversal=rev).data
        assert torch.equal(a, b) and torch.equal(a, c)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("R", [0, 1, 2])
def test_scatter_matches_oracle(gbg, oracle, dev, dtype, R):
    grid, g = make(gbg, oracle, origin=(0.3, -1.1, 2.0), dtype=dtype)
    rng = np.random.default_rng(200 + R)
    M, C = 301, 3 ** R
    pos = (np.array(grid.origin) + TWO_PI * (rng.random((M, 3)) * 1.4 - 0.2)).astype(dtype)
    q = rng.standard_normal((M, C)).astype(dtype)
    points = gbg.PointSet(to_dev(pos, dev))
    qv = gbg.AbstractPointValues(to_dev(q.reshape((M,) + (3,) * R, order="F"), dev), R)
    for scheme in scheme_list(gbg):
        got = gbg.anterpolate(grid, points, qv, scheme).data.cpu().numpy().reshape((-1, C), order="F")
        want = oracle.scatter(g, np.zeros(grid.grid_size + (C,), dtype, order="F"), pos, q,
                              scheme.coefficients).reshape((-1, C), order="F")
        assert relerr(got, want) <= TOL[dtype], (scheme, relerr(got, want))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_scatter_alpha_beta_and_nan_overwrite(gbg, oracle, dev, dtype):
    # interpolation_transfer.jl:158-180, 287-296
    grid, g = make(gbg, oracle, dtype=dtype)
    rng = np.random.default_rng(11)
    M = 64
    pos = (TWO_PI * rng.random((M, 3))).astype(dtype)
    q = rng.random((M, 3)).astype(dtype)
    points = gbg.PointSet(to_dev(pos, dev))
    qv = gbg.VectorPointValues(to_dev(q, dev))
    cr = gbg.CatmullRom
    shape = grid.grid_size + (3,)
    prior = rng.standard_normal(shape).astype(dtype)
    for alpha, beta in ((1.0, 0.0), (3.0, 0.0), (1.0, 1.0), (-1.5, 0.5), (2.0, -3.0)):
        fd = gbg.VectorFieldPhysical(to_dev(prior, dev), grid)
        gbg.anterpolate_(fd, points, qv, cr, alpha, beta)
        want = oracle.scatter(g, np.asfortranarray(prior.copy()), pos, q, cr.coefficients, alpha, beta)
        assert relerr(fd.data.cpu().numpy(), want) <= TOL[dtype]
    nanf = gbg.VectorFieldPhysical(to_dev(np.full(shape, np.nan, dtype), dev), grid)
    gbg.anterpolate_(nanf, points, qv, cr, 1.0, 0.0)
    assert torch.isfinite(nanf.data).all()
    # alpha = 0, beta = 2 is a pure rescale, bitwise
    dest = gbg.VectorFieldPhysical(to_dev(prior, dev), grid)
    gbg.anterpolate_(dest, points, qv, cr, 0.0, 2.0)
    assert np.array_equal(dest.data.cpu().numpy(), 2 * prior)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_scatter_deterministic_and_order_free(gbg, oracle, dev, dtype):
    grid, g = make(gbg, oracle, n=(12, 10, 9), dtype=dtype)
    rng = np.random.default_rng(5)
    M = 3000
    pos = (0.3 * rng.random((M, 3))).astype(dtype)  # heavy contention in a few cells
    q = rng.random((M, 1)).astype(dtype)
    points = gbg.PointSet(to_dev(pos, dev))
    qv = gbg.ScalarPointValues(to_dev(q[:, 0], dev))
    order = gbg.point_traversal_order(grid, points)
    a = gbg.anterpolate(grid, points, qv, gbg.CatmullRom).data
    b = gbg.anterpolate(grid, points, qv, gbg.CatmullRom).data
    c = gbg.anterpolate(grid, points, qv, gbg.CatmullRom, traversal=order).data
    assert torch.equal(a, b) and torch.equal(a, c)
    want = oracle.scatter(g, np.zeros(grid.grid_size, dtype, order="F"), pos, q, gbg.CatmullRom.coefficients)
    assert relerr(a.cpu().numpy(), want) <= TOL[dtype]
    assert np.isclose(a.double().sum().item(), q.sum(dtype=np.float64), rtol=1e-10 if dtype == np.float64 else 1e-5)


def test_adjointness_fp64(gbg, oracle, dev):
    grid, g = make(gbg, oracle, n=(20, 18, 16))
    rng = np.random.default_rng(9)
    M = 1000
    pos = TWO_PI * rng.random((M, 3))
    points = gbg.PointSet(to_dev(pos, dev))
    for R in (0, 1, 2):
        C = 3 ** R
        f = rng.standard_normal(grid.grid_size + (3,) * R)
        q = rng.standard_normal((M,) + (3,) * R)
        field = gbg.AbstractFieldPhysical(to_dev(f, dev), grid, R)
        qv = gbg.AbstractPointValues(to_dev(q, dev), R)
        for scheme in (gbg.CatmullRom, gbg.LalescuSpline(6), gbg.LagrangeSpline(8)):
            Wf = gbg.interpolate(field, points, scheme).data
            Wtq = gbg.anterpolate(grid, points, qv, scheme).data
            lhs = torch.sum(Wf * torch.from_numpy(q).to(dev)).item()
            rhs = torch.sum(torch.from_numpy(f).to(dev) * Wtq).item()
            scale = Wf.norm().item() * np.linalg.norm(q)
            assert abs(lhs - rhs) / scale <= 1e-13


def test_adversarial_cases(gbg, oracle, dev):
    rng = np.random.default_rng(3)
    # non-zero origin + strongly anisotropic grid (interpolation_transfer.jl:201-217)
    grid, g = make(gbg, oracle, n=(10, 8, 12), domain=(TWO_PI, 0.5, 40.0), origin=(-1.3, 7.0, 100.0))
    M = 50
    pos = np.stack([grid.origin[d] + grid.domain_size[d] * rng.random(M) for d in range(3)], 1)
    f = rng.random((10, 8, 12))
    q = rng.random(M)
    field = gbg.ScalarFieldPhysical(to_dev(f, dev), grid)
    points = gbg.PointSet(to_dev(pos, dev))
    got = gbg.interpolate(field, points, gbg.CatmullRom).data.cpu().numpy()
    assert relerr(got[:, None], oracle.gather(g, f, pos, gbg.CatmullRom.coefficients)) <= 1e-13
    dep = gbg.anterpolate(grid, points, gbg.ScalarPointValues(to_dev(q, dev)), gbg.CatmullRom).data.cpu().numpy()
    want = oracle.scatter(g, np.zeros((10, 8, 12), order="F"), pos, q[:, None], gbg.CatmullRom.coefficients)
    assert relerr(dep, want) <= 1e-13
    # points exactly on nodes (219-227)
    grid, g = make(gbg, oracle, n=(8, 8, 8))
    dx = TWO_PI / 8
    idx = [(0, 0, 0), (2, 3, 4), (7, 7, 7), (0, 7, 3)]
    coords = np.array([[dx * i[d] for d in range(3)] for i in idx])
    f = rng.random((8, 8, 8))
    v = gbg.interpolate(gbg.ScalarFieldPhysical(to_dev(f, dev), grid), gbg.PointSet(to_dev(coords, dev)),
                        gbg.CatmullRom).data.cpu().numpy()
    assert np.allclose(v, [f[i] for i in idx], rtol=1e-12)
    # stencil wider than the grid (229-236)
    grid, g = make(gbg, oracle, n=(4, 4, 4))
    pos = TWO_PI * rng.random((30, 3))
    f = rng.random((4, 4, 4))
    q = rng.random(30)
    pts = gbg.PointSet(to_dev(pos, dev))
    for scheme in (gbg.LagrangeSpline(8), gbg.LagrangeSpline(10)):
        got = gbg.interpolate(gbg.ScalarFieldPhysical(to_dev(f, dev), grid), pts, scheme).data.cpu().numpy()
        assert relerr(got[:, None], oracle.gather(g, f, pos, scheme.coefficients)) <= 1e-13
        dep = gbg.anterpolate(grid, pts, gbg.ScalarPointValues(to_dev(q, dev)), scheme).data.cpu().numpy()
        want = oracle.scatter(g, np.zeros((4, 4, 4), order="F"), pos, q[:, None], scheme.coefficients)
        assert relerr(dep, want) <= 1e-13
    # heavy contention: 4000 points in one cell (238-246)
    grid, g = make(gbg, oracle, n=(8, 8, 8))
    pos = 0.25 * rng.random((4000, 3))
    q = rng.random(4000)
    dep = gbg.anterpolate(grid, gbg.PointSet(to_dev(pos, dev)), gbg.ScalarPointValues(to_dev(q, dev)),
                          gbg.CatmullRom).data.cpu().numpy()
    want = oracle.scatter(g, np.zeros((8, 8, 8), order="F"), pos, q[:, None], gbg.CatmullRom.coefficients)
    assert relerr(dep, want) <= 1e-13
    assert np.isclose(dep.sum(), q.sum(), rtol=1e-12)


def test_scatter_high_coverage_cancelling_sums(gbg, oracle, dev):
    """Points packed into a few tight blobs, so a node is reached by thousands of points
    (the fixed-point sums shift by several bits, as at the headline's 1e7 clustered points),
    with N(0,1) quantities whose sums cancel: the error stays within the Float64 bar
    relative to max|oracle| and carries no bias (each contribution's rounding averages out
    instead of adding up)."""
    import os
    from gbgperiodicfields_gb300.workloads import clustered_points
    grid, g = make(gbg, oracle, n=(64, 64, 64))
    M = 300_000
    pos = clustered_points(M, seed=11, cluster_fraction=0.5, nblobs=20, sigma=0.05)
    q = np.random.default_rng(12).standard_normal((M, 3))
    pts = gbg.PointSet(to_dev(pos, dev))
    qv = gbg.VectorPointValues(to_dev(q, dev))
    for scheme in (gbg.CatmullRom, gbg.LalescuSpline(6)):
        dep = gbg.anterpolate(grid, pts, qv, scheme).data.cpu().numpy()
        want = oracle.scatter(g, np.zeros((64, 64, 64, 3), order="F"), pos, q, scheme.coefficients,
                              nthreads=os.cpu_count() or 1)
        assert relerr(dep, want) <= 1e-13
        assert abs((dep - want).mean()) <= 1e-16 * np.abs(want).max()


def test_single_and_empty(gbg, oracle, dev):
    grid, g = make(gbg, oracle, n=(8, 8, 8))
    f = np.random.default_rng(0).random((8, 8, 8))
    field = gbg.ScalarFieldPhysical(to_dev(f, dev), grid)
    one = gbg.PointSet(to_dev(np.array([[1.1, 2.2, 0.7]]), dev))
    assert gbg.interpolate(field, one, gbg.CatmullRom).data.shape == (1,)
    dep = gbg.anterpolate(grid, one, gbg.ScalarPointValues(torch.tensor([2.5], dtype=torch.float64, device=dev)),
                          gbg.CatmullRom)
    assert abs(dep.data.sum().item() - 2.5) <= 1e-12
    empty = gbg.PointSet(torch.zeros((0, 3), dtype=torch.float64, device=dev))
    assert gbg.interpolate(field, empty, gbg.CatmullRom).data.shape == (0,)
    dep0 = gbg.anterpolate(grid, empty, gbg.ScalarPointValues(torch.zeros(0, dtype=torch.float64, device=dev)),
                           gbg.CatmullRom)
    assert dep0.data.abs().max().item() == 0
    # the callable field(x) (Interpolation.jl:1229-1235)
    v = field([1.1, 2.2, 0.7])
    want = oracle.gather(g, f, np.array([[1.1, 2.2, 0.7]]), gbg.CatmullRom.coefficients)[0, 0]
    assert abs(v - want) <= 1e-13 * abs(want)


def test_nonfinite_position_is_reported(gbg, dev):
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    field = gbg.ScalarFieldPhysical(torch.rand((8, 8, 8), dtype=torch.float64, device=dev), grid)
    pts = gbg.PointSet(torch.tensor([[1.0, 2.0, 3.0], [float("nan"), 1.0, 1.0]], dtype=torch.float64, device=dev))
    with pytest.raises(gbg.InexactError):
        gbg.interpolate(field, pts, gbg.CatmullRom)
    with pytest.raises(gbg.InexactError):
        gbg.anterpolate(grid, pts, gbg.ScalarPointValues(torch.ones(2, dtype=torch.float64, device=dev)), gbg.CatmullRom)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_traversal_order_matches_oracle_bitwise(gbg, oracle, dev, dtype):
    # test/point_traversal_order.jl:29-57; the device sort is stable, so it reproduces the
    # oracle's order exactly.
    grid, g = make(gbg, oracle, n=(16, 12, 20), domain=(TWO_PI, 2 * TWO_PI, 3 * TWO_PI),
                   origin=(-1, 0, 0.5), dtype=dtype)
    rng = np.random.default_rng(2026)
    M = 700
    pos = np.stack([-1 + TWO_PI * rng.random(M), 2 * TWO_PI * rng.random(M),
                    0.5 + 3 * TWO_PI * rng.random(M)], 1).astype(dtype)
    pos[:3] = [[np.nan, 0, 0], [np.inf, 1, 1], [-1e30, 2, 2]]
    points = gbg.PointSet(to_dev(pos, dev))
    for tile in (1, 2, 3, 4, 8, 32):
        got = gbg.point_traversal_order(grid, points, tile).indices.cpu().numpy()
        want = oracle.traversal_order(g, pos, tile)
        assert np.array_equal(got, want), tile
    with pytest.raises(gbg.ArgumentError):
        gbg.point_traversal_order(grid, points, 0)
    # in-place rebuild with caller scratch (point_traversal_order!)
    order = gbg.point_traversal_order(grid, points)
    storage = order.indices
    scratch = gbg.PointTraversalOrderScratch(grid, points)
    assert gbg.point_traversal_order_(order, grid, points, scratch) is order
    assert order.indices is storage
    assert np.array_equal(order.indices.cpu().numpy(), oracle.traversal_order(g, pos, 4))
    half = gbg.PointSet(points.positions[: M // 2])
    with pytest.raises(gbg.ArgumentError):
        gbg.point_traversal_order_(order, grid, points, gbg.PointTraversalOrderScratch(grid, half))
    with pytest.raises(gbg.ArgumentError):
        gbg.point_traversal_order_(order, grid, half, scratch)


def test_traversal_validation_on_device(gbg, dev):
    n = 50
    with pytest.raises(gbg.ArgumentError):
        gbg.PointTraversalOrder(torch.ones(n, dtype=torch.int32, device=dev))
    with pytest.raises(gbg.ArgumentError):
        gbg.PointTraversalOrder(torch.arange(2, n + 2, dtype=torch.int32, device=dev))
    gbg.PointTraversalOrder(torch.arange(n, 0, -1, dtype=torch.int32, device=dev))
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    field = gbg.ScalarFieldPhysical(torch.rand((8, 8, 8), dtype=torch.float64, device=dev), grid)
    pts = gbg.PointSet(TWO_PI * torch.rand((n, 3), dtype=torch.float64, device=dev))
    host_order = gbg.PointTraversalOrder(torch.arange(1, n + 1, dtype=torch.int32))
    with pytest.raises(gbg.ArgumentError):
        gbg.interpolate(field, pts, gbg.CatmullRom, traversal=host_order)


def test_config1_parity(gbg, oracle, dev):
    """64^3 Float64 scalar field from random Fourier modes, 1e5 uniform points, cubic:
    gather and scatter against the oracle, and the adjointness of the GPU pair."""
    from gbgperiodicfields_gb300.workloads import spectral_field, uniform_points
    grid = gbg.Grid3D((64, 64, 64), (TWO_PI,) * 3)
    g = oracle.grid_dict(grid.grid_size)
    f = spectral_field((64, 64, 64), 1, kmax=8, seed=1)[..., 0]
    pos = uniform_points(100_000, seed=2)
    q = np.random.default_rng(3).standard_normal(100_000)
    field = gbg.ScalarFieldPhysical(to_dev(f, dev), grid)
    points = gbg.PointSet(to_dev(pos, dev))
    got = gbg.interpolate(field, points, gbg.CatmullRom).data
    want = oracle.gather(g, f, pos, gbg.CatmullRom.coefficients)
    assert relerr(got.cpu().numpy()[:, None], want) <= 1e-13
    dep = gbg.anterpolate(grid, points, gbg.ScalarPointValues(to_dev(q, dev)), gbg.CatmullRom).data
    want_dep = oracle.scatter(g, np.zeros((64, 64, 64), order="F"), pos, q[:, None], gbg.CatmullRom.coefficients)
    assert relerr(dep.cpu().numpy(), want_dep) <= 1e-13
    lhs = torch.dot(got, torch.from_numpy(q).to(dev)).item()
    rhs = torch.sum(torch.from_numpy(f).to(dev) * dep).item()
    assert abs(lhs - rhs) / (got.norm().item() * np.linalg.norm(q)) <= 1e-13


def _abs_scatter(coeffs, n, pos, q, dx):
    """Per node and component, sum over points of |w_x w_y w_z| |q| (numpy, FP64): the
    magnitude that bounds the rounding error of any FP64 sum of the node's contributions."""
    n2 = coeffs.shape[0]
    half = n2 // 2
    ci = pos / dx
    base = np.floor(ci).astype(np.int64)
    t = ci - base
    w = []
    for d in range(3):
        # Horner over the powers, every node at once: w[p, i] = sum_r c[i, r] t_p^r
        acc = np.zeros((len(pos), n2))
        for r in range(coeffs.shape[1] - 1, -1, -1):
            acc = acc * t[:, d:d + 1] + coeffs[:, r][None, :]
        w.append(np.abs(acc))
    A = np.zeros(tuple(n) + (q.shape[1],))
    for i in range(n2):
        for j in range(n2):
            for k in range(n2):
                wt = w[0][:, i] * w[1][:, j] * w[2][:, k]
                ix = np.mod(base[:, 0] - half + 1 + i, n[0])
                iy = np.mod(base[:, 1] - half + 1 + j, n[1])
                iz = np.mod(base[:, 2] - half + 1 + k, n[2])
                for c in range(q.shape[1]):
                    np.add.at(A[..., c], (ix, iy, iz), wt * np.abs(q[:, c]))
    return A


@pytest.mark.parametrize("width", [4, 6])
def test_scatter_per_node_accuracy_across_magnitudes(gbg, oracle, dev, width):
    """Quantities spanning eight decades by region (1, 1e-3, 1e-6, 1e-8 by z slab), one
    component all zero and one scaled by 1e-4: every node of the FP64 scatter is within
    1e-12 of the sum of its contributions' magnitudes, as any FP64 sum of that node's
    contributions is (the reference's atomic adds included) -- not only relative to the
    largest value in the field -- and the zero component is exactly zero."""
    n = (24, 20, 32)
    grid, g = make(gbg, oracle, n=n)
    rng = np.random.default_rng(300 + width)
    M = 30000
    pos = np.asfortranarray(TWO_PI * rng.random((M, 3)))
    slab = np.minimum((pos[:, 2] / TWO_PI * 4).astype(int), 3)
    q = rng.standard_normal((M, 3)) * np.array([1.0, 1e-3, 1e-6, 1e-8])[slab][:, None]
    q[:, 1] = 0.0
    q[:, 2] *= 1e-4
    q = np.asfortranarray(q)
    scheme = gbg.CatmullRom if width == 4 else gbg.LalescuSpline(6)
    points = gbg.PointSet(to_dev(pos, dev))
    got = gbg.anterpolate(grid, points, gbg.VectorPointValues(to_dev(q, dev)), scheme).data.cpu().numpy()
    want = oracle.scatter(g, np.zeros(n + (3,), order="F"), pos, q, scheme.coefficients)
    A = _abs_scatter(np.asarray(scheme.coefficients), n, pos, q, TWO_PI / np.array(n))
    assert np.all(got[..., 1] == 0.0)
    err = np.abs(got - want)
    assert np.all(err <= 1e-12 * A), float(np.max(err / np.maximum(A, 1e-300)))
    # nodes reached only by the smallest slab's points (z cells 24..31): relative error per
    # node where the sum is not a cancellation
    half = width // 2
    zn = np.arange(n[2])
    small = (zn >= 3 * n[2] // 4 + half) & (zn <= n[2] - half)
    sel = np.abs(want[:, :, small, 0]) > 1e-3 * A[:, :, small, 0]
    rel = np.abs(got[:, :, small, 0] - want[:, :, small, 0])[sel] / np.abs(want[:, :, small, 0])[sel]
    assert rel.size > 100 and rel.max() <= 1e-11


def test_scatter_exact_zeros_on_nodes(gbg, oracle, dev):
    """Nodes the reference leaves exactly zero stay exactly zero: with Float64 positions on
    grid nodes, the nodes reached only with weight 0; in either precision, a component whose
    quantities are all zero."""
    n = (12, 10, 8)
    for dtype in (np.float64, np.float32):
        grid, g = make(gbg, oracle, n=n, dtype=dtype)
        rng = np.random.default_rng(11)
        cells = rng.integers(0, 8, size=(200, 3))
        pos = np.asfortranarray((cells * (TWO_PI / np.array(n))).astype(dtype))
        q = rng.standard_normal((200, 3)).astype(dtype)
        q[:, 2] = 0
        q = np.asfortranarray(q)
        points = gbg.PointSet(to_dev(pos, dev))
        got = gbg.anterpolate(grid, points, gbg.VectorPointValues(to_dev(q, dev)), gbg.CatmullRom).data.cpu().numpy()
        want = oracle.scatter(g, np.zeros(n + (3,), dtype, order="F"), pos, q, gbg.CatmullRom.coefficients)
        assert np.all(got[..., 2] == 0)
        if dtype == np.float64:
            assert (want == 0).sum() > 0.5 * want.size
            assert np.all(got[want == 0] == 0)
        assert relerr(got, want) <= TOL[dtype]
