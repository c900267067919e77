"""Pins the CPU oracle to the reference's own known-answer tests for the transfer path.

Each test names the reference test it restates (GBGPeriodicFields.jl,
test/interpolation_transfer.jl, test/point_traversal_order.jl and
test/exhaustive/references.jl).  The reference cannot run here (no Julia), so these
checks, written from the reference's tests, are what pins the oracle.
"""
import numpy as np
import pytest

TWO_PI = 2 * np.pi


def spline_weights(oracle, coeffs, t):
    # test/interpolation_transfer.jl:14 -- coefficients * [t^p for p in 0:M2-1]
    return coeffs @ np.array([t ** p for p in range(coeffs.shape[1])])


def sample(fn, grid, ncomp=1):
    """Fields.jl:484-503 -- values at x0 + (i-1)*dx in the grid's element type."""
    dt = grid["dtype"].type
    nx, ny, nz = grid["n"]
    o = [dt(v) for v in grid["origin"]]
    d = [dt(v) for v in grid["spacing"]]
    xs = o[0] + np.arange(nx, dtype=dt) * d[0]
    ys = o[1] + np.arange(ny, dtype=dt) * d[1]
    zs = o[2] + np.arange(nz, dtype=dt) * d[2]
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    vals = fn(X, Y, Z)
    if ncomp == 1:
        return np.asfortranarray(np.asarray(vals, dtype=dt))
    return np.asfortranarray(np.stack([np.asarray(v, dtype=dt) for v in vals], axis=-1))


# ------------------------------------------------------------- weights


@pytest.mark.parametrize("n,m", [(0, 0), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2), (2, 4),
                                 (3, 1), (3, 3)])
def test_partition_of_unity_lalescu(oracle, n, m):
    # interpolation_transfer.jl:19-26
    c = oracle.lalescu(2 * n + 2, m)
    for t in np.arange(0, 1.0001, 0.1):
        assert abs(spline_weights(oracle, c, t).sum() - 1.0) < 1e-12


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4])
def test_partition_of_unity_lagrange(oracle, n):
    # interpolation_transfer.jl:27-31
    c = oracle.lagrange(2 * n + 2)
    for t in np.arange(0, 1.0001, 0.1):
        assert abs(spline_weights(oracle, c, t).sum() - 1.0) < 1e-12


def test_catmull_rom_closed_form(oracle):
    # interpolation_transfer.jl:34-37
    def cr(t):
        return np.array([-0.5 * t + t ** 2 - 0.5 * t ** 3, 1 - 2.5 * t ** 2 + 1.5 * t ** 3,
                         0.5 * t + 2 * t ** 2 - 1.5 * t ** 3, -0.5 * t ** 2 + 0.5 * t ** 3])
    c = oracle.lalescu(4)
    for t in np.arange(0, 1.0001, 0.1):
        assert np.abs(spline_weights(oracle, c, t) - cr(t)).max() < 1e-12
        # the Horner evaluation the kernels use (Interpolation.jl:440-446) agrees too
        assert np.abs(oracle.axis_weights(c, t) - cr(t)).max() < 1e-12


@pytest.mark.parametrize("n", [1, 2, 3])
def test_linear_at_zero_smoothness(oracle, n):
    # interpolation_transfer.jl:41-49
    c = oracle.lalescu(2 * n + 2, 0)
    for t in np.arange(0, 1.0001, 0.1):
        w = spline_weights(oracle, c, t)
        assert abs(w[n] - (1 - t)) < 1e-12
        assert abs(w[n + 1] - t) < 1e-12
        rest = np.delete(w, [n, n + 1])
        assert np.abs(rest).sum() < 1e-12


@pytest.mark.parametrize("n", [1, 2, 3])
def test_lagrange_cardinal_basis(oracle, n):
    # interpolation_transfer.jl:52-60
    c = oracle.lagrange(2 * n + 2)
    offsets = np.arange(-n, n + 2)

    def lag(t):
        return np.array([np.prod([(t - offsets[j]) / (offsets[i] - offsets[j])
                                  for j in range(len(offsets)) if j != i])
                         for i in range(len(offsets))])
    for t in np.arange(0, 1.0001, 0.1):
        assert np.abs(spline_weights(oracle, c, t) - lag(t)).max() < 1e-10


def test_validity_refusals(oracle):
    # interpolation_transfer.jl:63-67
    oracle.lalescu(4, 2)
    for w, m in ((4, 3), (2, 1), (0, None)):
        with pytest.raises(ValueError):
            oracle.lalescu(w, m)
    with pytest.raises(ValueError):
        oracle.lagrange(0)


TURTLE = {
    # test/interpolation_transfer.jl:70-87: TurTLE's beta_n{n}_m{m}, deriv 0
    (1, 1): lambda x: [x * (x * (-x / 2 + 1) - 1 / 2), x ** 2 * (3 * x / 2 - 5 / 2) + 1,
                       x * (x * (-3 * x / 2 + 2) + 1 / 2), x ** 2 * (x / 2 - 1 / 2)],
    (1, 2): lambda x: [x * (x * (x * (x * (x - 5 / 2) + 3 / 2) + 1 / 2) - 1 / 2),
                       x ** 2 * (x * (x * (-3 * x + 15 / 2) - 9 / 2) - 1) + 1,
                       x * (x * (x * (x * (3 * x - 15 / 2) + 9 / 2) + 1 / 2) + 1 / 2),
                       x ** 3 * (x * (-x + 5 / 2) - 3 / 2)],
    (2, 1): lambda x: [x * (x * (x / 12 - 1 / 6) + 1 / 12), x * (x * (-7 * x / 12 + 5 / 4) - 2 / 3),
                       x ** 2 * (4 * x / 3 - 7 / 3) + 1, x * (x * (-4 * x / 3 + 5 / 3) + 2 / 3),
                       x * (x * (7 * x / 12 - 1 / 2) - 1 / 12), x ** 2 * (-x / 12 + 1 / 12)],
}


@pytest.mark.parametrize("nm", sorted(TURTLE))
def test_turtle_pins(oracle, nm):
    n, m = nm
    c = oracle.lalescu(2 * n + 2, m)
    for t in np.arange(0, 1.0001, 0.05):
        assert np.abs(spline_weights(oracle, c, t) - np.array(TURTLE[nm](t))).max() < 1e-12


def test_fornberg_known_weights(oracle):
    # The centred 3-point stencil: first derivative (-1/2, 0, 1/2), second (1, -2, 1).
    w = oracle.fornberg(0.0, [-1.0, 0.0, 1.0], 2)
    assert np.allclose(w[:, 0], [0, 1, 0], atol=1e-15)
    assert np.allclose(w[:, 1], [-0.5, 0, 0.5], atol=1e-15)
    assert np.allclose(w[:, 2], [1, -2, 1], atol=1e-15)


def test_walk_is_mod(oracle):
    # test/point_traversal_order.jl:238-272
    for extent in range(1, 13):
        for width in range(1, 17):
            nb = (width - 2) // 2
            for base in (-40, -7, -1, 0, 1, 5, 39, 1000, -1000, 10 ** 7, -10 ** 7):
                idx = oracle.walk(base, nb, extent, width)
                want = [(base + (i - nb)) % extent for i in range(width)]
                assert list(idx) == want


# ------------------------------------------------------------- transfers

@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_polynomial_reproduction(oracle, dtype):
    # interpolation_transfer.jl:96-124
    dt = np.dtype(dtype).type
    g = oracle.grid_dict((16, 15, 14), dtype=dtype)
    rng = np.random.default_rng(20260609)
    M = 64
    tol = 1e-10 if dtype == np.float64 else 1e-3
    coords = (dt(0.3 * TWO_PI) + dt(0.4 * TWO_PI) * rng.random((M, 3)).astype(dtype)).astype(dtype)
    lin = lambda x, y, z: dt(0.3) + dt(0.7) * x - dt(0.4) * y + dt(0.2) * z
    quad = lambda x, y, z: dt(1) + x - dt(0.5) * y ** 2 + dt(0.3) * x * z
    cr = oracle.lalescu(4)
    for fn in (lin, quad):
        v = oracle.gather(g, sample(fn, g), coords, cr)[:, 0]
        want = fn(coords[:, 0], coords[:, 1], coords[:, 2])
        assert np.allclose(v, want, rtol=tol)
    vf = sample(lambda x, y, z: (lin(x, y, z), -quad(x, y, z), dt(2) * lin(x, y, z)), g, 3)
    vv = oracle.gather(g, vf, coords, cr)
    X, Y, Z = coords.T
    assert np.allclose(vv, np.stack([lin(X, Y, Z), -quad(X, Y, Z), 2 * lin(X, Y, Z)], 1), rtol=tol)
    cubic = lambda x, y, z: dt(0.2) + x - dt(0.1) * y ** 3 + dt(0.4) * x * y * z
    inner = (dt(0.4 * TWO_PI) + dt(0.2 * TWO_PI) * rng.random((M, 3)).astype(dtype)).astype(dtype)
    vc = oracle.gather(g, sample(cubic, g), inner, oracle.lagrange(8))[:, 0]
    assert np.allclose(vc, cubic(*inner.T), rtol=1e-8 if dtype == np.float64 else 1e-2)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("R", [0, 1, 2])
def test_adjointness(oracle, dtype, R):
    # interpolation_transfer.jl:126-156 (including the measure-weighted form)
    g = oracle.grid_dict((16, 15, 14), dtype=dtype)
    rng = np.random.default_rng(7 + R)
    M, C = 64, 3 ** R
    tol = 1e-10 if dtype == np.float64 else 1e-3
    pos = (TWO_PI * rng.random((M, 3))).astype(dtype)
    f = np.asfortranarray(rng.random((16, 15, 14, C)).astype(dtype))
    q = np.asfortranarray(rng.random((M, C)).astype(dtype))
    Wf = oracle.gather(g, f, pos, oracle.lalescu(4))
    Wtq = oracle.scatter(g, np.zeros_like(f, order="F"), pos, q, oracle.lalescu(4))
    lhs = np.dot(Wf.ravel(order="F").astype(np.float64), q.ravel(order="F"))
    rhs = np.dot(f.ravel(order="F").astype(np.float64), Wtq.ravel(order="F"))
    assert abs(lhs - rhs) <= tol * abs(lhs)
    N = 16 * 15 * 14
    assert np.isclose(M * (lhs / (M * C)), N * (rhs / (N * C)), rtol=tol)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_conservation_alpha_beta(oracle, dtype):
    # interpolation_transfer.jl:158-180
    dt = np.dtype(dtype).type
    g = oracle.grid_dict((16, 15, 14), dtype=dtype)
    rng = np.random.default_rng(11)
    M = 64
    pos = (TWO_PI * rng.random((M, 3))).astype(dtype)
    q = rng.random((M, 1)).astype(dtype)
    cr = oracle.lalescu(4)
    shape = (16, 15, 14)
    dep = oracle.scatter(g, np.zeros(shape, dtype, order="F"), pos, q, cr)
    assert np.isclose(dep.sum(dtype=np.float64), q.sum(dtype=np.float64),
                      rtol=1e-10 if dtype == np.float64 else 1e-4)
    over = oracle.scatter(g, np.full(shape, np.nan, dtype, order="F"), pos, q, cr, dt(1), dt(0))
    assert np.isfinite(over).all()
    assert np.allclose(over, dep, rtol=1e-12 if dtype == np.float64 else 1e-4)
    scaled = oracle.scatter(g, dep.copy(order="F"), pos, q, cr, dt(3), dt(0))
    assert np.allclose(scaled, 3 * dep, rtol=1e-10 if dtype == np.float64 else 1e-3)
    acc = oracle.scatter(g, dep.copy(order="F"), pos, q, cr, dt(1), dt(1))
    assert np.allclose(acc, 2 * dep, rtol=1e-10 if dtype == np.float64 else 1e-3)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_periodicity(oracle, dtype):
    # interpolation_transfer.jl:182-188
    dt = np.dtype(dtype).type
    g = oracle.grid_dict((16, 15, 14), dtype=dtype)
    f = sample(lambda x, y, z: np.sin(x) + np.cos(2 * y) + np.sin(3 * z), g)
    base = np.array([[1.1, 2.2, 0.7]], dtype=dtype)
    shifted = (base + dt(TWO_PI) * np.array([[1, -1, 2]], dtype=dtype)).astype(dtype)
    a = oracle.gather(g, f, base, oracle.lalescu(4))
    b = oracle.gather(g, f, shifted, oracle.lalescu(4))
    assert np.allclose(a, b, rtol=1e-12 if dtype == np.float64 else 1e-4)


def _adjoint_ok(oracle, g, f, pos, q, c, rtol=1e-9):
    Wf = oracle.gather(g, f, pos, c)
    Wtq = oracle.scatter(g, np.zeros_like(f, order="F"), pos, q, c)
    lhs = np.dot(Wf.ravel(order="F"), np.asarray(q).ravel(order="F"))
    rhs = np.dot(f.ravel(order="F"), Wtq.ravel(order="F"))
    return np.isclose(lhs, rhs, rtol=rtol)


def _conserves(oracle, g, shape, pos, q, c, rtol=1e-9):
    dep = oracle.scatter(g, np.zeros(shape, order="F"), pos, q, c)
    return np.isclose(dep.sum(), np.asarray(q).sum(), rtol=rtol)


def test_adversarial_anisotropic_origin(oracle):
    # interpolation_transfer.jl:201-217
    g = oracle.grid_dict((10, 8, 12), domain=(TWO_PI, 0.5, 40.0), origin=(-1.3, 7.0, 100.0))
    rng = np.random.default_rng(3)
    M = 50
    dx = g["spacing"]
    org = g["origin"]
    ns = g["n"]
    coords = np.stack([org[d] + dx[d] * (1.5 + (ns[d] - 4) * rng.random(M)) for d in range(3)], 1)
    lin = lambda x, y, z: 0.5 + 0.3 * x - 1.1 * y + 0.02 * z
    v = oracle.gather(g, sample(lin, g), coords, oracle.lalescu(4))[:, 0]
    assert np.allclose(v, lin(*coords.T), rtol=1e-9)
    whole = np.stack([org[d] + g["domain"][d] * rng.random(M) for d in range(3)], 1)
    q = rng.random((M, 1))
    f = np.asfortranarray(rng.random((10, 8, 12)))
    assert _adjoint_ok(oracle, g, f, whole, q, oracle.lalescu(4))
    assert _conserves(oracle, g, (10, 8, 12), whole, q, oracle.lalescu(4))


def test_points_on_nodes(oracle):
    # interpolation_transfer.jl:219-227
    g = oracle.grid_dict((8, 8, 8))
    f = sample(lambda x, y, z: np.sin(x) * np.cos(y) + np.sin(z), g)
    dx = TWO_PI / 8
    idx = [(1, 1, 1), (3, 4, 5), (8, 8, 8), (1, 8, 4)]
    coords = np.array([[dx * (i[d] - 1) for d in range(3)] for i in idx])
    v = oracle.gather(g, f, coords, oracle.lalescu(4))[:, 0]
    want = [f[i[0] - 1, i[1] - 1, i[2] - 1] for i in idx]
    assert np.allclose(v, want, rtol=1e-12)


def test_stencil_wider_than_grid(oracle):
    # interpolation_transfer.jl:229-236
    g = oracle.grid_dict((4, 4, 4))
    rng = np.random.default_rng(5)
    pos = TWO_PI * rng.random((30, 3))
    q = rng.random((30, 1))
    f = np.asfortranarray(rng.random((4, 4, 4)))
    assert _adjoint_ok(oracle, g, f, pos, q, oracle.lagrange(8))
    assert _conserves(oracle, g, (4, 4, 4), pos, q, oracle.lagrange(8))


def test_heavy_contention(oracle):
    # interpolation_transfer.jl:238-246
    g = oracle.grid_dict((8, 8, 8))
    rng = np.random.default_rng(6)
    pos = 0.25 * rng.random((4000, 3))
    q = rng.random((4000, 1))
    assert _conserves(oracle, g, (8, 8, 8), pos, q, oracle.lalescu(4))
    assert _adjoint_ok(oracle, g, np.asfortranarray(rng.random((8, 8, 8))), pos, q, oracle.lalescu(4))


def test_tensor_order_three(oracle):
    # interpolation_transfer.jl:248-256
    g = oracle.grid_dict((6, 6, 6))
    rng = np.random.default_rng(8)
    pos = TWO_PI * rng.random((20, 3))
    f = np.asfortranarray(rng.random((6, 6, 6, 27)))
    q = np.asfortranarray(rng.random((20, 27)))
    assert oracle.gather(g, f, pos, oracle.lalescu(4)).shape == (20, 27)
    assert _adjoint_ok(oracle, g, f, pos, q, oracle.lalescu(4))
    dep = oracle.scatter(g, np.zeros((6, 6, 6, 27), order="F"), pos, q, oracle.lalescu(4))
    assert np.isclose(dep.sum(), q.sum(), rtol=1e-9)


def test_higher_smooth_schemes(oracle):
    # interpolation_transfer.jl:258-274
    g = oracle.grid_dict((20, 20, 20))
    rng = np.random.default_rng(9)
    M = 40
    dx = TWO_PI / 20
    coords = dx * (4.0 + 11.0 * rng.random((M, 3)))
    cubic = lambda x, y, z: 1.0 + x - 0.5 * y ** 2 + 0.3 * x * z - 0.05 * y ** 3
    whole = TWO_PI * rng.random((M, 3))
    q = rng.random((M, 1))
    for c in (oracle.lalescu(6, 1), oracle.lalescu(8, 2)):
        v = oracle.gather(g, sample(cubic, g), coords, c)[:, 0]
        assert np.allclose(v, cubic(*coords.T), rtol=1e-8)
        assert _adjoint_ok(oracle, g, np.asfortranarray(rng.random((20, 20, 20))), whole, q, c)
        assert _conserves(oracle, g, (20, 20, 20), whole, q, c)


def test_single_point_and_empty(oracle):
    # interpolation_transfer.jl:276-282 and 312-319
    g = oracle.grid_dict((8, 8, 8))
    pos = np.array([[1.1, 2.2, 0.7]])
    f = sample(lambda x, y, z: np.sin(x), g)
    assert oracle.gather(g, f, pos, oracle.lalescu(4)).shape == (1, 1)
    dep = oracle.scatter(g, np.zeros((8, 8, 8), order="F"), pos, np.array([[2.5]]), oracle.lalescu(4))
    assert np.isclose(dep.sum(), 2.5, rtol=1e-12)
    empty = np.zeros((0, 3))
    assert oracle.gather(g, f, empty, oracle.lalescu(4)).shape == (0, 1)
    dep0 = oracle.scatter(g, np.zeros((8, 8, 8), order="F"), empty, np.zeros((0, 1)), oracle.lalescu(4))
    assert np.abs(dep0).max() == 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_alpha_zero_is_pure_rescale(oracle, dtype):
    # interpolation_transfer.jl:292-296 (bitwise ==)
    dt = np.dtype(dtype).type
    g = oracle.grid_dict((8, 7, 6), dtype=dtype)
    rng = np.random.default_rng(31)
    pos = (TWO_PI * rng.random((5, 3))).astype(dtype)
    q = rng.random((5, 3)).astype(dtype)
    before = np.asfortranarray(rng.random((8, 7, 6, 3)).astype(dtype))
    dest = oracle.scatter(g, before.copy(order="F"), pos, q, oracle.lalescu(4), dt(0), dt(2))
    assert np.array_equal(dest, 2 * before)


def test_independent_catmull_rom_reference(oracle):
    """test/exhaustive/references.jl:590-654 -- an independent Catmull-Rom gather and
    scatter written from the closed-form weights, restated here in numpy."""
    def cr(t):
        return np.array([-0.5 * t ** 3 + t ** 2 - 0.5 * t, 1.5 * t ** 3 - 2.5 * t ** 2 + 1,
                         -1.5 * t ** 3 + 2 * t ** 2 + 0.5 * t, 0.5 * t ** 3 - 0.5 * t ** 2])

    g = oracle.grid_dict((9, 7, 8), origin=(0.3, -0.2, 1.0))
    N = np.array(g["n"])
    dx = np.array(g["spacing"])
    o = np.array(g["origin"])
    rng = np.random.default_rng(12)
    M = 37
    for R in (0, 1, 2):
        C = 3 ** R
        pos = o + np.array(g["domain"]) * (rng.random((M, 3)) * 1.2 - 0.1)
        f = np.asfortranarray(rng.random((9, 7, 8, C)))
        q = np.asfortranarray(rng.random((M, C)))
        flat = f.reshape((-1, C), order="F")
        ref_out = np.zeros((M, C))
        ref_dep = np.zeros_like(flat)
        for p in range(M):
            base = np.floor((pos[p] - o) / dx).astype(int)
            t = (pos[p] - o) / dx - base
            w = [cr(t[d]) for d in range(3)]
            for i in range(4):
                for j in range(4):
                    for k in range(4):
                        n1 = (base[0] + i - 1) % N[0]
                        n2 = (base[1] + j - 1) % N[1]
                        n3 = (base[2] + k - 1) % N[2]
                        ww = w[0][i] * w[1][j] * w[2][k]
                        idx = n1 + N[0] * n2 + N[0] * N[1] * n3
                        ref_out[p] += ww * flat[idx]
                        ref_dep[idx] += ww * q[p]
        out = oracle.gather(g, f, pos, oracle.lalescu(4))
        dep = oracle.scatter(g, np.zeros_like(f, order="F"), pos, q, oracle.lalescu(4))
        assert np.allclose(out, ref_out, rtol=1e-12, atol=1e-13)
        assert np.allclose(dep.reshape((-1, C), order="F"), ref_dep, rtol=1e-12, atol=1e-13)


def test_traversal_is_invariant_for_gather(oracle):
    # test/point_traversal_order.jl:60-117 (the gather is bitwise equal under any order)
    g = oracle.grid_dict((14, 16, 12), domain=(TWO_PI, TWO_PI, 2 * TWO_PI), origin=(0.25, -2, 0))
    rng = np.random.default_rng(4242)
    M = 600
    pos = np.stack([0.25 + TWO_PI * rng.random(M), -2 + TWO_PI * rng.random(M),
                    2 * TWO_PI * rng.random(M)], 1)
    f = np.asfortranarray(rng.random((14, 16, 12, 3)))
    order = oracle.traversal_order(g, pos)
    for c in (oracle.lalescu(4), oracle.lalescu(6, 1), oracle.lagrange(4)):
        a = oracle.gather(g, f, pos, c)
        b = oracle.gather(g, f, pos, c, traversal=order)
        r = oracle.gather(g, f, pos, c, traversal=order[::-1].copy())
        assert np.array_equal(a, b) and np.array_equal(a, r)


# ------------------------------------------------------------ traversal order

@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_traversal_order_is_sorted_bijection(oracle, dtype):
    # test/point_traversal_order.jl:29-57
    dt = np.dtype(dtype).type
    g = oracle.grid_dict((16, 12, 20), domain=(TWO_PI, 2 * TWO_PI, 3 * TWO_PI),
                         origin=(-1, 0, 0.5), dtype=dtype)
    rng = np.random.default_rng(2026)
    M = 700
    pos = np.stack([dt(-1) + dt(TWO_PI) * rng.random(M).astype(dtype),
                    dt(2 * TWO_PI) * rng.random(M).astype(dtype),
                    dt(0.5) + dt(3 * TWO_PI) * rng.random(M).astype(dtype)], 1).astype(dtype)
    for tile in (1, 2, 3, 4, 8, 32):
        order = oracle.traversal_order(g, pos, tile)
        assert sorted(order.tolist()) == list(range(1, M + 1))
        tiles = [max(-(-g["n"][d] // tile), 1) for d in range(3)]
        edge = [dt(g["domain"][d]) / dt(tiles[d]) for d in range(3)]

        def key(p):
            i = [min(max(int(np.floor((pos[p, d] - dt(g["origin"][d])) / edge[d])), 0), tiles[d] - 1)
                 for d in range(3)]
            return 1 + i[0] + tiles[0] * (i[1] + tiles[1] * i[2])
        keys = [key(p - 1) for p in order]
        assert keys == sorted(keys)
    with pytest.raises(ValueError):
        oracle.traversal_order(g, pos, 0)
    assert len(oracle.traversal_order(g, np.zeros((0, 3), dtype))) == 0
    far = np.full((3, 3), 1000, dtype=dtype)
    assert sorted(oracle.traversal_order(g, far).tolist()) == [1, 2, 3]


def test_tile_index_saturates(oracle):
    # test/point_traversal_order.jl:212-235
    inv = 64 / TWO_PI
    assert oracle.tile_index(np.nan, 0.0, inv, 64) == 0
    assert oracle.tile_index(np.inf, 0.0, inv, 64) == 63
    assert oracle.tile_index(-np.inf, 0.0, inv, 64) == 0
    assert oracle.tile_index(1e300, 0.0, inv, 64) == 63
    assert oracle.tile_index(-1e300, 0.0, inv, 64) == 0
    assert oracle.tile_index(0.0, 0.0, inv, 64) == 0
    tiles = (1300, 1300, 1300)
    far = [t - 1 for t in tiles]
    key = 2 + far[0] + tiles[0] * (far[1] + tiles[1] * far[2])
    assert key == np.prod(tiles, dtype=np.int64) + 1
    wild = np.array([[np.nan, 0.0, 0.0], [np.inf, 1.0, 1.0], [-np.inf, 2.0, 2.0], [1e300, 3.0, 3.0]])
    assert len(oracle.traversal_order(oracle.grid_dict((8, 8, 8)), wild)) == 4


def test_wrap_coordinate(oracle):
    # Points.jl:1245-1249: mod into [o, o+L), the excluded endpoint folded, non-finite passes.
    L = TWO_PI
    assert oracle.wrap_coordinate(L + 0.5, L, 0.0) == pytest.approx(0.5)
    assert oracle.wrap_coordinate(-0.5, L, 0.0) == pytest.approx(L - 0.5)
    assert oracle.wrap_coordinate(-1e-300, L, 0.0) == 0.0  # r + y rounds to y, folded to 0
    assert np.isnan(oracle.wrap_coordinate(np.inf, L, 0.0))
    assert oracle.wrap_coordinate(3.0, 2.0, 1.5) == 3.0  # already in [1.5, 3.5)
    assert oracle.wrap_coordinate(3.6, 2.0, 1.5) == pytest.approx(1.6)
