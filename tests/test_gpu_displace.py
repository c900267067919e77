"""GPU tests of displace!/wrap! (Points.jl:1382-1490) and of the fused displace + re-bin
of the resident form, following the reference's test/displacement.jl cases (values
regenerated here): the n-term displacement equals the term-by-term sum bitwise, the
destination/source and aliased forms, zero terms, torus displacement == cover displacement
then wrap! bitwise, the fold of the excluded endpoint, non-finite coordinates, the domain
following the origin.  Parity with the oracle's restatement is bitwise (the arithmetic is
the reference's: products and sums rounded separately, Julia's float mod)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TWO_PI = 2 * np.pi


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def setup(gbg, T, M=257, seed=3):
    rng = np.random.default_rng(seed)
    L = (TWO_PI, 2 * TWO_PI, 3 * TWO_PI)
    tdt = torch.float64 if T == np.float64 else torch.float32
    grid = gbg.Grid3D((8, 12, 16), L, dtype=tdt)
    X0 = np.asfortranarray((rng.random((M, 3)) * TWO_PI).astype(T))
    secs = [np.asfortranarray(rng.standard_normal((M, 3)).astype(T)) for _ in range(3)]
    coefs = (0.31, -1.2, 0.07)
    return grid, X0, secs, coefs, tdt


def ps(gbg, a):
    return gbg.PointSet(torch.from_numpy(np.asfortranarray(a)).cuda())


def vpv(gbg, a):
    return gbg.VectorPointValues(torch.from_numpy(np.asfortranarray(a)).cuda())


def pos(p):
    return p.positions.cpu().numpy()


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_cover_displacement_bitwise(gbg, oracle, dev, T):
    grid, X0, secs, coefs, _ = setup(gbg, T)
    points = ps(gbg, X0)
    assert gbg.displace_(points, (coefs[0], vpv(gbg, secs[0]))) is points
    assert np.array_equal(pos(points), X0 + T(coefs[0]) * secs[0])
    points = ps(gbg, X0)
    gbg.displace_(points, *[(c, vpv(gbg, v)) for c, v in zip(coefs, secs)])
    want = X0.copy()
    for c, v in zip(coefs, secs):
        want += T(c) * v
    assert np.array_equal(pos(points), want)
    assert np.array_equal(pos(points), oracle.displace(X0, list(zip(coefs, secs))))


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_destination_source_and_aliased_forms(gbg, oracle, dev, T):
    grid, X0, secs, coefs, _ = setup(gbg, T)
    source, dest = ps(gbg, X0), ps(gbg, np.zeros_like(X0))
    terms = [(coefs[0], vpv(gbg, secs[0])), (coefs[1], vpv(gbg, secs[1]))]
    gbg.displace_(dest, source, *terms)
    assert np.array_equal(pos(source), X0)
    assert np.array_equal(pos(dest), (X0 + T(coefs[0]) * secs[0]) + T(coefs[1]) * secs[1])
    aliased = ps(gbg, X0)
    gbg.displace_(aliased, aliased, *terms)
    assert np.array_equal(pos(aliased), pos(dest))
    # zero terms copy; with a grid, copy and wrap
    d2 = ps(gbg, np.ones_like(X0))
    gbg.displace_(d2, source)
    assert np.array_equal(pos(d2), X0)


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_torus_displacement_equals_cover_then_wrap(gbg, oracle, dev, T):
    grid, X0, secs, coefs, _ = setup(gbg, T)
    g = {"domain": grid.domain_size, "origin": grid.origin}
    terms = [(c, vpv(gbg, v)) for c, v in zip(coefs, secs)]
    fused, unfused = ps(gbg, X0), ps(gbg, X0)
    gbg.displace_(fused, grid, *terms)
    gbg.displace_(unfused, *terms)
    gbg.wrap_(unfused, grid)
    assert np.array_equal(pos(fused), pos(unfused))
    assert np.array_equal(pos(fused), oracle.displace(X0, list(zip(coefs, secs)), g))
    for a in range(3):
        col = pos(fused)[:, a]
        assert (col >= 0).all() and (col < T(grid.domain_size[a])).all()
    # far positions (ten periods out) come back to the same representative up to roundoff
    far_in = X0 + T(10) * np.array(grid.domain_size, dtype=T)[None, :]
    far = ps(gbg, far_in)
    gbg.displace_(far, far, grid)
    assert np.array_equal(pos(far), oracle.displace(far_in, [], g))


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_wrap_edge_cases(gbg, oracle, dev, T):
    grid, X0, secs, coefs, tdt = setup(gbg, T)
    g = {"domain": grid.domain_size, "origin": grid.origin}
    tiny = -np.finfo(T).eps * T(16)
    p = ps(gbg, np.array([[tiny, tiny, tiny], [-1e-20, -1e-30, 0.0]], dtype=T))
    gbg.wrap_(p, grid)
    got = pos(p)
    for a in range(3):
        assert (got[:, a] >= 0).all() and (got[:, a] < T(grid.domain_size[a])).all()
    nonfinite = np.array([[np.nan, 1, 1], [np.inf, 1, 1], [-np.inf, 1, 1]], dtype=T)
    p = ps(gbg, nonfinite)
    gbg.wrap_(p, grid)
    got = pos(p)
    assert np.isnan(got[:, 0]).all() and np.isfinite(got[:, 1:]).all()
    # the fundamental domain follows the origin
    shifted = gbg.Grid3D((8, 12, 16), grid.domain_size, origin=(1.0, -2.0, 0.5), dtype=tdt)
    rng = np.random.default_rng(9)
    raw = (rng.random((257, 3)) * 40 - 20).astype(T)
    p = ps(gbg, raw)
    gbg.wrap_(p, shifted)
    got = pos(p)
    assert np.array_equal(got, oracle.displace(raw, [], {"domain": shifted.domain_size, "origin": shifted.origin}))
    for a in range(3):
        o = T(shifted.origin[a])
        assert (got[:, a] >= o).all() and (got[:, a] < o + T(shifted.domain_size[a])).all()


def test_fused_displace_rebin_equals_displace_then_build(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(4)
    grid = gbg.Grid3D((24, 20, 18), (TWO_PI,) * 3, origin=(0.2, -0.3, 0.1))
    M, C = 5000, 3
    X0 = np.asfortranarray(np.array(grid.origin) + TWO_PI * rng.random((M, 3)))
    v = np.asfortranarray(rng.standard_normal((M, 3)))
    src = torch.from_numpy(X0).cuda()
    vt = torch.from_numpy(v).cuda()
    # fused: displace by 0.4 * v, wrap, and bin in one pass
    dst = gbg.empty_colmajor((M, 3), torch.float64, "cuda")
    fused = resident.PointBins(grid, M).build_displaced(dst, src, [(0.4, vt)], wrap=True)
    # unfused: displace_ + wrap through the drop-in API, then build
    moved = gbg.PointSet(src.clone())
    gbg.displace_(moved, grid, (0.4, gbg.VectorPointValues(vt)))
    assert torch.equal(dst, moved.positions)
    plain = resident.PointBins(grid, M).build(moved.positions)
    assert torch.equal(fused.order(), plain.order())
    f = np.asfortranarray(rng.standard_normal(grid.grid_size + (C,)))
    field = resident.ResidentField(grid, C, max_stencil_width=4).load(torch.from_numpy(f).cuda())
    a = resident.interpolate_binned(field, fused, gbg.CatmullRom)
    b = resident.interpolate_binned(field, plain, gbg.CatmullRom)
    assert torch.equal(a, b)
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    want = oracle.gather(g, f, dst.cpu().numpy(), gbg.CatmullRom.coefficients)
    assert np.abs(a.double().cpu().numpy() - want).max() / np.abs(want).max() <= 1e-5
    # in place (dst is src) gives the same positions
    src2 = torch.from_numpy(X0).cuda()
    resident.PointBins(grid, M).build_displaced(src2, src2, [(0.4, vt)], wrap=True)
    assert torch.equal(src2, dst)


def test_permute_keeps_state_binned(gbg, dev):
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(5)
    grid = gbg.Grid3D((16, 16, 16), (TWO_PI,) * 3)
    M = 3000
    x = torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((M, 3)))).cuda()
    q = gbg.colmajor(torch.randn((M, 4), device="cuda"))
    bins = resident.PointBins(grid, M).build(x)
    perm = bins.order().long() - 1
    assert torch.equal(bins.permute(x), x[perm])
    assert torch.equal(bins.permute(q), q[perm])
    # after the permutation the points are in binned order: rebuilding gives the identity
    again = resident.PointBins(grid, M).build(bins.permute(x))
    assert torch.equal(again.order().long() - 1, torch.arange(M, device="cuda"))


def test_particle_loop_matches_oracle(gbg, oracle, dev):
    """Three steps of x <- wrap(x + dt * u(x)) with the FP64 drop-in gather and
    displace_, against the same loop on the oracle: positions within 1e-12."""
    rng = np.random.default_rng(6)
    grid = gbg.Grid3D((20, 18, 16), (TWO_PI,) * 3)
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    u = np.asfortranarray(rng.standard_normal(grid.grid_size + (3,)))
    field = gbg.VectorFieldPhysical(torch.from_numpy(u).cuda(), grid)
    x_h = np.asfortranarray(TWO_PI * rng.random((400, 3)))
    pts = gbg.PointSet(torch.from_numpy(x_h).cuda())
    dt = 0.05
    for _ in range(3):
        vel = gbg.interpolate(field, pts, gbg.CatmullRom)
        gbg.displace_(pts, grid, (dt, vel))
        v_h = oracle.gather(g, u, x_h, gbg.CatmullRom.coefficients)
        x_h = oracle.displace(x_h, [(dt, v_h)], {"domain": grid.domain_size, "origin": grid.origin})
    assert np.abs(pts.positions.cpu().numpy() - x_h).max() <= 1e-12
