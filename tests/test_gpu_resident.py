"""GPU tests of the resident precision form: FP32 ghost-padded storage, FP64 positions
binned on the device, the TMA-staged gather and the deterministic scatter.

Errors are measured against the FP64 oracle on the FP64 field, relative to max|oracle|:
the precision form's bar is 1e-5.  The binned order is integer work and is compared
bitwise with a host-side stable sort of the same keys."""
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


def relerr(got, want):
    return np.abs(np.asarray(got, np.float64) - want).max() / max(np.abs(want).max(), 1e-300)


def setup(gbg, oracle, n, ncomp, m, seed, origin=(0.0, 0.0, 0.0), brick=None, width=6):
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(seed)
    grid = gbg.Grid3D(n, (TWO_PI,) * 3, origin=origin)
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    f = np.asfortranarray(rng.standard_normal(n + (ncomp,)))
    pos = np.asfortranarray(np.array(origin) + TWO_PI * (rng.random((m, 3)) * 1.3 - 0.15))
    q = np.asfortranarray(rng.standard_normal((m, ncomp)))
    field = resident.ResidentField(grid, ncomp, max_stencil_width=width).load(torch.from_numpy(f).cuda())
    bins = resident.PointBins(grid, m, brick=brick).build(torch.from_numpy(pos).cuda())
    return resident, grid, g, f, pos, q, field, bins


@pytest.mark.parametrize("ncomp", [1, 3, 9, 12])
@pytest.mark.parametrize("width", [2, 4, 6, 8])
def test_staged_gather_matches_fp64_oracle(gbg, oracle, dev, ncomp, width):
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (24, 20, 18), ncomp, 3000, 10 + width,
                                                       origin=(0.3, -0.7, 1.1), width=8)
    scheme = {2: gbg.LalescuSpline(2, 0), 4: gbg.CatmullRom, 6: gbg.LalescuSpline(6), 8: gbg.LagrangeSpline(8)}[width]
    got = resident.interpolate_binned(field, bins, scheme, dtype=torch.float64).cpu().numpy()
    want = oracle.gather(g, f, pos, scheme.coefficients)
    assert relerr(got, want) <= 1e-5
    # and against the FP64 oracle on the FP32-rounded field: the arithmetic alone
    f32 = np.asfortranarray(f.astype(np.float32).astype(np.float64))
    assert relerr(got, oracle.gather(g, f32, pos, scheme.coefficients)) <= 2e-6


@pytest.mark.parametrize("ncomp", [1, 3, 12])
@pytest.mark.parametrize("width", [4, 6])
def test_staged_scatter_matches_fp64_oracle_and_is_deterministic(gbg, oracle, dev, ncomp, width):
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (20, 22, 18), ncomp, 4000, 30 + width)
    scheme = gbg.CatmullRom if width == 4 else gbg.LalescuSpline(6)
    qt = torch.from_numpy(q).cuda()
    resident.anterpolate_binned(field, bins, scheme, qt, 1.0, 0.0)
    a = field.read()
    want = oracle.scatter(g, np.zeros(grid.grid_size + (ncomp,), order="F"), pos, q, scheme.coefficients)
    assert relerr(a.cpu().numpy(), want) <= 1e-5
    resident.anterpolate_binned(field, bins, scheme, qt, 1.0, 0.0)
    assert torch.equal(a, field.read())
    # alpha / beta: field = 2*W^T q - 0.5*field
    resident.anterpolate_binned(field, bins, scheme, qt, 2.0, -0.5)
    want2 = 2 * want - 0.5 * want
    assert relerr(field.read().cpu().numpy(), want2) <= 1e-5


def test_clustered_points_and_empty_bins(gbg, oracle, dev):
    from gbgperiodicfields_gb300.workloads import clustered_points
    resident, grid, g, f, _, _, field, bins = setup(gbg, oracle, (32, 32, 32), 3, 10, 5)
    pos = clustered_points(20000, seed=4, nblobs=5, sigma=0.05)
    q = np.asfortranarray(np.random.default_rng(6).standard_normal((20000, 3)))
    bins = resident.PointBins(grid, 20000).build(torch.from_numpy(pos).cuda())
    got = resident.interpolate_binned(field, bins, gbg.CatmullRom, dtype=torch.float64).cpu().numpy()
    assert relerr(got, oracle.gather(g, f, pos, gbg.CatmullRom.coefficients)) <= 1e-5
    resident.anterpolate_binned(field, bins, gbg.CatmullRom, torch.from_numpy(q).cuda())
    want = oracle.scatter(g, np.zeros((32, 32, 32, 3), order="F"), pos, q, gbg.CatmullRom.coefficients)
    assert relerr(field.read().cpu().numpy(), want) <= 1e-5
    # zero points: the scatter with beta = 0 clears the field
    empty = resident.PointBins(grid, 0).build(torch.zeros((0, 3), dtype=torch.float64, device="cuda"))
    resident.anterpolate_binned(field, empty, gbg.CatmullRom, torch.zeros((0, 3), dtype=torch.float64, device="cuda"))
    assert field.read().abs().max().item() == 0.0


def test_bins_order_is_a_stable_brick_sort(gbg, oracle, dev):
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (30, 26, 22), 3, 5000, 8, brick=(11, 8, 8))
    order = bins.order().cpu().numpy()
    # host restatement of the keys: brick-major, then cell within the brick
    n = np.array(grid.grid_size)
    b = np.array([11, 8, 8])
    nb = -(-n // b)
    inv = n / np.array(grid.domain_size)
    u = np.floor((pos - np.array(grid.origin)) * inv).astype(np.int64)
    c = np.mod(u, n)
    br = c // b
    loc = c - br * b
    key = ((br[:, 2] * nb[1] + br[:, 1]) * nb[0] + br[:, 0]) * b.prod() + (loc[:, 2] * b[1] + loc[:, 1]) * b[0] + loc[:, 0]
    want = np.argsort(key, kind="stable") + 1
    assert np.array_equal(order, want)


def test_positions_far_outside_wrap(gbg, oracle, dev):
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (16, 16, 16), 3, 500, 9)
    shifted = pos + TWO_PI * np.array([3.0, -7.0, 12.0])
    b2 = resident.PointBins(grid, 500).build(torch.from_numpy(np.asfortranarray(shifted)).cuda())
    a = resident.interpolate_binned(field, bins, gbg.CatmullRom).cpu().numpy()
    b = resident.interpolate_binned(field, b2, gbg.CatmullRom).cpu().numpy()
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()


def test_nonfinite_position_flagged(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import resident
    grid = gbg.Grid3D((16, 16, 16), (TWO_PI,) * 3)
    pos = torch.tensor([[1.0, 2.0, 3.0], [float("nan"), 0.0, 0.0]], dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    resident.PointBins(grid, 2).build(pos, status)
    torch.cuda.synchronize()
    assert int(status.item()) & gbg._lib.GBG_DEV_NONFINITE


def test_bins_order_with_a_crowded_cell(gbg, oracle, dev):
    """A cell holding more than 1024 points sends the counting sort to the radix sort: the
    order is still the stable brick sort."""
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (20, 18, 16), 3, 3000, 41, brick=(11, 8, 8))
    rng = np.random.default_rng(42)
    crowd = np.asfortranarray(np.vstack([pos, np.full((2500, 3), 0.5) + 0.01 * rng.random((2500, 3))]))
    bins = resident.PointBins(grid, len(crowd), brick=(11, 8, 8)).build(torch.from_numpy(crowd).cuda())
    order = bins.order().cpu().numpy()
    n = np.array(grid.grid_size)
    b = np.array([11, 8, 8])
    nb = -(-n // b)
    c = np.mod(np.floor((crowd - np.array(grid.origin)) * (n / np.array(grid.domain_size))).astype(np.int64), n)
    br = c // b
    loc = c - br * b
    key = ((br[:, 2] * nb[1] + br[:, 1]) * nb[0] + br[:, 0]) * b.prod() + (loc[:, 2] * b[1] + loc[:, 1]) * b[0] + loc[:, 0]
    assert np.array_equal(order, np.argsort(key, kind="stable") + 1)
    # the points' records follow that order too (the fallback gathers them again)
    got = resident.interpolate_binned(field, bins, gbg.CatmullRom, dtype=torch.float64).cpu().numpy()
    assert relerr(got, oracle.gather(g, f, crowd, gbg.CatmullRom.coefficients)) <= 1e-5


def test_nonfinite_quantity_is_reported(gbg, oracle, dev):
    """A NaN quantity in the binned scatter sets GBG_DEV_NONFINITE in the status word."""
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (16, 16, 16), 3, 2000, 51)
    q = q.copy(order="F")
    q[100, 1] = np.nan
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    resident.anterpolate_binned(field, bins, gbg.CatmullRom, torch.from_numpy(q).cuda(), 1.0, 0.0, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) & gbg._lib.GBG_DEV_NONFINITE


def test_compensated_scatter_at_high_coverage(gbg, oracle, dev):
    """Thousands of points per cell (400000 points in eight neighbouring cells): every node
    sums of order 10^5 contributions of one sign.  One plain FP32 running sum per node
    drifts with the number of terms; compensated summation of the chunk sums stays at the
    FP32 rounding of the weights and quantities.  Errors against the FP64 oracle, relative
    to max|oracle| (the precision form's bar is 1e-5)."""
    from gbgperiodicfields_gb300 import resident
    grid = gbg.Grid3D((16, 16, 16), (TWO_PI,) * 3)
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    rng = np.random.default_rng(31)
    m = 400_000
    h = TWO_PI / 16
    cells = rng.integers(6, 8, size=(m, 3))
    pos = np.asfortranarray((cells + rng.random((m, 3))) * h)
    q = np.asfortranarray(1.0 + 0.1 * rng.standard_normal((m, 3)))
    want = oracle.scatter(g, np.zeros((16, 16, 16, 3), order="F"), pos, q, gbg.CatmullRom.coefficients)
    field = resident.ResidentField(grid, 3, max_stencil_width=4)
    bins = resident.PointBins(grid, m).build(torch.from_numpy(pos).cuda())
    qt = torch.from_numpy(q).cuda()
    errs = {}
    for comp in (True, False):
        bins.set_compensated(comp)
        resident.anterpolate_binned(field, bins, gbg.CatmullRom, qt, 1.0, 0.0)
        errs[comp] = relerr(field.read().cpu().numpy(), want)
    assert errs[True] <= 1e-6, errs
    assert errs[True] * 10 <= errs[False], errs


def test_compensation_leaves_single_chunk_regions_unchanged(gbg, oracle, dev):
    """At ordinary densities every brick region fits in one chunk: the compensated and the
    plain scatter give the same bits."""
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (32, 24, 20), 12, 3000, 61)
    qt = torch.from_numpy(q).cuda()
    out = []
    for comp in (True, False):
        bins.set_compensated(comp)
        resident.anterpolate_binned(field, bins, gbg.CatmullRom, qt, 1.0, 0.0)
        out.append(field.read())
    assert torch.equal(out[0], out[1])


@pytest.mark.parametrize("ncomp", [3, 12])
@pytest.mark.parametrize("width", [2, 4, 6, 8])
def test_direct_gather_of_sparse_points(gbg, oracle, dev, ncomp, width):
    """A point set sparse on its grid (under four points a brick) is gathered straight from
    the field, with the staged kernels' per-point arithmetic: it matches the oracle, and a
    point's values are bitwise those it gets inside a dense set (staged tiles)."""
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(90 + width)
    n = (40, 36, 32)
    grid = gbg.Grid3D(n, (TWO_PI,) * 3, origin=(0.2, -0.4, 0.6))
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    f = np.asfortranarray(rng.standard_normal(n + (ncomp,)))
    field = resident.ResidentField(grid, ncomp, max_stencil_width=8).load(torch.from_numpy(f).cuda())
    scheme = {2: gbg.LalescuSpline(2, 0), 4: gbg.CatmullRom, 6: gbg.LalescuSpline(6), 8: gbg.LagrangeSpline(8)}[width]
    dense = np.asfortranarray(np.array(grid.origin) + TWO_PI * (rng.random((60000, 3)) * 1.2 - 0.1))
    sparse = np.asfortranarray(dense[:25])
    got = {}
    for name, pos in (("sparse", sparse), ("dense", dense)):
        bins = resident.PointBins(grid, pos.shape[0], brick=(11, 8, 8)).build(torch.from_numpy(pos).cuda())
        assert (pos.shape[0] < 4 * bins_count(bins)) == (name == "sparse")
        got[name] = resident.interpolate_binned(field, bins, scheme, dtype=torch.float32).cpu()
    assert torch.equal(got["sparse"], got["dense"][:25])
    want = oracle.gather(g, f, sparse, scheme.coefficients)
    assert relerr(got["sparse"].double().numpy(), want) <= 1e-5


@pytest.mark.parametrize("ncomp", [3, 12])
@pytest.mark.parametrize("width", [2, 4, 6, 8])
@pytest.mark.parametrize("beta", [0.0, 1.0, 0.5])
def test_sparse_scatter_regions_from_neighbour_lists(gbg, oracle, dev, ncomp, width, beta):
    """A sparse set's scatter builds each brick's region from the neighbouring bricks' point
    lists: bitwise the result of the per-cell tables, and within the bar of the oracle --
    including points in one cell and across the periodic wrap."""
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(120 + width)
    n = (40, 36, 32)
    grid = gbg.Grid3D(n, (TWO_PI,) * 3, origin=(0.2, -0.4, 0.6))
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    scheme = {2: gbg.LalescuSpline(2, 0), 4: gbg.CatmullRom, 6: gbg.LalescuSpline(6), 8: gbg.LagrangeSpline(8)}[width]
    pos = np.array(grid.origin) + TWO_PI * (rng.random((200, 3)) * 1.2 - 0.1)
    pos[:5] = pos[5]                                   # a crowded cell
    pos[10:14] = np.array(grid.origin) + 1e-9          # at the wrap
    pos = np.asfortranarray(pos)
    q = np.asfortranarray(rng.standard_normal((200, ncomp)))
    prior = np.asfortranarray(rng.standard_normal(n + (ncomp,)))
    bins = resident.PointBins(grid, 200, brick=(11, 8, 8)).build(torch.from_numpy(pos).cuda())
    assert 200 < 4 * bins_count(bins)
    outs = []
    for allow in (True, False):
        bins.set_sparse_regions(allow)
        dest = resident.ResidentField(grid, ncomp, max_stencil_width=8).load(torch.from_numpy(prior).cuda())
        resident.anterpolate_binned(dest, bins, scheme, torch.from_numpy(q).cuda(), 1.0, beta)
        outs.append(dest.read())
    assert torch.equal(outs[0], outs[1])
    want = oracle.scatter(g, prior.copy(order="F"), pos, q, scheme.coefficients, 1.0, beta)
    assert relerr(outs[0].cpu().numpy(), want) <= 1e-5


def bins_count(bins):
    nb = [-(-n // b) for n, b in zip(bins.grid.grid_size, bins.brick)]
    return nb[0] * nb[1] * nb[2]


@pytest.mark.parametrize("comp", [True, False], ids=["compensated", "plain"])
def test_multi_chunk_scatter_is_independent_of_the_launch_shape(gbg, oracle, dev, comp):
    """Dense points make every brick region span several chunks; the chunks, and so where
    the compensated summation folds, depend on the brick alone, so every threads-per-CTA
    choice gives the same bits -- and both stay within the precision form's bar."""
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (24, 20, 16), 12, 120000, 83)
    bins.set_compensated(comp)
    qt = torch.from_numpy(q).cuda()
    outs = []
    for threads in (0, 64, 128, 256):
        bins.set_launch(0, threads)
        resident.anterpolate_binned(field, bins, gbg.CatmullRom, qt, 1.0, 0.0)
        outs.append(field.read())
    for o in outs[1:]:
        assert torch.equal(o, outs[0])
    want = oracle.scatter(g, np.zeros(grid.grid_size + (12,), order="F"), pos, q, gbg.CatmullRom.coefficients)
    assert relerr(outs[0].cpu().numpy(), want) <= 1e-5


def test_plain_scatter_is_independent_of_brick_and_chunking(gbg, oracle, dev):
    """Plain FP32 running sums carry across chunks exactly, and a node's order (its stencil's
    rows z outer, y inner, then its points in binned order) is the same whatever brick holds
    it; so dense points scattered with a brick whose regions fit one chunk and with one
    whose regions need several give the same bits."""
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(131)
    n = (30, 24, 24)
    grid = gbg.Grid3D(n, (TWO_PI,) * 3)
    m = 2 * n[0] * n[1] * n[2]
    pos = torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((m, 3)))).cuda()
    q = torch.from_numpy(np.asfortranarray(rng.standard_normal((m, 12)))).float().cuda()
    outs = []
    for brick in ((3, 4, 4), (15, 8, 8)):
        bins = resident.PointBins(grid, m, brick=brick).build(pos)
        bins.set_compensated(False)
        dest = resident.ResidentField(grid, 12, max_stencil_width=4)
        resident.anterpolate_binned(dest, bins, gbg.CatmullRom, q)
        outs.append(dest.read())
    assert torch.equal(outs[0], outs[1])


def test_bounded_tile_wait_reports_timeout(gbg, oracle, dev):
    """A staged gather whose tile wait is allowed a single poll gives up on tiles still in
    flight: the status word says GBG_DEV_TIMEOUT, the call returns, and the context stays
    usable -- with the default limit the next gather matches the oracle."""
    resident, grid, g, f, pos, q, field, bins = setup(gbg, oracle, (48, 40, 32), 12, 40000, 71)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    bins.set_wait_limit(1)
    resident.interpolate_binned(field, bins, gbg.CatmullRom, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) & gbg._lib.GBG_DEV_TIMEOUT
    bins.set_wait_limit(0)
    status.zero_()
    got = resident.interpolate_binned(field, bins, gbg.CatmullRom, dtype=torch.float64, status=status).cpu().numpy()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert relerr(got, oracle.gather(g, f, pos, gbg.CatmullRom.coefficients)) <= 1e-5


def test_host_read_and_import_equal_the_device_path(gbg, dev):
    """A field read to the host is the device read, bitwise, taken after the export kernel
    has finished (a large field, so an early host read would see unwritten data); a host
    array imports like the same array on the device."""
    from gbgperiodicfields_gb300 import resident
    grid = gbg.Grid3D((128, 128, 128), (TWO_PI,) * 3)
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    data = torch.randn((12, 128, 128, 128), device=dev, generator=g).permute(3, 2, 1, 0)
    f = resident.ResidentField(grid, 12, max_stencil_width=4).load(data)
    for _ in range(3):
        host = f.read(dtype=torch.float32, device="cpu")
        assert host.device.type == "cpu" and host.stride() == (1, 128, 128 * 128, 128 ** 3)
        assert torch.equal(host, data.cpu())
    h = resident.ResidentField(grid, 12, max_stencil_width=4).load(data.cpu())
    assert torch.equal(h.read(dtype=torch.float32), data)
    with pytest.raises(gbg.ArgumentError):
        resident.PointBins(grid, 10).build(torch.zeros((10, 3), dtype=torch.float64))


def test_bins_split_at_extreme_positions(gbg, oracle, dev):
    """The FP64 fixed-point split far from the box: u = x * n/L * 2^32 (one rounding, origin 0),
    floor(u) split into cell and fraction.  Positions up to 5.7e8 (u near 6e18, close to the
    9.2e18 limit) bin like the host's exact keys and gather like the same points in the box;
    positions past the limit are reported as non-finite."""
    from gbgperiodicfields_gb300 import resident
    n = 16
    grid = gbg.Grid3D((n, n, n), (TWO_PI,) * 3)
    rng = np.random.default_rng(77)
    pos = TWO_PI * rng.random((600, 3))
    field = resident.ResidentField(grid, 3, max_stencil_width=4).load(
        torch.from_numpy(np.asfortranarray(rng.standard_normal((n, n, n, 3)))).cuda())
    inside = resident.PointBins(grid, 600, brick=(8, 8, 8)).build(torch.from_numpy(np.asfortranarray(pos)).cuda())
    want = resident.interpolate_binned(field, inside, gbg.CatmullRom).cpu().numpy()
    for shift in ([1e7, -3e7, 9e7], [-9e7, 5e6, -1e3]):
        far = np.asfortranarray(pos + TWO_PI * np.array(shift))
        bins = resident.PointBins(grid, 600, brick=(8, 8, 8)).build(torch.from_numpy(far).cuda())
        # host keys: the same single-rounding product and floor, then the periodic cell
        u = far * (n / TWO_PI * 4294967296.0)
        c = np.mod(np.floor(u).astype(np.int64) >> 32, n)
        br, loc = c // 8, c % 8
        key = ((br[:, 2] * 2 + br[:, 1]) * 2 + br[:, 0]) * 512 + (loc[:, 2] * 8 + loc[:, 1]) * 8 + loc[:, 0]
        assert np.array_equal(bins.order().cpu().numpy(), np.argsort(key, kind="stable") + 1)
        got = resident.interpolate_binned(field, bins, gbg.CatmullRom).cpu().numpy()
        assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    beyond = torch.tensor([[1.0, 2.0, 3.0], [9e8, 0.5, 0.5], [0.5, -9e8, 0.5]], dtype=torch.float64, device=dev)
    resident.PointBins(grid, 3, brick=(8, 8, 8)).build(beyond, status)
    torch.cuda.synchronize()
    assert int(status.item()) & gbg._lib.GBG_DEV_NONFINITE
