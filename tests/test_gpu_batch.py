"""GPU tests of the batched form: instances of uneven sizes (grids, components, point
counts, stencil widths) in one persistent gather launch and one persistent scatter launch,
and beside them instances large enough to run through the single-instance kernels.
Each instance's batched result must equal its single-instance result bitwise (the same
arithmetic in the same order) and the FP64 oracle within the precision form's 1e-5; the
whole step (bins builds + batch) is also replayed from a captured CUDA graph."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TWO_PI = 2 * np.pi


def relerr(got, want):
    return np.abs(np.asarray(got, np.float64) - want).max() / max(np.abs(want).max(), 1e-300)


def make_instances(gbg, oracle, seed=0, specs=None):
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(seed)
    if specs is None:
        specs = [((16, 16, 16), 1, 700, gbg.CatmullRom), ((24, 20, 18), 3, 5000, gbg.LalescuSpline(6)),
                 ((32, 32, 32), 12, 20000, gbg.CatmullRom), ((20, 22, 24), 9, 3000, gbg.CatmullRom),
                 ((18, 18, 18), 3, 1500, gbg.LagrangeSpline(8)), ((28, 16, 20), 4, 9000, gbg.LalescuSpline(6))]
    insts = []
    for n, C, M, scheme in specs:
        grid = gbg.Grid3D(n, (TWO_PI,) * 3, origin=(0.1, -0.2, 0.3))
        g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
        f = np.asfortranarray(rng.standard_normal(n + (C,)))
        pos = np.asfortranarray(np.array(grid.origin) + TWO_PI * rng.random((M, 3)))
        q = np.asfortranarray(rng.standard_normal((M, C)))
        field = resident.ResidentField(grid, C, max_stencil_width=8).load(torch.from_numpy(f).cuda())
        dest = resident.ResidentField(grid, C, max_stencil_width=8)
        pos_t = torch.from_numpy(pos).cuda()
        bins = resident.PointBins(grid, M).build(pos_t)
        insts.append(dict(field=field, bins=bins, scheme=scheme, dest=dest, grid=grid, g=g, f=f, pos=pos, q=q, pos_t=pos_t,
                          out=gbg.empty_colmajor((M, C), torch.float32, "cuda"),
                          qt=gbg.colmajor(torch.from_numpy(q).float().cuda())))
    return resident, insts


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def mixed_specs(gbg):
    """Instances below 1024 points, which share the persistent launches, beside larger
    ones, which the batch runs through the single-instance kernels."""
    return [((16, 16, 16), 1, 700, gbg.CatmullRom), ((40, 36, 32), 3, 70000, gbg.LalescuSpline(6)),
            ((20, 22, 24), 9, 600, gbg.CatmullRom), ((48, 48, 48), 4, 90000, gbg.CatmullRom),
            ((18, 18, 18), 3, 1500, gbg.LagrangeSpline(8))]


@pytest.mark.parametrize("mixed", [False, True], ids=["pooled", "pooled+direct"])
def test_batch_matches_single_and_oracle(gbg, oracle, dev, mixed):
    resident, insts = make_instances(gbg, oracle, specs=mixed_specs(gbg) if mixed else None)
    batch = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], out=i["out"], dest=i["dest"],
                                 q=i["qt"], alpha=1.0, beta=0.0) for i in insts])
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    batch.run(status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    for inst in insts:
        single = resident.interpolate_binned(inst["field"], inst["bins"], inst["scheme"])
        assert torch.equal(single, inst["out"])
        assert relerr(inst["out"].cpu().numpy(), oracle.gather(inst["g"], inst["f"], inst["pos"],
                                                               inst["scheme"].coefficients)) <= 1e-5
        got = inst["dest"].read().cpu().numpy()
        want = oracle.scatter(inst["g"], np.zeros(inst["grid"].grid_size + (inst["q"].shape[1],), order="F"),
                              inst["pos"], inst["q"], inst["scheme"].coefficients)
        assert relerr(got, want) <= 1e-5
        resident.anterpolate_binned(inst["field"], inst["bins"], inst["scheme"], inst["qt"])
        assert torch.equal(inst["field"].read(), inst["dest"].read())


@pytest.mark.parametrize("mixed", [False, True], ids=["pooled", "pooled+direct"])
def test_batch_step_in_cuda_graph(gbg, oracle, dev, mixed):
    resident, insts = make_instances(gbg, oracle, seed=5, specs=mixed_specs(gbg) if mixed else None)
    batch = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], out=i["out"], dest=i["dest"],
                                 q=i["qt"]) for i in insts])

    def step():
        for inst in insts:
            inst["bins"].build(inst["pos_t"])
        batch.run()

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()  # warm-up outside capture (sets kernel attributes)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    ref_out = [i["out"].clone() for i in insts]
    ref_dest = [i["dest"].read() for i in insts]
    for i in insts:
        i["out"].zero_()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    graph.replay()
    graph.replay()
    torch.cuda.synchronize()
    for i, o, d in zip(insts, ref_out, ref_dest):
        assert torch.equal(i["out"], o)
        assert torch.equal(i["dest"].read(), d)


def test_autotune_persists_and_keeps_results(gbg, oracle, dev, tmp_path, monkeypatch):
    """The tuner's choice (brick, threads per CTA) changes the launch shape only: results
    stay within the precision form's tolerance of the default configuration, and the
    choice is cached per problem class."""
    from gbgperiodicfields_gb300 import autotune, resident
    monkeypatch.setenv("GBG_TUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(21)
    grid = gbg.Grid3D((40, 36, 32), (TWO_PI,) * 3)
    g = oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin)
    M, C = 30000, 3
    pos = np.asfortranarray(TWO_PI * rng.random((M, 3)))
    pos_t = torch.from_numpy(pos).cuda()
    res = autotune.tune(grid, C, gbg.CatmullRom, pos_t, bricks=((11, 8, 8), (7, 4, 4)),
                        gather_threads=(256, 512), scatter_threads=(128, 256), reps=1)
    assert len(res["trials"]) == 2 and res["brick"] in ([11, 8, 8], [7, 4, 4])
    chosen = autotune.choose(grid.grid_size, C, gbg.CatmullRom, M)
    assert chosen["source"] == "cache" and chosen["brick"] == res["brick"]
    f = np.asfortranarray(rng.standard_normal(grid.grid_size + (C,)))
    q = np.asfortranarray(rng.standard_normal((M, C)))
    field = resident.ResidentField(grid, C, max_stencil_width=4).load(torch.from_numpy(f).cuda())
    bins = autotune.apply(resident.PointBins(grid, M, brick=chosen["brick"]).build(pos_t), chosen)
    got = resident.interpolate_binned(field, bins, gbg.CatmullRom).cpu().numpy()
    assert relerr(got, oracle.gather(g, f, pos, gbg.CatmullRom.coefficients)) <= 1e-5
    dest = resident.ResidentField(grid, C, max_stencil_width=4)
    resident.anterpolate_binned(dest, bins, gbg.CatmullRom, torch.from_numpy(q).float().cuda())
    want = oracle.scatter(g, np.zeros(grid.grid_size + (C,), order="F"), pos, q, gbg.CatmullRom.coefficients)
    assert relerr(dest.read().cpu().numpy(), want) <= 1e-5
    # every thread choice gives the same bits for the scatter (integer accumulation)
    ref = dest.read()
    for gt, st in ((128, 64), (512, 256), (256, 128)):
        bins.set_launch(gt, st)
        d2 = resident.ResidentField(grid, C, max_stencil_width=4)
        resident.anterpolate_binned(d2, bins, gbg.CatmullRom, torch.from_numpy(q).float().cuda())
        assert torch.equal(d2.read(), ref)
        assert torch.equal(resident.interpolate_binned(field, bins, gbg.CatmullRom),
                           torch.from_numpy(got).cuda())


def test_batch_reports_nonfinite_from_a_direct_instance(gbg, oracle, dev):
    """An instance large enough to run through the single-instance kernels inside the batch
    still reports a non-finite quantity in the batch's status word."""
    resident, insts = make_instances(gbg, oracle, seed=3, specs=mixed_specs(gbg))
    big = insts[1]
    assert big["pos"].shape[0] >= 1024
    big["qt"][17, 1] = float("nan")
    batch = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], out=i["out"], dest=i["dest"],
                                 q=i["qt"], alpha=1.0, beta=0.0) for i in insts])
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    batch.run(status)
    torch.cuda.synchronize()
    assert int(status.item()) & gbg._lib.GBG_DEV_NONFINITE


def test_batched_bins_builds_match_single_builds(gbg, oracle, dev):
    """gbg_bins_build_batch over uneven instances (and one bins twice, built in call order)
    gives every bins the binned order and the results of its own single build."""
    from gbgperiodicfields_gb300 import resident
    resident_, insts = make_instances(gbg, oracle, seed=11)
    want = [i["bins"].order().clone() for i in insts]
    fresh = [resident.PointBins(i["grid"], i["pos"].shape[0], brick=i["bins"].brick) for i in insts]
    decoy = gbg.colmajor(torch.rand_like(insts[0]["pos_t"]) * TWO_PI)
    pairs = [(fresh[0], decoy)] + [(b, i["pos_t"]) for b, i in zip(fresh, insts)]
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    resident.build_bins(pairs, status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    for b, w, i in zip(fresh, want, insts):
        assert torch.equal(b.order(), w)
        assert torch.equal(resident.interpolate_binned(i["field"], b, i["scheme"]),
                           resident.interpolate_binned(i["field"], i["bins"], i["scheme"]))
