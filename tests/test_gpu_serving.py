"""GPU tests of the serving form: requests of mixed kinds and sizes over resident fields,
admitted by memory and batched onto stream slots as they arrive.

The central property: every request's result is the same alone and in the mix.  "Alone"
runs the requests one at a time (one slot, runs of one request, each waited for before
the next is submitted); "in the mix" submits them all at once to several slots with runs
of several requests.  Gathers and scatters on the same field keep their arrival order in
both, so the results must agree bitwise (the batched kernels do the single-instance
arithmetic in the same order), and agree with the FP64 oracle of the same serial
sequence within the precision form's 1e-5.  Failures are injected on the host only: a
poisoned position, a forced allocation failure, a deadline already passed."""
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


FIELD_SPECS = {"A": ((24, 20, 18), 3), "B": ((32, 32, 32), 1), "C": ((16, 16, 20), 9)}


def make_fields(gbg, oracle, seed=3):
    from gbgperiodicfields_gb300 import resident
    rng = np.random.default_rng(seed)
    fields, host = {}, {}
    for name, (n, C) in FIELD_SPECS.items():
        grid = gbg.Grid3D(n, (TWO_PI,) * 3, origin=(0.2, -0.1, 0.05))
        f = np.asfortranarray(rng.standard_normal(n + (C,)))
        fields[name] = resident.ResidentField(grid, C, max_stencil_width=8).load(torch.from_numpy(f).cuda())
        host[name] = dict(grid=grid, g=oracle.grid_dict(grid.grid_size, grid.domain_size, grid.origin), f=f)
    return fields, host


def make_requests(gbg, host, seed=11):
    """An arrival sequence that interleaves gathers and scatters on shared fields."""
    rng = np.random.default_rng(seed)
    plan = [("g", "A", gbg.CatmullRom, 900), ("g", "B", gbg.LalescuSpline(6), 2500),
            ("s", "C", gbg.CatmullRom, 1200, 2.0, 0.5), ("g", "C", gbg.CatmullRom, 700),
            ("g", "A", gbg.LagrangeSpline(4), 1600), ("s", "A", gbg.LalescuSpline(6), 3000, 1.0, 1.0),
            ("g", "A", gbg.CatmullRom, 500), ("s", "B", gbg.CatmullRom, 4000, 1.0, 0.0),
            ("g", "B", gbg.CatmullRom, 800), ("s", "A", gbg.CatmullRom, 600, -1.5, 1.0),
            ("g", "A", gbg.LagrangeSpline(8), 2000), ("g", "C", gbg.LalescuSpline(6), 1000)]
    reqs = []
    for p in plan:
        kind, name, scheme, M = p[:4]
        grid = host[name]["grid"]
        pos = np.asfortranarray(np.array(grid.origin) + TWO_PI * (rng.random((M, 3)) * 1.2 - 0.1))
        r = dict(kind=kind, field=name, scheme=scheme, pos=pos)
        if kind == "s":
            r.update(q=np.asfortranarray(rng.standard_normal((M, FIELD_SPECS[name][1]))), alpha=p[4], beta=p[5])
        reqs.append(r)
    return reqs


def submit(server, fields, r):
    pos = torch.from_numpy(r["pos"]).cuda()
    if r["kind"] == "g":
        return server.interpolate(fields[r["field"]], pos, r["scheme"])
    q = torch.from_numpy(r["q"]).float().cuda()
    return server.anterpolate(fields[r["field"]], pos, r["scheme"], q, r["alpha"], r["beta"])


def run_alone(gbg, oracle, host, reqs):
    from gbgperiodicfields_gb300 import serving
    fields, _ = make_fields(gbg, oracle)
    outs = []
    with serving.Server(slots=1, max_batch=1, timeout=30.0) as server:
        for r in reqs:
            t = submit(server, fields, r)
            out = server.result(t)
            outs.append(None if out is None else out.clone())
        server.drain()
    return outs, {k: f.read() for k, f in fields.items()}


def run_mixed(gbg, oracle, reqs, slots=3, max_batch=4):
    from gbgperiodicfields_gb300 import serving
    fields, _ = make_fields(gbg, oracle)
    with serving.Server(slots=slots, max_batch=max_batch, timeout=30.0) as server:
        tickets = [submit(server, fields, r) for r in reqs]
        outs = [server.result(t) for t in tickets]
        server.drain()
        stats = server.stats()
    return outs, {k: f.read() for k, f in fields.items()}, stats


def test_results_same_alone_and_in_the_mix(gbg, oracle, dev):
    _, host = make_fields(gbg, oracle)
    reqs = make_requests(gbg, host)
    alone_out, alone_fields = run_alone(gbg, oracle, host, reqs)
    for slots, mb in ((3, 4), (6, 16), (2, 2)):
        mixed_out, mixed_fields, stats = run_mixed(gbg, oracle, reqs, slots, mb)
        assert stats["completed"] == len(reqs) and stats["failed"] == 0
        for a, m in zip(alone_out, mixed_out):
            assert (a is None) == (m is None)
            if a is not None:
                assert torch.equal(a, m)
        for k in FIELD_SPECS:
            assert torch.equal(alone_fields[k], mixed_fields[k])
    # and the serial sequence against the FP64 oracle
    state = {k: h["f"].copy(order="F") for k, h in host.items()}
    for r, out in zip(reqs, alone_out):
        h = host[r["field"]]
        if r["kind"] == "g":
            want = oracle.gather(h["g"], state[r["field"]], r["pos"], r["scheme"].coefficients)
            assert relerr(out.cpu().numpy(), want) <= 1e-5
        else:
            st = np.asfortranarray(r["beta"] * state[r["field"]])
            W = oracle.scatter(h["g"], np.zeros_like(st, order="F"), r["pos"], r["q"], r["scheme"].coefficients)
            state[r["field"]] = np.asfortranarray(st + r["alpha"] * W)
    for k in FIELD_SPECS:
        assert relerr(alone_fields[k].cpu().numpy(), state[k]) <= 1e-5


def test_served_gather_equals_direct_call(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import resident, serving
    fields, host = make_fields(gbg, oracle)
    rng = np.random.default_rng(5)
    pos = torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((3000, 3)))).cuda()
    bins = resident.PointBins(host["A"]["grid"], 3000).build(pos)
    direct = resident.interpolate_binned(fields["A"], bins, gbg.CatmullRom)
    with serving.Server(slots=2, max_batch=8) as server:
        served = server.result(server.interpolate(fields["A"], pos, gbg.CatmullRom))
    assert torch.equal(direct, served)


def test_poisoned_request_fails_alone(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import serving
    fields, host = make_fields(gbg, oracle)
    rng = np.random.default_rng(8)
    good = [torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((500, 3)))).cuda() for _ in range(3)]
    bad = good[1].clone()
    bad[17, 1] = float("nan")
    with serving.Server(slots=2, max_batch=8) as server:
        t = [server.interpolate(fields["A"], good[0], gbg.CatmullRom),
             server.interpolate(fields["A"], bad, gbg.CatmullRom),
             server.interpolate(fields["B"], good[2], gbg.CatmullRom)]
        codes = [server.wait(x) for x in t]
    assert codes == [0, gbg._lib.GBG_ENONFINITE, 0]


def test_injected_allocation_failure_and_deadline(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import serving
    fields, host = make_fields(gbg, oracle)
    rng = np.random.default_rng(9)
    pos = torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((800, 3)))).cuda()
    with serving.Server(slots=2, max_batch=1, timeout=30.0) as server:
        ref = server.result(server.interpolate(fields["A"], pos, gbg.CatmullRom)).clone()
        server.inject(gbg._lib.GBG_FAULT_ALLOC, 1)
        assert server.wait(server.interpolate(fields["A"], pos, gbg.CatmullRom)) == gbg._lib.GBG_ENOMEM
        server.inject(gbg._lib.GBG_FAULT_DEADLINE, 1)
        assert server.wait(server.interpolate(fields["A"], pos, gbg.CatmullRom)) == gbg._lib.GBG_ETIMEOUT
        server.drain()  # the expired run still completes on the device and is retired
        assert torch.equal(server.result(server.interpolate(fields["A"], pos, gbg.CatmullRom)), ref)
        server.drain()
        st = server.stats()
        assert st["hbm_in_use"] == 0 and st["failed"] == 2 and st["completed"] == 2


def test_budget_refusal_and_admission_by_memory(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import serving
    fields, host = make_fields(gbg, oracle)
    rng = np.random.default_rng(10)
    pos = torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((20000, 3)))).cuda()
    with serving.Server(slots=4, max_batch=8, hbm_budget=1 << 20) as server:
        with pytest.raises(gbg.GBGError):
            server.interpolate(fields["A"], pos, gbg.CatmullRom)  # needs more than the whole budget
    # a budget that holds one request at a time: everything still completes, serially
    small = pos[:3000]
    with serving.Server(slots=4, max_batch=8) as probe:
        probe.result(probe.interpolate(fields["A"], small, gbg.CatmullRom))
        one = probe.stats()["hbm_peak"]
    with serving.Server(slots=4, max_batch=8, hbm_budget=int(one * 1.5)) as server:
        ts = [server.interpolate(fields["A"], small, gbg.CatmullRom) for _ in range(6)]
        outs = [server.result(t) for t in ts]
        st = server.stats()
    assert st["hbm_peak"] <= int(one * 1.5) and st["completed"] == 6 and st["runs"] == 6
    for o in outs[1:]:
        assert torch.equal(o, outs[0])


def test_latency_counters(gbg, oracle, dev):
    from gbgperiodicfields_gb300 import serving
    fields, host = make_fields(gbg, oracle)
    rng = np.random.default_rng(12)
    with serving.Server(slots=4, max_batch=4) as server:
        ts = []
        for i in range(20):
            M = int(rng.integers(100, 5000))
            pos = torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((M, 3)))).cuda()
            ts.append(server.interpolate(fields["ABC"[i % 3]], pos, gbg.CatmullRom))
        for t in ts:
            assert server.wait(t) == 0
        st = server.stats(reset=True)
        assert st["completed"] == 20 and 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
        assert st["runs"] <= 20 and st["points"] > 0
        assert server.stats()["completed"] == 0
