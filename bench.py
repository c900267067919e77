#!/usr/bin/env python
"""Benchmark of the particle gather/scatter path on GB300.

Workload (the benchmark's plain-FP64-at-scale configuration): a 256^3 Float64
3-component velocity field (random Fourier modes |k| <= 64, |k|^(-11/6) spectrum,
divergence projected out) on [0, 2pi)^3 and 1e7 points, 70% uniform + 30% in 1000
Gaussian blobs of sigma = 0.05.  One step = build the traversal order, then cubic
(CatmullRom) gather + scatter and quintic (LalescuSpline(6)) gather + scatter: 4
particle-evaluations per point per step (one evaluation = one point x one field, all
components, one transfer).  Inputs are synthetic and seeded; the field (403 MB) and the
point arrays are larger than L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  With --impl reference it times the reference's CPU path
(the oracle's OpenMP restatement of the reference's KernelAbstractions CPU kernels) on
the host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-evals/s (gather+scatter) at fixed error vs FP64; serving p50/p99 ms"
UNIT = "particle-evals/s"
N_GRID = (256, 256, 256)
NCOMP = 3
M_POINTS = 10_000_000
KMAX = 64
WORKLOAD = ("256^3 Float64 3-component velocity field (|k|<=64, |k|^-11/6, divergence-free), "
            "1e7 points (70% uniform + 30% in 1000 Gaussian blobs, sigma=0.05), "
            "cubic + quintic gather and scatter per step, traversal order rebuilt per step")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the precision, batched and served forms (reported beside the headline)")
    ap.add_argument("--no-peaks", action="store_true",
                    help="skip the FP64 peak measurement (a cuBLAS DGEMM), e.g. under a profiler's launch list")
    ap.add_argument("--case", choices=sorted(PROFILE_CASES),
                    help="run one small fixed case twice and exit (the inputs of the ncu captures in profiles/)")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- workload

def make_inputs_host(seed: int = 1):
    from __graft_entry__ import load_package
    load_package()
    from gbgperiodicfields_gb300.workloads import clustered_points
    pos = clustered_points(M_POINTS, seed=seed + 1)
    q = np.asfortranarray(np.random.Generator(np.random.PCG64(seed + 2)).standard_normal((M_POINTS, NCOMP)))
    return pos, q


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# The main kernel of each timed call of the headline step.
KERNEL_NAMES = {"gather_cubic": "k_gather_plain<double, 4, 4, 3>", "gather_quintic": "k_gather_plain<double, 6, 6, 3>",
                "scatter_cubic": "k_scatter_fixed64<double, 4>", "scatter_quintic": "k_scatter_fixed64<double, 6>"}

# DRAM bytes (read + write) per launch of those kernels on this workload, from one ncu capture
# of dram__bytes_read.sum + dram__bytes_write.sum (one pass) on the full-size step (the timed
# step's launches; the warm-up step's agree to 0.1%).
NCU_TRAFFIC = {"gather_cubic": 5867726592, "scatter_cubic": 2899915520,
               "gather_quintic": 6046056192, "scatter_quintic": 5924986624}

# What bounds those kernels, from the ncu captures summarised in profiles/ (not measured in
# this run): the scatters run on the integer pipes, the gathers on the FP64 pipe.
_SCATTER_LIMITER = {"pipe": "integer issue (signed 64-bit high products, shared 32-bit atomics)",
                    "issue_active_pct": 70.1, "fma_heavy_pct": 56.4, "alu_pct": 53.1, "dram_pct": 2.6,
                    "source": "ncu --set full, 256^3 x 3, 4e6 clustered points, quintic "
                              "(profiles/fp64_scatter_k_scatter_fixed64_256cube_c3_4e6_quintic.md)"}
NCU_LIMITER = {"scatter_cubic": _SCATTER_LIMITER, "scatter_quintic": _SCATTER_LIMITER,
               "gather_cubic": {"pipe": "FP64 (the quintic gather's capture)",
                                "source": "profiles/fp64_gather_k_gather_plain_256cube_c3_4e6_quintic.md"},
               "gather_quintic": {"pipe": "FP64", "fp64_pipe_pct": 94.4,
                                  "source": "profiles/fp64_gather_k_gather_plain_256cube_c3_4e6_quintic.md"}}


def fp64_peak_tflops() -> float:
    """FP64 throughput of this GPU, measured: the best of a few cuBLAS DGEMMs."""
    import torch
    n = 8192
    a = torch.randn((n, n), dtype=torch.float64, device="cuda")
    b = torch.randn((n, n), dtype=torch.float64, device="cuda")
    torch.mm(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    del a, b
    return best


def algorithmic_bytes(m: int, ncomp: int, n: int, s: int, beta_nonzero=False) -> dict:
    """Compulsory traffic per call: every input read once, every output written once."""
    gather = m * (3 * s + ncomp * s) + n * ncomp * s
    scatter = m * (3 * s + ncomp * s) + (2 if beta_nonzero else 1) * n * ncomp * s
    return {"gather": gather, "scatter": scatter}


# -------------------------------------------------------------- GB300 arm

def run_gb300(args, rank, world):
    import ctypes
    import torch
    from __graft_entry__ import load_package
    gbg = load_package()
    from gbgperiodicfields_gb300.workloads import spectral_field

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = gbg._lib.load()
    grid = gbg.Grid3D(N_GRID, (2 * np.pi,) * 3)
    gC = grid.c()
    cubic, quintic = gbg.CatmullRom, gbg.LalescuSpline(6)
    schemes = [cubic, quintic]

    pos_h, q_h = make_inputs_host()
    field = spectral_field(N_GRID, NCOMP, kmax=KMAX, seed=1, project=True, device=dev)
    pos = torch.from_numpy(pos_h).to(dev)
    q = torch.from_numpy(q_h).to(dev)
    out = gbg.empty_colmajor((M_POINTS, NCOMP), torch.float64, dev)
    dep = gbg.empty_colmajor(N_GRID + (NCOMP,), torch.float64, dev)
    order = torch.empty(M_POINTS, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)

    nb = ctypes.c_size_t()
    gbg._lib.check(lib.gbg_point_traversal_order_workspace_size(gC, M_POINTS, 4, ctypes.byref(nb)))
    ws_order = torch.empty(nb.value, dtype=torch.uint8, device=dev)
    need = 0
    for s in schemes:
        gbg._lib.check(lib.gbg_anterpolate_workspace_size(gC, gbg._lib.GBG_F64, NCOMP, M_POINTS, s.c(), ctypes.byref(nb)))
        need = max(need, nb.value)
    ws_scatter = torch.empty(need, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    # per-call CUDA events on the launching stream, and per call the main kernel alone
    # (gbg_set_kernel_timing_events: events recorded by the library around that kernel)
    timings = {"order": [], "gather_cubic": [], "scatter_cubic": [], "gather_quintic": [], "scatter_quintic": []}
    kernel_times = {k: [] for k in timings if k != "order"}

    def timed(kev, fn):
        gbg._lib.check(lib.gbg_set_kernel_timing_events(kev[0].cuda_event, kev[1].cuda_event))
        try:
            fn()
        finally:
            lib.gbg_set_kernel_timing_events(None, None)

    def step(record):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        kev = {k: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for k in kernel_times}
        for a, b in kev.values():  # the handles exist once recorded
            a.record(stream)
            b.record(stream)
        ev[0].record(stream)
        gbg._lib.check(lib.gbg_point_traversal_order(gC, gbg._lib.GBG_F64, pos.data_ptr(), M_POINTS, 4,
                                                     order.data_ptr(), ws_order.data_ptr(), ws_order.numel(), sh))
        ev[1].record(stream)
        k = 2
        for name, s in (("cubic", cubic), ("quintic", quintic)):
            timed(kev["gather_" + name], lambda: gbg._lib.check(lib.gbg_interpolate(
                gC, gbg._lib.GBG_F64, NCOMP, field.data_ptr(), pos.data_ptr(), M_POINTS, order.data_ptr(), s.c(),
                out.data_ptr(), status.data_ptr(), sh)))
            ev[k].record(stream)
            timed(kev["scatter_" + name], lambda: gbg._lib.check(lib.gbg_anterpolate(
                gC, gbg._lib.GBG_F64, NCOMP, dep.data_ptr(), pos.data_ptr(), M_POINTS, q.data_ptr(), None, s.c(),
                1.0, 0.0, ws_scatter.data_ptr(), ws_scatter.numel(), status.data_ptr(), sh)))
            ev[k + 1].record(stream)
            k += 2
        if record is not None:
            record.append((ev, kev))

    for _ in range(args.warmup):
        step(None)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = lib.gbg_kernel_launches()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    evs = []
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(args.steps):
        step(evs)
    end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = lib.gbg_kernel_launches() - launches0
    ms_total = start.elapsed_time(end)
    for ev, kev in evs:
        names = list(timings)
        for i, nm in enumerate(names):
            timings[nm].append(ev[i].elapsed_time(ev[i + 1]))
        for nm, (a, b) in kev.items():
            kernel_times[nm].append(a.elapsed_time(b))
    if int(status.item()) != 0:
        raise RuntimeError(f"device status {int(status.item())}")
    if rank == 0 and not args.no_cpu:
        # the last timed step's quintic outputs, checked against the oracle after the CPU
        # baseline has run (oracle_check)
        _LAST_OUTPUTS.update(field=np.asfortranarray(field.cpu().numpy()), gather=np.asfortranarray(out.cpu().numpy()),
                             scatter=np.asfortranarray(dep.cpu().numpy()))

    ms_total = reduce_max(ms_total, world, dev)
    evals_per_step = 4 * M_POINTS
    value = world * evals_per_step * args.steps / (ms_total / 1e3)

    # roofline of the dominant kernel (by its own event-timed duration): algorithmic bytes
    # per launch against the HBM copy peak, and algorithmic FP64 flops (2 * width^3 * C per
    # point) against the FP64 peak measured here with a cuBLAS DGEMM
    avg = {k: float(np.mean(v)) for k, v in timings.items()}
    kavg = {k: float(np.mean(v)) for k, v in kernel_times.items()}
    peak, peak_kind = peaks()
    ab = algorithmic_bytes(M_POINTS, NCOMP, int(np.prod(N_GRID)), 8)
    dominant = max(kavg, key=kavg.get)
    dom_bytes = ab["scatter"] if dominant.startswith("scatter") else ab["gather"]
    achieved = dom_bytes / (kavg[dominant] / 1e3) / 1e9
    width = 6 if dominant.endswith("quintic") else 4
    dom_flops = 2 * width ** 3 * NCOMP * M_POINTS
    fp64_peak = None if args.no_peaks else fp64_peak_tflops()
    fp64_achieved = dom_flops / (kavg[dominant] / 1e3) / 1e12

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "grid": list(N_GRID), "ncomp": NCOMP, "points": M_POINTS,
                   "schemes": ["CatmullRom", "LalescuSpline(6)"], "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (field 403 MB)"},
        "per_call_ms": avg,
        "kernel_ms": kavg,
        "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dominant], "call": dominant, "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": NCU_TRAFFIC.get(dominant), "algorithmic_bytes": dom_bytes,
                     "fp64": {"achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                              "frac": fp64_achieved / fp64_peak if fp64_peak else None,
                              "algorithmic_flops": dom_flops,
                              "peak_source": "cuBLAS DGEMM 8192^3 measured in this run"},
                     "limiter": NCU_LIMITER.get(dominant)},
        "clocks": clk,
        "gpu_launches": int(launches),
    }

    if not args.no_e2e:
        result["e2e"] = e2e_gb300(args, gbg, lib, grid, field, pos_h, q_h, dev, stream)
    if not args.no_forms:
        del field, pos, q, out, dep, ws_scatter, ws_order
        torch.cuda.empty_cache()
        launches1 = lib.gbg_kernel_launches()
        result["precision_form"] = precision_form(gbg, lib, dev, peak)
        result["batched_form"] = batched_form(gbg, dev)
        result["served_form"] = served_form(gbg, dev)
        result["nufft_form"] = nufft_form(gbg, lib, dev)
        result["forms_gpu_launches"] = int(lib.gbg_kernel_launches() - launches1)
    return result


def e2e_gb300(args, gbg, lib, grid, field_dev, pos_h, q_h, dev, stream):
    """The same step through the C ABI with host buffers: every step copies the inputs
    from pinned host memory and reads every result back.  The copies run on their own
    streams, as a caller of the stream-ordered ABI would run them: the uploads on one, the
    downloads on another, each transfer waiting only for the inputs it reads, and two sets
    of device buffers so that a step's uploads overlap the previous step's work.  Every byte
    still crosses inside the timed region."""
    import torch
    gC = grid.c()
    cs = stream
    sh = cs.cuda_stream
    up = torch.cuda.Stream(device=dev)
    down = torch.cuda.Stream(device=dev)
    f_h = field_dev.cpu().pin_memory()  # column-major (Nx,Ny,Nz,3) host copy
    pos_p = torch.from_numpy(pos_h).pin_memory()
    q_p = torch.from_numpy(q_h).pin_memory()
    out_h = [torch.empty((NCOMP, M_POINTS), dtype=torch.float64).pin_memory() for _ in range(2)]
    dep_h = [torch.empty(f_h.shape[::-1], dtype=torch.float64).pin_memory() for _ in range(2)]
    schemes = [gbg.CatmullRom, gbg.LalescuSpline(6)]
    sets = []
    for _ in range(2):
        sets.append({
            "f": gbg.empty_colmajor(N_GRID + (NCOMP,), torch.float64, dev),
            "pos": gbg.empty_colmajor((M_POINTS, 3), torch.float64, dev),
            "q": gbg.empty_colmajor((M_POINTS, NCOMP), torch.float64, dev),
            "order": torch.empty(M_POINTS, dtype=torch.int32, device=dev),
            "out": [gbg.empty_colmajor((M_POINTS, NCOMP), torch.float64, dev) for _ in range(2)],
            "dep": [gbg.empty_colmajor(N_GRID + (NCOMP,), torch.float64, dev) for _ in range(2)],
            "free": torch.cuda.Event(),
        })
        sets[-1]["free"].record(cs)

    def step(k):
        S = sets[k & 1]
        ev = {name: torch.cuda.Event() for name in ("pos", "f", "q")}
        up.wait_event(S["free"])  # this set's previous step is done (its results are read back)
        with torch.cuda.stream(up):
            S["pos"].copy_(pos_p, non_blocking=True)
            ev["pos"].record(up)
            S["f"].copy_(f_h, non_blocking=True)
            ev["f"].record(up)
            S["q"].copy_(q_p, non_blocking=True)
            ev["q"].record(up)
        cs.wait_event(ev["pos"])
        gbg._lib.check(lib.gbg_point_traversal_order(gC, gbg._lib.GBG_F64, S["pos"].data_ptr(), M_POINTS, 4,
                                                     S["order"].data_ptr(), None, 0, sh))
        cs.wait_event(ev["f"])
        cs.wait_event(ev["q"])
        for i, s in enumerate(schemes):
            gbg._lib.check(lib.gbg_interpolate(gC, gbg._lib.GBG_F64, NCOMP, S["f"].data_ptr(), S["pos"].data_ptr(),
                                               M_POINTS, S["order"].data_ptr(), s.c(), S["out"][i].data_ptr(), None, sh))
            g_done = torch.cuda.Event()
            g_done.record(cs)
            gbg._lib.check(lib.gbg_anterpolate(gC, gbg._lib.GBG_F64, NCOMP, S["dep"][i].data_ptr(), S["pos"].data_ptr(),
                                               M_POINTS, S["q"].data_ptr(), None, s.c(), 1.0, 0.0, None, 0, None, sh))
            s_done = torch.cuda.Event()
            s_done.record(cs)
            down.wait_event(g_done)
            with torch.cuda.stream(down):
                out_h[i].copy_(S["out"][i].T, non_blocking=True)
            down.wait_event(s_done)
            with torch.cuda.stream(down):
                dep_h[i].copy_(S["dep"][i].permute(3, 2, 1, 0), non_blocking=True)
        S["free"].record(down)

    step(0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = max(2, args.steps // 2)
    e0.record(cs)
    up.wait_stream(cs)
    for k in range(n):
        step(k)
    cs.wait_stream(down)
    cs.wait_stream(up)
    e1.record(cs)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    h2d = f_h.numel() * 8 + pos_p.numel() * 8 + q_p.numel() * 8
    d2h = sum(t.numel() * 8 for t in out_h) + sum(t.numel() * 8 for t in dep_h)
    return {"value": 4 * M_POINTS / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "overlap": "uploads and downloads on their own streams, two buffer sets"}


# ------------------------------------------------- precision / batched / served forms

def _time_ms(fn, reps=3):
    """Minimum over reps of CUDA-event time (warm-up call first)."""
    import torch
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def _kernel_ms(lib, fn, reps=3):
    """Minimum over reps of the library's main kernel alone (timing events recorded by the
    library around it, on its stream)."""
    import torch
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        b.record()
        lib.gbg_set_kernel_timing_events(a.cuda_event, b.cuda_event)
        try:
            fn()
        finally:
            lib.gbg_set_kernel_timing_events(None, None)
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def _rel_errors(got, want):
    """max and RMS of |got - want|, relative to max|want| and RMS(want)."""
    import torch
    d = (got.double() - want.double())
    w = want.double()
    return {"max_rel": float(d.abs().max() / w.abs().max().clamp_min(1e-300)),
            "rms_rel": float(d.square().mean().sqrt() / w.square().mean().sqrt().clamp_min(1e-300))}


def precision_form(gbg, lib, dev, peak):
    """512^3 field of 3 + 9 components (velocity and its gradient tensor, stored as one
    12-component resident FP32 field), 3.2e7 uniform points, cubic gather and scatter
    through the resident form; errors against the FP64 drop-in path (itself pinned to the
    oracle at <= 1e-13) and the speed-up over that FP64 path on the same inputs."""
    import torch
    from gbgperiodicfields_gb300 import resident
    from gbgperiodicfields_gb300.workloads import spectral_field, uniform_points
    n, C, M = (512, 512, 512), 12, 32_000_000
    grid = gbg.Grid3D(n, (2 * np.pi,) * 3)
    f64 = spectral_field(n, 3, kmax=64, seed=3, project=True, gradient=True, device=dev, dtype=torch.float64)
    field = resident.ResidentField(grid, C, max_stencil_width=4).load(f64)
    pos_r = torch.from_numpy(uniform_points(M, seed=4)).to(dev)
    q64_r = gbg.colmajor(torch.randn((M, C), dtype=torch.float64, device=dev))
    bins = resident.PointBins(grid, M)
    out = gbg.empty_colmajor((M, C), torch.float32, dev)
    dest = resident.ResidentField(grid, C, max_stencil_width=4)
    scheme = gbg.CatmullRom
    # points in arrival (random) order: every gathered value lands at a random row
    q32_r = gbg.colmajor(q64_r.float())
    random_order = {"bins": _time_ms(lambda: bins.build(pos_r)),
                    "gather": _time_ms(lambda: resident.interpolate_binned(field, bins, scheme, out=out)),
                    "scatter": _time_ms(lambda: resident.anterpolate_binned(dest, bins, scheme, q32_r, 1.0, 0.0))}
    # the particle state kept in binned order on the device (re-sorted once, as a
    # particle code does when it moves its points), the configuration reported
    perm = bins.order().long() - 1
    pos = gbg.colmajor(pos_r[perm])
    q64 = gbg.colmajor(q64_r[perm])
    q32 = gbg.colmajor(q64.float())
    del pos_r, q64_r, q32_r, perm
    # the autotuner picks the bin brick and the threads per CTA for this problem
    from gbgperiodicfields_gb300 import autotune
    tuned = autotune.tune(grid, C, scheme, pos, bricks=((11, 8, 8), (7, 8, 8), (15, 8, 8)), reps=1, persist=False)
    bins = autotune.apply(resident.PointBins(grid, M, brick=tuned["brick"]).build(pos), tuned)
    t_bins = _time_ms(lambda: bins.build(pos))
    t_gather = _time_ms(lambda: resident.interpolate_binned(field, bins, scheme, out=out))
    t_scatter = _time_ms(lambda: resident.anterpolate_binned(dest, bins, scheme, q32, 1.0, 0.0))
    k_gather = _kernel_ms(lib, lambda: resident.interpolate_binned(field, bins, scheme, out=out))
    k_scatter = _kernel_ms(lib, lambda: resident.anterpolate_binned(dest, bins, scheme, q32, 1.0, 0.0))
    # the FP64 drop-in on the same inputs: reference values and the speed comparison
    gC = grid.c()
    sh = torch.cuda.current_stream().cuda_stream
    out64 = gbg.empty_colmajor((M, C), torch.float64, dev)
    dep64 = gbg.empty_colmajor(n + (C,), torch.float64, dev)
    order = torch.empty(M, dtype=torch.int32, device=dev)

    def plain_step():
        gbg._lib.check(lib.gbg_point_traversal_order(gC, gbg._lib.GBG_F64, pos.data_ptr(), M, 4, order.data_ptr(),
                                                     None, 0, sh))
        gbg._lib.check(lib.gbg_interpolate(gC, gbg._lib.GBG_F64, C, f64.data_ptr(), pos.data_ptr(), M,
                                           order.data_ptr(), scheme.c(), out64.data_ptr(), None, sh))
        gbg._lib.check(lib.gbg_anterpolate(gC, gbg._lib.GBG_F64, C, dep64.data_ptr(), pos.data_ptr(), M,
                                           q64.data_ptr(), None, scheme.c(), 1.0, 0.0, None, 0, None, sh))
    t_plain = _time_ms(plain_step, reps=1)
    err_g = _rel_errors(out, out64)
    err_s = _rel_errors(dest.read(), dep64)
    alg = algorithmic_bytes(M, C, int(np.prod(n)), 4)
    step = t_bins + t_gather + t_scatter
    res = {
        "workload": "512^3 x (3+9) FP32 resident field (velocity + gradient, |k|<=64), 3.2e7 uniform points "
                    "kept in binned order, cubic gather + scatter, bins rebuilt per step",
        "value": 2 * M / (step / 1e3), "unit": UNIT,
        "per_call_ms": {"bins": t_bins, "gather": t_gather, "scatter": t_scatter},
        "kernel_ms": {"gather": k_gather, "scatter": k_scatter},
        "tuned": {k: tuned[k] for k in ("brick", "gather_threads", "scatter_threads")},
        "random_order_ms": random_order,
        "roofline": {
            "gather": {"bound": "hbm", "kernel": "k_gather_staged4<4, 12, float>",
                       "achieved": alg["gather"] / (k_gather / 1e3) / 1e9, "peak": peak,
                       "unit": "GB/s", "frac": alg["gather"] / (k_gather / 1e3) / 1e9 / peak,
                       "algorithmic_bytes": alg["gather"]},
            "scatter": {"bound": "hbm", "kernel": "k_scatter_nodes<4, 1, 12>",
                        "achieved": alg["scatter"] / (k_scatter / 1e3) / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": alg["scatter"] / (k_scatter / 1e3) / 1e9 / peak,
                        "algorithmic_bytes": alg["scatter"]}},
        "error_vs_fp64": {"gather": err_g, "scatter": err_s},
        "plain_fp64_ms": t_plain, "speedup_vs_plain_fp64": t_plain / step,
    }
    del f64, field, dest, out64, dep64, q64, q32, pos, bins, out
    torch.cuda.empty_cache()
    return res


def nufft_form(gbg, lib, dev, n=128, M=2_000_000, samples=32):
    """The NUFFT spectral transfer: a band-limited 128^3 3-component field in spectral
    representation (|k| <= 32), 2e6 uniform points, type 2 (interpolate) and type 1
    (anterpolate) at FP64 tolerance 1e-6 (window width 8) and FP32 tolerance 1e-4 (width 6),
    oversampling 2.  Error of the gather against the exact DirectDFT sum at a sample of
    points (computed here with torch on the device), and the adjoint identity
    M<Wf,q> = N<f,W^T q> for the whole deposit."""
    import torch
    from gbgperiodicfields_gb300.workloads import spectral_field, uniform_points
    res = {"workload": f"{n}^3 x 3 spectral field (|k|<=32), {M:.0e} uniform points, oversampling 2, "
                       "type 2 + type 1 per step", "unit": UNIT}
    pos64 = torch.from_numpy(uniform_points(M, seed=12)).to(dev)
    for dtype, tol in ((torch.float64, 1e-6), (torch.float32, 1e-4)):
        grid = gbg.Grid3D((n,) * 3, (2 * np.pi,) * 3, dtype=dtype)
        phys = spectral_field((n,) * 3, 3, kmax=32, seed=13, project=True, device=dev, dtype=dtype)
        fh = gbg.to_spectral(gbg.VectorFieldPhysical(phys, grid))
        plan = gbg.NUFFT(fh, tolerance=tol)
        pts = gbg.PointSet(gbg.colmajor(pos64.to(dtype)))
        q = gbg.VectorPointValues(gbg.colmajor(torch.randn((M, 3), dtype=dtype, device=dev)))
        out = gbg.VectorPointValues(gbg.empty_colmajor((M, 3), dtype, dev))
        dep = gbg.VectorFieldSpectral(torch.zeros_like(fh.data), grid)
        t2 = _time_ms(lambda: gbg.interpolate_(out, fh, pts, plan))
        t1 = _time_ms(lambda: gbg.anterpolate_(dep, pts, q, plan))
        k2 = _kernel_ms(lib, lambda: gbg.interpolate_(out, fh, pts, plan))
        k1 = _kernel_ms(lib, lambda: gbg.anterpolate_(dep, pts, q, plan))
        # the exact sum at a sample of points
        F = fh.data.to(torch.complex128)
        k = [torch.fft.rfftfreq(n, 1.0 / n, device=dev, dtype=torch.float64) if d == 0 else
             torch.fft.fftfreq(n, 1.0 / n, device=dev, dtype=torch.float64) for d in range(3)]
        alpha = torch.full((n // 2 + 1,), 2.0, dtype=torch.float64, device=dev)
        alpha[0] = 1.0
        alpha[-1] = 1.0
        P = pos64[:samples]
        exact = torch.empty((samples, 3), dtype=torch.float64, device=dev)
        for i in range(samples):
            ph = (torch.exp(1j * k[0] * P[i, 0])[:, None, None] * torch.exp(1j * k[1] * P[i, 1])[None, :, None]
                  * torch.exp(1j * k[2] * P[i, 2])[None, None, :])
            exact[i] = (alpha[:, None, None, None] * torch.real(F * ph[..., None])).sum(dim=(0, 1, 2)) / float(n ** 3)
        got = out.data[:samples].to(torch.float64)
        err = float((got - exact).abs().max() / exact.abs().max())
        left = float((out.data.to(torch.float64) * q.data.to(torch.float64)).sum())
        D = dep.data.to(torch.complex128)
        right = float((alpha[:, None, None, None] * torch.real(F * torch.conj(D))).sum()) / float(n ** 3)
        res["f64" if dtype == torch.float64 else "f32"] = {
            "tolerance": tol, "window_width": plan.width, "window_shape": plan.beta,
            "per_call_ms": {"interpolate": t2, "anterpolate": t1},
            "kernel_ms": {"gather": k2, "spread": k1},
            "value": 2 * M / ((t1 + t2) / 1e3),
            "max_rel_error_vs_directdft": err,
            "adjoint_rel_gap": abs(left - right) / max(abs(left), 1e-300),
        }
        del phys, fh, plan, pts, q, out, dep, F, D
        torch.cuda.empty_cache()
    return res


def batched_form(gbg, dev):
    """64 instances of uneven sizes (grids 32^3..256^3, 1/3/9 components, 1e3..1e6
    points log-uniform, cubic or quintic) as one batch (instances below 1024 points in one
    persistent gather launch and one persistent scatter launch, the others through the
    single-instance kernels), the whole step (bins builds + batch) replayed from a CUDA
    graph; beside it the same work launched instance by instance."""
    import torch
    from gbgperiodicfields_gb300 import autotune, resident
    rng = np.random.default_rng(7)
    insts = []
    for _ in range(64):
        nn = int(rng.choice([32, 64, 128, 256]))
        C = int(rng.choice([1, 3, 9]))
        M = int(np.exp(rng.uniform(np.log(1e3), np.log(1e6))))
        scheme = gbg.CatmullRom if rng.random() < 0.5 else gbg.LalescuSpline(6)
        grid = gbg.Grid3D((nn,) * 3, (2 * np.pi,) * 3)
        field = resident.ResidentField(grid, C, max_stencil_width=6).load(
            torch.randn((C, nn, nn, nn), device=dev).permute(3, 2, 1, 0))
        dest = resident.ResidentField(grid, C, max_stencil_width=6)
        pos = gbg.colmajor(torch.rand((M, 3), dtype=torch.float64, device=dev) * 2 * np.pi)
        cfg = autotune.choose(grid.grid_size, C, scheme, M)
        bins = autotune.apply(resident.PointBins(grid, M, brick=cfg["brick"]).build(pos), cfg)
        insts.append(dict(field=field, dest=dest, bins=bins, scheme=scheme, pos=pos, M=M,
                          out=gbg.empty_colmajor((M, C), torch.float32, dev),
                          q=gbg.colmajor(torch.randn((M, C), device=dev))))
    total = sum(i["M"] for i in insts)
    batch = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], out=i["out"], dest=i["dest"],
                                 q=i["q"]) for i in insts])

    def step():
        for i in insts:
            i["bins"].build(i["pos"])
        batch.run()

    def seq():
        for i in insts:
            i["bins"].build(i["pos"])
            resident.interpolate_binned(i["field"], i["bins"], i["scheme"], out=i["out"])
            resident.anterpolate_binned(i["dest"], i["bins"], i["scheme"], i["q"])

    t_seq = _time_ms(seq)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    t_graph = _time_ms(lambda: graph.replay())
    res = {"workload": "64 instances: grids {32,64,128,256}^3, C in {1,3,9}, M log-uniform 1e3..1e6, "
                       "cubic/quintic, FP32 resident, bricks from the autotuner; bins + the batch (persistent "
                       "launches below 1024 points, single-instance kernels above), CUDA graph",
           "points": int(total), "value": 2 * total / (t_graph / 1e3), "unit": UNIT,
           "ms_per_step": t_graph, "sequential_ms": t_seq}
    del insts, batch, graph
    torch.cuda.empty_cache()
    return res


def served_form(gbg, dev, requests=240, seed=9):
    """Poisson requests over 8 resident FP32 3-component fields of 128^3..512^3, request
    sizes log-uniform in [1e4, 4e6] points, 70% gathers and 30% scatters (beta = 1 into
    the field), at 80% of the capacity measured first with a full backlog."""
    import torch
    from gbgperiodicfields_gb300 import resident, serving
    rng = np.random.default_rng(seed)
    sizes = [128, 192, 256, 320, 384, 448, 512, 512]
    fields, grids = [], []
    for k, nn in enumerate(sizes):
        grid = gbg.Grid3D((nn,) * 3, (2 * np.pi,) * 3)
        grids.append(grid)
        fields.append(resident.ResidentField(grid, 3, max_stencil_width=4).load(
            torch.randn((3, nn, nn, nn), device=dev).permute(3, 2, 1, 0)))
    # a pool of request inputs, made before the clock starts
    pool = []
    for _ in range(64):
        M = int(np.exp(rng.uniform(np.log(1e4), np.log(4e6))))
        pos = gbg.colmajor(torch.rand((M, 3), dtype=torch.float64, device=dev) * 2 * np.pi)
        pool.append(dict(M=M, pos=pos, q=gbg.colmajor(torch.randn((M, 3), device=dev)),
                         out=gbg.empty_colmajor((M, 3), torch.float32, dev)))
    torch.cuda.synchronize()
    scheme = gbg.CatmullRom
    plan = [(int(rng.integers(0, 8)), int(rng.integers(0, len(pool))), rng.random() < 0.3) for _ in range(requests)]

    def issue(server, r):
        fi, pi, is_scatter = r
        p = pool[pi]
        if is_scatter:
            return server.anterpolate(fields[fi], p["pos"], scheme, p["q"], 1.0, 1.0)
        return server.interpolate(fields[fi], p["pos"], scheme, out=p["out"])

    with serving.Server(slots=4, max_batch=8, timeout=60.0) as server:
        # capacity: the whole plan as one backlog
        for r in plan[:16]:
            issue(server, r)
        server.drain()
        server.stats(reset=True)
        t0 = time.perf_counter()
        tickets = [issue(server, r) for r in plan]
        server.drain()
        t_cap = time.perf_counter() - t0
        for t in tickets:
            server.wait(t)
        cap = server.stats(reset=True)
        capacity = requests / t_cap
        # open loop at 80% of capacity
        rate = 0.8 * capacity
        gaps = rng.exponential(1.0 / rate, requests)
        t0 = time.perf_counter()
        due = t0
        tickets = []
        for r, g in zip(plan, gaps):
            due += g
            while True:
                now = time.perf_counter()
                if now >= due:
                    break
                time.sleep(min(due - now, 0.0005))
            tickets.append(issue(server, r))
        server.drain()
        wall = time.perf_counter() - t0
        codes = [server.wait(t) for t in tickets]
        st = server.stats()
    pts = sum(pool[r[1]]["M"] for r in plan)
    res = {"workload": "8 resident FP32 3-component fields (128^3..512^3), Poisson requests, M log-uniform "
                       "1e4..4e6, 70% gather / 30% scatter (beta=1), cubic; 4 slots, runs of <= 8",
           "requests": requests, "capacity_req_s": capacity, "capacity_points_s": pts / t_cap,
           "offered_req_s": rate, "load": 0.8,
           "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
           "throughput_req_s": requests / wall, "throughput_points_s": pts / wall,
           "runs": st["runs"], "failed": int(sum(1 for c in codes if c != 0)),
           "hbm_peak_bytes": int(st["hbm_peak"]),
           "backlog_p50_ms": cap["p50_ms"], "backlog_p99_ms": cap["p99_ms"]}
    del fields, pool
    torch.cuda.empty_cache()
    return res


def reduce_max(value: float, world: int, device) -> float:
    """The largest value over the ranks (the whole job's time is its slowest replica's)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------- CPU baseline

_LAST_OUTPUTS: dict = {}


def oracle_check(pos_h, q_h):
    """The last timed step's quintic gather and scatter (all 1e7 points) against the oracle
    on the same inputs and the same field, run over all host cores: max and RMS error
    relative to max|oracle|, beside the Float64 bar the parity tests hold (1e-13)."""
    if not _LAST_OUTPUTS:
        return None
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    o = _LAST_OUTPUTS
    g = oracle.grid_dict(N_GRID)
    coeffs = oracle.lalescu(6)
    cores = os.cpu_count() or 1
    p, qq = np.asfortranarray(pos_h), np.asfortranarray(q_h)
    t0 = time.perf_counter()
    want_g = oracle.gather(g, o["field"], p, coeffs, nthreads=cores)
    want_s = oracle.scatter(g, np.zeros(o["field"].shape, order="F"), p, qq, coeffs, 1.0, 0.0, nthreads=cores)

    def rel(got, want):
        d = got.reshape(want.shape, order="F") - want
        scale = float(np.abs(want).max())
        return {"max_rel": float(np.abs(d).max() / scale), "rms_rel": float(np.sqrt(np.mean(d * d)) / scale)}

    res = {"gather_quintic": rel(o["gather"], want_g), "scatter_quintic": rel(o["scatter"], want_s), "bar": 1e-13,
           "points": M_POINTS, "oracle_seconds": round(time.perf_counter() - t0, 1)}
    _LAST_OUTPUTS.clear()
    return res


def cpu_sample_rate(pos_h, q_h, field_h, target_seconds: float):
    """Times the reference's CPU path (oracle, OpenMP over all host cores) on a bounded
    sample of the points: the same four transfers per point as a GPU step."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from __graft_entry__ import load_package
    load_package()
    g = oracle.grid_dict(N_GRID)
    cubic, quintic = oracle.lalescu(4), oracle.lalescu(6)
    cores = os.cpu_count() or 1
    dep = np.zeros(field_h.shape, order="F")

    def run(m):
        p = np.asfortranarray(pos_h[:m])
        qq = np.asfortranarray(q_h[:m])
        t0 = time.perf_counter()
        for c in (cubic, quintic):
            trav = oracle.traversal_order(g, p)
            oracle.gather(g, field_h, p, c, traversal=trav, nthreads=cores)
            oracle.scatter(g, dep, p, qq, c, 1.0, 0.0, traversal=trav, nthreads=cores)
        return time.perf_counter() - t0

    m = 100_000
    t = run(m)
    m2 = int(min(M_POINTS, max(m, m * target_seconds / max(t, 1e-3) * 0.8)))
    t2 = run(m2)
    return {"value": 4 * m2 / t2, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{m2} of the {M_POINTS} points (all four transfers, traversal order per transfer), "
                      f"full 256^3x3 field, {t2:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    from __graft_entry__ import load_package
    load_package()
    from gbgperiodicfields_gb300.workloads import spectral_field
    import torch
    torch.set_num_threads(os.cpu_count() or 1)
    pos_h, q_h = make_inputs_host()
    field_h = spectral_field(N_GRID, NCOMP, kmax=KMAX, seed=1, project=True, device="cpu")
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps))
    rates = []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_sample_rate(pos_h, q_h, field_h, 1.0)
    for _ in range(args.steps):
        rates.append(cpu_sample_rate(pos_h, q_h, field_h, per_step))
    value = float(np.median([r["value"] for r in rates]))
    base = rates[-1]
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 4 * M_POINTS / value * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "grid": list(N_GRID), "ncomp": NCOMP, "points": M_POINTS,
                       "schemes": ["CatmullRom", "LalescuSpline(6)"], "parallelism": "host threads"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------------------- profiling cases

def case_resident(n=256, C=12, M=4_000_000, brick=(15, 8, 8), threads=256):
    """256^3 x 12 FP32 resident field (0.85 GB), 4e6 uniform points in binned order,
    cubic gather and scatter, twice, at the precision form's tuned launch shape (15x8x8
    bricks, 256 threads for both kernels)."""
    import torch
    from __graft_entry__ import load_package
    gbg = load_package()
    from gbgperiodicfields_gb300 import resident
    from gbgperiodicfields_gb300.workloads import uniform_points
    dev = torch.device("cuda:0")
    grid = gbg.Grid3D((n,) * 3, (2 * np.pi,) * 3)
    field = resident.ResidentField(grid, C, max_stencil_width=4).load(
        torch.randn((C, n, n, n), device=dev).permute(3, 2, 1, 0))
    pos = torch.from_numpy(uniform_points(M, seed=2)).to(dev)
    bins = resident.PointBins(grid, M, brick=brick).build(pos)
    pos = gbg.colmajor(pos[bins.order().long() - 1])
    bins.build(pos)
    bins.set_launch(threads, threads)
    out = gbg.empty_colmajor((M, C), torch.float32, dev)
    q = gbg.colmajor(torch.randn((M, C), dtype=torch.float32, device=dev))
    for _ in range(2):
        bins.build(pos)
        resident.interpolate_binned(field, bins, gbg.CatmullRom, out=out)
        resident.anterpolate_binned(field, bins, gbg.CatmullRom, q)
    torch.cuda.synchronize()


def case_resident_full():
    """The precision form's step at full size: 512^3 x 12 FP32 resident field, 3.2e7
    points in binned order, bins + cubic gather + scatter, twice (for a one-pass launch
    list only)."""
    case_resident(n=512, C=12, M=32_000_000)


def case_nufft(n=64, M=500_000):
    """NUFFT on a 64^3 x 3 spectral field with 5e5 uniform points, type 2 then type 1, at
    FP64 tolerance 1e-6 (window width 8) and FP32 tolerance 1e-4 (width 6); twice."""
    import torch
    from __graft_entry__ import load_package
    gbg = load_package()
    from gbgperiodicfields_gb300.workloads import spectral_field, uniform_points
    dev = torch.device("cuda:0")
    pos = torch.from_numpy(uniform_points(M, seed=2)).to(dev)
    runs = []
    for dtype, tol in ((torch.float64, 1e-6), (torch.float32, 1e-4)):
        grid = gbg.Grid3D((n,) * 3, (2 * np.pi,) * 3, dtype=dtype)
        fh = gbg.to_spectral(gbg.VectorFieldPhysical(spectral_field((n,) * 3, 3, kmax=16, seed=1, project=True,
                                                                    device=dev, dtype=dtype), grid))
        pts = gbg.PointSet(gbg.colmajor(pos.to(dtype)))
        q = gbg.VectorPointValues(gbg.colmajor(torch.randn((M, 3), dtype=dtype, device=dev)))
        runs.append((grid, fh, gbg.NUFFT(fh, tolerance=tol), pts, q))
    for _ in range(2):
        for grid, fh, plan, pts, q in runs:
            gbg.interpolate(fh, pts, plan)
            gbg.anterpolate(grid, pts, q, plan)
    torch.cuda.synchronize()


def case_plain(n=256, M=4_000_000):
    """256^3 x 3 FP64 field (403 MB, above L2), 4e6 clustered points, quintic
    (LalescuSpline(6)) scatter and gather through the drop-in API, twice."""
    import torch
    from __graft_entry__ import load_package
    gbg = load_package()
    from gbgperiodicfields_gb300.workloads import clustered_points
    dev = torch.device("cuda:0")
    grid = gbg.Grid3D((n,) * 3, (2 * np.pi,) * 3)
    pts = gbg.PointSet(torch.from_numpy(clustered_points(M, seed=3)).to(dev))
    q = gbg.VectorPointValues(gbg.colmajor(torch.randn((M, 3), dtype=torch.float64, device=dev)))
    f = gbg.VectorFieldPhysical(gbg.colmajor(torch.randn((n, n, n, 3), dtype=torch.float64, device=dev)), grid)
    order = gbg.point_traversal_order(grid, pts)
    s = gbg.LalescuSpline(6)
    for _ in range(2):
        gbg.anterpolate_(f, pts, q, s, 1.0, 0.0)
        gbg.interpolate(f, pts, s, traversal=order)
    torch.cuda.synchronize()


PROFILE_CASES = {"resident_256c12_4e6": case_resident, "resident_512c12_3p2e7": case_resident_full,
                 "plain_256c3_4e6_quintic": case_plain, "nufft_64c3_5e5": case_nufft}


def main():
    args = parse()
    if args.case:
        PROFILE_CASES[args.case]()
        print(json.dumps({"case": args.case, "ok": True}))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group(backend)
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_gb300(args, rank, world)
        if rank == 0 and not args.no_cpu:
            pos_h, q_h = make_inputs_host()
            from gbgperiodicfields_gb300.workloads import spectral_field
            field_h = spectral_field(N_GRID, NCOMP, kmax=KMAX, seed=1, project=True, device="cpu")
            res["cpu_baseline"] = cpu_sample_rate(pos_h, q_h, field_h, args.cpu_seconds)
            res["error_vs_oracle"] = oracle_check(pos_h, q_h)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
