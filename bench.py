#!/usr/bin/env python
"""Benchmark of the particle gather/scatter path on GB300.

Headline workload (the precision form, the largest configuration that fits one GPU): a
512^3 field of 3 velocity components plus the 9-component velocity-gradient tensor (random
Fourier modes |k| <= 64, |k|^(-11/6) spectrum, divergence projected out, the gradient
computed spectrally), held as one 12-component FP32 resident field; 3.2e7 uniform points
with FP64 positions (FP64 is kept for the periodic wrap and the cell/fraction split only);
cubic (CatmullRom) splines.  One step = rebuild the device cell bins from the positions,
gather the 12 components at every point, scatter 12 quantities per point into a second
resident field (beta = 0): 2 particle-evaluations per point per step (one evaluation = one
point x one transfer of the 12-component field).  The caller's particle state is kept in
binned order (as a particle code re-orders its arrays after moving them), and the bins are
rebuilt from those positions every step.  Inputs are synthetic and seeded; the field
(6.6 GB) and the point arrays are larger than L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `e2e` is the same step through the C ABI from host
buffers: every step uploads the field, the positions and the quantities from pinned host
memory and reads the gathered values and the deposited field back.  `--impl reference`
times the reference's CPU path (the oracle's OpenMP restatement of the reference's
KernelAbstractions CPU kernels: traversal order, gather, atomic scatter) on the host cores,
each step on a block of the same points against the full FP64 field.  Secondary keys: the
FP64 drop-in on the same inputs, the plain-FP64-at-scale workload (256^3 x 3, 1e7
clustered points, cubic + quintic), the batched, served and NUFFT forms, and oracle checks.
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

# headline: the precision form at full size
N3 = (512, 512, 512)
C3 = 12
M3 = 32_000_000
KMAX3 = 64


def workload_config():
    """The headline workload's description (the same dict in both arms)."""
    wl = (f"{N3[0]}^3 x (3 velocity + 9 velocity-gradient) FP32 resident field (|k|<={KMAX3}, |k|^-11/6, "
          f"divergence-free), FP64 positions, {M3:.1e} uniform points kept in binned order, cubic "
          "(CatmullRom); per step: bins rebuilt, gather of the 12 components, scatter of 12 quantities (beta=0)")
    fb = N3[0] * N3[1] * N3[2] * C3 * 4
    return {"workload": wl, "grid": list(N3), "ncomp": C3, "points": M3, "scheme": "CatmullRom",
            "storage": "f32 field, f64 positions", "evals_per_point_per_step": 2, "parallelism": "replicas",
            "l2": f"inputs larger than L2 (field {fb / 1e9:.2f} GB), no flush" if fb > 2 ** 27 else "field within L2"}


def shrink_workload(k: int):
    """Divides the headline grid by k per axis and the points by k^3 (the harness's own CPU
    tests run the reference arm this way; the line's config records the sizes used)."""
    global N3, M3, KMAX3
    if k > 1:
        N3 = tuple(n // k for n in N3)
        M3 = M3 // k ** 3
        KMAX3 = max(2, KMAX3 // k)

# secondary: plain FP64 at scale
N2G = (256, 256, 256)
NCOMP2 = 3
M2 = 10_000_000
KMAX2 = 64

# reference arm / CPU baseline: points per step of the CPU port
CPU_BLOCK = 2_000_000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and the oracle checks")
    ap.add_argument("--cpu-block", type=int, default=CPU_BLOCK,
                    help="points per step of the CPU port (reference arm and CPU baseline)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the secondary workloads (FP64 drop-in, plain FP64 at scale, batched, served, NUFFT)")
    ap.add_argument("--shrink", type=int, default=1,
                    help="divide the headline grid by K per axis and the points by K^3 (harness tests only)")
    ap.add_argument("--case", choices=sorted(PROFILE_CASES),
                    help="run one small fixed case twice and exit (the inputs of the committed ncu captures)")
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


# --------------------------------------------------------------- inputs

def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(m: int, ncomp: int, n: int, s: int, beta_nonzero=False) -> dict:
    """Compulsory traffic per call: every input read once, every output written once;
    positions are FP64 (24 B per point), values and quantities s bytes each."""
    gather = m * (24 + ncomp * s) + n * ncomp * s
    scatter = m * (24 + ncomp * s) + (2 if beta_nonzero else 1) * n * ncomp * s
    return {"gather": gather, "scatter": scatter}


def c3_points_host():
    """The 3.2e7 uniform FP64 positions, (M, 3) column-major, in generation order."""
    from __graft_entry__ import load_package
    load_package()
    from gbgperiodicfields_gb300.workloads import uniform_points
    return uniform_points(M3, seed=4)


def c3_quantities_host(rows=None):
    """The scatter's N(0,1) quantities, (M, 12) Float32 in generation order (row blocks of
    one seeded stream, so a block of rows can be made without the rest)."""
    out = np.empty((M3, C3), dtype=np.float32, order="F") if rows is None else None
    blk = min(1_000_000, M3)
    lo, hi = (0, M3) if rows is None else rows
    parts = []
    for b in range(lo // blk, (hi + blk - 1) // blk):
        g = np.random.Generator(np.random.PCG64([5, b]))
        v = g.standard_normal((blk, C3), dtype=np.float32)
        a, z = max(lo, b * blk), min(hi, (b + 1) * blk)
        if out is not None:
            out[a:z] = v[a - b * blk:z - b * blk]
        else:
            parts.append(v[a - b * blk:z - b * blk])
    return out if out is not None else np.asfortranarray(np.concatenate(parts, axis=0))


# -------------------------------------------------------------- GB300 arm

def _events(n):
    import torch
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def run_gb300(args, rank, world):
    import torch
    from __graft_entry__ import load_package
    gbg = load_package()
    from gbgperiodicfields_gb300 import autotune, resident
    from gbgperiodicfields_gb300.workloads import spectral_field

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = gbg._lib.load()
    grid = gbg.Grid3D(N3, (2 * np.pi,) * 3)
    scheme = gbg.CatmullRom
    peak, peak_kind = peaks()

    # inputs: the FP64 field (kept for the FP64 comparison and the oracle), its FP32
    # resident copy, the points in binned order and their quantities
    f64 = spectral_field(N3, 3, kmax=KMAX3, seed=3, project=True, gradient=True, device=dev, dtype=torch.float64)
    field = resident.ResidentField(grid, C3, max_stencil_width=4).load(f64)
    pos_gen = torch.from_numpy(c3_points_host()).to(dev)
    bins = resident.PointBins(grid, M3).build(pos_gen)
    perm = bins.order().long() - 1
    pos = gbg.colmajor(pos_gen[perm])
    q_gen = torch.from_numpy(c3_quantities_host()).to(dev)
    q32 = gbg.colmajor(q_gen[perm])
    del q_gen
    perm_h = perm.cpu().numpy()  # binned slot -> generation index
    del perm, pos_gen
    torch.cuda.empty_cache()
    # bin brick and threads per CTA from the autotuner, timed on these points
    tuned = autotune.tune(grid, C3, scheme, pos, bricks=((11, 8, 8), (7, 8, 8), (15, 8, 8)), reps=1, persist=False)
    bins = autotune.apply(resident.PointBins(grid, M3, brick=tuned["brick"]).build(pos), tuned)
    out = gbg.empty_colmajor((M3, C3), torch.float32, dev)
    dest = resident.ResidentField(grid, C3, max_stencil_width=4)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    names = ("bins", "gather", "scatter")
    calls = {k: [] for k in names}
    kernels = {"gather": [], "scatter": []}

    def timed_kernel(kev, fn):
        gbg._lib.check(lib.gbg_set_kernel_timing_events(kev[0].cuda_event, kev[1].cuda_event))
        try:
            fn()
        finally:
            lib.gbg_set_kernel_timing_events(None, None)

    def step(record):
        ev = _events(4)
        kev = {k: tuple(_events(2)) for k in kernels}
        for a, b in kev.values():  # the handles exist once recorded
            a.record(stream)
            b.record(stream)
        ev[0].record(stream)
        bins.build(pos, status)
        ev[1].record(stream)
        timed_kernel(kev["gather"], lambda: resident.interpolate_binned(field, bins, scheme, out=out))
        ev[2].record(stream)
        timed_kernel(kev["scatter"], lambda: resident.anterpolate_binned(dest, bins, scheme, q32, 1.0, 0.0))
        ev[3].record(stream)
        if record is not None:
            record.append((ev, kev))

    for _ in range(max(3, args.warmup)):
        step(None)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = lib.gbg_kernel_launches()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    evs = []
    start, end = _events(2)
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
        for i, nm in enumerate(names):
            calls[nm].append(ev[i].elapsed_time(ev[i + 1]))
        for nm, (a, b) in kev.items():
            kernels[nm].append(a.elapsed_time(b))
    if int(status.item()) != 0:
        raise RuntimeError(f"device status {int(status.item())}")
    ms_total = reduce_max(ms_total, world, dev)
    value = world * 2 * M3 * args.steps / (ms_total / 1e3)

    avg = {k: float(np.mean(v)) for k, v in calls.items()}
    kavg = {k: float(np.mean(v)) for k, v in kernels.items()}
    alg = algorithmic_bytes(M3, C3, int(np.prod(N3)), 4)
    kname = {"gather": "k_gather_staged4<4, 12, float>", "scatter": "k_scatter_nodes<4, 1, 12>"}
    per_kernel = {k: {"kernel": kname[k], "ms": kavg[k], "algorithmic_bytes": alg[k],
                      "achieved": alg[k] / (kavg[k] / 1e3) / 1e9,
                      "frac": alg[k] / (kavg[k] / 1e3) / 1e9 / peak} for k in kavg}
    dominant = max(kavg, key=kavg.get)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 position split)", "data": "synthetic (seeded)",
        "config": workload_config(),
        "per_call_ms": avg,
        "kernel_ms": kavg,
        "roofline": {"bound": "hbm", "kernel": kname[dominant], "call": dominant,
                     "achieved": per_kernel[dominant]["achieved"], "peak": peak, "unit": "GB/s",
                     "frac": per_kernel[dominant]["frac"], "peak_source": peak_kind,
                     "traffic": None, "algorithmic_bytes": alg[dominant], "per_kernel": per_kernel,
                     "note": "achieved = algorithmic bytes / the kernel's CUDA-event time on its stream over the "
                             "timed steps; DRAM traffic per launch is in the committed ncu summaries"},
        "tuned": {**{k: tuned[k] for k in ("brick", "gather_threads", "scatter_threads")},
                  "trials": [{k: (round(v, 3) if isinstance(v, float) else v) for k, v in t.items()}
                             for t in tuned["trials"]]},
        "clocks": clk,
        "gpu_launches": int(launches),
    }

    # the points of the oracle checks and of the CPU legs: a uniform stride over the slots
    check_idx = np.arange(0, M3, max(1, M3 // 1_000_000))[:1_000_000]
    if rank == 0 and not args.no_cpu:
        idx_t = torch.from_numpy(check_idx).to(dev)
        _LAST.update(gather_rows=out[idx_t].double().cpu().numpy(), check_idx=check_idx, perm_h=perm_h)
        # the scatter of the same sample on its own (a deposit of all 3.2e7 points cannot
        # be restated on the host in bench time)
        sub_pos = gbg.colmajor(pos[idx_t])
        sub_q = gbg.colmajor(q32[idx_t])
        sub_bins = resident.PointBins(grid, len(check_idx)).build(sub_pos)
        sub_dest = resident.ResidentField(grid, C3, max_stencil_width=4)
        resident.anterpolate_binned(sub_dest, sub_bins, scheme, sub_q, 1.0, 0.0)
        _LAST.update(scatter_field=sub_dest.read(torch.float32).cpu().numpy(), f64_host=f64.cpu().numpy())
        del sub_pos, sub_q, sub_bins, sub_dest, idx_t

    if not args.no_e2e:
        result["e2e"] = e2e_c3(args, gbg, grid, scheme, field, dest, bins, pos, q32, f64, dev, stream)
    if not args.no_forms:
        result["fp64_dropin_same_inputs"] = fp64_dropin_same_inputs(gbg, lib, grid, scheme, f64, pos, q32, out, dest,
                                                                     result["ms_per_step"], dev)
    del field, dest, bins, out, pos, q32, f64
    torch.cuda.empty_cache()
    if not args.no_forms:
        launches1 = lib.gbg_kernel_launches()
        result["plain_fp64_form"] = plain_fp64_form(args, gbg, lib, dev, peak)
        result["batched_form"] = batched_form(gbg, dev)
        result["served_form"] = served_form(gbg, dev)
        result["nufft_form"] = nufft_form(gbg, lib, dev)
        result["forms_gpu_launches"] = int(lib.gbg_kernel_launches() - launches1)
    return result


def e2e_c3(args, gbg, grid, scheme, field, dest, bins, pos_dev, q_dev, f64, dev, stream):
    """The headline step through the C ABI from host buffers.  Every step uploads the
    field (FP32, the reference's column-major layout), the positions and the quantities
    from pinned host memory, imports the field into the resident layout, rebuilds the bins,
    gathers, scatters, exports the deposit to the reference layout and reads the gathered
    values and the deposit back.  The copies run on their own streams, as a caller of the
    stream-ordered ABI would run them (uploads on one, downloads on another, each waiting
    only for what it moves), with two sets of device buffers so that one step's uploads
    overlap the previous step's work; every byte still crosses inside the timed region."""
    import torch
    from gbgperiodicfields_gb300 import resident
    cs = stream
    up = torch.cuda.Stream(device=dev)
    down = torch.cuda.Stream(device=dev)
    f_h = f64.to(torch.float32).cpu().pin_memory()  # (Nx, Ny, Nz, 12) column-major
    pos_h = pos_dev.cpu().pin_memory()
    q_h = q_dev.cpu().pin_memory()
    out_h = [torch.empty((C3, M3), dtype=torch.float32).pin_memory() for _ in range(2)]
    dep_h = [torch.empty((C3,) + N3[::-1], dtype=torch.float32).pin_memory() for _ in range(2)]
    sets = []
    for _ in range(2):
        sets.append({"f": gbg.empty_colmajor(N3 + (C3,), torch.float32, dev),
                     "pos": gbg.empty_colmajor((M3, 3), torch.float64, dev),
                     "q": gbg.empty_colmajor((M3, C3), torch.float32, dev),
                     "out": gbg.empty_colmajor((M3, C3), torch.float32, dev),
                     "dep": gbg.empty_colmajor(N3 + (C3,), torch.float32, dev),
                     "free": torch.cuda.Event()})
        sets[-1]["free"].record(cs)
    lib = gbg._lib.load()

    def step(k):
        S = sets[k & 1]
        ev = {name: torch.cuda.Event() for name in ("pos", "f", "q")}
        up.wait_event(S["free"])  # this set's previous step has been read back
        with torch.cuda.stream(up):
            S["pos"].copy_(pos_h, non_blocking=True)
            ev["pos"].record(up)
            S["f"].copy_(f_h, non_blocking=True)
            ev["f"].record(up)
            S["q"].copy_(q_h, non_blocking=True)
            ev["q"].record(up)
        cs.wait_event(ev["pos"])
        bins.build(S["pos"])
        cs.wait_event(ev["f"])
        field.load(S["f"])
        resident.interpolate_binned(field, bins, scheme, out=S["out"])
        g_done = torch.cuda.Event()
        g_done.record(cs)
        cs.wait_event(ev["q"])
        resident.anterpolate_binned(dest, bins, scheme, S["q"], 1.0, 0.0)
        gbg._lib.check(lib.gbg_field_export(dest.handle, gbg._lib.GBG_F32, S["dep"].data_ptr(), cs.cuda_stream))
        s_done = torch.cuda.Event()
        s_done.record(cs)
        down.wait_event(g_done)
        with torch.cuda.stream(down):
            out_h[k & 1].copy_(S["out"].T, non_blocking=True)
        down.wait_event(s_done)
        with torch.cuda.stream(down):
            dep_h[k & 1].copy_(S["dep"].permute(3, 2, 1, 0), non_blocking=True)
        S["free"].record(down)

    step(0)
    step(1)
    torch.cuda.synchronize()
    e0, e1 = _events(2)
    n = max(3, args.steps // 2)
    e0.record(cs)
    up.wait_stream(cs)
    for k in range(n):
        step(k)
    cs.wait_stream(down)
    cs.wait_stream(up)
    e1.record(cs)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    h2d = f_h.numel() * 4 + pos_h.numel() * 8 + q_h.numel() * 4
    d2h = out_h[0].numel() * 4 + dep_h[0].numel() * 4
    res = {"value": 2 * M3 / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": n,
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "overlap": "uploads and downloads on their own streams, two device buffer sets"}
    del sets, f_h, pos_h, q_h, out_h, dep_h
    torch.cuda.empty_cache()
    return res


def fp64_dropin_same_inputs(gbg, lib, grid, scheme, f64, pos, q32, out32, dest, precision_ms, dev):
    """The FP64 drop-in (gbg_point_traversal_order + gbg_interpolate + gbg_anterpolate on
    the reference's layouts, itself pinned to the oracle at 1e-13) on the headline's inputs:
    its step time beside the precision form's, and the precision form's error against it
    over every point and every node (max and RMS, relative to max|FP64| and RMS(FP64))."""
    import torch
    gC = grid.c()
    sh = torch.cuda.current_stream().cuda_stream
    q64 = gbg.colmajor(q32.double())
    out64 = gbg.empty_colmajor((M3, C3), torch.float64, dev)
    dep64 = gbg.empty_colmajor(N3 + (C3,), torch.float64, dev)
    order = torch.empty(M3, dtype=torch.int32, device=dev)

    def plain_step():
        gbg._lib.check(lib.gbg_point_traversal_order(gC, gbg._lib.GBG_F64, pos.data_ptr(), M3, 4, order.data_ptr(),
                                                     None, 0, sh))
        gbg._lib.check(lib.gbg_interpolate(gC, gbg._lib.GBG_F64, C3, f64.data_ptr(), pos.data_ptr(), M3,
                                           order.data_ptr(), scheme.c(), out64.data_ptr(), None, sh))
        gbg._lib.check(lib.gbg_anterpolate(gC, gbg._lib.GBG_F64, C3, dep64.data_ptr(), pos.data_ptr(), M3,
                                           q64.data_ptr(), None, scheme.c(), 1.0, 0.0, None, 0, None, sh))
    t_plain = _time_ms(plain_step, reps=2)
    res = {"ms_per_step": t_plain, "precision_ms_per_step": precision_ms,
           "speedup_of_precision_form": t_plain / precision_ms,
           "precision_error_vs_fp64": {"gather": _rel_errors(out32, out64), "scatter": _rel_errors(dest.read(), dep64)}}
    del q64, out64, dep64, order
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------- secondary workloads

def _time_ms(fn, reps=3):
    """Minimum over reps of CUDA-event time (warm-up call first)."""
    import torch
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = _events(2)
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
        a, b = _events(2)
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
    d = (got.double() - want.double())
    w = want.double()
    return {"max_rel": float(d.abs().max() / w.abs().max().clamp_min(1e-300)),
            "rms_rel": float(d.square().mean().sqrt() / w.square().mean().sqrt().clamp_min(1e-300))}


def plain_fp64_form(args, gbg, lib, dev, peak):
    """The plain-FP64-at-scale workload through the drop-in C ABI: 256^3 x 3 FP64 velocity
    field (|k| <= 64, divergence-free), 1e7 points (70% uniform + 30% in 1000 Gaussian
    blobs, sigma 0.05); per step the traversal order, then cubic and quintic gather and
    scatter (4 evaluations per point).  The last step's four outputs are kept for the
    oracle check over all 1e7 points."""
    import torch
    from gbgperiodicfields_gb300.workloads import clustered_points, spectral_field
    grid = gbg.Grid3D(N2G, (2 * np.pi,) * 3)
    gC = grid.c()
    schemes = {"cubic": gbg.CatmullRom, "quintic": gbg.LalescuSpline(6)}
    pos_h = clustered_points(M2, seed=2)
    q_h = np.asfortranarray(np.random.Generator(np.random.PCG64(3)).standard_normal((M2, NCOMP2)))
    field = spectral_field(N2G, NCOMP2, kmax=KMAX2, seed=1, project=True, device=dev)
    pos = torch.from_numpy(pos_h).to(dev)
    q = torch.from_numpy(q_h).to(dev)
    outs = {k: gbg.empty_colmajor((M2, NCOMP2), torch.float64, dev) for k in schemes}
    deps = {k: gbg.empty_colmajor(N2G + (NCOMP2,), torch.float64, dev) for k in schemes}
    order = torch.empty(M2, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    sh = torch.cuda.current_stream().cuda_stream
    timings = {"order": [], **{f"{c}_{k}": [] for k in schemes for c in ("gather", "scatter")}}
    kernel = {f"{c}_{k}": [] for k in schemes for c in ("gather", "scatter")}

    def step():
        ev = _events(6)
        ev[0].record()
        gbg._lib.check(lib.gbg_point_traversal_order(gC, gbg._lib.GBG_F64, pos.data_ptr(), M2, 4,
                                                     order.data_ptr(), None, 0, sh))
        ev[1].record()
        i = 1
        for k, s in schemes.items():
            for c in ("gather", "scatter"):
                a, b = _events(2)
                a.record()
                b.record()
                lib.gbg_set_kernel_timing_events(a.cuda_event, b.cuda_event)
                try:
                    if c == "gather":
                        gbg._lib.check(lib.gbg_interpolate(gC, gbg._lib.GBG_F64, NCOMP2, field.data_ptr(),
                                                           pos.data_ptr(), M2, order.data_ptr(), s.c(),
                                                           outs[k].data_ptr(), status.data_ptr(), sh))
                    else:
                        gbg._lib.check(lib.gbg_anterpolate(gC, gbg._lib.GBG_F64, NCOMP2, deps[k].data_ptr(),
                                                           pos.data_ptr(), M2, q.data_ptr(), None, s.c(), 1.0, 0.0,
                                                           None, 0, status.data_ptr(), sh))
                finally:
                    lib.gbg_set_kernel_timing_events(None, None)
                i += 1
                ev[i].record()
                kernel[f"{c}_{k}"].append((a, b))
        return ev

    step()
    torch.cuda.synchronize()
    for v in kernel.values():
        v.clear()
    e0, e1 = _events(2)
    steps = max(3, min(args.steps, 10))
    evs = []
    e0.record()
    for _ in range(steps):
        evs.append(step())
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    names = list(timings)
    for ev in evs:
        for i, nm in enumerate(names):
            timings[nm].append(ev[i].elapsed_time(ev[i + 1]))
    kms = {k: float(np.mean([a.elapsed_time(b) for a, b in v])) for k, v in kernel.items()}
    if int(status.item()) != 0:
        raise RuntimeError(f"device status {int(status.item())}")
    alg = algorithmic_bytes(M2, NCOMP2, int(np.prod(N2G)), 8)
    res = {"workload": "256^3 Float64 3-component velocity field (|k|<=64, |k|^-11/6, divergence-free), 1e7 points "
                       "(70% uniform + 30% in 1000 Gaussian blobs, sigma=0.05), traversal order + cubic and quintic "
                       "gather and scatter per step",
           "value": 4 * M2 / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
           "per_call_ms": {k: float(np.mean(v)) for k, v in timings.items()}, "kernel_ms": kms,
           "hbm_frac": {k: (alg["gather"] if k.startswith("gather") else alg["scatter"]) / (v / 1e3) / 1e9 / peak
                        for k, v in kms.items()},
           "fp64_flops_frac_note": "the FP64 kernels are bound by the FP64 pipe (GB300 FP64 is 1/58 of FP32)"}
    _LAST.update(c2_field=np.asfortranarray(field.cpu().numpy()), c2_pos=pos_h, c2_q=q_h,
                 c2_out={k: np.asfortranarray(v.cpu().numpy()) for k, v in outs.items()},
                 c2_dep={k: np.asfortranarray(v.cpu().numpy()) for k, v in deps.items()})
    del field, pos, q, outs, deps, order
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
    points log-uniform, cubic or quintic) as one batch, the whole step (batched bins builds
    + batch) replayed from a CUDA graph; beside it the same work launched instance by
    instance, and a breakdown by phase.  Each instance class (grid, components, scheme,
    density) takes the brick and launch shape the autotuner measures on its own points."""
    import torch
    from gbgperiodicfields_gb300 import autotune, resident
    rng = np.random.default_rng(7)
    insts, tuned = [], {}
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
        k = autotune.key(grid.grid_size, C, scheme, M)
        if k not in tuned:
            tuned[k] = autotune.tune(grid, C, scheme, pos, bricks=((11, 8, 8), (15, 8, 8), (7, 8, 8), (7, 4, 4)),
                                     reps=1, persist=False)
        cfg = tuned[k]
        bins = autotune.apply(resident.PointBins(grid, M, brick=cfg["brick"]).build(pos), cfg)
        insts.append(dict(field=field, dest=dest, bins=bins, scheme=scheme, pos=pos, M=M,
                          out=gbg.empty_colmajor((M, C), torch.float32, dev),
                          q=gbg.colmajor(torch.randn((M, C), device=dev))))
        torch.cuda.empty_cache()
    total = sum(i["M"] for i in insts)
    batch = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], out=i["out"], dest=i["dest"],
                                 q=i["q"]) for i in insts])
    gathers = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], out=i["out"]) for i in insts])
    scatters = resident.Batch([dict(field=i["field"], bins=i["bins"], scheme=i["scheme"], dest=i["dest"], q=i["q"])
                               for i in insts])

    def step():
        resident.build_bins([(i["bins"], i["pos"]) for i in insts])
        batch.run()

    def seq():
        for i in insts:
            i["bins"].build(i["pos"])
            resident.interpolate_binned(i["field"], i["bins"], i["scheme"], out=i["out"])
            resident.anterpolate_binned(i["dest"], i["bins"], i["scheme"], i["q"])

    t_seq = _time_ms(seq)
    phases = {"bins_builds": _time_ms(lambda: resident.build_bins([(i["bins"], i["pos"]) for i in insts])),
              "gathers": _time_ms(gathers.run), "scatters": _time_ms(scatters.run), "batch": _time_ms(batch.run)}
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
                       "cubic/quintic, FP32 resident, bricks and threads from the autotuner per class; "
                       "batched bins builds + the batch, CUDA graph",
           "points": int(total), "value": 2 * total / (t_graph / 1e3), "unit": UNIT,
           "ms_per_step": t_graph, "sequential_ms": t_seq, "phase_ms": phases,
           "tuned_classes": len(tuned),
           "paths": {"pooled_instances": sum(1 for i in insts if i["M"] < 1024),
                     "sparse_instances": sum(1 for i in insts if i["M"] < 4 * i["bins"].nbricks_count()),
                     "instances": len(insts)}}
    del insts, batch, gathers, scatters, graph
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


# ----------------------------------------------------------- CPU legs

_LAST: dict = {}


def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    return oracle


def cpu_transfer_step(oracle, g, field_h, dep_h, pos_h, q_h, lo, hi, coeffs, cores):
    """The reference's CPU path on points lo..hi-1: its traversal order, the gather of
    every component at those points, and the atomic scatter of their quantities into the
    full field (beta = 0, so the field is cleared first, as anterpolate! does).  Returns
    the wall time."""
    p = np.asfortranarray(pos_h[lo:hi])
    qq = np.asfortranarray(q_h[lo:hi].astype(np.float64))
    t0 = time.perf_counter()
    trav = oracle.traversal_order(g, p)
    oracle.gather(g, field_h, p, coeffs, traversal=trav, nthreads=cores)
    oracle.scatter(g, dep_h, p, qq, coeffs, 1.0, 0.0, traversal=trav, nthreads=cores)
    return time.perf_counter() - t0


def cpu_baseline(field_h, block: int, reps: int = 3):
    """The reference's CPU path (the oracle's OpenMP restatement, all host cores) on the
    headline workload: blocks of `block` of the 3.2e7 points against the full 512^3 x 12
    FP64 field, timed per block (the best of `reps`)."""
    oracle = _oracle()
    g = oracle.grid_dict(N3)
    coeffs = oracle.lalescu(4)
    cores = os.cpu_count() or 1
    pos_h = c3_points_host()
    dep_h = np.empty(field_h.shape, order="F")
    best = float("inf")
    for r in range(reps):
        lo = r * block
        q_h = c3_quantities_host((lo, lo + block))
        best = min(best, cpu_transfer_step(oracle, g, field_h, dep_h, pos_h[lo:lo + block], q_h, 0, block,
                                           coeffs, cores))
    return {"value": 2 * block / best, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{block} of the {M3} points per timed block (traversal order, gather of 12 components, "
                      f"atomic scatter into the full 512^3 x 12 FP64 field with beta=0), best of {reps}: {best:.2f} s"}


def oracle_checks():
    """The headline's gather (last timed step) at 1e6 points spread over the slots, and the
    precision-form scatter of those points on their own, against the FP64 oracle on the
    full FP64 field; the plain-FP64 workload's four outputs over all 1e7 points.  Errors
    are max and RMS relative to max|oracle|."""
    if not _LAST:
        return None
    oracle = _oracle()
    cores = os.cpu_count() or 1
    res = {}

    def rel(got, want):
        # one component (the last axis) at a time, so no full-size temporaries are made
        got = np.asarray(got).reshape(want.shape, order="F")
        scale, dmax, dsq = 0.0, 0.0, 0.0
        for c in range(want.shape[-1]):
            w = want[..., c]
            d = got[..., c].astype(np.float64) - w
            scale = max(scale, float(np.abs(w).max()))
            dmax = max(dmax, float(np.abs(d).max()))
            dsq += float(np.sum(d * d))
        return {"max_rel": dmax / scale, "rms_rel": float(np.sqrt(dsq / want.size)) / scale}

    if "gather_rows" in _LAST:
        t0 = time.perf_counter()
        g = oracle.grid_dict(N3)
        c = oracle.lalescu(4)
        idx = _LAST["check_idx"]
        gen = _LAST["perm_h"][idx]  # generation indices of the checked slots
        pos_h = c3_points_host()
        p = np.asfortranarray(pos_h[gen])
        del pos_h
        f = _LAST.pop("f64_host")
        want_g = oracle.gather(g, f, p, c, nthreads=cores)
        qall = np.empty((len(gen), C3), dtype=np.float32)
        order = np.argsort(gen)
        blk = 1_000_000
        for b in np.unique(gen // blk):
            sel = order[(gen[order] // blk) == b]
            rows = c3_quantities_host((int(b) * blk, int(b) * blk + blk))
            qall[sel] = rows[gen[sel] - int(b) * blk]
        want_s = oracle.scatter(g, np.empty(f.shape, order="F"), p, np.asfortranarray(qall.astype(np.float64)), c,
                                1.0, 0.0, nthreads=cores)
        del f
        res["precision_form"] = {"points": int(len(idx)), "bar": 1e-5,
                                 "gather": rel(_LAST.pop("gather_rows"), want_g),
                                 "scatter": rel(_LAST.pop("scatter_field"), want_s),
                                 "oracle_seconds": round(time.perf_counter() - t0, 1)}
        del want_s
    if "c2_field" in _LAST:
        t0 = time.perf_counter()
        g = oracle.grid_dict(N2G)
        f, p, qq = _LAST.pop("c2_field"), _LAST.pop("c2_pos"), _LAST.pop("c2_q")
        outs, deps = _LAST.pop("c2_out"), _LAST.pop("c2_dep")
        r = {"points": M2, "bar": 1e-13}
        for name, width in (("cubic", 4), ("quintic", 6)):
            cf = oracle.lalescu(width)
            r["gather_" + name] = rel(outs[name], oracle.gather(g, f, p, cf, nthreads=cores))
            r["scatter_" + name] = rel(deps[name], oracle.scatter(g, np.zeros(f.shape, order="F"), p, qq, cf, 1.0, 0.0,
                                                                  nthreads=cores))
        r["oracle_seconds"] = round(time.perf_counter() - t0, 1)
        res["plain_fp64_form"] = r
    _LAST.clear()
    return res


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU path on the headline workload, on this
    machine's host cores.  Every step runs the traversal order, the gather and the atomic
    scatter (into the full FP64 field, cleared first) on the next block of the points; the
    whole K-step region is timed, and the warm-up steps run first on smaller blocks."""
    if rank != 0:
        return None
    from __graft_entry__ import load_package
    load_package()
    from gbgperiodicfields_gb300.workloads import spectral_field
    import torch
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    oracle = _oracle()
    g = oracle.grid_dict(N3)
    coeffs = oracle.lalescu(4)
    field_h = spectral_field(N3, 3, kmax=KMAX3, seed=3, project=True, gradient=True, device="cpu")
    pos_h = c3_points_host()
    dep_h = np.empty(field_h.shape, order="F")
    block = min(int(args.cpu_block), M3 // 2)
    wblock = max(1, block // 10)
    for w in range(args.warmup):
        lo = (w * wblock) % (M3 - wblock)
        q_w = c3_quantities_host((lo, lo + wblock))
        cpu_transfer_step(oracle, g, field_h, dep_h, pos_h[lo:lo + wblock], q_w, 0, wblock, coeffs, cores)
    qs = [c3_quantities_host(((k * block) % (M3 - block), (k * block) % (M3 - block) + block))
          for k in range(args.steps)]
    times = []
    t0 = time.perf_counter()
    for k in range(args.steps):
        lo = (k * block) % (M3 - block)
        times.append(cpu_transfer_step(oracle, g, field_h, dep_h, pos_h[lo:lo + block], qs[k], 0, block, coeffs,
                                       cores))
    total = time.perf_counter() - t0
    value = 2 * block * args.steps / total
    sample = (f"{block} of the {M3} points per step (the next block each step; traversal order, gather of 12 "
              f"components, atomic scatter into the full 512^3 x 12 FP64 field with beta=0), {args.steps} steps "
              f"timed back to back: {total:.1f} s")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "per_step_s": [round(t, 3) for t in times]}


# ------------------------------------------------------- profiling cases

def case_resident(n=256, C=12, M=4_000_000, brick=(15, 8, 8), gather_threads=512, scatter_threads=256):
    """256^3 x 12 FP32 resident field (0.85 GB), 4e6 uniform points in binned order,
    bins + cubic gather and scatter, twice, at 15x8x8 bricks, 512 gather and 256 scatter
    threads (the tuned launch shape)."""
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
    bins.set_launch(gather_threads, scatter_threads)
    out = gbg.empty_colmajor((M, C), torch.float32, dev)
    q = gbg.colmajor(torch.randn((M, C), dtype=torch.float32, device=dev))
    for _ in range(2):
        bins.build(pos)
        resident.interpolate_binned(field, bins, gbg.CatmullRom, out=out)
        resident.anterpolate_binned(field, bins, gbg.CatmullRom, q)
    torch.cuda.synchronize()


def case_resident_full():
    """The headline step at full size: 512^3 x 12 FP32 resident field, 3.2e7 points in
    binned order, bins + cubic gather + scatter, twice (for a one-pass launch list only)."""
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


def case_plain(n=256, M=4_000_000, width=6):
    """256^3 x 3 FP64 field (403 MB, above L2), 4e6 clustered points, scatter and gather
    through the drop-in API (quintic by default), twice."""
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
    s = gbg.LalescuSpline(width) if width != 4 else gbg.CatmullRom
    for _ in range(2):
        gbg.anterpolate_(f, pts, q, s, 1.0, 0.0)
        gbg.interpolate(f, pts, s, traversal=order)
    torch.cuda.synchronize()


def case_plain_cubic():
    """The same as plain_256c3_4e6_quintic with the cubic (CatmullRom) scheme."""
    case_plain(width=4)


PROFILE_CASES = {"resident_256c12_4e6": case_resident, "resident_512c12_3p2e7": case_resident_full,
                 "plain_256c3_4e6_quintic": case_plain, "plain_256c3_4e6_cubic": case_plain_cubic,
                 "nufft_64c3_5e5": case_nufft}


def main():
    args = parse()
    if args.case:
        PROFILE_CASES[args.case]()
        print(json.dumps({"case": args.case, "ok": True}))
        return
    shrink_workload(args.shrink)
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
            f = _LAST.get("f64_host")
            if f is not None:
                res["cpu_baseline"] = cpu_baseline(f, min(args.cpu_block, 2_000_000, M3 // 4))
            res["error_vs_oracle"] = oracle_checks()
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
