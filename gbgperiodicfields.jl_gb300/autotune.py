"""Autotuner of the resident and batched forms' launch shape: the bin (brick) edges, the
field's ghost width (halo) and the threads per CTA of the binned gather and scatter.

`tune()` times candidate configurations on the caller's grid, component count, scheme
and a sample of its positions (CUDA events, best of a few runs), and persists the winner
in a JSON cache keyed by (grid, components, stencil width and powers, storage dtype,
points-per-cell bucket).  `choose()` returns the cached choice for a problem, or the
rule-of-thumb configuration when nothing has been tuned for it.

The candidates keep the gather's shared-memory tile conflict-free (tile row of brick_x +
width - 1 nodes, 2 modulo 4 for width 4) where they can and leave at least two bricks
per SM for small grids."""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

import torch

from . import _lib

DEFAULT_BRICK = (11, 8, 8)
BRICKS = ((11, 8, 8), (7, 8, 8), (15, 8, 8), (11, 4, 4), (7, 4, 4), (11, 12, 8), (3, 4, 4))
GATHER_THREADS = (256, 512)
SCATTER_THREADS = (128, 256)


def cache_path() -> Path:
    p = os.environ.get("GBG_TUNE_CACHE")
    if p:
        return Path(p)
    return Path.home() / ".cache" / "gbgperiodicfields_gb300" / "tune.json"


def _density_bucket(npoints: int, grid_size) -> int:
    cells = math.prod(int(n) for n in grid_size)
    return int(round(math.log2(max(npoints, 1) / cells)))


def key(grid_size, ncomp: int, scheme, npoints: int, dtype: str = "f32") -> str:
    n = "x".join(str(int(v)) for v in grid_size)
    return (f"{n}|C{int(ncomp)}|w{scheme.stencil_width}m{scheme.c().num_powers}|{dtype}"
            f"|d{_density_bucket(npoints, grid_size)}")


def _load() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store(entries: dict):
    p = cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(entries, indent=1, sort_keys=True))
    os.replace(tmp, p)


def heuristic(grid_size, ncomp: int, scheme, npoints: int) -> dict:
    """Default brick unless the grid has fewer than two default bricks per SM; then the
    largest candidate that gives at least that many."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 152

    def nbricks(b):
        return math.prod(-(-int(n) // e) for n, e in zip(grid_size, b))

    if nbricks(DEFAULT_BRICK) >= 2 * sms:
        brick = DEFAULT_BRICK
    else:
        enough = [b for b in BRICKS if nbricks(b) >= 2 * sms]
        brick = max(enough, key=math.prod) if enough else min(BRICKS, key=math.prod)
    return {"brick": list(brick), "gather_threads": 0, "scatter_threads": 0,
            "max_stencil_width": int(scheme.stencil_width), "source": "heuristic"}


def choose(grid_size, ncomp: int, scheme, npoints: int) -> dict:
    """The tuned configuration for this problem class, else the heuristic one."""
    got = _load().get(key(grid_size, ncomp, scheme, npoints))
    if got:
        return dict(got, source="cache")
    return heuristic(grid_size, ncomp, scheme, npoints)


def _time(fn, reps: int) -> float:
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


def tune(grid, ncomp: int, scheme, positions: torch.Tensor, *, bricks=BRICKS, gather_threads=GATHER_THREADS,
         scatter_threads=SCATTER_THREADS, reps: int = 3, persist: bool = True) -> dict:
    """Time every candidate on these positions and keep the fastest gather + scatter."""
    from .resident import PointBins, ResidentField, anterpolate_binned, interpolate_binned
    from .api import colmajor, empty_colmajor
    positions = colmajor(positions)
    m = int(positions.shape[0])
    width = int(scheme.stencil_width)
    n = tuple(int(v) for v in grid.grid_size)
    field = ResidentField(grid, ncomp, max_stencil_width=width)
    field.load(torch.randn((ncomp,) + n[::-1], device=positions.device).permute(3, 2, 1, 0))
    dest = ResidentField(grid, ncomp, max_stencil_width=width)
    out = empty_colmajor((m, ncomp), torch.float32, positions.device)
    q = colmajor(torch.randn((m, ncomp), device=positions.device))
    trials = []
    for brick in bricks:
        try:
            bins = PointBins(grid, m, brick=brick).build(positions)
        except (_lib.GBGError, _lib.ArgumentError):
            continue
        best_g = best_s = None
        for gt in gather_threads:
            try:
                bins.set_launch(gt, 0)
                t = _time(lambda: interpolate_binned(field, bins, scheme, out=out), reps)
            except (_lib.GBGError, _lib.ArgumentError):
                continue
            if best_g is None or t < best_g[1]:
                best_g = (gt, t)
        for stt in scatter_threads:
            try:
                bins.set_launch(0, stt)
                t = _time(lambda: anterpolate_binned(dest, bins, scheme, q), reps)
            except (_lib.GBGError, _lib.ArgumentError):
                continue
            if best_s is None or t < best_s[1]:
                best_s = (stt, t)
        if best_g and best_s:
            trials.append({"brick": list(brick), "gather_threads": best_g[0], "scatter_threads": best_s[0],
                           "gather_ms": best_g[1], "scatter_ms": best_s[1], "ms": best_g[1] + best_s[1]})
    if not trials:
        raise _lib.GBGError(_lib.GBG_EUNSUPPORTED, "no candidate configuration ran")
    win = min(trials, key=lambda t: t["ms"])
    result = {"brick": win["brick"], "gather_threads": win["gather_threads"],
              "scatter_threads": win["scatter_threads"], "max_stencil_width": width,
              "ms": win["ms"], "trials": trials}
    if persist:
        entries = _load()
        entries[key(n, ncomp, scheme, m)] = {k: v for k, v in result.items() if k != "trials"}
        _store(entries)
    return result


def apply(bins, config: dict):
    """Set a chosen configuration's launch knobs on bins built with its brick."""
    return bins.set_launch(int(config.get("gather_threads", 0)), int(config.get("scatter_threads", 0)))
