"""Serving form over the C ABI (gbg_server_*): resident fields, gather/scatter requests
admitted by free device memory and batched as they arrive onto stream slots, with
p50/p99 latency and throughput counters.

The loop itself is native (a C++ progress thread in libgbg_gb300.so); this module keeps
the request's tensors alive until the request has completed and orders the server's
work after the caller's stream with one CUDA event per request."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _lib
from .api import _DTYPE_CODE, colmajor, empty_colmajor
from .resident import ResidentField


@dataclass
class Ticket:
    id: int
    kind: int
    out: torch.Tensor | None
    keep: tuple


class Server:
    """A request loop over resident fields.

    slots       runs in flight at once (one CUDA stream each)
    max_batch   requests merged into one batched launch
    hbm_budget  device bytes the server may hold for requests (0: half the free memory)
    timeout     deadline of one run's device work, in seconds
    """

    def __init__(self, slots: int = 4, max_batch: int = 16, brick=None, hbm_budget: int = 0,
                 timeout: float = 10.0):
        cfg = _lib.ServerConfigC()
        cfg.slots = int(slots)
        cfg.max_batch = int(max_batch)
        for d in range(3):
            cfg.brick[d] = int(brick[d]) if brick is not None else 0
        cfg.hbm_budget_bytes = int(hbm_budget)
        cfg.timeout_seconds = float(timeout)
        h = ctypes.c_void_p()
        _lib.check(_lib.load().gbg_server_create(ctypes.byref(cfg), ctypes.byref(h)), "gbg_server_create")
        self.handle = h
        self.timeout = float(timeout)
        self._tickets: dict[int, Ticket] = {}

    # -- requests
    def _submit(self, kind, field: ResidentField, positions, scheme, out=None, q=None, alpha=1.0, beta=0.0):
        positions = colmajor(positions)
        if positions.dim() != 2 or positions.shape[1] != 3 or not positions.is_cuda:
            raise _lib.ArgumentError("positions must be a (M, 3) CUDA tensor")
        m = int(positions.shape[0])
        r = _lib.RequestC()
        r.kind = kind
        r.pos_dtype = _DTYPE_CODE[positions.dtype]
        r.field = field.handle
        r.scheme = scheme.c()
        r.positions = positions.data_ptr()
        r.npoints = m
        if out is not None:
            r.out = out.data_ptr()
        if q is not None:
            r.q = q.data_ptr()
        r.alpha = float(alpha)
        r.beta = float(beta)
        ready = torch.cuda.Event()
        ready.record(torch.cuda.current_stream())
        r.ready_event = ready.cuda_event
        t = ctypes.c_int64()
        _lib.check(_lib.load().gbg_server_submit(self.handle, ctypes.byref(r), ctypes.byref(t)), "gbg_server_submit")
        tk = Ticket(int(t.value), kind, out, (positions, q, ready, field))
        self._tickets[tk.id] = tk
        return tk

    def interpolate(self, field: ResidentField, positions: torch.Tensor, scheme, out: torch.Tensor | None = None):
        """Queue a gather of field at positions; out is FP32 (M, ncomp), column-major."""
        m = int(positions.shape[0])
        if out is None:
            out = empty_colmajor((m, field.ncomp), torch.float32, "cuda")
        if out.dtype != torch.float32 or tuple(out.shape) != (m, field.ncomp) or not out.is_cuda:
            raise _lib.ArgumentError("out must be a Float32 (M, ncomp) CUDA tensor")
        out = colmajor(out)
        return self._submit(_lib.GBG_REQ_INTERPOLATE, field, positions, scheme, out=out)

    def anterpolate(self, field: ResidentField, positions: torch.Tensor, scheme, q: torch.Tensor,
                    alpha: float = 1.0, beta: float = 0.0):
        """Queue field = alpha * W^T q + beta * field; q is FP32 (M, ncomp)."""
        if not q.is_cuda:
            raise _lib.ArgumentError("q must be a CUDA tensor")
        q = colmajor(q.to(torch.float32))
        if tuple(q.shape) != (int(positions.shape[0]), field.ncomp):
            raise _lib.DimensionMismatch("q must be (M, ncomp)")
        return self._submit(_lib.GBG_REQ_ANTERPOLATE, field, positions, scheme, q=q, alpha=alpha, beta=beta)

    def wait(self, ticket: Ticket, timeout: float | None = None) -> int:
        """Wait for a request; returns its status code (0 = GBG_OK).  Raises GBGError
        (GBG_ETIMEOUT) if it is still pending after `timeout` seconds."""
        res = ctypes.c_int32()
        st = _lib.load().gbg_server_wait(self.handle, ticket.id,
                                         float(self.timeout * 4 if timeout is None else timeout), ctypes.byref(res))
        _lib.check(st, "gbg_server_wait")
        self._tickets.pop(ticket.id, None)
        return int(res.value)

    def result(self, ticket: Ticket, timeout: float | None = None):
        """Wait and raise on a failed request; returns the gather's output (or None)."""
        _lib.check(self.wait(ticket, timeout), f"request {ticket.id}")
        return ticket.out

    def drain(self, timeout: float | None = None):
        _lib.check(_lib.load().gbg_server_drain(self.handle, float(self.timeout * 4 if timeout is None else timeout)),
                   "gbg_server_drain")

    def stats(self, reset: bool = False) -> dict:
        c = _lib.ServerCountersC()
        _lib.check(_lib.load().gbg_server_stats(self.handle, int(reset), ctypes.byref(c)), "gbg_server_stats")
        return {name: getattr(c, name) for name, _ in c._fields_}

    def inject(self, fault: int, count: int = 1):
        _lib.check(_lib.load().gbg_server_inject(self.handle, int(fault), int(count)), "gbg_server_inject")

    def close(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            st = _lib.load().gbg_server_destroy(h)
            self.handle = None
            self._tickets.clear()
            _lib.check(st, "gbg_server_destroy")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan(kinds, fields, nbytes, free_bytes: int, max_batch: int) -> int:
    """The server's admission rule on its own (gbg_server_plan): how many queued requests
    from the head form the next run."""
    n = len(kinds)
    k = (ctypes.c_int32 * max(n, 1))(*kinds)
    f = (ctypes.c_uint64 * max(n, 1))(*fields)
    b = (ctypes.c_size_t * max(n, 1))(*nbytes)
    out = ctypes.c_int32()
    _lib.check(_lib.load().gbg_server_plan(k, f, b, n, int(free_bytes), int(max_batch), ctypes.byref(out)),
               "gbg_server_plan")
    return int(out.value)
