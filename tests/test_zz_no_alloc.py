"""The allocation-free scatter, gbg_anterpolate_noalloc, against gbg_anterpolate.

Some callers cannot allocate device memory while they run: a host that reserves the GPU's
memory up front and hands out only its own pool, or a caller held to the reference's rule
that the in-place anterpolate! allocates nothing.  For them the library keeps a fixed
64 MiB scratch array compiled into its device image, and gbg_anterpolate_noalloc uses it
instead of allocating.  This test calls that entry point through the C ABI twice in a row
(the second call on different inputs, so stale contents left by the first call would
show) and checks each result against the FP64 oracle, with the tolerance the other
scatter tests use, and against the allocating entry point's (both are deterministic, so
the results agree bitwise).  Around the two calls it checks that no device memory was
taken: the device's free memory, torch's reserved bytes and the default memory pool's
used-memory high-water mark are unchanged.  It runs alone in a fresh process or after
every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi


class _DeviceMemory:
    """Snapshots of the device's memory through the CUDA driver API: free bytes
    (cuMemGetInfo) and the default pool's used-memory high-water mark
    (cuMemPoolGetAttribute), which reset() brings down to the pool's current use."""
    USED_MEM_HIGH = 8  # CU_MEMPOOL_ATTR_USED_MEM_HIGH

    def __init__(self, ordinal):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), ordinal) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def reset(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def snapshot(self):
        torch.cuda.synchronize()
        free, total, high = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_uint64()
        assert self.cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
        assert self.cu.cuMemPoolGetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(high)) == 0
        return dict(free=free.value, pool_high=high.value, torch_reserved=torch.cuda.memory_reserved())


def _scatter(gbg, lib, grid, field, pos, q, scheme, alpha, beta, noalloc, status=None):
    m = pos.shape[0]
    if status is None:
        status = torch.zeros(1, dtype=torch.int32, device=field.device)
    status.zero_()
    stream = torch.cuda.current_stream().cuda_stream
    dt = gbg._lib.GBG_F64 if field.dtype == torch.float64 else gbg._lib.GBG_F32
    ncomp = field.shape[3] if field.dim() == 4 else 1
    if noalloc:
        st = lib.gbg_anterpolate_noalloc(grid.c(), dt, ncomp, field.data_ptr(), pos.data_ptr(), m, q.data_ptr(),
                                         scheme.c(), alpha, beta, status.data_ptr(), stream)
    else:
        nbytes = ctypes.c_size_t()
        gbg._lib.check(lib.gbg_anterpolate_workspace_size(grid.c(), dt, ncomp, m, scheme.c(), ctypes.byref(nbytes)))
        ws = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device=field.device)
        st = lib.gbg_anterpolate(grid.c(), dt, ncomp, field.data_ptr(), pos.data_ptr(), m, q.data_ptr(), None,
                                 scheme.c(), alpha, beta, ws.data_ptr(), ws.numel(), status.data_ptr(), stream)
    gbg._lib.check(st, "anterpolate")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return field


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-13), (torch.float32, 2e-5)])
def test_noalloc_matches_oracle_and_allocating_scatter_twice(gbg, oracle, dtype, tol):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda:0")
    lib = gbg._lib.load()
    n = (24, 20, 18)
    origin = (0.2, -0.5, 1.0)
    grid = gbg.Grid3D(n, (TWO_PI,) * 3, origin=origin, dtype=dtype)
    g = oracle.grid_dict(n, (TWO_PI,) * 3, origin)
    rng = np.random.default_rng(77)
    cases = []
    for m, scheme, alpha, beta in ((5000, gbg.CatmullRom, 1.0, 0.0), (3000, gbg.LalescuSpline(6), 0.5, 2.0)):
        pos = np.asfortranarray(TWO_PI * rng.random((m, 3)) - 1.0)
        q = np.asfortranarray(rng.standard_normal((m, 3)))
        prior = np.asfortranarray(rng.standard_normal(n + (3,)))
        if dtype == torch.float32:  # the oracle sees the very values the GPU sees
            pos, q, prior = (np.asfortranarray(a.astype(np.float32).astype(np.float64)) for a in (pos, q, prior))
        cases.append((pos, q, prior, scheme, alpha, beta))
    dev_t = lambda a: gbg.colmajor(torch.from_numpy(a).to(dev, dtype))
    # the allocating entry point first: its kernels share the library's device image with
    # the static scratch, so the image is loaded before the memory snapshots
    wants = [_scatter(gbg, lib, grid, dev_t(prior), dev_t(pos), dev_t(q), scheme, alpha, beta, noalloc=False)
             for pos, q, prior, scheme, alpha, beta in cases]
    inputs = [(dev_t(pos), dev_t(q), dev_t(prior)) for pos, q, prior, *_ in cases]
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    mem = _DeviceMemory(dev.index or 0)
    mem.reset()
    before = mem.snapshot()
    gots = [_scatter(gbg, lib, grid, prior_t, pos_t, q_t, c[3], c[4], c[5], noalloc=True, status=status)
            for (pos_t, q_t, prior_t), c in zip(inputs, cases)]
    after = mem.snapshot()
    assert after == before, (before, after)
    for call, ((pos, q, prior, scheme, alpha, beta), got, want) in enumerate(zip(cases, gots, wants)):
        ref = oracle.scatter(g, prior.copy(order="F"), pos, q, scheme.coefficients, alpha, beta)
        err = np.abs(got.cpu().numpy().astype(np.float64) - ref).max() / np.abs(ref).max()
        assert err <= tol, (call, err)
        assert torch.equal(got, want), call


def test_noalloc_refuses_oversized_problems(gbg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = gbg._lib.load()
    grid = gbg.Grid3D((64, 64, 64), (TWO_PI,) * 3)
    # 10^6 Float64 points of 9 components need far more than the 64 MiB static scratch;
    # the size check happens before any pointer is touched.
    st = lib.gbg_anterpolate_noalloc(grid.c(), gbg._lib.GBG_F64, 9, 1, 1, 1_000_000, 1, gbg.CatmullRom.c(),
                                     1.0, 0.0, None, None)
    assert st == gbg._lib.GBG_EUNSUPPORTED
    assert "static scratch" in gbg._lib.last_error()
