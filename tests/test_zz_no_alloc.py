"""The allocation-free scatter, gbg_anterpolate_noalloc, against gbg_anterpolate.

Some callers cannot allocate device memory while they run: a host that reserves the GPU's
memory up front and hands out only its own pool, or a caller held to the reference's rule
that the in-place anterpolate! allocates nothing.  For them the library keeps a fixed
64 MiB scratch array compiled into its device image, and gbg_anterpolate_noalloc uses it
instead of allocating.  This test calls that entry point through the C ABI twice in a row
(the second call on different inputs, so stale contents left by the first call would
show) and checks each result against the allocating entry point's, with the tolerance the
other scatter tests use (here both are deterministic, so the results also agree bitwise).
It runs alone in a fresh process or after every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi


def _scatter(gbg, lib, grid, field, pos, q, scheme, alpha, beta, noalloc):
    m = pos.shape[0]
    status = torch.zeros(1, dtype=torch.int32, device=field.device)
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
def test_noalloc_matches_allocating_scatter_twice(gbg, dtype, tol):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda:0")
    lib = gbg._lib.load()
    grid = gbg.Grid3D((24, 20, 18), (TWO_PI,) * 3, origin=(0.2, -0.5, 1.0), dtype=dtype)
    rng = np.random.default_rng(77)
    for call, (m, scheme, alpha, beta) in enumerate(((5000, gbg.CatmullRom, 1.0, 0.0),
                                                     (3000, gbg.LalescuSpline(6), 0.5, 2.0))):
        pos = gbg.colmajor(torch.from_numpy(np.asfortranarray(
            TWO_PI * rng.random((m, 3)) - 1.0)).to(dev, dtype))
        q = gbg.colmajor(torch.from_numpy(np.asfortranarray(rng.standard_normal((m, 3)))).to(dev, dtype))
        prior = gbg.colmajor(torch.from_numpy(np.asfortranarray(rng.standard_normal((24, 20, 18, 3)))).to(dev, dtype))
        want = _scatter(gbg, lib, grid, prior.clone(memory_format=torch.preserve_format), pos, q, scheme,
                        alpha, beta, noalloc=False)
        got = _scatter(gbg, lib, grid, prior.clone(memory_format=torch.preserve_format), pos, q, scheme,
                       alpha, beta, noalloc=True)
        err = (got - want).abs().max().item() / want.abs().max().item()
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
