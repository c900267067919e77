"""GPU tests of the checkpoint of resident serving state: resident fields, the bins'
configuration and positions, point values and schemes written to one HDF5 file and
restored.  The restored fields hold the same bits, the rebuilt bins the same binned
order, and the binned gather and scatter on the restored state give bitwise the results
of the original state; a read scheme interpolates bitwise like the one written
(the reference's test/hdf5.jl:286-330 claim)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TWO_PI = 2 * math.pi


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def test_resident_state_round_trips_bitwise(gbg, dev, tmp_path):
    from gbgperiodicfields_gb300 import checkpoint as ck
    from gbgperiodicfields_gb300 import h5, resident
    rng = np.random.default_rng(31)
    grid = gbg.Grid3D((40, 36, 32), (TWO_PI,) * 3, origin=(0.1, -0.2, 0.3))
    M = 60000
    f12 = resident.ResidentField(grid, 12, max_stencil_width=6).load(
        torch.from_numpy(np.asfortranarray(rng.standard_normal((40, 36, 32, 12)))).cuda())
    f3 = resident.ResidentField(grid, 3, max_stencil_width=4).load(
        torch.from_numpy(np.asfortranarray(rng.standard_normal((40, 36, 32, 3)))).cuda())
    pos = gbg.colmajor(torch.from_numpy(np.asfortranarray(TWO_PI * rng.random((M, 3)) - 1.0)).cuda())
    bins = resident.PointBins(grid, M, brick=(11, 8, 8)).build(pos)
    bins.set_launch(128, 128)
    q = gbg.colmajor(torch.from_numpy(np.asfortranarray(rng.standard_normal((M, 12)))).float().cuda())
    scheme = gbg.LalescuSpline(6)

    def results(fa, fb, b, s):
        g12 = resident.interpolate_binned(fa, b, s)
        g3 = resident.interpolate_binned(fb, b, gbg.CatmullRom)
        dest = resident.ResidentField(grid, 12, max_stencil_width=6)
        resident.anterpolate_binned(dest, b, s, q)
        torch.cuda.synchronize()
        return g12, g3, dest.read(dtype=torch.float32)

    want = results(f12, f3, bins, scheme)
    p = tmp_path / "state.h5"
    ck.save_state(p, resident={"u": f12, "v": f3}, bins={"b": (bins, pos)}, schemes={"s": scheme},
                  values={"q": gbg.AbstractPointValues(q[:, :3].cpu(), 1)}, attrs={"iteration": 17})
    state = ck.load_state(p)
    r12, r3 = state["resident"]["u"], state["resident"]["v"]
    rbins, rpos = state["bins"]["b"]
    assert state["attrs"]["iteration"] == 17
    assert r12.ncomp == 12 and r3.ncomp == 3 and r12.grid == grid and r3.max_stencil_width == 4
    assert torch.equal(r12.read(dtype=torch.float32), f12.read(dtype=torch.float32))
    assert torch.equal(r3.read(dtype=torch.float32), f3.read(dtype=torch.float32))
    assert torch.equal(rpos, pos) and rbins.brick == (11, 8, 8)
    assert torch.equal(rbins.order(), bins.order())
    assert state["schemes"]["s"] == scheme
    assert torch.equal(state["values"]["q"].data.cpu(), q[:, :3].cpu())
    got = results(r12, r3, rbins, state["schemes"]["s"])
    for a, b in zip(got, want):
        assert torch.equal(a, b)
    # the 3-component resident field is a reference VectorFieldPhysical group of Float32
    with h5.File(p) as f:
        assert f["resident/v"].attrs["type"] == "GBGPeriodicFields.VectorFieldPhysical"
        assert f["resident/u"].attrs["type"] == ck.RESIDENT_TAG
        fld = ck.read_field(f["resident"], "v")
        assert fld.data.dtype == torch.float32 and tuple(fld.data.shape) == (40, 36, 32, 3)
        assert torch.equal(fld.data, f3.read(dtype=torch.float32, device="cpu"))


def test_read_scheme_interpolates_bitwise_like_the_written_one(gbg, dev, tmp_path):
    from gbgperiodicfields_gb300 import checkpoint as ck
    from gbgperiodicfields_gb300 import h5
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    field = gbg.sample_field(lambda x, y, z: torch.sin(x) * torch.cos(y) + 0.3 * torch.sin(z), grid)
    points = gbg.PointSet(gbg.colmajor(TWO_PI * torch.rand(16, 3, dtype=torch.float64)).cuda())
    for scheme in (gbg.CatmullRom, gbg.LagrangeSpline(6), gbg.LalescuSpline(8, smoothness=2)):
        p = tmp_path / "behave.h5"
        with h5.File(p, "a") as f:
            if "behave" in f:
                del f["behave"]
            ck.write_scheme(f, "behave", scheme)
        with h5.File(p) as f:
            back = ck.read_scheme(f, "behave")
        assert torch.equal(gbg.interpolate(field, points, back).data, gbg.interpolate(field, points, scheme).data)
