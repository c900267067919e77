"""HDF5 persistence on the CPU: the format layer (h5.py) against files libhdf5 wrote, and
the reference's persistence verbs (checkpoint.py) through the cases of the reference's
test/hdf5.jl -- exact round trips of every field type, the point layer and the schemes,
self-describing attributes, the schema checks on tampered files, read_field! with its
refusals, and copy-free writes and reads.

Two files written by libhdf5 pin the reader: the reference's own example output
(examples/figures/HIST_CUDA_giant.h5 -- superblock 2, dense link storage in a fractal
heap indexed by a version 2 B-tree, checksummed metadata) and scipy's MATLAB 7.3 test
file (superblock 0 behind a 512-byte user block, symbol-table groups).  Each test that
reads one is skipped where that file is absent."""
import math
import os
import tracemalloc

import numpy as np
import pytest
import torch

TWO_PI = 2 * math.pi
REF_HIST = "/root/reference/examples/figures/HIST_CUDA_giant.h5"


def _scipy_v73():
    try:
        import scipy.io.matlab as m
    except ImportError:
        return None
    p = os.path.join(os.path.dirname(m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    return p if os.path.exists(p) else None


@pytest.fixture(scope="module")
def mods(gbg):
    from gbgperiodicfields_gb300 import checkpoint, h5
    return gbg, h5, checkpoint


def _rand(shape, dtype, rng):
    if dtype in (torch.complex64, torch.complex128):
        real = torch.float32 if dtype == torch.complex64 else torch.float64
        a = torch.complex(torch.from_numpy(rng.random(shape)).to(real), torch.from_numpy(rng.random(shape)).to(real))
    else:
        a = torch.from_numpy(rng.random(shape)).to(dtype)
    from gbgperiodicfields_gb300 import colmajor
    return colmajor(a)


# ------------------------------------------------------------------ the format layer


def test_lookup3_known_answers(mods):
    _, h5, _ = mods
    # the values printed by the driver of Bob Jenkins' lookup3.c
    assert h5.lookup3(b"") == 0xDEADBEEF
    assert h5.lookup3(b"Four score and seven years ago") == 0x17770551
    assert h5.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.mark.skipif(not os.path.exists(REF_HIST), reason="the reference's example output is not present")
def test_reads_the_reference_written_file(mods):
    """A file HDF5.jl (libhdf5) wrote for the reference: every checksum on the way
    (superblock, object headers, fractal heap, B-tree) verifies, and the bundle decodes."""
    _, h5, _ = mods
    with h5.File(REF_HIST) as f:
        assert f._reader.sb_version == 2
        keys = set(f.keys())
        assert {"t", "E", "eps_t", "N", "L_box", "backend", "ek_k", "ek_E"} <= keys
        assert f["N"].read() == 320
        assert f["L_box"].read() == pytest.approx(TWO_PI, rel=1e-15)
        assert f["backend"].read() == "CUDA"
        t, E, eps = f["t"].read(), f["E"].read(), f["eps_t"].read()
        assert t.shape == E.shape == eps.shape == (23000,)
        assert np.all(np.diff(t) > 0) and np.all(np.isfinite(E)) and np.all(eps > 0)
        assert f["ek_k"].read().dtype == np.float32 and f["ek_k"].shape == f["ek_E"].shape
        for k in keys:
            v = f[k].read()
            if isinstance(v, np.ndarray) and v.dtype.kind == "f":
                assert np.all(np.isfinite(v)), k


@pytest.mark.skipif(_scipy_v73() is None, reason="scipy's MATLAB 7.3 test file is not present")
def test_reads_a_superblock_0_file_behind_a_user_block(mods):
    _, h5, _ = mods
    with h5.File(_scipy_v73()) as f:
        assert f._reader.sb_version == 0 and f._reader.base == 512
        d = f["testdouble"]
        assert d.attrs["MATLAB_class"] == "double"
        np.testing.assert_array_equal(d.read().ravel(), np.arange(9) * (math.pi / 4))


def test_written_files_are_self_consistent(mods, tmp_path):
    """What the writer lays out: superblock 2 whose end-of-file address is the file's
    size, and checksummed headers that the reader verifies on the way back."""
    _, h5, _ = mods
    p = tmp_path / "x.h5"
    rng = np.random.default_rng(3)
    a = np.asfortranarray(rng.standard_normal((5, 4, 3)))
    with h5.File(p, "w") as f:
        f["a"] = a
        f["s"] = "text"
        f["i"] = 7
        f["z"] = np.asfortranarray(rng.standard_normal((3, 2)) + 1j * rng.standard_normal((3, 2)))
        g = f.create_group("g/h") if False else f.create_group("g")
        g.create_group("h").attrs["x"] = np.array([1.5, 2.5])
        f.attrs["note"] = "root"
    raw = p.read_bytes()
    assert raw[:8] == h5.SIGNATURE and raw[8] == 2
    assert int.from_bytes(raw[28:36], "little") == len(raw)
    with h5.File(p) as f:
        np.testing.assert_array_equal(f["a"].read(), a)
        assert f["a"].read().flags.f_contiguous and f["a"].shape == (5, 4, 3)
        assert f["s"].read() == "text" and f["i"].read() == 7
        assert f["z"].read().dtype == np.complex128
        np.testing.assert_array_equal(f["g/h"].attrs["x"], [1.5, 2.5])
        assert f.attrs["note"] == "root"
    # the stored dataspace is the reversed shape (HDF5.jl's convention): dims (3, 4, 5)
    with h5.File(p) as f:
        reader, dt, dims, layout = f["a"]._stored
        assert dims == (3, 4, 5)


def test_modify_keeps_untouched_data_and_exceptions_write_nothing(mods, tmp_path):
    _, h5, _ = mods
    p = tmp_path / "m.h5"
    big = np.asfortranarray(np.arange(200000, dtype=np.float64).reshape(100, 2000, order="F"))
    with h5.File(p, "w") as f:
        f["big"] = big
        f["drop"] = np.ones(3)
        f["big"].attrs["a"] = 1
    with h5.File(p, "r+") as f:
        del f["drop"]
        del f["big"].attrs["a"]
        f["big"].attrs["b"] = "two"
        f.create_group("new")["v"] = np.float32(1.25)
    with h5.File(p) as f:
        assert set(f.keys()) == {"big", "new"}
        np.testing.assert_array_equal(f["big"].read(), big)
        assert dict(f["big"].attrs) == {"b": "two"}
        v = f["new/v"].read()
        assert v == 1.25 and f["new/v"].dtype == np.float32
    before = p.read_bytes()
    with pytest.raises(RuntimeError):
        with h5.File(p, "r+") as f:
            del f["big"]
            raise RuntimeError("abandon")
    assert p.read_bytes() == before
    assert [n for n in os.listdir(tmp_path) if n.startswith(".h5tmp")] == []
    with h5.File(tmp_path / "new.h5", "a") as f:  # "a" (Julia's "cw") creates
        f["x"] = np.zeros(2)
    with h5.File(tmp_path / "new.h5", "cw") as f:
        assert "x" in f
        f["y"] = 1


def test_dataset_data_is_captured_when_written(mods, tmp_path):
    """Like HDF5's own write: a change to the array after the write does not reach the
    file."""
    _, h5, _ = mods
    a = np.zeros((4, 4), order="F")
    p = tmp_path / "c.h5"
    with h5.File(p, "w") as f:
        f["a"] = a
        a[:] = 5
        np.testing.assert_array_equal(f["a"].read(), 0)
    with h5.File(p) as f:
        np.testing.assert_array_equal(f["a"].read(), 0)


@pytest.mark.parametrize("level", [None, 0, 6])
def test_chunked_datasets_round_trip(mods, tmp_path, level):
    """Chunked datasets (edge chunks stored whole; deflated when a level is given) read back
    exactly through the reader's chunk B-tree walk: before close from the chunk list, after
    close from the file, and after a rewrite in append mode (which stores them whole).  300
    chunks need a second B-tree level (64 chunks a leaf)."""
    _, h5, _ = mods
    rng = np.random.default_rng(5)
    cases = {"f64": (rng.standard_normal((13, 7, 5)), (4, 3, 2)),
             "i32": (rng.integers(-9, 9, (40, 30, 3)).astype(np.int32), (2, 2, 3)),
             "c128": (rng.standard_normal((9, 4)) + 1j * rng.standard_normal((9, 4)), (5, 4)),
             "f32": (rng.standard_normal(100).astype(np.float32), (7,))}
    p = tmp_path / "chunked.h5"
    with h5.File(p, "w") as f:
        for name, (a, ch) in cases.items():
            ds = f.create_dataset(name, np.asfortranarray(a), chunks=ch, compression=level)
            np.testing.assert_array_equal(ds.read(), a)
    with h5.File(p) as f:
        for name, (a, ch) in cases.items():
            layout = f[name]._stored[3]
            assert layout["class"] == "chunked" and layout["filters"] == ([] if level is None else [1])
            assert tuple(layout["chunk"]) == tuple(reversed(ch))
            got = f[name].read()
            assert got.dtype == a.dtype and got.shape == a.shape
            np.testing.assert_array_equal(got, a)
            out = np.empty(a.shape, a.dtype, order="F")
            np.testing.assert_array_equal(f[name].read_into(out), a)
    with h5.File(p, "a") as f:
        f.create_dataset("more", np.arange(3.0))
    with h5.File(p) as f:
        for name, (a, _) in cases.items():
            np.testing.assert_array_equal(f[name].read(), a)


def test_chunked_dataset_refusals(mods, tmp_path):
    _, h5, _ = mods
    with h5.File(tmp_path / "r.h5", "w") as f:
        with pytest.raises(h5.H5Error):
            f.create_dataset("a", np.zeros((4, 4)), chunks=(2,))           # one extent per axis
        with pytest.raises(h5.H5Error):
            f.create_dataset("b", np.zeros((4, 4)), chunks=(0, 2))         # extents >= 1
        with pytest.raises(h5.H5Error):
            f.create_dataset("c", np.zeros((4, 4)), compression=4)         # deflate needs chunks
        with pytest.raises(h5.H5Error):
            f.create_dataset("d", "text", chunks=(1,))                     # numeric arrays only
        with pytest.raises(h5.H5Error):
            f.create_dataset("e", np.zeros((4, 4)), chunks=(2, 2), compression=12)


# ------------------------------------------------------------------ fields


@pytest.mark.parametrize("T", [torch.float64, torch.float32], ids=["Float64", "Float32"])
def test_exact_round_trip_every_field_type(mods, tmp_path, T):
    gbg, h5, ck = mods
    C = torch.complex128 if T == torch.float64 else torch.complex64
    rng = np.random.default_rng(1)
    grid = gbg.Grid3D((8, 8, 6), (TWO_PI, 4 * math.pi, TWO_PI), origin=(0.1, 0.2, 0.3), dtype=T)
    fields = {
        "scalar_physical": gbg.ScalarFieldPhysical(_rand((8, 8, 6), T, rng), grid),
        "scalar_spectral": gbg.ScalarFieldSpectral(_rand((5, 8, 6), C, rng), grid),
        "vector_physical": gbg.VectorFieldPhysical(_rand((8, 8, 6, 3), T, rng), grid),
        "vector_spectral": gbg.VectorFieldSpectral(_rand((5, 8, 6, 3), C, rng), grid),
        "tensor_physical": gbg.TensorFieldPhysical(_rand((8, 8, 6, 3, 3), T, rng), grid),
        "tensor_spectral": gbg.TensorFieldSpectral(_rand((5, 8, 6, 3, 3), C, rng), grid),
    }
    p = tmp_path / "fields.h5"
    with h5.File(p, "w") as f:
        for name, fld in fields.items():
            ck.write_field(f, name, fld)
    with h5.File(p) as f:
        for name, fld in fields.items():
            r = ck.read_field(f, name)
            assert type(r) is type(fld) and ck._field_tag(r) == ck._field_tag(fld)
            assert torch.equal(r.data, fld.data) and r.data.dtype == fld.data.dtype
            assert r.tensor_order == fld.tensor_order
            assert r.grid == grid
            assert (r.grid.grid_size, r.grid.domain_size, r.grid.origin, r.grid.grid_spacing) == (
                grid.grid_size, grid.domain_size, grid.origin, grid.grid_spacing)
            assert ck._layout_of(r).fft_dims == ck._layout_of(fld).fft_dims


@pytest.mark.parametrize("T", [torch.float64, torch.float32], ids=["Float64", "Float32"])
def test_permuted_rfft_layout_round_trips(mods, tmp_path, T):
    gbg, h5, ck = mods
    C = torch.complex128 if T == torch.float64 else torch.complex64
    grid = gbg.Grid3D((8, 7, 6), (TWO_PI, 4 * math.pi, TWO_PI), dtype=T)
    layout = gbg.RealFourierLayout((2, 1, 3))
    f0 = gbg.VectorFieldSpectral(_rand((8, 4, 6, 3), C, np.random.default_rng(2)), grid, layout=layout)
    p = tmp_path / "perm.h5"
    with h5.File(p, "w") as f:
        ck.write_field(f, "permuted", f0)
    with h5.File(p) as f:
        r = ck.read_field(f, "permuted")
        assert r.layout.fft_dims == (2, 1, 3) and torch.equal(r.data, f0.data) and r.grid.dtype == T


def test_snapshot_bundle_with_the_consumers_own_data(mods, tmp_path):
    gbg, h5, ck = mods
    rng = np.random.default_rng(4)
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    u = gbg.VectorFieldPhysical(_rand((8, 8, 8, 3), torch.float64, rng), grid)
    w = gbg.VectorFieldPhysical(_rand((8, 8, 8, 3), torch.float64, rng), grid)
    p = tmp_path / "snap.h5"
    with h5.File(p, "w") as f:
        f["note"] = "run-42"
        snap = f.create_group("step_0100")
        ck.write_field(snap, "velocity", u)
        snap["vorticity"] = w  # the sugar
        snap.attrs["time"] = 1.25
        snap.attrs["iteration"] = 100
    with h5.File(p) as f:
        assert torch.equal(ck.read_field(f, "step_0100/velocity").data, u.data)
        assert torch.equal(ck.read_field(f["step_0100"], "vorticity").data, w.data)
        assert f["step_0100"].attrs["time"] == 1.25 and f["step_0100"].attrs["iteration"] == 100
        assert f["note"].read() == "run-42"


def test_field_groups_are_self_describing(mods, tmp_path):
    gbg, h5, ck = mods
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    p = tmp_path / "sd.h5"
    with h5.File(p, "w") as f:
        ck.write_field(f, "u", gbg.ScalarFieldSpectral(_rand((5, 8, 8), torch.complex128, np.random.default_rng(5)),
                                                      grid))
        g = ck.write_field(f, "probe", gbg.ScalarFieldSpectral(torch.zeros(5, 8, 8, dtype=torch.complex128), grid))
        assert {"type", "version", "representation", "tensor_order", "grid_size"} <= set(g.attrs)
    with h5.File(p) as f:
        a = f["u"].attrs
        assert a["type"] == "GBGPeriodicFields.ScalarFieldSpectral" and a["version"] == 1
        assert a["representation"] == "spectral" and a["tensor_order"] == 0
        assert list(a["grid_size"]) == [8, 8, 8] and set(f["u"].keys()) == {"data"}


def test_field_error_paths(mods, tmp_path):
    gbg, h5, ck = mods
    ArgumentError = gbg.ArgumentError
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    mk = lambda: gbg.ScalarFieldPhysical(_rand((8, 8, 8), torch.float64, np.random.default_rng(6)), grid)
    p = tmp_path / "err.h5"
    with h5.File(p, "w") as f:
        f["plain"] = np.array([1.0, 2.0])
        ck.write_field(f, "field", mk())
        f.create_group("tagless")
        ck.write_field(f, "bogus_tag", mk())
        f["bogus_tag"].attrs["type"] = "GBGPeriodicFields.NoSuchField"
        ck.write_field(f, "no_data", mk())
        del f["no_data"]["data"]
        ck.write_field(f, "no_geometry", mk())
        del f["no_geometry"].attrs["grid_size"]
    with h5.File(p) as f:
        for name in ("plain", "absent", "tagless", "bogus_tag", "no_data", "no_geometry"):
            with pytest.raises(ArgumentError):
                ck.read_field(f, name)
        ck.read_field(f, "field")


def test_grid_round_trips_exactly_and_tampering_is_refused(mods, tmp_path):
    gbg, h5, ck = mods
    ArgumentError = gbg.ArgumentError
    sizes, extent = (8, 8, 8), (TWO_PI,) * 3
    canonical = [e / n for e, n in zip(extent, sizes)]
    perturbed = tuple(float(np.nextafter(np.nextafter(c, np.inf), np.inf)) for c in canonical)
    assert list(perturbed) != canonical
    grid = gbg.Grid3D(sizes, extent, grid_spacing=perturbed)
    field = gbg.ScalarFieldPhysical(_rand(sizes, torch.float64, np.random.default_rng(8)), grid)
    p = tmp_path / "exact.h5"
    with h5.File(p, "w") as f:
        ck.write_field(f, "f", field)
    with h5.File(p) as f:
        back = ck.read_field(f, "f")
    assert back.grid.grid_spacing == perturbed and back.grid == grid and torch.equal(back.data, field.data)
    plain = gbg.ScalarFieldPhysical(_rand((4, 4, 4), torch.float64, np.random.default_rng(9)),
                                    gbg.Grid3D((4, 4, 4), (TWO_PI,) * 3))
    for attribute, value in (("version", 99), ("representation", "spectral"), ("eltype", "Float32"),
                             ("tensor_order", 2)):
        q = tmp_path / f"{attribute}.h5"
        with h5.File(q, "w") as f:
            ck.write_field(f, "f", plain)
        with h5.File(q, "r+") as f:
            del f["f"].attrs[attribute]
            f["f"].attrs[attribute] = value
        with h5.File(q) as f:
            with pytest.raises(ArgumentError):
                ck.read_field(f, "f")
    q = tmp_path / "clean.h5"
    with h5.File(q, "w") as f:
        ck.write_field(f, "f", plain)
    with h5.File(q) as f:
        assert torch.equal(ck.read_field(f, "f").data, plain.data)


@pytest.mark.parametrize("T", [torch.float64, torch.float32], ids=["Float64", "Float32"])
def test_read_field_into_an_existing_field(mods, tmp_path, T):
    gbg, h5, ck = mods
    ArgumentError = gbg.ArgumentError
    C = torch.complex128 if T == torch.float64 else torch.complex64
    sizes = (8, 6, 5)
    grid = gbg.Grid3D(sizes, (TWO_PI, 4 * math.pi, TWO_PI), dtype=T)
    layout = gbg.RealFourierLayout((2, 1, 3))
    rng = np.random.default_rng(10)

    def physical(R, data):
        f = gbg.AbstractFieldPhysical(data, grid, R)
        f.layout = layout
        return f

    spectral = lambda R, data: gbg.AbstractFieldSpectral(data, grid, R, layout)
    pshape = lambda R: sizes + (3,) * R
    sshape = lambda R: (8, 4, 5) + (3,) * R
    p = tmp_path / "into.h5"
    with h5.File(p, "w") as f:
        for R in (0, 1, 2):
            ck.write_field(f, f"f1_{R}", physical(R, _rand(pshape(R), T, rng)))
            ck.write_field(f, f"f2_{R}", spectral(R, _rand(sshape(R), C, rng)))
    from gbgperiodicfields_gb300 import zeros_colmajor
    with h5.File(p) as f:
        for R in (0, 1, 2):
            for k, make, shape, dt in ((1, physical, pshape, T), (2, spectral, sshape, C)):
                name = f"f{k}_{R}"
                stored = f[name]["data"].read()
                dest = make(R, zeros_colmajor(shape(R), dt, "cpu"))
                assert ck.read_field_(dest, f, name) is dest
                np.testing.assert_array_equal(dest.data.numpy(), stored)
        other_T = torch.float32 if T == torch.float64 else torch.float64

        def sentinel(fld):
            fld.data.fill_(7)
            return fld

        other_grid = gbg.Grid3D(sizes, (TWO_PI, 4 * math.pi, TWO_PI), dtype=other_T)
        wrong_layout = gbg.AbstractFieldPhysical(zeros_colmajor(pshape(1), T, "cpu"), grid, 1)
        refusals = (sentinel(physical(0, zeros_colmajor(pshape(0), T, "cpu"))),
                    sentinel(spectral(1, zeros_colmajor(sshape(1), C, "cpu"))),
                    sentinel(gbg.AbstractFieldPhysical(zeros_colmajor(pshape(1), other_T, "cpu"), other_grid, 1)),
                    sentinel(wrong_layout),
                    sentinel(physical(1, zeros_colmajor(pshape(1), T, "cpu"))) if False else None)
        box = gbg.Grid3D(sizes, (TWO_PI,) * 3, dtype=T)
        other_box = gbg.AbstractFieldPhysical(zeros_colmajor(pshape(1), T, "cpu"), box, 1)
        other_box.layout = layout
        for dest in [r for r in refusals if r is not None] + [sentinel(other_box)]:
            with pytest.raises(ArgumentError):
                ck.read_field_(dest, f, "f1_1")
            assert bool((dest.data == 7).all())
        CO = torch.complex64 if T == torch.float64 else torch.complex128
        spec_other = gbg.AbstractFieldSpectral(zeros_colmajor(sshape(1), CO, "cpu"), other_grid, 1, layout)
        with pytest.raises(ArgumentError) as e:
            ck.read_field_(spec_other, f, "f2_1")
        msg = str(e.value)
        want_T = "Float64" if T == torch.float64 else "Float32"
        other_name = "Float32" if T == torch.float64 else "Float64"
        assert f"holds a {want_T} field" in msg and f"destination is {other_name}" in msg and "Complex" not in msg


@pytest.mark.parametrize("T", [torch.float64, torch.float32], ids=["Float64", "Float32"])
def test_writes_and_reads_copy_nothing(mods, tmp_path, T):
    """At 24^3 a vector field is 324 KiB in Float64; the verbs' own bookkeeping must stay
    far below that (a field-sized copy would not)."""
    gbg, h5, ck = mods
    big = gbg.Grid3D((24, 24, 24), (TWO_PI,) * 3, dtype=T)
    rng = np.random.default_rng(12)
    field = gbg.VectorFieldPhysical(_rand((24, 24, 24, 3), T, rng), big)
    from gbgperiodicfields_gb300 import zeros_colmajor
    dest = gbg.VectorFieldPhysical(zeros_colmajor((24, 24, 24, 3), T, "cpu"), big)
    nbytes = field.data.numel() * field.data.element_size()
    p = tmp_path / "copy.h5"
    with h5.File(p, "w") as f:
        ck.write_field(f, "warm", field)
        tracemalloc.start()
        ck.write_field(f, "u", field)
        _, peak = tracemalloc.get_traced_memory()
        tracemalloc.stop()
        assert peak < nbytes // 8, peak
    with h5.File(p) as f:
        ck.read_field_(dest, f, "u")
        tracemalloc.start()
        ck.read_field_(dest, f, "u")
        _, peak = tracemalloc.get_traced_memory()
        tracemalloc.stop()
        assert peak < nbytes // 8, peak
        assert torch.equal(dest.data, field.data)


# ------------------------------------------------------------------ points


@pytest.mark.parametrize("T", [torch.float64, torch.float32], ids=["Float64", "Float32"])
def test_exact_round_trip_point_layer(mods, tmp_path, T):
    gbg, h5, ck = mods
    M = 5
    rng = np.random.default_rng(7)
    positions = gbg.PointSet(_rand((M, 3), T, rng) * TWO_PI)
    scalars = gbg.ScalarPointValues(_rand((M,), T, rng))
    vectors = gbg.VectorPointValues(_rand((M, 3), T, rng))
    tensors = gbg.TensorPointValues(_rand((M, 3, 3), T, rng))
    third = gbg.TensorPointValues(_rand((M, 3, 3, 3), T, rng), 3)
    p = tmp_path / "pts.h5"
    with h5.File(p, "w") as f:
        ck.write_points(f, "positions", positions)
        ck.write_points(f, "scalars", scalars)
        ck.write_points(f, "vectors", vectors)
        ck.write_points(f, "tensors", tensors)
        f["third"] = third
    with h5.File(p) as f:
        back = ck.read_points(f, "positions")
        assert isinstance(back, gbg.PointSet) and torch.equal(back.positions, positions.positions)
        assert back.positions.dtype == T and back.npoints == M
        for name, orig, order in (("scalars", scalars, 0), ("vectors", vectors, 1), ("tensors", tensors, 2),
                                  ("third", third, 3)):
            b = ck.read_points(f, name)
            assert isinstance(b, gbg.AbstractPointValues) and b.tensor_order == order
            assert torch.equal(b.data, orig.data) and b.data.dtype == T and b.npoints == M


def test_point_groups_are_self_describing_and_separate(mods, tmp_path):
    gbg, h5, ck = mods
    ArgumentError = gbg.ArgumentError
    rng = np.random.default_rng(11)
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    positions = gbg.PointSet(_rand((4, 3), torch.float64, rng) * TWO_PI)
    p = tmp_path / "sep.h5"
    with h5.File(p, "w") as f:
        ck.write_points(f, "positions", positions)
        ck.write_points(f, "q", gbg.VectorPointValues(_rand((4, 3), torch.float64, rng)))
        assert {"type", "version", "npoints"} <= set(ck.write_points(f, "probe", positions).attrs)
        ck.write_field(f, "u", gbg.VectorFieldPhysical(_rand((8, 8, 8, 3), torch.float64, rng), grid))
    with h5.File(p) as f:
        a = f["positions"].attrs
        assert a["type"] == "GBGPeriodicFields.PointSet" and a["npoints"] == 4
        assert "tensor_order" not in a and "grid_size" not in a
        assert f["q"].attrs["tensor_order"] == 1
        assert ck.read_field(f, "u").tensor_order == 1
        with pytest.raises(ArgumentError):
            ck.read_points(f, "u")
        with pytest.raises(ArgumentError):
            ck.read_field(f, "positions")


def test_point_error_paths(mods, tmp_path):
    gbg, h5, ck = mods
    ArgumentError = gbg.ArgumentError
    pts = lambda: gbg.PointSet(torch.rand(3, 3, dtype=torch.float64))
    p = tmp_path / "perr.h5"
    with h5.File(p, "w") as f:
        f["plain_points"] = np.array([1.0, 2.0])
        ck.write_points(f, "bogus_tag", pts())
        f["bogus_tag"].attrs["type"] = "GBGPeriodicFields.NoSuchPointThing"
        ck.write_points(f, "no_data", pts())
        del f["no_data"]["data"]
        f.create_group("tagless_points")
        ck.write_points(f, "future", pts())
        f["future"].attrs["version"] = 99
    with h5.File(p) as f:
        for name in ("plain_points", "absent", "tagless_points", "bogus_tag", "no_data", "future"):
            with pytest.raises(ArgumentError):
                ck.read_points(f, name)


# ------------------------------------------------------------------ schemes


def test_schemes_round_trip_through_their_parameters(mods, tmp_path):
    gbg, h5, ck = mods
    schemes = (gbg.CatmullRom, gbg.LalescuSpline(2, smoothness=0), gbg.LalescuSpline(8, smoothness=2),
               gbg.LalescuSpline(6, smoothness=4), gbg.LagrangeSpline(2), gbg.LagrangeSpline(8), gbg.DirectDFT())
    p = tmp_path / "schemes.h5"
    with h5.File(p, "w") as f:
        for i, s in enumerate(schemes):
            g = ck.write_scheme(f, f"s{i}", s)
            assert isinstance(g, h5.Group) and "data" not in g
        f["sugar"] = gbg.CatmullRom
    with h5.File(p) as f:
        for i, s in enumerate(schemes):
            back = ck.read_scheme(f, f"s{i}")
            assert type(back) is type(s) and back == s
            if hasattr(s, "coefficients"):
                assert back.stencil_width == s.stencil_width
                np.testing.assert_array_equal(back.coefficients, s.coefficients)  # identical weights
        assert ck.read_scheme(f, "sugar") == gbg.CatmullRom


def test_nufft_refused_and_malformed_scheme_groups_caught(mods, tmp_path):
    gbg, h5, ck = mods
    ArgumentError = gbg.ArgumentError

    class FakeNUFFT(gbg.NUFFT):  # a NUFFT instance without building plans (no device here)
        def __init__(self):
            pass

    p = tmp_path / "serr.h5"
    with h5.File(p, "w") as f:
        with pytest.raises(ArgumentError):
            ck.write_scheme(f, "nufft", FakeNUFFT())
        with pytest.raises(ArgumentError):
            f["nufft_sugar"] = FakeNUFFT()
        ck.write_scheme(f, "impossible", gbg.LalescuSpline(4, smoothness=1))
        f["impossible"].attrs["smoothness"] = 9
        ck.write_scheme(f, "future", gbg.CatmullRom)
        f["future"].attrs["version"] = 99
        ck.write_scheme(f, "alien_eltype", gbg.CatmullRom)
        f["alien_eltype"].attrs["eltype"] = "Float16"
        ck.write_scheme(f, "single_eltype", gbg.CatmullRom)
        f["single_eltype"].attrs["eltype"] = "Float32"
        ck.write_scheme(f, "no_param", gbg.CatmullRom)
        del f["no_param"].attrs["stencil_width"]
        ck.write_scheme(f, "wrong_tag", gbg.CatmullRom)
        f["wrong_tag"].attrs["type"] = "GBGPeriodicFields.NotAScheme"
        f.create_group("bare")
        f["plain_dataset"] = np.array([1.0, 2.0, 3.0])
    with h5.File(p) as f:
        assert "nufft" not in f and "nufft_sugar" not in f
        for name in ("impossible", "future", "alien_eltype", "no_param", "wrong_tag", "bare", "plain_dataset",
                     "absent"):
            with pytest.raises(ArgumentError):
                ck.read_scheme(f, name)
        assert ck.read_scheme(f, "single_eltype") == gbg.CatmullRom
    # schema version 1 stored the half-width `neighbours` (width 2n + 2)
    with h5.File(p, "r+") as f:
        for label, tag, params in (("v1_lalescu", "LalescuSpline", {"neighbours": 3, "smoothness": 2}),
                                   ("v1_lagrange", "LagrangeSpline", {"neighbours": 1})):
            g = f.create_group(label)
            g.attrs["type"] = "GBGPeriodicFields." + tag
            g.attrs["version"] = 1
            g.attrs["eltype"] = "Float64"
            for k, v in params.items():
                g.attrs[k] = v
    with h5.File(p) as f:
        assert ck.read_scheme(f, "v1_lalescu") == gbg.LalescuSpline(8, smoothness=2)
        assert ck.read_scheme(f, "v1_lagrange") == gbg.LagrangeSpline(4)
        assert f["future"].attrs["version"] == 99
    with h5.File(p, "r+") as f:
        g = ck.write_scheme(f, "v2", gbg.LalescuSpline(6, smoothness=1))
        assert g.attrs["version"] == 2 and g.attrs["stencil_width"] == 6 and g.attrs["smoothness"] == 1
        assert "neighbours" not in g.attrs


def test_every_scheme_is_persistable_or_a_recorded_refusal(mods, tmp_path):
    gbg, h5, ck = mods
    from gbgperiodicfields_gb300 import api, nufft
    refused = {"NUFFT"}
    concrete = {c.__name__ for mod in (api, nufft) for c in vars(mod).values()
                if isinstance(c, type) and c.__module__ == mod.__name__
                and (issubclass(c, api._SplineScheme) or c.__name__ in ("NUFFT", "DirectDFT")) and not c.__name__.startswith("_")}
    assert concrete >= {"LalescuSpline", "LagrangeSpline", "DirectDFT", "NUFFT"}
    representative = {"LalescuSpline": gbg.CatmullRom, "LagrangeSpline": gbg.LagrangeSpline(4),
                      "DirectDFT": gbg.DirectDFT()}
    for name in concrete - refused:
        assert name in representative
        p = tmp_path / f"cov_{name}.h5"
        with h5.File(p, "w") as f:
            ck.write_scheme(f, "s", representative[name])
        with h5.File(p) as f:
            assert ck.read_scheme(f, "s") == representative[name]


def test_direct_dft_is_a_record_not_a_transfer(mods):
    gbg, _, _ = mods
    grid = gbg.Grid3D((8, 8, 8), (TWO_PI,) * 3)
    field = gbg.ScalarFieldPhysical(torch.zeros(8, 8, 8, dtype=torch.float64), grid)
    with pytest.raises(gbg.MethodError):
        gbg.interpolate(field, gbg.PointSet(torch.zeros(1, 3, dtype=torch.float64)), gbg.DirectDFT())
