"""HDF5 snapshot files (the reference solver's Print_Out format, cuPentCahnADI.cu:103-140) and
checkpoint / resume of Cahn-Hilliard grids through them.

CPU tests: the library's reader and the test-side parser (tests/h5_format.py) both read a file that
the HDF5 library itself wrote (scipy's MATLAB 7.3 test file, which is HDF5 behind a 512-byte user
block) and give the values that scipy reads from the same matrix saved in MATLAB's older format;
then the library's writer is checked structurally by that parser and by round trips.
GPU tests: a grid saved and resumed continues bit for bit like one that never stopped."""
import math
import struct
from pathlib import Path

import numpy as np
import pytest

from tests.h5_format import H5File


def _scipy_data():
    scipy = pytest.importorskip("scipy")
    import scipy.io
    d = Path(scipy.__file__).parent / "io" / "matlab" / "tests" / "data"
    h5, twin = d / "testhdf5_7.4_GLNX86.mat", d / "testdouble_7.1_GLNX86.mat"
    if not h5.exists() or not twin.exists():
        pytest.skip("scipy's MATLAB test files are not installed")
    return h5, scipy.io.loadmat(str(twin))["testdouble"]


def test_reader_reads_a_file_written_by_the_hdf5_library(built):
    h5, expect = _scipy_data()
    got = built.h5_read(h5, "testdouble")
    # MATLAB stores the 1 x 9 row column-major: HDF5 dims (9, 1)
    assert got.shape == (9, 1)
    assert np.array_equal(got.ravel(), expect.ravel())


def test_test_parser_reads_a_file_written_by_the_hdf5_library():
    h5, expect = _scipy_data()
    f = H5File(h5.read_bytes())
    assert f.sb == 512 and f.base == 512
    # the end-of-file address counts the user block; every other address is relative to the base
    assert f.eof == len(h5.read_bytes())
    assert np.array_equal(f.read("testdouble").ravel(), expect.ravel())
    # the conventions the writer follows, as the HDF5 library wrote them
    ds = f.datasets["testdouble"]
    assert ds["fill"][:4] == bytes([1, 2, 2, 1])
    assert f.heap[f.heap_free:f.heap_free + 8] == struct.pack("<Q", 1)   # free list ends at offset 1
    assert f.btree_keys[0] == 0 and f.name_at(0) == ""


def _write(built, path, datasets):
    built.h5_write(path, datasets)
    return H5File(Path(path).read_bytes())


def test_writer_layout_follows_the_format(built, tmp_path):
    rng = np.random.default_rng(7)
    c = rng.uniform(-0.1, 0.1, (64, 64))
    f = _write(built, tmp_path / "s.nc", {"c": c, "c_old": c * 0.5, "t": np.array([[0.25]])})
    assert f.eof == (tmp_path / "s.nc").stat().st_size
    assert (f.leaf_k, f.internal_k, f.base) == (4, 16, 0)
    assert f.root_entry["cache"] == 1 and f.root_entry["scratch"] == (f.btree_addr, f.heap_addr)
    assert f.heap_names == ["c", "c_old", "t"]
    h5lib_float64 = bytes.fromhex("11203f000800000000004000340b0034ff030000")
    for name, ds in f.datasets.items():
        assert ds["dtype"] == h5lib_float64, name
        assert ds["nbytes"] == 8 * int(np.prod(ds["shape"]))
        assert ds["addr"] % 8 == 0 and ds["addr"] + ds["nbytes"] <= f.eof
    assert f.datasets["c"]["shape"] == (64, 64)
    assert np.array_equal(f.read("c"), c)
    assert np.array_equal(f.read("t"), [[0.25]])


@pytest.mark.parametrize("count", [1, 3, 8])
def test_writer_round_trip_bit_exact(built, tmp_path, count):
    rng = np.random.default_rng(count)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -1.7976931348623157e308, 1.0 / 3.0])
    data = {}
    for k in range(count):
        a = rng.standard_normal((3 + k, 1 + 2 * k))
        a.ravel()[: min(a.size, specials.size)] = specials[: min(a.size, specials.size)]
        data[f"d{7 - k}_{k}"] = a
    p = tmp_path / "r.h5"
    f = _write(built, p, data)
    assert sorted(f.datasets) == sorted(data)
    for name, a in data.items():
        got = built.h5_read(p, name)
        assert got.shape == a.shape
        assert got.tobytes() == a.tobytes(), name          # bit for bit, NaN payloads and -0.0 included
        assert f.read(name).tobytes() == a.tobytes()


def test_rank_0_and_1_datasets(built, tmp_path):
    p = tmp_path / "v.h5"
    built.h5_write(p, {"scalar": 2.5, "vec": np.arange(5.0)})
    assert built.h5_read(p, "scalar").shape == (1, 1)
    assert np.array_equal(built.h5_read(p, "vec").ravel(), np.arange(5.0))


def test_user_block_is_skipped(built, tmp_path):
    """A user block shifts the superblock to 512 and every address by the base address."""
    a = np.arange(12.0).reshape(3, 4)
    p = tmp_path / "plain.h5"
    built.h5_write(p, {"c": a})
    blob = bytearray(p.read_bytes())
    struct.pack_into("<Q", blob, 24, 512)          # base address = the superblock's new position
    struct.pack_into("<Q", blob, 40, len(blob) + 512)   # end-of-file address, user block included
    q = tmp_path / "ub.h5"
    q.write_bytes(bytes(512) + bytes(blob))
    assert np.array_equal(built.h5_read(q, "c"), a)
    assert np.array_equal(H5File(q.read_bytes()).read("c"), a)


def test_errors_are_reported_not_fatal(built, tmp_path):
    p = tmp_path / "e.h5"
    built.h5_write(p, {"c": np.zeros((2, 2))})
    with pytest.raises(built.CustenError, match="no dataset named missing"):
        built.h5_read(p, "missing")
    (tmp_path / "not.h5").write_bytes(b"plain text, not HDF5" * 10)
    with pytest.raises(built.CustenError, match="not an HDF5 file"):
        built.h5_read(tmp_path / "not.h5", "c")
    (tmp_path / "cut.h5").write_bytes(p.read_bytes()[:300])
    with pytest.raises(built.CustenError):
        built.h5_read(tmp_path / "cut.h5", "c")
    with pytest.raises(built.CustenError, match="cannot open"):
        built.h5_read(tmp_path / "absent.h5", "c")
    with pytest.raises(built.CustenError):
        built.h5_write(p, {f"d{k}": np.zeros(1) for k in range(9)})
    with pytest.raises(built.CustenError):
        built.h5_write(p, {"a/b": np.zeros(1)})


def test_snapshot_name_matches_the_reference():
    import custen_gb300 as cs
    assert cs.snapshot_name(0.1) == "cahn_hilliard_0.1000000000.nc"
    assert cs.snapshot_name(12.5) == "cahn_hilliard_12.5000000000.nc"


# ---------------------------------------------------------------- checkpoint / resume on the GPU

def _c0(n, seed):
    return np.random.default_rng(seed).uniform(-0.1, 0.1, (n, n))


@pytest.mark.gpu
def test_resume_is_bit_identical(gpu, tmp_path):
    sizes = [64, 96]
    straight = gpu.CahnHilliardBatch(sizes)
    for k, n in enumerate(sizes):
        straight.set_state(k, _c0(n, 10 + k))
    straight.step(7)
    expect = [straight.state(k) for k in range(len(sizes))]
    straight.close()

    first = gpu.CahnHilliardBatch(sizes)
    for k, n in enumerate(sizes):
        first.set_state(k, _c0(n, 10 + k))
    first.step(3)
    for k in range(len(sizes)):
        first.save(k, tmp_path / f"g{k}.nc", time=3 * 0.1 * 2 * math.pi / sizes[k])
    first.close()

    resumed = gpu.CahnHilliardBatch(sizes)
    for k in range(len(sizes)):
        t = resumed.load(k, tmp_path / f"g{k}.nc")
        assert t == 3 * 0.1 * 2 * math.pi / sizes[k]
    resumed.step(4)
    for k in range(len(sizes)):
        cur, old = resumed.state(k)
        assert np.array_equal(cur, expect[k][0]) and np.array_equal(old, expect[k][1])
    resumed.close()


@pytest.mark.gpu
def test_resume_from_a_reference_style_snapshot(gpu, tmp_path):
    """A file holding only "c" (what the reference writes) starts both time levels from it."""
    n = 64
    c = _c0(n, 3)
    p = tmp_path / gpu.snapshot_name(0.0)
    gpu.h5_write(p, {"c": c})
    a = gpu.CahnHilliardBatch([n])
    assert math.isnan(a.load(0, p))
    b = gpu.CahnHilliardBatch([n])
    b.set_state(0, c)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.state(0)[0], b.state(0)[0])
    with pytest.raises(gpu.CustenError, match="snapshot grid is 64 x 64"):
        gpu.CahnHilliardBatch([96]).load(0, p)
    a.close()
    b.close()
