"""HDF5 data and result files (``ptylab_gb300.io``): the reader pinned to a
file libhdf5 wrote and to the published lookup3 vectors, the writer checked
against libhdf5's on-disk conventions, and the measurement / result file
semantics pinned to goldens the reference's own ``ExperimentalData`` and
``saveResults`` produced (tests/golden/make_hdf5_golden.py)."""

from __future__ import annotations

import struct
import types
from pathlib import Path

import numpy as np
import pytest

from ptylab_gb300 import ExperimentalData
from ptylab_gb300.io import hdf5, readHdf5
from ptylab_gb300.Reconstruction import Reconstruction

GOLDEN_DIR = Path(__file__).parent / "golden"
INPUTS = GOLDEN_DIR / "hdf5"
MODES = {"cpm_simulation": "CPM", "cpm_encoder_transposed": "CPM", "fpm_leds": "FPM", "cpm_gzip": "CPM",
         "cpm_missing_zo": "CPM"}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN_DIR / "hdf5_golden.npz")


# ---------------------------------------------------------------- format


def test_lookup3_published_vectors():
    # the self-test vectors of Bob Jenkins' lookup3.c
    assert hdf5.lookup3(b"") == 0xDEADBEEF
    assert hdf5.lookup3(b"Four score and seven years ago") == 0x17770551
    assert hdf5.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


def _libhdf5_mat_file():
    try:
        import scipy.io.matlab as m
    except ImportError:
        return None
    p = Path(m.__file__).parent / "tests" / "data" / "testhdf5_7.4_GLNX86.mat"
    return p if p.exists() else None


def test_reads_a_file_libhdf5_wrote():
    """MATLAB 7.3 writes through libhdf5: a 512-byte user block, superblock
    version 0, a symbol-table root group, a contiguous float64 dataset with
    an attribute.  The file ships with SciPy's test data."""
    p = _libhdf5_mat_file()
    if p is None:
        pytest.skip("SciPy's MATLAB 7.3 test file is not installed")
    assert hdf5.is_hdf5(p)
    with hdf5.File(p) as f:
        assert f.keys() == ["testdouble"]
        d = f["testdouble"]
        assert d.shape == (9, 1) and d.dtype == np.float64
        np.testing.assert_array_equal(np.array(d).ravel(), np.arange(9) * np.pi / 4)
        assert d.attrs == {"MATLAB_class": b"double"}


def _parse_v1_header(buf, addr):
    version, _, nmsgs, refcount, size = struct.unpack_from("<BBHII", buf, addr)
    assert version == 1 and refcount == 1
    pos, msgs = addr + 16, []
    while pos < addr + 16 + size:
        mtype, msize, flags = struct.unpack_from("<HHB", buf, pos)
        assert msize % 8 == 0, "v1 object header messages are 8-byte aligned"
        msgs.append((mtype, buf[pos + 8:pos + 8 + msize]))
        pos += 8 + msize
    assert pos == addr + 16 + size and len(msgs) == nmsgs
    return msgs


def test_writer_follows_libhdf5_conventions(tmp_path):
    """The structures libhdf5 validates when it opens a file, checked byte by
    byte on a written file (the same layout as the MATLAB/libhdf5 file)."""
    p = tmp_path / "w.h5"
    names = [f"d{i:02d}" for i in range(11)]  # two symbol-table nodes
    with hdf5.File(p, "w") as f:
        for i, n in enumerate(names):
            f.create_dataset(n, data=np.full((i + 1, 3), i, dtype=np.float32))
    buf = p.read_bytes()
    assert buf[:8] == hdf5.SIGNATURE
    assert buf[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    leaf_k, internal_k = struct.unpack_from("<HH", buf, 16)
    assert (leaf_k, internal_k) == (4, 16)
    base, freespace, eof, driver = struct.unpack_from("<4Q", buf, 24)
    assert base == 0 and freespace == hdf5.UNDEF and driver == hdf5.UNDEF and eof == len(buf)
    _, root, cache, _, btree, heap = struct.unpack_from("<QQIIQQ", buf, 56)
    assert cache == 1
    # local heap: "" at 0, names 8-aligned, a free block ending the list with 1
    assert buf[heap:heap + 4] == b"HEAP"
    dsize, free, daddr = struct.unpack_from("<QQQ", buf, heap + 8)
    assert buf[daddr:daddr + 8] == bytes(8)
    nxt, fsize = struct.unpack_from("<QQ", buf, daddr + free)
    assert nxt == 1 and free % 8 == 0 and free + fsize == dsize and fsize >= 16
    # group B-tree node, keys = heap offsets of the last name in each child
    assert buf[btree:btree + 6] == b"TREE\x00\x00"
    entries = struct.unpack_from("<H", buf, btree + 6)[0]
    assert entries == 2
    heapnames = buf[daddr:daddr + dsize]
    keys = struct.unpack_from(f"<{2 * entries + 1}Q", buf, btree + 24)[0::2]
    children = struct.unpack_from(f"<{2 * entries + 1}Q", buf, btree + 24)[1::2]
    keynames = [heapnames[k:heapnames.index(b"\0", k)].decode() for k in keys]
    assert keynames == ["", "d07", "d10"]
    seen = []
    for c in children:
        assert buf[c:c + 6] == b"SNOD\x01\x00"
        n = struct.unpack_from("<H", buf, c + 6)[0]
        for j in range(n):
            noff, oh = struct.unpack_from("<QQ", buf, c + 8 + 40 * j)
            seen.append(heapnames[noff:heapnames.index(b"\0", noff)].decode())
            msgs = _parse_v1_header(buf, oh)
            assert [m[0] for m in msgs] == [hdf5.MSG_DATASPACE, hdf5.MSG_DATATYPE, hdf5.MSG_LAYOUT]
            layout = msgs[2][1]
            version, cls, addr, size = struct.unpack_from("<BBQQ", layout)
            assert (version, cls) == (3, 1) and addr + size <= eof
    assert seen == sorted(names)
    msgs = _parse_v1_header(buf, root)
    assert msgs[0][0] == hdf5.MSG_SYMBOL_TABLE and struct.unpack_from("<QQ", msgs[0][1]) == (btree, heap)


def test_datatype_encodings_match_libhdf5():
    """float64 as in the libhdf5 file; h5py's complex compound and boolean
    enum."""
    assert hdf5._encode_datatype(np.dtype("<f8")).hex() == "11203f000800000000004000340b0034ff030000"
    assert hdf5._encode_datatype(np.dtype("<f4")).hex() == "11201f000400000000002000170800177f000000"
    c = hdf5._encode_datatype(np.dtype("<c8"))
    assert c[:8] == bytes([0x16, 2, 0, 0, 8, 0, 0, 0]) and len(c) == 8 + 2 * (8 + 32 + 20)
    assert hdf5._decode_datatype(hdf5._Cursor(c)) == np.dtype({"names": ["r", "i"], "formats": ["<f4", "<f4"],
                                                               "offsets": [0, 4], "itemsize": 8})
    assert hdf5._decode_datatype(hdf5._Cursor(hdf5._encode_datatype(np.dtype(bool)))) == np.dtype(bool)


ROUND_TRIP = {
    "f2": np.linspace(-3, 3, 7, dtype=np.float16),
    "f4": np.random.default_rng(0).standard_normal((3, 4, 5)).astype(np.float32),
    "f8_big_endian": np.arange(6, dtype=">f8").reshape(2, 3),
    "i1": np.arange(-5, 5, dtype=np.int8),
    "u2": np.arange(9, dtype=np.uint16).reshape(3, 3),
    "i8": np.array([-(2**62), 2**62]),
    "c8": (np.arange(6) + 1j * np.arange(6)[::-1]).astype(np.complex64).reshape(2, 3),
    "c16": np.array([1e300 - 1e-300j]),
    "bool": np.array([[True, False], [False, True]]),
    "bytes": np.array([b"probe", b"obj"]),
    "scalar_f4": np.float32(0.25),
    "scalar_i8": np.int64(-3),
    "empty": np.zeros((0, 4), np.float32),
    "a long name with spaces": np.ones(3),
}


def test_round_trip_types_and_shapes(tmp_path):
    p = tmp_path / "rt.h5"
    with hdf5.File(p, "w") as f:
        for k, v in ROUND_TRIP.items():
            f.create_dataset(k, data=v)
    with hdf5.File(p) as f:
        assert f.keys() == sorted(ROUND_TRIP)
        for k, v in ROUND_TRIP.items():
            got = f[k][()]
            want = np.asarray(v)
            assert got.shape == want.shape, k
            assert got.dtype == want.dtype.newbyteorder("="), k
            np.testing.assert_array_equal(got, want, err_msg=k)


@pytest.mark.parametrize("opts", [
    dict(chunks=(4, 5, 3)),
    dict(chunks=(1, 16, 16), compression="gzip"),
    dict(chunks=True, compression="gzip", compression_opts=9, shuffle=True),
    dict(chunks=(2, 2, 2)),  # thousands of chunks: a three-level index
])
def test_round_trip_chunked(tmp_path, opts):
    rng = np.random.default_rng(5)
    data = rng.integers(0, 5000, (37, 16, 23)).astype(np.float32)
    p = tmp_path / "c.h5"
    with hdf5.File(p, "w") as f:
        f.create_dataset("ptychogram", data=data, **opts)
        f.create_dataset("cplx", data=(data[:3] + 1j).astype(np.complex64), **opts)
    with hdf5.File(p) as f:
        np.testing.assert_array_equal(f["ptychogram"][()], data)
        np.testing.assert_array_equal(f["cplx"][()], (data[:3] + 1j).astype(np.complex64))


def test_many_datasets_and_limits(tmp_path):
    p = tmp_path / "many.h5"
    with hdf5.File(p, "w") as f:
        for i in range(256):
            f[f"x{i}"] = np.array([i])
    with hdf5.File(p) as f:
        assert len(f) == 256 and int(f["x255"][()][0]) == 255
    with pytest.raises(NotImplementedError):
        with hdf5.File(tmp_path / "too_many.h5", "w") as f:
            for i in range(257):
                f[f"x{i}"] = np.array([i])


def test_errors(tmp_path):
    bad = tmp_path / "not.h5"
    bad.write_bytes(b"\0" * 4096)
    assert not hdf5.is_hdf5(bad)
    with pytest.raises(hdf5.HDF5FormatError):
        hdf5.File(bad)
    p = tmp_path / "ok.h5"
    with hdf5.File(p, "w") as f:
        f["a"] = np.ones(2)
        with pytest.raises(ValueError):
            f["a"] = np.ones(2)
        with pytest.raises(ValueError):
            f.create_dataset("g/a", data=np.ones(2))
        with pytest.raises(NotImplementedError):
            f.create_dataset("o", data=np.array([object()]))
        with pytest.raises(NotImplementedError):
            f.create_dataset("lzf", data=np.ones(4), compression="lzf")
    with hdf5.File(p) as f:
        with pytest.raises(KeyError):
            f["b"]
        assert "a" in f and "b" not in f
    # a file abandoned by an exception is not written
    q = tmp_path / "abandoned.h5"
    with pytest.raises(RuntimeError):
        with hdf5.File(q, "w") as f:
            f["a"] = np.ones(2)
            raise RuntimeError
    assert not q.exists()
    with pytest.raises(ValueError):
        hdf5.File(p, "a")


def test_truncated_file_is_rejected(tmp_path):
    p = tmp_path / "t.h5"
    with hdf5.File(p, "w") as f:
        f["a"] = np.arange(1000.0)
    buf = p.read_bytes()
    (tmp_path / "cut.h5").write_bytes(buf[: len(buf) - 100])
    with hdf5.File(tmp_path / "cut.h5") as f:
        with pytest.raises(hdf5.HDF5FormatError):
            f["a"][()]


# ---------------------------------------------------------------- PtyLab semantics


def test_scalify_and_checks(tmp_path):
    assert readHdf5.scalify(np.array([[3.5]])) == 3.5 and isinstance(readHdf5.scalify(np.array([2])), int)
    assert readHdf5.scalify(np.ones((2, 1))).shape == (2,)
    with pytest.raises(FileNotFoundError):
        readHdf5.loadInputData(tmp_path / "none.hdf5", [], [])
    other = tmp_path / "x.txt"
    other.write_bytes(b"")
    with pytest.raises(NotImplementedError):
        readHdf5.loadInputData(other, [], [])
    with pytest.raises(KeyError):
        readHdf5.checkDataFields(INPUTS / "cpm_missing_zo.hdf5", ["ptychogram", "zo"])
    assert readHdf5.getOrientation(INPUTS / "cpm_missing_zo.hdf5") is None
    assert readHdf5.getOrientation(INPUTS / "cpm_encoder_transposed.hdf5") == 3


@pytest.mark.parametrize("tag", sorted(MODES))
def test_measurement_files_match_reference(golden, tag):
    """ExperimentalData(file) against the reference's ExperimentalData on the
    same file: every field bit-identical, the same fields None, the same
    error for a file missing a required field."""
    path = INPUTS / f"{tag}.hdf5"
    if f"{tag}/error" in golden.files:
        errors = {"KeyError": KeyError, "FileNotFoundError": FileNotFoundError}
        with pytest.raises(errors[str(golden[f"{tag}/error"])]):
            ExperimentalData(str(path), operationMode=MODES[tag])
        return
    ed = ExperimentalData(str(path), operationMode=MODES[tag])
    none = {str(x) for x in golden[f"{tag}/none"]}
    checked = 0
    for key in golden.files:
        if not key.startswith(tag + "/") or key in (f"{tag}/none",):
            continue
        field = key.split("/", 1)[1]
        want = golden[key]
        got = np.asarray(getattr(ed, field))
        assert got.shape == want.shape, field
        assert got.dtype == want.dtype, field
        np.testing.assert_array_equal(got, want, err_msg=field)
        checked += 1
    for field in none:
        assert getattr(ed, field, None) is None, field
    assert checked >= 10


def test_set_orientation_all_cases():
    frames = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)
    T = lambda a: np.transpose(a, (0, 2, 1))
    want = {0: frames, 1: frames[..., ::-1], 2: frames[:, ::-1], 3: frames[:, ::-1, ::-1],
            4: T(frames), 5: T(frames)[..., ::-1], 6: T(frames)[:, ::-1], 7: T(frames)[:, ::-1, ::-1]}
    for o, w in want.items():
        ed = ExperimentalData("test:nodata")
        ed.ptychogram = frames.copy()
        ed.setOrientation(o)
        np.testing.assert_array_equal(ed.ptychogram, w)
        assert ed.ptychogram.flags.c_contiguous
    ed = ExperimentalData("test:nodata")
    with pytest.raises(ValueError):
        ed.setOrientation(8)
    with pytest.raises(TypeError):
        ed.setOrientation(1.0)


def _result_namespace(golden_attrs):
    ns = types.SimpleNamespace(**golden_attrs)
    ns.data = types.SimpleNamespace(operationMode="CPM")
    ns.logger = __import__("logging").getLogger("test")
    return ns


def test_save_results_match_reference(golden, tmp_path):
    """saveResults writes the reference's dataset names, types and values."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_hdf5_golden", GOLDEN_DIR / "make_hdf5_golden.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    ns = _result_namespace(gen.result_inputs())
    p = tmp_path / "res.hdf5"
    Reconstruction.saveResults(ns, str(p), type="all")
    with hdf5.File(p) as f:
        assert f.keys() == [str(x) for x in golden["result/names"]]
        for k in f.keys():
            got, want = f[k][()], golden[f"result/{k}"]
            assert got.dtype == want.dtype and got.shape == want.shape, k
            np.testing.assert_array_equal(got, want, err_msg=k)
    with pytest.raises(NotImplementedError):
        Reconstruction.saveResults(ns, str(p), type="everything")


def test_results_load_back(tmp_path):
    """saveResults -> load / loadResults / load_object / load_probe."""
    ed = ExperimentalData(str(INPUTS / "cpm_simulation.hdf5"))
    from ptylab_gb300 import Params

    rec = Reconstruction(ed, Params())
    rec.npsm = 2
    rec.initializeObjectProbe()
    rng = np.random.default_rng(3)
    rec.probe = (rec.probe * rng.random(rec.probe.shape)).astype(np.complex64)
    rec.object = (rec.object * (1 + 1j * rng.random(rec.object.shape))).astype(np.complex64)
    rec.error = [2.0, 1.0]
    p = tmp_path / "recon.hdf5"
    rec.saveResults(str(p))
    probe, obj = rec.probe.copy(), rec.object.copy()
    np.testing.assert_array_equal(Reconstruction.loadResults(str(p), "probe"), probe)
    rec.object = None
    rec.load_object(str(p))
    np.testing.assert_array_equal(rec.object, obj)
    rec.probe = None
    rec.load_probe(str(p))
    np.testing.assert_array_equal(rec.probe, probe)
    rec.npsm = 3
    rec.shape_P = (1, 1, 3, 1, rec.Np, rec.Np)
    with pytest.raises(RuntimeError):
        rec.load_probe(str(p))
    rec.load(str(p))
    np.testing.assert_array_equal(rec.error, np.float32([2.0, 1.0]))
    # a reconstruction started from the saved one
    rec2 = Reconstruction(ed, Params())
    rec2.npsm = 2
    rec2.initialProbe = rec2.initialObject = "recon"
    rec2.initialProbe_filename = str(p)
    rec2.initializeObjectProbe()
    np.testing.assert_array_equal(rec2.probe, probe)
    np.testing.assert_array_equal(rec2.object, obj)
    for name in ("probe", "object"):
        q = tmp_path / f"{name}.hdf5"
        rec.saveResults(str(q), type=name, squeeze=True)
        with hdf5.File(q) as f:
            assert f[name].shape == np.squeeze(getattr(rec, name)).shape


def test_easy_initialize_from_files():
    """PtyLab's easyInitialize (PtyLab/__init__.py:11-58) on measurement files."""
    import ptylab_gb300 as P

    d, rec, params, monitor, engine = P.easyInitialize(str(INPUTS / "cpm_simulation.hdf5"), engine=P.Engines.mPIE)
    assert type(engine).__name__ == "mPIE" and rec.probe.shape[-1] == d.ptychogram.shape[-1]
    d, rec, params, monitor, engine, calib = P.easyInitialize(str(INPUTS / "fpm_leds.hdf5"), operationMode="FPM")
    assert type(engine).__name__ == "ePIE" and type(calib).__name__ == "IlluminationCalibration"
    assert params.positionOrder == "NA" and params.probeBoundary
    with pytest.raises(NotImplementedError):
        P.easyInitialize(str(INPUTS / "cpm_simulation.hdf5"), operationMode="XYZ")


@pytest.mark.parametrize("step", ["reduce", "crop", "crop_odd", "bin"])
def test_data_preparation_matches_reference(golden, step):
    """reduce_positions / cropCenter / binData on a loaded file, against the
    reference's ExperimentalData on the same file (ExperimentalData.py:151-190)."""
    ed = ExperimentalData(str(INPUTS / "cpm_simulation.hdf5"))
    {"reduce": lambda: ed.reduce_positions(1, 5), "crop": lambda: ed.cropCenter(10),
     "crop_odd": lambda: ed.cropCenter(7), "bin": lambda: ed.binData(2)}[step]()
    for key in ("ptychogram", "encoder"):
        want = golden[f"prep_{step}/{key}"]
        got = np.asarray(getattr(ed, key))
        assert got.dtype == want.dtype and got.shape == want.shape
        np.testing.assert_array_equal(got, want)
    with pytest.raises(TypeError):
        ed.cropCenter(4.0)


def test_io_benchmark_runs(capsys, tmp_path):
    """python -m ptylab_gb300.io.benchmark at a tiny size: both layouts, read
    back equal to what was written."""
    import json

    from ptylab_gb300.io import benchmark

    benchmark.main(["--frames", "6", "--Nd", "32", "--reps", "1", "--dir", str(tmp_path)])
    lines = [json.loads(x) for x in capsys.readouterr().out.strip().splitlines()]
    assert [x["layout"] for x in lines] == ["contiguous", "gzip"]
    assert all(x["read"] > 0 and x["write"] > 0 for x in lines) and "fromfile" in lines[0]


def test_reconstruction_geometry_properties():
    """Detector / object coordinates, detection NA and depth of field
    (Reconstruction.py:583-598, 652-672, 712-724)."""
    from ptylab_gb300 import Params

    ed = ExperimentalData(str(INPUTS / "cpm_simulation.hdf5"))
    rec = Reconstruction(ed, Params())
    n, d = rec.Nd, rec.dxd
    np.testing.assert_array_equal(rec.xd, np.linspace(-n / 2, n / 2, n) * d)
    assert rec.Xd.shape == (n, n) and np.array_equal(rec.Xd[0], rec.xd) and np.array_equal(rec.Yd[:, 0], rec.xd)
    np.testing.assert_array_equal(rec.xo, np.linspace(-rec.No / 2, rec.No / 2, rec.No) * rec.dxo)
    assert rec.Xo.shape == (rec.No, rec.No)
    assert rec.NAd == rec.Ld / (2 * rec.zo) and rec.DoF == rec.wavelength / rec.NAd**2


def test_matlab_73_file_loads_through_readHdf5(tmp_path):
    """A MATLAB 7.3 .mat file is HDF5 (written by libhdf5 with a 512-byte
    user block); loadInputData reads it as PtyLab's PyTables path does."""
    import shutil

    p = _libhdf5_mat_file()
    if p is None:
        pytest.skip("SciPy's MATLAB 7.3 test file is not installed")
    mat = tmp_path / "measurement.mat"
    shutil.copy(p, mat)
    readHdf5.checkDataFields(mat, ["testdouble"])
    got = readHdf5.loadInputData(mat, ["testdouble"], ["absent"])
    np.testing.assert_array_equal(got["testdouble"], np.arange(9) * np.pi / 4)
    assert got["absent"] is None
    assert readHdf5.getOrientation(mat) is None
