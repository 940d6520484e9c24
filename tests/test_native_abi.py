"""The C-ABI library builds, loads without a GPU and exports every symbol include/ptyg.h declares."""

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from ptylab_gb300 import _build, _native

    if not _native.LIB_PATH.exists():
        _build.build()
    return _native.load_library()


def declared_functions():
    text = (ROOT / "include" / "ptyg.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:PTYG_API\s+)?(?:int|size_t|const char\*)\s+(ptyg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_bound_functions():
    from ptylab_gb300 import _native

    assert declared_functions() == _native.exported_symbols()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version_and_error_string_without_gpu(lib):
    assert lib.ptyg_version() == 1000
    assert isinstance(lib.ptyg_last_error(), bytes)


def test_invalid_geometry_is_rejected_before_touching_a_device(lib):
    import ctypes as C

    from ptylab_gb300 import _native

    g = _native.Geometry(Np=48, No=64, nosm=1, npsm=1, nslice=1, num_frames=1, num_scans=1)
    plan = C.c_void_p()
    st = lib.ptyg_plan_create(C.byref(g), C.byref(plan))
    assert st == _native.PTYG_ERR_UNSUPPORTED
    assert b"Np=48" in lib.ptyg_last_error()
    with pytest.raises(NotImplementedError):
        _native.check(st, "ptyg_plan_create")


def test_status_codes_map_to_reference_exceptions():
    from ptylab_gb300 import _native

    assert _native._EXC[_native.PTYG_ERR_INVALID] is ValueError
    assert _native._EXC[_native.PTYG_ERR_UNSUPPORTED] is NotImplementedError
    assert _native._EXC[_native.PTYG_ERR_DEVICE] is ImportError


_C_TYPES = {"int32_t": "c_int", "float": "c_float", "double": "c_double"}


def declared_structs():
    """{struct name: [(field, ctype-ish)]} from the typedef'd structs of include/ptyg.h."""
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "ptyg.h").read_text(), flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (ptyg_\w+) \{(.*?)\} \1;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"(?:const\s+)?(\w+)\s*(\**)\s*(.+)", decl)
            base, ptr, names = m.groups()
            for n in names.split(","):
                n = n.strip()
                star = ptr or ("*" if n.startswith("*") else "")
                n = n.lstrip("*").strip()
                fields.append((n, "c_void_p" if star else _C_TYPES.get(base, base)))
        out[name] = fields
    return out


@pytest.mark.parametrize(
    "cname,pyname",
    [("ptyg_geometry", "Geometry"), ("ptyg_update_params", "UpdateParams"), ("ptyg_scan_buffers", "ScanBuffers"),
     ("ptyg_multislice", "Multislice"), ("ptyg_projection", "Projection")],
)
def test_ctypes_structs_match_the_header(cname, pyname):
    """Field names, order and types of the ctypes mirrors equal the C structs."""
    import ctypes as C

    from ptylab_gb300 import _native

    want = declared_structs()[cname]
    got = []
    for n, t in getattr(_native, pyname)._fields_:
        kind = {C.c_int32: "c_int", C.c_int: "c_int", C.c_float: "c_float", C.c_double: "c_double"}.get(t, "c_void_p")
        got.append((n, kind))
    assert got == want


def test_new_entry_points_reject_bad_arguments_before_touching_a_device(lib):
    """Argument checks of the wavelength-set propagators, the several-
    wavelength and CTA-size plan fields, the stitcher and the convolution
    path switch run on the host: the errors come back without a GPU."""
    import ctypes as C

    from ptylab_gb300 import _native

    dummy = C.c_void_p(16)
    # nsets must divide the batch; SCALED_ASP takes one table set
    assert lib.ptyg_propagate_sets(3, 0, 64, 4, 3, dummy, dummy, dummy, dummy, None, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_propagate_sets(4, 0, 64, 4, 2, dummy, dummy, dummy, dummy, None, None) == _native.PTYG_ERR_INVALID
    # a propagator of ptyg_propagate is not a set propagator, and the tables are required
    assert lib.ptyg_propagate_sets(0, 0, 64, 4, 1, dummy, dummy, dummy, dummy, None, None) == _native.PTYG_ERR_UNSUPPORTED
    assert lib.ptyg_propagate_sets(5, 0, 64, 4, 1, dummy, dummy, dummy, None, None, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_propagate_sets(6, 0, 48, 4, 1, dummy, dummy, dummy, dummy, None, None) == _native.PTYG_ERR_UNSUPPORTED
    # several wavelengths: not with e3PIE; CTA sizes: multiples of 32 in range
    plan = C.c_void_p()
    g = _native.Geometry(Np=64, No=128, nosm=1, npsm=1, nslice=1, num_frames=4, num_scans=1,
                         engine=_native.ENGINES["e3PIE"], nlambda=2)
    assert lib.ptyg_plan_create(C.byref(g), C.byref(plan)) == _native.PTYG_ERR_UNSUPPORTED
    assert b"wavelengths" in lib.ptyg_last_error()
    for threads in (100, 64, 1024):
        g = _native.Geometry(Np=64, No=128, nosm=1, npsm=1, nslice=1, num_frames=4, num_scans=1,
                             engine=_native.ENGINES["ePIE"], threads=threads)
        assert lib.ptyg_plan_create(C.byref(g), C.byref(plan)) == _native.PTYG_ERR_INVALID
    g = _native.Geometry(Np=64, No=128, nosm=1, npsm=1, nslice=1, num_frames=4, num_scans=1,
                         engine=_native.ENGINES["ePIE"], probe_in_smem=3)
    assert lib.ptyg_plan_create(C.byref(g), C.byref(plan)) == _native.PTYG_ERR_INVALID
    g = _native.Geometry(Np=64, No=128, nosm=1, npsm=1, nslice=1, num_frames=4, num_scans=1,
                         engine=_native.ENGINES["ePIE"], propagator=_native.PROPAGATORS["asp"], asp_table_in_smem=-1)
    assert lib.ptyg_plan_create(C.byref(g), C.byref(plan)) == _native.PTYG_ERR_INVALID
    assert b"asp_table_in_smem" in lib.ptyg_last_error()
    # the stitcher needs its buffers and No >= Np
    assert lib.ptyg_stitch(None, dummy, 1, 32, 64, dummy, dummy, dummy, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_stitch(dummy, dummy, 1, 64, 32, dummy, dummy, dummy, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_nn_conv3_path(1) == 0


def test_calibration_and_reference_entry_points_validate_first(lib):
    """The FPM calibration calls and the interferometric readout refuse bad
    arguments with the documented status before any device work."""
    import ctypes as C

    from ptylab_gb300 import _native

    d = C.c_void_p(16)
    host = (C.c_double * 4)(1.0, 0.5, 0.25, 0.125)
    # frame sizes outside the transforms'; counts and pointers
    assert lib.ptyg_calib_spectra(2, 48, d, d, d, d, d, d, d, None) == _native.PTYG_ERR_UNSUPPORTED
    assert lib.ptyg_calib_spectra(0, 64, d, d, d, d, d, d, d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_spectra(2, 64, d, None, d, d, d, d, d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_normalise(-1, 64, d, d, C.c_float(1.0), None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_normalise(0, 64, d, d, C.c_float(1.0), None) == _native.PTYG_OK
    assert lib.ptyg_calib_gaussian(2, 64, 64, host, d, d, None) == _native.PTYG_ERR_UNSUPPORTED
    assert lib.ptyg_calib_gaussian(2, 64, 3, None, d, d, None) == _native.PTYG_ERR_UNSUPPORTED
    assert lib.ptyg_calib_gaussian(0, 64, 3, host, d, d, None) == _native.PTYG_OK
    # circle search: radii and angles at most 64, a search grid of at most 255
    assert lib.ptyg_calib_arcs(64, d, 1, d, d, d, 0, host, 4, host, host, 3, d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_arcs(64, d, 1, d, d, d, 65, host, 4, host, host, 3, d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_arcs(64, d, 1, d, d, d, 4, host, 65, host, host, 3, d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_arcs(64, d, 1, d, d, d, 4, host, 4, host, host, 256, d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_arcs(64, d, 0, d, d, d, 4, host, 4, host, host, 3, d, None) == _native.PTYG_OK
    assert lib.ptyg_calib_arcs(64, d, 1, d, d, d, 4, host, 4, host, None, 3, d, None) == _native.PTYG_ERR_INVALID
    # candidate RMSE
    assert lib.ptyg_calib_rms(96, d, d, 2, d, d, C.c_double(5.0), d, None) == _native.PTYG_ERR_UNSUPPORTED
    assert lib.ptyg_calib_rms(64, d, d, -1, d, d, C.c_double(5.0), d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_rms(64, d, d, 2, d, d, C.c_double(-1.0), d, None) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_calib_rms(64, d, d, 0, d, d, C.c_double(5.0), d, None) == _native.PTYG_OK
    # the interferometric field readout needs a plan
    assert lib.ptyg_plan_get_reference(None, 0, d, None) == _native.PTYG_ERR_INVALID
