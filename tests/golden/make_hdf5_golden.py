"""Golden fixtures for PtyLab's HDF5 data and result files.

Test infrastructure only.  Writes small measurement files (the layouts of
PtyLab/io/generateSimulationData.py:124-135 and of hand-made CPM/FPM files:
scalars as (1,) arrays, an encoder stored transposed, orientations 3, 5 and
6, a gzip-compressed ptychogram, a file missing a required field) with
``ptylab_gb300.io.hdf5``, then loads each through the REFERENCE's own
``ExperimentalData`` (PtyLab/ExperimentalData/ExperimentalData.py:86-149,
PtyLab/io/readHdf5.py) and writes a result file through the reference's
``Reconstruction.saveResults`` (PtyLab/Reconstruction/Reconstruction.py:510-576).
The reference's PyTables / h5py calls go to thin shims over this package's
HDF5 reader and writer (neither library is installed here), so what is pinned
is the reference's host logic on top of the file access: which fields are
read, scalars, the encoder transposition and centring, the orientation
flips, the result file's dataset names, types and values.

Run from the repository root with the reference checked out:

    python tests/golden/make_hdf5_golden.py --reference <path of a PtyLab.py checkout>

Outputs: ``tests/golden/hdf5/*.hdf5`` (inputs) and
``tests/golden/hdf5_golden.npz``.
"""

from __future__ import annotations

import argparse
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

from ptylab_gb300.io import hdf5  # noqa: E402

OUT_DIR = HERE / "hdf5"
GOLDEN = HERE / "hdf5_golden.npz"

MEASUREMENT_FIELDS = (
    "ptychogram", "encoder", "wavelength", "dxd", "zo", "zled", "magnification", "NA",
    "entrancePupilDiameter", "spectralDensity", "theta", "emptyBeam",
    "Nd", "xd", "Ld", "numFrames", "energyAtPos", "maxProbePower",
)


def _frames(rng, n, N):
    # distinct, asymmetric frames so every flip and transpose is visible
    base = np.arange(N * N, dtype=np.float32).reshape(N, N)
    return (base[None] * (1 + np.arange(n, dtype=np.float32))[:, None, None]
            + rng.random((n, N, N), dtype=np.float32))


def write_inputs():
    rng = np.random.default_rng(2024)
    OUT_DIR.mkdir(exist_ok=True)
    files = {}

    # generateSimulationData.py:124-135 layout
    p = OUT_DIR / "cpm_simulation.hdf5"
    with hdf5.File(p, "w") as hf:
        hf.create_dataset("ptychogram", data=_frames(rng, 6, 16), dtype="f")
        hf.create_dataset("encoder", data=rng.standard_normal((6, 2)) * 1e-5, dtype="f")
        hf.create_dataset("binningFactor", data=1, dtype="i")
        hf.create_dataset("dxd", data=(7.2e-6,), dtype="f")
        hf.create_dataset("Nd", data=(16,), dtype="i")
        hf.create_dataset("No", data=(64,), dtype="i")
        hf.create_dataset("zo", data=(0.05,), dtype="f")
        hf.create_dataset("wavelength", data=(632.8e-9,), dtype="f")
        hf.create_dataset("entrancePupilDiameter", data=(3e-5,), dtype="f")
        hf.create_dataset("orientation", data=0)
    files["cpm_simulation"] = (p, "CPM")

    # encoder stored (2, n): transposed and centred on load; orientation 3
    p = OUT_DIR / "cpm_encoder_transposed.hdf5"
    with hdf5.File(p, "w") as hf:
        hf.create_dataset("ptychogram", data=_frames(rng, 5, 12), dtype="f")
        hf.create_dataset("encoder", data=rng.standard_normal((2, 5)) * 1e-5 + 3e-5, dtype="f")
        hf.create_dataset("dxd", data=np.array([[6.5e-6]]))
        hf.create_dataset("zo", data=0.1)
        hf.create_dataset("wavelength", data=np.array([[5e-7]], dtype=np.float32))
        hf.create_dataset("spectralDensity", data=np.array([4.9e-7, 5e-7, 5.1e-7]))
        hf.create_dataset("theta", data=(12.5,), dtype="f")
        hf.create_dataset("orientation", data=np.array([3], dtype=np.int32))
    files["cpm_encoder_transposed"] = (p, "CPM")

    # FPM required + optional fields; orientation 5 (transpose, then columns)
    p = OUT_DIR / "fpm_leds.hdf5"
    with hdf5.File(p, "w") as hf:
        hf.create_dataset("ptychogram", data=_frames(rng, 9, 10), dtype="f")
        g = np.stack(np.meshgrid(np.arange(-1, 2), np.arange(-1, 2)), -1).reshape(-1, 2) * 4e-3
        hf.create_dataset("encoder", data=g)
        hf.create_dataset("dxd", data=(6.5e-6,), dtype="f")
        hf.create_dataset("zled", data=(0.07,), dtype="f")
        hf.create_dataset("magnification", data=(4.0,), dtype="f")
        hf.create_dataset("wavelength", data=(6.25e-7,), dtype="f")
        hf.create_dataset("NA", data=(0.1,), dtype="f")
        hf.create_dataset("orientation", data=5)
    files["fpm_leds"] = (p, "FPM")

    # compressed, chunked ptychogram; orientation 6 (transpose, then rows)
    p = OUT_DIR / "cpm_gzip.hdf5"
    with hdf5.File(p, "w") as hf:
        hf.create_dataset("ptychogram", data=_frames(rng, 7, 16), dtype="f", chunks=(1, 16, 16),
                          compression="gzip", shuffle=True)
        hf.create_dataset("encoder", data=rng.standard_normal((7, 2)) * 1e-5)
        hf.create_dataset("dxd", data=(4.5e-6,), dtype="f")
        hf.create_dataset("zo", data=(0.03,), dtype="f")
        hf.create_dataset("wavelength", data=(1.3e-8,), dtype="f")
        hf.create_dataset("emptyBeam", data=rng.random((16, 16), dtype=np.float32))
        hf.create_dataset("orientation", data=6)
    files["cpm_gzip"] = (p, "CPM")

    # a required field missing
    p = OUT_DIR / "cpm_missing_zo.hdf5"
    with hdf5.File(p, "w") as hf:
        hf.create_dataset("ptychogram", data=_frames(rng, 2, 8), dtype="f")
        hf.create_dataset("encoder", data=np.zeros((2, 2)))
        hf.create_dataset("dxd", data=(4.5e-6,), dtype="f")
        hf.create_dataset("wavelength", data=(1.3e-8,), dtype="f")
    files["cpm_missing_zo"] = (p, "CPM")
    return files


def result_inputs():
    """Attributes of a finished CPM reconstruction, for ``saveResults``."""
    rng = np.random.default_rng(7)
    probe = (rng.standard_normal((1, 1, 2, 1, 8, 8)) + 1j * rng.standard_normal((1, 1, 2, 1, 8, 8))).astype(np.complex64)
    obj = (rng.standard_normal((1, 1, 1, 1, 20, 20)) + 1j * rng.standard_normal((1, 1, 1, 1, 20, 20))).astype(np.complex64)
    return dict(
        probe=probe, object=obj, error=[3.5, 2.25, 1.125], _zo=0.05, wavelength=632.8e-9,
        dxp=1.1e-5, purityProbe=0.93, purityObject=1.0, encoder_corrected=rng.standard_normal((6, 2)) * 1e-5,
        theta=None,
    )


class _TablesNode:
    def __init__(self, f, name):
        self._f = f
        self.name = name

    def read(self):
        return self._f[self.name][()]


class _TablesRoot:
    def __init__(self, f):
        self._f = f

    def __getitem__(self, key):
        if key not in self._f:
            raise KeyError(key)
        return _TablesNode(self._f, key)

    def __contains__(self, key):
        return key in self._f


class _TablesFile:
    def __init__(self, path, mode="r"):
        self._f = hdf5.File(path, "r")
        self.root = _TablesRoot(self._f)

    def list_nodes(self, where):
        return [_TablesNode(self._f, k) for k in self._f.keys()]

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self._f.close()
        return False


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()

    from refload import load_reference

    load_reference(args.reference)
    import importlib

    # the package re-exports classes under its module names: go by module path
    ref_ed = importlib.import_module("PtyLab.ExperimentalData.ExperimentalData")
    ref_read = importlib.import_module("PtyLab.io.readHdf5")
    ref_rec = importlib.import_module("PtyLab.Reconstruction.Reconstruction")

    tables_shim = types.SimpleNamespace(open_file=_TablesFile)
    h5py_shim = types.SimpleNamespace(File=hdf5.File)
    ref_read.tables = tables_shim
    ref_read.h5py = h5py_shim
    ref_rec.h5py = h5py_shim

    out = {}
    for tag, (path, mode) in write_inputs().items():
        try:
            ed = ref_ed.ExperimentalData(str(path), operationMode=mode)
        except Exception as e:  # noqa: BLE001 - the error type is the fixture
            out[f"{tag}/error"] = np.array(type(e).__name__)
            continue
        none = []
        for field in MEASUREMENT_FIELDS:
            if not hasattr(ed, field):
                continue
            v = getattr(ed, field)
            if v is None:
                none.append(field)
            else:
                out[f"{tag}/{field}"] = np.asarray(v)
        out[f"{tag}/none"] = np.array(none)

    # data preparation on a loaded file (ExperimentalData.py:151-190)
    for step, call in (("reduce", lambda e: e.reduce_positions(1, 5)), ("crop", lambda e: e.cropCenter(10)),
                       ("crop_odd", lambda e: e.cropCenter(7)), ("bin", lambda e: e.binData(2))):
        ed = ref_ed.ExperimentalData(str(OUT_DIR / "cpm_simulation.hdf5"), operationMode="CPM")
        call(ed)
        out[f"prep_{step}/ptychogram"] = np.asarray(ed.ptychogram)
        out[f"prep_{step}/encoder"] = np.asarray(ed.encoder)

    attrs = result_inputs()
    ns = types.SimpleNamespace(**attrs)
    ns.data = types.SimpleNamespace(operationMode="CPM")
    res = OUT_DIR.parent / "_result_tmp.hdf5"
    ref_rec.Reconstruction.saveResults(ns, str(res), type="all")
    with hdf5.File(res, "r") as f:
        out["result/names"] = np.array(f.keys())
        for k in f.keys():
            out[f"result/{k}"] = f[k][()]
    res.unlink()
    np.savez(GOLDEN, **out)
    print(f"wrote {GOLDEN} ({len(out)} arrays)")


if __name__ == "__main__":
    main()
