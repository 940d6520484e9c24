"""Record what the GB300 engines take from PtyLab's own objects (a test fixture).

Usage (needs the PtyLab.py source tree)::

    python tests/golden/make_ptylab_objects.py --reference /path/to/PtyLab.py

For each case, the reference builds its own ExperimentalData, Params and
Reconstruction (its GUI/HDF5 imports stubbed by refload.py) on a small
Fermat-spiral scan, seeds and draws its initial guesses, and the objects are
handed to ``ptylab_gb300.Engines.<engine>``.  The fixture
``ptylab_objects_<case>.npz`` stores, from those objects:

* ``in_*``  -- the raw inputs (ptychogram, encoder, geometry scalars);
* ``host_*`` -- the host state the engine moves to the GPU (_host_state), the
  plan geometry (_geometry), the step scalars (_update_params) and the
  propagator tables (_host_tables), after the engine's host preparation
  (_prepare_host, which mutates the objects the way PtyLab's own preparation
  does);
* ``out_*`` -- the reference engine's own result on a copy of the same
  objects after ITERS iterations (object, probe, error curve).

``tests/test_ptylab_objects.py`` rebuilds the objects with the package's own
classes from ``in_*`` and checks that the engines take exactly ``host_*``
from them; with the reference tree present it also does this live.
"""

from __future__ import annotations

import argparse
import copy
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

SEED = 20240607
ITERS = 3
CASES = {
    # case: (engine, npsm, engine attributes)
    "epie": ("ePIE", 1, {}),
    "mpie_modes": ("mPIE", 2, {"alphaObject": 0.25, "alphaProbe": 0.25}),
    "qnewton": ("qNewton", 1, {}),
}


def dataset():
    from make_golden import fermat_scan_dataset

    return fermat_scan_dataset(nd=32, n_pos=24)


def ptylab_objects(classes, d, npsm):
    """ExperimentalData, Params and Reconstruction built the PtyLab way with
    `classes` (the reference's, or the package's own), seeded guesses drawn."""
    ExperimentalData, Params, Reconstruction = classes
    data = ExperimentalData(None, "CPM")
    for k in ("ptychogram", "encoder", "dxd", "wavelength", "zo", "entrancePupilDiameter"):
        setattr(data, k, d[k])
    data.spectralDensity = None
    data.theta = None
    data.emptyBeam = None
    data._setData()
    params = Params()
    params.gpuSwitch = False
    params.propagatorType = "Fraunhofer"
    params.positionOrder = "sequential"
    params.fftshiftSwitch = False
    rec = Reconstruction(data, params)
    rec.nlambda, rec.nosm, rec.npsm, rec.nslice = 1, 1, npsm, 1
    np.random.seed(SEED)
    rec.initializeObjectProbe()
    return data, params, rec


def engine_host_packet(engine):
    """The engine's host preparation, then everything it moves to the GPU."""
    engine._pre_prepare()
    engine._prepare_host()
    out = {}
    for k, v in engine._host_state().items():
        out[f"host_{k}"] = np.asarray(v)
    g = engine._geometry()
    for name, _ in g._fields_:
        out[f"host_geom_{name}"] = np.int64(getattr(g, name))
    u = engine._update_params()
    for name, _ in u._fields_:
        out[f"host_upd_{name}"] = np.float64(getattr(u, name))
    for name, tab in zip(("fresnel", "asp", "slice"), engine._host_tables()):
        if tab is not None:
            out[f"host_table_{name}"] = np.asarray(tab)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="path to the PtyLab.py source tree")
    ap.add_argument("--out", default=str(HERE), help="directory for the fixtures")
    args = ap.parse_args()
    from refload import load_reference

    load_reference(args.reference)
    from PtyLab import Engines as RefEngines
    from PtyLab.ExperimentalData.ExperimentalData import ExperimentalData
    from PtyLab.Monitor.Monitor import DummyMonitor
    from PtyLab.Params.Params import Params
    from PtyLab.Reconstruction.Reconstruction import Reconstruction

    from ptylab_gb300 import Engines

    d = dataset()
    for case, (eng_name, npsm, attrs) in CASES.items():
        data, params, rec = ptylab_objects((ExperimentalData, Params, Reconstruction), d, npsm)
        run = copy.deepcopy((data, params, rec))
        eng = getattr(Engines, eng_name)(rec, data, params, DummyMonitor())
        for k, v in attrs.items():
            setattr(eng, k, v)
        packet = engine_host_packet(eng)
        rdata, rparams, rrec = run
        ref = getattr(RefEngines, eng_name)(rrec, rdata, rparams, DummyMonitor())
        ref.numIterations = ITERS
        for k, v in attrs.items():
            setattr(ref, k, v)
        np.random.seed(SEED)
        ref.reconstruct()
        out = dict(
            meta_engine=np.array(eng_name), meta_npsm=np.int64(npsm), meta_seed=np.int64(SEED),
            meta_iters=np.int64(ITERS),
            **{f"meta_attr_{k}": np.float64(v) for k, v in attrs.items()},
            **{f"in_{k}": np.asarray(v) for k, v in d.items() if k != "operationMode"},
            **packet,
            out_object=np.asarray(rrec.object), out_probe=np.asarray(rrec.probe),
            out_error=np.asarray(rrec.error, dtype=np.float64),
        )
        path = Path(args.out) / f"ptylab_objects_{case}.npz"
        np.savez_compressed(path, **out)
        print(f"wrote {path.name}: {len(packet)} host entries")


if __name__ == "__main__":
    main()
