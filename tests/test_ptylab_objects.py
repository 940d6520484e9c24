"""The engines take PtyLab's own ExperimentalData, Params and Reconstruction.

tests/golden/make_ptylab_objects.py builds those objects with the reference
itself, hands them to ptylab_gb300.Engines.<engine>, and records everything
the engine then moves to the GPU (host state, plan geometry, step scalars,
propagator tables) with the reference engine's own result on the same
objects.  Here:
  - the package's own classes, built the same way from the same inputs, give
    exactly the recorded host state (so the GPU path sees identical inputs
    from PtyLab's objects and from the package's);
  - with the reference tree present, the recording is redone live from
    PtyLab's objects (in a separate process, since the reference needs its
    GUI imports stubbed) and must match the committed fixture bit for bit;
  - on the GPU, the engines reproduce the reference's result on those objects.
"""

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_err

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem[len("ptylab_objects_"):] for p in GOLDEN.glob("ptylab_objects_*.npz"))
# the PtyLab.py source tree: PTYLAB_REFERENCE, else a checkout beside this repository
REF = os.environ.get("PTYLAB_REFERENCE") or str(Path(__file__).resolve().parents[2] / "reference")


def _fixture(case):
    with np.load(GOLDEN / f"ptylab_objects_{case}.npz") as f:
        return {k: f[k] for k in f.files}


def _engine_from_clones(fx):
    """The case rebuilt with the package's own classes, as the fixture script builds PtyLab's."""
    sys.path.insert(0, str(GOLDEN))
    from make_ptylab_objects import ptylab_objects

    from ptylab_gb300 import DummyMonitor, Engines, ExperimentalData, Params, Reconstruction

    d = {k[3:]: fx[k] for k in fx if k.startswith("in_")}
    data, params, rec = ptylab_objects((ExperimentalData, Params, Reconstruction), d, int(fx["meta_npsm"]))
    eng = getattr(Engines, str(fx["meta_engine"]))(rec, data, params, DummyMonitor())
    for k in fx:
        if k.startswith("meta_attr_"):
            setattr(eng, k[len("meta_attr_"):], float(fx[k]))
    return eng, rec


@pytest.mark.parametrize("case", CASES)
def test_package_objects_give_the_host_state_ptylabs_objects_gave(case):
    sys.path.insert(0, str(GOLDEN))
    from make_ptylab_objects import engine_host_packet

    fx = _fixture(case)
    eng, _ = _engine_from_clones(fx)
    got = engine_host_packet(eng)
    want = {k: v for k, v in fx.items() if k.startswith("host_")}
    assert sorted(got) == sorted(want)
    for k in want:
        assert got[k].dtype == want[k].dtype, k
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)


@pytest.mark.skipif(not (Path(REF) / "PtyLab").is_dir(), reason="the PtyLab.py source tree is absent")
def test_live_ptylab_objects_match_the_fixture(tmp_path):
    r = subprocess.run([sys.executable, str(GOLDEN / "make_ptylab_objects.py"), "--reference", REF,
                        "--out", str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    for case in CASES:
        want = _fixture(case)
        with np.load(tmp_path / f"ptylab_objects_{case}.npz") as f:
            got = {k: f[k] for k in f.files}
        assert sorted(got) == sorted(want)
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"{case}: {k}")


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_engines_reproduce_the_reference_on_its_objects(case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fx = _fixture(case)
    eng, rec = _engine_from_clones(fx)
    eng.numIterations = int(fx["meta_iters"])
    np.random.seed(int(fx["meta_seed"]))
    eng.reconstruct()
    errs = {k: rel_err(np.asarray(getattr(rec, k)), fx[f"out_{k}"]) for k in ("object", "probe", "error")}
    floor = _reference_spread(fx)
    print(case, "gpu vs reference", errs, "reference c64 vs c128", floor)
    for k, e in errs.items():
        assert e < max(1e-3, 3 * floor[k]), (k, e, floor[k])


def _reference_spread(fx):
    """The reference's own complex64 result against a complex128 oracle run
    from the same host state: its FP32 noise floor on this case (the bar the
    other fixture tests use: max(1e-3, 3 x this spread))."""
    from oracle import ptyoracle as O

    Np, No = int(fx["host_geom_Np"]), int(fx["host_geom_No"])
    wl, zo, dxd = float(fx["in_wavelength"]), float(fx["in_zo"]), float(fx["in_dxd"])
    g = O.Geometry(Np=Np, No=No, dxp=wl * zo / (Np * dxd), wavelength=wl, zo=zo, npsm=int(fx["meta_npsm"]))
    attrs = {k[len("meta_attr_"):]: float(fx[k]) for k in fx if k.startswith("meta_attr_")}
    s = O.Settings(engine=str(fx["meta_engine"]), entrancePupilDiameter=float(fx["in_entrancePupilDiameter"]), **attrs)
    pty = fx["host_ptychogram"].astype(np.float64)
    st = O.State(object=fx["host_object"].astype(np.complex128), probe=fx["host_probe"].astype(np.complex128))
    np.random.seed(int(fx["meta_seed"]))
    r = O.OracleEngine(s, g, st, pty, fx["host_positions"], np.sum(np.abs(fx["host_ptychogram"]), axis=(-1, -2)))
    r = r.reconstruct(int(fx["meta_iters"]))
    return {k: rel_err(fx[f"out_{k}"], np.asarray(getattr(r, k))) for k in ("object", "probe", "error")}
