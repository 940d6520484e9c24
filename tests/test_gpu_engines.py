"""GB300 engines against the reference's own outputs (fixtures) and the oracle.

Parity metric: relative Frobenius error, as in the reference's GPU-vs-CPU
test (tests/regression/test_engine_regression.py:140-175).  The reference
accepts 1e-3 there (its CuPy/cuFFT path measured 1e-8 ... 2.2e-4); this suite
uses the same 1e-3 bound on the 2-5 iteration fixtures and records the
measured values in the assertion messages.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import fixture_names, load_fixture, rel_err
from test_host_logic import containers

pytestmark = pytest.mark.gpu
TOL_FIXTURE = 1e-3
IN_SCOPE = [n for n in fixture_names("reg_") + fixture_names("scan_") if "e3pie" not in n]


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def run_fixture_gpu(fx, engine_name=None, iters=None):
    from ptylab_gb300 import DummyMonitor, Engines

    m, i, d, p, rec = containers(fx)
    rec.initialGuessObject = i["init_object"].copy()
    rec.initialGuessProbe = i["init_probe"].copy()
    rec.object = i["init_object"].copy()
    rec.probe = i["init_probe"].copy()
    eng = getattr(Engines, engine_name or str(m["engine"]))(rec, d, p, DummyMonitor())
    eng.numIterations = int(m["iters"]) if iters is None else iters
    np.random.seed(int(m["seed"]))
    eng.reconstruct()
    return rec, eng


@pytest.mark.parametrize("name", IN_SCOPE)
def test_engine_matches_reference_fixture(torch_cuda, name):
    fx = load_fixture(name)
    rec, _ = run_fixture_gpu(fx)
    errs = {k: rel_err(getattr(rec, k), fx[f"out_{k}"]) for k in ("object", "probe", "error", "errorAtPos")}
    assert rec.object.dtype == np.complex64 and rec.probe.dtype == np.complex64
    assert rec.object.shape == fx["out_object"].shape and rec.probe.shape == fx["out_probe"].shape
    assert all(v < TOL_FIXTURE for v in errs.values()), f"{name}: {errs}"
    if "out_detectorError" in fx:
        assert rel_err(rec.detectorError, fx["out_detectorError"]) < TOL_FIXTURE
    if "out_objectMomentum" in fx:
        assert rel_err(rec.objectMomentum, fx["out_objectMomentum"]) < 1e-2
        assert rel_err(rec.probeMomentum, fx["out_probeMomentum"]) < 1e-2


def test_stepwise_equals_reconstruct(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_random")
    rec_a, _ = run_fixture_gpu(fx)
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    eng = Engines.ePIE(rec, d, p, DummyMonitor())
    eng.numIterations = int(m["iters"])
    np.random.seed(int(m["seed"]))
    steps = list(eng.reconstruct_stepwise())
    assert len(steps) == int(m["iters"]) * d.numFrames
    np.testing.assert_array_equal(rec.object, rec_a.object)
    np.testing.assert_array_equal(rec.probe, rec_a.probe)
    np.testing.assert_array_equal(rec.error, rec_a.error)


def test_unsupported_switch_raises(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("reg_epie_fraunhofer")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    p.intensityConstraint = "poission"
    eng = Engines.ePIE(rec, d, p, DummyMonitor())
    with pytest.raises(NotImplementedError):
        eng.reconstruct()


def test_asp_with_fftshift_raises_value_error(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_asp")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    p.fftshiftSwitch = True
    with pytest.raises(ValueError):
        Engines.ePIE(rec, d, p, DummyMonitor()).reconstruct()


def test_position_outside_object_raises(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_random")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    rec.encoder_corrected = rec.encoder_corrected * 100
    with pytest.raises(ValueError):
        Engines.ePIE(rec, d, p, DummyMonitor()).reconstruct()


def test_batched_scans_equal_single_runs(torch_cuda):
    """G independent scans in one launch (one cluster each) reproduce G single-scan launches bitwise."""
    torch = torch_cuda
    from ptylab_gb300 import _native
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    lib = _native.require(0)
    G, Np, No, nf = 3, 64, 192, 30
    scans = []
    for g in range(G):
        d, p, rec, _, _ = cpm_problem(ScanSpec(Np=Np, No=No, num_positions=nf, seed=100 + g), engine_seed=g)
        scans.append((d, rec))

    def run(scan_ids):
        geom = _native.Geometry(Np=Np, No=No, nosm=1, npsm=1, nslice=1, num_frames=nf, num_scans=len(scan_ids),
                                engine=0, propagator=0, fftshift=0, fpm=0, cluster=0)
        plan = C.c_void_p()
        _native.check(lib.ptyg_plan_create(C.byref(geom), C.byref(plan)))
        keep, outs = [], []
        for s, g in enumerate(scan_ids):
            d, rec = scans[g]
            obj = torch.from_numpy(rec.object.copy()).cuda()
            prb = torch.from_numpy(rec.probe.copy()).cuda()
            pos = torch.from_numpy(rec.positions.astype(np.int32)).cuda()
            order = torch.arange(nf, dtype=torch.int32, device="cuda")
            data = torch.from_numpy(d.ptychogram).cuda()
            b = _native.ScanBuffers(object=obj.data_ptr(), probe=prb.data_ptr(), positions=pos.data_ptr(),
                                    order=order.data_ptr())
            _native.check(lib.ptyg_plan_bind_scan(plan, s, C.byref(b), data.data_ptr(), None))
            keep += [obj, prb, pos, order, data, b]
            outs.append((obj, prb))
        u = _native.UpdateParams(beta_object=0.25, beta_probe=0.25, probe_weight=1.0)
        for _ in range(3):
            _native.check(lib.ptyg_plan_run(plan, C.byref(u), 0, nf, 0, None))
        torch.cuda.synchronize()
        lib.ptyg_plan_destroy(plan)
        return [(o.cpu().numpy(), q.cpu().numpy()) for o, q in outs]

    batched = run(list(range(G)))
    for g in range(G):
        single = run([g])[0]
        np.testing.assert_array_equal(batched[g][0], single[0])
        np.testing.assert_array_equal(batched[g][1], single[1])


@pytest.mark.parametrize("engine", ["ePIE", "mPIE"])
def test_config0_size_against_oracle(torch_cuda, engine):
    """Np=64, No=256, 100 Fermat positions, 20 iterations: GB300 vs the complex64 oracle
    (the reference's algorithm) from the same seeded guesses."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    d, p, rec, _, _ = cpm_problem(ScanSpec())
    obj0, prb0 = rec.object.copy(), rec.probe.copy()
    eng = getattr(Engines, engine)(rec, d, p, DummyMonitor())
    eng.numIterations = 20
    np.random.seed(5)
    eng.reconstruct()
    g = O.Geometry(Np=64, No=256, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo)
    s = O.Settings(engine=engine, entrancePupilDiameter=d.entrancePupilDiameter)
    st = O.State(object=obj0, probe=prb0)
    np.random.seed(5)
    ref = O.OracleEngine(s, g, st, d.ptychogram, rec.positions, d.energyAtPos).reconstruct(20)
    errs = {k: rel_err(getattr(rec, k), getattr(ref, k)) for k in ("object", "probe", "error")}
    # ePIE: 1e-4 (spec bound); mPIE: bounded by the reference's own c64-vs-c128 spread
    tol = {"ePIE": 1e-3, "mPIE": 1e-2}[engine]
    assert all(v < tol for v in errs.values()), f"{engine}: {errs}"
    print(f"{engine} C0 x20 vs oracle: {errs}")
