"""Host-side logic of the drop-in against the reference fixtures and the oracle (no GPU)."""

from pathlib import Path

import numpy as np
import pytest

from conftest import fixture_names, load_fixture
from oracle import ptyoracle as O
from ptylab_gb300 import ExperimentalData, Params, Reconstruction, _tables


def containers(fx):
    """Build the package's ExperimentalData/Params/Reconstruction from a fixture."""
    m = {k[5:]: fx[k] for k in fx if k.startswith("meta_")}
    i = {k[3:]: fx[k] for k in fx if k.startswith("in_")}
    mode = str(m["operationMode"])
    d = ExperimentalData(None, mode)
    d.ptychogram = i["ptychogram"]
    d.encoder = i["encoder"]
    d.dxd = float(m["dxd"])
    d.wavelength = float(i["wavelength"])
    if mode == "CPM":
        d.zo = float(i["zo"])
        d.entrancePupilDiameter = float(i["entrancePupilDiameter"])
    else:
        d.zled = float(m["zled"])
        d.magnification = float(m["magnification"])
        d.NA = float(m["NA"])
    d._setData()
    p = Params()
    p.propagatorType = str(m["propagator"])
    p.positionOrder = str(m["order"])
    p.fftshiftSwitch = bool(m["fftshift"])
    p.probeBoundary = bool(m["probeBoundary"])
    p.orthogonalizationSwitch = bool(m["orthogonalizationSwitch"])
    p.orthogonalizationFrequency = int(m["orthogonalizationFrequency"])
    # intensity-projection switches and their tables (absent from older fixtures)
    p.intensityConstraint = str(m.get("intensityConstraint", "standard"))
    p.adaptiveDenoisingSwitch = bool(m.get("adaptiveDenoisingSwitch", False))
    p.backgroundModeSwitch = bool(m.get("backgroundModeSwitch", False))
    p.FourierMaskSwitch = bool(m.get("FourierMaskSwitch", False))
    p.saveMemory = bool(m.get("saveMemory", False))
    p.probePowerCorrectionSwitch = bool(m.get("probePowerCorrectionSwitch", False))
    if bool(m.get("intensityMask", False)):
        p.intensityMask = True
    if "W" in i:
        d.W = np.array(i["W"], copy=True)
    if "intensityScaling" in i:
        p.intensityScaling = np.array(i["intensityScaling"], copy=True)
    rec = Reconstruction(d, p, No=int(i["No"]) if mode == "FPM" else None)
    nl, nos, nps, nsl = (int(v) for v in m["modes"])
    rec.nlambda, rec.nosm, rec.npsm, rec.nslice = nl, nos, nps, nsl
    if "spectralDensity" in i:
        rec.spectralDensity = np.array(i["spectralDensity"], copy=True)
    if nsl > 1:
        rec.dz = float(i["dz"])
        rec.refrIndex = 1.0
    if "intensity_mask" in i:
        rec.intensity_mask = np.array(i["intensity_mask"], copy=True)
    return m, i, d, p, rec


@pytest.mark.parametrize("name", fixture_names("reg_") + fixture_names("scan_"))
def test_geometry_positions_and_seeded_guesses(name):
    """Reconstruction.positions, No, dxp and the seeded initial guesses match the reference."""
    fx = load_fixture(name)
    m, i, d, p, rec = containers(fx)
    assert rec.No == int(i["No"])
    assert rec.dxp == pytest.approx(float(i["dxp"]), rel=1e-15)
    np.testing.assert_array_equal(rec.positions, i["positions"])
    np.testing.assert_array_equal(d.energyAtPos, i["energyAtPos"])
    np.random.seed(int(m["seed"]))
    rec.initializeObjectProbe()
    np.testing.assert_array_equal(rec.object, i["init_object"])
    np.testing.assert_array_equal(rec.probe, i["init_probe"])
    assert d.entrancePupilDiameter == pytest.approx(float(i["entrancePupilDiameter"]), rel=1e-15)


def test_random_order_and_momentum_draws_follow_the_global_rng():
    """A shuffle then rand(n) consumes the legacy RNG like a shuffle then n x rand(1)
    (BaseEngine.py:646-653, mPIE.py:170)."""
    np.random.seed(3)
    idx = np.arange(40)
    np.random.shuffle(idx)
    batch = np.random.rand(40)
    np.random.seed(3)
    idx2 = np.arange(40)
    np.random.shuffle(idx2)
    single = np.array([np.random.rand(1)[0] for _ in range(40)])
    np.testing.assert_array_equal(idx, idx2)
    np.testing.assert_array_equal(batch, single)


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_tables_match_the_oracle(n):
    dxp, lam, z = 1.3e-5, 632.8e-9, 0.05
    np.testing.assert_array_equal(_tables.fresnel_chirp(z, lam, n, dxp), O.quad_phase(z, lam, n, dxp))
    np.testing.assert_array_equal(
        _tables.angular_spectrum_tf(z, lam, n, n * dxp), O.aspw_transfer_function(z, lam, n, n * dxp)
    )
    np.testing.assert_array_equal(
        _tables.asp_detector_tf(z, lam, n, n * dxp)[None, None, None, None],
        O.asp_transfer_function(1, 1, n, z, lam, n * dxp),
    )


def _bitrev5(l):
    return int(f"{l:05b}"[::-1], 2)


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_fourier_layout_is_a_permutation(n):
    """slot s = 32 r + l holds frequency k = r + E*bitrev5(l) (kernel layout); a bijection."""
    E = n // 32
    k = np.array([(s >> 5) + E * _bitrev5(s & 31) for s in range(n)])
    assert sorted(k.tolist()) == list(range(n))
    # the inverse used by from_fourier_layout: s = 32*(k % E) + bitrev5(k // E)
    s_back = np.array([32 * (kk % E) + _bitrev5(kk // E) for kk in k])
    np.testing.assert_array_equal(s_back, np.arange(n))


def test_multislice_transfer_function_matches_the_oracle():
    """e3PIE.py:62-69: aspw at dz, wavelength / refrIndex, Np, Lp."""
    dz, lam, n, Np, dxp = 10e-6, 13.5e-9, 1.0, 256, 20e-9
    np.testing.assert_array_equal(
        _tables.multislice_tf(dz, lam, n, Np, Np * dxp), O.aspw_transfer_function(dz, lam / n, Np, Np * dxp)
    )


def test_mqnewton_host_logic():
    """mqNewton.py:50-79: defaults, the method lookup, and the second moments
    the kernel carries as scalars (uniform real arrays)."""
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_mqnewton_adam")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    rec.initialGuessObject, rec.initialGuessProbe = rec.object.copy(), rec.probe.copy()
    eng = Engines.mqNewton(rec, d, p, DummyMonitor())
    assert (eng.beta1, eng.beta2, eng.betaObject_m, eng.betaProbe_m, eng.momentum_method) == (0.5, 0.5, 0.25, 0.25, "ADAM")
    assert p.momentumAcceleration
    np.testing.assert_array_equal(rec.objectBuffer, rec.object)
    assert not np.any(rec.objectMomentum) and rec.objectMomentum.shape == rec.object.shape
    eng.initializeAdaptiveMomentum()
    assert eng._second_moments() == [0.0, 0.0]
    rec.objectMomentum_v = np.full(rec.object.shape, np.complex64(0.25))
    assert eng._second_moments()[0] == 0.25
    rec.objectMomentum_v.flat[3] = 1.0  # what a second reconstruct() produces
    with pytest.raises(NotImplementedError):
        eng._second_moments()
    eng.momentum_method = "Adagrad"
    with pytest.raises(AttributeError):
        eng.initializeAdaptiveMomentum()


def test_reconstruct_batch_rejects_mismatched_engines():
    """Engines that cannot share one launch are refused before any device work."""
    from ptylab_gb300 import DummyMonitor, Engines

    def make(name, **over):
        fx = load_fixture(name)
        m, i, d, p, rec = containers(fx)
        rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
        rec.initialGuessObject, rec.initialGuessProbe = rec.object.copy(), rec.probe.copy()
        eng = Engines.ePIE(rec, d, p, DummyMonitor())
        for k, v in over.items():
            setattr(eng, k, v)
        return eng

    with pytest.raises(ValueError, match="update parameters"):
        Engines.reconstruct_batch([make("scan_epie_random"), make("scan_epie_random", betaObject=0.5)])
    with pytest.raises(ValueError, match="geometry"):
        Engines.reconstruct_batch([make("scan_epie_random"), make("reg_epie_fraunhofer")])
    with pytest.raises(ValueError, match="one class"):
        fx = load_fixture("scan_epie_random")
        m, i, d, p, rec = containers(fx)
        rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
        Engines.reconstruct_batch([make("scan_epie_random"), Engines.qNewton(rec, d, p, DummyMonitor())])


def test_several_wavelengths_are_checked_before_device_work():
    """nlambda > 1 runs with ePIE, mPIE, qNewton and mqNewton (not e3PIE);
    ASP refuses it as PtyLab's does (Operators.py:866-869) and polychromeASP
    needs a wavelength per slot."""
    from ptylab_gb300 import DummyMonitor, Engines

    def setup(engine, propagator, spectral=True):
        fx = load_fixture("reg_epie_polychrome")
        m, i, d, p, rec = containers(fx)
        p.propagatorType = propagator
        if not spectral:
            rec.spectralDensity = np.atleast_1d(rec.wavelength)
        rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
        rec.initialGuessObject, rec.initialGuessProbe = rec.object.copy(), rec.probe.copy()
        return getattr(Engines, engine)(rec, d, p, DummyMonitor())

    setup("mqNewton", "polychromeASP")._check_supported()
    setup("mPIE", "polychromeASP")._check_supported()
    setup("qNewton", "polychromeASP")._check_supported()
    with pytest.raises(ValueError):
        setup("ePIE", "ASP")._check_supported()
    with pytest.raises(ValueError):
        setup("ePIE", "polychromeASP", spectral=False)._check_supported()
    setup("ePIE", "polychromeASP")._check_supported()
    setup("ePIE", "Fraunhofer")._check_supported()


def test_beam_width_and_overlap_match_reference():
    """getBeamWidth / getOverlap (BaseEngine.py:744-818) against the
    reference's own methods on the same probe and positions."""
    import types

    from ptylab_gb300.Engines.BaseEngine import BaseEngine

    g = np.load(Path(__file__).parent / "golden" / "analysis_golden.npz")
    rec = types.SimpleNamespace(**{k[3:]: g[k] for k in g.files if k.startswith("in_")})
    rec.Np, rec.dxp = int(rec.Np), float(rec.dxp)
    eng = types.SimpleNamespace(reconstruction=rec)
    by, bx = BaseEngine.getBeamWidth(eng)
    np.testing.assert_allclose(by, g["beamWidthY"], rtol=1e-12)
    np.testing.assert_allclose(bx, g["beamWidthX"], rtol=1e-12)
    eng.getBeamWidth = lambda: BaseEngine.getBeamWidth(eng)
    for a, b in ((0, 3), (2, 7), (5, 5)):
        lin, area = BaseEngine.getOverlap(eng, a, b)
        np.testing.assert_allclose(lin, g[f"linear_{a}_{b}"], rtol=1e-12)
        np.testing.assert_allclose(area, g[f"area_{a}_{b}"], rtol=1e-6)
