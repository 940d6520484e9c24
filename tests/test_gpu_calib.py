"""FPM illumination calibration on the GPU (``ptyg_calib_*`` and
``ptylab_gb300.CalibrationFPM``) against the oracle and the reference's
goldens.

Tolerances: the window product, frame sums, pupil masks and the decisions
are exact; the FP32 transforms differ from NumPy's pocketfft in summation
order (1e-5 relative); SciPy's Gaussian and bilinear sampling are followed
operation by operation (1e-6 relative, SciPy builds may contract to FMA);
candidate RMSEs come from complex64 transforms where the reference uses
complex128 (1e-5 relative).  End to end, every integer decision (brightfield
split, per-LED positions, fitted positions) must equal the reference's.
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).parent.parent / "oracle"))

import calib_oracle as co  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"
CASES = sorted(p.stem[len("calib_"):] for p in GOLDEN.glob("calib_*.npz"))


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def load_case(name):
    g = np.load(GOLDEN / f"calib_{name}.npz")
    settings = {}
    for k, v in zip(g["calib_keys"], g["calib_values"]):
        v = str(v)
        settings[str(k)] = v == "True" if v in ("True", "False") else v
    return g, settings


def rel(a, b):
    """Largest difference relative to the largest magnitude (complex-safe)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a.astype(np.complex128) - b)) / max(float(np.max(np.abs(b))), 1e-30))


@pytest.mark.parametrize("N", [64, 128, 256])
def test_fourier_images(torch_cuda, N):
    from ptylab_gb300.CalibrationFPM import _Device, gaussian_half_weights, hann_window

    rng = np.random.default_rng(N)
    frames = rng.poisson(200.0, (9, N, N)).astype(np.float32)
    dev = _Device()
    w = hann_window((N, N))
    windowed, sums, spectra, ft, norm = dev.spectra(frames, w)
    ref_win = frames.copy()
    ref_win *= w[None]
    np.testing.assert_array_equal(dev.to_host(windowed), ref_win)
    np.testing.assert_allclose(dev.to_host(sums), ref_win.astype(np.float64).sum((1, 2)), rtol=1e-12)
    ref_spec = co.ifft2c(ref_win)
    assert rel(dev.to_host(spectra), ref_spec) < 1e-5
    ref_ft = np.abs(ref_spec)
    assert rel(dev.to_host(ft), ref_ft) < 1e-5
    assert rel(dev.to_host(norm), np.mean(ref_ft, 0)) < 1e-5
    # normalisation and smoothing on identical input
    ft_in = torch_cuda.from_numpy(ref_ft).cuda()
    norm_in = torch_cuda.from_numpy(np.mean(ref_ft, 0)).cuda()
    floor = np.float32(2 * np.mean(np.mean(ref_ft, 0)[: N // 4]))
    dev.normalise(ft_in, norm_in, floor)
    want = np.abs(ref_ft / np.maximum(np.mean(ref_ft, 0), floor))
    np.testing.assert_array_equal(dev.to_host(ft_in), want)
    dev.gaussian(ft_in, 3)
    want_g = np.stack([co.gaussian(x, 3) for x in want])
    assert rel(dev.to_host(ft_in), want_g) < 1e-6
    r, hw = gaussian_half_weights(3)
    assert r == 12 and hw.size == 13


def test_circle_search_and_rms(torch_cuda):
    from ptylab_gb300.CalibrationFPM import IlluminationCalibration

    g, settings = load_case("similarity")
    rec = types.SimpleNamespace(Np=int(g["Np"]), No=int(g["No"]), dxp=float(g["dxp"]), dxo=float(g["dxp"]),
                                wavelength=float(g["wavelength"]), NA=float(g["NA_in"]), zled=float(g["zled"]),
                                positions=g["positions"].copy())
    data = types.SimpleNamespace(ptychogram=g["ptychogram"].astype(np.float32), encoder=g["encoder"].copy())
    ic = IlluminationCalibration(rec, data)
    ic.initialize_error_search_space()
    oracle = co.CalibrationOracle(rec.Np, rec.No, rec.dxp, rec.wavelength, rec.NA)
    frames = g["ptychogram"].astype(np.float32)[:12]
    FT = oracle.convertToFourierSpace(frames)  # windows frames in place
    dev = ic._device()
    ft_dev = torch_cuda.from_numpy(FT).cuda()
    radii = np.mgrid[4.0:-0.5:-0.5] + ic.apertRadiusPixel
    positions = np.array([[0, 0], [5, -7], [-20, 13], [33, 30], [-41, -2], [12, 44]])
    cs = ic._circle_search(ft_dev, np.arange(len(positions)) % len(FT), positions, radii)
    for t, p in enumerate(positions):
        want = oracle.circle_search(FT[t % len(FT)], p, radii)
        assert rel(cs[t], want) < 1e-6
    # RMSE of candidate shifts
    img = torch_cuda.from_numpy(frames).cuda()
    spectra = dev.ifft2c(img)
    cand_led = [0, 0, 0, 3, 3, 7]
    q = [(0, 0), (2, -1), (-3, 4), (10, -9), (11, -9), (-5, 6)]
    got = dev.rms(spectra, img, cand_led, q, ic.apertRadiusPixel)
    F = co.ifft2c(frames)
    want = np.array([co.rms_of_candidates(frames[l], F[l], [(0, 0)], qq, ic.apertRadiusPixel)[0]
                     for l, qq in zip(cand_led, q)])
    np.testing.assert_allclose(got, want, rtol=1e-5)


@pytest.mark.parametrize("name", CASES)
def test_calibration_matches_reference(torch_cuda, name):
    from ptylab_gb300.CalibrationFPM import IlluminationCalibration

    g, settings = load_case(name)
    rec = types.SimpleNamespace(Np=int(g["Np"]), No=int(g["No"]), dxp=float(g["dxp"]), dxo=float(g["dxp"]),
                                wavelength=float(g["wavelength"]), NA=float(g["NA_in"]), zled=float(g["zled"]),
                                positions=g["positions"].copy())
    data = types.SimpleNamespace(ptychogram=g["ptychogram"].astype(np.float32), encoder=g["encoder"].copy())
    ic = IlluminationCalibration(rec, data)
    for k, v in settings.items():
        setattr(ic, k, v)
    np.random.seed(1234)
    m = ic.runCalibration()
    np.testing.assert_array_equal(ic.brightfieldIndices, g["brightfield"])
    assert ic.apertRadiusPixel == float(g["radius"])
    assert rec.NA == pytest.approx(float(g["NA"]), rel=1e-15)
    np.testing.assert_array_equal(ic.positionsFitted, g["positionsFitted"])
    np.testing.assert_allclose(m.params, g["matrix"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(data.encoder, g["encoder_out"], rtol=0, atol=1e-12)
    oracle = co.CalibrationOracle(rec.Np, rec.No, rec.dxp, rec.wavelength, float(g["NA_in"]), **settings)
    np.random.seed(1234)
    oracle.run(g["ptychogram"].astype(np.float32), g["positions"])
    np.testing.assert_array_equal(ic.calibrated_positions, oracle.calibrated_positions)


def test_single_frame_rmse_api(torch_cuda):
    """calculateRMSE, the reference's per-frame entry point."""
    from ptylab_gb300.CalibrationFPM import IlluminationCalibration

    g, settings = load_case("affine_small")
    rec = types.SimpleNamespace(Np=int(g["Np"]), No=int(g["No"]), dxp=float(g["dxp"]), dxo=float(g["dxp"]),
                                wavelength=float(g["wavelength"]), NA=float(g["NA_in"]), zled=float(g["zled"]),
                                positions=g["positions"].copy())
    ic = IlluminationCalibration(rec, types.SimpleNamespace(ptychogram=None, encoder=None))
    ic.initialize_error_search_space()
    oracle = co.CalibrationOracle(rec.Np, rec.No, rec.dxp, rec.wavelength, rec.NA)
    frame = g["ptychogram"][24].astype(np.float32)
    cand = np.array([[a, b] for a in range(0, 13, 3) for b in range(0, 13, 4)])
    got = ic.calculateRMSE(frame, cand, (-2, 3))
    want = oracle.calculateRMSE(frame, cand, (-2, 3))[:3]
    assert tuple(int(x) for x in got[:2]) == tuple(int(x) for x in want[:2]) and bool(got[2]) == bool(want[2])
