"""The FPM illumination-calibration oracle (oracle/calib_oracle.py) against
goldens the reference's own ``IlluminationCalibration`` produced
(tests/golden/make_calib_golden.py): every per-LED search decision, the
brightfield split, radius, NA, transform, fitted positions and encoder."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).parent.parent / "oracle"))

import calib_oracle as co  # noqa: E402

GOLDEN = Path(__file__).parent / "golden"
CASES = sorted(p.stem[len("calib_"):] for p in GOLDEN.glob("calib_*.npz"))


def load_case(name):
    g = np.load(GOLDEN / f"calib_{name}.npz")
    settings = {}
    for k, v in zip(g["calib_keys"], g["calib_values"]):
        v = str(v)
        settings[str(k)] = v == "True" if v in ("True", "False") else v
    return g, settings


def run_oracle(g, settings, record=None):
    c = co.CalibrationOracle(int(g["Np"]), int(g["No"]), float(g["dxp"]), float(g["wavelength"]), float(g["NA_in"]),
                             **settings)
    if record is not None:
        orig = c.calculateRMSE

        def logged(image, cand, position):
            ex, ey, edge, rms = orig(image, cand, position)
            record.append([float(position[0]), float(position[1]), ex, ey, int(edge), len(cand)])
            return ex, ey, edge, rms

        c.calculateRMSE = logged
    np.random.seed(1234)
    m, NA, epd, fitted = c.run(g["ptychogram"].astype(np.float32), g["positions"])
    return c, m, NA, epd, fitted


def test_cases_present():
    assert set(CASES) >= {"similarity", "translation_radius", "affine_small"}


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    g, settings = load_case(name)
    rec = []
    c, m, NA, epd, fitted = run_oracle(g, settings, rec)
    np.testing.assert_array_equal(c.brightfieldIndices, g["brightfield"])
    np.testing.assert_array_equal(np.array(rec), g["decisions"])
    assert c.apertRadiusPixel == pytest.approx(float(g["radius"]), rel=0, abs=0)
    assert NA == pytest.approx(float(g["NA"]), rel=1e-15)
    assert epd == pytest.approx(float(g["entrancePupilDiameter"]), rel=1e-15)
    np.testing.assert_allclose(m.params, g["matrix"], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(fitted, g["positionsFitted"])
    enc = co.encoder_update(g["encoder"], m.params, float(g["wavelength"]), float(g["dxp"]), int(g["Np"]),
                            float(g["zled"]))
    np.testing.assert_allclose(enc, g["encoder_out"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("name", CASES[:1])
def test_fourier_images_match_reference(name):
    g, settings = load_case(name)
    c = co.CalibrationOracle(int(g["Np"]), int(g["No"]), float(g["dxp"]), float(g["wavelength"]), float(g["NA_in"]))
    frames = g["ptychogram"].astype(np.float32)
    ft = c.convertToFourierSpace(frames)
    np.testing.assert_array_equal(ft[[0, len(ft) // 2]], g["ft_frames"])


def test_restated_routines():
    # Hann: symmetric, zero at the corners' radius, one at the centre
    w = co.hann_window((64, 64))
    assert w.shape == (64, 64) and np.allclose(w, w.T) and np.allclose(w, w[::-1, ::-1])
    assert w.max() <= 1 and w.min() >= 0 and w[0, 0] == 0 and w[32, 32] > 0.99
    # Umeyama recovers an exact similarity
    rng = np.random.default_rng(0)
    src = rng.standard_normal((12, 2))
    t = 0.3
    M = np.array([[1.2 * np.cos(t), -1.2 * np.sin(t), 3.0], [1.2 * np.sin(t), 1.2 * np.cos(t), -1.0], [0, 0, 1]])
    dst = co.matrix_transform(src, M)
    np.testing.assert_allclose(co.umeyama(src, dst, True), M, atol=1e-12)
    # RANSAC ignores an outlier
    dst_bad = dst.copy()
    dst_bad[3] += 50
    model, inl = co.ransac((src, dst_bad), co.SimilarityTransform, 2, 0.5, max_trials=1000)
    assert not inl[3] and inl.sum() == 11
    np.testing.assert_allclose(model.params, M, atol=1e-10)
    # gaussian weights as scipy builds them
    r, wts = co.gaussian_weights(3)
    assert r == 12 and abs(wts.sum() - 1) < 1e-15
