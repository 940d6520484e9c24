"""Host side of ``ptylab_gb300.CalibrationFPM`` on the CPU: the batched
search (every LED's rounds together, the device calls' contract) with the
five device calls emulated in the reference's NumPy/SciPy arithmetic, against
the oracle and the reference's goldens; plus the host routines it shares
with the oracle's restatements."""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).parent.parent / "oracle"))

import calib_oracle as co  # noqa: E402

from ptylab_gb300 import CalibrationFPM as cal  # noqa: E402

GOLDEN = Path(__file__).parent / "golden"
CASES = sorted(p.stem[len("calib_"):] for p in GOLDEN.glob("calib_*.npz"))


class NumpyDevice:
    """The contract of the ptyg_calib_* calls, in the reference's arithmetic."""

    def __init__(self, oracle):
        self.oracle = oracle
        self.calls = {"arcs": 0, "rms": 0}

    def take(self, arr, idx):
        return np.ascontiguousarray(arr[np.asarray(idx)])

    def to_host(self, arr):
        return np.asarray(arr)

    def upload(self, arr):
        return np.ascontiguousarray(arr, dtype=np.float32)

    def ifft2c(self, images):
        return co.ifft2c(np.asarray(images, dtype=np.float32))

    def spectra(self, frames, window):
        windowed = np.asarray(frames, dtype=np.float32).copy()
        windowed *= window[None]
        sums = np.sum(windowed.astype(np.float64), (1, 2))
        spectra = co.ifft2c(windowed)
        ft = np.abs(spectra)
        return windowed, sums, spectra, ft, np.mean(ft, 0)

    def normalise(self, ft, norm, floor_value):
        ft[...] = np.abs(ft / np.maximum(norm, floor_value))

    def gaussian(self, images, sigma, out=None):
        out = images if out is None else out
        for i in range(len(images)):
            out[i] = co.gaussian(images[i], sigma)
        return out

    def arcs(self, images, task_image, task_pos, task_keep, radii, sin_a, cos_a, search):
        self.calls["arcs"] += 1
        out = []
        for ti, pos, keep in zip(task_image, task_pos, task_keep):
            arcs = self.oracle.circular_arcs(pos, radii)
            ref_keep = np.all((arcs[..., 0] > -np.inf), axis=(0, 1, 2))  # shape check only
            assert arcs.shape[3] == bin(int(keep)).count("1") and ref_keep.size == arcs.shape[3]
            out.append(self.oracle.circle_search(images[ti], pos, radii))
        return np.array(out, dtype=np.float32)

    def rms(self, spectra, images, cand_led, cand_q, radius):
        self.calls["rms"] += 1
        out = []
        for led, (q0, q1) in zip(cand_led, cand_q):
            out.append(co.rms_of_candidates(images[led], spectra[led], [(0, 0)], (q0, q1), radius)[0])
        return np.array(out)


def load_case(name):
    g = np.load(GOLDEN / f"calib_{name}.npz")
    settings = {}
    for k, v in zip(g["calib_keys"], g["calib_values"]):
        v = str(v)
        settings[str(k)] = v == "True" if v in ("True", "False") else v
    return g, settings


def build(g, settings):
    rec = types.SimpleNamespace(Np=int(g["Np"]), No=int(g["No"]), dxp=float(g["dxp"]), dxo=float(g["dxp"]),
                                wavelength=float(g["wavelength"]), NA=float(g["NA_in"]), zled=float(g["zled"]),
                                positions=g["positions"].copy())
    data = types.SimpleNamespace(ptychogram=g["ptychogram"].astype(np.float32), encoder=g["encoder"].copy())
    ic = cal.IlluminationCalibration(rec, data)
    for k, v in settings.items():
        setattr(ic, k, v)
    oracle = co.CalibrationOracle(rec.Np, rec.No, rec.dxp, rec.wavelength, rec.NA, **settings)
    ic._dev = NumpyDevice(oracle)
    return ic, rec, data, oracle


@pytest.mark.parametrize("name", CASES)
def test_batched_search_matches_reference(name):
    g, settings = load_case(name)
    ic, rec, data, oracle = build(g, settings)
    np.random.seed(1234)
    m = ic.runCalibration()
    np.testing.assert_array_equal(ic.brightfieldIndices, g["brightfield"])
    assert ic.apertRadiusPixel == float(g["radius"])
    assert rec.NA == pytest.approx(float(g["NA"]), rel=1e-15)
    assert rec.entrancePupilDiameter == pytest.approx(float(g["entrancePupilDiameter"]), rel=1e-15)
    np.testing.assert_allclose(m.params, g["matrix"], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(ic.positionsFitted, g["positionsFitted"])
    np.testing.assert_allclose(data.encoder, g["encoder_out"], rtol=0, atol=1e-15)
    # the per-LED end points equal the oracle's LED-by-LED search
    np.random.seed(1234)
    oracle.run(g["ptychogram"].astype(np.float32), g["positions"])
    np.testing.assert_array_equal(ic.calibrated_positions, oracle.calibrated_positions)
    assert ic.failed_position_calib == oracle.failed
    # batched: one circle search and one RMSE batch per round, not per LED
    assert ic._dev.calls["rms"] == ic.rounds <= 6
    assert ic.rounds == int(np.max(oracle.rounds))


def test_host_routines_equal_the_restatements():
    for n in (32, 64, 128, 256):
        np.testing.assert_array_equal(cal.hann_window((n, n)), co.hann_window((n, n)))
    r, w = cal.gaussian_half_weights(3)
    r2, w2 = co.gaussian_weights(3)
    assert r == r2 and np.array_equal(w, w2[r2:])
    rng = np.random.default_rng(1)
    src = rng.standard_normal((15, 2)) * 10
    for cls_a, cls_b in ((cal.SimilarityTransform, co.SimilarityTransform),
                         (cal.EuclideanTransform, co.EuclideanTransform),
                         (cal.AffineTransform, co.AffineTransform)):
        M = np.array([[0.9, -0.1, 2.0], [0.1, 0.9, -3.0], [0, 0, 1]])
        dst = cal.matrix_transform(src, M) + rng.standard_normal((15, 2)) * 0.1
        ma, _ = cal.ransac((src, dst), cls_a, 2, 0.5, max_trials=500)
        mb, _ = co.ransac((src, dst), cls_b, 2, 0.5, max_trials=500)
        np.testing.assert_array_equal(ma.params, mb.params)
    pts = np.column_stack([np.arange(30), np.r_[np.full(20, 5.0), np.full(10, 90.0)] + rng.random(30)])
    np.testing.assert_array_equal(cal.kmeans2_labels(pts), co.kmeans2_labels(pts))


def test_keep_angles_equal_the_full_filter():
    """The extreme-shift filter keeps exactly the angles the reference's
    full filter (every radius and grid shift) keeps."""
    g, settings = load_case(CASES[0])
    ic, rec, data, oracle = build(g, settings)
    ic.initialize_error_search_space()
    radii = np.mgrid[4.0:-0.5:-0.5] + ic.apertRadiusPixel
    for pos in [(0, 0), (40, -3), (-45, 44), (50, 50), (-60, 0), (10, 61)]:
        keep = ic._keep_angles(pos, radii)
        arcs = oracle.circular_arcs(pos, radii)
        assert bin(keep).count("1") == arcs.shape[3]
        ic.radiusScanRangeInit = radii
        np.testing.assert_array_equal(ic.generateCircularArcsVectorized(np.array(pos)), arcs)


def test_plot_and_sizes_are_refused():
    g, settings = load_case(CASES[0])
    ic, *_ = build(g, settings)
    ic.plot = True
    with pytest.raises(NotImplementedError):
        ic.runCalibration()


def test_calibrated_encoder_reaches_positions_after_reset():
    """As in the reference, the calibration rewrites the data's encoder; the
    reconstruction's positions follow after reset_positioncorrection()."""
    from ptylab_gb300 import ExperimentalData, Params, Reconstruction

    g, settings = load_case("affine_small")
    d = ExperimentalData(None, "FPM")
    d.ptychogram = g["ptychogram"].astype(np.float32)
    d.encoder = g["encoder"].copy()
    d.dxd = float(g["dxp"]) * 4.0
    d.magnification = 4.0
    d.zled = float(g["zled"])
    d.wavelength = float(g["wavelength"])
    d.NA = float(g["NA_in"])
    d._setData()
    rec = Reconstruction(d, Params(), No=int(g["No"]))
    np.testing.assert_array_equal(rec.positions, g["positions"])
    ic = cal.IlluminationCalibration(rec, d)
    for k, v in settings.items():
        setattr(ic, k, v)
    ic._dev = NumpyDevice(co.CalibrationOracle(rec.Np, rec.No, rec.dxp, rec.wavelength, rec.NA, **settings))
    ic.runCalibration()
    np.testing.assert_allclose(d.encoder, g["encoder_out"], rtol=0, atol=1e-15)
    np.testing.assert_array_equal(rec.positions, g["positions"])  # encoder_corrected untouched
    rec.reset_positioncorrection()
    assert not np.array_equal(rec.positions, g["positions"])


def test_refused_sizes_and_plotting():
    g, settings = load_case(CASES[0])
    ic, rec, data, oracle = build(g, settings)
    with pytest.raises(NotImplementedError):
        ic.plotCalibration(None, None, None)
    ic.img_size = 96
    with pytest.raises(NotImplementedError):
        ic._fourier(np.zeros((2, 96, 96), np.float32))


def test_public_steps_take_host_arrays():
    """PtyLab's own callers pass NumPy arrays to the two search steps."""
    g, settings = load_case("affine_small")
    ic, rec, data, oracle = build(g, settings)
    frames = g["ptychogram"].astype(np.float32)
    FT = oracle.convertToFourierSpace(frames)  # windows frames in place
    bf = g["brightfield"]
    init = g["positions"] - int(g["No"]) // 2 + int(g["Np"]) // 2
    m, fitted = ic.findPositionCalibrationMatrix(frames[bf], FT[bf], init[bf])
    np.random.seed(1234)
    oracle.run(g["ptychogram"].astype(np.float32), g["positions"])
    np.testing.assert_array_equal(ic.calibrated_positions, oracle.calibrated_positions)
    old, new = ic.findCalibratedRadius(frames[bf], FT[bf], init[bf])
    assert old == pytest.approx(ic.apertRadiusPixel_init) and new > 0
