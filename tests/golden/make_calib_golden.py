"""Golden fixtures for the FPM illumination calibration.

Test infrastructure only.  Simulates FPM scans whose LED array is misaligned
(``ptylab_gb300.simulate.simulate_fpm``: rotated, shifted, a wrong NA) and
runs the REFERENCE's ``IlluminationCalibration.runCalibration``
(PtyLab/Reconstruction/CalibrationFPM.py:830-919) on them.  scikit-image is
not installed here, so its routines the reference calls (``window``,
``gaussian``, ``ransac``, the transforms, ``matrix_transform``) are replaced
by the restatements in ``oracle/calib_oracle.py``; scikit-learn's KMeans and
SciPy's ``map_coordinates`` are the real ones.  Recorded per case: the
brightfield frames, every ``calculateRMSE`` decision, the calibrated
aperture radius and NA, the transform, the fitted positions and the updated
encoder, plus the Fourier-domain images of two frames.

    python tests/golden/make_calib_golden.py --reference <path of a PtyLab.py checkout>

Output: ``tests/golden/calib_<case>.npz``; each holds its own inputs.
"""

from __future__ import annotations

import argparse
import importlib
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT / "oracle"))

import calib_oracle as co  # noqa: E402

from ptylab_gb300.simulate import FPMSpec, simulate_fpm  # noqa: E402

CASES = {
    # default fit on a rotated and shifted LED array
    "similarity": dict(spec=dict(Np=128, No=512, grid=9, photons=1e5, amp_contrast=0.2, phase_scale=0.3 * np.pi,
                                 led_rotation_deg=1.5, led_shift=(7e-4, -5e-4)),
                       calib=dict()),
    # the reference example's settings: radius calibration and a translation
    # fit, the aperture given 8 % too small
    "translation_radius": dict(spec=dict(Np=128, No=512, grid=9, photons=1e5, amp_contrast=0.2,
                                         phase_scale=0.3 * np.pi, led_shift=(6e-4, 4e-4), NA=0.092, true_NA=0.1),
                               calib=dict(calibrateRadius=True, fit_mode="Translation")),
    # a small scan, affine fit
    "affine_small": dict(spec=dict(Np=64, No=256, grid=7, photons=1e5, amp_contrast=0.2, phase_scale=0.3 * np.pi,
                                   led_rotation_deg=-2.0, led_shift=(-4e-4, 3e-4)),
                         calib=dict(fit_mode="AffineTransform")),
}


def inputs(spec_kw):
    spec = FPMSpec(**spec_kw)
    I, enc, _, _, dxp = simulate_fpm(spec)
    conv = -(1 / spec.wavelength) * dxp * spec.Np
    pos = np.round(conv * enc / np.sqrt(enc[:, 0] ** 2 + enc[:, 1] ** 2 + spec.zled**2)[..., None])
    pos = (pos + spec.No // 2 - spec.Np // 2).astype(int)
    return spec, I, enc, dxp, pos


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    from refload import load_reference

    load_reference(args.reference)
    cal = importlib.import_module("PtyLab.Reconstruction.CalibrationFPM")
    cal.window = lambda kind, shape: co.hann_window(shape)
    cal.gaussian = lambda img, sigma, preserve_range=False: co.gaussian(img, sigma)
    cal.ransac = co.ransac
    cal.EuclideanTransform = co.EuclideanTransform
    cal.SimilarityTransform = co.SimilarityTransform
    cal.AffineTransform = co.AffineTransform
    cal.matrix_transform = co.matrix_transform
    cal.print = lambda *a, **k: None

    for name, case in CASES.items():
        spec, I, enc, dxp, pos = inputs(case["spec"])
        rec = types.SimpleNamespace(Np=spec.Np, No=spec.No, dxp=dxp, dxo=dxp, wavelength=spec.wavelength,
                                    NA=spec.NA, zled=spec.zled, positions=pos.copy())
        data = types.SimpleNamespace(ptychogram=I.copy(), encoder=enc.copy())
        ic = cal.IlluminationCalibration(rec, data)
        for k, v in case["calib"].items():
            setattr(ic, k, v)
        decisions = []
        orig = ic.calculateRMSE

        def logged(image, candidates, position, _orig=orig):
            ex, ey, edge = _orig(image, candidates, position)
            decisions.append([float(position[0]), float(position[1]), ex, ey, int(edge), len(candidates)])
            return ex, ey, edge

        ic.calculateRMSE = logged
        ft_probe = {}
        orig_ft = ic.convertToFourierSpace

        def ft_logged(p, _orig=orig_ft):
            ft = _orig(p)
            ft_probe["ft"] = ft[[0, len(ft) // 2]].copy()
            return ft

        ic.convertToFourierSpace = ft_logged
        np.random.seed(1234)
        m = ic.runCalibration()
        assert np.array_equal(I, np.round(I)) and I.min() >= 0  # Poisson counts: stored as integers
        out = dict(
            ptychogram=I.astype(np.uint32), encoder=enc, positions=pos, dxp=dxp, Np=spec.Np, No=spec.No, wavelength=spec.wavelength,
            NA_in=spec.NA, zled=spec.zled, calib_keys=np.array(list(case["calib"].keys())),
            calib_values=np.array([str(v) for v in case["calib"].values()]),
            brightfield=np.asarray(ic.brightfieldIndices), decisions=np.array(decisions),
            radius=ic.apertRadiusPixel, NA=rec.NA, entrancePupilDiameter=rec.entrancePupilDiameter,
            matrix=m.params, positionsFitted=ic.positionsFitted, encoder_out=data.encoder,
            ft_frames=ft_probe["ft"],
        )
        np.savez_compressed(HERE / f"calib_{name}.npz", **out)
        print(name, "brightfield", int(np.sum(out["brightfield"])), "decisions", len(decisions),
              "radius", round(float(out["radius"]), 3), "NA", out["NA"])


if __name__ == "__main__":
    main()
