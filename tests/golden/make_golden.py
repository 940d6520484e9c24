"""Record golden fixtures by running the PtyLab.py reference's own NumPy path.

Usage (needs the reference source tree; run where it is present)::

    python tests/golden/make_golden.py /path/to/PtyLab.py

What it writes, all under ``tests/golden/``:

* ``reg_<name>.npz`` -- the nine configurations of the reference's
  engine regression suite (``tests/regression/test_engine_regression.py:47-57``)
  on the dataset of ``tests/regression/conftest.py:22-51`` rebuilt in NumPy.
  Before writing, each result is checked against the reference's own committed
  golden (``tests/regression/data/<name>.npz``); the script aborts unless the
  relative Frobenius error is exactly 0, so these fixtures are the reference's
  goldens reproduced, with the inputs stored beside them.
* ``prop_<name>.npz`` -- forward/back propagation of the seeded initial probe
  for all eight propagators, three wavelengths for the polychrome ones
  (``tests/regression/test_propagator_regression.py:27-82``), likewise checked
  against ``propagator_<name>.npz``.
* ``scan_<name>.npz`` -- cases the regression dataset cannot exercise (its 16
  frames all round to one pixel position): a Fermat-spiral CPM scan with
  random position order, mPIE momentum, mqNewton (ADAM, NADAM, plain
  momentum), mixed states, orthogonalisation, fftshiftSwitch, Fresnel/ASP,
  multislice, and an FPM LED-array scan with 'NA' order and probeBoundary.
  These are outputs of the unmodified reference.

``--only NAME [NAME ...]`` rewrites just those fixtures (file stems such as
``scan_mqnewton_adam``); the others are left untouched.

Every fixture stores its inputs (ptychogram, encoder, geometry scalars, the
seeded initial object/probe, pixel positions) and outputs (object, probe, error
curve, errorAtPos) so the tests need neither the reference nor h5py.
"""

from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

SEED = 20240607  # tests/regression/test_engine_regression.py:41


# ----------------------------------------------------------------------------
# datasets
# ----------------------------------------------------------------------------
def regression_dataset(nd=32, grid=4, seed=SEED):
    """NumPy rebuild of tests/regression/conftest.py:22-51 (h5py stores encoder as float32)."""
    rng = np.random.default_rng(seed)
    n_frames = grid * grid
    step = 3e-6
    coords = (np.arange(grid) - (grid - 1) / 2) * step
    yy, xx = np.meshgrid(coords, coords, indexing="ij")
    encoder = np.stack([yy.ravel(), xx.ravel()], axis=1)
    encoder = encoder + rng.normal(0, step / 50, encoder.shape)
    field = rng.random((n_frames, nd, nd))
    spectrum = np.fft.fftshift(np.fft.fft2(field), axes=(-2, -1))
    ky = np.fft.fftshift(np.fft.fftfreq(nd))
    mask = (ky[:, None] ** 2 + ky[None, :] ** 2) < 0.25**2
    pty = np.abs(np.fft.ifft2(np.fft.ifftshift(spectrum * mask, axes=(-2, -1)))) ** 2
    pty = (pty / pty.max()).astype(np.float32)
    return dict(
        operationMode="CPM",
        ptychogram=pty,
        encoder=encoder.astype(np.float32),
        dxd=75e-6,
        zo=0.05,
        wavelength=632.8e-9,
        entrancePupilDiameter=400e-6,
    )


def _smooth_field(rng, n, sigma):
    k = np.fft.fftfreq(n)
    g = np.exp(-2 * (np.pi * sigma) ** 2 * (k[:, None] ** 2 + k[None, :] ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(rng.standard_normal((n, n))) * g))
    f -= f.min()
    return f / max(f.max(), 1e-30)


def fermat_scan_dataset(nd=32, n_pos=24, step_px=4.0, seed=7):
    """A small CPM Fermat-spiral scan simulated with the centred Fraunhofer model."""
    rng = np.random.default_rng(seed)
    wavelength, zo, dxd = 632.8e-9, 0.05, 75e-6
    dxp = wavelength * zo / (nd * dxd)
    golden = np.pi * (3 - np.sqrt(5))
    i = np.arange(n_pos)
    r = step_px * np.sqrt(i) * 0.9
    th = i * golden
    enc_px = np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
    encoder = (enc_px * dxp).astype(np.float32)
    no = int(2 * np.ceil(np.abs(enc_px).max()) + 2 * nd + 2)
    obj = (0.7 + 0.3 * _smooth_field(rng, no, 3.0)) * np.exp(1j * np.pi * _smooth_field(rng, no, 3.0))
    yy, xx = np.mgrid[:nd, :nd] - nd / 2
    rad = nd / 5
    probe = (np.hypot(yy, xx) < rad) * np.exp(1j * 2 * np.pi * (yy**2 + xx**2) / rad**2)
    pos = np.round(enc_px).astype(int) + no // 2 - nd // 2
    pty = np.empty((n_pos, nd, nd), np.float32)
    for j, (py, px) in enumerate(pos):
        esw = obj[py : py + nd, px : px + nd] * probe
        spec = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(esw), norm="ortho"))
        pty[j] = np.abs(spec) ** 2
    pty = (pty / pty.max() * 1e4).astype(np.float32)
    pty = rng.poisson(pty).astype(np.float32)
    return dict(
        operationMode="CPM",
        ptychogram=pty,
        encoder=encoder,
        dxd=dxd,
        zo=zo,
        wavelength=wavelength,
        entrancePupilDiameter=2 * rad * dxp,
    )


def fpm_dataset(nd=32, grid=5, seed=11):
    """A small FPM LED-array scan: low-res images of a spectrum patch times a circular pupil."""
    rng = np.random.default_rng(seed)
    wavelength, dxd, mag, zled, pitch, na = 625e-9, 6.5e-6, 4.0, 0.08, 4e-3, 0.1
    dxp = dxd / mag
    c = (np.arange(grid) - (grid - 1) / 2) * pitch
    yy, xx = np.meshgrid(c, c, indexing="ij")
    encoder = np.stack([yy.ravel(), xx.ravel()], axis=1)
    conv = -(1 / wavelength) * dxp * nd
    shift = np.round(conv * encoder / np.sqrt(encoder[:, 0] ** 2 + encoder[:, 1] ** 2 + zled**2)[..., None])
    no = int(2 * np.abs(shift).max() + nd + 8)
    no += no % 2
    obj = (0.6 + 0.4 * _smooth_field(rng, no, 2.0)) * np.exp(1j * 2 * _smooth_field(rng, no, 2.0))
    spectrum = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(obj), norm="ortho"))
    pupil_d = 2 * dxp**2 * nd * na / wavelength
    x = np.linspace(-nd / 2, nd / 2, nd) * dxp
    X, Y = np.meshgrid(x, x)
    pupil = (X**2 + Y**2) < (pupil_d / 2) ** 2
    pos = (shift + no // 2 - nd // 2).astype(int)
    pty = np.empty((grid * grid, nd, nd), np.float32)
    for j, (py, px) in enumerate(pos):
        img = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(spectrum[py : py + nd, px : px + nd] * pupil), norm="ortho"))
        pty[j] = np.abs(img) ** 2
    pty = (pty / pty.max() * 5e3).astype(np.float32)
    pty = rng.poisson(pty).astype(np.float32)
    return dict(
        operationMode="FPM",
        ptychogram=pty,
        encoder=encoder,
        dxd=dxd,
        zled=zled,
        wavelength=wavelength,
        magnification=mag,
        NA=na,
        No=no,
    )


# ----------------------------------------------------------------------------
# running the reference
# ----------------------------------------------------------------------------
def _experimental_data(ref, d):
    ExperimentalData = ref["ExperimentalData"]
    data = ExperimentalData(None, d["operationMode"])
    keys = ["ptychogram", "encoder", "dxd", "wavelength"]
    if d["operationMode"] == "CPM":
        keys += ["zo", "entrancePupilDiameter"]
        data.spectralDensity = None
        data.theta = None
        data.emptyBeam = None
    else:
        keys += ["zled", "magnification", "NA"]
        data.entrancePupilDiameter = None
    for k in keys:
        setattr(data, k, d[k])
    data._setData()
    return data


def run_case(ref, d, case):
    """Run one configuration through the reference; return (inputs, outputs)."""
    np_ = np
    data = _experimental_data(ref, d)
    params = ref["Params"]()
    params.gpuSwitch = False
    params.propagatorType = case.get("propagator", "Fraunhofer")
    params.positionOrder = case.get("order", "sequential")
    params.fftshiftSwitch = case.get("fftshift", False)
    for k, v in case.get("params", {}).items():
        setattr(params, k, v)
    extra_inputs = {}
    if case.get("W"):
        # experimentalData.W for FourierMaskSwitch: a detector-plane disc
        n = d["ptychogram"].shape[-1]
        yy, xx = np.mgrid[:n, :n] - n / 2
        data.W = (np.hypot(yy, xx) < 0.4 * n).astype(np.float32)
        extra_inputs["W"] = data.W.copy()
    if case.get("intensityScaling"):
        # the fluctuation constraint writes params.intensityScaling, which
        # Params never creates (BaseEngine.py:931): the caller provides it
        params.intensityScaling = np.ones(d["ptychogram"].shape[0])
        extra_inputs["intensityScaling"] = params.intensityScaling.copy()
    if "No" in d:
        # the reconstruction derives No from the scan unless it is set first
        Reconstruction = ref["Reconstruction"]
        Reconstruction.No = d["No"]
    rec = ref["Reconstruction"](data, params)
    if "No" in d:
        del ref["Reconstruction"].No
        rec.No = d["No"]
    nl, nos, nps, nsl = case.get("modes", (1, 1, 1, 1))
    rec.nlambda, rec.nosm, rec.npsm, rec.nslice = nl, nos, nps, nsl
    if nl > 1:
        # tests/regression/test_engine_regression.py:78-80
        base = float(np.atleast_1d(rec.wavelength)[0])
        rec.spectralDensity = base * np.linspace(0.98, 1.02, nl)
        extra_inputs["spectralDensity"] = np.asarray(rec.spectralDensity, dtype=np.float64).copy()
    if nsl > 1:
        rec.dz = case.get("dz", 1e-4)
        rec.refrIndex = 1.0
    np_.random.seed(SEED)
    rec.initializeObjectProbe()
    if case.get("intensity_mask"):
        # reconstruction.intensity_mask for params.intensityMask: 1 inside, 0.5 on a ring, 0 in one corner
        n = rec.Np
        yy, xx = np.mgrid[:n, :n] - n / 2
        r = np.hypot(yy, xx)
        m = np.where(r < 0.35 * n, 1.0, 0.5).astype(np.float32)
        m[: n // 8, : n // 8] = 0.0
        rec.intensity_mask = m
        extra_inputs["intensity_mask"] = m.copy()
    init_object = rec.object.copy()
    init_probe = rec.probe.copy()
    engine = getattr(ref["Engines"], case["engine"])(rec, data, params, ref["DummyMonitor"]())
    engine.numIterations = case["iters"]
    for k, v in case.get("engine_attrs", {}).items():
        setattr(engine, k, v)
    if case.get("engine_attrs", {}).get("momentum_method") == "momentum":
        # mqNewton's plain-momentum method passes objectMomentum_v through
        # untouched, but reads it (mqNewton.py:188-199): give it one
        rec.objectMomentum_v = np.zeros_like(rec.object)
        rec.probeMomentum_v = np.zeros_like(rec.probe)
    positions = np.asarray(rec.positions).copy()
    # record the order each iteration used: 'NA' is np.argsort of LED distances,
    # whose tie order differs between NumPy's x86 and Arm sort kernels
    orders = []
    set_order = engine.setPositionOrder

    def recording_set_order():
        set_order()
        orders.append(np.asarray(engine.positionIndices).copy())

    engine.setPositionOrder = recording_set_order
    np_.random.seed(SEED)
    engine.reconstruct()
    inputs = dict(
        ptychogram=np.asarray(d["ptychogram"]),
        encoder=np.asarray(d["encoder"]),
        init_object=init_object,
        init_probe=init_probe,
        positions=positions,
        No=np.int64(rec.No),
        Np=np.int64(rec.Np),
        dxp=np.float64(rec.dxp),
        wavelength=np.float64(rec.wavelength),
        zo=np.float64(rec.zo),
        entrancePupilDiameter=np.float64(data.entrancePupilDiameter),
        energyAtPos=np.asarray(data.energyAtPos),
        orders=np.stack(orders),
        **extra_inputs,
    )
    if nsl > 1:
        inputs["dz"] = np.float64(rec.dz)
    outputs = dict(
        object=np.asarray(rec.object),
        probe=np.asarray(rec.probe),
        error=np.asarray(rec.error, dtype=np.float64),
        errorAtPos=np.asarray(rec.errorAtPos, dtype=np.float64),
    )
    if case["engine"] in ("mPIE", "mqNewton"):
        outputs["objectMomentum"] = np.asarray(rec.objectMomentum)
        outputs["probeMomentum"] = np.asarray(rec.probeMomentum)
    if case["engine"] == "mqNewton":
        outputs["objectBuffer"] = np.asarray(rec.objectBuffer)
        outputs["probeBuffer"] = np.asarray(rec.probeBuffer)
        if case.get("engine_attrs", {}).get("momentum_method", "ADAM") != "momentum":
            outputs["objectMomentum_v"] = np.asarray(rec.objectMomentum_v)
            outputs["probeMomentum_v"] = np.asarray(rec.probeMomentum_v)
    if case.get("keep_detector_error", False):
        outputs["detectorError"] = np.asarray(rec.detectorError, dtype=np.float64)
    if getattr(params, "backgroundModeSwitch", False):
        outputs["background"] = np.asarray(rec.background)
    if case.get("intensityScaling"):
        outputs["intensityScaling"] = np.asarray(params.intensityScaling)
    if getattr(params, "intensityConstraint", "standard") == "interferometric":
        outputs["reference"] = np.asarray(rec.reference)
    return inputs, outputs


# tests/regression/test_propagator_regression.py:27-36: wavelengths per propagator
PROPAGATORS = {
    "fraunhofer": 1, "fresnel": 1, "asp": 1, "scaledasp": 1, "identity": 1,
    "polychromeasp": 3, "scaledpolychromeasp": 3, "twosteppolychrome": 3,
}


def run_propagator(ref, d, prop):
    """tests/regression/test_propagator_regression.py:39-82."""
    nlambda = PROPAGATORS[prop]
    data = _experimental_data(ref, d)
    params = ref["Params"]()
    params.gpuSwitch = False
    params.propagatorType = prop
    params.fftshiftSwitch = False
    rec = ref["Reconstruction"](data, params)
    rec.nlambda = nlambda
    if nlambda > 1:
        base = float(np.atleast_1d(rec.wavelength)[0])
        rec.spectralDensity = base * np.linspace(0.98, 1.02, nlambda)
    np.random.seed(SEED)
    rec.initializeObjectProbe()
    Operators = ref["Operators"]
    field = rec.probe.copy()
    rec.esw = field
    _, fwd = Operators.object2detector(field, params, rec)
    rec.ESW = fwd
    _, back = Operators.detector2object(fwd, params, rec)
    inputs = dict(
        field=field,
        Np=np.int64(rec.Np),
        dxp=np.float64(rec.dxp),
        wavelength=np.float64(rec.wavelength),
        zo=np.float64(rec.zo),
        Lp=np.float64(rec.Lp),
        dxd=np.float64(rec.dxd),
        spectralDensity=np.atleast_1d(np.asarray(rec.spectralDensity, dtype=np.float64)),
        nlambda=np.int64(nlambda),
    )
    outputs = dict(
        forward=np.asarray(fwd),
        back=np.asarray(back),
        error=np.array([np.linalg.norm(fwd.ravel()), np.linalg.norm(back.ravel())]),
    )
    return inputs, outputs


REG_CONFIGS = {
    # tests/regression/test_engine_regression.py:47-57 (all nine rows)
    "epie_fraunhofer": dict(
        engine="ePIE", propagator="Fraunhofer", modes=(1, 1, 1, 1), iters=3, keep_detector_error=True
    ),
    "epie_asp": dict(engine="ePIE", propagator="ASP", modes=(1, 1, 1, 1), iters=3),
    "epie_fresnel": dict(engine="ePIE", propagator="Fresnel", modes=(1, 1, 1, 1), iters=3),
    "epie_mixed_state": dict(engine="ePIE", propagator="Fraunhofer", modes=(1, 2, 3, 1), iters=3),
    "epie_polychrome": dict(engine="ePIE", propagator="polychromeASP", modes=(3, 1, 1, 1), iters=2),
    "mpie_single": dict(engine="mPIE", propagator="Fraunhofer", modes=(1, 1, 1, 1), iters=3),
    "mpie_mixed_state": dict(engine="mPIE", propagator="Fraunhofer", modes=(1, 2, 3, 1), iters=3),
    "qnewton_single": dict(engine="qNewton", propagator="Fraunhofer", modes=(1, 1, 1, 1), iters=3),
    "e3pie_multislice": dict(engine="e3PIE", propagator="Fraunhofer", modes=(1, 1, 1, 3), iters=2),
}

SCAN_CONFIGS = {
    # several wavelengths (tests/regression/test_engine_regression.py:78-80 spectral density)
    "qnewton_polychrome": dict(engine="qNewton", propagator="polychromeASP", modes=(3, 1, 2, 1), iters=3),
    "mpie_polychrome": dict(engine="mPIE", propagator="polychromeASP", modes=(2, 2, 1, 1), iters=3, order="random"),
    "epie_random": dict(engine="ePIE", order="random", iters=4, keep_detector_error=True),
    "epie_fftshift": dict(engine="ePIE", order="random", fftshift=True, iters=3),
    "epie_fresnel": dict(engine="ePIE", propagator="Fresnel", iters=3),
    "epie_asp": dict(engine="ePIE", propagator="ASP", iters=3),
    "mpie_mixed_random": dict(engine="mPIE", order="random", modes=(1, 1, 2, 1), iters=5),
    "mpie_objmodes": dict(engine="mPIE", modes=(1, 2, 2, 1), iters=3),
    "mpie_orth": dict(
        engine="mPIE",
        order="random",
        modes=(1, 1, 3, 1),
        iters=4,
        params=dict(orthogonalizationSwitch=True, orthogonalizationFrequency=2),
    ),
    "qnewton": dict(engine="qNewton", order="random", iters=3),
    "e3pie": dict(engine="e3PIE", modes=(1, 1, 1, 3), iters=3, dz=2e-4),
    "e3pie_asp": dict(engine="e3PIE", propagator="ASP", modes=(1, 1, 1, 2), iters=2, dz=2e-4),
    "mqnewton_adam": dict(engine="mqNewton", order="random", iters=3),
    "mqnewton_nadam_orth": dict(
        engine="mqNewton",
        order="random",
        modes=(1, 1, 2, 1),
        iters=4,
        engine_attrs=dict(momentum_method="NADAM"),
        params=dict(orthogonalizationSwitch=True, orthogonalizationFrequency=2),
    ),
    "mqnewton_momentum": dict(engine="mqNewton", iters=3, engine_attrs=dict(momentum_method="momentum")),
    # mqNewton over three wavelengths: qNewton's steps summed over them
    # (mqNewton.py:226-251), the adaptive momentum on every wavelength's copy
    "mqnewton_polychrome": dict(engine="mqNewton", order="random", modes=(3, 1, 2, 1), iters=3),
    # intensity-projection switches (BaseEngine.py:870-1012, 1805-1822)
    # the unsquared constraints need an initial probe of the data's power
    "epie_poission": dict(
        engine="ePIE", order="random", iters=3,
        params=dict(intensityConstraint="poission", probePowerCorrectionSwitch=True),
    ),
    "mpie_exponential_denoise": dict(
        engine="mPIE", iters=3, params=dict(intensityConstraint="exponential", adaptiveDenoisingSwitch=True)
    ),
    "epie_background_fmask": dict(
        engine="ePIE", order="random", iters=3, W=True, keep_detector_error=True,
        params=dict(backgroundModeSwitch=True, FourierMaskSwitch=True),
    ),
    "epie_fluctuation": dict(
        engine="ePIE", iters=3, intensityScaling=True,
        params=dict(intensityConstraint="fluctuation", probePowerCorrectionSwitch=True),
    ),
    "epie_intensity_mask": dict(engine="ePIE", iters=3, intensity_mask=True, params=dict(intensityMask=True)),
    # the interferometric constraint: a detector-plane reference field,
    # updated at every position (BaseEngine.py:371-374, 883-891, 975-982)
    "epie_interferometric": dict(engine="ePIE", iters=3, params=dict(intensityConstraint="interferometric")),
    "mpie_interferometric_modes": dict(
        engine="mPIE", modes=(1, 1, 2, 1), iters=3, params=dict(intensityConstraint="interferometric")
    ),
    # ... uncentred transforms (no centring sign on the field), Fresnel, and
    # three wavelengths (one field per wavelength and mode)
    "qnewton_interferometric_fftshift": dict(
        engine="qNewton", fftshift=True, iters=3, params=dict(intensityConstraint="interferometric")
    ),
    "epie_interferometric_fresnel": dict(
        engine="ePIE", propagator="Fresnel", iters=3, params=dict(intensityConstraint="interferometric")
    ),
    "epie_interferometric_polychrome": dict(
        engine="ePIE", modes=(3, 1, 1, 1), iters=3, params=dict(intensityConstraint="interferometric")
    ),
    "epie_asp_denoise_background": dict(
        engine="ePIE", propagator="ASP", iters=3, params=dict(adaptiveDenoisingSwitch=True, backgroundModeSwitch=True)
    ),
    "qnewton_savememory_background": dict(
        engine="qNewton", iters=3, W=True, params=dict(saveMemory=True, backgroundModeSwitch=True, FourierMaskSwitch=True)
    ),
    # e3PIE's detector projection is BaseEngine's, every switch included (e3PIE.py:118)
    "e3pie_exponential_fmask": dict(
        engine="e3PIE", modes=(1, 1, 1, 3), iters=3, dz=2e-4, order="random", W=True, keep_detector_error=True,
        params=dict(intensityConstraint="exponential", FourierMaskSwitch=True),
    ),
    "e3pie_background_denoise_modes": dict(
        engine="e3PIE", modes=(1, 1, 2, 2), iters=3, dz=2e-4,
        params=dict(backgroundModeSwitch=True, adaptiveDenoisingSwitch=True),
    ),
    "e3pie_fluctuation": dict(
        engine="e3PIE", modes=(1, 1, 1, 2), iters=3, dz=2e-4, intensityScaling=True,
        params=dict(intensityConstraint="fluctuation", probePowerCorrectionSwitch=True),
    ),
    "e3pie_asp_exponential_mask": dict(
        engine="e3PIE", propagator="ASP", modes=(1, 1, 1, 2), iters=2, dz=2e-4, intensity_mask=True,
        params=dict(intensityConstraint="exponential", intensityMask=True),
    ),
}

FPM_CONFIGS = {
    "qnewton_fpm": dict(engine="qNewton", order="NA", iters=3, params=dict(probeBoundary=True)),
    "mpie_fpm": dict(engine="mPIE", order="NA", iters=3, params=dict(probeBoundary=True)),
    # the FPM example's engine (example_scripts/exampleReconstructionFPM.py:66-75)
    "mqnewton_nadam_fpm": dict(
        engine="mqNewton", order="NA", iters=3, engine_attrs=dict(momentum_method="NADAM"),
        params=dict(probeBoundary=True),
    ),
    # ... with the example's adaptive denoising (exampleReconstructionFPM.py:54-60)
    "mqnewton_nadam_fpm_denoise": dict(
        engine="mqNewton", order="NA", iters=3, engine_attrs=dict(momentum_method="NADAM"),
        params=dict(probeBoundary=True, adaptiveDenoisingSwitch=True),
    ),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference", help="path to the PtyLab.py source tree")
    ap.add_argument("--out", default=str(HERE))
    ap.add_argument("--only", nargs="*", default=None, help="fixture stems to (re)write")
    args = ap.parse_args()
    wanted = (lambda stem: True) if not args.only else (lambda stem: stem in args.only)

    from refload import load_reference

    load_reference(args.reference)
    from PtyLab import Engines
    from PtyLab.ExperimentalData.ExperimentalData import ExperimentalData
    from PtyLab.Monitor.Monitor import DummyMonitor
    from PtyLab.Operators import Operators
    from PtyLab.Params.Params import Params
    from PtyLab.Reconstruction.Reconstruction import Reconstruction

    ref = dict(
        Engines=Engines,
        ExperimentalData=ExperimentalData,
        DummyMonitor=DummyMonitor,
        Operators=Operators,
        Params=Params,
        Reconstruction=Reconstruction,
    )
    out = Path(args.out)
    gold = Path(args.reference) / "tests" / "regression" / "data"

    def rel(a, b):
        return float(np.linalg.norm((np.asarray(a) - b).ravel()) / max(np.linalg.norm(np.ravel(b)), 1e-30))

    def save(path, meta, inputs, outputs):
        arrs = {f"in_{k}": v for k, v in inputs.items()}
        arrs.update({f"out_{k}": v for k, v in outputs.items()})
        for k, v in meta.items():
            arrs[f"meta_{k}"] = np.asarray(v)
        np.savez_compressed(path, **arrs)

    d = regression_dataset()
    for name, case in REG_CONFIGS.items():
        if not wanted(f"reg_{name}"):
            continue
        inputs, outputs = run_case(ref, d, case)
        g = np.load(gold / f"{name}.npz")
        for key in g.files:
            e = rel(outputs[key], g[key])
            if e != 0.0:
                raise SystemExit(f"{name}: {key} differs from the reference golden by {e:.3e}")
        save(out / f"reg_{name}.npz", _meta(case, d), inputs, outputs)
        print(f"reg_{name}: matches {gold.name}/{name}.npz exactly")

    for prop in PROPAGATORS:
        if not wanted(f"prop_{prop}"):
            continue
        inputs, outputs = run_propagator(ref, d, prop)
        g = np.load(gold / f"propagator_{prop}.npz")
        for key in g.files:
            e = rel(outputs[key], g[key])
            # the fields must be bit-identical; the stored norms may differ in
            # the last bit (np.linalg.norm's BLAS sums in its own order)
            if e > (2.3e-16 if key == "error" else 0.0):
                raise SystemExit(f"propagator {prop}: {key} differs by {e:.3e}")
        save(out / f"prop_{prop}.npz", dict(propagator=prop), inputs, outputs)
        print(f"prop_{prop}: matches propagator_{prop}.npz exactly")

    ds = fermat_scan_dataset()
    for name, case in SCAN_CONFIGS.items():
        if not wanted(f"scan_{name}"):
            continue
        inputs, outputs = run_case(ref, ds, case)
        save(out / f"scan_{name}.npz", _meta(case, ds), inputs, outputs)
        print(f"scan_{name}: recorded (error {outputs['error'][-1]:.5g})")

    df = fpm_dataset()
    for name, case in FPM_CONFIGS.items():
        if not wanted(f"scan_{name}"):
            continue
        inputs, outputs = run_case(ref, df, case)
        save(out / f"scan_{name}.npz", _meta(case, df), inputs, outputs)
        print(f"scan_{name}: recorded (error {outputs['error'][-1]:.5g})")


def _meta(case, d):
    nl, nos, nps, nsl = case.get("modes", (1, 1, 1, 1))
    params = dict(case.get("params", {}))
    return dict(
        engine=case["engine"],
        propagator=case.get("propagator", "Fraunhofer"),
        order=case.get("order", "sequential"),
        fftshift=bool(case.get("fftshift", False)),
        operationMode=d["operationMode"],
        modes=np.array([nl, nos, nps, nsl]),
        iters=case["iters"],
        seed=SEED,
        probeBoundary=bool(params.get("probeBoundary", False)),
        orthogonalizationSwitch=bool(params.get("orthogonalizationSwitch", False)),
        orthogonalizationFrequency=int(params.get("orthogonalizationFrequency", 10)),
        dxd=d["dxd"],
        zled=d.get("zled", 0.0),
        magnification=d.get("magnification", 0.0),
        NA=d.get("NA", 0.0),
        momentum_method=case.get("engine_attrs", {}).get("momentum_method", "ADAM"),
        intensityConstraint=params.get("intensityConstraint", "standard"),
        adaptiveDenoisingSwitch=bool(params.get("adaptiveDenoisingSwitch", False)),
        backgroundModeSwitch=bool(params.get("backgroundModeSwitch", False)),
        FourierMaskSwitch=bool(params.get("FourierMaskSwitch", False)),
        intensityMask=bool(params.get("intensityMask", False)),
        saveMemory=bool(params.get("saveMemory", False)),
        probePowerCorrectionSwitch=bool(params.get("probePowerCorrectionSwitch", False)),
    )


if __name__ == "__main__":
    os.environ.setdefault("TQDM_DISABLE", "1")
    main()
