"""Seeded synthetic CPM/FPM scans with the shapes of the benchmark configurations.

No dataset ships with PtyLab's benchmarks (its bench_engines.py synthesises
random data too), so these stand in for measured data: a Fermat-spiral scan
over a Gaussian-random-field object, a circular probe with defocus phase (or
orthogonal Hermite-Gauss modes), Fraunhofer intensities scaled to a peak
photon count with Poisson noise.  Forward model: I = sum_modes |fft2c(O_patch * P)|^2,
the model the engines invert (PtyLab/Engines/BaseEngine.py:870-1012).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .ExperimentalData import ExperimentalData
from .Params import Params
from .Reconstruction import Reconstruction


def fft2c(x):
    ax = (-2, -1)
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(x, axes=ax), norm="ortho"), axes=ax)


def gaussian_random_field(rng, n, sigma_px):
    """Smooth field in [0, 1]: white noise low-passed by a Gaussian of sigma_px pixels."""
    k = np.fft.fftfreq(n)
    g = np.exp(-2 * (np.pi * sigma_px) ** 2 * (k[:, None] ** 2 + k[None, :] ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(rng.standard_normal((n, n))) * g))
    f -= f.min()
    return f / max(f.max(), 1e-30)


def fermat_spiral(n, step_px):
    """n points on a Fermat spiral whose nearest-neighbour spacing is about step_px."""
    golden = np.pi * (3 - np.sqrt(5))
    i = np.arange(n)
    r = step_px * np.sqrt(i) * 0.55
    return np.stack([r * np.cos(i * golden), r * np.sin(i * golden)], axis=1)


def hermite_gauss_modes(Np, waist_px, n_modes, powers):
    yy, xx = np.mgrid[:Np, :Np] - Np / 2
    u, v = xx / waist_px, yy / waist_px
    herm = [lambda t: np.ones_like(t), lambda t: 2 * t, lambda t: 4 * t**2 - 2, lambda t: 8 * t**3 - 12 * t]
    orders = [(0, 0), (1, 0), (0, 1), (1, 1), (2, 0), (0, 2), (2, 1), (1, 2)]
    modes = []
    for m in range(n_modes):
        a, b = orders[m]
        f = herm[a](u) * herm[b](v) * np.exp(-(u**2 + v**2) / 2)
        f = f / np.sqrt(np.sum(np.abs(f) ** 2)) * np.sqrt(powers[m])
        modes.append(f.astype(np.complex128))
    return np.stack(modes)


@dataclass
class ScanSpec:
    Np: int = 64
    No: int = 256
    num_positions: int = 100
    npsm: int = 1
    step_fraction: float = 0.25
    probe_radius_fraction: float = 1 / 8
    photons: float = 1e5
    phase_max: float = np.pi
    amp_min: float = 1.0
    sigma_px: float = 4.0
    seed: int = 20240607
    wavelength: float = 632.8e-9
    zo: float = 0.05
    dxd: float = 75e-6
    # "fermat" (spiral) or "raster" (a square grid spanning the object, each
    # position moved by a seeded uniform jitter of up to jitter_px pixels)
    scan: str = "fermat"
    jitter_px: float = 0.0
    # multislice object: nslice weak-phase slices dz apart, the exit wave
    # carried between them by the angular spectrum (e3PIE.py:99-124)
    nslice: int = 1
    dz: float = 0.0


def _scan_pixels(spec: ScanSpec, rng, step):
    if spec.scan == "raster":
        n = int(round(np.sqrt(spec.num_positions)))
        if n * n != spec.num_positions:
            raise ValueError("a raster scan needs a square number of positions")
        span = spec.No - spec.Np - 2 - 2 * spec.jitter_px
        g = (np.arange(n) - (n - 1) / 2) * (span / max(n - 1, 1))
        yy, xx = np.meshgrid(g, g, indexing="ij")
        pos = np.stack([yy.ravel(), xx.ravel()], axis=1)
        return pos + rng.uniform(-spec.jitter_px, spec.jitter_px, pos.shape)
    pos = fermat_spiral(spec.num_positions, step)
    span = spec.No - spec.Np - 2
    if np.abs(pos).max() * 2 > span:
        pos *= span / (2 * np.abs(pos).max())
    return pos


def simulate_cpm(spec: ScanSpec):
    """Return (ptychogram float32, encoder metres, true object, true probe, dxp);
    the true probe is scaled to the photon count of the intensities."""
    rng = np.random.default_rng(spec.seed)
    Np, No = spec.Np, spec.No
    dxp = spec.wavelength * spec.zo / (Np * spec.dxd)
    R = spec.probe_radius_fraction * Np
    step = spec.step_fraction * 2 * R
    pos = _scan_pixels(spec, rng, step)
    encoder = pos * dxp
    if spec.nslice > 1:
        # weak-phase slices, amplitude 1, phase in [0, phase_max]
        obj = np.stack([np.exp(1j * spec.phase_max * gaussian_random_field(rng, No, spec.sigma_px))
                        for _ in range(spec.nslice)])
        from ._tables import multislice_tf

        H = np.fft.ifftshift(multislice_tf(spec.dz, spec.wavelength, 1.0, Np, Np * dxp))
    else:
        amp = spec.amp_min + (1 - spec.amp_min) * gaussian_random_field(rng, No, spec.sigma_px)
        phase = spec.phase_max * gaussian_random_field(rng, No, spec.sigma_px)
        obj = amp * np.exp(1j * phase)
    yy, xx = np.mgrid[:Np, :Np] - Np / 2
    r = np.hypot(yy, xx)
    if spec.npsm == 1:
        probe = ((r < R) * np.exp(1j * 2 * np.pi * (r / R) ** 2))[None]
    else:
        # Hermite-Gauss modes whose fundamental falls to 1/e in amplitude at
        # the pupil radius R, the footprint of the circular pupil guess
        powers = [1.0 / 2**m for m in range(spec.npsm)]
        probe = hermite_gauss_modes(Np, R / np.sqrt(2), spec.npsm, powers) * np.exp(1j * 2 * np.pi * (r / R) ** 2)
    rows_cols = np.round(encoder / dxp).astype(int) + No // 2 - Np // 2
    I = np.empty((spec.num_positions, Np, Np), np.float64)
    for j, (py, px) in enumerate(rows_cols):
        if spec.nslice > 1:
            w = obj[0, py : py + Np, px : px + Np] * probe
            for sl in range(1, spec.nslice):
                w = np.fft.ifft2(np.fft.fft2(w) * H) * obj[sl, py : py + Np, px : px + Np]
            I[j] = np.sum(np.abs(fft2c(w)) ** 2, axis=0)
            continue
        patch = obj[py : py + Np, px : px + Np]
        I[j] = np.sum(np.abs(fft2c(patch[None] * probe)) ** 2, axis=0)
    scale = spec.photons / I.max()
    I *= scale
    probe = probe * np.sqrt(scale)  # the probe that generates these intensities
    I = rng.poisson(I).astype(np.float32)
    return I, encoder, obj, probe, dxp


def cpm_problem(spec: ScanSpec, engine_seed: int = 20240607):
    """ExperimentalData, Params and a Reconstruction with seeded initial guesses for `spec`."""
    I, encoder, obj, probe, dxp = simulate_cpm(spec)
    d = ExperimentalData(None, "CPM")
    d.ptychogram = I
    d.encoder = encoder
    d.dxd = spec.dxd
    d.zo = spec.zo
    d.wavelength = spec.wavelength
    d.entrancePupilDiameter = 2 * spec.probe_radius_fraction * spec.Np * dxp * 1.2
    d._setData()
    p = Params()
    p.positionOrder = "sequential"
    rec = Reconstruction(d, p, No=spec.No)
    rec.npsm = spec.npsm
    if spec.nslice > 1:
        rec.nslice = spec.nslice
        rec.dz = spec.dz
        rec.refrIndex = 1.0
    np.random.seed(engine_seed)
    rec.initializeObjectProbe()
    return d, p, rec, obj, probe


@dataclass
class FPMSpec:
    """LED-array Fourier ptychography: grid x grid LEDs, low-res Np images of a
    No x No high-resolution spectrum (the object's centred Fourier transform)."""

    Np: int = 128
    No: int = 512
    grid: int = 15
    pitch: float = 4e-3
    zled: float = 80e-3
    wavelength: float = 625e-9
    dxd: float = 6.5e-6
    magnification: float = 4.0
    NA: float = 0.1
    photons: float = 5e4
    sigma_px: float = 4.0
    seed: int = 20240607
    # misalignment of the LED array the images are made with; the returned
    # encoder stays the nominal grid (what an illumination calibration fixes)
    led_rotation_deg: float = 0.0
    led_shift: tuple = (0.0, 0.0)
    true_NA: float | None = None
    # object contrast: amplitude 1 - amp_contrast * (1 - field), phase phase_scale * field
    amp_contrast: float = 0.5
    phase_scale: float = np.pi


def simulate_fpm(spec: FPMSpec):
    """Return (ptychogram float32, encoder metres, true object, pupil, dxp)."""
    rng = np.random.default_rng(spec.seed)
    Np, No = spec.Np, spec.No
    dxp = spec.dxd / spec.magnification
    c = (np.arange(spec.grid) - (spec.grid - 1) / 2) * spec.pitch
    yy, xx = np.meshgrid(c, c, indexing="ij")
    encoder = np.stack([yy.ravel(), xx.ravel()], axis=1)
    amp = 1.0 - spec.amp_contrast + spec.amp_contrast * gaussian_random_field(rng, No, spec.sigma_px)
    phase = spec.phase_scale * gaussian_random_field(rng, No, spec.sigma_px)
    obj = amp * np.exp(1j * phase)
    spectrum = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(obj), norm="ortho"))
    NA = spec.NA if spec.true_NA is None else spec.true_NA
    pupil_d = 2 * dxp**2 * Np * NA / spec.wavelength
    x = np.linspace(-Np / 2, Np / 2, Np) * dxp
    X, Y = np.meshgrid(x, x)
    pupil = (X**2 + Y**2) < (pupil_d / 2) ** 2
    conv = -(1 / spec.wavelength) * dxp * Np
    leds = encoder
    if spec.led_rotation_deg or any(spec.led_shift):
        t = np.deg2rad(spec.led_rotation_deg)
        rot = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
        leds = encoder @ rot.T + np.asarray(spec.led_shift, dtype=np.float64)
    shift = np.round(conv * leds / np.sqrt(leds[:, 0] ** 2 + leds[:, 1] ** 2 + spec.zled**2)[..., None])
    pos = (shift + No // 2 - Np // 2).astype(int)
    I = np.empty((len(pos), Np, Np), np.float64)
    for j, (py, px) in enumerate(pos):
        I[j] = np.abs(fft2c(spectrum[py : py + Np, px : px + Np] * pupil)) ** 2
    I *= spec.photons / I.max()
    I = rng.poisson(I).astype(np.float32)
    return I, encoder, obj, pupil, dxp


def fpm_problem(spec: FPMSpec, engine_seed: int = 20240607):
    """ExperimentalData, Params and a Reconstruction (FPM: 'upsampled' object,
    circular pupil) for `spec`, with PtyLab's FPM defaults ('NA' order,
    probeBoundary, PtyLab/__init__.py:54-55)."""
    I, encoder, obj, pupil, dxp = simulate_fpm(spec)
    d = ExperimentalData(None, "FPM")
    d.ptychogram = I
    d.encoder = encoder
    d.dxd = spec.dxd
    d.zled = spec.zled
    d.wavelength = spec.wavelength
    d.magnification = spec.magnification
    d.NA = spec.NA
    d._setData()
    p = Params()
    p.positionOrder = "NA"
    p.probeBoundary = True
    rec = Reconstruction(d, p, No=spec.No)
    np.random.seed(engine_seed)
    rec.initializeObjectProbe()
    return d, p, rec, obj, pupil


# ---------------------------------------------------------------- configurations
# The four benchmark workloads of the plain reconstruction loop, as engine
# name, scan description and iteration count.
#   C0  CPM ePIE, Fraunhofer, Np 64, No 256, 100 Fermat positions (~75 % overlap),
#       circular pupil of radius Np/8 with 2 pi of defocus at the rim, phase in
#       [0, pi], 1e5 photons; 20 iterations, beta 0.25, sequential order
#   C1  CPM mPIE, 4 Hermite-Gauss probe modes (powers 1 : 0.5 : 0.25 : 0.125),
#       Np 128, No 512, 400 Fermat positions (~70 % overlap), amplitude in
#       [0.6, 1], phase in [0, 2 pi], 1e6 photons; alpha = beta = 0.25,
#       friction 0.7, feedback 0.3, random order with momentum; 50 iterations
#   C2  multislice (e3PIE): 4 weak-phase slices (<= 0.3 rad) 10 um apart,
#       13.5 nm wavelength, 20 nm pixels, Np 256, No 768, 30 x 30 raster with
#       +-2 px jitter; 30 iterations
#   C3  FPM qNewton: 15 x 15 LEDs at 4 mm pitch, 80 mm away, 128 x 128 images
#       (6.5 um pixels, 4x magnification), NA 0.1, 625 nm, spectrum 512 x 512,
#       5e4 photons; 'NA' order, probeBoundary; 50 iterations
CONFIG_ENGINES = {"C0": "ePIE", "C1": "mPIE", "C2": "e3PIE", "C3": "qNewton"}
CONFIG_ITERATIONS = {"C0": 20, "C1": 50, "C2": 30, "C3": 50}


def config_spec(name: str, seed: int | None = None):
    """ScanSpec / FPMSpec of benchmark configuration `name` (C0 ... C3)."""
    kw = {} if seed is None else {"seed": seed}
    if name == "C0":
        return ScanSpec(**kw)
    if name == "C1":
        return ScanSpec(Np=128, No=512, num_positions=400, npsm=4, step_fraction=0.3, probe_radius_fraction=1 / 4,
                        photons=1e6, phase_max=2 * np.pi, amp_min=0.6, sigma_px=4.0, **kw)
    if name == "C2":
        return ScanSpec(Np=256, No=768, num_positions=900, scan="raster", jitter_px=2.0, probe_radius_fraction=0.2,
                        wavelength=13.5e-9, zo=0.05, dxd=13.5e-9 * 0.05 / (256 * 20e-9), photons=1e5,
                        phase_max=0.3, nslice=4, dz=10e-6, **kw)
    if name == "C3":
        return FPMSpec(**kw)
    raise ValueError(f"unknown configuration {name!r}")


def config_problem(name: str, seed: int | None = None, engine_seed: int = 20240607):
    """(engine name, ExperimentalData, Params, Reconstruction) of configuration
    `name` with seeded data and initial guesses, ready for
    ``getattr(Engines, engine)(rec, d, p, monitor)``."""
    spec = config_spec(name, seed)
    if name == "C3":
        d, p, rec, _, _ = fpm_problem(spec, engine_seed=engine_seed)
    else:
        d, p, rec, _, _ = cpm_problem(spec, engine_seed=engine_seed)
    if name == "C1":
        p.positionOrder = "random"
    return CONFIG_ENGINES[name], d, p, rec


def configure_engine(name: str, engine, iterations: int | None = None):
    """The configuration's engine scalars (mPIE: alpha 0.25 as C1 states; the
    other scalars are the engines' own defaults: beta 0.25 for ePIE / mPIE /
    e3PIE, friction 0.7, feedback 0.3; qNewton beta 1, reg 1)."""
    if name == "C1":
        engine.alphaObject = engine.alphaProbe = 0.25
    engine.numIterations = CONFIG_ITERATIONS[name] if iterations is None else iterations
    return engine
