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


def simulate_cpm(spec: ScanSpec):
    """Return (ptychogram float32, encoder metres, true object, true probe, dxp);
    the true probe is scaled to the photon count of the intensities."""
    rng = np.random.default_rng(spec.seed)
    Np, No = spec.Np, spec.No
    dxp = spec.wavelength * spec.zo / (Np * spec.dxd)
    R = spec.probe_radius_fraction * Np
    step = spec.step_fraction * 2 * R
    pos = fermat_spiral(spec.num_positions, step)
    span = No - Np - 2
    if np.abs(pos).max() * 2 > span:
        pos *= span / (2 * np.abs(pos).max())
    encoder = pos * dxp
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
