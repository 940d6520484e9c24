"""Host-built propagation tables (double precision, rounded to complex64 on upload).

Same formulas as PtyLab's cached builders, evaluated once per geometry:
  * Fresnel chirp  Q = exp(i*pi/(lambda*z)*(x^2+y^2)), x = linspace(-Np/2, Np/2, Np)*dxp
    (PtyLab/Operators/_propagation_kernels.py:16-36)
  * band-limited angular-spectrum transfer function on the centred frequency
    grid f = arange(-N/2, N/2)/L, with the circular band limit
    f_max = L/(lambda*sqrt(L^2+4z^2)) and evanescent cut (PtyLab/Operators/Operators.py:631-684)
  * the scaled angular spectrum's chirps Q1 (source plane) and Q2 (Fourier
    plane) with their band limits (Operators.py:706-760)
"""

from __future__ import annotations

from functools import lru_cache

import numpy as np


@lru_cache(maxsize=32)
def fresnel_chirp(zo: float, wavelength: float, Np: int, dxp: float) -> np.ndarray:
    x = np.linspace(-Np / 2, Np / 2, int(Np)) * dxp
    X, Y = np.meshgrid(x, x)
    q = np.exp(1.0j * np.pi / (wavelength * zo) * (X**2 + Y**2))
    q.setflags(write=False)
    return q


@lru_cache(maxsize=32)
def angular_spectrum_tf(z: float, wavelength: float, N: int, L: float, bandlimit: bool = True) -> np.ndarray:
    az = abs(z)
    k = 2 * np.pi / wavelength
    f = np.arange(-N / 2, N / 2) / L
    Fx, Fy = np.meshgrid(f, f)
    f_max = L / (wavelength * np.sqrt(L**2 + 4 * az**2))
    window = (Fx**2 + Fy**2) < (2 * f_max / 2) ** 2
    arg = 1 - (Fx * wavelength) ** 2 - (Fy * wavelength) ** 2
    mask = (arg > 0) if bandlimit else np.ones_like(arg, dtype=bool)
    phase = k * az * np.sqrt(np.clip(arg, 0, np.inf))
    H = mask * (np.cos(phase) + 1j * np.sin(phase))
    if z < 0:
        H = H.conj()
    H = H * window
    H.setflags(write=False)
    return H


def asp_detector_tf(zo: float, wavelength: float, Np: int, Lp: float) -> np.ndarray:
    """The detector ASP transfer function as the engines use it: rounded to
    complex64 first (Operators.py:861-893), centred."""
    return angular_spectrum_tf(float(zo), float(wavelength), int(Np), float(Lp)).astype(np.complex64)


def multislice_tf(dz: float, wavelength: float, refr_index: float, Np: int, Lp: float) -> np.ndarray:
    """Slice-to-slice transfer function of e3PIE (e3PIE.py:62-69), centred, complex128."""
    return angular_spectrum_tf(float(dz), float(wavelength) / float(refr_index), int(Np), float(Lp))


@lru_cache(maxsize=32)
def scaled_asp_tables(z: float, wavelength: float, N: int, dx: float, dq: float):
    """(Q1, Q2) complex64 of the scaled angular spectrum from grid spacing dx
    to dq over z (the Fresnel-approximation method with band limits
    r1^2 < (lambda z / (2 dx (1 - m)))^2 and f^2 < (m / (2 z lambda df))^2,
    m = dq/dx, df = 1/(N dx)), evaluated in float64 and rounded as
    PtyLab stores them (Operators.py:954-988)."""
    k = 2 * np.pi / wavelength
    x1 = np.arange(-N // 2, N // 2) * dx
    X1, Y1 = np.meshgrid(x1, x1)
    r1sq = X1**2 + Y1**2
    f = np.arange(-N // 2, N // 2) / (N * dx)
    FX, FY = np.meshgrid(f, f)
    fsq = FX**2 + FY**2
    m = dq / dx
    q1 = np.exp(1.0j * k / 2 * (1 - m) / z * r1sq)
    q2 = np.exp(-1.0j * np.pi**2 * 2 * z / m / k * fsq)
    if m != 1:
        r_max = wavelength * z / (2 * dx * (1 - m))
        q1 = q1 * ((X1**2 + Y1**2) < r_max**2)
    f_max = m / (2 * z * wavelength * (1 / (N * dx)))
    q2 = q2 * ((FX**2 + FY**2) < f_max**2)
    q1, q2 = q1.astype(np.complex64), q2.astype(np.complex64)
    q1.setflags(write=False)
    q2.setflags(write=False)
    return q1, q2


def polychrome_asp_tf(zo: float, wavelengths: tuple, Np: int, Lp: float) -> np.ndarray:
    """One centred transfer function per wavelength, (nlambda, Np, Np) complex64
    (Operators.py:909-951)."""
    return np.stack([angular_spectrum_tf(float(zo), float(w), int(Np), float(Lp)) for w in wavelengths]).astype(
        np.complex64
    )


def two_step_polychrome_tables(zo: float, wavelengths: tuple, Np: int, Lp: float, dxp: float):
    """(transfer functions over zo*(1 - l0/l) per wavelength l, (nlambda, Np, Np);
    the Fresnel chirp of the first wavelength, (Np, Np)), complex64
    (Operators.py:1033-1077)."""
    l0 = float(wavelengths[0])
    tf = np.stack(
        [angular_spectrum_tf(float(zo) * (1 - l0 / float(w)), float(w), int(Np), float(Lp)) for w in wavelengths]
    )
    return tf.astype(np.complex64), fresnel_chirp(float(zo), l0, int(Np), float(dxp)).astype(np.complex64)
