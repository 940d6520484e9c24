"""Host-built propagation tables (double precision, rounded to complex64 on upload).

Same formulas as PtyLab's cached builders, evaluated once per geometry:
  * Fresnel chirp  Q = exp(i*pi/(lambda*z)*(x^2+y^2)), x = linspace(-Np/2, Np/2, Np)*dxp
    (PtyLab/Operators/_propagation_kernels.py:16-36)
  * band-limited angular-spectrum transfer function on the centred frequency
    grid f = arange(-N/2, N/2)/L, with the circular band limit
    f_max = L/(lambda*sqrt(L^2+4z^2)) and evanescent cut (PtyLab/Operators/Operators.py:631-684)
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
