"""CPU oracle for the per-position ptychography reconstruction loop.

TEST INFRASTRUCTURE ONLY.  This module restates, in NumPy, the algorithm of the
PtyLab.py reference (version 0.3.1) for the path the GB300 package accelerates:
the ePIE / mPIE / qNewton / mqNewton / e3PIE position loops, the standard intensity
projection, the Fraunhofer / Fresnel / ASP propagators, the error metrics, the
position order and the seeded initial guesses.  Only ``tests/``, the package's
``smoke()`` entry and ``bench.py``'s CPU-baseline leg may import it, and only as
the checker or the timed CPU baseline; the package never calls it.

Every function names the reference file:line it follows.  NumPy dtype
promotion is reproduced on purpose (complex64 state, float32 intensities, the
complex128 promotion of the Fresnel chirp and the multislice transfer
function), so that on the reference's golden datasets this restatement agrees
with the reference to the last bit; ``tests/test_oracle_golden.py`` pins that
against fixtures recorded from the reference itself.

Random numbers come from NumPy's legacy global generator exactly where the
reference draws them: ``np.random.shuffle`` of the position order
(``PtyLab/Engines/BaseEngine.py:646-653``) and mPIE's per-position momentum
draw ``np.random.rand(1) > 0.95`` (``PtyLab/Engines/mPIE.py:170``).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np


# ----------------------------------------------------------------------------
# transforms and propagators
# ----------------------------------------------------------------------------
def fft2c(x, fftshiftSwitch=False):
    """Unitary centred 2D DFT over the last two axes (PtyLab/utils/utils.py:12-28)."""
    if fftshiftSwitch:
        return np.fft.fft2(x, norm="ortho")
    ax = (-2, -1)
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(x, axes=ax), norm="ortho"), axes=ax)


def ifft2c(x, fftshiftSwitch=False):
    """Unitary centred inverse 2D DFT (PtyLab/utils/utils.py:31-47)."""
    if fftshiftSwitch:
        return np.fft.ifft2(x, norm="ortho")
    ax = (-2, -1)
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(x, axes=ax), norm="ortho"), axes=ax)


def circ(x, y, D):
    """Binary disc of diameter D (PtyLab/utils/utils.py:50-59)."""
    return (x**2 + y**2) < (D / 2) ** 2


def quad_phase(zo, wavelength, Np, dxp):
    """Fresnel chirp exp(i*pi/(lambda*z)*(x^2+y^2)), complex128, x from linspace
    (PtyLab/Operators/_propagation_kernels.py:16-36)."""
    x_p = np.linspace(-Np / 2, Np / 2, int(Np)) * dxp
    Xp, Yp = np.meshgrid(x_p, x_p)
    return np.exp(1.0j * np.pi / (wavelength * zo) * (Xp**2 + Yp**2))


def aspw_transfer_function(z, wavelength, N, L, bandlimit=True):
    """Band-limited angular-spectrum transfer function, complex128, centred frequency grid
    (PtyLab/Operators/Operators.py:631-684)."""
    a_z = abs(z)
    k = 2 * np.pi / wavelength
    X = np.arange(-N / 2, N / 2) / L
    Fx, Fy = np.meshgrid(X, X)
    f_max = L / (wavelength * np.sqrt(L**2 + 4 * a_z**2))
    W = np.array(circ(Fx, Fy, 2 * f_max))
    exponent = 1 - (Fx * wavelength) ** 2 - (Fy * wavelength) ** 2
    mask = exponent > 0
    if not bandlimit:
        mask = 0 * mask + 1
    exponent = np.clip(exponent, 0, np.inf)
    angle = k * a_z * np.sqrt(exponent)
    H = np.array(mask * (np.cos(angle) + 1j * np.sin(angle)))
    if z < 0:
        H = H.conj()
    return H * W


def scaled_asp_tables(z, wavelength, N, dx, dq):
    """Q1 (source-plane chirp) and Q2 (Fourier-plane chirp) of the scaled
    angular spectrum with its band limits (PtyLab/Operators/Operators.py:706-760,
    bandlimit=True), rounded to complex64 as the propagator stores them
    (Operators.py:954-988).  The expressions keep the reference's operation
    order so the float64 values, and hence their complex64 rounding, agree."""
    k = 2 * np.pi / wavelength
    x1 = np.arange(-N // 2, N // 2) * dx
    X1, Y1 = np.meshgrid(x1, x1)
    r1sq = X1**2 + Y1**2
    f = np.arange(-N // 2, N // 2) / (N * dx)
    FX, FY = np.meshgrid(f, f)
    fsq = FX**2 + FY**2
    m = dq / dx
    Q1 = np.exp(1.0j * k / 2 * (1 - m) / z * r1sq)
    Q2 = np.exp(-1.0j * np.pi**2 * 2 * z / m / k * fsq)
    if m != 1:
        r1sq_max = wavelength * z / (2 * dx * (1 - m))
        Q1 = Q1 * np.array(circ(X1, Y1, 2 * r1sq_max))
    fsq_max = m / (2 * z * wavelength * (1 / (N * dx)))
    Q2 = Q2 * np.array(circ(FX, FY, 2 * fsq_max))
    return Q1.astype(np.complex64), Q2.astype(np.complex64)


def _per_wavelength(tables):
    """Stack per-wavelength Np x Np tables as (nlambda, 1, 1, 1, Np, Np): they
    broadcast over modes and slices as the reference's (nlambda, nosm, npsm,
    1, Np, Np) copies do."""
    return np.stack(tables)[:, None, None, None]


def polychrome_asp_tf(g):
    """(Operators.py:909-951): one centred transfer function per wavelength of
    spectralDensity, complex128 on the CPU path (no dtype given there)."""
    return _per_wavelength([aspw_transfer_function(g.zo, lam, g.Np, g.Lp) for lam in g.spectralDensity])


def scaled_polychrome_asp_tables(g):
    """(Operators.py:990-1030): scaledASP's Q1, Q2 per wavelength, complex64."""
    q = [scaled_asp_tables(g.zo, lam, g.Np, g.dxo, g.dxd) for lam in g.spectralDensity]
    return _per_wavelength([a for a, _ in q]), _per_wavelength([b for _, b in q])


def two_step_polychrome_tables(g):
    """(Operators.py:1033-1077): transfer functions over zo*(1 - l0/l) at each
    wavelength l (complex128) and the Fresnel chirp of the first wavelength."""
    sd = g.spectralDensity
    tf = _per_wavelength([aspw_transfer_function(g.zo * (1 - sd[0] / lam), lam, g.Np, g.Lp) for lam in sd])
    return tf, quad_phase(g.zo, sd[0], g.Np, g.dxp)


def asp_transfer_function(nosm, npsm, Np, zo, wavelength, Lp):
    """ASP detector transfer function as the engines use it: complex64, shape
    (1, nosm, npsm, 1, Np, Np) (PtyLab/Operators/Operators.py:861-893)."""
    tf = aspw_transfer_function(zo, wavelength, Np, Lp)
    return np.array([[[[tf] for _ in range(npsm)] for _ in range(nosm)]], dtype=np.complex64)


@dataclass
class Geometry:
    Np: int
    No: int
    dxp: float
    wavelength: float
    zo: float
    nlambda: int = 1
    nosm: int = 1
    npsm: int = 1
    nslice: int = 1
    dz: float = 0.0
    refrIndex: float = 1.0
    dxd: float = 0.0
    spectralDensity: tuple = ()

    @property
    def Lp(self):
        return self.Np * self.dxp

    @property
    def dxo(self):
        return self.dxp

    @property
    def xp(self):
        return np.linspace(-self.Np / 2, self.Np / 2, int(self.Np)) * self.dxp

    @property
    def Xp(self):
        return np.meshgrid(self.xp, self.xp)[0]

    @property
    def Yp(self):
        return np.meshgrid(self.xp, self.xp)[1]


def object2detector(fields, propagator, fftshift, g: Geometry):
    """Forward propagators (PtyLab/Operators/Operators.py:27-50, 77-113, 155-215, 576-584)."""
    p = propagator.lower()
    if p == "fraunhofer":
        return fft2c(fields, fftshift)
    if p == "fresnel":
        return fft2c(fields * quad_phase(g.zo, g.wavelength, fields.shape[-1], g.dxp), fftshift)
    if p == "asp":
        if fftshift:
            raise ValueError("ASP propagator only works with fftshiftswitch == False")
        tf = np.fft.ifftshift(asp_transfer_function(g.nosm, g.npsm, g.Np, g.zo, g.wavelength, g.Lp), axes=(-2, -1))
        return ifft2c(fft2c(fields, True) * tf, True)
    if p in ("polychromeasp", "scaledasp", "scaledpolychromeasp", "twosteppolychrome") and fftshift:
        raise ValueError(f"{propagator} propagatorType works only with fftshiftSwitch = False")
    if p == "polychromeasp":  # Operators.py:458-505
        return ifft2c(fft2c(fields) * polychrome_asp_tf(g))
    if p == "scaledasp":  # Operators.py:313-350
        Q1, Q2 = scaled_asp_tables(g.zo, g.wavelength, g.Np, g.dxo, g.dxd)
        return ifft2c(fft2c(fields * Q1) * Q2)
    if p == "scaledpolychromeasp":  # Operators.py:378-423
        Q1, Q2 = scaled_polychrome_asp_tables(g)
        return ifft2c(fft2c(fields * Q1) * Q2)
    if p == "twosteppolychrome":  # Operators.py:233-282
        tf, qp = two_step_polychrome_tables(g)
        return fft2c(ifft2c(fft2c(fields) * tf) * qp)
    if p == "identity":  # Operators.py:508-533: multiplication by complex128 ones
        return fields * (quad_phase(1e-3, 532e-9, g.Np, g.dxp) * 0 + 1)
    raise NotImplementedError(propagator)


def detector2object(fields, propagator, fftshift, g: Geometry):
    """Inverse propagators (PtyLab/Operators/Operators.py:53-74, 116-152, 218-230, 561-573)."""
    p = propagator.lower()
    if p == "fraunhofer":
        return ifft2c(fields, fftshift)
    if p == "fresnel":
        return ifft2c(fields, fftshift) * quad_phase(g.zo, g.wavelength, g.Np, g.dxp).conj()
    if p == "asp":
        if fftshift:
            raise ValueError("ASP propagator only works with fftshiftswitch == False")
        tf = np.fft.ifftshift(asp_transfer_function(g.nosm, g.npsm, g.Np, g.zo, g.wavelength, g.Lp), axes=(-2, -1))
        return ifft2c(fft2c(fields, True) * tf.conj(), True)
    if p in ("polychromeasp", "scaledasp", "scaledpolychromeasp", "twosteppolychrome") and fftshift:
        raise ValueError(f"{propagator} propagatorType works only with fftshiftSwitch = False")
    if p == "polychromeasp":  # Operators.py:536-558
        return ifft2c(fft2c(fields) * polychrome_asp_tf(g).conj())
    if p == "scaledasp":  # Operators.py:346-375
        Q1, Q2 = scaled_asp_tables(g.zo, g.wavelength, g.Np, g.dxo, g.dxd)
        return ifft2c(fft2c(fields) * Q2.conj()) * Q1.conj()
    if p == "scaledpolychromeasp":  # Operators.py:419-455
        Q1, Q2 = scaled_polychrome_asp_tables(g)
        return ifft2c(fft2c(fields) * Q2.conj()) * Q1.conj()
    if p == "twosteppolychrome":  # Operators.py:270-275 (the field part of the pair returned at :285-310)
        tf, qp = two_step_polychrome_tables(g)
        return ifft2c(fft2c(fields * qp.conj()) * tf.conj())
    if p == "identity":
        return fields * (quad_phase(1e-3, 532e-9, g.Np, g.dxp) * 0 + 1)
    raise NotImplementedError(propagator)


# ----------------------------------------------------------------------------
# geometry, scan positions, order, initial guesses
# ----------------------------------------------------------------------------
def positions_cpm(encoder, dxo, No, Np):
    """round(encoder/dxo) + No//2 - Np//2 as int (PtyLab/Reconstruction/Reconstruction.py:21-31)."""
    positions = np.round(encoder / dxo)
    positions = positions + No // 2 - Np // 2
    return positions.astype(int)


def positions_fpm(encoder, dxo, Np, wavelength, zled, No):
    """LED angles to spectrum-patch corners (PtyLab/Reconstruction/Reconstruction.py:689-706)."""
    conv = -(1 / wavelength) * dxo * Np
    positions = np.round(
        conv * encoder / np.sqrt(encoder[:, 0] ** 2 + encoder[:, 1] ** 2 + zled**2)[..., None]
    )
    positions = positions + No // 2 - Np // 2
    return positions.astype(int)


def derive_No(positions_fn, Np):
    """Object size from the scan extent (PtyLab/Reconstruction/Reconstruction.py:194-204)."""
    pos = positions_fn(Np * 2**2)
    range_pixels = np.max(pos, axis=0) - np.min(pos, axis=0)
    range_pixels = np.max(range_pixels) + Np * 2
    if range_pixels % 2 == 1:
        range_pixels += 1
    return int(np.max([Np, range_pixels]))


def position_order(order, num_frames, n_error, positions):
    """BaseEngine.setPositionOrder (PtyLab/Engines/BaseEngine.py:637-665)."""
    if order == "sequential":
        return np.arange(num_frames)
    if order == "random":
        idx = np.arange(num_frames)
        if n_error >= 2:
            np.random.shuffle(idx)
        return idx
    if order == "NA":
        rows = positions[:, 0] - np.mean(positions[:, 0])
        cols = positions[:, 1] - np.mean(positions[:, 1])
        return np.argsort(np.sqrt(rows**2 + cols**2))
    raise ValueError("position order not properly set")


def initial_object_ones(shape):
    """'ones' initial guess, consumes the global RNG (PtyLab/utils/initializationFunctions.py:34-35)."""
    return (np.ones(shape) + 0.001 * np.random.rand(*shape)).astype(np.complex64)


def initial_probe_circ(shape, Xp, Yp, diameter):
    """'circ' initial probe (PtyLab/utils/initializationFunctions.py:37-48)."""
    pupil = circ(Xp, Yp, diameter)
    f = np.ones(shape, dtype=np.complex64) + 0.001 * np.random.rand(*shape)
    f *= pupil
    return f.astype(np.complex64)


def initial_object_upsampled(shape, ptychogram, No, Np):
    """FPM 'upsampled' initial spectrum (PtyLab/utils/initializationFunctions.py:56-62)."""
    low_res = ifft2c(np.sqrt(np.mean(ptychogram, 0)))
    pad = (int((No - Np) / 2), int((No - Np) / 2))
    up = np.pad(low_res, pad, mode="constant", constant_values=0)
    return (np.ones(shape) * up).astype(np.complex64)


# ----------------------------------------------------------------------------
# engines
# ----------------------------------------------------------------------------
@dataclass
class Settings:
    """The Params switches on this path (PtyLab/Params/Params.py:41-195) plus engine scalars."""

    engine: str = "ePIE"
    propagator: str = "Fraunhofer"
    order: str = "sequential"
    fftshift: bool = False
    operationMode: str = "CPM"
    saveMemory: bool = False
    probeBoundary: bool = False
    orthogonalizationSwitch: bool = False
    orthogonalizationFrequency: int = 10
    probePowerCorrectionSwitch: bool = False
    absorbingProbeBoundary: bool = False
    absorbingProbeBoundaryAleph: float = 5e-2
    entrancePupilDiameter: float = 0.0
    betaObject: Optional[float] = None
    betaProbe: Optional[float] = None
    alphaObject: float = 0.1
    alphaProbe: float = 0.1
    feedbackM: float = 0.3
    frictionM: float = 0.7
    regObject: float = 1.0
    regProbe: float = 1.0
    # projection switches (Params.py:60-120; BaseEngine.py:870-1012)
    intensityConstraint: str = "standard"
    adaptiveDenoisingSwitch: bool = False
    backgroundModeSwitch: bool = False
    FourierMaskSwitch: bool = False
    intensityMask: bool = False
    # mqNewton (mqNewton.py:50-66)
    beta1: float = 0.5
    beta2: float = 0.5
    betaObject_m: float = 0.25
    betaProbe_m: float = 0.25
    momentum_method: str = "ADAM"


_DEFAULT_BETAS = {"ePIE": (0.25, 0.25), "mPIE": (0.25, 0.25), "qNewton": (1, 1), "mqNewton": (1, 1), "e3PIE": (0.25, 0.25)}


@dataclass
class State:
    object: np.ndarray
    probe: np.ndarray
    error: np.ndarray = field(default_factory=lambda: np.zeros(0))
    errorAtPos: Optional[np.ndarray] = None
    detectorError: Optional[np.ndarray] = None
    objectMomentum: Optional[np.ndarray] = None
    probeMomentum: Optional[np.ndarray] = None
    objectBuffer: Optional[np.ndarray] = None
    probeBuffer: Optional[np.ndarray] = None
    objectMomentum_v: Optional[np.ndarray] = None
    probeMomentum_v: Optional[np.ndarray] = None
    purityProbe: float = 1.0
    background: Optional[np.ndarray] = None  # backgroundModeSwitch (float64, Np x Np)
    reference: Optional[np.ndarray] = None  # 'interferometric': detector-plane reference field
    intensityScaling: Optional[np.ndarray] = None  # 'fluctuation': per-frame scaling (params.intensityScaling)


class OracleEngine:
    """One engine run: the position loop of ePIE.py:68-118, mPIE.py:110-195,
    qNewton.py:63-99 or e3PIE.py:71-190, with BaseEngine's projection,
    error metrics and the in-scope constraints."""

    def __init__(self, s: Settings, g: Geometry, state: State, ptychogram, positions, energyAtPos, Xp=None, Yp=None,
                 W=None, intensity_mask=None):
        self.s = s
        self.W = W  # experimentalData.W (FourierMaskSwitch)
        self.intensity_mask = intensity_mask  # reconstruction.intensity_mask (params.intensityMask)
        self.g = g
        self.st = state
        self.ptychogram = np.asarray(ptychogram)
        self.positions = np.asarray(positions)
        self.energyAtPos = np.asarray(energyAtPos)
        bo, bp = _DEFAULT_BETAS[s.engine]
        self.betaObject = bo if s.betaObject is None else s.betaObject
        self.betaProbe = bp if s.betaProbe is None else s.betaProbe
        self.fftshiftFlag = False
        self.momentumAcceleration = s.engine in ("mPIE", "mqNewton")
        self._loop = 0
        self.Xp = g.Xp if Xp is None else Xp
        self.Yp = g.Yp if Yp is None else Yp
        if s.engine == "mPIE":
            # mPIE.py:73-94: zero momenta, buffers from the current guess
            st = self.st
            if st.objectMomentum is None:
                st.objectMomentum = np.zeros_like(st.object)
            if st.probeMomentum is None:
                st.probeMomentum = np.zeros_like(st.probe)
        if s.engine == "mqNewton":
            # mqNewton.py:41-47: zero momenta, buffers from the guess at construction
            st = self.st
            st.objectMomentum = np.zeros_like(st.object)
            st.probeMomentum = np.zeros_like(st.probe)
            st.objectBuffer = st.object.copy()
            st.probeBuffer = st.probe.copy()
        if s.engine == "e3PIE":
            # e3PIE.py:62-69: ifftshifted aspw TF for the slice spacing, complex128
            H = aspw_transfer_function(g.dz, g.wavelength / g.refrIndex, g.Np, g.Lp)
            self.H = np.fft.ifftshift(H)

    # BaseEngine._prepareReconstruction subset (BaseEngine.py:96-111)
    def prepare(self):
        s, st, g = self.s, self.st, self.g
        if s.propagator == "ASP" and s.fftshift:
            raise ValueError("ASP propagatorType works only with fftshiftSwitch = False")
        if s.fftshift and not self.fftshiftFlag:  # _checkFFT BaseEngine.py:405-420
            self.ptychogram = np.fft.ifftshift(self.ptychogram, axes=(-1, -2))
            if self.W is not None:
                self.W = np.fft.ifftshift(self.W, axes=(-1, -2))
            self.fftshiftFlag = True
        if s.backgroundModeSwitch:  # _checkMISC BaseEngine.py:361-364
            st.background = 1e-1 * np.ones((g.Np, g.Np))
        if s.intensityConstraint == "interferometric":  # BaseEngine.py:371-374 (float64 ones)
            st.reference = np.ones(st.probe[0, 0, 0, 0, ...].shape)
        if s.probePowerCorrectionSwitch:  # BaseEngine.py:227-235
            maxProbePower = np.sqrt(np.max(np.sum(self.ptychogram, (-1, -2))))
            st.probe = st.probe / np.sqrt(np.sum(st.probe * st.probe.conj())) * maxProbePower
        # _probeWindow BaseEngine.py:237-266
        self.probeWindow = None
        if not s.saveMemory or s.absorbingProbeBoundary:
            self.probeWindow = np.exp(
                -(((self.Xp**2 + self.Yp**2) / (2 * (3 / 4 * g.Np * g.dxp / 2.355) ** 2)) ** 10)
            )
        if s.probeBoundary:
            self.probeWindow = circ(self.Xp, self.Yp, s.entrancePupilDiameter + s.entrancePupilDiameter * 0.2)
        # _initializeErrors BaseEngine.py:199-225
        nf = self.ptychogram.shape[0]
        if s.saveMemory:
            st.detectorError = 0
        elif st.detectorError is None:
            st.detectorError = np.zeros((nf, g.Np, g.Np))
        if st.errorAtPos is None:
            st.errorAtPos = np.zeros((nf, 1), dtype=np.float32)

    # BaseEngine.intensityProjection (BaseEngine.py:870-1012) with the
    # standard / poission / exponential / fluctuation constraints, adaptive
    # denoising (:1805-1822), the background mode and the Fourier / intensity
    # masks; NumPy's dtype rules as in the reference (the float64 background
    # is added in place to the float32 estimate, so the estimate stays float32)
    def intensity_projection(self, j, esw):
        s, st = self.s, self.st
        gimmel = 1e-10
        ESW = object2detector(esw, s.propagator, s.fftshift, self.g)
        if s.intensityConstraint == "interferometric":  # BaseEngine.py:883-888
            Iest = np.sum(np.abs(ESW + st.reference) ** 2, axis=(0, 1, 2))[-1]
        else:
            Iest = np.sum(np.abs(ESW) ** 2, axis=(0, 1, 2))[-1]
        if s.backgroundModeSwitch:
            Iest += st.background
        Imeas = self.ptychogram[j]
        cur = abs(Imeas - Iest)  # getRMSD BaseEngine.py:843-868
        if s.saveMemory:
            self.st.errorAtPos[j] = np.sum(cur * self.W) if s.FourierMaskSwitch else np.sum(cur)
        else:
            self.st.detectorError[j] = cur
        if s.adaptiveDenoisingSwitch:  # BaseEngine.adaptiveDenoising
            Am = Imeas**0.5
            Ae = np.abs(Iest) ** 0.5
            noise = np.abs(np.mean(Am - Ae))
            Am = Am - noise
            Am[Am < 0] = 0
            Imeas = Am**2
        c = s.intensityConstraint
        if c == "fluctuation":
            if s.FourierMaskSwitch:
                aleph = np.sum(Imeas * Iest * self.W) / np.sum(Imeas * Imeas * self.W)
            else:
                aleph = np.sum(Imeas * Iest) / np.sum(Imeas * Imeas)
            st.intensityScaling[j] = aleph
            frac = (1 + aleph) / 2 * Imeas / (Iest + gimmel)
        elif c == "exponential":
            x = cur / (Iest + gimmel)
            W = np.exp(-0.05 * x)
            frac = np.sqrt(Imeas / (Iest + gimmel))
            frac = W * frac + (1 - W)
        elif c == "poission":
            frac = Imeas / (Iest + gimmel)
        elif c in ("standard", "interferometric"):
            frac = np.sqrt(Imeas / (Iest + gimmel))
        else:
            raise ValueError("intensity constraint not properly specified!")
        if c == "interferometric":  # BaseEngine.py:975-982: the reference takes the ESW's shape
            temp = (ESW + st.reference) * frac - ESW
            ESW = (ESW + st.reference) * frac - st.reference
            st.reference = temp
        elif s.intensityMask:
            ESW = ESW * (frac * self.intensity_mask + (self.intensity_mask - 1))
        else:
            ESW = ESW * frac
        if s.backgroundModeSwitch:
            upd = (1 + 1 / self.ptychogram.shape[0] * (np.sqrt(frac) - 1)) ** 2
            st.background = st.background * upd * self.W if s.FourierMaskSwitch else st.background * upd
        return detector2object(ESW, s.propagator, s.fftshift, self.g)

    # BaseEngine.getErrorMetrics (BaseEngine.py:819-841)
    def error_metrics(self):
        st = self.st
        if not self.s.saveMemory:
            if self.s.FourierMaskSwitch:
                st.errorAtPos = np.sum(np.abs(st.detectorError) * self.W, axis=(-1, -2))
            else:
                st.errorAtPos = np.sum(np.abs(st.detectorError), axis=(-1, -2))
        st.errorAtPos = st.errorAtPos / (self.energyAtPos + 1e-20)
        st.error = np.append(st.error, np.sum(st.errorAtPos))

    # ---------------------------------------------------------------- updates
    def epie_object(self, patch, D):  # ePIE.py:128-143
        P = self.st.probe
        frac = P.conj() / np.max(np.sum(np.abs(P) ** 2, axis=(0, 1, 2, 3)))
        return patch + self.betaObject * np.sum(frac * D, axis=(0, 2, 3), keepdims=True)

    def epie_probe(self, patch, D):  # ePIE.py:145-160
        frac = patch.conj() / np.max(np.sum(np.abs(patch) ** 2, axis=(0, 1, 2, 3)))
        return self.st.probe + self.betaProbe * np.sum(frac * D, axis=(0, 1, 3), keepdims=True)

    def mpie_object(self, patch, D):  # mPIE.py:226-251
        P = self.st.probe
        absP2 = np.abs(P) ** 2
        Pmax = np.max(np.sum(absP2, axis=(0, 1, 2, 3)), axis=(-1, -2))
        a = self.s.alphaObject
        if self.s.operationMode == "FPM":
            frac = abs(P) / Pmax * P.conj() / (a * Pmax + (1 - a) * absP2)
        else:
            frac = P.conj() / (a * Pmax + (1 - a) * absP2)
        return patch + self.betaObject * np.sum(frac * D, axis=2, keepdims=True)

    def mpie_probe(self, patch, D, weight=1):  # mPIE.py:253-270
        absO2 = np.abs(patch) ** 2
        Omax = np.max(np.sum(absO2, axis=(0, 1, 2, 3)), axis=(-1, -2))
        a = self.s.alphaProbe
        frac = patch.conj() / (a * Omax + (1 - a) * absO2)
        return self.st.probe + weight * self.betaProbe * np.sum(frac * D, axis=1, keepdims=True)

    def mpie_momentum(self):  # mPIE.py:196-224
        st, s = self.st, self.s
        grad = st.objectBuffer - st.object
        st.objectMomentum = grad + s.frictionM * st.objectMomentum
        st.object = st.object - s.feedbackM * st.objectMomentum
        st.objectBuffer = st.object.copy()
        grad = st.probeBuffer - st.probe
        st.probeMomentum = grad + s.frictionM * st.probeMomentum
        st.probe = st.probe - s.feedbackM * st.probeMomentum
        st.probeBuffer = st.probe.copy()

    def qn_object(self, patch, D):  # qNewton.py:108-122
        P = self.st.probe
        Pmax = np.max(np.sum(np.abs(P), axis=(0, 1, 2, 3)))
        frac = np.abs(P) / Pmax * P.conj() / (np.abs(P) ** 2 + self.s.regObject)
        return patch + self.betaObject * np.sum(frac * D, axis=(0, 2, 3), keepdims=True)

    def qn_probe(self, patch, D):  # qNewton.py:124-140
        Omax = np.max(np.sum(np.abs(self.st.object), axis=(0, 1, 2, 3)))
        frac = np.abs(patch) / Omax * patch.conj() / (np.abs(patch) ** 2 + self.s.regProbe)
        return self.st.probe + self.betaProbe * np.sum(frac * D, axis=(0, 1, 3), keepdims=True)

    def adaptive_step(self, grad, m, v, itr):  # mqNewton.py:142-182
        """(update, first moment, second moment) of the chosen momentum method."""
        s = self.s
        if s.momentum_method == "momentum":
            m = grad + s.frictionM * m
            return m, m, v
        b1s = 1 - s.beta1**itr
        b2s = 1 - s.beta2**itr
        nsq = np.linalg.norm(grad.ravel(), 2) ** 2
        m = s.beta1 * m + (1 - s.beta1) * grad
        v = s.beta2 * v + (1 - s.beta2) * nsq
        m_hat = m / b1s
        denom = (v / b2s) ** 0.5 + 1e-8
        if s.momentum_method == "ADAM":
            return m_hat / denom, m, v
        if s.momentum_method == "NADAM":
            return (s.beta1 * m_hat + grad * (1 - s.beta1) / b1s) / denom, m, v
        raise AttributeError(s.momentum_method)

    def mq_momentum(self):  # mqNewton.py:184-224
        st, s = self.st, self.s
        itr = self._loop + 1
        u, st.objectMomentum, st.objectMomentum_v = self.adaptive_step(
            st.objectBuffer - st.object, st.objectMomentum, st.objectMomentum_v, itr
        )
        st.object = st.object - s.betaObject_m * u
        st.objectBuffer = st.object.copy()
        u, st.probeMomentum, st.probeMomentum_v = self.adaptive_step(
            st.probeBuffer - st.probe, st.probeMomentum, st.probeMomentum_v, itr
        )
        st.probe = st.probe - s.betaProbe_m * u
        st.probeBuffer = st.probe.copy()

    def e3_object(self, patch, D, localProbe):  # e3PIE.py:192-208
        frac = localProbe.conj() / np.max(np.sum(np.abs(localProbe) ** 2, axis=(0, 1, 2)))
        return patch + self.betaObject * np.sum(frac * D, axis=(0, 2), keepdims=True)

    def e3_probe(self, patch, D, localProbe, beth):  # e3PIE.py:210-225
        frac = patch.conj() / np.max(np.sum(np.abs(patch) ** 2, axis=(0, 1, 2)))
        return localProbe + beth * np.sum(frac * D, axis=(0, 1), keepdims=True)

    # ------------------------------------------------------------- one position
    def position(self, j, momentum_draw=None):
        st, g = self.st, self.g
        row, col = self.positions[j]
        sy = slice(row, row + g.Np)
        sx = slice(col, col + g.Np)
        patch = st.object[..., sy, sx].copy()
        eng = self.s.engine
        if eng == "e3PIE":
            return self._e3pie_position(j, patch, sy, sx)
        esw = patch * st.probe
        eswUpdate = self.intensity_projection(j, esw)
        D = eswUpdate - esw
        if eng == "ePIE":
            st.object[..., sy, sx] = self.epie_object(patch, D)
            st.probe = self.epie_probe(patch, D)
        elif eng == "mPIE":
            st.object[..., sy, sx] = self.mpie_object(patch, D)
            st.probe = self.mpie_probe(patch, D, 1)
            if momentum_draw is not None and momentum_draw > 0.95:
                self.mpie_momentum()
        elif eng == "qNewton":
            st.object[..., sy, sx] = self.qn_object(patch, D)
            st.probe = self.qn_probe(patch, D)
        elif eng == "mqNewton":  # mqNewton.py:112-126
            st.object[..., sy, sx] = self.qn_object(patch, D)
            st.probe = self.qn_probe(patch, D)
            self.mq_momentum()
        else:
            raise NotImplementedError(eng)

    def _e3pie_position(self, j, patch, sy, sx):  # e3PIE.py:99-173
        st, H = self.st, self.H
        S = self.g.nslice
        st.esw[:, :, :, 0, ...] = patch[:, :, :, 0, ...] * st.probe[:, :, :, 0, ...]
        for s in range(1, S):
            st.probe[:, :, :, s, ...] = np.fft.ifft2(np.fft.fft2(st.esw[:, :, :, s - 1, ...]) * H)
            st.esw[:, :, :, s, ...] = st.probe[:, :, :, s, ...] * patch[:, :, :, s, ...]
        eswUpdate = self.intensity_projection(j, st.esw)
        D = (eswUpdate - st.esw)[:, :, :, -1, ...]
        for t in range(S - 1):
            s = S - 1 - t
            st.object[..., s, sy, sx] = self.e3_object(patch[:, :, :, s, ...], D, st.probe[:, :, :, s, ...])
            st.probe[:, :, :, s, ...] = self.e3_probe(patch[:, :, :, s, ...], D, st.probe[:, :, :, s, ...], 0.9)
            D = np.fft.ifft2(np.fft.fft2(st.probe[:, :, :, s, ...]) * H.conj()) - st.esw[:, :, :, s - 1, ...]
        st.object[..., 0, sy, sx] = self.e3_object(patch[:, :, :, 0, ...], D, st.probe[:, :, :, 0, ...])
        st.probe[:, :, :, 0, ...] = self.e3_probe(patch[:, :, :, 0, ...], D, st.probe[:, :, :, 0, ...], self.betaProbe)

    # ------------------------------------------------------------- constraints
    def apply_constraints(self, loop):  # BaseEngine.applyConstraints subset (BaseEngine.py:1440-1500)
        s, st = self.s, self.st
        if s.orthogonalizationSwitch and np.mod(loop, s.orthogonalizationFrequency) == 0:
            self.orthogonalization()
        if s.probePowerCorrectionSwitch:
            maxProbePower = np.sqrt(np.max(np.sum(self.ptychogram, (-1, -2))))
            st.probe = st.probe / np.sqrt(np.sum(st.probe * st.probe.conj())) * maxProbePower
        if s.probeBoundary:
            st.probe *= self.probeWindow
        if s.absorbingProbeBoundary:
            aleph = s.absorbingProbeBoundaryAleph
            st.probe = (1 - aleph) * st.probe + aleph * st.probe * self.probeWindow

    def orthogonalization(self):  # BaseEngine.py:1614-1669 with utils.py:130-211 (snapShots)
        st, g = self.st, self.g
        if g.npsm > 1:
            for l in range(g.nlambda):
                for sl in range(g.nslice):
                    p = st.probe[l, 0, :, sl, :, :]
                    modes, evals, V = snapshot_modes(p)
                    st.probe[l, 0, :, sl, :, :] = modes
                    st.purityProbe = float(np.sqrt(np.sum(np.asarray(evals) ** 2)))
                    if self.momentumAcceleration:
                        for name in ("probeBuffer", "probeMomentum"):
                            arr = getattr(st, name)
                            q = arr[l, 0, :, sl, :, :].reshape((g.npsm, g.Np**2))
                            arr[l, 0, :, sl, :, :] = (np.array(V) @ q).reshape((g.npsm, g.Np, g.Np))
        elif g.nosm > 1:
            for l in range(g.nlambda):
                for sl in range(g.nslice):
                    o = st.object[l, :, 0, sl, :, :]
                    modes, evals, V = snapshot_modes(o)
                    st.object[l, :, 0, sl, :, :] = modes
                    if self.momentumAcceleration:
                        for name in ("objectBuffer", "objectMomentum"):
                            arr = getattr(st, name)
                            q = arr[l, :, 0, sl, :, :].reshape((g.nosm, g.No**2))
                            arr[l, :, 0, sl, :, :] = (np.array(V) @ q).reshape((g.nosm, g.No, g.No))

    # ------------------------------------------------------------- driver
    def reconstruct(self, num_iterations):
        """Run like Engine.reconstruct(): prepare, then iterations of
        (order, positions, error metric, constraints); returns the state."""
        self.prepare()
        st = self.st
        if self.s.engine == "mPIE":  # mPIE.py:103-105
            st.objectBuffer = st.object.copy()
            st.probeBuffer = st.probe.copy()
        if self.s.engine == "e3PIE":  # e3PIE.py:75
            st.esw = st.probe.copy()
        if self.s.engine == "mqNewton" and self.s.momentum_method in ("ADAM", "NADAM"):
            # initializeAdaptiveMomentum (mqNewton.py:68-79)
            st.objectMomentum_v = st.objectMomentum.copy()
            st.probeMomentum_v = st.probeMomentum.copy()
        nf = self.ptychogram.shape[0]
        for loop in range(num_iterations):
            self._loop = loop
            order = position_order(self.s.order, nf, len(st.error), self.positions)
            for j in order:
                draw = np.random.rand(1)[0] if self.s.engine == "mPIE" else None
                self.position(int(j), draw)
            self.error_metrics()
            self.apply_constraints(loop)
        return st


def snapshot_modes(p):
    """Gram-matrix mode orthogonalisation (PtyLab/utils/utils.py:130-175)."""
    p2D = p.reshape(p.shape[0], p.shape[1] * p.shape[2])
    G = np.dot(p2D.conj(), np.transpose(p2D))
    w, V = np.linalg.eigh(G)
    order = np.argsort(w)[::-1]
    s = np.sqrt(np.clip(w[order].real, 0.0, None))
    evals = s**2 / np.sum(s**2)
    V = np.ascontiguousarray(V[:, order].T)
    modes = np.dot(V, p2D).reshape(p.shape)
    return modes, evals, V


# ----------------------------------------------------------------------------
# convenience: run a fixture's configuration
# ----------------------------------------------------------------------------
def run_fixture(fx, iters=None, dtype=None):
    """Run the configuration stored in a golden fixture (dict of arrays, see
    tests/golden/make_golden.py) from its recorded initial guess; returns State.
    ``dtype=np.complex128`` runs the same algorithm in double precision
    (intensities float64), the precision reference for the FP32 paths."""
    m = {k[5:]: fx[k] for k in fx if k.startswith("meta_")}
    i = {k[3:]: fx[k] for k in fx if k.startswith("in_")}
    nl, nos, nps, nsl = (int(v) for v in m["modes"])
    g = Geometry(
        Np=int(i["Np"]),
        No=int(i["No"]),
        dxp=float(i["dxp"]),
        wavelength=float(i["wavelength"]),
        zo=float(i["zo"]),
        nlambda=nl,
        nosm=nos,
        npsm=nps,
        nslice=nsl,
        dz=float(i.get("dz", 0.0)),
        dxd=float(m.get("dxd", 0.0)),
        spectralDensity=tuple(np.atleast_1d(i["spectralDensity"])) if "spectralDensity" in i else (float(i["wavelength"]),),
    )
    s = Settings(
        momentum_method=str(m.get("momentum_method", "ADAM")),
        engine=str(m["engine"]),
        propagator=str(m["propagator"]),
        order=str(m["order"]),
        fftshift=bool(m["fftshift"]),
        operationMode=str(m["operationMode"]),
        probeBoundary=bool(m["probeBoundary"]),
        orthogonalizationSwitch=bool(m["orthogonalizationSwitch"]),
        orthogonalizationFrequency=int(m["orthogonalizationFrequency"]),
        entrancePupilDiameter=float(i["entrancePupilDiameter"]),
        intensityConstraint=str(m.get("intensityConstraint", "standard")),
        adaptiveDenoisingSwitch=bool(m.get("adaptiveDenoisingSwitch", False)),
        backgroundModeSwitch=bool(m.get("backgroundModeSwitch", False)),
        FourierMaskSwitch=bool(m.get("FourierMaskSwitch", False)),
        intensityMask=bool(m.get("intensityMask", False)),
        saveMemory=bool(m.get("saveMemory", False)),
        probePowerCorrectionSwitch=bool(m.get("probePowerCorrectionSwitch", False)),
    )
    cdt = np.complex64 if dtype is None else dtype
    fdt = np.float64 if cdt == np.complex128 else np.float32
    st = State(object=np.array(i["init_object"], dtype=cdt), probe=np.array(i["init_probe"], dtype=cdt))
    if "intensityScaling" in i:
        st.intensityScaling = np.array(i["intensityScaling"], dtype=np.float64)
    W = np.array(i["W"]) if "W" in i else None
    mask = np.array(i["intensity_mask"]) if "intensity_mask" in i else None
    if dtype is not None:
        W = None if W is None else W.astype(fdt)
        mask = None if mask is None else mask.astype(fdt)
    eng = OracleEngine(s, g, st, np.asarray(i["ptychogram"], dtype=fdt), i["positions"], i["energyAtPos"],
                       W=W, intensity_mask=mask)
    np.random.seed(int(m["seed"]))
    return eng.reconstruct(int(m["iters"]) if iters is None else iters)


# ----------------------------------------------------------------------------
# multislice forward model (the model e3PIE inverts) and its reference gradient
# ----------------------------------------------------------------------------
def multislice_forward(obj, probe, positions, H_shifted):
    """I_j = sum_p |fft2c(psi_{S-1})|^2, psi_0 = O_0[patch] P, psi_s = ifft2(fft2(psi_{s-1}) H) O_s[patch]
    (e3PIE.py:99-118 with the Fraunhofer detector); obj (S, No, No), probe (npsm, Np, Np)."""
    S = obj.shape[0]
    Np = probe.shape[-1]
    out = np.empty((len(positions), Np, Np))
    for j, (r, c) in enumerate(positions):
        psi = obj[0, r : r + Np, c : c + Np] * probe
        for s in range(1, S):
            psi = np.fft.ifft2(np.fft.fft2(psi) * H_shifted) * obj[s, r : r + Np, c : c + Np]
        out[j] = np.sum(np.abs(fft2c(psi)) ** 2, axis=0)
    return out


def e3pie_last_slice_delta(obj, probe, position, H_shifted, Imeas):
    """For one position and one probe mode: the last slice's incident field
    P_{S-1} and e3PIE's DELTA = eswUpdate - esw of the last slice after the
    standard intensity projection (e3PIE.py:99-123, BaseEngine.py:870-1012)."""
    S = obj.shape[0]
    Np = probe.shape[-1]
    r, c = position
    P = probe
    psi = obj[0, r : r + Np, c : c + Np] * P
    for s in range(1, S):
        P = np.fft.ifft2(np.fft.fft2(psi) * H_shifted)
        psi = P * obj[s, r : r + Np, c : c + Np]
    Psi = fft2c(psi)
    Iest = np.sum(np.abs(Psi) ** 2, axis=0)
    frac = np.sqrt(Imeas / (Iest + 1e-10))
    return P, ifft2c(Psi * frac) - psi
