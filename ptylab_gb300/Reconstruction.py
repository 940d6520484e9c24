"""Reconstruction state, mirroring PtyLab's ``Reconstruction``
(PtyLab/Reconstruction/Reconstruction.py:34-876) for what the loop reads and
writes: geometry (dxp, Np, No), pixel positions, the 6-D object/probe arrays
and their seeded initial guesses, and the mPIE momentum arrays.

The engines only read attributes, so PtyLab's own Reconstruction works with
them unchanged; this class exists so the package is usable (and testable)
where PtyLab and its HDF5 dependencies are not installed.
"""

from __future__ import annotations

import logging
from copy import copy

import numpy as np

from .ExperimentalData import ExperimentalData


def circ(x, y, D):
    """Binary disc of diameter D (PtyLab/utils/utils.py:50-59)."""
    return (x**2 + y**2) < (D / 2) ** 2


def _ifft2c(x):
    ax = (-2, -1)
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(x, axes=ax), norm="ortho"), axes=ax)


def calculate_pixel_positions(encoder_corrected, dxo, No, Np, asint):
    """round(encoder/dxo) + No//2 - Np//2 (Reconstruction.py:21-31); numpy round is half-to-even."""
    positions = np.round(encoder_corrected / dxo)
    positions = positions + No // 2 - Np // 2
    if asint:
        positions = positions.astype(int)
    return positions


def initialProbeOrObject(shape, type_of_init, data, logger=None):
    """Seeded initial guesses (PtyLab/utils/initializationFunctions.py:10-62).

    Consumes NumPy's legacy global RNG exactly as the reference does, so a
    ``np.random.seed`` before ``initializeObjectProbe`` reproduces its guesses.
    """
    if type(type_of_init) is np.ndarray:
        return type_of_init
    if type_of_init == "ones":
        return np.ones(shape) + 0.001 * np.random.rand(*shape)
    if type_of_init == "circ":
        pupil = circ(data.Xp, data.Yp, data.data.entrancePupilDiameter)
        initial_field = np.ones(shape, dtype=np.complex64) + 0.001 * np.random.rand(*shape)
        initial_field *= pupil
        return initial_field
    if type_of_init == "upsampled":
        low_res = _ifft2c(np.sqrt(np.mean(data.data.ptychogram, 0)))
        pad_size = (int((data.No - data.Np) / 2), int((data.No - data.Np) / 2))
        upsampled = np.pad(low_res, pad_size, mode="constant", constant_values=0)
        return np.ones(shape) * upsampled
    raise NotImplementedError(f"initial guess {type_of_init!r} is not supported here (ones, circ, upsampled)")


class Reconstruction(object):
    listOfReconstructionPropertiesCPM = ["wavelength", "dxd", "theta", "spectralDensity", "entrancePupilDiameter"]
    listOfReconstructionPropertiesFPM = ["wavelength", "dxd", "zled", "NA"]

    def __init__(self, data: ExperimentalData, params, No=None):
        self.zMomentum = 0
        self.wavelength = None
        self._zo = None
        self.dxd = None
        self.theta = None
        self.encoder_corrected = None
        self.logger = logging.getLogger("Reconstruction")
        self.data = data
        self.params = params
        if No is not None:
            self.No = int(No)
        self.copyAttributesFromExperiment(data)
        self.computeParameters()
        self.initializeSettings()
        self.possible_GPU_fields = [
            "probe", "object", "probeBuffer", "objectBuffer", "probeMomentum", "objectMomentum",
            "detectorError", "background", "reference", "intensity_mask", "H",
        ]

    def copyAttributesFromExperiment(self, data):
        """Reconstruction.py:99-123."""
        keys = (
            self.listOfReconstructionPropertiesCPM
            if self.data.operationMode == "CPM"
            else self.listOfReconstructionPropertiesFPM
        )
        for key in keys:
            setattr(self, key, copy(getattr(data, key, None)))
        if self.data.operationMode == "CPM":
            self.zo = getattr(data, "zo")
        if self.encoder_corrected is None:
            self.encoder_corrected = data.encoder.copy()

    @property
    def zo(self):
        return self._zo

    @zo.setter
    def zo(self, new_value):
        """Reconstruction.py:135-145: dxp follows zo in CPM."""
        self._zo = new_value
        if self.data.operationMode == "CPM":
            self.dxp = self.wavelength * self._zo / self.Ld
        elif self.data.operationMode == "FPM":
            self.zled = self._zo

    def computeParameters(self):
        """Reconstruction.py:155-204."""
        if self.data.operationMode == "CPM":
            if self.data.entrancePupilDiameter is None:
                self.data.entrancePupilDiameter = self.Lp / 3
            if self.spectralDensity is None:
                self.spectralDensity = np.atleast_1d(self.wavelength)
        elif self.data.operationMode == "FPM":
            self.dxp = self.dxd / self.data.magnification
            self.zo = self.zled
            if self.NA is None:
                self.data.entrancePupilDiameter = self.Lp / 2
                self.NA = self.data.entrancePupilDiameter * self.wavelength / (2 * self.dxp**2 * self.Np)
            else:
                self.data.entrancePupilDiameter = 2 * self.dxp**2 * self.Np * self.NA / self.wavelength
        if not hasattr(self, "No"):
            self.No = self.Np * 2**2
            range_pixels = np.max(self.positions, axis=0) - np.min(self.positions, axis=0)
            range_pixels = np.max(range_pixels) + self.Np * 2
            if range_pixels % 2 == 1:
                range_pixels += 1
            self.No = int(np.max([self.Np, range_pixels]))

    def initializeSettings(self):
        """Reconstruction.py:302-334."""
        self.nlambda = 1
        self.nosm = 1
        self.npsm = 1
        self.nslice = 1
        self.purityProbe = 1.0
        self.purityObject = 1.0
        self.purityProbeHist = []
        self.positions0 = self.positions.copy()
        if self.data.operationMode == "FPM":
            self.initialObject = "upsampled"
            self.initialProbe = "circ"
        else:
            self.initialProbe = "circ"
            self.initialObject = "ones"

    def initializeObjectProbe(self, force=True):
        """Reconstruction.py:346-354: object first, then probe (RNG order)."""
        self.initializeObject(force=force)
        self.initializeProbe(force=force)
        self.object = self.initialGuessObject.copy()
        self.probe = self.initialGuessProbe.copy()

    def initializeObject(self, type_of_init=None, force=True):
        if type_of_init is not None:
            self.initialObject = type_of_init
        self.shape_O = (self.nlambda, self.nosm, 1, self.nslice, self.No, self.No)
        self.initialGuessObject = initialProbeOrObject(self.shape_O, self.initialObject, self, self.logger).astype(
            np.complex64
        )

    def initializeProbe(self, force=False):
        if self.data.entrancePupilDiameter is None:
            self.data.entrancePupilDiameter = self.Lp / 3
        self.shape_P = (self.nlambda, 1, self.npsm, self.nslice, int(self.Np), int(self.Np))
        self.initialGuessProbe = initialProbeOrObject(self.shape_P, self.initialProbe, self).astype(np.complex64)

    def initializeObjectMomentum(self):
        self.objectMomentum = np.zeros_like(self.initialGuessObject)

    def initializeProbeMomentum(self):
        self.probeMomentum = np.zeros_like(self.initialGuessProbe)

    # ------------------------------------------------------------ geometry
    @property
    def Nd(self):
        return self.data.ptychogram.shape[1]

    @property
    def Ld(self):
        return self.Nd * self.dxd

    @property
    def Np(self):
        return self.Nd

    @property
    def Lp(self):
        return self.Np * self.dxp

    @property
    def xp(self):
        return np.linspace(-self.Np / 2, self.Np / 2, int(self.Np)) * self.dxp

    @property
    def Xp(self):
        return np.meshgrid(self.xp, self.xp)[0]

    @property
    def Yp(self):
        return np.meshgrid(self.xp, self.xp)[1]

    @property
    def dxo(self):
        return self.dxp

    @property
    def Lo(self):
        return self.No * self.dxo

    @property
    def positions(self):
        """Patch corners in pixels (Reconstruction.py:676-710)."""
        if self.data.operationMode == "FPM":
            conv = -(1 / self.wavelength) * self.dxo * self.Np
            positions = np.round(
                conv
                * self.encoder_corrected
                / np.sqrt(
                    self.encoder_corrected[:, 0] ** 2 + self.encoder_corrected[:, 1] ** 2 + self.zled**2
                )[..., None]
            )
            positions = positions + self.No // 2 - self.Np // 2
            return positions.astype(int)
        return calculate_pixel_positions(self.encoder_corrected, self.dxo, self.No, self.Np, asint=True)
