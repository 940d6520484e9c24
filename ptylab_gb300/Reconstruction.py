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

    def reset_positioncorrection(self):
        """Positions from the data's encoder again (Reconstruction.py:136-138),
        e.g. after an illumination calibration rewrote it."""
        self.encoder_corrected = self.data.encoder.copy()

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
        if self.initialObject == "recon":
            # Reconstruction.py:370-372 reads the object from the file named
            # by initialProbe_filename
            self.initialGuessObject = self.loadResults(self.initialProbe_filename, datatype="object")
            return
        self.initialGuessObject = initialProbeOrObject(self.shape_O, self.initialObject, self, self.logger).astype(
            np.complex64
        )

    def initializeProbe(self, force=False):
        if self.data.entrancePupilDiameter is None:
            self.data.entrancePupilDiameter = self.Lp / 3
        self.shape_P = (self.nlambda, 1, self.npsm, self.nslice, int(self.Np), int(self.Np))
        if self.initialProbe == "recon":
            self.initialGuessProbe = self.loadResults(self.initialProbe_filename, datatype="probe")
            return
        self.initialGuessProbe = initialProbeOrObject(self.shape_P, self.initialProbe, self).astype(np.complex64)

    def initializeObjectMomentum(self):
        self.objectMomentum = np.zeros_like(self.initialGuessObject)

    def initializeProbeMomentum(self):
        self.probeMomentum = np.zeros_like(self.initialGuessProbe)

    # ------------------------------------------------------------ result files
    @staticmethod
    def loadResults(fileName, datatype="probe"):
        """One array of a result file (Reconstruction.py:377-384)."""
        from .io import hdf5

        with hdf5.File(fileName, "r") as archive:
            data = np.copy(np.array(archive[datatype]))
        return data

    def load_object(self, filename):
        """The object of an earlier reconstruction, cut to ``shape_O``
        (Reconstruction.py:420-450)."""
        from .io import hdf5

        with hdf5.File(filename, "r") as archive:
            obj = np.array(archive["object"])
            stored = obj.shape
        obj = obj[tuple(slice(0, n) for n in self.shape_O)]
        if obj.shape != tuple(self.shape_O):
            raise RuntimeError(
                f"Shape of saved probe cannot be extended to shape of required probe. File: {stored}. Need: {self.shape_O}"
            )
        self.object = obj

    def load_probe(self, filename, expand_npsm=False, center_phase=False):
        """The probe of an earlier reconstruction, its centre cut to
        ``shape_P`` (Reconstruction.py:452-483)."""
        from .io import hdf5

        if center_phase:
            raise NotImplementedError("center_phase needs scikit-image's phase_cross_correlation")
        with hdf5.File(filename, "r") as archive:
            probe = np.array(archive["probe"])
        n_read = probe.shape[-1]
        Np = int(self.Np)
        ss = slice(max(n_read // 2 - Np // 2, 0), min(max(n_read // 2 - Np // 2 + Np, 0), n_read))
        stored = probe.shape
        probe = probe[: self.nlambda, :1, : self.npsm, : self.nslice, ss, ss]
        if probe.shape != tuple(self.shape_P):
            raise RuntimeError(
                f"Shape of saved probe cannot be extended to shape of required probe. File: {stored}. Need: {self.shape_P}"
            )
        self.probe = probe

    def load(self, filename):
        """The arrays ``saveResults`` wrote (Reconstruction.py:495-508)."""
        from .io import hdf5

        with hdf5.File(filename, "r") as archive:
            for key in ("probe", "object", "error", "wavelength", "dxp", "purityProbe", "purityObject", "zo"):
                setattr(self, key, np.array(archive[key]))
            if "theta" in archive.keys():
                self.theta = np.array(archive["theta"])

    def saveResults(self, fileName="recent", type="all", squeeze=False):
        """Write the reconstruction as HDF5 with the reference's dataset names
        and types (Reconstruction.py:510-576)."""
        from .io import hdf5

        allowed_save_types = ["all", "object", "probe", "probe_stack"]
        if type not in allowed_save_types:
            raise NotImplementedError(f"Only {allowed_save_types} are allowed keywords for type")
        squeezefun = np.squeeze if squeeze else (lambda x: x)
        host = lambda x: x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)
        if type == "all":
            probe, obj = host(self.probe), host(self.object)
            if self.data.operationMode == "CPM":
                with hdf5.File(fileName, "w") as hf:
                    hf.create_dataset("probe", data=probe, dtype="complex64")
                    hf.create_dataset("object", data=obj, dtype="complex64")
                    hf.create_dataset("error", data=np.asarray(self.error), dtype="f")
                    hf.create_dataset("zo", data=self._zo, dtype="f")
                    hf.create_dataset("wavelength", data=self.wavelength, dtype="f")
                    hf.create_dataset("dxp", data=self.dxp, dtype="f")
                    hf.create_dataset("purityProbe", data=self.purityProbe, dtype="f")
                    hf.create_dataset("purityObject", data=self.purityObject, dtype="f")
                    hf.create_dataset("I object", data=abs(obj), dtype="f")
                    hf.create_dataset("I probe", data=abs(probe), dtype="f")
                    hf.create_dataset("encoder_corrected", data=host(self.encoder_corrected))
                    if getattr(self, "theta", None) is not None:
                        hf.create_dataset("theta", data=self.theta, dtype="f")
            if self.data.operationMode == "FPM":
                with hdf5.File(fileName, "w") as hf:
                    hf.create_dataset("probe", data=probe, dtype="complex64")
                    hf.create_dataset("object", data=obj, dtype="complex64")
                    hf.create_dataset("error", data=np.asarray(self.error), dtype="f")
                    hf.create_dataset("zled", data=self.zled, dtype="f")
                    hf.create_dataset("wavelength", data=self.wavelength, dtype="f")
                    hf.create_dataset("dxp", data=self.dxp, dtype="f")
        elif type == "probe":
            with hdf5.File(fileName, "w") as hf:
                hf.create_dataset("probe", data=squeezefun(host(self.probe)), dtype="complex64")
        elif type == "object":
            with hdf5.File(fileName, "w") as hf:
                hf.create_dataset("object", data=squeezefun(host(self.object)), dtype="complex64")
        elif type == "probe_stack":
            with hdf5.File(str(fileName) + "_probe_stack.hdf5", "w") as hf:
                hf.create_dataset("probe_stack", data=host(self.probe_stack.get()), dtype="complex64")
        self.logger.info("The reconstruction results (%s) have been saved", type)

    # ------------------------------------------------------------ geometry
    @property
    def Nd(self):
        return self.data.ptychogram.shape[1]

    @property
    def Ld(self):
        return self.Nd * self.dxd

    # detector and object coordinates, detection NA and depth of field
    # (Reconstruction.py:583-598, 652-672, 712-724)
    @property
    def xd(self):
        return np.linspace(-self.Nd / 2, self.Nd / 2, int(self.Nd)) * self.dxd

    @property
    def Xd(self):
        return np.meshgrid(self.xd, self.xd)[0]

    @property
    def Yd(self):
        return np.meshgrid(self.xd, self.xd)[1]

    @property
    def xo(self):
        return np.linspace(-self.No / 2, self.No / 2, int(self.No)) * self.dxo

    @property
    def Xo(self):
        return np.meshgrid(self.xo, self.xo)[0]

    @property
    def Yo(self):
        return np.meshgrid(self.xo, self.xo)[1]

    @property
    def NAd(self):
        return self.Ld / (2 * self.zo)

    @property
    def DoF(self):
        return self.wavelength / self.NAd**2

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
