"""Measurement container, mirroring PtyLab's ``ExperimentalData``
(PtyLab/ExperimentalData/ExperimentalData.py:21-288) for the fields the
reconstruction loop reads.  ``loadData`` reads PtyLab's HDF5 measurement
files through ``ptylab_gb300.io`` (no h5py or PyTables needed); the fields
can also be assigned directly, followed by ``_setData()``.
"""

from __future__ import annotations

import logging

import numpy as np


class ExperimentalData:
    def __init__(self, filename=None, operationMode="CPM"):
        self.logger = logging.getLogger("ExperimentalData")
        self.operationMode = operationMode
        self._setFields()
        if filename is not None:
            self.loadData(filename)
        self.fields_to_transfer = ["emptyBeam", "ptychogram", "ptychogramDownsampled", "W"]

    def _setFields(self):
        """Required/optional fields per operation mode (ExperimentalData.py:48-84)."""
        if self.operationMode == "CPM":
            self.requiredFields = ["ptychogram", "wavelength", "encoder", "dxd", "zo"]
            self.optionalFields = ["entrancePupilDiameter", "spectralDensity", "theta", "emptyBeam"]
            for f in self.optionalFields:
                setattr(self, f, getattr(self, f, None))
        elif self.operationMode == "FPM":
            self.requiredFields = ["ptychogram", "wavelength", "encoder", "dxd", "zled", "magnification"]
            self.optionalFields = ["NA"]
            self.NA = getattr(self, "NA", None)
            self.entrancePupilDiameter = getattr(self, "entrancePupilDiameter", None)
        else:
            raise ValueError('operationMode is not properly set, choose "CPM" or "FPM"')

    def loadData(self, filename=None):
        """Load a measurement file (ExperimentalData.py:86-149): the stub
        ``test:nodata``, or an .hdf5/.h5/.mat (HDF5-based) file holding the
        mode's required fields and any of its optional ones."""
        import os

        from .io import readHdf5

        if str(filename) == "test:nodata":
            self.filename = filename
            self.ptychogram = np.zeros((1, 16, 16), dtype=np.float32)
            self.encoder = np.zeros((1, 2), dtype=np.float64)
            self.wavelength = 500e-9
            self.dxd = 6.5e-6
            self.zo = 0.1
            self.entrancePupilDiameter = None
            self.spectralDensity = None
            self.theta = None
            self.emptyBeam = None
            self._setData()
            return
        if not os.path.exists(filename) and str(filename).startswith("example:"):
            raise FileNotFoundError(
                f"{filename}: PtyLab's example datasets are downloaded files that this package does not ship"
            )
        self.filename = filename
        readHdf5.checkDataFields(self.filename, self.requiredFields)
        measurementDict = readHdf5.loadInputData(self.filename, self.requiredFields, self.optionalFields)
        for a in measurementDict.keys():
            attribute = str(a)
            if not isinstance(getattr(type(self), attribute, None), property):
                setattr(self, attribute, measurementDict[a])
            self.logger.debug("Setting %s", a)
        self._setData()
        # last: the orientation can change the ptychogram itself
        self.setOrientation(readHdf5.getOrientation(self.filename))

    def setOrientation(self, orientation, force_contiguous=True):
        """Flip/transpose the frames to the ptypy orientation convention
        (ExperimentalData.py:192-232): 0 none, 1 columns reversed, 2 rows
        reversed, 3 both, 4 transposed, 5-7 transposed then reversed as 1-3."""
        if orientation is None:
            return
        if not isinstance(orientation, int):
            raise TypeError("Orientation value is not valid.")
        if orientation == 0:
            return
        if orientation < 0 or orientation > 7:
            raise ValueError(f"Orientation {orientation} is not implemented")
        if orientation >= 4:
            self.ptychogram = np.transpose(self.ptychogram, (0, 2, 1))
        if orientation in (1, 3, 5, 7):
            self.ptychogram = np.flip(self.ptychogram, axis=-1)
        if orientation in (2, 3, 6, 7):
            self.ptychogram = np.flip(self.ptychogram, axis=-2)
        if force_contiguous:
            self.ptychogram = np.ascontiguousarray(self.ptychogram)

    def reduce_positions(self, start, end):
        """Keep frames and encoder rows [start, end) (ExperimentalData.py:151-156)."""
        self.ptychogram = self.ptychogram[start:end]
        self.encoder = self.encoder[start:end]

    def cropCenter(self, size):
        """Crop every frame to size x size about the centre, starting one
        pixel past N // 2 - size // 2 as PtyLab does (ExperimentalData.py:158-171)."""
        if not isinstance(size, int):
            raise TypeError("Crop value is not valid. Int expected")
        first = self.ptychogram.shape[-1] // 2 - size // 2 + 1
        self.ptychogram = self.ptychogram[..., first:first + size, first:first + size]

    def binData(self, binning):
        """Average binning x binning pixel blocks of every frame into a float64
        ptychogram (ExperimentalData.py:173-190)."""
        n, ny, nx = self.ptychogram.shape
        frames = np.copy(self.ptychogram)
        out = np.zeros((n, ny // binning, nx // binning))
        for f in range(n):
            out[f] = frames[f].reshape(ny // binning, binning, nx // binning, binning).mean(axis=(1, 3))
        self.ptychogram = out

    def _setData(self):
        """Derived detector quantities (ExperimentalData.py:234-250)."""
        self.Nd = self.ptychogram.shape[-1]
        self.xd = np.linspace(-self.Nd / 2, self.Nd / 2, int(self.Nd)) * self.dxd
        self.Xd, self.Yd = np.meshgrid(self.xd, self.xd)
        self.Ld = self.Nd * self.dxd
        self.numFrames = self.ptychogram.shape[0]
        self.energyAtPos = np.sum(abs(self.ptychogram), (-1, -2))
        self.maxProbePower = np.sqrt(np.max(np.sum(self.ptychogram, (-1, -2))))

    def _move_data_to_cpu(self):
        """ExperimentalData.py:264-266.  The engines upload what they need
        into their own device buffers; the host arrays stay on the host."""

    def _move_data_to_gpu(self):
        """ExperimentalData.py:268-271: as ``_move_data_to_cpu``."""

    def relative_intensity(self, index):
        """Frame intensity relative to the brightest frames (ExperimentalData.py:273-288)."""
        if not hasattr(self, "_relative_intensity"):
            self._relative_intensity = self.ptychogram.mean((-2, -1))
            self._relative_intensity /= self._relative_intensity.mean() + 2 * self._relative_intensity.std()
        return self._relative_intensity[index]
