"""Measurement container, mirroring PtyLab's ``ExperimentalData``
(PtyLab/ExperimentalData/ExperimentalData.py:21-288) for the fields the
reconstruction loop reads.  HDF5 loading is not part of this package: assign
the fields (or pass PtyLab's own ExperimentalData to the engines) and call
``_setData()``.
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
        """Only the in-memory stub dataset (ExperimentalData.py:101-115) is supported."""
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
        raise NotImplementedError(
            "HDF5 loading is outside this package; load with PtyLab or assign the fields and call _setData()"
        )

    def _setData(self):
        """Derived detector quantities (ExperimentalData.py:234-250)."""
        self.Nd = self.ptychogram.shape[-1]
        self.xd = np.linspace(-self.Nd / 2, self.Nd / 2, int(self.Nd)) * self.dxd
        self.Xd, self.Yd = np.meshgrid(self.xd, self.xd)
        self.Ld = self.Nd * self.dxd
        self.numFrames = self.ptychogram.shape[0]
        self.energyAtPos = np.sum(abs(self.ptychogram), (-1, -2))
        self.maxProbePower = np.sqrt(np.max(np.sum(self.ptychogram, (-1, -2))))

    def relative_intensity(self, index):
        """Frame intensity relative to the brightest frames (ExperimentalData.py:273-288)."""
        if not hasattr(self, "_relative_intensity"):
            self._relative_intensity = self.ptychogram.mean((-2, -1))
            self._relative_intensity /= self._relative_intensity.mean() + 2 * self._relative_intensity.std()
        return self._relative_intensity[index]
