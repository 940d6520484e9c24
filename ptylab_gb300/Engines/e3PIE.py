"""e3PIE (multislice ePIE) on the GB300 kernels (PtyLab/Engines/e3PIE.py:29-225)."""

from __future__ import annotations

import numpy as np

from .. import _tables
from .BaseEngine import BaseEngine


class e3PIE(BaseEngine):
    engine_name = "e3PIE"

    def __init__(self, reconstruction, experimentalData, params, monitor):
        super().__init__(reconstruction, experimentalData, params, monitor)
        self.initializeReconstructionParams()

    def initializeReconstructionParams(self):
        """e3PIE.py:46-69: step sizes and the ifftshifted slice-to-slice
        angular-spectrum transfer function (dz, wavelength / refrIndex, Lp)."""
        self.betaProbe = 0.25
        self.betaObject = 0.25
        self.numIterations = 50
        rec = self.reconstruction
        rec.H = np.fft.ifftshift(self._slice_tf())

    def _slice_tf(self):
        rec = self.reconstruction
        Np = int(rec.Np)
        return _tables.multislice_tf(float(rec.dz), float(rec.wavelength), float(getattr(rec, "refrIndex", 1.0)),
                                     Np, Np * float(rec.dxp))

    def _check_supported(self):
        super()._check_supported()
        if int(self.reconstruction.nosm) != 1:
            raise NotImplementedError("e3PIE with object modes (nosm > 1) is not on this path")
        if int(self.reconstruction.nslice) > 6:
            raise NotImplementedError("e3PIE supports up to 6 slices")

    def _slice_table(self):
        return np.ascontiguousarray(self._slice_tf().astype(np.complex64))

    def reconstruct(self):
        """e3PIE.py:71-225: one kernel launch per iteration walks every position
        through the slices, the detector projection and back."""
        self._run_loop()

    def _finish(self):
        super()._finish()
        # product of all object slices (e3PIE.py:176)
        self.reconstruction.objectProd = np.prod(self.reconstruction.object, 3)
