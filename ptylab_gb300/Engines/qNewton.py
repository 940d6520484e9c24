"""qNewton on the GB300 kernels (PtyLab/Engines/qNewton.py:26-140)."""

from __future__ import annotations

from .BaseEngine import BaseEngine


class qNewton(BaseEngine):
    engine_name = "qNewton"

    def __init__(self, reconstruction, experimentalData, params, monitor):
        super().__init__(reconstruction, experimentalData, params, monitor)
        self.initializeReconstructionParams()

    def initializeReconstructionParams(self):
        """qNewton.py:43-52."""
        self.betaProbe = 1
        self.betaObject = 1
        self.regObject = 1
        self.regProbe = 1
        self.numIterations = 50

    def reconstruct(self, experimentalData=None):
        if experimentalData is not None:
            self.reconstruction.data = experimentalData
            self.experimentalData = experimentalData
        self._run_loop()
