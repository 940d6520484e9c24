"""ePIE on the GB300 kernels (PtyLab/Engines/ePIE.py:19-160)."""

from __future__ import annotations

from .BaseEngine import BaseEngine


class ePIE(BaseEngine):
    engine_name = "ePIE"

    def __init__(self, reconstruction, experimentalData, params, monitor):
        super().__init__(reconstruction, experimentalData, params, monitor)
        self.initializeReconstructionParams()

    def initializeReconstructionParams(self):
        """ePIE.py:35-42."""
        self.betaProbe = 0.25
        self.betaObject = 0.25
        self.numIterations = 50

    def reconstruct(self, experimentalData=None):
        """Run to completion: one kernel launch per iteration walks every position."""
        if experimentalData is not None:
            self.reconstruction.data = experimentalData
            self.experimentalData = experimentalData
        self._run_loop()

    def reconstruct_stepwise(self, experimentalData=None):
        """Generator variant (ePIE.py:53-126): yields ``(iteration, positionLoop)``
        after every position; each position is one kernel launch."""
        if experimentalData is not None:
            self.reconstruction.data = experimentalData
            self.experimentalData = experimentalData
        self._prepareReconstruction()
        nf = self.experimentalData.numFrames
        for loop in range(self.numIterations):
            self.setPositionOrder()
            self._upload_order()
            last = loop == self.numIterations - 1
            for positionLoop in range(nf):
                self._run_positions(positionLoop, 1, record_detector_error=last)
                yield loop, positionLoop
            self.getErrorMetrics()
            self.applyConstraints(loop)
        self._move_data_to_cpu(detector_error=self.numIterations > 0)
