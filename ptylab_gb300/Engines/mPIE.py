"""mPIE on the GB300 kernels (PtyLab/Engines/mPIE.py:29-270).

The momentum step fires after a position when ``np.random.rand(1) > 0.95``
(mPIE.py:170).  The draws for an iteration are taken on the host right after
that iteration's position shuffle, in position order, which consumes the
global RNG exactly like the reference's per-position draws, and passed to the
kernel as one flag byte per position.
"""

from __future__ import annotations

import numpy as np

from .BaseEngine import BaseEngine, _torch


class mPIE(BaseEngine):
    engine_name = "mPIE"

    def __init__(self, reconstruction, experimentalData, params, monitor):
        super().__init__(reconstruction, experimentalData, params, monitor)
        self.initializeReconstructionParams()
        self.params.momentumAcceleration = True
        self.name = "mPIE"

    def initializeReconstructionParams(self):
        """mPIE.py:73-94."""
        self.betaProbe = 0.25
        self.betaObject = 0.25
        self.alphaProbe = 0.1
        self.alphaObject = 0.1
        self.feedbackM = 0.3
        self.frictionM = 0.7
        self.numIterations = 50
        rec = self.reconstruction
        rec.objectMomentum = np.zeros_like(rec.initialGuessObject)
        rec.probeMomentum = np.zeros_like(rec.initialGuessProbe)
        rec.objectBuffer = np.array(rec.object, copy=True)
        rec.probeBuffer = np.array(rec.probe, copy=True)
        rec.probeWindow = np.abs(np.asarray(rec.probe))

    def _check_supported(self):
        super()._check_supported()
        if getattr(self.params, "weigh_probe_updates_by_intensity", False):
            raise NotImplementedError("weigh_probe_updates_by_intensity is not supported by the GB300 mPIE")
        if hasattr(self, "patches"):
            raise NotImplementedError("keepPatches is not supported by the GB300 mPIE")

    def _state_fields(self):
        return ["object", "probe", "objectBuffer", "probeBuffer", "objectMomentum", "probeMomentum"]

    def _scan_buffers(self):
        b = super()._scan_buffers()
        rec = self.reconstruction
        b.object_buffer = rec.objectBuffer.data_ptr()
        b.object_momentum = rec.objectMomentum.data_ptr()
        b.probe_buffer = rec.probeBuffer.data_ptr()
        b.probe_momentum = rec.probeMomentum.data_ptr()
        return b

    def reconstruct(self, experimentalData=None, reconstruction=None, vis_after_each_iteration=None):
        self.changeExperimentalData(experimentalData)
        self.changeOptimizable(reconstruction)
        self._vis = vis_after_each_iteration
        self._run_loop()

    def _loop_begin(self):
        # buffers follow the object/probe as they stand after preparation (mPIE.py:103-105)
        rec = self.reconstruction
        rec.objectBuffer.copy_(rec.object)
        rec.probeBuffer.copy_(rec.probe)

    def _loop_order(self, loop):
        self.setPositionOrder()
        draws = np.random.rand(self.experimentalData.numFrames)
        self._upload_order(momentum=draws > 0.95)

    def _loop_end(self, loop):
        super()._loop_end(loop)
        vis = getattr(self, "_vis", None)
        if callable(vis):
            self._resolve_errors()  # the callback sees this iteration's error
            vis(loop, self.reconstruction)
