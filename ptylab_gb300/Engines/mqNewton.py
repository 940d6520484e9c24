"""mqNewton on the GB300 kernels (PtyLab/Engines/mqNewton.py:26-251).

qNewton's object and probe steps (identical to qNewton.py:108-140), followed
after every position by a momentum step on the whole object and the whole
probe: plain momentum, ADAM or NADAM (``momentum_method``,
mqNewton.py:142-224).  The kernel runs the step over the object in the same
launch as the position loop.

In the reference the second moments ``objectMomentum_v`` / ``probeMomentum_v``
are arrays that start as copies of the first moments (zero for a fresh engine)
and gain the same real scalar in every element at every ADAM/NADAM step, so
the kernel carries one float32 per scan for the object and one for the probe;
they are written back as full arrays.  A second ``reconstruct()`` on the same
engine seeds them from the non-zero first moments (mqNewton.py:75-79), which
makes them non-uniform: that case raises NotImplementedError.
"""

from __future__ import annotations

import logging

import numpy as np

from .. import _native
from .BaseEngine import BaseEngine, _torch


class mqNewton(BaseEngine):
    engine_name = "mqNewton"

    def __init__(self, reconstruction, experimentalData, params, monitor):
        super().__init__(reconstruction, experimentalData, params, monitor)
        self.logger = logging.getLogger("mqNewton")
        self.initializeReconstructionParams()
        rec = self.reconstruction
        # Reconstruction.initializeObjectMomentum / initializeProbeMomentum
        # (Reconstruction.py:416-420) and the buffers (mqNewton.py:43-47)
        rec.objectMomentum = np.zeros_like(rec.initialGuessObject)
        rec.probeMomentum = np.zeros_like(rec.initialGuessProbe)
        rec.objectBuffer = np.array(rec.object, copy=True)
        rec.probeBuffer = np.array(rec.probe, copy=True)
        self.params.momentumAcceleration = True

    def initializeReconstructionParams(self):
        """mqNewton.py:50-66."""
        self.betaProbe = 1
        self.betaObject = 1
        self.regObject = 1
        self.regProbe = 1
        self.beta1 = 0.5
        self.beta2 = 0.5
        self.betaProbe_m = 0.25
        self.betaObject_m = 0.25
        self.feedbackM = 0.3
        self.frictionM = 0.7
        self.momentum_method = "ADAM"
        self.numIterations = 50

    def initializeAdaptiveMomentum(self):
        """mqNewton.py:68-79: resolve the method by name; ADAM and NADAM start
        their second moments from copies of the first moments."""
        method = self.momentum_method
        if method not in _native.MOMENTUM_METHODS:
            raise AttributeError(f"type object 'mqNewton' has no momentum method {method!r}")
        self.logger.info("Momentum mqNewton used: %s", method)
        if method in ("ADAM", "NADAM"):
            rec = self.reconstruction
            rec.objectMomentum_v = _host_copy(rec.objectMomentum)
            rec.probeMomentum_v = _host_copy(rec.probeMomentum)

    def _state_fields(self):
        return ["object", "probe", "objectBuffer", "probeBuffer", "objectMomentum", "probeMomentum"]

    def _second_moments(self):
        """The scalar every element of objectMomentum_v / probeMomentum_v holds."""
        rec = self.reconstruction
        out = []
        for name in ("objectMomentum_v", "probeMomentum_v"):
            if self.momentum_method == "momentum":
                out.append(0.0)
                continue
            v = np.asarray(getattr(rec, name)).ravel()
            v0 = v[0] if v.size else np.complex64(0)
            if v.size and (np.any(v != v0) or np.imag(v0) != 0):
                raise NotImplementedError(
                    f"{name} is not a uniform real array (a second reconstruct() seeds it from the first "
                    "moments, mqNewton.py:75-79); the GB300 mqNewton carries the second moment as one "
                    "scalar: reset objectMomentum and probeMomentum to zero before reconstructing again"
                )
            out.append(float(np.float32(np.real(v0))))
        return out

    def _scan_buffers(self):
        b = super()._scan_buffers()
        rec = self.reconstruction
        b.object_momentum = rec.objectMomentum.data_ptr()
        b.probe_buffer = rec.probeBuffer.data_ptr()
        b.probe_momentum = rec.probeMomentum.data_ptr()
        b.second_moment = self._dev["moment2"].data_ptr()
        return b

    def _update_params(self):
        u = super()._update_params()
        u.momentum_method = _native.MOMENTUM_METHODS[self.momentum_method]
        u.beta1 = float(self.beta1)
        u.beta2 = float(self.beta2)
        itr = self._loop + 1  # mqNewton.py:121-122 pass loop + 1
        u.beta1_scale = float(np.float32(1 - self.beta1**itr))
        u.beta2_scale = float(np.float32(1 - self.beta2**itr))
        u.beta_object_m = float(self.betaObject_m)
        u.beta_probe_m = float(self.betaProbe_m)
        return u

    def _device_extras(self):
        torch = _torch()
        self._dev["moment2"] = torch.tensor(self._second_moments(), dtype=torch.float32, device=self._dev["device"])

    def reconstruct(self, experimentalData=None):
        if experimentalData is not None:
            self.reconstruction.data = experimentalData
            self.experimentalData = experimentalData
        self._run_loop()

    def _pre_prepare(self):
        self.initializeAdaptiveMomentum()
        rec = self.reconstruction
        if not np.array_equal(_host_copy(rec.objectBuffer), _host_copy(rec.object)):
            raise NotImplementedError(
                "objectBuffer differs from the object: the GB300 mqNewton keeps them equal (the object was "
                "changed after the engine was built; build the engine again)"
            )
        self._loop = 0

    def _loop_order(self, loop):
        self._loop = loop
        super()._loop_order(loop)

    def _finish(self):
        rec = self.reconstruction
        # the buffers equal the object and probe after the last step
        # (mqNewton.py:203, 224); the kernel keeps only the probe buffer
        rec.objectBuffer.copy_(rec.object)
        vO, vP = (float(x) for x in self._dev["moment2"].cpu())
        super()._finish()
        if self.momentum_method in ("ADAM", "NADAM"):
            rec.objectMomentum_v = np.full(rec.objectMomentum.shape, np.complex64(vO))
            rec.probeMomentum_v = np.full(rec.probeMomentum.shape, np.complex64(vP))


def _host_copy(x):
    """A NumPy copy of a host array or a torch tensor."""
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy().copy()
    return np.array(x, copy=True)
