"""Quasi-Newton gradient engine for multislice ptychography on the GB300 kernels.

The reference reconstructs multislice scans with e3PIE only
(PtyLab/Engines/e3PIE.py:29-225); this engine reconstructs the same model (the
object slices O_s and the entrance probe P: psi_0 = O_0[patch] P, psi_s =
ifft2(fft2(psi_{s-1}) H) O_s[patch], I = sum_modes |fft2c(psi_{S-1})|^2,
e3PIE.py:99-118) by steps along the gradient of the amplitude loss
L = sum (sqrt(I) - sqrt(I_meas))^2, taken with the hand-written adjoint of the
differentiable model (ptyg_multislice_amplitude_gradient) and scaled per pixel
the way qNewton scales its updates (qNewton.py:108-140):

    O_s += betaObject * sqrt(W_s / max W_s) / (W_s + regObject) * sum conj(u_s) DELTA_s
    P   += betaProbe  * sqrt(V / max V)     / (V + regProbe)    * sum conj(O_0) DELTA_0

with W_s the illumination of slice s (sum of |incident field|^2 over the
step's positions and modes), V the summed |O_0[patch]|^2, and DELTA the
back-propagated exit-wave correction (the gradient is -2 conj(.) DELTA).
For one position and one slice this is qNewton's object and probe step.
The positions of an iteration, in the order setPositionOrder draws, are taken
`batchSize` at a time: one step per batch, so batchSize = 1 is the
position-by-position form of the other engines.  Only the entrance probe is
reconstructed; the probe's further slices are left as given.

Every slice and the probe take their step at once against the same residual, so full
steps (qNewton's betas of 1) overshoot by about the number of slices; the
default betas are 0.5.  The entrance probe is first scaled to the data's
power, as PtyLab's probePowerCorrectionSwitch does once at the start
(PtyLab/Engines/BaseEngine.py:227-236): a probe far off the data's scale makes the
first steps diverge.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _native, _tables
from .BaseEngine import BaseEngine, _torch


class e3qNewton(BaseEngine):
    engine_name = "e3qNewton"

    def __init__(self, reconstruction, experimentalData, params, monitor):
        super().__init__(reconstruction, experimentalData, params, monitor)
        self.betaObject = 0.5
        self.betaProbe = 0.5
        self.regObject = 1.0
        self.regProbe = 1.0
        self.numIterations = 30
        self.batchSize = 64

    def _check_supported(self):
        p, rec = self.params, self.reconstruction
        if p.propagatorType.lower() != "fraunhofer":
            raise NotImplementedError("e3qNewton models a Fraunhofer detector")
        if p.fftshiftSwitch:
            raise NotImplementedError("e3qNewton runs with fftshiftSwitch = False")
        if int(rec.nosm) != 1 or int(getattr(rec, "nlambda", 1)) != 1:
            raise NotImplementedError("e3qNewton: one object mode and one wavelength")
        if self._projection_switches_on():
            raise NotImplementedError("e3qNewton runs the standard intensity projection only")
        if int(rec.Np) not in (32, 64, 128, 256):
            raise NotImplementedError("e3qNewton: Np must be 32, 64, 128 or 256")
        if int(self.batchSize) < 1:
            raise ValueError("batchSize must be at least 1")

    def _slice_table(self):
        rec = self.reconstruction
        Np = int(rec.Np)
        H = _tables.multislice_tf(float(getattr(rec, "dz", 0.0) or 0.0), float(rec.wavelength),
                                  float(getattr(rec, "refrIndex", 1.0)), Np, Np * float(rec.dxp))
        return np.ascontiguousarray(np.fft.ifftshift(H).astype(np.complex64))

    def reconstruct(self):
        self._begin()
        for loop in range(int(self.numIterations)):
            self._iterate(loop)
        self._end()

    def _begin(self):
        """Validation, and the state, data and step buffers on the GPU."""
        torch = _torch()
        self._prepare_host()
        rec, d = self.reconstruction, self.experimentalData
        if not self.params.probePowerCorrectionSwitch:  # (with the switch on, _prepare_host has done it)
            rec.probe = np.asarray(rec.probe) / np.sqrt(np.sum(np.abs(np.asarray(rec.probe)) ** 2)) * d.maxProbePower
        if not torch.cuda.is_available():
            raise ImportError("no CUDA device: the GB300 engines need an sm_103a GPU")
        dev = torch.device("cuda", torch.cuda.current_device())
        lib = _native.require(dev.index)
        Np, No, S, npsm = int(rec.Np), int(rec.No), int(rec.nslice), int(rec.npsm)
        nf = int(d.numFrames)
        obj_full = np.asarray(rec.object)
        prb_full = np.asarray(rec.probe)
        if obj_full.shape != (1, 1, 1, S, No, No) or prb_full.shape != (1, 1, npsm, S, Np, Np):
            raise ValueError(f"object {obj_full.shape} / probe {prb_full.shape} do not match the geometry")
        positions = np.asarray(rec.positions).astype(np.int64)
        if positions.min() < 0 or positions.max() > No - Np:
            raise ValueError(f"scan positions fall outside the {No}x{No} object (patch {Np})")
        self._positions_host = positions
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)  # noqa: E731
        B = min(int(self.batchSize), nf)
        geom = _native.Multislice(Np=Np, No=No, npsm=npsm, nslice=S, num_frames=B, chunk=B)
        ws_bytes = lib.ptyg_multislice_workspace_bytes(C.byref(geom))
        O = t(obj_full[0, 0, 0], torch.complex64)  # (S, No, No)
        P = t(prb_full[0, 0, :, 0], torch.complex64)  # (npsm, Np, Np)
        self._dev = {
            "device": dev, "lib": lib, "geom": geom, "B": B, "ws_bytes": ws_bytes,
            "O": O, "P": P, "obj_full": obj_full, "prb_full": prb_full,
            "pos": t(positions.astype(np.int32), torch.int32),
            "meas": t(d.ptychogram, torch.float32),
            "H": t(self._slice_table(), torch.complex64) if S > 1 else None,
            "ws": torch.empty(ws_bytes, dtype=torch.uint8, device=dev),
            "gO": torch.zeros_like(O), "gP": torch.zeros_like(P),
            "wO": torch.zeros(O.shape, dtype=torch.float32, device=dev),
            "wP": torch.zeros(P.shape, dtype=torch.float32, device=dev),
            "err": torch.zeros((max(int(self.numIterations), 1), nf), dtype=torch.float64, device=dev),
            "scratch": torch.zeros(64, dtype=torch.float32, device=dev),
            "order": torch.empty(nf, dtype=torch.int32, device=dev),
        }
        self._loops = 0

    def _iterate(self, loop):
        """One iteration: the host-drawn order, then one gradient pass and one
        quasi-Newton step of object slices and probe per batch of positions."""
        torch = _torch()
        D = self._dev
        lib, geom, B = D["lib"], D["geom"], D["B"]
        rec = self.reconstruction
        nf = int(self.experimentalData.numFrames)
        S, npsm, No, Np = int(rec.nslice), int(rec.npsm), int(rec.No), int(rec.Np)
        stream = torch.cuda.current_stream(D["device"]).cuda_stream
        if loop >= D["err"].shape[0]:
            D["err"] = torch.cat([D["err"], torch.zeros_like(D["err"])])
        err = D["err"][loop]
        self._err_n = loop  # iterations run so far (setPositionOrder's count of recorded errors)
        self.setPositionOrder()
        D["order"].copy_(torch.from_numpy(np.asarray(self.positionIndices, dtype=np.int32)))
        hptr = D["H"].data_ptr() if D["H"] is not None else None
        for first in range(0, nf, B):
            geom.num_frames = min(B, nf - first)
            _native.check(lib.ptyg_multislice_amplitude_gradient(
                C.byref(geom), D["O"].data_ptr(), D["P"].data_ptr(), D["pos"].data_ptr(), hptr,
                D["order"].data_ptr() + 4 * first, D["meas"].data_ptr(), D["gO"].data_ptr(), D["gP"].data_ptr(),
                D["wO"].data_ptr(), D["wP"].data_ptr(), err.data_ptr(), D["ws"].data_ptr(), D["ws_bytes"], stream),
                "ptyg_multislice_amplitude_gradient")
            _native.check(lib.ptyg_qn_step(D["O"].data_ptr(), D["gO"].data_ptr(), D["wO"].data_ptr(), S, No * No,
                                           float(self.betaObject), float(self.regObject), D["scratch"].data_ptr(),
                                           stream), "ptyg_qn_step")
            _native.check(lib.ptyg_qn_step(D["P"].data_ptr(), D["gP"].data_ptr(), D["wP"].data_ptr(), npsm, Np * Np,
                                           float(self.betaProbe), float(self.regProbe), D["scratch"].data_ptr(),
                                           stream), "ptyg_qn_step")
        self._loops = loop + 1

    def _end(self):
        """Errors and the reconstruction back to the host as NumPy arrays."""
        torch = _torch()
        D = self._dev
        rec = self.reconstruction
        torch.cuda.current_stream(D["device"]).synchronize()
        self._err_n = 0
        for row in D["err"][: self._loops].cpu().numpy():
            self._append_errors(row)
        obj_full = D["obj_full"].astype(np.complex64, copy=True)
        prb_full = D["prb_full"].astype(np.complex64, copy=True)
        obj_full[0, 0, 0] = D["O"].cpu().numpy()
        prb_full[0, 0, :, 0] = D["P"].cpu().numpy()
        rec.object, rec.probe = obj_full, prb_full
        rec.objectProd = np.prod(rec.object, 3)
        self._dev = {}
