"""Host control of the GB300 engines, mirroring PtyLab's ``BaseEngine``
(PtyLab/Engines/BaseEngine.py:69-1858) for the per-position path.

What stays on the host, as in the reference: switch validation, the
fftshift of the data, the position order (same NumPy calls, same global RNG),
the per-iteration error metric and the in-scope constraints.  What moves to
the GPU: the whole walk over the scan positions of an iteration, which is one
``ptyg_plan_run`` launch (libptyg.so, sm_103a), and the constraint kernels.

State lives in torch CUDA tensors while ``reconstruct()`` runs
(``reconstruction.object`` / ``.probe`` and, for mPIE, the buffers and
momenta are replaced by device tensors, as the reference replaces them by CuPy
arrays) and is written back as NumPy complex64 arrays at the end
(ePIE.py:123-126).  There is no CPU code path: without libptyg.so and an
sm_103a device every engine raises ImportError.
"""

from __future__ import annotations

import ctypes as C
import logging

import numpy as np

from .. import _native, _tables
from ..Reconstruction import circ

_UPLOAD_SLOTS = 3  # iterations the host may queue ahead of the GPU

# Switches whose branches are not on this path; PtyLab default for all is off.
_UNSUPPORTED = (
    "CPSCswitch",
    "positionCorrectionSwitch",
    "OPRP",
    "objectTVregSwitch",
    "modulusEnforcedProbeSwitch",
    "l2reg",
    "probeSpectralPowerCorrectionSwitch",
    "probeSmoothenessSwitch",
    "objectSmoothenessSwitch",
    "absObjectSwitch",
    "absProbeSwitch",
    "objectContrastSwitch",
    "couplingSwitch",
    "binaryProbeSwitch",
    "PSDestimationSwitch",
    "TV_autofocus",
    "map_position_to_z_change",
)


def _host(x):
    """A NumPy view of a host array or a torch tensor."""
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _torch():
    import torch

    return torch


class BaseEngine(object):
    engine_name = "BaseEngine"
    _err_n = 0  # iterations whose frame sums wait on the device (_record_errors)
    _err_dev = None
    _batch = None  # the shared per-iteration state of reconstruct_batch (Engines/batch.py)
    _batch_row = 0

    def __init__(self, reconstruction, experimentalData, params, monitor):
        self.betaObject = 0.25
        self.reconstruction = reconstruction
        self.experimentalData = experimentalData
        self.params = params
        self.monitor = monitor
        try:
            self.monitor.reconstruction = reconstruction
        except AttributeError:
            pass
        self.logger = logging.getLogger(self.engine_name)
        self._plan = None
        self._owns_plan = True
        self._scan = 0  # this engine's scan in the (possibly shared) launch plan
        self._dev = {}

    # --------------------------------------------------------- validation
    def _check_supported(self):
        p, rec = self.params, self.reconstruction
        ic = p.intensityConstraint
        if ic == "interferometric":
            if self.engine_name not in ("ePIE", "mPIE", "qNewton"):
                raise NotImplementedError("the interferometric constraint runs with the GB300 ePIE, mPIE and qNewton")
            if p.propagatorType.lower() not in ("fraunhofer", "fresnel"):
                raise NotImplementedError("the interferometric constraint runs with the Fraunhofer and Fresnel propagators")
        if ic not in _native.INTENSITY_CONSTRAINTS:
            raise ValueError("intensity constraint not properly specified!")  # BaseEngine.py:963-964
        if ic == "fluctuation" and not hasattr(p, "intensityScaling"):
            # the reference writes params.intensityScaling[positionIndex] (BaseEngine.py:931),
            # which Params never creates: the caller must provide it
            raise AttributeError("'Params' object has no attribute 'intensityScaling'")
        if p.FourierMaskSwitch and getattr(self.experimentalData, "W", None) is None:
            raise ValueError("FourierMaskSwitch needs experimentalData.W")
        if getattr(p, "intensityMask", False) and getattr(rec, "intensity_mask", None) is None:
            raise ValueError("params.intensityMask needs reconstruction.intensity_mask")
        if ic == "interferometric" and self.engine_name == "e3PIE":
            raise NotImplementedError("the GB300 e3PIE runs every projection switch but the interferometric constraint")
        for name in _UNSUPPORTED:
            if getattr(p, name, False):
                raise NotImplementedError(f"params.{name} is not supported by the GB300 engines")
        if getattr(p, "comStabilizationSwitch", None) not in (None, False):
            raise NotImplementedError("params.comStabilizationSwitch is not supported by the GB300 engines")
        nl = int(getattr(rec, "nlambda", 1))
        if nl != 1 and self.engine_name not in ("ePIE", "mPIE", "qNewton", "mqNewton"):
            raise NotImplementedError(f"nlambda = {nl}: several wavelengths run with the GB300 ePIE, mPIE, qNewton and mqNewton")
        if nl != 1 and getattr(p, "orthogonalizationSwitch", False):
            raise NotImplementedError("orthogonalizationSwitch with several wavelengths is not on this path")
        kind = p.propagatorType.lower()
        if kind not in ("fraunhofer", "fresnel", "asp", "polychromeasp"):
            raise NotImplementedError(f"propagatorType {p.propagatorType!r} is not on this path")
        if kind == "asp" and nl > 1:  # Operators.py:866-869
            raise ValueError("For multi-wavelength, polychromeASP needs to be used instead of ASP")
        if kind == "polychromeasp" and np.atleast_1d(rec.spectralDensity).size < nl:
            raise ValueError(f"reconstruction.spectralDensity holds fewer than nlambda = {nl} wavelengths")

    def _checkMISC(self):
        """BaseEngine.py:376-403."""
        if self.params.probePowerCorrectionSwitch and self.params.modulusEnforcedProbeSwitch:
            raise ValueError(
                "probePowerCorrectionSwitch and modulusEnforcedProbeSwitch can not simultaneously be switched on!"
            )
        if self.params.propagatorType.lower() in ("asp", "polychromeasp") and self.params.fftshiftSwitch:
            raise ValueError("ASP propagatorType works only with fftshiftSwitch = False")
        rec = self.reconstruction
        if self.params.backgroundModeSwitch:  # BaseEngine.py:361-364
            rec.background = 1e-1 * np.ones((rec.Np, rec.Np))
        if self.params.intensityConstraint == "fluctuation":  # BaseEngine.py:367-369
            self.intensityScaling = np.ones(self.experimentalData.numFrames)
        if self.params.intensityConstraint == "interferometric":  # BaseEngine.py:371-374
            rec.reference = np.ones((int(rec.Np), int(rec.Np)))

    def _projection_switches_on(self):
        p = self.params
        return (p.intensityConstraint != "standard" or p.adaptiveDenoisingSwitch or p.backgroundModeSwitch
                or p.FourierMaskSwitch or bool(getattr(p, "intensityMask", False)))

    def _checkFFT(self):
        """Shift the data once so the uncentred transform applies (BaseEngine.py:405-450)."""
        d = self.experimentalData
        W = getattr(d, "W", None)
        if self.params.fftshiftSwitch:
            if self.params.fftshiftFlag == 0:
                d.ptychogram = np.fft.ifftshift(d.ptychogram, axes=(-1, -2))
                if W is not None:
                    d.W = np.fft.ifftshift(W, axes=(-1, -2))
                self.params.fftshiftFlag = 1
        else:
            if self.params.fftshiftFlag == 1:
                d.ptychogram = np.fft.fftshift(d.ptychogram, axes=(-1, -2))
                if W is not None:
                    d.W = np.fft.fftshift(W, axes=(-1, -2))
                self.params.fftshiftFlag = 0

    def _initialProbePowerCorrection(self):
        if self.params.probePowerCorrectionSwitch:
            rec = self.reconstruction
            rec.probe = (
                rec.probe / np.sqrt(np.sum(rec.probe * rec.probe.conj())) * self.experimentalData.maxProbePower
            )

    def _probeWindow(self):
        """BaseEngine.py:237-266."""
        rec = self.reconstruction
        self.probeWindow = None
        if not self.params.saveMemory or self.params.absorbingProbeBoundary:
            self.probeWindow = np.exp(
                -(((rec.Xp**2 + rec.Yp**2) / (2 * (3 / 4 * rec.Np * rec.dxp / 2.355) ** 2)) ** 10)
            )
        if self.params.probeBoundary:
            d = self.experimentalData.entrancePupilDiameter
            self.probeWindow = circ(rec.Xp, rec.Yp, d + d * 0.2)

    def _initializeErrors(self):
        """BaseEngine.py:199-225; detectorError is filled at the end of the run."""
        rec = self.reconstruction
        if self.params.saveMemory:
            rec.detectorError = 0
        if not hasattr(rec, "errorAtPos"):
            rec.errorAtPos = np.zeros((self.experimentalData.numFrames, 1), dtype=np.float32)
        if not hasattr(rec, "error"):
            rec.error = []

    def _prepareReconstruction(self):
        self._prepare_host()
        self._checkGPU()

    def _prepare_host(self):
        """BaseEngine._prepareReconstruction (BaseEngine.py:96-111) up to the device move."""
        self._check_supported()
        self._checkMISC()
        self._checkFFT()
        self._initialProbePowerCorrection()
        self._probeWindow()
        self._initializeErrors()

    # --------------------------------------------------------- device state
    def _engine_code(self):
        return _native.ENGINES[self.engine_name]

    def _state_fields(self):
        return ["object", "probe"]

    def _to_device(self, x, dtype):
        torch = _torch()
        dev = self._dev["device"]
        if isinstance(x, torch.Tensor):
            return x.to(device=dev, dtype=dtype).contiguous()
        return torch.from_numpy(np.ascontiguousarray(np.asarray(x))).to(device=dev, dtype=dtype)

    def _checkGPU(self):
        """Move the state to the GPU and build the launch plan (BaseEngine.py:613-635)."""
        self._device_state()
        self._plan_and_bind()

    def _host_state(self):
        """What the device path takes from PtyLab's objects, read and checked
        on the host: the state arrays (object, probe, and the engine's
        buffers), the scan positions and the ptychogram, as NumPy arrays.  The
        engines read nothing else from the objects on the way to the GPU but
        the scalars of _geometry, _update_params and _host_tables."""
        rec, d = self.reconstruction, self.experimentalData
        Np, No = int(rec.Np), int(rec.No)
        nosm, npsm, nslice = int(rec.nosm), int(rec.npsm), int(rec.nslice)
        nl = int(getattr(rec, "nlambda", 1))
        # (a state array that is already a torch tensor is passed through as it
        # is; NumPy arrays of the right dtype are not copied: everything here
        # is only read, on its way to the GPU)
        out = {}
        for name in self._state_fields():
            v = getattr(rec, name)
            out[name] = v if hasattr(v, "detach") else np.asarray(v).astype(np.complex64, copy=False)
        if tuple(out["object"].shape) != (nl, nosm, 1, nslice, No, No):
            raise ValueError(f"object shape {tuple(out['object'].shape)} != {(nl, nosm, 1, nslice, No, No)}")
        if tuple(out["probe"].shape) != (nl, 1, npsm, nslice, Np, Np):
            raise ValueError(f"probe shape {tuple(out['probe'].shape)} != {(nl, 1, npsm, nslice, Np, Np)}")
        nf = int(d.numFrames)
        positions = np.asarray(rec.positions).astype(np.int64)
        if positions.shape != (nf, 2):
            raise ValueError(f"positions shape {positions.shape} != {(nf, 2)}")
        if positions.min() < 0 or positions.max() > No - Np:
            raise ValueError(f"scan positions fall outside the {No}x{No} object (patch {Np})")
        out["positions"] = positions
        out["ptychogram"] = np.asarray(_host(d.ptychogram)).astype(np.float32, copy=False)
        return out

    def _device_state(self):
        """The reconstruction state, data, positions and order buffers on the GPU."""
        torch = _torch()
        if not getattr(self.params, "gpuSwitch", True):
            self.logger.warning("params.gpuSwitch is False; the GB300 engines always run on the GPU")
        if not torch.cuda.is_available():
            raise ImportError("no CUDA device: the GB300 engines need an sm_103a GPU")
        device = torch.device("cuda", torch.cuda.current_device())
        lib = _native.require(device.index)
        rec, d, p = self.reconstruction, self.experimentalData, self.params
        host = self._host_state()
        self._dev = {"device": device, "lib": lib}
        for name in self._state_fields():
            setattr(rec, name, self._to_device(host[name], torch.complex64))
        nf = int(d.numFrames)
        positions = host["positions"]
        self._positions_host = positions
        self._dev["positions"] = torch.from_numpy(positions.astype(np.int32)).to(device)
        self._dev["data"] = self._to_device(host["ptychogram"], torch.float32)
        self._dev["order"] = torch.zeros(nf, dtype=torch.int32, device=device)
        self._dev["flags"] = torch.zeros(nf, dtype=torch.uint8, device=device)
        # a ring of pinned staging buffers for the per-iteration order and
        # momentum flags: the host fills slot n while the copies of earlier
        # iterations may still be queued; slot n's event (its last copy)
        # is waited on before the slot is reused.  Allocated at the first
        # upload (a batch stages every scan's rows in its own ring instead)
        self._upload_ring = None
        self._upload_events = [None] * _UPLOAD_SLOTS
        self._uploads = 0
        self._err_dev = None  # per-iteration frame sums awaiting readback
        self._err_n = 0

    def _geometry(self, num_scans=1, throughput=0):
        rec, d, p = self.reconstruction, self.experimentalData, self.params
        return _native.Geometry(
            Np=int(rec.Np), No=int(rec.No), nosm=int(rec.nosm), npsm=int(rec.npsm), nslice=int(rec.nslice),
            num_frames=int(d.numFrames), num_scans=num_scans, engine=self._engine_code(),
            propagator=_native.PROPAGATORS[p.propagatorType.lower()], fftshift=int(bool(p.fftshiftSwitch)),
            fpm=int(d.operationMode == "FPM"), cluster=int(getattr(self, "cluster", 0) or 0), throughput=throughput,
            threads=int(getattr(self, "threads", 0) or 0),
            nlambda=int(getattr(rec, "nlambda", 1)),
            asp_table_in_smem=int(getattr(self, "aspTableInSmem", 0) or 0),
        )

    def _plan_and_bind(self, plan=None, scan=0, num_scans=1, throughput=0):
        """Create the launch plan (or join `plan` as scan `scan`) and bind this
        engine's buffers to it."""
        lib = self._dev["lib"]
        self._release_plan()
        if plan is None:
            plan = C.c_void_p()
            _native.check(lib.ptyg_plan_create(C.byref(self._geometry(num_scans, throughput)), C.byref(plan)),
                          "ptyg_plan_create")
            self._owns_plan = True
            self._plan, self._scan = plan, scan
            self._set_tables()
        else:
            self._owns_plan = False
            self._plan, self._scan = plan, scan
        self._set_projection()
        self._device_extras()
        self._bind()
        self.params.gpuFlag = 1

    def _host_tables(self):
        """The propagator tables the plan takes (Fresnel chirp, ASP transfer
        function(s), slice transfer function), computed on the host."""
        rec, p = self.reconstruction, self.params
        Np = int(rec.Np)
        q = h = sh = None
        kind = p.propagatorType.lower()
        if kind == "fresnel":
            q = np.ascontiguousarray(
                _tables.fresnel_chirp(float(rec.zo), float(rec.wavelength), Np, float(rec.dxp)).astype(np.complex64)
            )
        elif kind == "asp":
            h = np.ascontiguousarray(_tables.asp_detector_tf(float(rec.zo), float(rec.wavelength), Np, Np * float(rec.dxp)))
        elif kind == "polychromeasp":
            # one transfer function per wavelength of spectralDensity (Operators.py:909-951)
            wl = tuple(float(w) for w in np.atleast_1d(rec.spectralDensity)[: int(rec.nlambda)])
            h = np.ascontiguousarray(_tables.polychrome_asp_tf(float(rec.zo), wl, Np, Np * float(rec.dxp)))
        return q, h, self._slice_table()

    def _set_tables(self):
        lib = self._dev["lib"]
        q, h, sh = self._host_tables()
        self._tables_keepalive = (q, h, sh)
        ptr = lambda a: a.ctypes.data if a is not None else None  # noqa: E731
        _native.check(lib.ptyg_plan_set_tables(self._plan, ptr(q), ptr(h), ptr(sh)), "ptyg_plan_set_tables")

    def _set_projection(self):
        """The projection switches and their tables (BaseEngine.py:870-1012)."""
        if not self._projection_switches_on():
            return
        torch = _torch()
        p, rec, d = self.params, self.reconstruction, self.experimentalData
        lib = self._dev["lib"]
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        mask_on = bool(getattr(p, "intensityMask", False))
        pr = _native.Projection(
            intensity_constraint=_native.INTENSITY_CONSTRAINTS[p.intensityConstraint],
            adaptive_denoising=int(bool(p.adaptiveDenoisingSwitch)), background_mode=int(bool(p.backgroundModeSwitch)),
            fourier_mask=int(bool(p.FourierMaskSwitch)), intensity_mask=int(mask_on),
        )
        tab = lambda a: self._to_device(np.broadcast_to(np.asarray(a, dtype=np.float32), (rec.Np, rec.Np)), torch.float32)  # noqa: E731
        W = tab(d.W) if p.FourierMaskSwitch else None
        M = tab(_host(rec.intensity_mask)) if mask_on else None
        self._dev["W"], self._dev["intensity_mask"] = W, M
        _native.check(
            lib.ptyg_plan_set_projection(self._plan, C.byref(pr), W.data_ptr() if W is not None else None,
                                         M.data_ptr() if M is not None else None, stream),
            "ptyg_plan_set_projection",
        )
        if p.backgroundModeSwitch:
            bg = tab(rec.background)
            self._dev["background"] = bg
            _native.check(lib.ptyg_plan_set_background(self._plan, self._scan, bg.data_ptr(), stream), "ptyg_plan_set_background")

    def _slice_table(self):
        return None

    def _device_extras(self):
        """Engine-specific device state created before the scan is bound."""

    def _scan_buffers(self):
        rec = self.reconstruction
        b = _native.ScanBuffers()
        b.object = rec.object.data_ptr()
        b.probe = rec.probe.data_ptr()
        b.positions = self._dev["positions"].data_ptr()
        b.order = self._dev["order"].data_ptr()
        b.momentum_flags = self._dev["flags"].data_ptr()
        return b

    def _bind(self):
        torch = _torch()
        lib = self._dev["lib"]
        self._buffers = self._scan_buffers()
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        _native.check(
            lib.ptyg_plan_bind_scan(self._plan, self._scan, C.byref(self._buffers), self._dev["data"].data_ptr(), stream),
            "ptyg_plan_bind_scan",
        )

    def _release_plan(self):
        if self._plan is not None and self._plan.value and self._owns_plan:
            _native.load_library().ptyg_plan_destroy(self._plan)
        self._plan = None

    def __del__(self):
        try:
            self._release_plan()
        except Exception:
            pass

    def _update_params(self):
        u = _native.UpdateParams()
        u.beta_object = float(self.betaObject)
        u.beta_probe = float(getattr(self, "betaProbe", 0.25))
        u.alpha_object = float(getattr(self, "alphaObject", 0.1))
        u.alpha_probe = float(getattr(self, "alphaProbe", 0.1))
        u.reg_object = float(getattr(self, "regObject", 1.0))
        u.reg_probe = float(getattr(self, "regProbe", 1.0))
        u.friction = float(getattr(self, "frictionM", 0.7))
        u.feedback = float(getattr(self, "feedbackM", 0.3))
        u.probe_weight = 1.0
        u.slice_beta = 0.9
        return u

    def _upload_order(self, momentum=None):
        if self._batch is not None:  # staged for the batch's one copy
            self._batch.stage(self._batch_row, self.positionIndices, momentum)
            return
        torch = _torch()
        if self._upload_ring is None:
            nf = int(self.experimentalData.numFrames)
            self._upload_ring = [
                (torch.zeros(nf, dtype=torch.int32).pin_memory(), torch.zeros(nf, dtype=torch.uint8).pin_memory())
                for _ in range(_UPLOAD_SLOTS)
            ]
        slot = self._uploads % _UPLOAD_SLOTS
        if self._upload_events[slot] is not None:
            self._upload_events[slot].synchronize()
        order_host, flags_host = self._upload_ring[slot]
        order_host.copy_(torch.from_numpy(np.asarray(self.positionIndices, dtype=np.int32)))
        self._dev["order"].copy_(order_host, non_blocking=True)
        if momentum is not None:
            flags_host.copy_(torch.from_numpy(np.asarray(momentum, dtype=np.uint8)))
            self._dev["flags"].copy_(flags_host, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self._dev["device"]))
        self._upload_events[slot] = ev
        self._uploads += 1

    def _run_positions(self, start, count, record_detector_error=False):
        torch = _torch()
        lib = self._dev["lib"]
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        u = self._update_params()
        _native.check(
            lib.ptyg_plan_run(self._plan, C.byref(u), int(start), int(count), int(bool(record_detector_error)), stream),
            "ptyg_plan_run",
        )

    # ------------------------------------------------------ the iteration loop
    # reconstruct() = prepare; _loop_begin; per iteration: _loop_order, one
    # launch over every position, _loop_end; _finish.  reconstruct_batch()
    # runs the same hooks for many engines sharing one launch.
    def _pre_prepare(self):
        """Engine set-up that PtyLab does before _prepareReconstruction."""

    def _loop_begin(self):
        """After the device move, before the first iteration."""

    def _loop_order(self, loop):
        self.setPositionOrder()
        self._upload_order()

    def _loop_end(self, loop):
        self._record_errors()
        self.applyConstraints(loop)
        self.showReconstruction(loop)

    def _finish(self):
        self._resolve_errors()
        self._move_data_to_cpu(detector_error=self.numIterations > 0)

    def _run_loop(self):
        self._pre_prepare()
        self._prepareReconstruction()
        self._loop_begin()
        nf = self.experimentalData.numFrames
        for loop in range(self.numIterations):
            self._loop_order(loop)
            self._run_positions(0, nf, record_detector_error=(loop == self.numIterations - 1))
            self._loop_end(loop)
        self._finish()

    # ------------------------------------------------------ host control
    def setPositionOrder(self):
        """BaseEngine.py:637-665 (same NumPy calls, same global RNG)."""
        nf = self.experimentalData.numFrames
        order = self.params.positionOrder
        if order == "sequential":
            self.positionIndices = np.arange(nf)
        elif order == "random":
            self.positionIndices = np.arange(nf)
            if len(self.reconstruction.error) + self._err_n >= 2:
                np.random.shuffle(self.positionIndices)
        elif order == "NA":
            pos = self._positions_host
            rows = pos[:, 0] - np.mean(pos[:, 0])
            cols = pos[:, 1] - np.mean(pos[:, 1])
            self.positionIndices = np.argsort(np.sqrt(rows**2 + cols**2))
        else:
            raise ValueError("position order not properly set")

    def getErrorMetrics(self):
        """BaseEngine.py:819-841, from the per-frame FP64 sums of |I_meas - I_est|."""
        torch = _torch()
        self._resolve_errors()
        nf = self.experimentalData.numFrames
        err = np.empty(nf, dtype=np.float64)
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        _native.check(
            self._dev["lib"].ptyg_plan_frame_errors(self._plan, self._scan, err.ctypes.data, stream), "ptyg_plan_frame_errors"
        )
        self._append_errors(err)

    def _record_errors(self):
        """getErrorMetrics without waiting for the GPU: this iteration's
        per-frame sums go to a device row (queued on the stream), and
        _resolve_errors turns the rows into rec.errorAtPos and rec.error in
        iteration order once, so the host can queue the next iteration while
        this one runs."""
        if self._batch is not None:  # the batch sums every scan's frames in one launch
            return
        torch = _torch()
        nf = self.experimentalData.numFrames
        if self._err_dev is None or self._err_n == self._err_dev.shape[0]:
            grown = torch.empty((max(int(self.numIterations), 1) + self._err_n, nf), dtype=torch.float64,
                                device=self._dev["device"])
            if self._err_n:
                grown[: self._err_n].copy_(self._err_dev[: self._err_n])
            self._err_dev = grown
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        _native.check(
            self._dev["lib"].ptyg_plan_frame_errors_device(self._plan, self._scan, self._err_dev[self._err_n].data_ptr(),
                                                           stream),
            "ptyg_plan_frame_errors_device",
        )
        self._err_n += 1

    def _resolve_errors(self):
        if not self._err_n:
            return
        rows = self._err_dev[: self._err_n].cpu().numpy()
        if self._batch is not None:
            self._err_dev = self._err_dev[self._err_n :]  # the batch's later rows
        self._err_n = 0
        for err in rows:
            self._append_errors(err)

    def _append_errors(self, err):
        rec = self.reconstruction
        nf = self.experimentalData.numFrames
        energy = np.asarray(self.experimentalData.energyAtPos)
        if self.params.saveMemory:
            # getRMSD stores one sum per position into errorAtPos (BaseEngine.py:857-866)
            eap = np.array(rec.errorAtPos, copy=True)
            eap[...] = err.reshape((nf,) + (1,) * (eap.ndim - 1)).astype(eap.dtype)
            rec.errorAtPos = eap / (energy + 1e-20)
        else:
            rec.errorAtPos = err / (energy + 1e-20)
        rec.error = np.append(rec.error, np.sum(rec.errorAtPos))

    def applyConstraints(self, loop):
        """In-scope subset of BaseEngine.applyConstraints (BaseEngine.py:1440-1500), in place on the device."""
        p, rec = self.params, self.reconstruction
        if p.orthogonalizationSwitch and np.mod(loop, p.orthogonalizationFrequency) == 0:
            self.orthogonalization()
        if p.probePowerCorrectionSwitch:
            torch = _torch()
            norm = torch.sqrt(torch.sum(rec.probe * rec.probe.conj()))
            rec.probe.mul_(float(self.experimentalData.maxProbePower) / norm)
        if p.probeBoundary or p.absorbingProbeBoundary:
            torch = _torch()
            lib = self._dev["lib"]
            stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
            w = self._window_device()
            if p.probeBoundary:
                _native.check(
                    lib.ptyg_mul_window(rec.probe.data_ptr(), w.data_ptr(), rec.probe.numel(), w.numel(), stream),
                    "ptyg_mul_window",
                )
            if p.absorbingProbeBoundary:
                a = float(p.absorbingProbeBoundaryAleph)
                rec.probe.mul_((1 - a) + a * w.to(torch.complex64))

    def _window_device(self):
        torch = _torch()
        if "window" not in self._dev:
            w = np.asarray(self.probeWindow, dtype=np.float32)
            self._dev["window"] = torch.from_numpy(np.ascontiguousarray(w)).to(self._dev["device"])
        return self._dev["window"]

    def _orthogonalize(self, stack, companions=()):
        """Gram-matrix orthogonalisation of (modes, N, N) in place (utils.py:130-175):
        G on the device in FP64, eigh on the host, modes <- V^T stack."""
        torch = _torch()
        lib = self._dev["lib"]
        dev = self._dev["device"]
        stream = torch.cuda.current_stream(dev).cuda_stream
        m = int(stack.shape[0])
        n = int(stack[0].numel())
        G = torch.empty((m, m), dtype=torch.complex128, device=dev)
        src = stack.contiguous()
        _native.check(lib.ptyg_gram(src.data_ptr(), m, n, G.data_ptr(), stream), "ptyg_gram")
        w, V = np.linalg.eigh(G.cpu().numpy())
        order = np.argsort(w)[::-1]
        s = np.sqrt(np.clip(w[order].real, 0.0, None))
        evals = s**2 / np.sum(s**2)
        Vt = np.ascontiguousarray(V[:, order].T).astype(np.complex64)
        Vd = torch.from_numpy(Vt).to(dev)
        for arr in (stack,) + tuple(companions):
            a = arr.contiguous()
            out = torch.empty_like(a)
            _native.check(lib.ptyg_mix_modes(Vd.data_ptr(), a.data_ptr(), out.data_ptr(), m, n, stream), "ptyg_mix_modes")
            arr.copy_(out)
        return evals, Vt

    def orthogonalization(self):
        """BaseEngine.py:1614-1722 (probe modes first, else object modes)."""
        rec = self.reconstruction
        mom = bool(getattr(self.params, "momentumAcceleration", False))
        if rec.npsm > 1:
            for s in range(rec.nslice):
                comp = (rec.probeBuffer[0, 0, :, s], rec.probeMomentum[0, 0, :, s]) if mom else ()
                evals, V = self._orthogonalize(rec.probe[0, 0, :, s], comp)
                self.normalizedEigenvaluesProbe, self.MSPVprobe = evals, V
                rec.purityProbe = float(np.sqrt(np.sum(evals**2)))
                if hasattr(rec, "purityProbeHist"):
                    rec.purityProbeHist.append(rec.purityProbe)
        elif rec.nosm > 1:
            for s in range(rec.nslice):
                comp = (rec.objectBuffer[0, :, 0, s], rec.objectMomentum[0, :, 0, s]) if mom else ()
                evals, V = self._orthogonalize(rec.object[0, :, 0, s], comp)
                self.normalizedEigenvaluesObject, self.MSPVobject = evals, V
                rec.purityObject = float(np.sqrt(np.sum(evals**2)))

    def _detector_error_host(self):
        torch = _torch()
        d = self.experimentalData
        Np = int(self.reconstruction.Np)
        out = torch.empty((int(d.numFrames), Np, Np), dtype=torch.float32, device=self._dev["device"])
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        _native.check(
            self._dev["lib"].ptyg_plan_detector_error(self._plan, self._scan, out.data_ptr(), stream), "ptyg_plan_detector_error"
        )
        # PtyLab stores detectorError as float64: widen on the GPU, where it
        # costs nothing, rather than on one host core after the copy
        return out.to(torch.float64).cpu().numpy()

    def _check_status(self):
        st = C.c_int(0)
        torch = _torch()
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        _native.check(self._dev["lib"].ptyg_plan_status(self._plan, self._scan, C.byref(st), stream), "ptyg_plan_status")
        if st.value == 3:
            raise RuntimeError("device status 3: the ASP transfer function's copy into shared memory did not "
                               "complete within its bounded wait; this launch's results are not valid")
        if st.value != 0:
            raise RuntimeError(f"device status {st.value}: a scan position fell outside the object")

    def _move_data_to_cpu(self, detector_error=True):
        """Write the device state back as NumPy arrays (BaseEngine.py:543-611)."""
        torch = _torch()
        rec = self.reconstruction
        torch.cuda.current_stream(self._dev["device"]).synchronize()
        self._check_status()
        if detector_error and not self.params.saveMemory:
            rec.detectorError = self._detector_error_host()
        if self._projection_switches_on():
            self._projection_state_to_host()
        for name in self._state_fields():
            v = getattr(rec, name)
            if isinstance(v, torch.Tensor):
                setattr(rec, name, v.cpu().numpy())
        self._release_plan()
        self.params.gpuFlag = 0

    def _projection_state_to_host(self):
        """reconstruction.background (float64, as the reference keeps it) and
        params.intensityScaling, written in place like the reference does."""
        torch = _torch()
        p, rec = self.params, self.reconstruction
        lib = self._dev["lib"]
        stream = torch.cuda.current_stream(self._dev["device"]).cuda_stream
        if p.backgroundModeSwitch:
            bg = self._dev["background"]
            _native.check(lib.ptyg_plan_get_background(self._plan, self._scan, bg.data_ptr(), stream), "ptyg_plan_get_background")
            rec.background = bg.cpu().numpy().astype(np.float64)
        if p.intensityConstraint == "interferometric":
            # reconstruction.reference takes the exit wave's shape after the
            # first position (BaseEngine.py:975-982)
            shape = (int(getattr(rec, "nlambda", 1)), int(rec.nosm), int(rec.npsm), 1, int(rec.Np), int(rec.Np))
            ref = torch.empty(shape, dtype=torch.complex64, device=self._dev["device"])
            _native.check(lib.ptyg_plan_get_reference(self._plan, self._scan, ref.data_ptr(), stream),
                          "ptyg_plan_get_reference")
            rec.reference = ref.cpu().numpy()
        if p.intensityConstraint == "fluctuation":
            nf = self.experimentalData.numFrames
            out = np.empty(nf, dtype=np.float64)
            _native.check(lib.ptyg_plan_intensity_scaling(self._plan, self._scan, out.ctypes.data, stream),
                          "ptyg_plan_intensity_scaling")
            p.intensityScaling[...] = out

    def update_data(self, experimentalData, reconstruction=None):
        """BaseEngine.py:172-176."""
        self.experimentalData = experimentalData
        if reconstruction is not None:
            self.reconstruction = reconstruction

    def getBeamWidth(self):
        """FWHM widths (y, x) of the probe's last-slice intensity, summed over
        wavelengths and modes, from its second moments (BaseEngine.py:744-768);
        also stored as reconstruction.beamWidthY / beamWidthX."""
        rec = self.reconstruction
        P = np.sum(np.abs(_host(rec.probe)[..., -1, :, :]) ** 2, axis=(0, 1, 2))
        P = P / np.sum(P, axis=(-1, -2))
        Xp, Yp = rec.Xp, rec.Yp
        xm = np.sum(Xp * P, axis=(-1, -2))
        ym = np.sum(Yp * P, axis=(-1, -2))
        xv = np.sum((Xp - xm) ** 2 * P, axis=(-1, -2))
        yv = np.sum((Yp - ym) ** 2 * P, axis=(-1, -2))
        c = 2 * np.sqrt(2 * np.log(2))  # standard deviation -> FWHM of a Gaussian
        rec.beamWidthX = c * np.sqrt(xv)
        rec.beamWidthY = c * np.sqrt(yv)
        return rec.beamWidthY, rec.beamWidthX

    def getOverlap(self, ind1, ind2):
        """Linear and area overlap of scan positions ind1 and ind2
        (BaseEngine.py:770-818), stored as reconstruction.linearOverlap and
        reconstruction.areaOverlap.  A host-side analysis of the probe for
        monitors and scripts, off the reconstruction path: its one transform
        is NumPy's."""
        rec = self.reconstruction
        pos = np.asarray(rec.positions)
        sy = abs(pos[ind2, 0] - pos[ind1, 0]) * rec.dxp
        sx = abs(pos[ind2, 1] - pos[ind1, 1]) * rec.dxp
        self.getBeamWidth()
        rec.linearOverlap = np.maximum(1 - np.sqrt(sx**2 + sy**2) / np.minimum(rec.beamWidthX, rec.beamWidthY), 0)
        Np = int(rec.Np)
        fx = np.arange(-Np // 2, Np // 2) * (1 / (Np * rec.dxp))
        Fx, Fy = np.meshgrid(fx, fx)
        ax = (-2, -1)  # centred unitary transform (utils.py:12-28)
        A = np.abs(_host(rec.probe)[:, 0, 0, -1, ...])
        Q = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(A, axes=ax), norm="ortho"), axes=ax)
        rec.areaOverlap = np.mean(
            np.abs(np.sum(Q**2 * np.exp(-1.0j * 2 * np.pi * (Fx * sx + Fy * sy)), axis=(-1, -2)))
            / np.sum(np.abs(Q) ** 2, axis=(-1, -2)),
            axis=0,
        )
        return rec.linearOverlap, rec.areaOverlap

    def convert2single(self):
        """BaseEngine.py:683-697: the reference leaves the dtype matching
        unimplemented; the GB300 engines are single precision throughout."""
        raise NotImplementedError()

    def changeExperimentalData(self, experimentalData):
        if experimentalData is not None:
            self.experimentalData = experimentalData

    def changeOptimizable(self, optimizable):
        if optimizable is not None:
            self.reconstruction = optimizable

    def showReconstruction(self, loop):
        """GUI monitors are outside this package; the DummyMonitor hooks are no-ops."""
        return None
