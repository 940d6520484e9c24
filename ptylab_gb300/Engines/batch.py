"""Many independent scans reconstructed side by side in one launch per iteration.

PtyLab reconstructs one scan per engine; a GB300 runs the position loop of
one scan on one thread-block cluster, so a single scan leaves most of the
GPU idle.  ``reconstruct_batch(engines)`` takes engines built the usual way
(``Engines.mPIE(reconstruction, experimentalData, params, monitor)`` ...),
one per scan, and runs them together: one launch plan with a cluster per
scan, one kernel launch per iteration for all of them.  Each engine keeps its
own state, position order, momentum draws, error curve and constraints, and
ends with its reconstruction back in NumPy exactly as ``reconstruct()``
leaves it.

The engines must be of one class and share the launch geometry (Np, No, mode
counts, slices, frames, propagator, fftshift, operation mode), the update
scalars, the propagator tables and the projection switches.  The global
NumPy RNG is consumed engine by engine within each iteration (order shuffle,
then mPIE's momentum draws), so a batched scan sees different draws than the
same engine run alone unless its order is deterministic.
"""

from __future__ import annotations

import numpy as np


def _same(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return np.array_equal(np.asarray(a), np.asarray(b))
    return a == b


def _check_compatible(engines):
    e0 = engines[0]
    if any(type(e) is not type(e0) for e in engines):
        raise ValueError("reconstruct_batch: all engines must be of one class")
    if len({id(e.reconstruction) for e in engines}) != len(engines):
        raise ValueError("reconstruct_batch: every engine needs its own reconstruction")
    geo = [f for f, _ in e0._geometry()._fields_ if f not in ("num_scans", "throughput")]
    g0 = e0._geometry()
    upd = [f for f, _ in e0._update_params()._fields_]
    u0 = e0._update_params()
    r0, p0 = e0.reconstruction, e0.params
    for e in engines[1:]:
        g = e._geometry()
        bad = [f for f in geo if getattr(g, f) != getattr(g0, f)]
        if bad:
            raise ValueError(f"reconstruct_batch: launch geometry differs ({', '.join(bad)})")
        u = e._update_params()
        bad = [f for f in upd if getattr(u, f) != getattr(u0, f)]
        if bad:
            raise ValueError(f"reconstruct_batch: update parameters differ ({', '.join(bad)})")
        if p0.propagatorType.lower() == "polychromeasp" and not _same(
            np.atleast_1d(e.reconstruction.spectralDensity), np.atleast_1d(r0.spectralDensity)
        ):
            raise ValueError("reconstruct_batch: reconstruction.spectralDensity differs (propagator tables)")
        for name in ("zo", "wavelength", "dxp"):
            if p0.propagatorType.lower() != "fraunhofer" and not _same(getattr(e.reconstruction, name),
                                                                       getattr(r0, name)):
                raise ValueError(f"reconstruct_batch: reconstruction.{name} differs (propagator tables)")
        for name in ("intensityConstraint", "adaptiveDenoisingSwitch", "backgroundModeSwitch", "FourierMaskSwitch"):
            if getattr(e.params, name) != getattr(p0, name):
                raise ValueError(f"reconstruct_batch: params.{name} differs")
        if e.numIterations != e0.numIterations:
            raise ValueError("reconstruct_batch: numIterations differs")


class _BatchState:
    """What the scans of a batch share per iteration: one device buffer of all
    scans' position orders and momentum flags (each scan's bound order is a
    row), filled from a ring of pinned host rows by one copy each, and one
    device row per iteration of all scans' per-frame error sums (each
    engine's error rows are a view of it).  With many scans, per-scan copies
    and launches would cost more host time than the iteration's kernel."""

    SLOTS = 3

    def __init__(self, engines):
        import torch

        e0 = engines[0]
        dev = e0._dev["device"]
        G, nf = len(engines), int(e0.experimentalData.numFrames)
        self.device, self.G, self.nf = dev, G, nf
        self.orders = torch.zeros((G, nf), dtype=torch.int32, device=dev)
        self.flags = torch.zeros((G, nf), dtype=torch.uint8, device=dev)
        self.ring = [(torch.zeros((G, nf), dtype=torch.int32).pin_memory(),
                      torch.zeros((G, nf), dtype=torch.uint8).pin_memory()) for _ in range(self.SLOTS)]
        # NumPy views of the pinned rows: a scan's order is staged by one
        # NumPy assignment (a torch row copy costs ~20x more host time, which
        # with 150 scans is the iteration's own kernel time)
        self.ring_np = [(o.numpy(), f.numpy()) for o, f in self.ring]
        self.events = [None] * self.SLOTS
        self.uploads = 0
        self.errs = torch.zeros((max(int(e0.numIterations), 1), G, nf), dtype=torch.float64, device=dev)
        self.n_err = 0
        self.staging = None
        self.any_flags = False

    def begin_upload(self):
        slot = self.uploads % self.SLOTS
        if self.events[slot] is not None:
            self.events[slot].synchronize()
        self.staging = self.ring[slot]
        self.staging_np = self.ring_np[slot]
        self.any_flags = False

    def stage(self, g, order, momentum):
        self.staging_np[0][g] = order
        if momentum is not None:
            self.staging_np[1][g] = momentum
            self.any_flags = True

    def end_upload(self):
        import torch

        self.orders.copy_(self.staging[0], non_blocking=True)
        if self.any_flags:
            self.flags.copy_(self.staging[1], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self.events[self.uploads % self.SLOTS] = ev
        self.uploads += 1

    def record_errors(self, engines):
        import torch

        from .. import _native

        e0 = engines[0]
        if self.n_err == self.errs.shape[0]:
            grown = torch.zeros((2 * self.errs.shape[0], self.G, self.nf), dtype=torch.float64, device=self.device)
            grown[: self.n_err].copy_(self.errs)
            # each engine's view moves to the grown buffer at the rows it has not read yet
            for g, e in enumerate(engines):
                e._err_dev = grown[self.n_err - e._err_n :, g, :]
            self.errs = grown
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _native.check(e0._dev["lib"].ptyg_plan_frame_errors_all_device(e0._plan, self.errs[self.n_err].data_ptr(), stream),
                      "ptyg_plan_frame_errors_all_device")
        self.n_err += 1
        for e in engines:
            e._err_n += 1


def begin_batch(engines, throughput=1):
    """Set-up half of ``reconstruct_batch``: validation, host preparation,
    device state, one launch plan with a cluster per scan.  Returns the list
    of engines; run ``iterate_batch`` for every loop, then ``finish_batch``."""
    engines = list(engines)
    for e in engines:
        e._pre_prepare()
    _check_compatible(engines)
    for e in engines:
        e._prepare_host()
    for e in engines:
        e._device_state()
    state = _BatchState(engines)
    for g, e in enumerate(engines):
        # the scan's order and flags are rows of the shared buffers (bound below)
        e._dev["order"], e._dev["flags"] = state.orders[g], state.flags[g]
        e._batch, e._batch_row = state, g
        e._err_dev, e._err_n = state.errs[:, g, :], 0
    e0 = engines[0]
    e0._plan_and_bind(num_scans=len(engines), throughput=throughput)
    for i, e in enumerate(engines[1:], 1):
        e._plan_and_bind(plan=e0._plan, scan=i)
    for e in engines:
        e._loop_begin()
    return engines


def iterate_batch(engines, loop):
    """One iteration of every scan: the host draws each order (and mPIE's
    momentum flags) into the shared staging rows, one copy moves them, one
    kernel launch walks all scans' positions, one launch sums every scan's
    frame errors, then each engine applies its constraints."""
    e0 = engines[0]
    state = e0._batch
    nf = e0.experimentalData.numFrames
    state.begin_upload()
    for e in engines:
        e._loop_order(loop)
    state.end_upload()
    e0._run_positions(0, nf, record_detector_error=(loop == e0.numIterations - 1))  # every bound scan
    state.record_errors(engines)
    for e in engines:
        e._loop_end(loop)


def finish_batch(engines):
    """Read every scan's results back into NumPy and release the plan."""
    for e in engines[1:]:
        e._finish()
    engines[0]._finish()  # the plan's owner last: it destroys the plan
    for e in engines:
        e._batch = None


def reconstruct_batch(engines):
    """Run ``engine.reconstruct()`` for every engine, all scans in one launch per iteration."""
    engines = list(engines)
    if not engines:
        return
    engines = begin_batch(engines)
    for loop in range(engines[0].numIterations):
        iterate_batch(engines, loop)
    finish_batch(engines)
