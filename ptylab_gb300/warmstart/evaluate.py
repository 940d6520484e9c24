"""Time to a normalised object error, plain mPIE against the learned warm start.

The evaluation scan: 1024 Fermat-spiral positions, Np = 128, No = 640, two
probe modes, Gaussian-random-field object (phase in [0, 2 pi], amplitude in
[0.5, 1]), 1e6-photon Poisson data.  The error of a reconstruction O against
the true object T
is e = min_{c,k} ||c exp(i k.r) O - T||_R / ||T||_R over complex c (global
phase and scale) and linear phase ramps k (an exact invariance of the data),
R the illuminated region (summed true-probe intensity above half its
maximum).
PtyLab defines no such metric: this is the package's own definition.

Both runs start from the same seeded initial guesses (PtyLab's 'ones' object
and 'circ' probe); the warm start replaces only the object guess by the
stitched network prediction.  Wall time counts the GPU work of every
iteration (and, for the warm start, the network inference and stitching),
measured with CUDA events; the error check after each iteration is not timed.
"""

from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from ..simulate import ScanSpec, cpm_problem

C4 = ScanSpec(Np=128, No=640, num_positions=1024, npsm=2, step_fraction=0.3, probe_radius_fraction=0.25,
              photons=1e6, phase_max=2 * np.pi, amp_min=0.5, sigma_px=4.0, seed=20241024)


def _torch():
    import torch

    return torch


def scanned_mask(positions, No, probe, level=0.5):
    """The illuminated region: pixels where the summed probe intensity of all
    positions exceeds `level` of its maximum."""
    Np = probe.shape[-1]
    ill = np.sum(np.abs(np.asarray(probe).reshape(-1, Np, Np)) ** 2, axis=0)
    acc = np.zeros((No, No))
    for r, c in np.asarray(positions):
        acc[r : r + Np, c : c + Np] += ill
    return acc > level * acc.max()


def normalized_error(obj, truth, mask):
    """min over a complex factor c and a linear phase ramp of
    ||c exp(i k.r) obj - truth|| / ||truth|| on the masked pixels.  Both are
    exact invariances of ptychographic data (a ramp in the object compensated
    by the opposite ramp in the probe leaves every intensity unchanged), so a
    reconstruction is judged modulo them.  The ramp: the peak of the 2x
    zero-padded Fourier transform of obj conj(truth), then a weighted
    least-squares plane through the remaining phase."""
    torch = _torch()
    o = torch.as_tensor(obj)
    o = o.reshape(o.shape[-2:]).to(torch.complex128)
    t = torch.as_tensor(truth, device=o.device).to(torch.complex128)
    m = torch.as_tensor(mask, device=o.device)
    n0, n1 = o.shape
    D = torch.where(m, torch.conj(o) * t, torch.zeros((), dtype=o.dtype, device=o.device))
    F = torch.fft.fft2(D, s=(2 * n0, 2 * n1))
    k = int(torch.argmax(F.abs()))
    ky, kx = k // (2 * n1), k % (2 * n1)
    ky = ky - 2 * n0 if ky >= n0 else ky
    kx = kx - 2 * n1 if kx >= n1 else kx
    yy = torch.arange(n0, device=o.device, dtype=torch.float64)[:, None]
    xx = torch.arange(n1, device=o.device, dtype=torch.float64)[None, :]
    ramp = 2 * np.pi * (ky * yy / (2 * n0) + kx * xx / (2 * n1))
    D1 = D * torch.exp(-1j * ramp)
    # plane through the residual phase (weights |D|), after removing its mean
    Dm = D1[m]
    ph0 = torch.angle(torch.sum(Dm))
    ph = torch.angle(Dm * torch.exp(-1j * ph0))
    w = Dm.abs()
    A = torch.stack([torch.ones_like(ph), yy.expand(n0, n1)[m], xx.expand(n0, n1)[m]], 1) * w[:, None]
    sol = torch.linalg.lstsq(A, ph * w).solution
    ramp = ramp + sol[1] * yy + sol[2] * xx
    o = o * torch.exp(1j * ramp)
    om, tm = o[m], t[m]
    c = torch.sum(torch.conj(om) * tm) / torch.sum(om.abs() ** 2)
    return float(torch.linalg.vector_norm(c * om - tm) / torch.linalg.vector_norm(tm))


@dataclass
class Run:
    label: str
    seconds: list  # cumulative GPU seconds after each iteration
    errors: list   # error after each iteration
    setup_seconds: float = 0.0

    def time_to(self, threshold):
        for s, e in zip(self.seconds, self.errors):
            if e <= threshold:
                return s
        return None


def mpie_iterations(eng, max_iters, truth, mask, threshold, label, setup_seconds=0.0, probe_first=0):
    """Run eng (an Engines.mPIE) one iteration at a time, as mPIE.reconstruct
    does, recording cumulative GPU time and the object error; stops at the
    threshold or after max_iters.  probe_first: the first iterations update
    the probe only (betaObject 0), so a probe guess can settle on an object
    that is already close (the hand-over from a warm start)."""
    torch = _torch()
    rec = eng.reconstruction
    eng._prepareReconstruction()
    if hasattr(rec, "objectBuffer"):  # mPIE.reconstruct: buffers follow the prepared state
        rec.objectBuffer.copy_(rec.object)
        rec.probeBuffer.copy_(rec.probe)
    nf = eng.experimentalData.numFrames
    dev = eng._dev["device"]
    t_dev = torch.as_tensor(truth, device=dev)
    m_dev = torch.as_tensor(mask, device=dev)
    stream = torch.cuda.current_stream(dev)
    run = Run(label, [], [], setup_seconds)
    total = setup_seconds
    beta_o = eng.betaObject
    for loop in range(max_iters):
        eng.betaObject = 0.0 if loop < probe_first else beta_o
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        eng.setPositionOrder()
        draws = np.random.rand(nf) if hasattr(rec, "objectBuffer") else None
        e0.record(stream)
        eng._upload_order(momentum=None if draws is None else draws > 0.95)
        eng._run_positions(0, nf, record_detector_error=False)
        eng.getErrorMetrics()
        eng.applyConstraints(loop)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        total += e0.elapsed_time(e1) / 1e3
        err = normalized_error(rec.object[0, 0, 0, 0], t_dev, m_dev)
        run.seconds.append(total)
        run.errors.append(err)
        if err <= threshold:
            break
    eng._move_data_to_cpu(detector_error=False)
    return run


def c4_problem(spec=C4, engine_seed=20240607):
    """(experimentalData, params, reconstruction, true object, true probe) of the evaluation scan."""
    d, p, rec, obj, probe = cpm_problem(spec, engine_seed=engine_seed)
    p.positionOrder = "random"
    return d, p, rec, obj, probe


def _mpie(d, p, rec):
    from ..Engines import mPIE
    from ..Monitor import DummyMonitor

    p.probePowerCorrectionSwitch = True
    eng = mPIE(rec, d, p, DummyMonitor())
    eng.alphaObject = eng.alphaProbe = 0.25
    eng.betaObject = eng.betaProbe = 0.25
    return eng


def compare(net, spec=C4, threshold=1e-2, max_iters=200, seed=5, batch=64, probe_first=(0,)):
    """Plain mPIE and warm-started mPIE on the evaluation scan: (plain Run,
    warm Run, warm-start error), with one warm Run per probe_first entry
    (a list of Runs when probe_first has several)."""
    torch = _torch()
    from .stitch import predict_object

    d, p, rec, obj, probe = c4_problem(spec)
    mask = scanned_mask(rec.positions, spec.No, probe)
    truth = obj.astype(np.complex64)
    obj0, prb0 = rec.object.copy(), rec.probe.copy()

    # warm-up (clocks, first launches), not timed
    np.random.seed(seed)
    mpie_iterations(_mpie(d, p, rec), 30, truth, mask, 0.0, "warm-up")
    d, p, rec, _, _ = c4_problem(spec)
    rec.object, rec.probe = obj0.copy(), prb0.copy()
    np.random.seed(seed)
    plain = mpie_iterations(_mpie(d, p, rec), max_iters, truth, mask, threshold, "plain mPIE")

    warms = []
    for pf in probe_first:
        d, p, rec, _, _ = c4_problem(spec)
        rec.object, rec.probe = obj0.copy(), prb0.copy()
        # warm-up of the inference (graph capture for this batch shape, first
        # launches), not timed, like the plain run's warm-up above
        predict_object(net, d.ptychogram, rec.positions, spec.No, spec.Np, batch=batch)
        torch.cuda.synchronize()
        warm_obj, setup = predict_object(net, d.ptychogram, rec.positions, spec.No, spec.Np, batch=batch)
        rec.object = warm_obj.reshape(rec.object.shape).astype(np.complex64)
        warm_err0 = normalized_error(warm_obj, truth, mask)
        np.random.seed(seed)
        label = "warm start + mPIE" + (f" (probe only for {pf} iterations)" if pf else "")
        warms.append(mpie_iterations(_mpie(d, p, rec), max_iters, truth, mask, threshold, label,
                                     setup_seconds=setup, probe_first=pf))
    return plain, (warms[0] if len(warms) == 1 else warms), warm_err0
