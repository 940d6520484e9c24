"""Training data and the training loop of the warm-start network.

The data are scans and reconstructions the plain method generates: seeded
simulated scans of the evaluation instrument (the same two-mode probe,
Gaussian-random-field objects, Fermat scans, 1e6-photon Poisson data), each
reconstructed by this package's GPU mPIE.  A training pair is a pattern and
the mPIE object patch at its position.

Loss per batch (B patterns of one scan):
  supervised: ||pred - c target||^2 / ||target||^2 over the probe footprint,
              c the unit phase that aligns them (a pattern fixes its patch only
              up to a global phase);
  physics:    ||sqrt(I_model(pred)) - sqrt(I_meas)||^2 / ||sqrt(I_meas)||^2 with
              I_model = sum_modes |fft2c(pred P_m)|^2, the scan's reconstructed
              probe P, evaluated by the differentiable forward model
              ``ptylab_gb300.autograd.multislice_intensity`` (one slice) whose
              backward is the hand-written adjoint.
The network's own backward pass and the Adam step are the package's kernels.
"""

from __future__ import annotations

import time
from dataclasses import replace

import numpy as np

from ..simulate import cpm_problem
from .evaluate import C4
from .stitch import blend_window, network_input

TRAIN_SPEC = replace(C4, No=320, num_positions=100, seed=0)


def _torch():
    import torch

    return torch


def make_training_set(n_scans, seed0=1000, spec=TRAIN_SPEC, mpie_iters=150, log=print, batch_scans=15):
    """Simulate n_scans scans and reconstruct them with the GPU mPIE,
    `batch_scans` at a time in one launch per iteration
    (Engines.reconstruct_batch): a list of {x: float32 [n, Np, Np] network
    inputs, target: complex64 [n, Np, Np] mPIE patches, truth: complex64
    [n, Np, Np] true patches, probe: complex64 (npsm, Np, Np) reconstructed,
    I: float32 [n, Np, Np] measured}."""
    from ..Engines import mPIE, reconstruct_batch
    from ..Monitor import DummyMonitor

    out = []
    t0 = time.perf_counter()
    Np = spec.Np
    for k0 in range(0, n_scans, max(1, batch_scans)):
        group = []
        for k in range(k0, min(n_scans, k0 + max(1, batch_scans))):
            d, p, rec, obj, _ = cpm_problem(replace(spec, seed=seed0 + k), engine_seed=seed0 + k)
            p.positionOrder = "random"
            p.probePowerCorrectionSwitch = True
            eng = mPIE(rec, d, p, DummyMonitor())
            eng.alphaObject = eng.alphaProbe = 0.25
            eng.betaObject = eng.betaProbe = 0.25
            eng.numIterations = mpie_iters
            group.append((eng, d, rec, obj))
        np.random.seed(seed0 + k0)
        if len(group) == 1:
            group[0][0].reconstruct()
        else:
            reconstruct_batch([g[0] for g in group])
        for _, d, rec, obj in group:
            o = np.asarray(rec.object)[0, 0, 0, 0]
            pos = np.asarray(rec.positions)
            tgt = np.stack([o[r : r + Np, c : c + Np] for r, c in pos]).astype(np.complex64)
            tru = np.stack([obj[r : r + Np, c : c + Np] for r, c in pos]).astype(np.complex64)
            out.append(dict(x=network_input(d.ptychogram), target=tgt, truth=tru,
                            I=np.asarray(d.ptychogram, np.float32),
                            probe=np.asarray(rec.probe)[0, 0, :, 0].astype(np.complex64)))
        if log:
            log(f"training scans: {len(out)}/{n_scans} ({time.perf_counter() - t0:.1f} s)")
    return out


def _phase_aligned_loss(pred, target, w):
    """sum_batch ||pred - c target||_w^2 / ||target||_w^2 / B with c = unit phase."""
    torch = _torch()
    ov = torch.sum(torch.conj(target) * pred * w, dim=(-2, -1), keepdim=True)
    c = (ov / (ov.abs() + 1e-12)).detach()
    num = torch.sum(torch.abs(pred - c * target) ** 2 * w, dim=(-2, -1))
    den = torch.sum(torch.abs(target) ** 2 * w, dim=(-2, -1))
    return torch.mean(num / den)


def _physics_loss(pred, probe, I_meas):
    """Amplitude misfit of the forward model through the hand-written adjoint:
    the B patches are tiled into a square mosaic object with one scan
    position per tile."""
    torch = _torch()
    from ..autograd import multislice_intensity

    B, Np, _ = pred.shape
    side = int(np.ceil(np.sqrt(B)))
    pad = side * side - B
    tiles = torch.cat([pred, torch.ones(pad, Np, Np, dtype=pred.dtype, device=pred.device)]) if pad else pred
    mosaic = tiles.reshape(side, side, Np, Np).permute(0, 2, 1, 3).reshape(1, side * Np, side * Np)
    pos = torch.tensor([[(j // side) * Np, (j % side) * Np] for j in range(B)], dtype=torch.int32, device=pred.device)
    I = multislice_intensity(mosaic.contiguous(), probe, pos)
    a_model = torch.sqrt(I + 1e-6)
    a_meas = torch.sqrt(I_meas)
    return torch.sum((a_model - a_meas) ** 2) / torch.sum(a_meas**2)


def train(net, data, steps, batch=16, lr=1e-3, lam_phys=0.5, seed=0, log=print, log_every=50, reducer=None):
    """Adam steps on batches of one scan each; returns the loss history.  The
    network's forward and backward passes run as CUDA graphs (bit-identical
    to the eager passes; ``net.enable_graphs(False)`` turns them off).
    ``reducer`` (dataparallel.network_reducer(net)) averages the gradients
    over the ranks between the backward pass and the Adam step, for
    data-parallel training where each rank passes its own shard of `data`."""
    torch = _torch()
    if net._graphs is None:
        net.enable_graphs()
    rng = np.random.default_rng(seed)
    dev = net.device
    Np = data[0]["x"].shape[-1]
    w = torch.as_tensor(blend_window(Np), device=dev)
    dev_data = [dict(x=torch.as_tensor(s["x"], device=dev), target=torch.as_tensor(s["target"], device=dev),
                     I=torch.as_tensor(s["I"], device=dev), probe=torch.as_tensor(s["probe"], device=dev))
                for s in data]
    hist = []
    t0 = time.perf_counter()
    for step in range(steps):
        s = dev_data[int(rng.integers(len(dev_data)))]
        idx = torch.as_tensor(rng.choice(s["x"].shape[0], size=batch, replace=False), device=dev)
        y = net.forward(s["x"][idx])
        out = y.detach().clone().requires_grad_(True)
        pred = torch.complex(out[..., 0], out[..., 1])
        l_sup = _phase_aligned_loss(pred, s["target"][idx], w)
        loss = l_sup
        l_phys = torch.zeros(())
        if lam_phys > 0:
            l_phys = _physics_loss(pred, s["probe"], s["I"][idx])
            loss = loss + lam_phys * l_phys
        loss.backward()
        net.backward(out.grad)
        if reducer is not None:
            reducer()
        net.adam_step(lr=lr)
        hist.append((float(l_sup.detach()), float(l_phys.detach())))
        if log and (step + 1) % log_every == 0:
            ls = np.mean([h[0] for h in hist[-log_every:]])
            lp = np.mean([h[1] for h in hist[-log_every:]])
            log(f"step {step + 1}/{steps}: supervised {ls:.4f} physics {lp:.4f} ({time.perf_counter() - t0:.1f} s)")
    net.check_status()
    return hist


def save_weights(net, path):
    """The FP32 master weights in the oracle's layout, as a compressed .npz."""
    p = net.export()
    np.savez_compressed(path, **{f"{k}_W": v[0].astype(np.float32) for k, v in p.items()},
                        **{f"{k}_b": v[1].astype(np.float32) for k, v in p.items()})


def load_weights(path, device=None):
    from .network import WarmStartNet, layer_specs

    z = np.load(path)
    params = {name: (z[f"{name}_W"].astype(np.float64), z[f"{name}_b"].astype(np.float64))
              for name, _, _, _ in layer_specs()}
    return WarmStartNet(params=params, device=device)
