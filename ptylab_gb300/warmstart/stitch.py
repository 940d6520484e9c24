"""Network inference over a scan and stitching of the predicted patches.

A diffraction pattern fixes its object patch only up to a global phase, so
each predicted patch is rotated onto the object stitched so far (the phase of
its overlap product) before it is added, in scan order (a Fermat spiral runs
from the centre outwards).  Patches are blended with a window matched to the
probe footprint; pixels no patch reaches keep PtyLab's 'ones' guess.
"""

from __future__ import annotations

import numpy as np

def _torch():
    import torch

    return torch


def network_input(ptychogram):
    """log(1 + I), standardised per pattern (zero mean, unit variance), float32."""
    x = np.log1p(np.maximum(np.asarray(ptychogram, dtype=np.float32), 0))
    mu = x.mean(axis=(-2, -1), keepdims=True)
    sd = x.std(axis=(-2, -1), keepdims=True) + 1e-6
    return ((x - mu) / sd).astype(np.float32)


def blend_window(Np, radius_fraction=0.25):
    yy, xx = np.mgrid[:Np, :Np] - Np / 2
    r = np.hypot(yy, xx) / (radius_fraction * Np)
    return np.exp(-0.5 * (r / 0.8) ** 2).astype(np.float32)


def predict_patches(net, ptychogram, batch=64):
    """Complex patches [n, Np, Np] (device tensor) for every pattern."""
    torch = _torch()
    x = torch.as_tensor(network_input(ptychogram), device=net.device)
    out = []
    for i in range(0, x.shape[0], batch):
        y = net.forward(x[i : i + batch])
        out.append(torch.complex(y[..., 0].clone(), y[..., 1].clone()))
    return torch.cat(out)


def stitch(patches, positions, No, window=None):
    """Phase-aligned, windowed average of patches [n, Np, Np] at (row, col) corners."""
    torch = _torch()
    n, Np, _ = patches.shape
    dev = patches.device
    w = torch.as_tensor(blend_window(Np) if window is None else window, device=dev)
    acc = torch.zeros(No, No, dtype=torch.complex64, device=dev)
    wsum = torch.zeros(No, No, dtype=torch.float32, device=dev)
    for j, (r, c) in enumerate(np.asarray(positions)):
        p = patches[j]
        a, ws = acc[r : r + Np, c : c + Np], wsum[r : r + Np, c : c + Np]
        ov = torch.sum(torch.conj(p) * a * w)  # overlap with what is there (zero for the first patch)
        mag = ov.abs()
        rot = torch.where(mag > 0, ov / torch.clamp(mag, min=1e-30), torch.ones_like(ov))
        acc[r : r + Np, c : c + Np] = a + rot * p * w
        ws += w
    out = torch.ones(No, No, dtype=torch.complex64, device=dev)
    m = wsum > 1e-3 * float(wsum.max())
    out[m] = acc[m] / wsum[m]
    return out


def predict_object(net, ptychogram, positions, No, Np, batch=64):
    """(initial object complex128 [No, No] on the host, GPU seconds of inference and stitching)."""
    torch = _torch()
    stream = torch.cuda.current_stream(net.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    obj = stitch(predict_patches(net, ptychogram, batch), positions, No)
    e1.record(stream)
    torch.cuda.synchronize(net.device)
    net.check_status()
    return obj.cpu().numpy().astype(np.complex128), e0.elapsed_time(e1) / 1e3
