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


def network_input_device(ptychogram, device):
    """network_input on the GPU (the same standardised log(1 + I), float32):
    the patterns go up once and are transformed where they land."""
    torch = _torch()
    x = torch.as_tensor(np.asarray(ptychogram, dtype=np.float32), device=device)
    x = torch.log1p(torch.clamp(x, min=0))
    mu = x.mean(dim=(-2, -1), keepdim=True)
    sd = x.std(dim=(-2, -1), keepdim=True, unbiased=False) + 1e-6
    return (x - mu) / sd


def predict_patches(net, ptychogram, batch=64):
    """Complex patches [n, Np, Np] (device tensor) for every pattern."""
    torch = _torch()
    x = network_input_device(ptychogram, net.device)
    out = []
    for i in range(0, x.shape[0], batch):
        y = net.forward(x[i : i + batch])
        out.append(torch.complex(y[..., 0].clone(), y[..., 1].clone()))
    return torch.cat(out)


def stitch(patches, positions, No, window=None):
    """Phase-aligned, windowed average of patches [n, Np, Np] at (row, col)
    corners: the patches are added in order by one CTA of ``ptyg_stitch``
    (each rotated onto the overlap with what is there), then divided by the
    summed window."""
    from .. import _native

    torch = _torch()
    n, Np, _ = patches.shape
    dev = patches.device
    lib = _native.require(dev.index or 0)
    w = torch.as_tensor(blend_window(Np) if window is None else window, device=dev).to(torch.float32).contiguous()
    acc = torch.zeros(No, No, dtype=torch.complex64, device=dev)
    wsum = torch.zeros(No, No, dtype=torch.float32, device=dev)
    pos = torch.as_tensor(np.ascontiguousarray(np.asarray(positions), dtype=np.int32), device=dev)
    p = patches.to(torch.complex64).contiguous()
    _native.check(lib.ptyg_stitch(p.data_ptr(), pos.data_ptr(), int(n), int(Np), int(No), w.data_ptr(),
                                  acc.data_ptr(), wsum.data_ptr(), torch.cuda.current_stream(dev).cuda_stream),
                  "ptyg_stitch")
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
