"""Differentiable multislice forward model on the GB300 kernels.

``multislice_intensity(object, probe, positions, slice_h)`` returns the
predicted diffraction intensities of every scan position,
I_j = sum_modes |fft2c(psi_{S-1,j})|^2 with psi_0 = O_0[patch_j] P and
psi_s = ifft2(fft2(psi_{s-1}) H) O_s[patch_j] -- the model e3PIE inverts
(PtyLab/Engines/e3PIE.py:99-118, Fraunhofer detector).  It is a
``torch.autograd.Function`` whose backward is the hand-written adjoint
(``ptyg_multislice_adjoint``): gradients of any real loss of I flow to the
object slices and the probe in PyTorch's complex convention
(dL/dRe + i dL/dIm).  The slice fields are recomputed per chunk of positions in
the backward pass instead of being stored for the whole scan.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native, _tables


def _torch():
    import torch

    return torch


def slice_transfer_function(dz, wavelength, Np, dxp, refr_index=1.0, device="cuda"):
    """ifftshifted slice-to-slice transfer function (e3PIE.py:62-69) as a device tensor."""
    torch = _torch()
    H = np.fft.ifftshift(_tables.multislice_tf(dz, wavelength, refr_index, Np, Np * dxp)).astype(np.complex64)
    return torch.from_numpy(np.ascontiguousarray(H)).to(device)


def _geometry(obj, probe, positions, chunk):
    S, No, _ = obj.shape
    npsm, Np, _ = probe.shape
    return _native.Multislice(Np=Np, No=No, npsm=npsm, nslice=S, num_frames=positions.shape[0], chunk=chunk)


def _check(obj, probe, positions):
    torch = _torch()
    if obj.dtype != torch.complex64 or probe.dtype != torch.complex64:
        raise ValueError("object and probe must be complex64")
    if not (obj.is_cuda and probe.is_cuda and positions.is_cuda):
        raise ValueError("object, probe and positions must be CUDA tensors")
    if obj.dim() != 3 or probe.dim() != 3 or positions.dim() != 2 or positions.shape[1] != 2:
        raise ValueError("shapes: object (nslice, No, No), probe (npsm, Np, Np), positions (n, 2)")
    Np, No = probe.shape[-1], obj.shape[-1]
    p = positions.cpu()
    if len(p) and (int(p.min()) < 0 or int(p.max()) > No - Np):
        raise ValueError("positions fall outside the object")


def _make_function():
    torch = _torch()

    class _MultisliceIntensity(torch.autograd.Function):
        @staticmethod
        def forward(ctx, obj, probe, positions, slice_h, chunk):
            lib = _native.require(obj.device.index or 0)
            obj, probe = obj.contiguous(), probe.contiguous()
            positions = positions.to(torch.int32).contiguous()
            g = _geometry(obj, probe, positions, chunk)
            ws_bytes = lib.ptyg_multislice_workspace_bytes(C.byref(g))
            ws = torch.empty(ws_bytes, dtype=torch.uint8, device=obj.device)
            out = torch.empty((positions.shape[0], probe.shape[-1], probe.shape[-1]), dtype=torch.float32,
                              device=obj.device)
            h = slice_h.contiguous() if slice_h is not None else None
            stream = torch.cuda.current_stream(obj.device).cuda_stream
            _native.check(
                lib.ptyg_multislice_forward(C.byref(g), obj.data_ptr(), probe.data_ptr(), positions.data_ptr(),
                                            h.data_ptr() if h is not None else None, out.data_ptr(), ws.data_ptr(),
                                            ws_bytes, stream),
                "ptyg_multislice_forward",
            )
            ctx.save_for_backward(obj, probe, positions, h if h is not None else torch.empty(0, device=obj.device))
            ctx.chunk = chunk
            ctx.has_h = h is not None
            return out

        @staticmethod
        def backward(ctx, grad_out):
            obj, probe, positions, h = ctx.saved_tensors
            lib = _native.require(obj.device.index or 0)
            g = _geometry(obj, probe, positions, ctx.chunk)
            ws_bytes = lib.ptyg_multislice_workspace_bytes(C.byref(g))
            ws = torch.empty(ws_bytes, dtype=torch.uint8, device=obj.device)
            gO = torch.zeros_like(obj)
            gP = torch.zeros_like(probe)
            gI = grad_out.to(torch.float32).contiguous()
            stream = torch.cuda.current_stream(obj.device).cuda_stream
            _native.check(
                lib.ptyg_multislice_adjoint(C.byref(g), obj.data_ptr(), probe.data_ptr(), positions.data_ptr(),
                                            h.data_ptr() if ctx.has_h else None, gI.data_ptr(), gO.data_ptr(),
                                            gP.data_ptr(), ws.data_ptr(), ws_bytes, stream),
                "ptyg_multislice_adjoint",
            )
            return gO, gP, None, None, None

    return _MultisliceIntensity


_FN = None


def multislice_intensity(obj, probe, positions, slice_h=None, chunk=64):
    """Predicted intensities (n, Np, Np) float32 of object slices (nslice, No, No)
    and probe modes (npsm, Np, Np), differentiable in both."""
    global _FN
    _check(obj, probe, positions)
    if obj.shape[0] > 1 and slice_h is None:
        raise ValueError("slice_h (slice_transfer_function) is required for more than one slice")
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(obj, probe, positions, slice_h, int(chunk))
