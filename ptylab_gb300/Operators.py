"""Drop-in for PtyLab's propagator dispatch (PtyLab/Operators/Operators.py:561-584, 1082-1103).

``object2detector(fields, params, reconstruction)`` and
``detector2object(fields, params, reconstruction)`` return
``(reconstruction.esw, propagated)`` like PtyLab's, for the Fraunhofer,
Fresnel and ASP propagators, computed by libptyg's sm_103a kernels
(``ptyg_propagate``).  Device placement follows the data
(test_propagator_regression.py:85-113): a torch CUDA tensor comes back as a
torch CUDA tensor on the same stream; a NumPy array is staged through the GPU
and comes back as a NumPy complex64 array.  Any leading shape is accepted; the
last two axes are the Np x Np field.
"""

from __future__ import annotations

import numpy as np

from . import _native, _tables

_KIND = {"fraunhofer": 0, "fresnel": 1, "asp": 2}
_table_cache: dict = {}


def _device_table(kind: int, reconstruction, Np: int, device, z=None):
    import torch

    if kind == 0:
        return None
    zo = float(reconstruction.zo if z is None else z)
    if kind == 1:
        key = ("fresnel", zo, float(reconstruction.wavelength), Np, float(reconstruction.dxp), str(device))
        if key not in _table_cache:
            q = _tables.fresnel_chirp(zo, float(reconstruction.wavelength), Np, float(reconstruction.dxp))
            _table_cache[key] = torch.from_numpy(np.ascontiguousarray(q.astype(np.complex64))).to(device)
        return _table_cache[key]
    Lp = float(reconstruction.Np * reconstruction.dxp) if hasattr(reconstruction, "Np") else Np * float(reconstruction.dxp)
    key = ("asp", zo, float(reconstruction.wavelength), Np, Lp, str(device))
    if key not in _table_cache:
        h = np.fft.ifftshift(_tables.asp_detector_tf(zo, float(reconstruction.wavelength), Np, Lp), axes=(-2, -1))
        _table_cache[key] = torch.from_numpy(np.ascontiguousarray(h)).to(device)
    return _table_cache[key]


def propagate(fields, kind: str, direction: int, fftshift: bool, reconstruction, z=None):
    """Run ptyg_propagate on ``fields`` (torch CUDA tensor or NumPy array)."""
    import torch

    k = _KIND[kind.lower()]
    if k == 2 and fftshift:
        raise ValueError("ASP propagator only works with fftshiftswitch == False")
    if getattr(reconstruction, "nlambda", 1) > 1:
        raise NotImplementedError("multi-wavelength propagators are not on this path")
    on_gpu = isinstance(fields, torch.Tensor)
    if on_gpu:
        if not fields.is_cuda:
            raise ValueError("torch fields must live on a CUDA device")
        x = fields.to(torch.complex64).contiguous()
        device = x.device
    else:
        device = torch.device("cuda", torch.cuda.current_device())
        x = torch.from_numpy(np.ascontiguousarray(np.asarray(fields), dtype=np.complex64)).to(device)
    lib = _native.require(device.index if device.index is not None else 0)
    Np = int(x.shape[-1])
    if x.shape[-2] != Np:
        raise ValueError(f"fields must be square in the last two axes, got {tuple(x.shape)}")
    batch = x.numel() // (Np * Np)
    out = torch.empty_like(x)
    table = _device_table(k, reconstruction, Np, device, z)
    stream = torch.cuda.current_stream(device).cuda_stream
    _native.check(
        lib.ptyg_propagate(
            k, int(direction), int(bool(fftshift)), Np, batch,
            x.data_ptr(), out.data_ptr(), table.data_ptr() if table is not None else None, None, stream,
        ),
        "ptyg_propagate",
    )
    if on_gpu:
        return out
    return out.cpu().numpy()


def _forward(kind):
    def fn(fields, params, reconstruction, z=None):
        return getattr(reconstruction, "esw", None), propagate(
            fields, kind, 0, bool(params.fftshiftSwitch), reconstruction, z
        )

    fn.__name__ = f"propagate_{kind}"
    return fn


def _inverse(kind):
    def fn(fields, params, reconstruction, z=None):
        return getattr(reconstruction, "esw", None), propagate(
            fields, kind, 1, bool(params.fftshiftSwitch), reconstruction, z
        )

    fn.__name__ = f"propagate_{kind}_inv"
    return fn


propagate_fraunhofer = _forward("fraunhofer")
propagate_fraunhofer_inv = _inverse("fraunhofer")
propagate_fresnel = _forward("fresnel")
propagate_fresnel_inv = _inverse("fresnel")
propagate_ASP = _forward("asp")
propagate_ASP_inv = _inverse("asp")

forward_lookup_dictionary = {
    "fraunhofer": propagate_fraunhofer,
    "fresnel": propagate_fresnel,
    "asp": propagate_ASP,
}
reverse_lookup_dictionary = {
    "fraunhofer": propagate_fraunhofer_inv,
    "fresnel": propagate_fresnel_inv,
    "asp": propagate_ASP_inv,
}


def _lookup(table, params):
    key = params.propagatorType.lower()
    if key not in table:
        raise NotImplementedError(f"propagatorType {params.propagatorType!r} is not on this path (Fraunhofer, Fresnel, ASP)")
    return table[key]


def object2detector(fields, params, reconstruction):
    """Operators.py:576-584."""
    if fields is None:
        fields = reconstruction.esw
    return _lookup(forward_lookup_dictionary, params)(fields, params, reconstruction)


def detector2object(fields, params, reconstruction):
    """Operators.py:561-573."""
    if fields is None:
        fields = reconstruction.ESW
    return _lookup(reverse_lookup_dictionary, params)(fields, params, reconstruction)
