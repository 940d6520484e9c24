"""Drop-in for PtyLab's propagator dispatch (PtyLab/Operators/Operators.py:561-584, 1082-1103).

``object2detector(fields, params, reconstruction)`` and
``detector2object(fields, params, reconstruction)`` return
``(reconstruction.esw, propagated)`` like PtyLab's, for all of PtyLab's
propagators: Fraunhofer, Fresnel and ASP (``ptyg_propagate``), and
polychromeASP, scaledASP, scaledPolychromeASP, twoStepPolychrome and
identity (``ptyg_propagate_sets``), computed by libptyg's sm_103a kernels.
Results are complex64 (PtyLab's CPU path promotes the polychrome and
two-step results to complex128 through its float64 tables; the tables here
are rounded to complex64).  Device placement follows the data
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


def _stage(fields):
    """(complex64 contiguous CUDA tensor, whether the caller passed a tensor)."""
    import torch

    on_gpu = isinstance(fields, torch.Tensor)
    if on_gpu:
        if not fields.is_cuda:
            raise ValueError("torch fields must live on a CUDA device")
        return fields.to(torch.complex64).contiguous(), True
    device = torch.device("cuda", torch.cuda.current_device())
    return torch.from_numpy(np.ascontiguousarray(np.asarray(fields), dtype=np.complex64)).to(device), False


def propagate(fields, kind: str, direction: int, fftshift: bool, reconstruction, z=None):
    """Run ptyg_propagate on ``fields`` (torch CUDA tensor or NumPy array)."""
    import torch

    k = _KIND[kind.lower()]
    if k == 2 and fftshift:
        raise ValueError("ASP propagator only works with fftshiftswitch == False")
    if k == 2 and getattr(reconstruction, "nlambda", 1) > 1:
        # Operators.py:866-869
        raise ValueError("For multi-wavelength, polychromeASP needs to be used instead of ASP")
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


def _wavelengths(reconstruction):
    nl = int(getattr(reconstruction, "nlambda", 1))
    sd = np.atleast_1d(np.asarray(getattr(reconstruction, "spectralDensity", reconstruction.wavelength), dtype=np.float64))
    if sd.size < nl:
        raise ValueError(f"spectralDensity has {sd.size} wavelengths for nlambda = {nl}")
    return tuple(float(w) for w in sd[:nl])


def _set_tables(kind, reconstruction, Np, device, z):
    """(table A, table B, number of sets, shape the tables broadcast to) on `device`."""
    import torch

    zo = float(reconstruction.zo if z is None else z)
    nl = int(getattr(reconstruction, "nlambda", 1))
    nosm, npsm = int(getattr(reconstruction, "nosm", 1)), int(getattr(reconstruction, "npsm", 1))
    Lp = Np * float(reconstruction.dxp)
    tab_shape = (nl, nosm, npsm, 1, Np, Np)
    if kind == "identity":
        return None, None, 1, (Np, Np)
    if kind == "scaledasp":
        if nl > 1:  # Operators.py:970-973
            raise ValueError("For multi-wavelength, scaledPolychromeASP needs to be used instead of scaledASP")
        key = (kind, zo, float(reconstruction.wavelength), Np, float(reconstruction.dxp), float(reconstruction.dxd))
        build = lambda: _tables.scaled_asp_tables(zo, float(reconstruction.wavelength), Np,
                                                  float(reconstruction.dxp), float(reconstruction.dxd))
        tab_shape = (1, nosm, npsm, 1, Np, Np)
    elif kind == "scaledpolychromeasp":
        wl = _wavelengths(reconstruction)
        key = (kind, zo, wl, Np, float(reconstruction.dxp), float(reconstruction.dxd))

        def build():
            q = [_tables.scaled_asp_tables(zo, w, Np, float(reconstruction.dxp), float(reconstruction.dxd)) for w in wl]
            return np.stack([a for a, _ in q]), np.stack([b for _, b in q])
    elif kind == "polychromeasp":
        wl = _wavelengths(reconstruction)
        key = (kind, zo, wl, Np, Lp)
        build = lambda: (_tables.polychrome_asp_tf(zo, wl, Np, Lp), None)
    else:  # twosteppolychrome
        wl = _wavelengths(reconstruction)
        key = (kind, zo, wl, Np, Lp, float(reconstruction.dxp))
        build = lambda: _tables.two_step_polychrome_tables(zo, wl, Np, Lp, float(reconstruction.dxp))
    key = key + (str(device),)
    if key not in _table_cache:
        a, b = build()
        up = lambda t: None if t is None else torch.from_numpy(np.ascontiguousarray(t, dtype=np.complex64)).to(device)
        _table_cache[key] = (up(a), up(b))
    a, b = _table_cache[key]
    return a, b, tab_shape[0], tab_shape


def propagate_sets(fields, kind: str, direction: int, fftshift: bool, reconstruction, z=None):
    """Run ptyg_propagate_sets on ``fields``: the fields are broadcast against
    the propagator's (nlambda, nosm, npsm, 1, Np, Np) tables as PtyLab's
    products broadcast them, so field f of the result reads wavelength set
    f // (fields per wavelength)."""
    import torch

    kind = kind.lower()
    if fftshift and kind != "identity":
        raise ValueError(f"{kind} propagatorType works only with fftshiftSwitch = False!")
    x, on_gpu = _stage(fields)
    device = x.device
    lib = _native.require(device.index if device.index is not None else 0)
    Np = int(x.shape[-1])
    if x.ndim < 2 or x.shape[-2] != Np:
        raise ValueError(f"fields must be square in the last two axes, got {tuple(x.shape)}")
    a, b, nsets, tab_shape = _set_tables(kind, reconstruction, Np, device, z)
    shape = np.broadcast_shapes(tuple(x.shape), tab_shape)
    if len(shape) > 6 and nsets > 1:
        raise ValueError(f"fields of shape {tuple(x.shape)}: the wavelength axis must lead a 6-axis array")
    # the tables are 6-axis with the wavelength first, so a 6-axis result is
    # wavelength-major: nsets consecutive blocks of fields
    if tuple(x.shape) != shape:
        x = x.expand(shape).contiguous()
    batch = x.numel() // (Np * Np)
    out = torch.empty_like(x)
    stream = torch.cuda.current_stream(device).cuda_stream
    _native.check(
        lib.ptyg_propagate_sets(
            _native.SET_PROPAGATORS[kind], int(direction), Np, batch, nsets, x.data_ptr(), out.data_ptr(),
            a.data_ptr() if a is not None else None, b.data_ptr() if b is not None else None, None, stream,
        ),
        "ptyg_propagate_sets",
    )
    return out if on_gpu else out.cpu().numpy()


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


def _set_forward(kind, name):
    def fn(fields, params, reconstruction, z=None):
        return getattr(reconstruction, "esw", None), propagate_sets(
            fields, kind, 0, bool(params.fftshiftSwitch), reconstruction, z
        )

    fn.__name__ = name
    return fn


def _set_inverse(kind, name):
    def fn(fields, params, reconstruction, z=None):
        return getattr(reconstruction, "esw", None), propagate_sets(
            fields, kind, 1, bool(params.fftshiftSwitch), reconstruction, z
        )

    fn.__name__ = name
    return fn


propagate_polychromeASP = _set_forward("polychromeasp", "propagate_polychromeASP")
propagate_polychromeASP_inv = _set_inverse("polychromeasp", "propagate_polychromeASP_inv")
propagate_scaledASP = _set_forward("scaledasp", "propagate_scaledASP")
propagate_scaledASP_inv = _set_inverse("scaledasp", "propagate_scaledASP_inv")
propagate_scaledPolychromeASP = _set_forward("scaledpolychromeasp", "propagate_scaledPolychromeASP")
propagate_scaledPolychromeASP_inv = _set_inverse("scaledpolychromeasp", "propagate_scaledPolychromeASP_inv")
propagate_twoStepPolychrome = _set_forward("twosteppolychrome", "propagate_twoStepPolychrome")


def propagate_twoStepPolychrome_inv(fields, params, reconstruction, z=None):
    """Operators.py:285-310: returns (the inverse of reconstruction.ESW, the
    inverse of fields), in that order, as PtyLab's does."""
    f = propagate_sets(fields, "twosteppolychrome", 1, bool(params.fftshiftSwitch), reconstruction, z)
    g = propagate_sets(reconstruction.ESW, "twosteppolychrome", 1, bool(params.fftshiftSwitch), reconstruction, z)
    return g, f


def propagate_identity(fields, params, reconstruction, inverse=False, z=None):
    """Operators.py:508-533: a copy of the fields (forward and inverse)."""
    return getattr(reconstruction, "esw", None), propagate_sets(fields, "identity", 0, False, reconstruction, z)


forward_lookup_dictionary = {
    "fraunhofer": propagate_fraunhofer,
    "fresnel": propagate_fresnel,
    "asp": propagate_ASP,
    "polychromeasp": propagate_polychromeASP,
    "scaledasp": propagate_scaledASP,
    "scaledpolychromeasp": propagate_scaledPolychromeASP,
    "twosteppolychrome": propagate_twoStepPolychrome,
    "identity": propagate_identity,
}
reverse_lookup_dictionary = {
    "fraunhofer": propagate_fraunhofer_inv,
    "fresnel": propagate_fresnel_inv,
    "asp": propagate_ASP_inv,
    "polychromeasp": propagate_polychromeASP_inv,
    "scaledasp": propagate_scaledASP_inv,
    "scaledpolychromeasp": propagate_scaledPolychromeASP_inv,
    "twosteppolychrome": propagate_twoStepPolychrome_inv,
    "identity": propagate_identity,
}


def _lookup(table, params):
    key = params.propagatorType.lower()
    if key not in table:  # PtyLab raises KeyError from its dictionaries (Operators.py:568-570)
        raise KeyError(key)
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
