"""ptyg_propagate (the Operators drop-in) against the reference fixtures and the oracle.

Tolerance: relative Frobenius error 1e-5 (FP32 transforms in a different
summation order than pocketfft; the reference's own GPU-vs-CPU bound for the
propagators is 1e-3, tests/regression/test_propagator_regression.py:108-113).
"""

from types import SimpleNamespace

import numpy as np
import pytest

from conftest import fixture_names, load_fixture, rel_err
from oracle import ptyoracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _rec(Np, dxp, wavelength, zo, dxd=None, spectralDensity=None, nlambda=1, nosm=1, npsm=1):
    sd = np.atleast_1d(wavelength if spectralDensity is None else spectralDensity)
    return SimpleNamespace(Np=Np, dxp=dxp, wavelength=wavelength, zo=zo, nlambda=nlambda, nosm=nosm, npsm=npsm,
                           dxd=dxp if dxd is None else dxd, spectralDensity=sd, esw=None, ESW=None)


@pytest.mark.parametrize("name", fixture_names("prop_"))
def test_propagator_fixtures(torch_cuda, name):
    from ptylab_gb300 import Operators, Params

    fx = load_fixture(name)
    p = Params()
    p.propagatorType = str(fx["meta_propagator"])
    p.fftshiftSwitch = False
    rec = _rec(int(fx["in_Np"]), float(fx["in_dxp"]), float(fx["in_wavelength"]), float(fx["in_zo"]),
               dxd=float(fx["in_dxd"]), spectralDensity=fx["in_spectralDensity"], nlambda=int(fx["in_nlambda"]))
    _, fwd = Operators.object2detector(fx["in_field"], p, rec)
    assert isinstance(fwd, np.ndarray) and fwd.shape == fx["out_forward"].shape
    assert rel_err(fwd, fx["out_forward"]) < TOL
    rec.ESW = fx["out_forward"]  # twoStepPolychrome's inverse also propagates reconstruction.ESW
    _, back = Operators.detector2object(fx["out_forward"], p, rec)
    assert rel_err(back, fx["out_back"]) < TOL
    # device follows the data: a CUDA tensor comes back as a CUDA tensor
    t = torch_cuda.from_numpy(fx["in_field"].astype(np.complex64)).cuda()
    _, fwd_t = Operators.object2detector(t, p, rec)
    assert fwd_t.is_cuda
    assert rel_err(fwd_t.cpu().numpy(), fx["out_forward"]) < TOL


@pytest.mark.parametrize("Np", [32, 64, 128, 256])
@pytest.mark.parametrize("prop", ["Fraunhofer", "Fresnel", "ASP"])
@pytest.mark.parametrize("fftshift", [False, True])
def test_propagators_match_oracle(torch_cuda, Np, prop, fftshift):
    from ptylab_gb300 import Operators, Params

    if prop == "ASP" and fftshift:
        pytest.skip("ASP rejects fftshiftSwitch (Operators.py:192-193)")
    rng = np.random.default_rng(Np)
    x = (rng.standard_normal((2, 3, Np, Np)) + 1j * rng.standard_normal((2, 3, Np, Np))).astype(np.complex64)
    dxp, lam, zo = 2e-6, 632.8e-9, 1e-3 if prop == "ASP" else 0.05
    p = Params()
    p.propagatorType = prop
    p.fftshiftSwitch = fftshift
    rec = _rec(Np, dxp, lam, zo)
    g = O.Geometry(Np=Np, No=Np, dxp=dxp, wavelength=lam, zo=zo)
    _, fwd = Operators.object2detector(x, p, rec)
    assert rel_err(fwd, O.object2detector(x.astype(np.complex128), prop, fftshift, g)) < TOL
    _, back = Operators.detector2object(x, p, rec)
    assert rel_err(back, O.detector2object(x.astype(np.complex128), prop, fftshift, g)) < TOL


@pytest.mark.parametrize("Np", [32, 64, 128, 256])
@pytest.mark.parametrize("prop", ["polychromeASP", "scaledASP", "scaledPolychromeASP", "twoStepPolychrome", "identity"])
def test_wavelength_set_propagators_match_oracle(torch_cuda, Np, prop):
    """Three wavelengths (one for scaledASP), two object modes, three probe
    modes: the (nlambda, 1, npsm, 1, Np, Np) probe-shaped input is broadcast
    against the (nlambda, nosm, npsm, 1, Np, Np) tables as PtyLab broadcasts
    it, and each wavelength block reads its own tables."""
    from ptylab_gb300 import Operators, Params

    nl = 1 if prop == "scaledASP" else 3
    rng = np.random.default_rng(Np + nl)
    shape = (nl, 1, 3, 1, Np, Np)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    dxp, dxd, lam, zo = 4e-6, 6e-6, 632.8e-9, 2e-3
    sd = lam * np.linspace(0.98, 1.02, nl)
    p = Params()
    p.propagatorType = prop
    rec = _rec(Np, dxp, lam, zo, dxd=dxd, spectralDensity=sd, nlambda=nl, nosm=2, npsm=3)
    g = O.Geometry(Np=Np, No=Np, dxp=dxp, wavelength=lam, zo=zo, dxd=dxd, nlambda=nl, nosm=2, npsm=3,
                   spectralDensity=tuple(sd))
    want_shape = shape if prop == "identity" else (nl, 2, 3, 1, Np, Np)
    xb = np.broadcast_to(x, want_shape).astype(np.complex128)
    _, fwd = Operators.object2detector(x, p, rec)
    assert fwd.shape == want_shape
    assert rel_err(fwd, O.object2detector(xb, prop, False, g)) < TOL
    rec.ESW = fwd
    _, back = Operators.detector2object(fwd, p, rec)
    assert rel_err(back, O.detector2object(fwd.astype(np.complex128), prop, False, g)) < TOL
    if prop != "identity":
        p.fftshiftSwitch = True
        with pytest.raises(ValueError):
            Operators.object2detector(x, p, rec)


def test_fraunhofer_round_trip_is_identity(torch_cuda):
    """tests/Operators/test_operators_integration.py:76-99 (unitary round trip)."""
    from ptylab_gb300 import Operators, Params

    rng = np.random.default_rng(1)
    x = (rng.standard_normal((4, 128, 128)) + 1j * rng.standard_normal((4, 128, 128))).astype(np.complex64)
    p = Params()
    rec = _rec(128, 1e-5, 632.8e-9, 0.05)
    for prop in ("Fraunhofer", "Fresnel"):
        p.propagatorType = prop
        _, f = Operators.object2detector(x, p, rec)
        _, b = Operators.detector2object(f, p, rec)
        assert rel_err(b, x) < 1e-6
        assert abs(np.linalg.norm(f) / np.linalg.norm(x) - 1) < 1e-6
