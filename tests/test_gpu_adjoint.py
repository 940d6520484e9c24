"""The differentiable multislice forward model and its hand-written adjoint.

* forward intensities against the complex128 oracle model;
* the adjoint against central finite differences (h = 1e-3) of the
  complex128 oracle model along 64 random directions, at a small size and at
  the config-2 field size (Np = 256, four slices, 13.5 nm, 20 nm pixels, 10 um);
* the gradient of the amplitude loss against the reference's own update
  direction: e3PIE moves the last object slice along conj(P_{S-1}) * DELTA
  (e3PIE.py:192-208), which is -1/2 of that gradient;
* chunking of positions does not change the result.
"""

import numpy as np
import pytest

from conftest import rel_err
from oracle import ptyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def problem(Np=64, No=128, S=3, npsm=1, n=6, seed=0, dz=10e-6, lam=13.5e-9, dxp=20e-9):
    rng = np.random.default_rng(seed)
    obj = ((0.85 + 0.15 * rng.random((S, No, No))) * np.exp(0.3j * rng.random((S, No, No)))).astype(np.complex64)
    yy, xx = np.mgrid[:Np, :Np] - Np / 2
    disc = (np.hypot(yy, xx) < Np / 4).astype(np.float64)
    probe = np.stack([disc * np.exp(2j * np.pi * rng.random((Np, Np)) * 0.1) * 0.5**m for m in range(npsm)])
    probe = probe.astype(np.complex64)
    pos = rng.integers(0, No - Np + 1, size=(n, 2)).astype(np.int32)
    H = np.fft.ifftshift(O.aspw_transfer_function(dz, lam, Np, Np * dxp))
    return obj, probe, pos, H


def to_dev(torch, obj, probe, pos, H):
    return (torch.from_numpy(obj).cuda(), torch.from_numpy(probe).cuda(), torch.from_numpy(pos).cuda(),
            torch.from_numpy(H.astype(np.complex64)).cuda())


def test_forward_matches_oracle(torch_cuda):
    from ptylab_gb300.autograd import multislice_intensity

    obj, probe, pos, H = problem(npsm=2)
    I = multislice_intensity(*to_dev(torch_cuda, obj, probe, pos, H), chunk=4).cpu().numpy()
    ref = O.multislice_forward(obj.astype(np.complex128), probe.astype(np.complex128), pos, H)
    assert rel_err(I, ref) < 1e-5


@pytest.mark.parametrize("shape", [dict(Np=64, No=128, S=3, npsm=2, n=6), dict(Np=256, No=384, S=4, npsm=1, n=3)])
def test_adjoint_matches_central_differences(torch_cuda, shape):
    torch = torch_cuda
    from ptylab_gb300.autograd import multislice_intensity

    obj, probe, pos, H = problem(**shape)
    rng = np.random.default_rng(1)
    w = rng.standard_normal((len(pos), shape["Np"], shape["Np"]))
    o_t, p_t, pos_t, H_t = to_dev(torch, obj, probe, pos, H)
    o_t.requires_grad_(True)
    p_t.requires_grad_(True)
    I = multislice_intensity(o_t, p_t, pos_t, H_t, chunk=2)
    (torch.from_numpy(w).cuda().float() * I).sum().backward()
    gO, gP = o_t.grad.cpu().numpy().astype(np.complex128), p_t.grad.cpu().numpy().astype(np.complex128)
    o64, p64 = obj.astype(np.complex128), probe.astype(np.complex128)

    def loss(o, p):
        return float(np.sum(w * O.multislice_forward(o, p, pos, H)))

    h = 1e-3
    worst = 0.0
    for _ in range(64):
        dO = rng.standard_normal(obj.shape) + 1j * rng.standard_normal(obj.shape)
        dP = rng.standard_normal(probe.shape) + 1j * rng.standard_normal(probe.shape)
        dO /= np.linalg.norm(dO)
        dP /= np.linalg.norm(dP)
        fd = (loss(o64 + h * dO, p64 + h * dP) - loss(o64 - h * dO, p64 - h * dP)) / (2 * h)
        an = float(np.sum(gO.real * dO.real + gO.imag * dO.imag) + np.sum(gP.real * dP.real + gP.imag * dP.imag))
        scale = np.linalg.norm(gO) + np.linalg.norm(gP)
        worst = max(worst, abs(fd - an) / scale)
    assert worst < 1e-4, f"worst directional-derivative mismatch {worst:.2e} (relative to |grad|)"


def test_amplitude_gradient_is_the_e3pie_update_direction(torch_cuda):
    torch = torch_cuda
    from ptylab_gb300.autograd import multislice_intensity

    obj, probe, pos, H = problem(Np=64, No=128, S=3, npsm=1, n=1)
    rng = np.random.default_rng(2)
    Imeas = (rng.random((64, 64)) * 50).astype(np.float32)
    o_t, p_t, pos_t, H_t = to_dev(torch, obj, probe, pos, H)
    o_t.requires_grad_(True)
    I = multislice_intensity(o_t, p_t, pos_t, H_t)
    # L = sum (sqrt(I) - sqrt(Imeas))^2 with the reference's 1e-10 guard: dL/dI = 1 - sqrt(Imeas / (I + 1e-10))
    g = 1 - torch.sqrt(torch.from_numpy(Imeas).cuda() / (I.detach()[0] + 1e-10))
    I[0].backward(g)
    r, c = pos[0]
    grad_last = o_t.grad[-1, r : r + 64, c : c + 64].cpu().numpy()
    P, delta = O.e3pie_last_slice_delta(obj.astype(np.complex128), probe.astype(np.complex128), pos[0], H,
                                        Imeas.astype(np.float64))
    expected = -2 * np.conj(P[0]) * delta[0]
    assert rel_err(grad_last, expected) < 1e-4


def test_chunking_does_not_change_the_result(torch_cuda):
    from ptylab_gb300.autograd import multislice_intensity

    obj, probe, pos, H = problem(n=9, npsm=2)
    args = to_dev(torch_cuda, obj, probe, pos, H)
    a = multislice_intensity(*args, chunk=2).cpu().numpy()
    b = multislice_intensity(*args, chunk=64).cpu().numpy()
    np.testing.assert_array_equal(a, b)
