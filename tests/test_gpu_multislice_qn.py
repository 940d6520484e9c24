"""The quasi-Newton multislice gradient engine (Engines.e3qNewton) and its two
entry points, ptyg_multislice_amplitude_gradient and ptyg_qn_step.

The reference has no gradient engine for multislice scans; it is checked
  - against PyTorch autograd of the amplitude loss through the differentiable
    model (whose adjoint is itself checked by central differences in
    test_gpu_adjoint.py), with the illuminations and per-frame errors;
  - against the reference's own qNewton step (qNewton.py:108-140) through the
    oracle: one position, one slice, the object step equal to the oracle's
    and the probe step parallel to it (the reference normalises the probe
    step by the whole object's maximum, this engine by the patch's);
  - at the C2 configuration (900 positions, 4 slices, Np 256): the error
    curve falls.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _lib():
    from ptylab_gb300 import _native

    return _native, _native.require(0)


def _gradient(torch, O, P, pos, H, meas, order=None, chunk=None):
    _native, lib = _lib()
    S, No, _ = O.shape
    npsm, Np, _ = P.shape
    n = pos.shape[0] if order is None else order.shape[0]
    g = _native.Multislice(Np=Np, No=No, npsm=npsm, nslice=S, num_frames=n, chunk=chunk or n)
    wsb = lib.ptyg_multislice_workspace_bytes(C.byref(g))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    gO, gP = torch.zeros_like(O), torch.zeros_like(P)
    wO = torch.zeros(O.shape, dtype=torch.float32, device="cuda")
    wP = torch.zeros(P.shape, dtype=torch.float32, device="cuda")
    err = torch.zeros(meas.shape[0], dtype=torch.float64, device="cuda")
    _native.check(lib.ptyg_multislice_amplitude_gradient(
        C.byref(g), O.data_ptr(), P.data_ptr(), pos.data_ptr(), H.data_ptr() if H is not None else None,
        order.data_ptr() if order is not None else None, meas.data_ptr(), gO.data_ptr(), gP.data_ptr(),
        wO.data_ptr(), wP.data_ptr(), err.data_ptr(), ws.data_ptr(), wsb, torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return gO, gP, wO, wP, err


def test_amplitude_gradient_matches_autograd(torch_cuda):
    """Gradients of L = sum (sqrt(I + 1e-10) - sqrt(I_meas))^2 against autograd
    through multislice_intensity; illuminations and |I_meas - I| per frame
    against PyTorch; a frame order that visits a subset in another order."""
    torch = torch_cuda
    from ptylab_gb300.autograd import multislice_intensity, slice_transfer_function

    rng = np.random.default_rng(3)
    Np, No, S, npsm, n = 64, 160, 3, 2, 7
    O = torch.from_numpy((np.exp(1j * 0.3 * rng.standard_normal((S, No, No))) *
                          (0.8 + 0.2 * rng.random((S, No, No)))).astype(np.complex64)).cuda()
    P = torch.from_numpy((rng.standard_normal((npsm, Np, Np)) + 1j * rng.standard_normal((npsm, Np, Np)))
                         .astype(np.complex64)).cuda()
    pos = torch.from_numpy(rng.integers(0, No - Np + 1, size=(n, 2)).astype(np.int32)).cuda()
    H = slice_transfer_function(2e-6, 13.5e-9, Np, 20e-9)
    meas = torch.from_numpy((rng.random((n, Np, Np)) * 4e3).astype(np.float32)).cuda()

    Oa, Pa = O.clone().requires_grad_(True), P.clone().requires_grad_(True)
    I = multislice_intensity(Oa, Pa, pos, H)
    L = ((I + 1e-10).sqrt() - meas.sqrt()).pow(2).sum()
    L.backward()
    gO, gP, wO, wP, err = _gradient(torch, O, P, pos, H, meas, chunk=3)
    assert rel_err(gO.cpu().numpy(), Oa.grad.cpu().numpy()) < 1e-4
    assert rel_err(gP.cpu().numpy(), Pa.grad.cpu().numpy()) < 1e-4
    Ih = I.detach()
    want_err = (meas - Ih).abs().sum(dim=(1, 2)).double()
    assert rel_err(err.cpu().numpy(), want_err.cpu().numpy()) < 1e-5
    # probe weight: sum_j |O_0[patch_j]|^2 in every mode plane
    p = pos.cpu().numpy()
    O0 = O[0].cpu().numpy()
    V = sum(np.abs(O0[y:y + Np, x:x + Np]) ** 2 for y, x in p)
    assert rel_err(wP[0].cpu().numpy(), V) < 1e-5 and rel_err(wP[1].cpu().numpy(), V) < 1e-5
    # slice 0's illumination: sum_j sum_p |P_p|^2 at the patches
    W0 = np.zeros((No, No))
    Pp = (np.abs(P.cpu().numpy()) ** 2).sum(0)
    for y, x in p:
        W0[y:y + Np, x:x + Np] += Pp
    assert rel_err(wO[0].cpu().numpy(), W0) < 1e-5

    # a subset of the frames in another order gives the gradient of that subset
    sub = [5, 0, 3]
    order = torch.tensor(sub, dtype=torch.int32, device="cuda")
    Ob, Pb = O.clone().requires_grad_(True), P.clone().requires_grad_(True)
    Is = multislice_intensity(Ob, Pb, pos[sub], H)
    ((Is + 1e-10).sqrt() - meas[sub].sqrt()).pow(2).sum().backward()
    gO2, gP2, _, _, err2 = _gradient(torch, O, P, pos, H, meas, order=order, chunk=2)
    assert rel_err(gO2.cpu().numpy(), Ob.grad.cpu().numpy()) < 1e-4
    assert rel_err(gP2.cpu().numpy(), Pb.grad.cpu().numpy()) < 1e-4
    e2 = err2.cpu().numpy()
    assert np.all(e2[[1, 2, 4, 6]] == 0) and np.all(e2[sub] > 0)


def test_one_position_step_is_qnewtons(torch_cuda):
    """One position, one slice, betas 1, regs 1: the object after the step is
    the oracle's qNewton object (qNewton.py:108-122) and the probe step is
    parallel to the oracle's (qNewton.py:124-140)."""
    torch = torch_cuda
    from oracle import ptyoracle as OR
    from ptylab_gb300 import simulate as SIM

    d, p, rec, _, _ = SIM.cpm_problem(SIM.ScanSpec(Np=64, No=160, num_positions=20, seed=4))
    obj0, prb0 = np.asarray(rec.object).copy(), np.asarray(rec.probe).copy()
    pos = np.asarray(rec.positions)[:1]
    data = np.asarray(d.ptychogram)[:1]
    g = OR.Geometry(Np=64, No=160, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo)
    s = OR.Settings(engine="qNewton", entrancePupilDiameter=d.entrancePupilDiameter)
    np.random.seed(0)
    ref = OR.OracleEngine(s, g, OR.State(object=obj0.copy(), probe=prb0.copy()), data, pos,
                          np.asarray(d.energyAtPos)[:1]).reconstruct(1)

    _native, lib = _lib()
    O = torch.from_numpy(obj0[0, 0, 0].astype(np.complex64)).cuda()      # (1, No, No)
    P = torch.from_numpy(prb0[0, 0, :, 0].astype(np.complex64)).cuda()   # (1, Np, Np)
    gpos = torch.from_numpy(pos.astype(np.int32)).cuda()
    meas = torch.from_numpy(data.astype(np.float32)).cuda()
    gO, gP, wO, wP, err = _gradient(torch, O, P, gpos, None, meas)
    scratch = torch.zeros(64, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    P_before = P.clone()
    _native.check(lib.ptyg_qn_step(O.data_ptr(), gO.data_ptr(), wO.data_ptr(), 1, 160 * 160, 1.0, 1.0,
                                   scratch.data_ptr(), st))
    _native.check(lib.ptyg_qn_step(P.data_ptr(), gP.data_ptr(), wP.data_ptr(), 1, 64 * 64, 1.0, 1.0,
                                   scratch.data_ptr(), st))
    torch.cuda.synchronize()
    got_obj = O.cpu().numpy()[0]
    want_obj = np.asarray(ref.object)[0, 0, 0, 0]
    e = rel_err(got_obj, want_obj)
    print(f"one-position qNewton object step: rel err {e:.2e}")
    assert e < 1e-5
    dp_got = (P - P_before).cpu().numpy().ravel()
    dp_want = (np.asarray(ref.probe)[0, 0, 0, 0] - prb0[0, 0, 0, 0]).ravel()
    cos = abs(np.vdot(dp_got, dp_want)) / (np.linalg.norm(dp_got) * np.linalg.norm(dp_want))
    print(f"probe step cosine {cos:.8f}")
    assert cos > 1 - 1e-5
    # the gradient pass's error is the reference's detector error of the position
    assert rel_err(err.cpu().numpy(), np.asarray(ref.errorAtPos).ravel() * np.asarray(d.energyAtPos)[:1]) < 1e-4


def test_config2_gradient_engine(torch_cuda):
    """C2 (900 positions on a jittered raster, 4 weak-phase slices 10 um apart,
    Np 256, No 768) through Engines.e3qNewton: three iterations, the error
    curve falls and the result keeps PtyLab's shapes and dtypes."""
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300 import simulate as SIM

    _, d, p, rec = SIM.config_problem("C2")
    eng = Engines.e3qNewton(rec, d, p, DummyMonitor())
    eng.numIterations = 3
    np.random.seed(2)
    eng.reconstruct()
    err = np.asarray(rec.error)
    print("e3qNewton C2 error curve", err)
    assert err.shape == (3,) and np.all(np.isfinite(err))
    assert err[1] < err[0] and err[2] < err[1]
    assert rec.object.shape == (1, 1, 1, 4, 768, 768) and rec.object.dtype == np.complex64
    assert rec.probe.shape == (1, 1, 1, 4, 256, 256) and rec.probe.dtype == np.complex64
