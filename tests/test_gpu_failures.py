"""Failure detection without a GPU fault.

* A bounded device wait that runs out: the network kernels' mbarrier waits
  poll a limited number of times (ptyg_nn_set_wait_policy).  The test injects
  a wait on a barrier that nothing arrives at, before the launch issues any
  copy or MMA; the wait runs out, the launch sets its status word, frees its
  tensor memory and returns, and the host raises TimeoutError.  The next
  launch on the same context then computes correctly.
* An allocation that cannot be satisfied (a plan whose intensities would need
  petabytes) comes back from the C ABI as PTYG_ERR_OOM -> MemoryError, and
  the library keeps working.
* A NaN in the measured intensities: no fault; NaN spreads exactly as it
  does in the reference's NumPy path (from the poisoned position on, through
  the shared probe, to every later patch), and the error curve is NaN.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ptylab_gb300 import _native

    return torch, _native, _native.require(0)


def _status_error(st):
    """The host side of a status word: TimeoutError when a bounded wait gave up."""
    if int(st.item()) != 0:
        st.zero_()
        raise TimeoutError("a bounded tensor-core wait gave up")


@pytest.mark.parametrize("kernel", ["gemm", "conv3", "dense_wgrad"])
def test_wait_that_runs_out_reports_timeout_and_context_survives(env, kernel):
    torch, _native, lib = env
    from oracle import nn_oracle as N

    rng = np.random.default_rng(3)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    bf = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).cuda().to(torch.bfloat16)  # noqa: E731
    if kernel == "gemm":
        M, Nn, K = 256, 128, 256
        A, B = rng.standard_normal((M, K)), rng.standard_normal((Nn, K))
        dA, dB = bf(A), bf(B)
        out = torch.empty(M, Nn, dtype=torch.float32, device="cuda")
        ref = N.bf16(A) @ N.bf16(B).T

        def launch():
            return lib.ptyg_nn_gemm(dA.data_ptr(), dB.data_ptr(), M, Nn, K, 1, out.data_ptr(), None, None, 0,
                                    st.data_ptr(), None)
    elif kernel == "conv3":
        Bn, H, W, Ci, Co = 1, 32, 32, 32, 32
        x = rng.standard_normal((Bn, H, W, Ci))
        w = rng.standard_normal((Co, 9, Ci)) / 17.0
        dx, dw = bf(x), bf(w.reshape(Co, -1))
        out = torch.empty(Bn * H * W, Co, dtype=torch.float32, device="cuda")
        ref = N.conv3(N.bf16(x), N.bf16(w), np.zeros(Co)).reshape(-1, Co)

        def launch():
            return lib.ptyg_nn_conv3(dx.data_ptr(), None, Ci, 0, Bn, H, W, dw.data_ptr(), Co, out.data_ptr(), None,
                                     None, 0, st.data_ptr(), None)
    else:
        Co, K, P = 64, 128, 512
        dY, X = rng.standard_normal((P, Co)), rng.standard_normal((P, K))
        ddY, dX = bf(dY), bf(X)
        out = torch.empty(1, Co, K, dtype=torch.float32, device="cuda")
        ref = (N.bf16(dY).T @ N.bf16(X))[None]

        def launch():
            return lib.ptyg_nn_dense_wgrad(ddY.data_ptr(), Co, dX.data_ptr(), K, P, 1, out.data_ptr(), st.data_ptr(),
                                           None)

    try:
        _native.check(lib.ptyg_nn_set_wait_policy(2000, 1))
        _native.check(launch())
        torch.cuda.synchronize()
        assert int(st.item()) == 1
        with pytest.raises(TimeoutError):
            _status_error(st)
    finally:
        _native.check(lib.ptyg_nn_set_wait_policy(1 << 26, 0))
    # the context is intact: the same launch now completes and is right
    _native.check(launch())
    torch.cuda.synchronize()
    _status_error(st)
    assert rel_err(out.cpu().numpy().reshape(ref.shape), ref) < 1e-5


def test_wait_policy_rejects_bad_arguments(env):
    _, _native, lib = env
    assert lib.ptyg_nn_set_wait_policy(0, 0) == _native.PTYG_ERR_INVALID
    assert lib.ptyg_nn_set_wait_policy(10, -1) == _native.PTYG_ERR_INVALID


def test_network_check_status_raises_timeout(env):
    """The warm-start network surfaces a run-out wait as TimeoutError and clears it."""
    torch, _native, lib = env
    from ptylab_gb300.warmstart.network import WarmStartNet

    net = WarmStartNet(seed=0)
    x = torch.zeros(2, 64, 64, device="cuda")
    try:
        _native.check(lib.ptyg_nn_set_wait_policy(2000, 1))
        net.forward(x)
        torch.cuda.synchronize()
        with pytest.raises(TimeoutError):
            net.check_status()
    finally:
        _native.check(lib.ptyg_nn_set_wait_policy(1 << 26, 0))
    net.forward(x)
    torch.cuda.synchronize()
    net.check_status()  # cleared, and the next pass is clean


def test_unsatisfiable_allocation_raises_memory_error(env):
    torch, _native, lib = env
    geom = _native.Geometry(Np=256, No=256, nosm=1, npsm=1, nslice=1, num_frames=1 << 27, num_scans=1, engine=0,
                            propagator=0, fftshift=0, fpm=0, cluster=0)
    plan = C.c_void_p()
    st = lib.ptyg_plan_create(C.byref(geom), C.byref(plan))
    assert st == _native.PTYG_ERR_OOM, lib.ptyg_last_error()
    with pytest.raises(MemoryError):
        _native.check(st, "ptyg_plan_create")
    # nothing leaked into the context: a normal plan still works
    geom.num_frames = 4
    _native.check(lib.ptyg_plan_create(C.byref(geom), C.byref(plan)))
    lib.ptyg_plan_destroy(plan)


def test_nan_in_intensities_spreads_like_the_reference(env):
    """One NaN pixel in frame 5 of a C0-size ePIE scan, 1 iteration."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    d, p, rec, _, _ = cpm_problem(ScanSpec(num_positions=30))
    d.ptychogram = d.ptychogram.copy()
    d.ptychogram[5, 30, 31] = np.nan
    obj0, prb0 = rec.object.copy(), rec.probe.copy()
    eng = Engines.ePIE(rec, d, p, DummyMonitor())
    eng.numIterations = 1
    eng.reconstruct()
    g = O.Geometry(Np=64, No=256, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo)
    s = O.Settings(engine="ePIE", entrancePupilDiameter=d.entrancePupilDiameter)
    with np.errstate(invalid="ignore"):
        ref = O.OracleEngine(s, g, O.State(object=obj0, probe=prb0), d.ptychogram, rec.positions,
                             d.energyAtPos).reconstruct(1)
    np.testing.assert_array_equal(np.isnan(rec.object), np.isnan(ref.object))
    np.testing.assert_array_equal(np.isnan(rec.probe), np.isnan(ref.probe))
    assert np.isnan(rec.probe).all() and np.isnan(np.asarray(rec.error)[-1])
    ok = ~np.isnan(ref.object)
    assert ok.any() and rel_err(rec.object[ok], ref.object[ok]) < 1e-4
