"""ptyg_propagate_noalloc, the propagator entry point that allocates no GPU memory.

It serves callers that cannot call cudaMalloc: code inside a host framework
that owns every device allocation, a real-time acquisition callback where
cudaMalloc's implicit synchronisation would stall the detector pipeline, or a
process that reserved all of HBM for its own buffers.  They pass only their
input and output; the scratch between the row and column passes is an 8 MiB
array built into libptyg.so.

Checked through the C ABI: two calls in a row per propagator and direction
give the same fields as ptyg_propagate (which uses allocated scratch), to the
1e-5 relative tolerance of the propagator tests (they share kernels, so the
result is in fact bitwise equal), and a batch above the built-in limit is
refused with PTYG_ERR_INVALID.  This file is collected last so a failure here
leaves every other test already run.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-5
MAX_POINTS = 1 << 20


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ptylab_gb300 import _native

    return torch, _native, _native.require(0)


def _tables(torch, Np):
    from ptylab_gb300 import _tables

    q = _tables.fresnel_chirp(0.05, 632.8e-9, Np, 1e-5).astype(np.complex64)
    h = np.fft.ifftshift(_tables.asp_detector_tf(1e-3, 632.8e-9, Np, Np * 2e-6))
    return {
        0: None,
        1: torch.from_numpy(np.ascontiguousarray(q)).cuda(),
        2: torch.from_numpy(np.ascontiguousarray(h)).cuda(),
    }


@pytest.mark.parametrize("propagator", [0, 1, 2])
@pytest.mark.parametrize("direction", [0, 1])
def test_noalloc_matches_allocating_entry_point_on_two_calls(env, propagator, direction):
    torch, _native, lib = env
    Np, batch = 128, 8
    tab = _tables(torch, Np)[propagator]
    tptr = tab.data_ptr() if tab is not None else None
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda").manual_seed(propagator * 2 + direction)
    for _ in range(2):  # the second call reuses the built-in scratch the first one left behind
        x = torch.randn((batch, Np, Np), dtype=torch.complex64, device="cuda", generator=g)
        ref = torch.empty_like(x)
        out = torch.empty_like(x)
        _native.check(lib.ptyg_propagate(propagator, direction, 0, Np, batch, x.data_ptr(), ref.data_ptr(),
                                         tptr, None, stream), "ptyg_propagate")
        _native.check(lib.ptyg_propagate_noalloc(propagator, direction, 0, Np, batch, x.data_ptr(),
                                                 out.data_ptr(), tptr, stream), "ptyg_propagate_noalloc")
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert rel_err(a, b) < TOL
        np.testing.assert_array_equal(a, b)


def test_noalloc_refuses_batches_above_its_scratch(env):
    torch, _native, lib = env
    Np = 128
    batch = MAX_POINTS // (Np * Np) + 1
    x = torch.zeros((1, Np, Np), dtype=torch.complex64, device="cuda")
    st = lib.ptyg_propagate_noalloc(0, 0, 0, Np, batch, x.data_ptr(), x.data_ptr(), None, None)
    assert st == _native.PTYG_ERR_INVALID
    assert b"exceeds" in lib.ptyg_last_error()
    # the largest batch that fits is accepted
    n = MAX_POINTS // (Np * Np)
    y = torch.randn((n, Np, Np), dtype=torch.complex64, device="cuda")
    z = torch.empty_like(y)
    _native.check(lib.ptyg_propagate_noalloc(0, 0, 0, Np, n, y.data_ptr(), z.data_ptr(), None, None))
    ref = torch.empty_like(y)
    _native.check(lib.ptyg_propagate(0, 0, 0, Np, n, y.data_ptr(), ref.data_ptr(), None, None, None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(z.cpu().numpy(), ref.cpu().numpy())
