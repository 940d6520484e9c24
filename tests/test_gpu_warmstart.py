"""The learned warm start end to end on the GPU: training data from the plain
method (simulated scans reconstructed by the GPU mPIE), training by the
package's own network kernels (supervised plus the physics loss through the
hand-written adjoint), inference and stitching on a held-out scan.

What the trained network gains over the method without it is measured
against the initial object it replaces (PtyLab's 'ones' guess): the stitched
prediction must be closer to the true object.  The time-to-error comparison
with plain mPIE is run by ``python -m ptylab_gb300.warmstart.benchmark``."""

from dataclasses import replace

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


def test_trained_network_improves_the_initial_object():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ptylab_gb300.warmstart import WarmStartNet
    from ptylab_gb300.warmstart import evaluate as EV
    from ptylab_gb300.warmstart import train as TR
    from ptylab_gb300.warmstart.stitch import predict_object

    data = TR.make_training_set(24, log=None)
    net = WarmStartNet(seed=1)
    hist = TR.train(net, data, 1500, batch=16, lr=3e-4, lam_phys=0.1, log=None)
    first, last = np.mean([h[0] for h in hist[:200]]), np.mean([h[0] for h in hist[-200:]])
    assert last < first, (first, last)
    spec = replace(EV.C4, num_positions=256, No=384, seed=777)  # held out: seed and size differ from training
    d, p, rec, obj, probe = EV.c4_problem(spec)
    mask = EV.scanned_mask(rec.positions, spec.No, probe)
    e_guess = EV.normalized_error(torch.as_tensor(rec.object), obj, mask)
    warm, seconds = predict_object(net, d.ptychogram, rec.positions, spec.No, spec.Np)
    e_warm = EV.normalized_error(torch.as_tensor(warm), obj, mask)
    print(f"object error: initial guess {e_guess:.4f}, warm start {e_warm:.4f} ({seconds:.3f} s inference + stitching)")
    assert e_warm < e_guess - 0.02, (e_guess, e_warm)


def _stitch_reference(torch, patches, positions, No, w):
    """The stitching rule restated with torch ops, one patch at a time."""
    n, Np, _ = patches.shape
    acc = torch.zeros(No, No, dtype=torch.complex128, device=patches.device)
    wsum = torch.zeros(No, No, dtype=torch.float64, device=patches.device)
    w = w.to(torch.float64)
    for j, (r, c) in enumerate(np.asarray(positions)):
        p = patches[j].to(torch.complex128)
        a = acc[r : r + Np, c : c + Np]
        ov = torch.sum(torch.conj(p) * a * w)
        rot = ov / ov.abs() if float(ov.abs()) > 0 else torch.ones((), dtype=ov.dtype, device=ov.device)
        acc[r : r + Np, c : c + Np] = a + rot * p * w
        wsum[r : r + Np, c : c + Np] += w
    return acc, wsum


def test_stitch_kernel_matches_the_rule(torch_cuda):
    """ptyg_stitch (one CTA walking the patches in order) against the rule
    in float64 torch: overlaps, rotations, window sums; patches with no
    overlap keep their own phase."""
    torch = torch_cuda
    from ptylab_gb300 import _native
    from ptylab_gb300.warmstart.stitch import blend_window

    rng = np.random.default_rng(3)
    n, Np, No = 60, 32, 112
    patches = torch.as_tensor((rng.standard_normal((n, Np, Np)) + 1j * rng.standard_normal((n, Np, Np)))
                              .astype(np.complex64)).cuda()
    positions = rng.integers(0, No - Np + 1, size=(n, 2)).astype(np.int32)
    positions[5] = (No - Np, No - Np)
    w = torch.as_tensor(blend_window(Np)).cuda()
    acc = torch.zeros(No, No, dtype=torch.complex64, device="cuda")
    wsum = torch.zeros(No, No, dtype=torch.float32, device="cuda")
    pos = torch.as_tensor(positions).cuda()
    lib = _native.require(0)
    _native.check(lib.ptyg_stitch(patches.data_ptr(), pos.data_ptr(), n, Np, No, w.data_ptr(), acc.data_ptr(),
                                  wsum.data_ptr(), None))
    torch.cuda.synchronize()
    ref_acc, ref_w = _stitch_reference(torch, patches, positions, No, w)
    assert rel_err(acc.cpu().numpy(), ref_acc.cpu().numpy()) < 1e-5
    assert rel_err(wsum.cpu().numpy(), ref_w.cpu().numpy()) < 1e-6


def test_network_input_on_the_device_matches_the_host_version(torch_cuda):
    from ptylab_gb300.warmstart.stitch import network_input, network_input_device

    rng = np.random.default_rng(8)
    I = rng.poisson(50.0 * rng.random((6, 64, 64))).astype(np.float32)
    got = network_input_device(I, "cuda").cpu().numpy()
    assert rel_err(got, network_input(I)) < 1e-6
