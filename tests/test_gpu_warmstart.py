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

pytestmark = pytest.mark.gpu


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
