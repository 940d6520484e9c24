"""Train the warm-start network on the GPU and time mPIE to a normalised
object error, plain against warm-started, on the evaluation scan.

    python -m ptylab_gb300.warmstart.benchmark [--scans 60] [--steps 3000]
        [--max-iters 1200] [--weights out.npz] [--photons 1e6]

--photons sets the dose of the evaluation scan, --train-photons that of the
training scans (both default to the configured 1e6), e.g. 1e9 for both to
see where the two runs go without the noise that stops plain mPIE near 2e-2.

Prints one JSON line: training time, the warm start's own object error, and
for both runs the GPU seconds to errors 1e-1, 3e-2 and 1e-2 (null where the
run stopped first), the iterations run and the final error.
"""

from __future__ import annotations

import argparse
import json
import time
from dataclasses import replace


def main():
    import torch

    from . import evaluate as EV
    from . import train as TR
    from .network import WarmStartNet

    ap = argparse.ArgumentParser()
    ap.add_argument("--scans", type=int, default=60)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--lam-phys", type=float, default=0.1)
    ap.add_argument("--max-iters", type=int, default=1200)
    ap.add_argument("--weights", default=None, help="save the trained weights here (.npz)")
    ap.add_argument("--photons", type=float, default=None, help="photons per pattern of the evaluation scan")
    ap.add_argument("--train-photons", type=float, default=None, help="photons per pattern of the training scans")
    ap.add_argument("--probe-first", default="0",
                    help="comma-separated: warm runs whose first N iterations update the probe only")
    ap.add_argument("--batch-scans", type=int, default=15, help="training scans reconstructed per launch")
    args = ap.parse_args()
    t0 = time.perf_counter()
    tspec = TR.TRAIN_SPEC if args.train_photons is None else replace(TR.TRAIN_SPEC, photons=args.train_photons)
    data = TR.make_training_set(args.scans, spec=tspec, log=None, batch_scans=args.batch_scans)
    t_data = time.perf_counter() - t0
    net = WarmStartNet(seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = TR.train(net, data, args.steps, batch=args.batch, lr=args.lr, lam_phys=args.lam_phys, log=None)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    if args.weights:
        TR.save_weights(net, args.weights)
    spec = EV.C4 if args.photons is None else replace(EV.C4, photons=args.photons)
    pfs = tuple(int(v) for v in args.probe_first.split(","))
    plain, warm, e0 = EV.compare(net, spec=spec, max_iters=args.max_iters, probe_first=pfs)
    warms = warm if isinstance(warm, list) else [warm]
    out = {
        "evaluation": f"1024-position Fermat scan, Np=128, No=640, npsm=2, {spec.photons:g} photons (synthetic, seeded)",
        "training": {"scans": args.scans, "patterns": args.scans * 100, "steps": args.steps, "batch": args.batch,
                     "photons": tspec.photons,
                     "data_seconds": round(t_data, 2), "train_seconds": round(t_train, 2),
                     "final_supervised_loss": float(sum(h[0] for h in hist[-100:]) / 100)},
        "warm_start_object_error": e0,
    }
    for r in (plain, *warms):
        out[r.label] = {"setup_seconds": r.setup_seconds, "iterations": len(r.errors), "final_error": r.errors[-1],
                        **{f"seconds_to_{t:g}": r.time_to(t) for t in (1e-1, 5e-2, 3e-2, 2e-2, 1e-2)}}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
