"""Time one layer of the warm-start network on the GPU: its 3x3 convolution
(forward) and its weight gradient, with random bf16 operands.

    python -m ptylab_gb300.warmstart.layer_bench [--layer d3a] [--batch 16] [--size 128] [--reps 20]
    python -m ptylab_gb300.warmstart.layer_bench --network [--batch 16] [--size 128] [--reps 20]

Prints the CUDA-event time and TFLOP/s of each; the layer names are those of
``layer_specs()``.  ``--network`` times the whole network's forward pass and
its backward pass (data and weight gradients of every layer) instead; the
FLOP counts are 2 M N K per GEMM (M pixels, N output channels, K = 9 x input
channels), the backward pass counting a weight gradient for every layer and
a data gradient for every layer but the first.
"""

from __future__ import annotations

import argparse


def main():
    import torch

    from .. import _native
    from .network import LEVELS, layer_specs

    ap = argparse.ArgumentParser()
    ap.add_argument("--layer", default="d3a")
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--size", type=int, default=128, help="pattern side (the network's input)")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--network", action="store_true", help="time the whole forward and backward passes")
    args = ap.parse_args()
    if args.network:
        return network_bench(args)
    lib = _native.require(0)
    spec = {name: (cins, co) for name, cins, co, _ in layer_specs(LEVELS)}
    if args.layer not in spec or args.layer in ("e1a", "head"):
        raise SystemExit(f"--layer: one of {[n for n in spec if n not in ('e1a', 'head')]}")
    level = {"e1": 1, "e2": 2, "e3": 3, "ba": 4, "bb": 4, "d3": 3, "d2": 2, "d1": 1}[args.layer[:2]]
    cins, co = spec[args.layer]
    c0, c1 = cins[0], (cins[1] if len(cins) > 1 else 0)
    B, H = args.batch, args.size >> (level - 1)
    W = H
    dev = "cuda"
    bf = torch.bfloat16
    x0 = torch.randn(B * H * W, c0, device=dev).to(bf)
    x1 = torch.randn(B * H * W, max(c1, 8), device=dev).to(bf)
    w = torch.randn(co, 9 * (c0 + c1), device=dev).to(bf)
    out = torch.empty(B * H * W, co, device=dev, dtype=bf)
    bias = torch.zeros(co, device=dev)
    dy = torch.randn(B * H * W, co, device=dev).to(bf)
    splits = 8
    part = torch.empty(splits, co, 9 * (c0 + c1), device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)

    def conv():
        _native.check(lib.ptyg_nn_conv3(x0.data_ptr(), x1.data_ptr() if c1 else None, c0, c1, B, H, W, w.data_ptr(), co,
                                        None, out.data_ptr(), bias.data_ptr(), 1, status.data_ptr(), None))

    def wgrad():
        _native.check(lib.ptyg_nn_conv3_wgrad(dy.data_ptr(), co, x0.data_ptr(), x1.data_ptr() if c1 else None, c0, c1,
                                              B, H, W, splits, part.data_ptr(), status.data_ptr(), None))

    flop = 2.0 * B * H * W * co * 9 * (c0 + c1)
    for name, f in (("conv3 forward", conv), ("weight gradient", wgrad)):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.reps):
            f()
        b.record()
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / args.reps / 1e3
        print(f"{args.layer} {name}: M={B * H * W} N={co} K={9 * (c0 + c1)}: {t * 1e6:.1f} us, {flop / t / 1e12:.1f} TFLOP/s")
    if int(status.item()) != 0:
        raise SystemExit("a tensor-core wait gave up")


def network_bench(args):
    import numpy as np
    import torch

    from .network import LEVELS, WarmStartNet, layer_specs

    level = {"e1": 1, "e2": 2, "e3": 3, "ba": 4, "bb": 4, "d3": 3, "d2": 2, "d1": 1, "he": 1}
    fwd = bwd = 0.0
    for name, cins, co, _ in layer_specs(LEVELS):
        side = args.size >> (level[name[:2]] - 1)
        k = (1 if name == "head" else 9) * sum(cins)
        f = 2.0 * args.batch * side * side * co * k
        fwd += f
        bwd += f if name == "e1a" else 2 * f
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.standard_normal((args.batch, args.size, args.size)).astype(np.float32)).cuda()
    dy = torch.as_tensor(rng.standard_normal((args.batch, args.size, args.size, 2)).astype(np.float32)).cuda()
    for mode in ("eager", "CUDA graphs"):
        net = WarmStartNet(seed=0)
        if mode != "eager":
            net.enable_graphs()
        _time_passes(net, x, dy, fwd, bwd, args, mode)


def _time_passes(net, x, dy, fwd, bwd, args, mode):
    import torch

    for name, f, flop in (("forward", lambda: net.forward(x), fwd), ("backward", lambda: net.backward(dy), bwd)):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.reps):
            f()
        b.record()
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / args.reps / 1e3
        print(f"network {name} ({mode}, batch {args.batch}, {args.size}x{args.size}): {t * 1e3:.3f} ms, "
              f"{flop / 1e9:.1f} GFLOP, {flop / t / 1e12:.1f} TFLOP/s")
    net.check_status()


if __name__ == "__main__":
    main()
