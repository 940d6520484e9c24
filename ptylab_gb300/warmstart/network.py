"""The warm-start network on the GB300 kernels (``csrc/ptyg_nn.cu``).

A 4-level convolutional encoder-decoder (channels 32/64/128/256, 3x3 'same'
convolutions with ReLU, 2x2 average pooling, nearest 2x upsampling, skip
connections by channel concatenation, a 1x1 output convolution) mapping
log-scaled diffraction patterns [B, H, W] to complex patches [B, H, W, 2]
(real, imaginary).  Activations are NHWC bfloat16, weights bfloat16 copies of
FP32 master weights, every convolution an implicit GEMM on the tcgen05 tensor
cores with FP32 accumulation, forward and backward.  PyTorch only provides
the buffers; every layer, its gradient and the Adam step are this package's
kernels.  The layer list and weight layout are those of ``oracle/nn_oracle.py``
(the CPU checker of these gradients).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _native

LEVELS = (32, 64, 128, 256)
HEAD_PAD = 8  # the 1x1 output convolution's 2 channels, padded for the GEMM's K multiple of 8
FIRST_K = 16  # the first layer's 9 taps of one channel, padded likewise


def layer_specs(levels=LEVELS):
    """(name, input channels of each concatenated source, output channels, relu) in forward order."""
    c1, c2, c3, c4 = levels
    return [
        ("e1a", (1,), c1, True), ("e1b", (c1,), c1, True),
        ("e2a", (c1,), c2, True), ("e2b", (c2,), c2, True),
        ("e3a", (c2,), c3, True), ("e3b", (c3,), c3, True),
        ("ba", (c3,), c4, True), ("bb", (c4,), c4, True),
        ("d3a", (c4, c3), c3, True), ("d3b", (c3,), c3, True),
        ("d2a", (c3, c2), c2, True), ("d2b", (c2,), c2, True),
        ("d1a", (c2, c1), c1, True), ("d1b", (c1,), c1, True),
        ("head", (c1,), 2, False),
    ]


def _torch():
    import torch

    return torch


class _Param:
    """FP32 master weights, BF16 copy, gradient and Adam moments of one tensor."""

    def __init__(self, value, device):
        torch = _torch()
        self.p = torch.as_tensor(np.ascontiguousarray(value, dtype=np.float32), device=device)
        self.p16 = self.p.to(torch.bfloat16)
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)


class WarmStartNet:
    """The encoder-decoder with hand-written forward and backward passes."""

    def __init__(self, params=None, seed=0, device=None, levels=LEVELS):
        """params: {name: (W, b)} in the oracle's layout (conv W [Co, 9, Ci],
        head W [2, Ci]); default He-normal from ``seed``."""
        torch = _torch()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.lib = _native.require(self.device.index or 0)
        self.levels = tuple(levels)
        self.specs = layer_specs(self.levels)
        if params is None:
            params = _he_init(seed, self.specs)
        self.W, self.b = {}, {}
        for name, cins, co, _ in self.specs:
            w, b = params[name]
            ci = sum(cins)
            if name == "head":
                wp = np.zeros((HEAD_PAD, ci))
                wp[:co] = w
                bp = np.zeros(HEAD_PAD)
                bp[:co] = b
            elif name == "e1a":
                wp = np.zeros((co, FIRST_K))
                wp[:, :9] = np.asarray(w).reshape(co, 9)
                bp = b
            else:
                wp = np.asarray(w).reshape(co, 9 * ci)
                bp = b
            self.W[name] = _Param(wp, self.device)
            self.b[name] = _Param(bp, self.device)
        self.step = 0
        self._shape = None
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._graphs = None  # enable_graphs(): {(pass, shape): (CUDAGraph, static input, output)}

    def enable_graphs(self, on=True):
        """Replay forward() and backward() as CUDA graphs, one captured per
        input shape (the ~60 forward and ~160 backward launches then cost
        one graph launch each, not one Python call each).  The passes keep
        their buffers across calls, so a captured graph stays valid until
        the shape changes."""
        self._graphs = {} if on else None

    def _replay(self, kind, fn, arg):
        """Run fn(arg) through the graph captured for (kind, arg's shape)."""
        torch = _torch()
        if self._shape is not None and tuple(arg.shape[:3]) != self._shape:
            # a new batch shape reallocates every buffer the graphs point at
            self._graphs.clear()
        key = (kind, tuple(arg.shape))
        entry = self._graphs.get(key)
        if entry is None:
            static = torch.empty_like(arg)
            static.copy_(arg)
            fn(static)  # eager run: allocates every buffer, sets kernel attributes
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                out = fn(static)
            entry = self._graphs[key] = (graph, static, out)
        graph, static, out = entry
        static.copy_(arg)
        graph.replay()
        return out

    # ---------------------------------------------------------------- plumbing
    def _stream(self):
        return _torch().cuda.current_stream(self.device).cuda_stream

    def _call(self, name, *args):
        _native.check(getattr(self.lib, name)(*args, self._stream()), name)

    def parameters(self):
        for name, _, _, _ in self.specs:
            yield self.W[name]
            yield self.b[name]

    def export(self):
        """{name: (W, b)} in the oracle's layout (float64, from the FP32 masters)."""
        out = {}
        for name, cins, co, _ in self.specs:
            w = self.W[name].p.double().cpu().numpy()
            b = self.b[name].p.double().cpu().numpy()
            ci = sum(cins)
            if name == "head":
                out[name] = (w[:co], b[:co])
            elif name == "e1a":
                out[name] = (w[:, :9].reshape(co, 9, 1), b)
            else:
                out[name] = (w.reshape(co, 9, ci), b)
        return out

    def export_grads(self):
        """The last backward()'s parameter gradients, {name: (dW, db)} in the oracle's layout."""
        out = {}
        for name, cins, co, _ in self.specs:
            w = self.W[name].g.double().cpu().numpy()
            b = self.b[name].g.double().cpu().numpy()
            ci = sum(cins)
            if name == "head":
                out[name] = (w[:co], b[:co])
            elif name == "e1a":
                out[name] = (w[:, :9].reshape(co, 9, 1), b)
            else:
                out[name] = (w.reshape(co, 9, ci), b)
        return out

    def _alloc(self, B, H, W):
        """Activation and gradient buffers for a batch of B patterns of H x W."""
        torch = _torch()
        if self._shape == (B, H, W):
            return
        dev, bf, f32 = self.device, torch.bfloat16, torch.float32
        sizes = {1: (H, W), 2: (H // 2, W // 2), 3: (H // 4, W // 4), 4: (H // 8, W // 8)}
        level = {"e1a": 1, "e1b": 1, "e2a": 2, "e2b": 2, "e3a": 3, "e3b": 3, "ba": 4, "bb": 4,
                 "d3a": 3, "d3b": 3, "d2a": 2, "d2b": 2, "d1a": 1, "d1b": 1, "head": 1}
        self.level, self.sizes = level, sizes
        a, g = {}, {}
        for name, cins, co, _ in self.specs:
            h, w = sizes[level[name]]
            M = B * h * w
            a[name] = torch.empty(M, HEAD_PAD if name == "head" else co, dtype=f32 if name == "head" else bf, device=dev)
            g[name] = torch.empty(M, HEAD_PAD if name == "head" else co, dtype=f32, device=dev)
        for k, lv, c in (("p1", 2, self.levels[0]), ("p2", 3, self.levels[1]), ("p3", 4, self.levels[2]),
                         ("u3", 3, self.levels[3]), ("u2", 2, self.levels[2]), ("u1", 1, self.levels[1])):
            h, w = sizes[lv]
            a[k] = torch.empty(B * h * w, c, dtype=bf, device=dev)
        self.a, self.gbuf = a, g
        self.x16 = torch.empty(B * H * W, dtype=bf, device=dev)
        self.col1 = torch.empty(B * H * W, FIRST_K, dtype=bf, device=dev)
        self.colsum = torch.empty(-(-(B * H * W) // 256) * 256, dtype=f32, device=dev)  # column-sum partials
        self._shape = (B, H, W)

    # ---------------------------------------------------------------- forward
    def _conv_fwd(self, name, srcs, lv):
        B = self._shape[0]
        h, w = self.sizes[lv]
        x0 = self.a[srcs[0]]
        x1 = self.a[srcs[1]] if len(srcs) > 1 else None
        c0 = x0.shape[1]
        c1 = x1.shape[1] if x1 is not None else 0
        co = self.a[name].shape[1]
        self._call("ptyg_nn_conv3", x0.data_ptr(), x1.data_ptr() if x1 is not None else None, c0, c1, B, h, w,
                   self.W[name].p16.data_ptr(), co, None, self.a[name].data_ptr(), self.b[name].p.data_ptr(), 1,
                   self.status.data_ptr())

    def forward(self, x):
        """x: float32 tensor [B, H, W] (H, W multiples of 8) -> float32 [B, H, W, 2]."""
        if self._graphs is not None:
            return self._replay("forward", self._forward, x)
        return self._forward(x)

    def _forward(self, x):
        torch = _torch()
        B, H, W = x.shape
        self._alloc(B, H, W)
        M = B * H * W
        self.x16.copy_(x.reshape(-1).to(torch.bfloat16))
        self._call("ptyg_nn_im2col1", self.x16.data_ptr(), B, H, W, FIRST_K, self.col1.data_ptr())
        self._call("ptyg_nn_gemm", self.col1.data_ptr(), self.W["e1a"].p16.data_ptr(), M, self.levels[0], FIRST_K, 1,
                   None, self.a["e1a"].data_ptr(), self.b["e1a"].p.data_ptr(), 1, self.status.data_ptr())
        self._conv_fwd("e1b", ["e1a"], 1)
        self._pool("e1b", "p1", 1)
        self._conv_fwd("e2a", ["p1"], 2)
        self._conv_fwd("e2b", ["e2a"], 2)
        self._pool("e2b", "p2", 2)
        self._conv_fwd("e3a", ["p2"], 3)
        self._conv_fwd("e3b", ["e3a"], 3)
        self._pool("e3b", "p3", 3)
        self._conv_fwd("ba", ["p3"], 4)
        self._conv_fwd("bb", ["ba"], 4)
        self._up("bb", "u3", 4)
        self._conv_fwd("d3a", ["u3", "e3b"], 3)
        self._conv_fwd("d3b", ["d3a"], 3)
        self._up("d3b", "u2", 3)
        self._conv_fwd("d2a", ["u2", "e2b"], 2)
        self._conv_fwd("d2b", ["d2a"], 2)
        self._up("d2b", "u1", 2)
        self._conv_fwd("d1a", ["u1", "e1b"], 1)
        self._conv_fwd("d1b", ["d1a"], 1)
        self._call("ptyg_nn_gemm", self.a["d1b"].data_ptr(), self.W["head"].p16.data_ptr(), M, HEAD_PAD,
                   self.levels[0], 1, self.a["head"].data_ptr(), None, self.b["head"].p.data_ptr(), 0,
                   self.status.data_ptr())
        return self.a["head"][:, :2].reshape(B, H, W, 2)

    def _pool(self, src, dst, lv):
        B = self._shape[0]
        h, w = self.sizes[lv]
        self._call("ptyg_nn_pool2", self.a[src].data_ptr(), self.a[dst].data_ptr(), B, h, w, self.a[src].shape[1])

    def _up(self, src, dst, lv):
        B = self._shape[0]
        h, w = self.sizes[lv]
        self._call("ptyg_nn_up2", self.a[src].data_ptr(), self.a[dst].data_ptr(), B, h, w, self.a[src].shape[1])

    # ---------------------------------------------------------------- backward
    def _splits(self, rows, cols, k):
        """Pixel ranges for a weight-gradient GEMM: about four CTAs per SM in all."""
        tiles = max(1, -(-rows // 128)) * max(1, -(-cols // 256))
        return int(max(1, min(-(-k // 64), 600 // tiles)))

    def _wgrad(self, name, launch, co, k, P):
        """dW [co, k] of layer `name` from the split-over-pixels GEMM `launch(splits, partials)`."""
        torch = _torch()
        s = self._splits(co, k, P)
        pb = -(-P // 64)
        s = min(s, pb)
        used = -(-P // (-(-pb // s) * 64))  # the split count the kernel uses (whole 64-pixel blocks)
        part = torch.empty(used, co, k, dtype=torch.float32, device=self.device)
        launch(s, part)
        self._call("ptyg_nn_reduce_splits", part.data_ptr(), self.W[name].g.data_ptr(), co * k, used)

    def _conv_bwd(self, name, srcs, lv, need_dx=True):
        """Upstream gradient in gbuf[name] (f32 [M, Co]); writes the parameter
        gradients and returns dX (f32 [M, sum of input channels]) or None."""
        torch = _torch()
        B = self._shape[0]
        h, w = self.sizes[lv]
        M = B * h * w
        y = self.a[name]
        co = y.shape[1]
        dpre16 = torch.empty(M, co, dtype=torch.bfloat16, device=self.device)
        dpre32 = torch.empty(M, co, dtype=torch.float32, device=self.device)
        self._call("ptyg_nn_relu_bwd", self.gbuf[name].data_ptr(), y.data_ptr(), dpre16.data_ptr(), dpre32.data_ptr(),
                   M * co)
        self._call("ptyg_nn_col_sum", dpre32.data_ptr(), self.colsum.data_ptr(), self.b[name].g.data_ptr(), M, co)
        x0 = self.a[srcs[0]]
        x1 = self.a[srcs[1]] if len(srcs) > 1 else None
        c0 = x0.shape[1]
        c1 = x1.shape[1] if x1 is not None else 0
        k = 9 * (c0 + c1)
        self._wgrad(name, lambda s, part: self._call(
            "ptyg_nn_conv3_wgrad", dpre16.data_ptr(), co, x0.data_ptr(), x1.data_ptr() if x1 is not None else None,
            c0, c1, B, h, w, s, part.data_ptr(), self.status.data_ptr()), co, k, M)
        if not need_dx:
            return None
        wf = torch.empty(c0 + c1, 9 * co, dtype=torch.bfloat16, device=self.device)
        self._call("ptyg_nn_flip_weights", self.W[name].p16.data_ptr(), wf.data_ptr(), co, c0 + c1)
        dx = torch.empty(M, c0 + c1, dtype=torch.float32, device=self.device)
        self._call("ptyg_nn_conv3", dpre16.data_ptr(), None, co, 0, B, h, w, wf.data_ptr(), c0 + c1, dx.data_ptr(),
                   None, None, 0, self.status.data_ptr())
        return dx

    def backward(self, dout):
        """dout: float32 [B, H, W, 2], the loss gradient w.r.t. forward()'s
        output; fills every parameter's .g."""
        if self._graphs is not None:
            self._replay("backward", self._backward, dout.contiguous())
            return
        self._backward(dout)

    def _backward(self, dout):
        torch = _torch()
        B, H, W = self._shape
        M = B * H * W
        c1, c2, c3, c4 = self.levels
        g = self.gbuf
        # head: 1x1 convolution, output channels padded to HEAD_PAD
        dh = torch.zeros(M, HEAD_PAD, dtype=torch.float32, device=self.device)
        dh[:, :2] = dout.reshape(M, 2)
        dh16 = torch.empty(M, HEAD_PAD, dtype=torch.bfloat16, device=self.device)
        self._call("ptyg_nn_cast_bf16", dh.data_ptr(), dh16.data_ptr(), M * HEAD_PAD)
        self._call("ptyg_nn_col_sum", dh.data_ptr(), self.colsum.data_ptr(), self.b["head"].g.data_ptr(), M, HEAD_PAD)
        self._wgrad("head", lambda s, part: self._call(
            "ptyg_nn_dense_wgrad", dh16.data_ptr(), HEAD_PAD, self.a["d1b"].data_ptr(), c1, M, s, part.data_ptr(),
            self.status.data_ptr()), HEAD_PAD, c1, M)
        wT = torch.empty(c1, HEAD_PAD, dtype=torch.bfloat16, device=self.device)
        self._call("ptyg_nn_transpose", self.W["head"].p16.data_ptr(), wT.data_ptr(), HEAD_PAD, c1)
        self._call("ptyg_nn_gemm", dh16.data_ptr(), wT.data_ptr(), M, c1, HEAD_PAD, 1, g["d1b"].data_ptr(), None,
                   None, 0, self.status.data_ptr())
        # decoder
        dx = self._conv_bwd("d1b", ["d1a"], 1)
        g["d1a"].copy_(dx)
        dx = self._conv_bwd("d1a", ["u1", "e1b"], 1)  # [M1, c2 + c1]
        self._up_bwd(dx, c2 + c1, 0, "d2b", 2, c2)
        self._call("ptyg_nn_slice_add", dx.data_ptr(), c2 + c1, c2, g["e1b"].data_ptr(), c1, M, 0)
        dx = self._conv_bwd("d2b", ["d2a"], 2)
        g["d2a"].copy_(dx)
        dx = self._conv_bwd("d2a", ["u2", "e2b"], 2)
        self._up_bwd(dx, c3 + c2, 0, "d3b", 3, c3)
        M2 = M // 4
        self._call("ptyg_nn_slice_add", dx.data_ptr(), c3 + c2, c3, g["e2b"].data_ptr(), c2, M2, 0)
        dx = self._conv_bwd("d3b", ["d3a"], 3)
        g["d3a"].copy_(dx)
        dx = self._conv_bwd("d3a", ["u3", "e3b"], 3)
        self._up_bwd(dx, c4 + c3, 0, "bb", 4, c4)
        M3 = M // 16
        self._call("ptyg_nn_slice_add", dx.data_ptr(), c4 + c3, c4, g["e3b"].data_ptr(), c3, M3, 0)
        # bottleneck and encoder
        dx = self._conv_bwd("bb", ["ba"], 4)
        g["ba"].copy_(dx)
        dx = self._conv_bwd("ba", ["p3"], 4)
        self._pool_bwd(dx, "e3b", 3)
        dx = self._conv_bwd("e3b", ["e3a"], 3)
        g["e3a"].copy_(dx)
        dx = self._conv_bwd("e3a", ["p2"], 3)
        self._pool_bwd(dx, "e2b", 2)
        dx = self._conv_bwd("e2b", ["e2a"], 2)
        g["e2a"].copy_(dx)
        dx = self._conv_bwd("e2a", ["p1"], 2)
        self._pool_bwd(dx, "e1b", 1)
        dx = self._conv_bwd("e1b", ["e1a"], 1)
        g["e1a"].copy_(dx)
        self._first_bwd()

    def _up_bwd(self, dcat, ld, coff, dst, lv_src, c):
        B = self._shape[0]
        h, w = self.sizes[lv_src]
        self._call("ptyg_nn_up2_bwd", dcat.data_ptr(), self.gbuf[dst].data_ptr(), B, h, w, c, ld, coff)

    def _pool_bwd(self, dpooled, dst, lv):
        """gbuf[dst] += the gradient through the 2x2 pooling of level lv's map."""
        B = self._shape[0]
        h, w = self.sizes[lv]
        self._call("ptyg_nn_pool2_bwd", dpooled.data_ptr(), self.gbuf[dst].data_ptr(), B, h, w, self.a[dst].shape[1])

    def _first_bwd(self):
        torch = _torch()
        B, H, W = self._shape
        M = B * H * W
        co = self.levels[0]
        dpre16 = torch.empty(M, co, dtype=torch.bfloat16, device=self.device)
        dpre32 = torch.empty(M, co, dtype=torch.float32, device=self.device)
        self._call("ptyg_nn_relu_bwd", self.gbuf["e1a"].data_ptr(), self.a["e1a"].data_ptr(), dpre16.data_ptr(),
                   dpre32.data_ptr(), M * co)
        self._call("ptyg_nn_col_sum", dpre32.data_ptr(), self.colsum.data_ptr(), self.b["e1a"].g.data_ptr(), M, co)
        self._wgrad("e1a", lambda s, part: self._call(
            "ptyg_nn_dense_wgrad", dpre16.data_ptr(), co, self.col1.data_ptr(), FIRST_K, M, s, part.data_ptr(),
            self.status.data_ptr()), co, FIRST_K, M)

    # ---------------------------------------------------------------- training
    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        self.step += 1
        for prm in self.parameters():
            self._call("ptyg_nn_adam", prm.p.data_ptr(), prm.g.data_ptr(), prm.m.data_ptr(), prm.v.data_ptr(),
                       prm.p16.data_ptr(), prm.p.numel(), lr, b1, b2, eps, self.step, weight_decay)

    def check_status(self):
        """Raise TimeoutError (PTYG_ERR_TIMEOUT's exception) when a bounded
        tensor-core wait of an earlier launch gave up; the status word is
        cleared so the network stays usable."""
        if int(self.status.item()) != 0:
            self.status.zero_()
            raise TimeoutError("a bounded tensor-core wait gave up in the warm-start network kernels")


def _he_init(seed, specs):
    rng = np.random.default_rng(seed)
    out = {}
    for name, cins, co, _ in specs:
        ci = sum(cins)
        if name == "head":
            w = rng.standard_normal((co, ci)) * np.sqrt(1.0 / ci)
        else:
            w = rng.standard_normal((co, 9, ci)) * np.sqrt(2.0 / (9 * ci))
        out[name] = (w, np.zeros(co))
    return out
