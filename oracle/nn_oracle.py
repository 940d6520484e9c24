"""CPU oracle of the warm-start network (encoder-decoder) and its gradients.

TEST INFRASTRUCTURE ONLY: the checker for ``ptylab_gb300.warmstart.network``,
never called by the package.  PtyLab has no network, so this oracle restates
the build's own architecture in NumPy (float64): 3x3 'same' convolutions
(NHWC activations, weights ``[Co][tap][Ci]`` with tap = 3 (dy+1) + (dx+1), the
decoder's inputs the channel concatenation [upsampled, skip]), ReLU, 2x2
average pooling, nearest 2x upsampling and a 1x1 output convolution, with
hand-written backward passes.  ``round_bf16=True`` rounds every tensor-core
operand (weights, layer inputs, backward gradients) to bfloat16 as the GPU
does, so the GPU can be compared at the precision it computes in; with
``round_bf16=False`` the gradients are exact and are themselves checked by
central finite differences in ``tests/test_nn_oracle.py``.
"""

from __future__ import annotations

import numpy as np

LEVELS = (32, 64, 128, 256)


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layer_specs(levels=LEVELS):
    """(name, kind, input channels of each concatenated source, output channels, relu)."""
    c1, c2, c3, c4 = levels
    return [
        ("e1a", "conv", (1,), c1, True), ("e1b", "conv", (c1,), c1, True),
        ("e2a", "conv", (c1,), c2, True), ("e2b", "conv", (c2,), c2, True),
        ("e3a", "conv", (c2,), c3, True), ("e3b", "conv", (c3,), c3, True),
        ("ba", "conv", (c3,), c4, True), ("bb", "conv", (c4,), c4, True),
        ("d3a", "conv", (c4, c3), c3, True), ("d3b", "conv", (c3,), c3, True),
        ("d2a", "conv", (c3, c2), c2, True), ("d2b", "conv", (c2,), c2, True),
        ("d1a", "conv", (c2, c1), c1, True), ("d1b", "conv", (c1,), c1, True),
        ("head", "head", (c1,), 2, False),
    ]


def init_params(seed=0, levels=LEVELS):
    """He-normal weights (float64), zero biases: {name: (W, b)}; conv W [Co, 9, Ci], head W [2, Ci]."""
    rng = np.random.default_rng(seed)
    out = {}
    for name, kind, cins, co, _ in layer_specs(levels):
        ci = sum(cins)
        if kind == "head":
            w = rng.standard_normal((co, ci)) * np.sqrt(1.0 / ci)
        else:
            w = rng.standard_normal((co, 9, ci)) * np.sqrt(2.0 / (9 * ci))
        out[name] = (w, np.zeros(co))
    return out


def _patches(x):
    """x [B, H, W, C] -> [B, H, W, 9, C] zero-padded 3x3 neighbourhoods."""
    B, H, W, C = x.shape
    xp = np.zeros((B, H + 2, W + 2, C), dtype=x.dtype)
    xp[:, 1:-1, 1:-1] = x
    return np.stack([xp[:, dy:dy + H, dx:dx + W] for dy in range(3) for dx in range(3)], axis=3)


def conv3(x, w, b):
    return np.einsum("bhwtc,otc->bhwo", _patches(x), w) + b


def conv3_bwd(x, w, dy):
    """Gradients of conv3 w.r.t. x, w, b for upstream gradient dy."""
    B, H, W, _ = x.shape
    dw = np.einsum("bhwtc,bhwo->otc", _patches(x), dy)
    db = dy.sum(axis=(0, 1, 2))
    dpat = np.einsum("bhwo,otc->bhwtc", dy, w)  # gradient of each patch entry
    dxp = np.zeros((B, H + 2, W + 2, x.shape[3]))
    t = 0
    for ddy in range(3):
        for ddx in range(3):
            dxp[:, ddy:ddy + H, ddx:ddx + W] += dpat[:, :, :, t]
            t += 1
    return dxp[:, 1:-1, 1:-1], dw, db


def pool2(x):
    B, H, W, C = x.shape
    return x.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool2_bwd(dy):
    return 0.25 * np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2)


def up2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up2_bwd(dy):
    B, H, W, C = dy.shape
    return dy.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


class Net:
    """The encoder-decoder: forward() caches what backward() needs."""

    def __init__(self, params, round_bf16=False):
        self.p = params
        self.r = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))

    def _conv(self, name, srcs, relu):
        w, b = self.p[name]
        x = np.concatenate([self.r(s) for s in srcs], axis=-1)
        pre = conv3(x, self.r(w), b)
        y = np.maximum(pre, 0) if relu else pre
        self.cache[name] = (x, y, relu, [s.shape[-1] for s in srcs])
        return self.r(y) if relu else y  # the GPU stores ReLU outputs in bf16

    def forward(self, x):
        self.cache = {}
        e1 = self._conv("e1b", [self._conv("e1a", [x], True)], True)
        e2 = self._conv("e2b", [self._conv("e2a", [pool2(e1)], True)], True)
        e3 = self._conv("e3b", [self._conv("e3a", [pool2(e2)], True)], True)
        bt = self._conv("bb", [self._conv("ba", [pool2(e3)], True)], True)
        d3 = self._conv("d3b", [self._conv("d3a", [up2(bt), e3], True)], True)
        d2 = self._conv("d2b", [self._conv("d2a", [up2(d3), e2], True)], True)
        d1 = self._conv("d1b", [self._conv("d1a", [up2(d2), e1], True)], True)
        w, b = self.p["head"]
        xin = self.r(d1)
        self.cache["head"] = xin
        return np.einsum("bhwc,oc->bhwo", xin, self.r(w)) + b

    def _conv_bwd(self, name, dy, grads):
        x, y, relu, splits = self.cache[name]
        w, _ = self.p[name]
        dpre = self.r(dy * (y > 0)) if relu else self.r(dy)
        dx, dw, db = conv3_bwd(x, self.r(w), dpre)
        grads[name] = (dw, db)
        out, c0 = [], 0
        for c in splits:
            out.append(dx[..., c0:c0 + c])
            c0 += c
        return out

    def backward(self, dout):
        """Parameter gradients {name: (dW, db)} for upstream gradient dout [B, H, W, 2]."""
        g = {}
        w, _ = self.p["head"]
        dout = self.r(dout)
        g["head"] = (np.einsum("bhwo,bhwc->oc", dout, self.cache["head"]), dout.sum(axis=(0, 1, 2)))
        dd1 = np.einsum("bhwo,oc->bhwc", dout, self.r(w))
        (dd1a,) = self._conv_bwd("d1b", dd1, g)
        du1, de1 = self._conv_bwd("d1a", dd1a, g)
        (dd2a,) = self._conv_bwd("d2b", up2_bwd(du1), g)
        du2, de2 = self._conv_bwd("d2a", dd2a, g)
        (dd3a,) = self._conv_bwd("d3b", up2_bwd(du2), g)
        du3, de3 = self._conv_bwd("d3a", dd3a, g)
        (dba,) = self._conv_bwd("bb", up2_bwd(du3), g)
        (dp3,) = self._conv_bwd("ba", dba, g)
        (de3a,) = self._conv_bwd("e3b", de3 + pool2_bwd(dp3), g)
        (dp2,) = self._conv_bwd("e3a", de3a, g)
        (de2a,) = self._conv_bwd("e2b", de2 + pool2_bwd(dp2), g)
        (dp1,) = self._conv_bwd("e2a", de2a, g)
        (de1a,) = self._conv_bwd("e1b", de1 + pool2_bwd(dp1), g)
        self._conv_bwd("e1a", de1a, g)
        return g
