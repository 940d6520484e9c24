"""The warm-start network's CPU oracle: its hand-written gradients against
central finite differences (float64, no rounding), on a small copy of the
architecture."""

import numpy as np

from oracle import nn_oracle as N


def test_oracle_gradients_match_finite_differences():
    levels = (8, 8, 16, 16)
    p = N.init_params(seed=1, levels=levels)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 16, 16, 1))
    R = rng.standard_normal((2, 16, 16, 2))

    def loss(params):
        return float(np.sum(N.Net(params).forward(x) * R))

    net = N.Net(p)
    net.forward(x)
    g = net.backward(R)
    h = 1e-6
    for name in ("e1a", "e2b", "ba", "d3a", "d1a", "head"):
        w, b = p[name]
        for which, arr, grad in (("W", w, g[name][0]), ("b", b, g[name][1])):
            d = rng.standard_normal(arr.shape)
            up = dict(p)
            dn = dict(p)
            up[name] = (w + h * d, b) if which == "W" else (w, b + h * d)
            dn[name] = (w - h * d, b) if which == "W" else (w, b - h * d)
            fd = (loss(up) - loss(dn)) / (2 * h)
            an = float(np.sum(grad * d))
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (name, which, fd, an)


def test_bf16_rounding_is_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = N.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125  # ties to even, then up
    assert abs(r[3] - (-3.140625)) < 1e-12 and r[4] == 0.0
