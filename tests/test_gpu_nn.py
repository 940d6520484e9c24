"""The warm-start network's tensor-core kernels against NumPy and the CPU oracle.

The GPU rounds every tensor-core operand to bfloat16 and accumulates in FP32;
the oracle (``oracle/nn_oracle.py``, itself checked by finite differences)
rounds at the same places and accumulates in float64, so the comparisons are
at bfloat16 precision: relative Frobenius errors of a few 1e-3.
"""

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


def _bf(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).cuda().to(torch.bfloat16)


@pytest.mark.parametrize(
    "M,N,K,splits,epi",
    [(128, 128, 64, 1, "f32"), (300, 64, 104, 1, "f32"), (257, 40, 16, 1, "f32"), (64, 200, 4096, 7, "f32"),
     (1000, 256, 576, 1, "bf16"), (96, 8, 8, 1, "f32"), (8, 32, 2048, 5, "f32")],
)
def test_gemm_matches_numpy(torch_cuda, M, N, K, splits, epi):
    torch = torch_cuda
    from oracle.nn_oracle import bf16
    from ptylab_gb300 import _native

    lib = _native.require(0)
    rng = np.random.default_rng(M + N + K)
    A, B = rng.standard_normal((M, K)), rng.standard_normal((N, K))
    bias = rng.standard_normal(N).astype(np.float32)
    ref = bf16(A) @ bf16(B).T
    dA, dB = _bf(torch, A), _bf(torch, B)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    if epi == "f32":
        kb = -(-K // 64)
        s = min(splits, kb)
        used = -(-K // (-(-kb // s) * 64))
        part = torch.empty(used, M, N, dtype=torch.float32, device="cuda")
        _native.check(lib.ptyg_nn_gemm(dA.data_ptr(), dB.data_ptr(), M, N, K, splits, part.data_ptr(), None, None, 0,
                                       st.data_ptr(), None))
        out = torch.empty(M, N, dtype=torch.float32, device="cuda")
        _native.check(lib.ptyg_nn_reduce_splits(part.data_ptr(), out.data_ptr(), M * N, used, None))
        got = out.cpu().numpy()
    else:
        db = torch.as_tensor(bias).cuda()
        out = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
        _native.check(lib.ptyg_nn_gemm(dA.data_ptr(), dB.data_ptr(), M, N, K, 1, None, out.data_ptr(), db.data_ptr(),
                                       1, st.data_ptr(), None))
        got = out.float().cpu().numpy()
        ref = np.maximum(ref + bias, 0)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert rel_err(got, ref) < (1e-5 if epi == "f32" else 5e-3), rel_err(got, ref)


def test_conv3_with_concatenation_matches_oracle(torch_cuda):
    torch = torch_cuda
    from oracle import nn_oracle as N
    from ptylab_gb300 import _native

    lib = _native.require(0)
    rng = np.random.default_rng(5)
    B, H, W, C0, C1, Co = 2, 16, 24, 32, 16, 40
    X0, X1 = rng.standard_normal((B, H, W, C0)), rng.standard_normal((B, H, W, C1))
    w = rng.standard_normal((Co, 9, C0 + C1))
    b = rng.standard_normal(Co).astype(np.float32)
    ref = N.conv3(np.concatenate([N.bf16(X0), N.bf16(X1)], -1), N.bf16(w), b)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.empty(B * H * W, Co, dtype=torch.float32, device="cuda")
    d0, d1, dw = _bf(torch, X0), _bf(torch, X1), _bf(torch, w.reshape(Co, -1))
    db = torch.as_tensor(b).cuda()
    _native.check(lib.ptyg_nn_conv3(d0.data_ptr(), d1.data_ptr(), C0, C1, B, H, W, dw.data_ptr(), Co, out.data_ptr(),
                                    None, db.data_ptr(), 0, st.data_ptr(), None))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert rel_err(out.cpu().numpy().reshape(B, H, W, Co), ref) < 1e-5


_SOURCES = {"e1b": ["e1a"], "e2a": ["p1"], "e2b": ["e2a"], "e3a": ["p2"], "e3b": ["e3a"], "ba": ["p3"], "bb": ["ba"],
            "d3a": ["u3", "e3b"], "d3b": ["d3a"], "d2a": ["u2", "e2b"], "d2b": ["d2a"], "d1a": ["u1", "e1b"],
            "d1b": ["d1a"]}


def test_network_forward_and_gradients_match_the_oracle(torch_cuda):
    """The output and every layer's weight and bias gradient of the full
    32/64/128/256 network on two 32 x 32 patterns.  The two forward passes
    agree to bfloat16 rounding; a ReLU whose input lies within that rounding of
    zero can open on one side and not the other, which for a zero-mean
    upstream gradient moves a gradient sum far more than rounding does, so
    the oracle's backward pass runs on the GPU's own activations (the GPU's
    forward is checked separately, layer by layer)."""
    torch = torch_cuda
    from oracle import nn_oracle as N
    from ptylab_gb300.warmstart import WarmStartNet

    params = N.init_params(seed=3)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((2, 32, 32)).astype(np.float32)
    R = rng.standard_normal((2, 32, 32, 2)).astype(np.float32)
    net = WarmStartNet(params=params)
    y = net.forward(torch.as_tensor(x).cuda())
    net.backward(torch.as_tensor(R).cuda())
    torch.cuda.synchronize()
    net.check_status()
    ref = N.Net(params, round_bf16=True)
    yo = ref.forward(x[..., None].astype(np.float64))
    assert rel_err(y.cpu().numpy(), yo) < 1e-2, rel_err(y.cpu().numpy(), yo)
    # each layer's forward from the GPU's inputs: bfloat16 rounding only
    for name, srcs in _SOURCES.items():
        B = 2
        xin = np.concatenate([net.a[s_].float().cpu().numpy() for s_ in srcs], axis=-1)
        hw = xin.shape[0] // B
        side = int(round(np.sqrt(hw)))
        xin = xin.reshape(B, side, side, -1)
        w, b = params[name]
        want = np.maximum(N.conv3(N.bf16(xin), N.bf16(w), b), 0)
        got_a = net.a[name].float().cpu().numpy().reshape(want.shape)
        assert rel_err(got_a, N.bf16(want)) < 5e-3, (name, rel_err(got_a, N.bf16(want)))
    # backward on the GPU's activations
    for name, srcs in _SOURCES.items():
        xin = np.concatenate([net.a[s_].float().cpu().numpy() for s_ in srcs], axis=-1)
        side = int(round(np.sqrt(xin.shape[0] // 2)))
        yl = net.a[name].float().cpu().numpy().reshape(2, side, side, -1)
        ref.cache[name] = (xin.reshape(2, side, side, -1).astype(np.float64), yl.astype(np.float64), True,
                           [net.a[s_].shape[1] for s_ in srcs])
    ref.cache["e1a"] = (N.bf16(x[..., None]), net.a["e1a"].float().cpu().numpy().reshape(2, 32, 32, -1), True, [1])
    ref.cache["head"] = net.a["d1b"].float().cpu().numpy().reshape(2, 32, 32, -1).astype(np.float64)
    go = ref.backward(R.astype(np.float64))
    got = net.export_grads()
    bad = {}
    for name in go:
        for k, (a, b) in enumerate(zip(got[name], go[name])):
            e = rel_err(a, b)
            if e > 1e-2:
                bad[(name, "Wb"[k])] = e
    assert not bad, bad


def test_training_steps_reduce_the_loss(torch_cuda):
    torch = torch_cuda
    from ptylab_gb300.warmstart import WarmStartNet

    rng = np.random.default_rng(6)
    x = torch.as_tensor(rng.standard_normal((4, 64, 64)).astype(np.float32)).cuda()
    t = torch.as_tensor(rng.standard_normal((4, 64, 64, 2)).astype(np.float32) * 0.1).cuda()
    t = t + torch.roll(t, 1, 1) + torch.roll(t, 1, 2)  # a little spatial structure
    net = WarmStartNet(seed=7)
    losses = []
    for _ in range(40):
        y = net.forward(x)
        d = y - t
        losses.append(float((d**2).mean()))
        net.backward(2 * d / d.numel())
        net.adam_step(lr=2e-3)
    torch.cuda.synchronize()
    net.check_status()
    assert losses[-1] < 0.3 * losses[0], losses


@pytest.mark.parametrize(
    "B,H,W,C0,C1,Co",
    [(2, 32, 32, 64, 32, 64), (1, 128, 128, 16, 0, 32), (3, 16, 16, 128, 128, 128), (2, 64, 64, 32, 0, 40),
     (1, 32, 32, 256, 128, 256)],
)
@pytest.mark.parametrize("path", [1, 0])
def test_conv3_tma_and_gather_paths_match_oracle(torch_cuda, B, H, W, C0, C1, Co, path):
    """The TMA-fed convolution (path 1; the shapes here all take it) and the
    cp.async gather (path 0) against the oracle: zero padding from the
    out-of-bounds fill, the second input of a concatenation, output channels
    beyond the last full tile, bf16 + bias + ReLU and f32 epilogues."""
    torch = torch_cuda
    from oracle import nn_oracle as N
    from ptylab_gb300 import _native

    lib = _native.require(0)
    rng = np.random.default_rng(B * H + C0 + C1 + Co)
    X0 = rng.standard_normal((B, H, W, C0))
    X1 = rng.standard_normal((B, H, W, C1)) if C1 else None
    w = rng.standard_normal((Co, 9, C0 + C1)) / np.sqrt(9 * (C0 + C1))
    b = rng.standard_normal(Co).astype(np.float32)
    xin = np.concatenate([N.bf16(X0), N.bf16(X1)], -1) if C1 else N.bf16(X0)
    ref = N.conv3(xin, N.bf16(w), b)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    d0, dw = _bf(torch, X0), _bf(torch, w.reshape(Co, -1))
    d1 = _bf(torch, X1) if C1 else None
    db = torch.as_tensor(b).cuda()
    _native.check(lib.ptyg_nn_conv3_path(path))
    try:
        f32 = torch.empty(B * H * W, Co, dtype=torch.float32, device="cuda")
        _native.check(lib.ptyg_nn_conv3(d0.data_ptr(), d1.data_ptr() if C1 else None, C0, C1, B, H, W, dw.data_ptr(),
                                        Co, f32.data_ptr(), None, db.data_ptr(), 0, st.data_ptr(), None))
        o16 = torch.empty(B * H * W, Co, dtype=torch.bfloat16, device="cuda")
        _native.check(lib.ptyg_nn_conv3(d0.data_ptr(), d1.data_ptr() if C1 else None, C0, C1, B, H, W, dw.data_ptr(),
                                        Co, None, o16.data_ptr(), db.data_ptr(), 1, st.data_ptr(), None))
        torch.cuda.synchronize()
    finally:
        lib.ptyg_nn_conv3_path(1)
    assert int(st.item()) == 0
    assert rel_err(f32.cpu().numpy().reshape(ref.shape), ref) < 1e-5
    assert rel_err(o16.float().cpu().numpy().reshape(ref.shape), np.maximum(ref, 0)) < 5e-3


def test_graph_replay_matches_eager_passes(torch_cuda):
    """forward/backward replayed from captured CUDA graphs give the eager
    passes' outputs and gradients bit for bit, across a change of batch
    shape (which recaptures)."""
    torch = torch_cuda
    from ptylab_gb300.warmstart import WarmStartNet

    rng = np.random.default_rng(11)
    eager, graphed = WarmStartNet(seed=5), WarmStartNet(seed=5)
    graphed.enable_graphs()
    for B in (2, 3, 2):
        x = torch.as_tensor(rng.standard_normal((B, 32, 32)).astype(np.float32)).cuda()
        dy = torch.as_tensor(rng.standard_normal((B, 32, 32, 2)).astype(np.float32)).cuda()
        for _ in range(2):  # the first call captures, the second replays
            ye = eager.forward(x).clone()
            yg = graphed.forward(x).clone()
            eager.backward(dy)
            graphed.backward(dy)
            torch.cuda.synchronize()
            assert torch.equal(ye, yg)
            ge, gg = eager.export_grads(), graphed.export_grads()
            for name in ge:
                for a, b in zip(ge[name], gg[name]):
                    np.testing.assert_array_equal(a, b)
    eager.check_status()
    graphed.check_status()
