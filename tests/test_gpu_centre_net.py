"""Centre-proposal CNN kernels against the numpy restatement (oracle/centre_net_ref.py): forward
outputs, loss and every parameter gradient of one batch, and a few Adam steps that fit it."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

import recview_gb300 as rv

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import centre_net_ref as R  # noqa: E402

pytestmark = pytest.mark.gpu
ORDER = [f"{k}{l}" for l in range(6) for k in ("w", "b")] + ["f0w", "f0b", "f1w", "f1b"]


def pack(p):
    return np.concatenate([p[k].ravel() for k in ORDER]).astype(np.float32)


def unpack(vec, like):
    out, o = {}, 0
    for k in ORDER:
        n = like[k].size
        out[k] = vec[o:o + n].reshape(like[k].shape)
        o += n
    return out


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    H, W, N = 64, 128, 3
    p = R.init_params(rng, H, W)
    for k in p:
        if k.startswith("b") or k.endswith("b"):
            p[k] = rng.normal(0, 0.05, p[k].shape).astype(np.float32)   # non-zero biases exercise db
    x = R.bf16(rng.normal(0, 1, (N, 4, H, W)).astype(np.float32))
    y = rng.normal(0, 1, N).astype(np.float32)
    d_x = torch.from_numpy(x).cuda().to(torch.bfloat16)
    return H, W, N, p, x, y, d_x


def make_net(gpu, H, W, N, p):
    net = C.c_void_p()
    assert gpu.RvCentreNetCreate(H, W, N, 1, C.byref(net)) == 0, rv.last_error()
    assert gpu.RvCentreNetNumParams(net) == pack(p).size
    flat = pack(p)
    assert gpu.RvCentreNetSetParams(net, flat.ctypes.data_as(C.POINTER(C.c_float))) == 0
    return net


def test_forward_matches_oracle(gpu, case):
    H, W, N, p, x, y, d_x = case
    net = make_net(gpu, H, W, N, p)
    try:
        mu, s = np.zeros(N, np.float32), np.zeros(N, np.float32)
        assert gpu.RvCentreNetForward(net, C.c_void_p(d_x.data_ptr()), N, mu.ctypes.data_as(C.POINTER(C.c_float)),
                                      s.ctypes.data_as(C.POINTER(C.c_float)), None) == 0
        mu_o, s_o, _ = R.forward(p, x)
        # FP32 sums in another order can flip a bf16 rounding of a stored activation: tiny deviations
        assert np.allclose(mu, mu_o, rtol=2e-2, atol=2e-3) and np.allclose(s, s_o, rtol=2e-2, atol=2e-3)
    finally:
        gpu.RvCentreNetDestroy(net)


def test_gradients_match_oracle(gpu, case):
    H, W, N, p, x, y, d_x = case
    net = make_net(gpu, H, W, N, p)
    try:
        g = np.zeros(pack(p).size, np.float32)
        loss = C.c_float()
        assert gpu.RvCentreNetGradients(net, C.c_void_p(d_x.data_ptr()), y.ctypes.data_as(C.POINTER(C.c_float)), N,
                                        C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float)), None) == 0
        loss_o, g_o, _ = R.loss_and_grads(p, x, y)
        assert abs(loss.value - loss_o) <= 1e-2 * abs(loss_o) + 1e-4
        gg = unpack(g, p)
        for k in ORDER:
            a, b = gg[k].astype(np.float64), g_o[k].astype(np.float64)
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert rel < 3e-2, (k, rel)
    finally:
        gpu.RvCentreNetDestroy(net)


def test_adam_steps_fit_a_batch(gpu, case):
    torch = pytest.importorskip("torch")
    H, W, N, p, x, y, d_x = case
    net = make_net(gpu, H, W, N, p)
    try:
        d_y = torch.from_numpy(y).cuda()
        losses = []
        for _ in range(60):
            l = C.c_float()
            assert gpu.RvCentreNetTrainStep(net, C.c_void_p(d_x.data_ptr()), C.cast(C.c_void_p(d_y.data_ptr()),
                                            C.POINTER(C.c_float)), N, 1e-3, C.byref(l), None) == 0
            losses.append(l.value)
        assert losses[-1] < losses[0] - 0.5, losses[::10]
    finally:
        gpu.RvCentreNetDestroy(net)
