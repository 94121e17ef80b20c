"""The numpy restatement of the centre-proposal network (oracle/centre_net_ref.py) against finite
differences in float64: the checker of the CNN kernels is itself checked here, on the CPU."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import centre_net_ref as R  # noqa: E402


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    H, W = 64, 64
    p = {k: v.astype(np.float64) for k, v in R.init_params(rng, H, W).items()}
    x = rng.normal(0, 1, (2, 4, H, W))
    y = np.array([0.3, -0.7])
    _, g, _ = R.loss_and_grads(p, x, y, bf16_store=False)
    for k in ("w0", "b0", "w2", "w5", "b5", "f0w", "f0b", "f1w", "f1b"):
        for _ in range(2):
            idx = tuple(int(rng.integers(0, d)) for d in p[k].shape)
            eps = 1e-6
            p[k][idx] += eps
            lp, _, _ = R.loss_and_grads(p, x, y, False)
            p[k][idx] -= 2 * eps
            lm, _, _ = R.loss_and_grads(p, x, y, False)
            p[k][idx] += eps
            fd, an = (lp - lm) / (2 * eps), g[k][idx]
            assert abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + 1e-9, (k, idx, fd, an)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.3, 0.0], np.float32)
    r = R.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0            # halfway rounds to even
    assert r[2] == np.float32(1.0078125) and r[3] == np.float32(1.0078125)
    assert r[5] == 0.0 and abs(r[4] + 3.3) < 0.02
