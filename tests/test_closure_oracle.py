"""The CPU restatement of the closure network: its backward pass against finite
differences (float64, no BF16 rounding), and the BF16 rounding helper."""
import numpy as np

from oracle import mlp_ref as M


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.0078125, -3.14159, 65504.0, 1e-20], dtype=np.float32)
    b = M.bf16(a)
    assert b[0] == 1.0 and b[1] == 1.0 and b[2] == 1.0078125  # 1 + 2^-8 ties to even (down)
    assert abs(b[3] + 3.140625) < 1e-6
    assert np.all(np.abs(b - a) <= np.abs(a) * 2.0 ** -8)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 7
    p = rng.normal(0, 0.1, M.param_count())
    x = rng.normal(0, 1, (n, M.IN))
    y = rng.normal(0, 1, (n, M.NY))
    xm, xs = np.zeros(M.IN), np.ones(M.IN)
    ym, ys = np.zeros(M.NY), np.ones(M.NY)
    loss, g = M.loss_and_grad(p, x, y, xm, xs, ym, ys, bf16_emul=False, dtype=np.float64)
    idx = rng.choice(p.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = M.loss_and_grad(q, x, y, xm, xs, ym, ys, bf16_emul=False, dtype=np.float64)
        q[i] -= 2 * h
        lm, _ = M.loss_and_grad(q, x, y, xm, xs, ym, ys, bf16_emul=False, dtype=np.float64)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
