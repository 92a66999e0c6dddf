"""CPU: the proposal network's numpy oracle.  Its backward pass, run without
the BF16 rounding, equals central finite differences of its loss in double
precision; BF16 rounding is round-to-nearest-even."""
import numpy as np

from oracle import mlp_oracle as mo


def _exact_loss_grad(w, x, t):
    # the same network in float64 without rounding: loss and analytic gradient
    w = np.asarray(w, np.float64)
    W1, b1, W2, b2 = w[0:512].reshape(32, 16), w[512:544], w[544:1568].reshape(32, 32), w[1568:1600]
    W3, b3 = w[1600:1632], w[1632]
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    y = h2 @ W3 + b3
    err = y - t
    B = x.shape[0]
    dy = 2 * err / B
    g = np.zeros(1633)
    g[1600:1632] = dy @ h2
    g[1632] = dy.sum()
    dh2 = np.where(z2 > 0, dy[:, None] * W3[None, :], 0)
    g[1568:1600] = dh2.sum(0)
    g[544:1568] = (dh2.T @ h1).reshape(-1)
    dh1 = np.where(z1 > 0, dh2 @ W2, 0)
    g[512:544] = dh1.sum(0)
    g[0:512] = (dh1.T @ x).reshape(-1)
    return float(np.mean(err * err)), g


def test_backward_formulas_match_finite_differences():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(64, 16))
    t = rng.uniform(size=64)
    w = rng.normal(size=1633) * 0.3
    l0, g = _exact_loss_grad(w, x, t)
    h = 1e-6
    for i in rng.choice(1633, 60, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (_exact_loss_grad(wp, x, t)[0] - _exact_loss_grad(wm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_rounded_oracle_close_to_exact():
    """The BF16-rounded oracle's gradient follows the exact one to BF16 precision."""
    rng = np.random.default_rng(2)
    x = rng.uniform(size=(256, 16)).astype(np.float32)
    t = rng.uniform(size=256).astype(np.float32)
    w = (rng.normal(size=1633) * 0.3).astype(np.float32)
    _, g_exact = _exact_loss_grad(w.astype(np.float64), mo.bf16(x).astype(np.float64), t.astype(np.float64))
    _, g = mo.loss_and_grad(w, x, t)
    assert np.linalg.norm(g - g_exact) <= 0.05 * np.linalg.norm(g_exact)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -3.14159, 0.0, 65504.0], np.float32)
    r = mo.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                        # tie -> even
    assert r[2] == np.float32(1.0 + 2 ** -7 + 2 ** -7) or r[2] == np.float32(1.0 + 2 ** -7)
    assert abs(r[3] - (-3.140625)) < 1e-6
    assert r[4] == 0.0
    assert (r.view(np.uint32) & 0xFFFF).max() == 0
