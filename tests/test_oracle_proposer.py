"""The proposer's CPU oracle: its analytic backward pass against float64
finite differences (no BF16 rounding), and its layout / mask."""
import numpy as np

from oracle import proposer as op


def test_layout_and_mask():
    lay, total = op.layout()
    assert total == 139632
    m = op.trainable_mask()
    p = op.init_params(1)
    assert np.all(p[~m] == 0)  # padding starts at zero


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    b = 2
    x = rng.uniform(0.0, 4.0, (b, 60, 80, 2))
    x[rng.uniform(size=x.shape) < 0.1] = 0.0
    p = op.init_params(7).astype(np.float64)
    p += 0.01 * rng.normal(size=p.shape) * op.trainable_mask()  # non-zero biases too
    t = rng.normal(size=(b, 6))
    out, cache = op.forward(p, x, quantize=False)
    loss, g = op.backward(cache, t)
    assert abs(loss - op.loss_only(p, x, t)) < 1e-12
    idx = rng.choice(np.flatnonzero(op.trainable_mask()), 40, replace=False)
    lay, _ = op.layout()
    # at least one entry from every tensor
    idx = np.concatenate([idx, [o for o, _ in lay]])
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (op.loss_only(pp, x, t) - op.loss_only(pm, x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1e-3, abs(fd)) + 1e-9, (i, fd, g[i])
