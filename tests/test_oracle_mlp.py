"""CPU tests of the proposer network's numpy oracle: its analytic gradient against central
finite differences (pins the oracle used by the device-gradient test).  No GPU."""
import numpy as np

from oracle import mlp_ref


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    din, W, n = 7, 16, 40
    npar = W * din + W + 2 * (W * W + W) + W + 1
    p = rng.normal(0, 0.4, npar)
    x = rng.normal(0, 1, (n, din))
    y = rng.uniform(size=n)  # soft targets exercise the same gradient
    sw = rng.uniform(0.5, 3.0, n)
    loss, g = mlp_ref.loss_and_grad(p, x, y, sw, din, W)
    h = 1e-6
    for k in rng.choice(npar, 60, replace=False):
        e = np.zeros(npar)
        e[k] = h
        fd = (mlp_ref.loss_and_grad(p + e, x, y, sw, din, W)[0] - mlp_ref.loss_and_grad(p - e, x, y, sw, din, W)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 1e-3], dtype=np.float32)
    r = mlp_ref.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-6
