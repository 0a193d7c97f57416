"""The refinement proposer's device kernels (bsa_mlp_*): forward pass, loss and gradients
against the FP64 numpy oracle with the same BF16 weights (FP32 accumulation on the device:
1e-4 relative), training on a separable problem, determinism."""
import numpy as np
import pytest

from bsalib_gb300 import api
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def test_gradients_match_oracle(bsalib):
    rng = np.random.default_rng(3)
    din, W, n = 13, 128, 300
    net = api.Mlp(din, W, seed=5)
    try:
        x = rng.normal(0, 1, (n, din)).astype(np.float32)
        y = rng.uniform(size=n).astype(np.float32)
        w = rng.uniform(0.5, 2.0, n).astype(np.float32)
        pb = net.params(bf16=True)
        assert np.array_equal(pb, mlp_ref.to_bf16(net.params()))
        loss, g = net.gradients(x, y, w)
        eloss, eg = mlp_ref.loss_and_grad(pb, x, y, w, din, W)
        assert abs(loss - eloss) <= 1e-5 * abs(eloss)
        assert np.max(np.abs(g - eg)) <= 1e-4 * np.max(np.abs(eg))
        prob = net.forward(x)
        logit, _ = mlp_ref.forward(pb, x, din, W)
        assert np.max(np.abs(prob - 1 / (1 + np.exp(-logit)))) < 1e-5
    finally:
        net.close()


def test_training_separable_and_deterministic(bsalib):
    rng = np.random.default_rng(0)
    x = rng.normal(0, 1, (4000, 6)).astype(np.float32)
    y = (x[:, 0] + 0.5 * x[:, 1] - 0.2 > 0).astype(np.float32)
    w = np.ones_like(y)
    params = []
    for _ in range(2):
        net = api.Mlp(6, 64, seed=11)
        try:
            loss = net.train(x, y, w, epochs=30, batch=256, lr=2e-3, seed=3)
            acc = np.mean((net.forward(x) > 0.5) == (y > 0.5))
            params.append(net.params())
        finally:
            net.close()
        assert loss < 0.1 and acc > 0.97
    assert np.array_equal(params[0], params[1])
