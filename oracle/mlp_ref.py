"""TEST INFRASTRUCTURE ONLY: an FP64 numpy restatement of the zone-refinement proposer
network (the library's bsa_mlp_* kernels) used to check the device forward pass, loss and
gradients.  Same architecture and flattened parameter order:
W1[W][din] b1[W] W2[W][W] b2[W] W3[W][W] b3[W] w4[W] b4, ReLU on the three hidden layers,
weighted binary cross-entropy on the logit averaged with the sample weights."""
import numpy as np


def unpack(p, din, W):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = []
    for shape in ((W, din), (W,), (W, W), (W,), (W, W), (W,), (W,), (1,)):
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    assert o == p.size
    return out


def forward(p, x, din, W):
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p, din, W)
    x = np.asarray(x, dtype=np.float64)
    z1 = np.maximum(x @ W1.T + b1, 0.0)
    z2 = np.maximum(z1 @ W2.T + b2, 0.0)
    z3 = np.maximum(z2 @ W3.T + b3, 0.0)
    logit = z3 @ w4 + b4[0]
    return logit, (x, z1, z2, z3)


def loss_and_grad(p, x, y, sw, din, W):
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p, din, W)
    logit, (x, z1, z2, z3) = forward(p, x, din, W)
    y = np.asarray(y, dtype=np.float64)
    sw = np.asarray(sw, dtype=np.float64)
    ws = sw.sum()
    l = np.log1p(np.exp(-np.abs(logit))) + np.maximum(logit, 0.0) - y * logit
    loss = float((sw * l).sum() / ws)
    dl = sw * (1.0 / (1.0 + np.exp(-logit)) - y) / ws
    g_w4 = z3.T @ dl
    g_b4 = np.array([dl.sum()])
    d3 = np.outer(dl, w4) * (z3 > 0)
    g_W3, g_b3 = d3.T @ z2, d3.sum(0)
    d2 = (d3 @ W3) * (z2 > 0)
    g_W2, g_b2 = d2.T @ z1, d2.sum(0)
    d1 = (d2 @ W2) * (z1 > 0)
    g_W1, g_b1 = d1.T @ x, d1.sum(0)
    g = np.concatenate([a.ravel() for a in (g_W1, g_b1, g_W2, g_b2, g_W3, g_b3, g_w4, g_b4)])
    return loss, g


def to_bf16(p):
    """Round FP32 values to bf16 (nearest even) and back, as the device's working copy."""
    a = np.asarray(p, dtype=np.float32).copy()
    u = a.view(np.uint32)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32)
