"""The surrogate network's BF16 tensor-core kernels (cs_mlp_*) against the
numpy restatement in oracle/mlp_oracle.py: forward outputs, the gradients of
every layer, and a short training run. Tolerances are norm-wise: both sides
round the same operands to bfloat16; the device accumulates in FP32, the
oracle in float64, so an intermediate occasionally rounds to the neighbouring
bfloat16 value."""
import numpy as np
import pytest

import crystalscatter_gb300 as cs
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def relnorm(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def make(n_in=8, hidden=256, n_out=384, seed=3):
    net = cs.SurrogateMLP(n_in, hidden, n_out, seed=seed)
    rng = np.random.default_rng(seed)
    layers = []
    for l in range(4):
        w0 = net.layer(l)["w"]
        w = (rng.standard_normal(w0.shape) / np.sqrt(w0.shape[1])).astype(np.float32)
        if l == 0:
            w[:, n_in:] = 0.0  # padded input columns
        b = (0.1 * rng.standard_normal(w0.shape[0])).astype(np.float32)
        net.set_layer(l, w, b)
        layers.append({"w": w, "b": b})
    return net, layers, rng


def test_forward_matches_oracle():
    import torch
    net, layers, rng = make()
    x = rng.uniform(-1, 1, (200, 8)).astype(np.float32)  # not a multiple of 128: padded rows
    y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    y_ref, _, _ = mlp_oracle.forward(layers, x)
    assert y.shape == y_ref.shape
    assert relnorm(y, y_ref) < 2e-3


def test_gradients_match_oracle():
    import torch
    net, layers, rng = make()
    x = rng.uniform(-1, 1, (256, 8)).astype(np.float32)
    t = rng.standard_normal((256, 384)).astype(np.float32)
    loss = net.gradients(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    loss_ref, grads = mlp_oracle.gradients(layers, x, t)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    for l in range(4):
        g = net.layer(l)
        assert relnorm(g["gw"], grads[l][0]) < 5e-3, l
        assert relnorm(g["gb"], grads[l][1]) < 5e-3, l


def test_training_lowers_loss():
    import torch
    net, _, rng = make(seed=5)
    x = rng.uniform(-1, 1, (1024, 8)).astype(np.float32)
    grid = np.linspace(-1, 1, 384, dtype=np.float32)
    t = np.sin(3 * x[:, :1] * grid[None, :] + x[:, 1:2]).astype(np.float32)  # smooth target family
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = net.train_step(xd, td, 1e-3)
    for _ in range(300):
        last = net.train_step(xd, td, 1e-3)
    assert last < 0.1 * first


def test_bilinear_upsample():
    import torch
    rng = np.random.default_rng(1)
    a = rng.standard_normal((3, 8, 8)).astype(np.float32)
    got = cs.upsample_bilinear(torch.from_numpy(a).cuda(), 4).cpu().numpy()
    f, s = 4, 8
    c = np.clip((np.arange(s * f) + 0.5) / f - 0.5, 0, s - 1)
    i0 = np.floor(c).astype(int)
    i1 = np.minimum(i0 + 1, s - 1)
    w = (c - i0).astype(np.float32)
    ref = ((1 - w)[None, :, None] * ((1 - w)[None, None, :] * a[:, i0][:, :, i0] + w[None, None, :] * a[:, i0][:, :, i1])
           + w[None, :, None] * ((1 - w)[None, None, :] * a[:, i1][:, :, i0] + w[None, None, :] * a[:, i1][:, :, i1]))
    assert np.abs(got - ref).max() < 1e-5
