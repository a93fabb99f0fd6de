"""The surrogate network restated in numpy (TEST INFRASTRUCTURE): the checker
for the library's BF16 tensor-core training kernels (cs_mlp_*).

Same architecture and roundings as the device code: every GEMM operand rounded
to bfloat16 (round to nearest even), products summed in float64 here (the device
sums in FP32), bias added in FP32, GELU (erf form) in FP32, the MSE gradient
2 (y - t) / (n * n_out) rounded to bfloat16, and the GELU derivative applied to
the FP32 input gradient before rounding to bfloat16.
"""
import numpy as np
from scipy.special import erf


def bf16(x):
    """round float32 values to the nearest bfloat16 (ties to even), as float32"""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def gelu(z):
    return (0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))).astype(np.float32)


def gelu_grad(z):
    z = z.astype(np.float64)
    return (0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)).astype(np.float32)


def forward(layers, x):
    """layers: list of 4 dicts {w (out x in_padded), b}; x (n x n_in).
    Returns output and the saved pre-activations / activations."""
    kin = layers[0]["w"].shape[1]
    a = np.zeros((x.shape[0], kin), np.float32)
    a[:, :x.shape[1]] = x
    a = bf16(a)
    acts, zs = [a], []
    for l in range(3):
        z = (a.astype(np.float64) @ bf16(layers[l]["w"]).T.astype(np.float64)).astype(np.float32) + layers[l]["b"]
        zs.append(z)
        a = bf16(gelu(z))
        acts.append(a)
    y = (a.astype(np.float64) @ bf16(layers[3]["w"]).T.astype(np.float64)).astype(np.float32) + layers[3]["b"]
    return y, zs, acts


def gradients(layers, x, t):
    """mean squared error and its gradients: list of (gw, gb) per layer"""
    y, zs, acts = forward(layers, x)
    n, nout = y.shape
    d = y - t
    loss = float(np.mean(d.astype(np.float64) ** 2))
    dz = bf16(2.0 * d / (n * nout))
    grads = [None] * 4
    for l in range(3, -1, -1):
        gw = (dz.astype(np.float64).T @ acts[l].astype(np.float64)).astype(np.float32)
        gb = dz.astype(np.float64).sum(axis=0).astype(np.float32)
        grads[l] = (gw, gb)
        if l == 0:
            break
        dh = (dz.astype(np.float64) @ bf16(layers[l]["w"]).astype(np.float64)).astype(np.float32)
        dz = bf16(dh * gelu_grad(zs[l - 1]))
    return loss, grads
