"""NumPy restatement of the surrogate network's forward and backward pass (test infrastructure
only): the checker of the tensor-core kernels of arbo_gpu_fit_gb300/csrc/mlp.cu. It rounds to
BF16 (nearest, ties to even) exactly where the kernels do — inputs, weights, hidden activations
and backward signals — and computes everything else in float64, so the GPU's FP32 results must
agree to accumulation-order rounding."""
from __future__ import annotations

import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward_backward(x, t, weights, biases, dims, n_out):
    """weights[l]: float32 [dims[l+1]][dims[l]] (padded), biases[l] [dims[l+1]]; x [n][n_in],
    t [n][n_out]. Returns (loss, dW list, db list, y)."""
    n = x.shape[0]
    L = len(weights)
    xin = np.zeros((n, dims[0]))
    xin[:, : x.shape[1]] = x
    a = bf16(xin.astype(np.float32))
    acts, zs = [a], []
    for l in range(L):
        wb = bf16(weights[l])
        z = (a @ wb.T).astype(np.float32).astype(np.float64) + biases[l].astype(np.float64)
        if l + 1 < L:
            z = z.astype(np.float32).astype(np.float64)
            zs.append(z)
            a = bf16(silu(z).astype(np.float32))
            acts.append(a)
        else:
            y = z
    e = np.zeros_like(y)
    e[:, :n_out] = y[:, :n_out] - t
    loss = float((e[:, :n_out] ** 2).mean())
    dz = bf16((2.0 * e / (n * n_out)).astype(np.float32))
    dws, dbs = [None] * L, [None] * L
    for l in range(L - 1, -1, -1):
        dws[l] = dz.T @ acts[l]
        dbs[l] = dz.sum(0)
        if l > 0:
            dh = dz @ bf16(weights[l])
            dz = bf16((dh.astype(np.float32) * dsilu(zs[l - 1]).astype(np.float32)).astype(np.float32))
    return loss, dws, dbs, y
