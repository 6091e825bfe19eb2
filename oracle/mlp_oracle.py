"""CPU restatement of the warm-start network's arithmetic (numpy).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU
forward and backward kernels (rismo2d_gb300/csrc/rg_mlp.cu).  The network has
no counterpart in the reference; this file states what the kernels compute:

  per node n:  h0 = x[n] (128 inputs, bf16)
               z_l = W_l h_{l-1} + b_l,  h_l = bf16(gelu(z_l))   l = 1, 2, 3 (128 wide)
               y   = W_4 h_3 + b_4                               (3 outputs)
  weights are bf16 (rounded from fp32 master copies), sums in fp32 or wider;
  loss = sum_n m[n] * sum_j (y[n,j] - t[n,j])^2 / sum_n m[n]
  gradients: the exact derivative of that loss with the bf16 roundings of
  weights and activations taken as identity (straight-through).
"""

from __future__ import annotations

import math

import numpy as np

D_IN = 128
D_H = 128
D_OUT = 3


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def gelu(z: np.ndarray) -> np.ndarray:
    erf = np.vectorize(math.erf, otypes=[np.float64])
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_grad(z: np.ndarray) -> np.ndarray:
    erf = np.vectorize(math.erf, otypes=[np.float64])
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params: dict, x: np.ndarray):
    """params: W1 (128x128), b1, W2, b2, W3, b3, W4 (3x128), b4 (fp32 masters).
    Returns y and the saved activations (h0..h3 as bf16 values, z1..z3)."""
    h = [bf16(x).astype(np.float64)]
    z = []
    for l in (1, 2, 3):
        W = bf16(params[f"W{l}"]).astype(np.float64)
        zl = h[-1] @ W.T + params[f"b{l}"].astype(np.float64)
        z.append(zl)
        h.append(bf16(gelu(zl).astype(np.float32)).astype(np.float64))
    W4 = bf16(params["W4"]).astype(np.float64)
    y = h[-1] @ W4.T + params["b4"].astype(np.float64)
    return y, h, z


def loss_and_grads(params: dict, x: np.ndarray, t: np.ndarray, m: np.ndarray):
    y, h, z = forward(params, x)
    cnt = max(float(np.sum(m)), 1.0)
    r = (y - t) * m[:, None]
    loss = float(np.sum(r * (y - t)) / cnt)
    dy = 2.0 * r / cnt
    g = {}
    g["W4"] = dy.T @ h[3]
    g["b4"] = dy.sum(axis=0)
    dh = dy @ bf16(params["W4"]).astype(np.float64)
    for l in (3, 2, 1):
        dz = dh * gelu_grad(z[l - 1])
        g[f"W{l}"] = dz.T @ h[l - 1]
        g[f"b{l}"] = dz.sum(axis=0)
        if l > 1:
            dh = dz @ bf16(params[f"W{l}"]).astype(np.float64)
    return loss, y, g
