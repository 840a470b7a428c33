"""CPU oracle of the conflict predictor network (float64 numpy). TEST INFRASTRUCTURE ONLY.

Restates the network the CUDA kernels compute (csmv-gpu-stm_gb300/csrc/mlp_kernels.cuh):
64 -> 128 -> 128 -> 1 with ReLU, ReLU, sigmoid, the weights W1, W2, w3 and the layer-1
activations rounded to bf16 (round to nearest even) as the kernels use them, biases in fp32,
and the gradient of the mean binary cross-entropy (straight through the activation rounding), so the kernels' forward and backward can be checked against it. Only tests/
import this module.
"""
from __future__ import annotations

import numpy as np

IN, HID = 64, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
N_PARAMS = OFF_B3 + 4


def bf16_round(a) -> np.ndarray:
    """float32 -> nearest bf16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def bf16_bits(a) -> np.ndarray:
    """uint16 bit patterns of bf16_round(a)."""
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def unpack(params):
    p = np.asarray(params, np.float32)
    w1 = bf16_round(p[OFF_W1:OFF_B1]).reshape(IN, HID).astype(np.float64)
    w2 = bf16_round(p[OFF_W2:OFF_B2]).reshape(HID, HID).astype(np.float64)
    w3 = bf16_round(p[OFF_W3:OFF_B3]).astype(np.float64)
    return (w1, p[OFF_B1:OFF_W2].astype(np.float64), w2, p[OFF_B2:OFF_W3].astype(np.float64), w3,
            float(p[OFF_B3]))


def forward(params, x, round_act=True):
    """x: [n, 64] (already bf16-representable). Returns (p, cache). round_act=False keeps the
    layer-1 activations in float64 (for checking the gradient by finite differences)."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    x = np.asarray(x, np.float64)
    a1 = x @ w1 + b1
    # the kernels feed layer 2 with bf16 activations
    h1 = np.maximum(a1, 0.0)
    if round_act:
        h1 = bf16_round(h1.astype(np.float32)).astype(np.float64)
    a2 = h1 @ w2 + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ w3 + b3
    p = 1.0 / (1.0 + np.exp(-z))
    return p, (x, h1, h2, z, w2, w3)


def loss_and_grads(params, x, y, round_act=True):
    """Mean BCE and its gradient w.r.t. the parameter block (bf16 weights treated as the
    variables, i.e. the straight-through gradient the kernels compute)."""
    p, (x, h1, h2, z, w2, w3) = forward(params, x, round_act)
    y = np.asarray(y, np.float64)
    n = x.shape[0]
    loss = float(np.mean(np.maximum(z, 0) - y * z + np.log1p(np.exp(-np.abs(z)))))
    dz = (p - y) / n
    g = np.zeros(N_PARAMS, np.float64)
    g[OFF_W3:OFF_B3] = h2.T @ dz
    g[OFF_B3] = dz.sum()
    dh2 = np.outer(dz, w3) * (h2 > 0)
    g[OFF_W2:OFF_B2] = (h1.T @ dh2).reshape(-1)
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = (dh2 @ w2.T) * (h1 > 0)
    g[OFF_W1:OFF_B1] = (x.T @ dh1).reshape(-1)
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    return loss, g


def adam(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (the kernels' update rule); returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v
