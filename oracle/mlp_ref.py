"""NumPy restatement of the surrogate MLP (forward, loss, hand-written
backward) with the device's BF16 roundings, in FP64 otherwise.

TEST INFRASTRUCTURE ONLY: the checker of the tensor-core MLP kernels
(dwarf-p-ice3_gb300/csrc/mlp.cu, surrogate.cu) in tests/.  The network has
no counterpart in the reference; this file states what the kernels compute:

    h_0 = bf16(x)
    z_l = h_{l-1} W_l^T + b_l,  h_l = bf16(GELU(z_l))      (hidden layers)
    y   = h_L W_out^T + b_out
    loss = mean over rows of  sum_r [ BCE(y_2r, t_2r) + t_2r (y_2r+1 - t_2r+1)^2 ]

with W in BF16 (the FP32 masters rounded to nearest even), the output
cotangent dY and the hidden cotangents dZ rounded to BF16 before they enter
a GEMM, and GELU in its tanh form.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    nan = np.isnan(f)
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


_K0 = np.sqrt(2.0 / np.pi)
_K1 = 0.044715 * _K0


def gelu(z):
    """GELU, tanh form (Hendrycks & Gimpel 2016); the kernels evaluate the
    tanh with the hardware approximation (relative error below 2^-10)."""
    return 0.5 * z * (1.0 + np.tanh(z * (_K0 + _K1 * z * z)))


def dgelu(z):
    th = np.tanh(z * (_K0 + _K1 * z * z))
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * (_K0 + 3.0 * _K1 * z * z)


def unpack(params: np.ndarray, layout: List[Tuple[int, int, int, int]]):
    """[(W [out][in], b [out])] per weight layer from the flat FP32 vector."""
    p = np.asarray(params, dtype=np.float32)
    return [(p[w:w + o * i].reshape(o, i), p[b:b + o]) for (w, b, o, i) in layout]


def _f32(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def _ident(x):
    return np.asarray(x, dtype=np.float64)


def forward(params, layout, x, quant: bool = True) -> Tuple[np.ndarray, Dict]:
    """quant=False: the same network entirely in FP64 (no BF16/FP32 roundings)."""
    q, r32 = (bf16, _f32) if quant else (_ident, _ident)
    layers = unpack(params, layout) if quant else [(np.asarray(W, np.float64), np.asarray(b, np.float64))
                                                   for (W, b) in unpack64(params, layout)]
    h = q(x)
    hs, zs = [h], []
    for (W, b) in layers[:-1]:
        z = r32(h @ q(W).T + np.asarray(b, np.float64))
        zs.append(z)
        h = q(gelu(z))
        hs.append(h)
    W, b = layers[-1]
    y = h @ q(W).T + np.asarray(b, np.float64)
    return y, {"h": hs, "z": zs}


def unpack64(params, layout):
    p = np.asarray(params, dtype=np.float64)
    return [(p[w:w + o * i].reshape(o, i), p[b:b + o]) for (w, b, o, i) in layout]


def loss_grad(params, layout, x, targets, quant: bool = True) -> Tuple[float, np.ndarray]:
    """Loss and gradient (flat, FP64) of one batch as the kernels form them
    (quant=False: exact FP64 backpropagation of the unrounded network)."""
    q, r32 = (bf16, _f32) if quant else (_ident, _ident)
    layers = unpack(params, layout) if quant else unpack64(params, layout)
    n = x.shape[0]
    y, st = forward(params, layout, x, quant)
    nr = y.shape[1] // 2
    logit, pred = y[:, 0::2], y[:, 1::2]
    act, val = targets[:, 0:2 * nr:2].astype(np.float64), targets[:, 1:2 * nr:2].astype(np.float64)
    p = 1.0 / (1.0 + np.exp(-logit))
    e = np.where(act > 0.5, pred - val, 0.0)
    loss = float(np.mean(np.sum(-(act * np.log(np.maximum(p, 1e-12)) + (1 - act) * np.log(np.maximum(1 - p, 1e-12)))
                                + e * e, axis=1)))
    dyf = np.empty_like(y)
    dyf[:, 0::2] = (p - act) / n
    dyf[:, 1::2] = 2.0 * e / n
    dyf = r32(dyf)
    g = np.zeros(sum(o * i + o for (_, _, o, i) in layout), dtype=np.float64)
    d = q(dyf)
    dfull = dyf
    for li in range(len(layers) - 1, -1, -1):
        wo, bo, o, i = layout[li]
        hin = st["h"][li]
        g[wo:wo + o * i] = (d.T @ hin).ravel()
        g[bo:bo + o] = dfull.sum(axis=0)
        if li > 0:
            W = q(layers[li][0])
            dz = r32((d @ W) * dgelu(st["z"][li - 1]))
            dfull = dz
            d = q(dz)
    return loss, g
