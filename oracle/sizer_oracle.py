"""CPU oracle of the learned tile sizer (test infrastructure only: tests import
it as the checker of the device kernels; nothing in the library calls it).

The network has no reference counterpart. This module restates, in numpy FP64,
what the device kernels compute:

* forward: x[16] -> relu(x W1 + b1)[64] -> relu(h1 W2 + b2)[64] -> h2 W3 + b3[4],
  with every parameter rounded to BF16 (round to nearest even) first, as the
  device's inference weights are;
* loss: mean over samples and the 3 used outputs of w (out - target)^2, with
  w = UNDER_WEIGHT where the first output (the max count) is below its target
  and 1 elsewhere;
* gradients of that loss with respect to every parameter, evaluated at the
  BF16-rounded parameters (the device trains FP32 master weights with the
  gradient of the BF16 network).

The flat parameter layout is W1[16][64], b1[64], W2[64][64], b2[64], W3[64][4],
b3[4], row-major with the input index first.
"""
from __future__ import annotations

import numpy as np

NF, NH, NO, NUSED = 16, 64, 4, 3
UNDER_WEIGHT = 4.0
SHAPES = [("W1", (NF, NH)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NH, NO)), ("b3", (NO,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16_round(p: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 -> FP32 with round to nearest, ties to even (NaN-free inputs)."""
    u = np.ascontiguousarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = params[o:o + n].reshape(shape)
        o += n
    return out


def pack(parts: dict) -> np.ndarray:
    return np.concatenate([np.asarray(parts[name], np.float64).reshape(-1) for name, _ in SHAPES])


def forward(params: np.ndarray, X: np.ndarray, quantize: bool = True):
    """Returns (out[n][4], h1, h2, z1, z2) in FP64."""
    p = bf16_round(params) if quantize else np.asarray(params, np.float32)
    P = {k: v.astype(np.float64) for k, v in unpack(p.astype(np.float64)).items()}
    X = np.asarray(X, np.float64)
    z1 = X @ P["W1"] + P["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ P["W2"] + P["b2"]
    h2 = np.maximum(z2, 0)
    out = h2 @ P["W3"] + P["b3"]
    return out, h1, h2, z1, z2


def loss_and_gradients(params: np.ndarray, X: np.ndarray, T: np.ndarray, quantize: bool = True):
    """Weighted squared error over the used outputs and its gradient (FP64)."""
    p = bf16_round(params) if quantize else np.asarray(params, np.float32)
    P = {k: v.astype(np.float64) for k, v in unpack(p.astype(np.float64)).items()}
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    n = len(X)
    out, h1, h2, _, _ = forward(params, X, quantize)
    err = np.zeros_like(out)
    err[:, :NUSED] = out[:, :NUSED] - T
    w = np.ones_like(out)
    w[:, 0] = np.where(err[:, 0] < 0, UNDER_WEIGHT, 1.0)
    loss = float((w * err ** 2)[:, :NUSED].sum() / (n * NUSED))
    dout = 2.0 * w * err / (n * NUSED)
    g = {"W3": h2.T @ dout, "b3": dout.sum(0)}
    dz2 = (dout @ P["W3"].T) * (h2 > 0)
    g["W2"] = h1.T @ dz2
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ P["W2"].T) * (h1 > 0)
    g["W1"] = X.T @ dz1
    g["b1"] = dz1.sum(0)
    return loss, pack(g)
