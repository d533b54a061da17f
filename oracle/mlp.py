"""CPU oracle of the learned preconditioner's network (test infrastructure:
only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it).

The network has no reference counterpart (the reference has no learned
component); this is the plain restatement that the GPU forward/backward is
checked against.  MLP 768 -> 256 -> 256 -> 256 -> 768 with ReLU between the
layers, parameters per layer W [out x in] (row-major) then b [out], loss =
mean (Y - T)^2.

Rounding contract shared with the GPU kernels: weights, layer inputs and
backward signals are rounded to BF16 (round to nearest even) before each
product; products accumulate in higher precision (FP64 here, FP32 on the
tensor cores); biases, loss and parameters are FP32.  `exact=True` drops the
BF16 rounding and works in FP64 throughout (for finite-difference checks).
"""
from __future__ import annotations

import numpy as np

LAYER_IN = (768, 256, 256, 256)
LAYER_OUT = (256, 256, 256, 768)


def nparams() -> int:
    return sum(o * i + o for i, o in zip(LAYER_IN, LAYER_OUT))


def bf16_bits(a) -> np.ndarray:
    """BF16 bit patterns of float32 values, round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16(a) -> np.ndarray:
    """Round float32 values to BF16 (returned as float32)."""
    return (bf16_bits(a).astype(np.uint32) << 16).view(np.float32)


def unpack(params: np.ndarray):
    out, o = [], 0
    for i, n in zip(LAYER_IN, LAYER_OUT):
        W = params[o:o + n * i].reshape(n, i)
        o += n * i
        b = params[o:o + n]
        o += n
        out.append((W, b))
    return out


def init_params(seed: int = 0, out_scale: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for l, (i, n) in enumerate(zip(LAYER_IN, LAYER_OUT)):
        sd = np.sqrt(2.0 / i) * (out_scale if l == 3 else 1.0)
        parts += [rng.normal(0.0, sd, n * i), rng.normal(0.0, 0.01, n)]
    return np.concatenate(parts).astype(np.float32)


def forward_backward(params, X, T, exact: bool = False):
    """Returns (Y, loss, grads) for one batch (rows of X and T)."""
    rnd = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: bf16(a).astype(np.float64))
    f32 = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: np.asarray(a, np.float32))
    layers = unpack(np.asarray(params, np.float64 if exact else np.float32))
    acts = [rnd(X)]  # BF16 inputs of each layer
    for l, (W, b) in enumerate(layers):
        z = f32(acts[-1] @ rnd(W).T) + f32(b)
        if l < 3:
            acts.append(rnd(np.maximum(f32(z), 0)))
        else:
            Y = f32(z)
    E = np.asarray(Y, np.float64) - np.asarray(T, np.float64)
    loss = float(np.mean(E * E))
    d = rnd(f32(2.0 * E / E.size))
    grads = [None] * 4
    for l in range(3, -1, -1):
        W, _ = layers[l]
        gW = f32(d.T @ acts[l])
        gb = f32(d.sum(axis=0))
        grads[l] = (gW, gb)
        if l > 0:
            dh = f32(d @ rnd(W))
            d = rnd(np.where(acts[l] > 0, dh, 0.0))
    flat = np.concatenate([np.concatenate([gW.ravel(), gb.ravel()]) for gW, gb in grads])
    return np.asarray(Y), loss, flat
