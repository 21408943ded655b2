"""CPU oracle of the learned warm-start network (TEST INFRASTRUCTURE ONLY).

Restates, in float64 NumPy, the network that csrc/mlp.cu trains and evaluates on the device, so
the GPU's loss and parameter gradients can be checked: hidden layers tanh(W h + b), a linear
output layer, mean squared error over all outputs.  The products use the parameters rounded to
BF16 (round to nearest even), as the device does; everything else is float64 here.  There is
no reference counterpart (the reference has no learned component); the layout of the parameter
vector follows include/ibgb300_learn.h: per layer W_l (dims[l+1] x dims[l], row-major), then b_l.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a: np.ndarray) -> np.ndarray:
    """float32 -> nearest BF16 (ties to even), returned as float32 (finite inputs)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray, dims: list[int]):
    """[(W_l, b_l)] views of the flat parameter vector."""
    out, off = [], 0
    for l in range(len(dims) - 1):
        n_in, n_out = dims[l], dims[l + 1]
        W = params[off: off + n_in * n_out].reshape(n_out, n_in)
        off += n_in * n_out
        b = params[off: off + n_out]
        off += n_out
        out.append((W, b))
    assert off == params.size
    return out


def _w(W: np.ndarray, bf16: bool) -> np.ndarray:
    return bf16_round(W).astype(np.float64) if bf16 else np.asarray(W, dtype=np.float64)


def forward(params: np.ndarray, dims: list[int], x: np.ndarray, bf16: bool = True):
    """Activations [x, h1, ..., y_hat] (float64), weights BF16-rounded unless ``bf16`` is False."""
    layers = unpack(np.asarray(params, dtype=np.float32 if bf16 else np.float64), dims)
    acts = [np.asarray(x, dtype=np.float64)]
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ _w(W, bf16).T + b.astype(np.float64)
        acts.append(np.tanh(z) if l + 1 < len(layers) else z)
    return acts


def loss_and_grad(params: np.ndarray, dims: list[int], x: np.ndarray, y: np.ndarray, bf16: bool = True):
    """Mean squared error over all outputs and its gradient with respect to the flat parameters
    (the weight gradient of a layer is dZ^T h with the BF16 forward; dh = dZ W_bf16)."""
    layers = unpack(np.asarray(params, dtype=np.float32 if bf16 else np.float64), dims)
    acts = forward(params, dims, x, bf16)
    yh = acts[-1]
    n = yh.size
    err = yh - np.asarray(y, dtype=np.float64)
    loss = float(np.sum(err * err) / n)
    dz = 2.0 * err / n
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        if l + 1 < len(layers):
            dz = dz * (1.0 - acts[l + 1] ** 2)
        gW = dz.T @ acts[l]
        gb = dz.sum(axis=0)
        grads[l] = (gW, gb)
        if l > 0:
            dz = dz @ _w(W, bf16)
    flat = np.concatenate([np.concatenate([gW.reshape(-1), gb]) for gW, gb in grads])
    return loss, flat
