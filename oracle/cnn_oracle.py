"""CPU FP64 oracle of the learned coarse-grid corrector network (test infrastructure).

There is no reference counterpart: the reference solver has no learned
component.  This restates the network the library defines (include/ns_gpu.h,
ns_cnn_*): six periodic 3x3 convolutions, 2 -> 64 -> 64 -> 64 -> 64 -> 64 -> 1
channels, GELU after every layer but the last, mean-squared-error loss, and
the exact gradients of that loss, in float64 numpy.  Parameters use the
library's flat layout: per layer the weights [3 dy + dx][ci][co] then the
biases [co]; tap (dy, dx) reads the input at offset (dy - 1, dx - 1) with
periodic wrap.  Only tests import this module.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

CHANNELS = [(2, 64), (64, 64), (64, 64), (64, 64), (64, 64), (64, 1)]


def unflatten(params: np.ndarray):
    """Flat parameter vector -> [(w [9][ci][co], b [co]), ...]."""
    out, off = [], 0
    for ci, co in CHANNELS:
        w = params[off:off + 9 * ci * co].reshape(9, ci, co)
        off += 9 * ci * co
        b = params[off:off + co]
        off += co
        out.append((w, b))
    assert off == params.size
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dy, dx):
    """x[b, (y + dy) % H, (x + dx) % W, c]."""
    return np.roll(np.roll(x, -dy, axis=1), -dx, axis=2)


def conv(x, w, b):
    """x [B][H][W][ci], w [9][ci][co] -> [B][H][W][co]."""
    out = np.zeros(x.shape[:3] + (w.shape[2],))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        out += _shift(x, dy - 1, dx - 1) @ w[tap]
    return out + b


def conv_input_grad(d, w):
    """Gradient with respect to the input of conv for output gradient d."""
    g = np.zeros(d.shape[:3] + (w.shape[1],))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        g += _shift(d @ w[tap].T, -(dy - 1), -(dx - 1))
    return g


def conv_weight_grad(x, d):
    gw = np.zeros((9, x.shape[3], d.shape[3]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        xs = _shift(x, dy - 1, dx - 1)
        gw[tap] = np.einsum("bhwi,bhwo->io", xs, d)
    return gw


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def loss_and_grads(params, inputs, targets, s0=1.0, s1=1.0, so=1.0, bf16_weights=True):
    """inputs [B][2][H][W], targets [B][H][W] (physical units); returns (loss, flat grads)."""
    layers = unflatten(np.asarray(params, dtype=np.float64))
    if bf16_weights:
        layers = [(bf16(w), b) for w, b in layers]
    x = np.stack([inputs[:, 0] * s0, inputs[:, 1] * s1], axis=-1).astype(np.float64)
    t = targets.astype(np.float64) * so
    acts, pres = [x], []
    for l, (w, b) in enumerate(layers):
        p = conv(acts[-1], w, b)
        pres.append(p)
        acts.append(gelu(p) if l < len(layers) - 1 else p)
    out = acts[-1][..., 0]
    n = out.size
    loss = float(np.sum((out - t) ** 2) / n)
    d = (2.0 * (out - t) / n)[..., None]
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        w, _ = layers[l]
        if l < len(layers) - 1:
            d = d * gelu_grad(pres[l])
        gw = conv_weight_grad(acts[l], d)
        gb = d.sum(axis=(0, 1, 2))
        grads.append((gw, gb))
        if l > 0:
            d = conv_input_grad(d, w)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
    return loss, flat


def gelu_tanh(x):
    """GELU in the tanh form of Hendrycks and Gimpel (2016)."""
    return 0.5 * x * (1.0 + np.tanh(np.sqrt(2.0 / np.pi) * (x + 0.044715 * x ** 3)))


def forward(params, inputs, s0=1.0, s1=1.0, so=1.0, bf16_hidden_inputs=False, inference=False):
    """Network output; bf16_hidden_inputs rounds the inputs of the four 64 -> 64
    layers to bfloat16, as the library's tensor-core path stores them.
    inference: the library's tensor-core inference path, which also applies GELU
    in its tanh form to the activations it stores as bfloat16 (the outputs of
    layers 0-3; the last hidden layer keeps the erf form and FP32)."""
    layers = [(bf16(w), b) for w, b in unflatten(np.asarray(params, dtype=np.float64))]
    x = np.stack([inputs[:, 0] * s0, inputs[:, 1] * s1], axis=-1).astype(np.float64)
    bf16_hidden_inputs = bf16_hidden_inputs or inference
    for l, (w, b) in enumerate(layers):
        if bf16_hidden_inputs and 1 <= l <= len(layers) - 2:
            x = bf16(x.astype(np.float32))
        x = conv(x, w, b)
        if l < len(layers) - 1:
            x = gelu_tanh(x) if (inference and l <= len(layers) - 3) else gelu(x)
    return x[..., 0] / so
