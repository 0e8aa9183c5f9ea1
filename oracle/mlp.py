"""TEST INFRASTRUCTURE ONLY: the MLP corrector in NumPy, against which the
tests compare the GPU's tensor-core forward and backward kernels (pibiti_gb300/csrc/sph_mlp.cu).

Double precision, with every value the GPU holds in BF16 rounded to BF16
at the same place: inputs, weights, hidden activations, and the output and
hidden gradients that feed the next product.  Parameter vector layout:
W1[16][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3].
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 16, 64, 3
SIZES = [("W1", (IN, HID)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)),
         ("W3", (HID, OUT)), ("b3", (OUT,))]
COUNT = sum(int(np.prod(s)) for _, s in SIZES)


def bf16(a) -> np.ndarray:
    """Round to BF16 (nearest, ties to even) and return as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def bf16_bits(a) -> np.ndarray:
    """BF16 bit patterns (uint16) of float values (nearest, ties to even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def split(params):
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = np.asarray(params[o:o + k], np.float64).reshape(shape)
        o += k
    return out


def init(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SIZES:
        if name.startswith("W"):
            parts.append(rng.normal(0, 1.0 / np.sqrt(shape[0]), size=shape).ravel())
        else:
            parts.append(np.zeros(shape).ravel())
    return np.concatenate(parts).astype(np.float32)


def forward(params, x, rounding: bool = True):
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    p = split(params)
    x = r(x)
    W1, W2, W3 = r(p["W1"]), r(p["W2"]), r(p["W3"])
    b1, b2, b3 = p["b1"], p["b2"], p["b3"]
    h1 = r(np.tanh(x @ W1 + b1))
    h2 = r(np.tanh(h1 @ W2 + b2))
    y = h2 @ W3 + b3
    return y, (x, h1, h2, W1, W2, W3)


def loss_and_grad(params, x, target, rounding: bool = True):
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    y, (xb, h1, h2, W1, W2, W3) = forward(params, x, rounding)
    n = len(x)
    e = y - np.asarray(target, np.float64)
    loss = float((e * e).sum() / (3 * n))
    dy = r(2.0 * e / (3 * n))
    dz2 = r((dy @ W3.T) * (1.0 - h2 * h2))
    dz1 = r((dz2 @ W2.T) * (1.0 - h1 * h1))
    g = {"W3": h2.T @ dy, "b3": dy.sum(0), "W2": h1.T @ dz2, "b2": dz2.sum(0),
         "W1": xb.T @ dz1, "b1": dz1.sum(0)}
    return loss, np.concatenate([g[name].ravel() for name, _ in SIZES])
