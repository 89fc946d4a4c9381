"""CPU restatement of the surrogate network's forward and backward passes --
TEST INFRASTRUCTURE ONLY (the checker of the GPU training kernels).

The network has no counterpart in the reference; this module restates the
library's own definition (48 -> 256 -> 256 -> 48, tanh-form GELU, mean
squared error over the 40 used outputs) in numpy, with the same bf16
roundings the tensor-core path applies to GEMM operands, so that the GPU
loss and gradients can be checked value by value.  With bf16=False it is
plain FP64 arithmetic, whose gradient is checked against finite differences.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT, N_USED = 48, 256, 48, 40
SHAPES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_OUT, N_HID)), ("b3", (N_OUT,))]
NUM_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(flat: np.ndarray) -> dict:
    out, off = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = flat[off:off + n].reshape(shape)
        off += n
    return out


def pack(parts: dict) -> np.ndarray:
    return np.concatenate([np.asarray(parts[name], dtype=np.float64).reshape(-1)
                           for name, _ in SHAPES])


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    u = 0.7978845608 * (z + 0.044715 * z ** 3)
    return 0.5 * z * (1.0 + np.tanh(u))


def gelu_grad(z):
    u = 0.7978845608 * (z + 0.044715 * z ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * 0.7978845608 * (1.0 + 0.134145 * z * z)


def forward(p: dict, x: np.ndarray, rb=True):
    r = bf16 if rb else (lambda a: np.asarray(a, dtype=np.float64))
    xb = r(x)
    z1 = xb @ r(p["W1"]).T + p["b1"]
    h1 = r(gelu(z1))
    z2 = h1 @ r(p["W2"]).T + p["b2"]
    h2 = r(gelu(z2))
    y = h2 @ r(p["W3"]).T + p["b3"]
    return {"xb": xb, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "y": y}


def loss_grad(flat: np.ndarray, x: np.ndarray, t: np.ndarray, rb=True):
    """Mean squared error over rows x 40 and its gradient (flat layout)."""
    r = bf16 if rb else (lambda a: np.asarray(a, dtype=np.float64))
    p = unpack(np.asarray(flat, dtype=np.float64))
    a = forward(p, x, rb)
    n = x.shape[0]
    diff = a["y"][:, :N_USED] - t
    loss = float(np.sum(diff * diff) / (n * N_USED))
    dy = np.zeros_like(a["y"])
    dy[:, :N_USED] = 2.0 * diff / (n * N_USED)
    dyb = r(dy)
    g = {"W3": dyb.T @ a["h2"], "b3": dy.sum(0)}
    dh2 = dyb @ r(p["W3"])
    dz2 = dh2 * gelu_grad(a["z2"])
    dz2b = r(dz2)
    g["W2"] = dz2b.T @ a["h1"]
    g["b2"] = dz2.sum(0)
    dh1 = dz2b @ r(p["W2"])
    dz1 = dh1 * gelu_grad(a["z1"])
    g["W1"] = r(dz1).T @ a["xb"]
    g["b1"] = dz1.sum(0)
    return loss, pack(g)
