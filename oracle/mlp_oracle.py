"""CPU FP64 reference of the learned-seed MLP's loss and gradient.

TEST INFRASTRUCTURE ONLY (the checker of pnjl_mlp_loss_grad).  It restates the network
3 -> 128 -> 128 -> 128 -> 5 with SiLU and applies BF16 rounding at the same points the GPU
kernels do -- the weights, the hidden activations h1..h3 and the back-propagated deltas of
layers 3 and 2 -- while computing everything else in FP64.  Parameter packing follows
pnjl_mlp_param_count(): W1[128][3], b1, W2[128][128], b2, W3[128][128], b3, W4[5][128], b4.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 3, 128, 5
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("W4", (OUT, H)), ("b4", (OUT,))]
PARAM_COUNT = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(flat):
    out, off = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[off:off + n], dtype=np.float64).reshape(shape)
        off += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def bf16(a):
    """Round to bfloat16 (round to nearest, ties to even) and return as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_grad(flat_params, x, y):
    """x [n,3] standardised inputs, y [n,5] standardised targets -> (loss, flat gradient)."""
    p = unpack(flat_params)
    W1, W2, W3, W4 = (bf16(p[k]) for k in ("W1", "W2", "W3", "W4"))
    n = x.shape[0]
    z1 = x @ W1.T + p["b1"]
    h1 = bf16(silu(z1))
    z2 = h1 @ W2.T + p["b2"]
    h2 = bf16(silu(z2))
    z3 = h2 @ W3.T + p["b3"]
    h3 = bf16(silu(z3))
    out = h3 @ W4.T + p["b4"]
    inv = 1.0 / (n * OUT)
    diff = out - y
    loss = float(np.sum(diff * diff) * inv)
    dout = 2.0 * diff * inv
    g = {"W4": dout.T @ h3, "b4": dout.sum(0)}
    d3 = bf16((dout @ W4) * silu_grad(z3))
    g["W3"], g["b3"] = d3.T @ h2, d3.sum(0)
    d2 = bf16((d3 @ W3) * silu_grad(z2))
    g["W2"], g["b2"] = d2.T @ h1, d2.sum(0)
    d1 = (d2 @ W2) * silu_grad(z1)
    g["W1"], g["b1"] = d1.T @ x, d1.sum(0)
    return loss, pack(g)


def forward(flat_params, x):
    p = unpack(flat_params)
    W1, W2, W3, W4 = (bf16(p[k]) for k in ("W1", "W2", "W3", "W4"))
    h1 = bf16(silu(x @ W1.T + p["b1"]))
    h2 = bf16(silu(h1 @ W2.T + p["b2"]))
    h3 = bf16(silu(h2 @ W3.T + p["b3"]))
    return h3 @ W4.T + p["b4"]
