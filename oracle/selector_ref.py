"""ORACLE -- test infrastructure only.

FP64 NumPy restatement of the selector MLP (12 -> 64 -> 64 -> 11, three softmax
heads) used to check the GPU kernels' logits and gradients.  Like the kernels,
every matrix-product operand is rounded to bfloat16 (round to nearest even);
products are then accumulated in FP64 here (FP32 on the GPU)."""
from __future__ import annotations

import numpy as np

IN, H, OUT = 16, 64, 16
NF, NO = 12, 11
HEADS = [(0, 2), (2, 8), (8, 11)]
OFF = {}
_o = 0
for name, size in [("W1", IN * H), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * OUT), ("b3", OUT)]:
    OFF[name] = (_o, size)
    _o += size
NPARAMS = _o


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float32)
    get = lambda k: p[OFF[k][0]:OFF[k][0] + OFF[k][1]].astype(np.float64)
    return (get("W1").reshape(IN, H), get("b1"), get("W2").reshape(H, H), get("b2"),
            get("W3").reshape(H, OUT), get("b3"))


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.zeros((len(x), IN))
    X[:, :NF] = x
    h1 = np.maximum(bf16(X) @ bf16(W1) + b1, 0)
    h1 = h1.astype(np.float32).astype(np.float64)  # the kernel keeps activations in fp32
    h2 = np.maximum(bf16(h1) @ bf16(W2) + b2, 0).astype(np.float32).astype(np.float64)
    z = bf16(h2) @ bf16(W3) + b3
    return X, h1, h2, z


def loss_grad(p, x, labels):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = len(x)
    X, h1, h2, z = forward(p, x)
    dz = np.zeros_like(z)
    loss = 0.0
    for hd, (lo, hi) in enumerate(HEADS):
        zz = z[:, lo:hi]
        m = zz.max(1, keepdims=True)
        e = np.exp(zz - m)
        s = e.sum(1, keepdims=True)
        lab = labels[:, hd]
        loss += float(np.sum(np.log(s[:, 0]) + m[:, 0] - zz[np.arange(n), lab]) / n)
        g = e / s
        g[np.arange(n), lab] -= 1.0
        dz[:, lo:hi] = g / n
    dz = dz.astype(np.float32).astype(np.float64)
    gW3 = bf16(h2).T @ bf16(dz)
    gb3 = dz.sum(0)
    d2 = (bf16(dz) @ bf16(W3).T) * (h2 > 0)
    d2 = d2.astype(np.float32).astype(np.float64)
    gW2 = bf16(h1).T @ bf16(d2)
    gb2 = d2.sum(0)
    d1 = (bf16(d2) @ bf16(W2).T) * (h1 > 0)
    d1 = d1.astype(np.float32).astype(np.float64)
    gW1 = bf16(X).T @ bf16(d1)
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    # padded inputs / outputs carry no gradient in the update
    return g, loss
