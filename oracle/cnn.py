"""FP64 numpy restatement of the learned preconditioner's network (test
infrastructure only): 5 bias-free 3x3 layers 2 -> 32 -> 32 -> 32 -> 32 -> 2 with
ReLU between layers, tensors [B][H][W][C], layer weights [9 taps][Cout][Cin]
(tap = 3*dy + dx for the offset (dy-1, dx-1)), zero padding, mean-squared-error
loss.  Used to check the GPU forward pass and weight gradients.  The network
has no reference counterpart, so there is nothing to pin beyond its definition.
"""
from __future__ import annotations

import numpy as np

CIN = [2, 32, 32, 32, 32]
COUT = [32, 32, 32, 32, 2]


def split(w):
    out, o = [], 0
    for ci, co in zip(CIN, COUT):
        n = 9 * ci * co
        out.append(np.asarray(w[o:o + n], dtype=np.float64).reshape(9, co, ci))
        o += n
    return out


def conv(x, W):
    B, H, Wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((B, H, Wd, W.shape[1]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        y += xp[:, dy:dy + H, dx:dx + Wd, :] @ W[tap].T
    return y


def bf16(a):
    """round to the nearest bfloat16 (ties to even), as the GPU stores activations"""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(w, x, round_bf16=False):
    """round_bf16 stores the hidden activations in bfloat16, as the GPU does"""
    Ws = split(w)
    acts = [np.asarray(x, dtype=np.float64)]
    a = acts[0]
    for l, W in enumerate(Ws):
        z = conv(a, W)
        a = np.maximum(z, 0.0) if l < 4 else z
        if round_bf16 and l < 4:
            a = bf16(a)
        acts.append(a)
    return a, acts


def gradients(w, x, t, round_bf16=False):
    """loss = mean((net(x) - t)^2); returns (loss, flat gradient).  round_bf16
    rounds hidden activations and the back-propagated hidden gradients to
    bfloat16 where the GPU stores them."""
    Ws = split(w)
    y, acts = forward(w, x, round_bf16)
    n = y.size
    d = 2.0 * (y - t) / n
    loss = float(np.sum((y - t) ** 2) / n)
    grads = [None] * 5
    for l in range(4, -1, -1):
        a = acts[l]
        B, H, Wd, _ = a.shape
        ap = np.pad(a, ((0, 0), (1, 1), (1, 1), (0, 0)))
        g = np.zeros_like(Ws[l])
        dxp = np.zeros_like(ap)
        for tap in range(9):
            dy, dx = divmod(tap, 3)
            xs = ap[:, dy:dy + H, dx:dx + Wd, :]
            g[tap] = np.einsum("bhwc,bhwd->dc", xs, d)
            dxp[:, dy:dy + H, dx:dx + Wd, :] += d @ Ws[l][tap]
        grads[l] = g
        if l > 0:
            d = dxp[:, 1:-1, 1:-1, :] * (acts[l] > 0)
            if round_bf16:
                d = bf16(d)
    return loss, np.concatenate([g.ravel() for g in grads])
