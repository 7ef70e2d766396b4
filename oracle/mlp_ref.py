"""CPU oracle of the warm-start network — TEST INFRASTRUCTURE ONLY.

numpy FP64 restatement of the forward and backward passes that libblpg's
kernels (blpg_mlp_*) perform, on the same packed parameter layout
(W_1 b_1 ... W_L b_L, W_l of shape out_pad x in_pad, row-major).  With
``emulate_bf16`` it rounds to BF16 exactly where the GPU stores BF16 (the
input, the weights, the post-ReLU activations and the gradients fed to the
GEMMs), so the GPU's gradients can be compared with it elementwise; without
it, it is a plain FP64 network for finite-difference checks.
"""
from __future__ import annotations

import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray, d_in_pad: int, hidden: int, layers: int, d_out_pad: int):
    Ws, bs = [], []
    off = 0
    for l in range(layers + 1):
        i = d_in_pad if l == 0 else hidden
        o = d_out_pad if l == layers else hidden
        Ws.append(params[off:off + o * i].reshape(o, i).astype(np.float64))
        off += o * i
        bs.append(params[off:off + o].astype(np.float64))
        off += o
    assert off == params.size
    return Ws, bs


def forward_backward(params, X, Y, d_in_pad, hidden, layers, d_out_pad, d_out,
                     emulate_bf16=True):
    """(loss, packed gradient) for rows X (B x d_in_pad), labels Y (B x d_out_pad)."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs = unpack(np.asarray(params), d_in_pad, hidden, layers, d_out_pad)
    B = X.shape[0]
    acts = [r(X)]
    for l in range(layers):
        h = np.maximum(acts[-1] @ r(Ws[l]).T + bs[l], 0.0)
        acts.append(r(h))
    z = acts[-1] @ r(Ws[layers]).T + bs[layers]
    valid = np.arange(d_out_pad) < d_out
    Y = np.asarray(Y, dtype=np.float64)
    zv, yv = z[:, valid], Y[:, valid]
    loss = float(np.sum(np.log1p(np.exp(-np.abs(zv))) + np.maximum(zv, 0) - yv * zv))
    dz = np.zeros_like(z)
    dz[:, valid] = (1.0 / (1.0 + np.exp(-zv)) - yv) / B
    gW = [None] * (layers + 1)
    gb = [None] * (layers + 1)
    for l in range(layers, -1, -1):
        xin = acts[l]
        gW[l] = r(dz).T @ xin
        gb[l] = dz.sum(0)
        if l == 0:
            break
        dh = r(dz) @ r(Ws[l])
        dz = dh * (acts[l] > 0)
    out = []
    for l in range(layers + 1):
        out.append(gW[l].ravel())
        out.append(gb[l])
    return loss, np.concatenate(out)


def forward(params, X, d_in_pad, hidden, layers, d_out_pad, emulate_bf16=True):
    """Logits of rows X (B x d_in_pad), as forward_backward computes them."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs = unpack(np.asarray(params), d_in_pad, hidden, layers, d_out_pad)
    h = r(X)
    for l in range(layers):
        h = r(np.maximum(h @ r(Ws[l]).T + bs[l], 0.0))
    return h @ r(Ws[layers]).T + bs[layers]


def init_params(d_in, d_in_pad, hidden, layers, d_out, d_out_pad, seed=0):
    """Small random parameters in the packed layout (padding zero)."""
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(layers + 1):
        i = d_in_pad if l == 0 else hidden
        o = d_out_pad if l == layers else hidden
        W = rng.normal(0, np.sqrt(2.0 / i), (o, i))
        if l == 0:
            W[:, d_in:] = 0
        if l == layers:
            W[d_out:, :] = 0
        parts += [W.ravel(), rng.normal(0, 0.1, o) * (np.arange(o) < (d_out if l == layers else o))]
    return np.concatenate(parts)
