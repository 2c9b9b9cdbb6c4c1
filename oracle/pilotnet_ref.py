"""CPU restatement of the learned pilot net (test infrastructure only).

The network has no counterpart in the reference; this file is the checker for
the GPU kernels in ``bmnd_gb300/csrc/pilotnet.cu``.  With ``bf16=True`` it
rounds the same quantities to BF16 that the GPU stores in BF16 (the weights,
the hidden activations and the hidden gradients), and accumulates in float64;
with ``bf16=False`` everything is float64, which is what the finite-difference
check of the backward pass uses.

Layout (same as the C ABI): parameters are one flat vector, layer by layer,
``W_l[tap][ci][co]`` then ``b_l[co]``; taps are in C order over the offsets
-1..1 per axis; activations are channels-last ``[batch, (D,) H, W, C]``.
"""

from __future__ import annotations

import itertools

import numpy as np


def bf16_round(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def offsets(ndim):
    return list(itertools.product((-1, 0, 1), repeat=ndim))


def layer_shapes(ndim, channels, layers):
    taps = 3 ** ndim
    shapes = []
    for l in range(layers):
        cin = 1 if l == 0 else channels
        cout = 1 if l == layers - 1 else channels
        shapes.append((taps, cin, cout))
    return shapes


def unflatten(params, ndim, channels, layers):
    ws, bs, off = [], [], 0
    for taps, cin, cout in layer_shapes(ndim, channels, layers):
        n = taps * cin * cout
        ws.append(params[off:off + n].reshape(taps, cin, cout))
        off += n
        bs.append(params[off:off + cout])
        off += cout
    assert off == params.size
    return ws, bs


def init_params(ndim, channels, layers, seed=0, out_scale=0.1):
    """He-normal initialisation; the residual branch starts small."""
    rng = np.random.default_rng(seed)
    parts = []
    shapes = layer_shapes(ndim, channels, layers)
    for l, (taps, cin, cout) in enumerate(shapes):
        std = np.sqrt(2.0 / (taps * cin))
        if l == len(shapes) - 1:
            std *= out_scale
        parts.append(rng.normal(0.0, std, size=taps * cin * cout))
        parts.append(np.zeros(cout))
    return np.concatenate(parts).astype(np.float32)


def anscombe(x):
    return (2.0 * np.sqrt(np.maximum(np.asarray(x, dtype=np.float32), 0.0) + np.float32(0.375))).astype(np.float32)


def _shift(x, off):
    """x[b, v + off, :] with zero padding; x is [B, *spatial, C]."""
    nd = len(off)
    pad = [(0, 0)] + [(1, 1)] * nd + [(0, 0)]
    xp = np.pad(x, pad)
    sl = [slice(None)] + [slice(1 + o, 1 + o + x.shape[1 + i]) for i, o in enumerate(off)] + [slice(None)]
    return xp[tuple(sl)]


def conv(x, w, ndim):
    """out[v, co] = sum_t sum_ci x[v + off_t, ci] w[t, ci, co] (float64)."""
    out = 0.0
    for t, off in enumerate(offsets(ndim)):
        out = out + np.tensordot(_shift(x, off), w[t].astype(np.float64), axes=([-1], [0]))
    return out


def conv_transpose(g, w, ndim):
    """gin[u, ci] = sum_t sum_co g[u - off_t, co] w[t, ci, co] (float64)."""
    out = 0.0
    for t, off in enumerate(offsets(ndim)):
        neg = tuple(-o for o in off)
        out = out + np.tensordot(_shift(g, neg), w[t].astype(np.float64), axes=([-1], [1]))
    return out


def wgrad(x, g, ndim):
    """dW[t, ci, co] = sum_v x[v + off_t, ci] g[v, co] (float64)."""
    taps = offsets(ndim)
    dw = np.zeros((len(taps), x.shape[-1], g.shape[-1]))
    gf = g.reshape(-1, g.shape[-1]).astype(np.float64)
    for t, off in enumerate(taps):
        xs = _shift(x, off).reshape(-1, x.shape[-1]).astype(np.float64)
        dw[t] = xs.T @ gf
    return dw


def forward(params, noisy, ndim, channels, layers, bf16=True, keep=False):
    """noisy: [B, *spatial] float32.  Returns (pilot, y, cache)."""
    rnd = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    ws, bs = unflatten(np.asarray(params, dtype=np.float32 if bf16 else np.float64), ndim, channels, layers)
    if bf16:
        ws = [bf16_round(w) for w in ws]
        bs = [bf16_round(b) for b in bs]
        a = anscombe(noisy)[..., None]
    else:
        a = (2.0 * np.sqrt(np.maximum(np.asarray(noisy, dtype=np.float64), 0.0) + 0.375))[..., None]
    acts = []
    h = a
    for l in range(layers - 1):
        z = conv(h, ws[l], ndim) + bs[l].astype(np.float64)
        h = rnd(np.maximum(z, 0.0))
        acts.append(h)
    r = conv(h, ws[-1], ndim)[..., 0] + float(bs[-1][0])
    y = a[..., 0].astype(np.float64) + r
    pilot = np.maximum((y / 2.0) ** 2 - 0.375, 0.0)
    cache = dict(a=a, acts=acts, ws=ws, bs=bs) if keep else None
    return pilot, y, cache


def loss_and_gradient(params, noisy, target, ndim, channels, layers, bf16=True):
    """Loss mean((y - A(target))^2) and its gradient (flat, parameter layout)."""
    rnd = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    _, y, c = forward(params, noisy, ndim, channels, layers, bf16=bf16, keep=True)
    t = anscombe(target).astype(np.float64) if bf16 else 2.0 * np.sqrt(
        np.maximum(np.asarray(target, dtype=np.float64), 0.0) + 0.375)
    n = y.size
    d = y - t
    loss = float(np.mean(d * d))
    gy = (2.0 / n) * d
    if bf16:
        gy = gy.astype(np.float32).astype(np.float64)
    ws, acts, a = c["ws"], c["acts"], c["a"]
    grads_w = [None] * layers
    grads_b = [None] * layers
    g = gy[..., None]
    grads_w[-1] = wgrad(acts[-1], g, ndim)
    grads_b[-1] = g.reshape(-1, 1).sum(axis=0)
    gh = rnd(conv_transpose(g, ws[-1], ndim) * (acts[-1] > 0))
    for l in range(layers - 2, 0, -1):
        grads_w[l] = wgrad(acts[l - 1], gh, ndim)
        grads_b[l] = gh.reshape(-1, gh.shape[-1]).sum(axis=0)
        gh = rnd(conv_transpose(gh, ws[l], ndim) * (acts[l - 1] > 0))
    grads_w[0] = wgrad(a, gh, ndim)
    grads_b[0] = gh.reshape(-1, gh.shape[-1]).sum(axis=0)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in zip(grads_w, grads_b)])
    return loss, flat, y
