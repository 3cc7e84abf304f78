"""FP64 numpy restatement of the warm-start U-Net (test infrastructure only).

The network has no counterpart in the reference: it is this library's learned warm start for the
nodal solve. This module restates exactly the architecture and parameter layout of the CUDA
implementation so that the tests can (1) check these analytic gradients against central finite
differences in FP64 and (2) check the GPU's BF16 tensor-core forward / backward against them.

Layout: activations are [Z, Y, X, C] arrays (channels last, interior voxels only; convolutions pad
with zeros). Parameters are one flat vector, layer by layer: w [taps][cout][cin_total] then b [cout].
Layers: encoder conv a / conv b per level (16, 32, 64, 128 channels; input 16 channels), decoder
conv a (input = concat(upsampled coarser output, skip)) / conv b for levels 2, 1, 0, and a 1x1x1
head with 16 outputs whose channel 0 is the prediction. GELU (tanh form) after every 3x3x3 conv;
2x2x2 average pooling down, nearest-neighbour upsampling up. Loss: mean over the domain voxels of
(prediction - target)^2.
"""
from __future__ import annotations

import numpy as np

LEVELS = 4
IN_C = 16
HEAD_C = 16
K = 0.7978845608028654  # sqrt(2 / pi)


def layer_specs(base=16):
    """(nin, cin0, cin1, cout, taps) per layer, in parameter order."""
    c = [base << l for l in range(LEVELS)]
    spec = []
    for l in range(LEVELS):
        spec.append((1, IN_C if l == 0 else c[l - 1], 0, c[l], 27))
        spec.append((1, c[l], 0, c[l], 27))
    for l in range(LEVELS - 2, -1, -1):
        spec.append((2, c[l + 1], c[l], c[l], 27))
        spec.append((1, c[l], 0, c[l], 27))
    spec.append((1, c[0], 0, HEAD_C, 1))
    return spec


def unpack(theta, base=16):
    """Flat parameters -> list of (w [taps, cout, cin_tot], b [cout])."""
    out, off = [], 0
    for nin, c0, c1, co, t in layer_specs(base):
        ct = c0 + c1
        w = theta[off:off + t * co * ct].reshape(t, co, ct)
        off += t * co * ct
        b = theta[off:off + co]
        off += co
        out.append((w, b))
    assert off == theta.size
    return out


def num_params(base=16):
    return sum(t * co * (c0 + c1) + co for _, c0, c1, co, t in layer_specs(base))


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(K * (x + 0.044715 * x ** 3)))


def dgelu(x):
    t = np.tanh(K * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * K * (1.0 + 3.0 * 0.044715 * x * x)


def _taps(ntaps):
    if ntaps == 1:
        return [(0, 0, 0)]
    return [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _shifted(xp, d, shape):
    z, y, x = shape
    dz, dy, dx = d
    return xp[1 + dz:1 + dz + z, 1 + dy:1 + dy + y, 1 + dx:1 + dx + x]


def conv(x, w, b):
    """Cross-correlation with zero padding: out[p] = b + sum_t x[p + t] @ w[t].T"""
    z, y, xx, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.broadcast_to(b, (z, y, xx, w.shape[1])).copy()
    for t, d in enumerate(_taps(w.shape[0])):
        out += _shifted(xp, d, (z, y, xx)) @ w[t].T
    return out


def conv_bwd(x, w, g):
    """Gradients of conv: (dx, dw, db) given upstream g = dL/d(out)."""
    z, y, xx, ci = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    gf = g.reshape(-1, g.shape[-1])
    for t, d in enumerate(_taps(w.shape[0])):
        xs = _shifted(xp, d, (z, y, xx))
        dw[t] = gf.T @ xs.reshape(-1, ci)
        dz, dy, dx = d
        dxp[1 + dz:1 + dz + z, 1 + dy:1 + dy + y, 1 + dx:1 + dx + xx] += g @ w[t]
    return dxp[1:-1, 1:-1, 1:-1], dw, gf.sum(axis=0)


def pool(x):
    z, y, xx, c = x.shape
    return x.reshape(z // 2, 2, y // 2, 2, xx // 2, 2, c).mean(axis=(1, 3, 5))


def pool_bwd(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 0), 2, 1), 2, 2) / 8.0


def upsample(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def upsample_bwd(g):
    z, y, xx, c = g.shape
    return g.reshape(z // 2, 2, y // 2, 2, xx // 2, 2, c).sum(axis=(1, 3, 5))


def forward(theta, x0, base=16):
    """x0: [Z, Y, X, 16]. Returns (prediction [Z, Y, X], cache)."""
    P = unpack(theta, base)
    cache = {"x0": x0}
    h = x0
    for l in range(LEVELS):
        if l > 0:
            h = pool(cache[("eb", l - 1)])
            cache[("pin", l)] = h
        pre = conv(h, *P[2 * l])
        cache[("ea_pre", l)], cache[("ea", l)] = pre, gelu(pre)
        pre = conv(cache[("ea", l)], *P[2 * l + 1])
        cache[("eb_pre", l)], cache[("eb", l)] = pre, gelu(pre)
    for l in range(LEVELS - 2, -1, -1):
        li = 2 * LEVELS + 2 * (LEVELS - 2 - l)
        src = cache[("eb", l + 1)] if l == LEVELS - 2 else cache[("db", l + 1)]
        up = upsample(src)
        cache[("up", l)] = up
        pre = conv(np.concatenate([up, cache[("eb", l)]], axis=-1), *P[li])
        cache[("da_pre", l)], cache[("da", l)] = pre, gelu(pre)
        pre = conv(cache[("da", l)], *P[li + 1])
        cache[("db_pre", l)], cache[("db", l)] = pre, gelu(pre)
    out = conv(cache[("db", 0)], *P[-1])
    cache["out"] = out
    return out[..., 0], cache


def loss_and_grad(theta, x0, target, dom, base=16):
    """MSE over voxels [:dom[2], :dom[1], :dom[0]] and its gradient (flat, like theta)."""
    P = unpack(theta, base)
    pred, cache = forward(theta, x0, base)
    mask = np.zeros(pred.shape, dtype=bool)
    mask[:dom[2], :dom[1], :dom[0]] = True
    n = mask.sum()
    diff = np.where(mask, pred - target, 0.0)
    loss = float((diff ** 2).sum() / n)
    grads = [None] * len(P)
    gout = np.zeros(cache["out"].shape)
    gout[..., 0] = 2.0 * diff / n
    dx, dw, db = conv_bwd(cache[("db", 0)], P[-1][0], gout)
    grads[-1] = (dw, db)
    G = dx * dgelu(cache[("db_pre", 0)])
    gskip = {}
    for l in range(LEVELS - 1):
        li = 2 * LEVELS + 2 * (LEVELS - 2 - l)
        dx, dw, db = conv_bwd(cache[("da", l)], P[li + 1][0], G)
        grads[li + 1] = (dw, db)
        G = dx * dgelu(cache[("da_pre", l)])
        xin = np.concatenate([cache[("up", l)], cache[("eb", l)]], axis=-1)
        dx, dw, db = conv_bwd(xin, P[li][0], G)
        grads[li] = (dw, db)
        cu = cache[("up", l)].shape[-1]
        gskip[l] = dx[..., cu:]
        pre_c = cache[("eb_pre", l + 1)] if l == LEVELS - 2 else cache[("db_pre", l + 1)]
        G = upsample_bwd(dx[..., :cu]) * dgelu(pre_c)
    for l in range(LEVELS - 1, -1, -1):
        dx, dw, db = conv_bwd(cache[("ea", l)], P[2 * l + 1][0], G)
        grads[2 * l + 1] = (dw, db)
        G = dx * dgelu(cache[("ea_pre", l)])
        xin = cache["x0"] if l == 0 else cache[("pin", l)]
        dx, dw, db = conv_bwd(xin, P[2 * l][0], G)
        grads[2 * l] = (dw, db)
        if l == 0:
            break
        G = (gskip[l - 1] + pool_bwd(dx)) * dgelu(cache[("eb_pre", l - 1)])
    flat = np.concatenate([np.concatenate([dw.ravel(), db.ravel()]) for dw, db in grads])
    return loss, flat


def init_params(seed=0, base=16):
    """He-normal weights, small head (only output channel 0), zero biases (same statistics as the
    CUDA initialiser; not the same numbers)."""
    rng = np.random.default_rng(seed)
    parts = []
    spec = layer_specs(base)
    for i, (nin, c0, c1, co, t) in enumerate(spec):
        ct = c0 + c1
        head = i == len(spec) - 1
        sd = 0.1 / np.sqrt(ct) if head else np.sqrt(2.0 / (t * ct))
        w = rng.standard_normal((t, co, ct)) * sd
        if head:
            w[:, 1:, :] = 0.0
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts)
