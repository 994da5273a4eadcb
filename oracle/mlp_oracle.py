"""TEST INFRASTRUCTURE, not part of the product: a numpy restatement of the
learned window's network (include/cor_window.h) to check the device's
forward pass and gradient.

The reference has no network, so there is nothing to pin this against but
mathematics: `check_backprop` compares the analytic gradient with central
differences in float64.  `forward`/`gradient` with bf16=True round what the
device keeps in BF16 (inputs, weights, hidden activations, the backward
dZ and dY) exactly as the device does (round to nearest even), accumulating
in float64, so the device differs only by FP32 summation order and by the
occasional BF16 rounding that order flips.
"""
from __future__ import annotations

import numpy as np

SHAPES = [(256, 19), (256,), (256, 256), (256,), (256, 256), (256,), (256, 256), (256,), (2, 256), (2,)]


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _split(p):
    out, o = [], 0
    for shp in SHAPES:
        n = int(np.prod(shp))
        out.append(np.asarray(p[o:o + n], np.float64).reshape(shp))
        o += n
    return out


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _f32(a):
    return np.asarray(a, np.float32).astype(np.float64)


def forward(p, x, bf16_mode=True):
    """-> (y, cache) for inputs x (n, 19)."""
    P = _split(p)
    r = bf16 if bf16_mode else (lambda a: np.asarray(a, np.float64))
    f = _f32 if bf16_mode else (lambda a: a)
    h = r(x)
    cache = [h]
    zs = []
    for l in range(4):
        W, b = r(P[2 * l]), P[2 * l + 1]
        z = f(h @ W.T + b)
        zs.append(z)
        h = r(_silu(z))
        cache.append(h)
    y = f(h @ r(P[8]).T + P[9])
    return y, (cache, zs)


def gradient(p, x, t, bf16_mode=True):
    """-> (loss, gradient in the parameter layout) of the mean squared error."""
    P = _split(p)
    r = bf16 if bf16_mode else (lambda a: np.asarray(a, np.float64))
    y, (hs, zs) = forward(p, x, bf16_mode)
    n = x.shape[0]
    e = y - t
    loss = float(np.sum(e * e) / (n * 2))
    d = (2.0 / (n * 2)) * e
    if bf16_mode:
        d = _f32(d)
    grads = [None] * 10
    grads[9] = d.sum(0)
    db = r(d)
    grads[8] = db.T @ hs[4]
    up = db @ r(P[8])
    for l in range(3, -1, -1):
        dz = up * _silu_grad(zs[l])
        if bf16_mode:
            dz = _f32(dz)
        grads[2 * l + 1] = dz.sum(0)
        dzb = r(dz)
        grads[2 * l] = dzb.T @ hs[l]
        if l > 0:
            up = dzb @ r(P[2 * l])
    return loss, np.concatenate([g.ravel() for g in grads])


def check_backprop(seed=0, n=6, eps=1e-6) -> float:
    """Largest |central difference - analytic gradient| / (1 + |gradient|) in
    float64 over sampled parameters of a random small problem."""
    rng = np.random.default_rng(seed)
    p = np.concatenate([rng.normal(0, 0.2, int(np.prod(s))) for s in SHAPES])
    x = rng.normal(0, 1, (n, 19))
    t = rng.normal(0, 1, (n, 2))
    _, g = gradient(p, x, t, bf16_mode=False)
    idx = rng.choice(p.size, 200, replace=False)
    idx = np.concatenate([idx, np.arange(p.size - 514, p.size)[:40]])
    worst = 0.0
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = gradient(q, x, t, bf16_mode=False)
        q[i] -= 2 * eps
        lm, _ = gradient(q, x, t, bf16_mode=False)
        num = (lp - lm) / (2 * eps)
        worst = max(worst, abs(num - g[i]) / (1.0 + abs(g[i])))
    return worst
