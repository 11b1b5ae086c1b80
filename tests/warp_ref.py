"""CPU reference of the learned warp (test infrastructure): the masked autoregressive MLP,
its |f|-weighted negative log-likelihood, the analytic gradient, and the sampler y -> x.
FP64 arithmetic on the same BF16-rounded weights the GPU kernels use."""
from __future__ import annotations

import numpy as np

H, K, ALPHA = 64, 16, 0.3
KP = K + 1


class Layout:
    def __init__(self, D):
        self.D, self.DK = D, D * KP
        o = 0
        self.oW1 = o; o += H * D; self.ob1 = o; o += H
        self.oW2 = o; o += H * H; self.ob2 = o; o += H
        self.oW3 = o; o += H * H; self.ob3 = o; o += H
        self.oW4 = o; o += self.DK * H; self.ob4 = o; o += self.DK
        self.n = o


def masks(D):
    L = Layout(D)
    m = np.ones(L.n)
    hd = 1 + np.arange(H) % (D - 1)
    m[L.oW1:L.ob1] = (hd[:, None] >= np.arange(1, D + 1)[None, :]).ravel()
    mm = (hd[:, None] >= hd[None, :]).ravel()
    m[L.oW2:L.ob2] = mm
    m[L.oW3:L.ob3] = mm
    od = np.arange(L.DK) // KP + 1
    m[L.oW4:L.ob4] = (od[:, None] > hd[None, :]).ravel()
    return m


def bf16(p):
    f = np.asarray(p, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, D):
    L = Layout(D)
    W1 = p[L.oW1:L.ob1].reshape(H, D); b1 = p[L.ob1:L.oW2]
    W2 = p[L.oW2:L.ob2].reshape(H, H); b2 = p[L.ob2:L.oW3]
    W3 = p[L.oW3:L.ob3].reshape(H, H); b3 = p[L.ob3:L.oW4]
    W4 = p[L.oW4:L.ob4].reshape(L.DK, H); b4 = p[L.ob4:]
    return W1, b1, W2, b2, W3, b3, W4, b4


def forward(p, X):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p, X.shape[1])
    x = 2 * X - 1
    a1 = x @ W1.T + b1; h1 = np.tanh(a1)
    a2 = h1 @ W2.T + b2; h2 = np.tanh(a2)
    a3 = h2 @ W3.T + b3; h3 = np.tanh(a3)
    lg = h3 @ W4.T + b4
    return x, h1, h2, h3, lg


def _heights(lg):
    """Knot heights v (unit-integral piecewise-linear density mixed with the uniform one)."""
    a = np.exp(lg - lg.max(axis=-1, keepdims=True))
    S = (a[..., :-1] + a[..., 1:]).sum(axis=-1, keepdims=True) / (2 * K)
    return a, S, (1 - ALPHA) * a / S + ALPHA


def loss_grad(p, X, w):
    """Loss -sum_i w_i log q(x_i) / sum w and its gradient w.r.t. the (BF16-rounded) weights."""
    D = X.shape[1]
    q = bf16(p)
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(q, D)
    wn = w / w.sum()
    x, h1, h2, h3, lg = forward(q, X)
    n = X.shape[0]
    lg = lg.reshape(n, D, KP)
    a, S, v = _heights(lg)
    S = S[..., 0]
    b = np.clip(np.floor(X * K).astype(int), 0, K - 1)
    t = X * K - b
    ab = np.take_along_axis(a, b[:, :, None], 2)[:, :, 0]
    ab1 = np.take_along_axis(a, (b + 1)[:, :, None], 2)[:, :, 0]
    mix = (1 - t) * ab + t * ab1
    qv = (1 - ALPHA) * mix / S + ALPHA
    loss = float(-(wn[:, None] * np.log(qv)).sum())
    k1 = -wn[:, None] * (1 - ALPHA) / (qv * S)
    k2 = mix / S / (2 * K)
    own = np.zeros_like(a)
    np.put_along_axis(own, b[:, :, None], (1 - t)[:, :, None], axis=2)
    own_b1 = np.zeros_like(a)
    np.put_along_axis(own_b1, (b + 1)[:, :, None], t[:, :, None], axis=2)
    nc = np.full(KP, 2.0)
    nc[0] = nc[-1] = 1.0
    dl = (k1[:, :, None] * a * (own + own_b1 - k2[:, :, None] * nc)).reshape(n, D * KP)
    g = np.zeros_like(p)
    L = Layout(D)
    g[L.oW4:L.ob4] = (dl.T @ h3).ravel(); g[L.ob4:] = dl.sum(0)
    d3 = (dl @ W4) * (1 - h3 * h3)
    g[L.oW3:L.ob3] = (d3.T @ h2).ravel(); g[L.ob3:L.oW4] = d3.sum(0)
    d2 = (d3 @ W3) * (1 - h2 * h2)
    g[L.oW2:L.ob2] = (d2.T @ h1).ravel(); g[L.ob2:L.oW3] = d2.sum(0)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    g[L.oW1:L.ob1] = (d1.T @ x).ravel(); g[L.ob1:L.oW2] = d1.sum(0)
    return loss, g


def warp_map(p, Y):
    """y -> (x, 1/q(x)) by sequential inversion of the per-dimension quadratic CDFs."""
    n, D = Y.shape
    q = bf16(p)
    X = np.zeros((n, D))
    wt = np.ones(n)
    for d in range(D):
        _, _, _, _, lg = forward(q, X)
        _, _, v = _heights(lg[:, d * KP:(d + 1) * KP])
        mass = 0.5 * (v[:, :-1] + v[:, 1:]) / K
        cum = np.cumsum(mass, axis=1)
        b = np.minimum((Y[:, d:d + 1] >= cum).sum(axis=1), K - 1)
        lo = np.where(b > 0, np.take_along_axis(cum, np.maximum(b - 1, 0)[:, None], 1)[:, 0], 0.0)
        vb = np.take_along_axis(v, b[:, None], 1)[:, 0]
        dv = np.take_along_axis(v, (b + 1)[:, None], 1)[:, 0] - vb
        r = np.maximum(Y[:, d] - lo, 0) * K
        t = 2 * r / (vb + np.sqrt(np.maximum(vb * vb + 2 * dv * r, 0)))
        t = np.clip(t, 0, 1 - 6e-8)
        X[:, d] = (b + t) / K
        wt /= vb + dv * t
    return X, wt
