"""CPU oracle of the surrogate network's forward and backward pass (test
infrastructure, float64 numpy).

It follows rebop_gb300/surrogate.py step for step, rounding to BF16 where the
GPU does (inputs, hidden activations, the gradients fed to the GEMMs), so the
GPU's tensor-core gradients can be checked against it; the only differences
left are FP32 accumulation and the fast exponential in the kernels.
"""

from __future__ import annotations

import numpy as np


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _softplus(x):
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def count_head(o, y, NC=32, KT=8):
    """Loss rows and gradient (before the 1/B of the mean) of the count-aware
    head: per species a block of NC class logits, then KT tail weight logits,
    means and raw scales; y rows (n_protein, n_dimer, residual_protein,
    residual_dimer)."""
    B = o.shape[0]
    HS = NC + 3 * KT
    loss = np.zeros(B)
    G = np.zeros_like(o)
    for sp in range(2):
        blk = o[:, sp * HS:(sp + 1) * HS]
        g = G[:, sp * HS:(sp + 1) * HS]
        n = y[:, sp]
        c = np.minimum(n, NC - 1).astype(int)
        lg = blk[:, :NC]
        lmax = lg.max(1, keepdims=True)
        logz = lmax + np.log(np.exp(lg - lmax).sum(1, keepdims=True))
        p = np.exp(lg - logz)
        loss += logz[:, 0] - lg[np.arange(B), c]
        g[:, :NC] = p
        g[np.arange(B), c] -= 1.0
        tail = c == NC - 1
        tw, tm, ts = blk[:, NC:NC + KT], blk[:, NC + KT:NC + 2 * KT], blk[:, NC + 2 * KT:]
        sg = _softplus(ts) + 1e-3
        e = (y[:, 2 + sp:3 + sp] - tm) / sg
        wmax = tw.max(1, keepdims=True)
        logw = wmax + np.log(np.exp(tw - wmax).sum(1, keepdims=True))
        lp = tw - logw - 0.5 * e ** 2 - np.log(sg) - 0.5 * np.log(2 * np.pi)
        m = lp.max(1, keepdims=True)
        ll = m + np.log(np.exp(lp - m).sum(1, keepdims=True))
        r = np.exp(lp - ll)
        w = np.exp(tw - logw)
        loss -= np.where(tail, ll[:, 0], 0.0)
        t = tail[:, None]
        g[:, NC:NC + KT] = np.where(t, w - r, 0.0)
        g[:, NC + KT:NC + 2 * KT] = np.where(t, -r * e / sg, 0.0)
        g[:, NC + 2 * KT:] = np.where(t, r * (1 - e ** 2) / sg * _sigmoid(ts), 0.0)
    return loss, G


def forward_backward(W, b, x, y, x_mean, x_std, K=8, head="mixture", tail=8):
    """W[i] [out][in], b[i] [out] (float64 copies of the BF16 / FP32 parameters),
    x [B][n_in], y [B][2] (mixture head: residuals) or [B][4] (count head:
    counts, residuals).  Returns (mean loss, dW list, db list)."""
    B = x.shape[0]
    h = bf16((x - x_mean) / x_std)
    H, Z = [h], []
    for i in range(len(W)):
        z = h @ bf16(W[i]).T + b[i]
        Z.append(z)
        if i < len(W) - 1:
            h = bf16(z * _sigmoid(z))
            H.append(h)
    o = Z[-1]
    if head == "count":
        rows, G = count_head(o, y, KT=tail)
        return _backward(W, H, Z, G / B, float(rows.mean()))
    logits, mu1, mu2 = o[:, :K], o[:, K:2 * K], o[:, 2 * K:3 * K]
    s1 = _softplus(o[:, 3 * K:4 * K]) + 1e-3
    s2 = _softplus(o[:, 4 * K:5 * K]) + 1e-3
    lmax = logits.max(1, keepdims=True)
    logz = lmax + np.log(np.exp(logits - lmax).sum(1, keepdims=True))
    e1 = (y[:, :1] - mu1) / s1
    e2 = (y[:, 1:] - mu2) / s2
    lp = logits - logz - 0.5 * (e1 ** 2 + e2 ** 2) - np.log(s1) - np.log(s2) - np.log(2 * np.pi)
    m = lp.max(1, keepdims=True)
    ll = m + np.log(np.exp(lp - m).sum(1, keepdims=True))
    r = np.exp(lp - ll)
    pi = np.exp(logits - logz)
    G = np.concatenate([pi - r, -r * e1 / s1, -r * e2 / s2,
                        r * (1 - e1 ** 2) / s1 * _sigmoid(o[:, 3 * K:4 * K]),
                        r * (1 - e2 ** 2) / s2 * _sigmoid(o[:, 4 * K:5 * K])], axis=1) / B
    return _backward(W, H, Z, G, float(-ll.mean()))


def _backward(W, H, Z, G, loss):
    dW, db = [None] * len(W), [None] * len(W)
    d = bf16(G)
    db[-1] = G.sum(0)
    for i in range(len(W) - 1, -1, -1):
        dW[i] = d.T @ H[i]
        if i == 0:
            break
        dh = d @ bf16(W[i])
        z = Z[i - 1]
        sg = _sigmoid(z)
        dz = dh * sg * (1 + z * (1 - sg))
        db[i - 1] = dz.sum(0)
        d = bf16(dz)
    return loss, dW, db
