"""CPU restatement of the learned warm start's network (test infrastructure).

numpy float64 forward and backward of the 39 -> 128 -> 128 -> 4 GELU MLP with
the same loss as the library's training kernel, and the same bf16 rounding of
every tensor-core operand (inputs, weights, hidden activations, output and
hidden gradients), so the GPU gradients can be compared element by element.
Also restates the pair features and shape descriptors.  Only the tests use
this module.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

NF, K1, HID, NO = 39, 48, 128, 4
OFF_W1, OFF_B1 = 0, 128 * 48
OFF_W2 = OFF_B1 + 128
OFF_B2 = OFF_W2 + 128 * 128
OFF_W3 = OFF_B2 + 128
OFF_B3 = OFF_W3 + 4 * 128
N_PARAMS = OFF_B3 + 4


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(128, 48), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(128, 128),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(4, 128), p[OFF_B3:N_PARAMS])


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward_backward(params, X, Y, logit_weight=0.5, emulate_bf16=True):
    """Returns (grad [N_PARAMS], (loss, dir loss, logit loss), y [n,4]) of the mean loss."""
    r = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(params)
    n = X.shape[0]
    Xb, W1b, W2b, W3b = r(X), r(W1), r(W2), r(W3)
    z1 = Xb @ W1b.T
    h1 = r(gelu(z1 + b1))
    z2 = h1 @ W2b.T
    h2 = r(gelu(z2 + b2))
    y = h2 @ W3b.T + b3
    u, s = y[:, :3], y[:, 3]
    nu = np.sqrt((u * u).sum(1) + 1e-12)
    d = u / nu[:, None]
    t, z = Y[:, :3].astype(np.float64), Y[:, 3].astype(np.float64)
    c = (d * t).sum(1)
    dy = np.zeros((n, 4))
    dy[:, :3] = -(t - c[:, None] * d) / nu[:, None] / n
    sig = 1.0 / (1.0 + np.exp(-s))
    dy[:, 3] = logit_weight * (sig - z) / n
    sp = np.maximum(s, 0) + np.log1p(np.exp(-np.abs(s)))
    ldir, llog = (1.0 - c).mean(), (sp - z * s).mean()
    dyb = r(dy)
    g = np.zeros(N_PARAMS)
    g[OFF_B3:N_PARAMS] = dy.sum(0)
    g[OFF_W3:OFF_B3] = (dyb.T @ h2).flatten()
    dz2 = (dyb @ W3b) * gelu_d(z2 + b2)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz2b = r(dz2)
    g[OFF_W2:OFF_B2] = (dz2b.T @ h1).flatten()
    dz1 = (dz2b @ W2b) * gelu_d(z1 + b1)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    gw1 = r(dz1).T @ Xb
    gw1[:, NF:] = 0.0
    g[OFF_W1:OFF_B1] = gw1.flatten()
    return g, (ldir + logit_weight * llog, ldir, llog), y


def shape_descriptors(batch):
    """16 floats per shape, as the library's k_shape_desc."""
    sh = batch.shapes
    out = np.zeros((len(sh), 16), np.float64)
    for i, rec in enumerate(sh):
        k = int(rec["kind"])
        out[i, k] = 1.0
        p = rec["p"].astype(np.float64)
        if k != 5:
            out[i, 6:9] = p[:3]
            out[i, 13] = {0: p[0], 1: math.sqrt(p[0] ** 2 + p[1] ** 2 + p[2] ** 2), 2: p[0] + p[1]}.get(
                k, math.sqrt(p[0] ** 2 + p[1] ** 2))
        else:
            pts = batch.hull_points[int(rec["hull_off"]):int(rec["hull_off"]) + int(rec["hull_n"]), :3]
            pts = pts.astype(np.float64)
            out[i, 6:9] = np.abs(pts).max(0)
            e = np.sort(np.linalg.eigvalsh(np.cov(pts.T, bias=True)))[::-1]
            out[i, 9:12] = np.sqrt(np.maximum(e, 0))
            out[i, 12] = math.log2(len(pts)) * 0.1
            out[i, 13] = np.sqrt((pts * pts).sum(1)).max()
    return out


def _qmul(a, b):
    ai, aj, ak, aw = a.T
    bi, bj, bk, bw = b.T
    return np.stack([aw * bi + ai * bw + aj * bk - ak * bj, aw * bj - ai * bk + aj * bw + ak * bi,
                     aw * bk + ai * bj - aj * bi + ak * bw, aw * bw - ai * bi - aj * bj - ak * bk], 1)


def _qrot_inv(q, v):
    qv = -q[:, :3]
    t = 2.0 * np.cross(qv, v)
    return v + q[:, 3:4] * t + np.cross(qv, t)


def pair_features(batch, desc=None):
    desc = shape_descriptors(batch) if desc is None else desc
    m1, m2 = batch.m1.astype(np.float64), batch.m2.astype(np.float64)
    da, db = desc[batch.g1], desc[batch.g2]
    sc = da[:, 13] + db[:, 13]
    sc = np.where(sc > 1e-6, sc, 1.0)
    t = _qrot_inv(m1[:, :4], m2[:, 4:7] - m1[:, 4:7]) / sc[:, None]
    qa = m1[:, :4].copy()
    qa[:, :3] *= -1
    q = _qmul(qa, m2[:, :4])
    q = np.where(q[:, 3:4] < 0, -q, q)
    X = np.zeros((batch.n_pairs, K1))
    X[:, 0:3], X[:, 3:7], X[:, 7:23], X[:, 23:39] = t, q, da, db
    return X
