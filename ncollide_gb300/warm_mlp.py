"""Learned warm start: training and use of the direction-predicting MLP.

The network (ncg_mlp.cu) maps a pair's relative pose and two shape
descriptors to GJK's first search direction plus a separation logit.  It is
trained on pairs that the plain GJK labels itself: the direction GJK/EPA
returns (the separating axis, or the EPA normal) expressed in the first
shape's frame, and whether GJK found an intersection.  Forward, backward and
the optimiser step all run in the library's CUDA kernels (tcgen05 tensor
cores, bf16 operands, f32 accumulation); this module only feeds batches.

    params = train(ctx, batch, epochs=20, batch_size=8192)
    ctx.set_mlp_params(params); ctx.set_warm_start(WARM_MLP)
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as N
from . import query as Q

N_PARAMS, N_INPUTS, HID, NF = N.MLP_N_PARAMS, N.MLP_N_INPUTS, 128, 39
OFF_W1, OFF_B1 = 0, 128 * 48
OFF_W2 = OFF_B1 + 128
OFF_B2 = OFF_W2 + 128 * 128
OFF_W3 = OFF_B2 + 128
OFF_B3 = OFF_W3 + 4 * 128


def _p(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def init_params(seed=0, device="cuda"):
    """Uniform(+-1/sqrt(fan_in)) weights, zero biases; padded inputs stay zero."""
    g = torch.Generator().manual_seed(seed)
    p = torch.zeros(N_PARAMS, dtype=torch.float32)
    w1 = (torch.rand((128, 48), generator=g) * 2 - 1) / math.sqrt(NF)
    w1[:, NF:] = 0
    p[OFF_W1:OFF_B1] = w1.flatten()
    p[OFF_W2:OFF_B2] = ((torch.rand((128, 128), generator=g) * 2 - 1) / math.sqrt(128)).flatten()
    p[OFF_W3:OFF_B3] = ((torch.rand((4, 128), generator=g) * 2 - 1) / math.sqrt(128)).flatten()
    return p.to(device)


def features(db: Q.DeviceBatch):
    """Shape descriptors [S,16] and pair features [N,48] on the device."""
    L = N.load()
    desc = torch.empty((max(db.n_shapes, 1), 16), dtype=torch.float32, device=db.m1.device)
    X = torch.empty((max(db.n_pairs, 1), N_INPUTS), dtype=torch.float32, device=db.m1.device)
    cb = db.c_struct()
    N.check(L.ncg_mlp_features(ctypes.byref(cb), _p(desc), _p(X), _stream()), "ncg_mlp_features")
    return desc[:db.n_shapes], X[:db.n_pairs]


def infer(db: Q.DeviceBatch, params):
    """The network's world-space unit start direction per pair."""
    L = N.load()
    desc = torch.empty((max(db.n_shapes, 1), 16), dtype=torch.float32, device=db.m1.device)
    out = torch.empty((max(db.n_pairs, 1), 3), dtype=torch.float32, device=db.m1.device)
    err = torch.zeros(1, dtype=torch.int32, device=db.m1.device)
    cb = db.c_struct()
    N.check(L.ncg_mlp_infer(ctypes.byref(cb), _p(params), _p(desc), _p(out), _p(err), _stream()), "ncg_mlp_infer")
    if int(err.item()) != 0:
        raise N.NcgError("ncg_mlp_infer: a tensor-core wait timed out")
    return out[:db.n_pairs]


def _qrot_inv(q, v):
    """Rotates v [N,3] by the inverse of unit quaternions q [N,4] (i, j, k, w)."""
    qv = -q[:, :3]
    t = 2.0 * torch.cross(qv, v, dim=1)
    return v + q[:, 3:4] * t + torch.cross(qv, t, dim=1)


def labels(ctx: Q.Context, db: Q.DeviceBatch):
    """Plain-GJK labels [N,4]: the returned direction in the first shape's frame
    and 1 when the pair intersects (contact with prediction 0, every pair by
    GJK/EPA)."""
    old = (ctx.dispatch, ctx.warm_start)
    ctx.set_dispatch(N.DISPATCH_SUPPORT_MAP)
    ctx.set_warm_start(N.WARM_NONE)
    o = Q.contact_batch(ctx, db, 0.0)
    ctx.set_dispatch(old[0])
    ctx.set_warm_start(old[1])
    d = _qrot_inv(db.m1[:, :4], o["dir"])
    d = d / d.norm(dim=1, keepdim=True).clamp_min(1e-12)
    return torch.cat([d, o["has_contact"].float()[:, None]], 1).contiguous()


class Trainer:
    """Adam on the library's gradient kernels."""

    def __init__(self, params, lr=2e-3, betas=(0.9, 0.999), eps=1e-8, logit_weight=0.5):
        self.params = params.contiguous()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.lr, self.betas, self.eps, self.logit_weight = lr, betas, eps, logit_weight
        self.step_no = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=self.params.device)
        self._partial = None
        self.grad = torch.empty(N_PARAMS + 4, dtype=torch.float32, device=self.params.device)

    def gradient(self, X, Y):
        """Mean-loss gradient of one batch; returns (grad [N_PARAMS], loss, dir loss, logit loss) on device."""
        n = X.shape[0]
        tiles = (n + 127) // 128
        if self._partial is None or self._partial.numel() < tiles * (N_PARAMS + 4):
            self._partial = torch.empty(tiles * (N_PARAMS + 4), dtype=torch.float32, device=X.device)
        L = N.load()
        N.check(L.ncg_mlp_grad(_p(self.params), _p(X.contiguous()), _p(Y.contiguous()), n,
                               ctypes.c_float(self.logit_weight), _p(self._partial), _p(self.grad), _p(self.err),
                               _stream()), "ncg_mlp_grad")
        return self.grad[:N_PARAMS], self.grad[N_PARAMS:N_PARAMS + 3]

    def step(self, X, Y):
        g, losses = self.gradient(X, Y)
        self.step_no += 1
        L = N.load()
        N.check(L.ncg_mlp_adam(_p(self.params), _p(self.m), _p(self.v), _p(self.grad), ctypes.c_float(self.lr),
                               ctypes.c_float(self.betas[0]), ctypes.c_float(self.betas[1]),
                               ctypes.c_float(self.eps), self.step_no, _stream()), "ncg_mlp_adam")
        return losses

    def check(self):
        if int(self.err.item()) != 0:
            raise N.NcgError("ncg_mlp_grad: a tensor-core wait timed out")


def train(X, Y, epochs=20, batch_size=8192, lr=2e-3, seed=0, params=None, log=None):
    """Trains on features X [N,48] and labels Y [N,4] (device tensors)."""
    tr = Trainer(init_params(seed, X.device) if params is None else params.clone(), lr=lr)
    gen = torch.Generator(device=X.device)
    gen.manual_seed(seed)
    n = X.shape[0]
    steps_per_epoch = max(1, n // batch_size)
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen, device=X.device)
        acc = torch.zeros(3, device=X.device)
        for s in range(steps_per_epoch):
            idx = perm[s * batch_size:(s + 1) * batch_size]
            acc += tr.step(X[idx], Y[idx])
        hist.append((acc / steps_per_epoch).tolist())
        if log:
            log(ep, hist[-1])
    tr.check()
    return tr.params, hist


def evaluate(X, Y, params, batch_size=65536):
    """Mean loss terms and the direction cosine / sign accuracy on held-out data."""
    tr = Trainer(params)
    tot = torch.zeros(3, device=X.device)
    nb = 0
    for s in range(0, X.shape[0], batch_size):
        _, losses = tr.gradient(X[s:s + batch_size], Y[s:s + batch_size])
        tot += losses
        nb += 1
    tr.check()
    return (tot / nb).tolist()
