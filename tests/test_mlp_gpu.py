"""Learned warm start on the GPU: features, inference and gradients of the
tensor-core kernels against the numpy oracle (oracle/mlp_oracle.py), a short
training run, and bit-exact GJK/EPA results with the network's directions."""
import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import warm_mlp as M
from ncollide_gb300 import workloads as W
from oracle import mlp_oracle as MO
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(MO.N_PARAMS, np.float32)
    p[MO.OFF_W1:MO.OFF_B1] = (rng.standard_normal((128, 48)) * 0.25 * (np.arange(48) < MO.NF)).flatten()
    p[MO.OFF_B1:MO.OFF_W2] = rng.standard_normal(128) * 0.1
    p[MO.OFF_W2:MO.OFF_B2] = rng.standard_normal(128 * 128) * 0.12
    p[MO.OFF_B2:MO.OFF_W3] = rng.standard_normal(128) * 0.1
    p[MO.OFF_W3:MO.OFF_B3] = rng.standard_normal(4 * 128) * 0.12
    p[MO.OFF_B3:] = rng.standard_normal(4) * 0.1
    return p


def test_features_match_oracle():
    b = W.mixed_convex(4096, seed=40)
    db = Q.DeviceBatch.from_host(b)
    desc, X = M.features(db)
    torch.cuda.synchronize()
    dref = MO.shape_descriptors(b)
    assert np.allclose(desc.cpu().numpy(), dref, rtol=1e-3, atol=1e-4)
    xref = MO.pair_features(b, dref)
    assert np.allclose(X.cpu().numpy(), xref, rtol=1e-3, atol=1e-4)


@pytest.mark.parametrize("n", [128, 1000])
def test_gradient_matches_oracle(n):
    b = W.mixed_convex(n, seed=41)
    db = Q.DeviceBatch.from_host(b)
    _, X = M.features(db)
    rng = np.random.default_rng(1)
    d = rng.standard_normal((n, 3))
    Y = np.concatenate([d / np.linalg.norm(d, axis=1, keepdims=True), rng.integers(0, 2, (n, 1))], 1)
    p = _params(2)
    tr = M.Trainer(torch.from_numpy(p).cuda())
    g, losses = tr.gradient(X, torch.from_numpy(Y.astype(np.float32)).cuda())
    torch.cuda.synchronize()
    tr.check()
    g = g.cpu().numpy().astype(np.float64)
    gref, lref, _ = MO.forward_backward(p, X.cpu().numpy(), Y, logit_weight=tr.logit_weight)
    assert np.allclose(losses.cpu().numpy(), lref, rtol=1e-4, atol=1e-6)
    blocks = {"W1": (MO.OFF_W1, MO.OFF_B1), "b1": (MO.OFF_B1, MO.OFF_W2), "W2": (MO.OFF_W2, MO.OFF_B2),
              "b2": (MO.OFF_B2, MO.OFF_W3), "W3": (MO.OFF_W3, MO.OFF_B3), "b3": (MO.OFF_B3, MO.N_PARAMS)}
    for name, (a, z) in blocks.items():
        err = np.linalg.norm(g[a:z] - gref[a:z]) / max(np.linalg.norm(gref[a:z]), 1e-12)
        assert err < 5e-3, (name, err)


def test_inference_matches_oracle():
    b = W.mixed_convex(3000, seed=42)
    db = Q.DeviceBatch.from_host(b)
    p = _params(3)
    d = M.infer(db, torch.from_numpy(p).cuda()).cpu().numpy().astype(np.float64)
    X = MO.pair_features(b)
    _, _, y = MO.forward_backward(p, X.astype(np.float32), np.tile([1.0, 0, 0, 0], (len(X), 1)))
    q = b.m1[:, :4].astype(np.float64)
    qv = q[:, :3]
    u = y[:, :3]
    t = 2.0 * np.cross(qv, u)
    w = u + q[:, 3:4] * t + np.cross(qv, t)
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    cos = (w * d).sum(1)
    assert np.all(np.abs(np.linalg.norm(d, axis=1) - 1) < 1e-5)
    assert np.mean(cos > 0.999) > 0.995, np.sort(cos)[:5]


def test_training_learns_and_warm_start_is_exact(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    train = Q.DeviceBatch.from_host(W.mixed_convex(1 << 16, seed=43))
    held = W.mixed_convex(8192, seed=44)
    dh = Q.DeviceBatch.from_host(held)
    _, X = M.features(train)
    Y = M.labels(ctx, train)
    params, hist = M.train(X, Y, epochs=6, batch_size=4096, lr=3e-3, seed=0)
    assert hist[-1][0] < 0.8 * hist[0][0], hist
    # the network's directions agree with plain GJK's final directions better
    # than the reference's default start normalize(t2 - t1) does
    _, Xh = M.features(dh)
    Yh = M.labels(ctx, dh)
    d = M.infer(dh, params)
    lab = Yh[:, :3]
    q = dh.m1[:, :4]
    qv = q[:, :3]
    t = 2.0 * torch.cross(qv, lab, dim=1)
    lab_w = lab + q[:, 3:4] * t + torch.cross(qv, t, dim=1)
    dflt = dh.m2[:, 4:7] - dh.m1[:, 4:7]
    dflt = dflt / dflt.norm(dim=1, keepdim=True)
    cos_net = (d * lab_w).sum(1).mean().item()
    cos_default = (dflt * lab_w).sum(1).mean().item()
    assert cos_net > cos_default, (cos_net, cos_default)
    # GJK/EPA with the network's start directions equals the oracle given them
    ctx.set_mlp_params(params)
    ctx.set_warm_start(N.WARM_MLP)
    got = Q.contact_batch(ctx, dh, 0.0, with_iters=True)
    ctx.set_warm_start(N.WARM_NONE)
    torch.cuda.synchronize()
    assert ctx.stats()["flags"] == 0
    r = O.query(held.with_init_dir(d.cpu().numpy()), O.CONTACT, O.MIXED, eps=-1.0, epa_tol=1e-6)
    assert np.array_equal(got["has_contact"].cpu().numpy(), r.tag)
    assert np.array_equal(got["status"].cpu().numpy().view(np.uint32), r.status)
    assert np.array_equal(got["iters"].cpu().numpy().view(np.uint32) & 0xffff, r.counters[:, 0])
    m = r.tag == 1
    c = got["contact"].cpu().numpy()
    want = np.concatenate([r.p1, r.p2, r.dir, r.value[:, None]], 1).astype(np.float32)
    assert np.array_equal(c[m], want[m])


def test_what_the_trained_network_gains_on_held_out_pairs(ctx_factory):
    """What the trained network gains over the default start, measured on
    held-out pairs.  Its directions are closer to GJK's final directions than
    the reference's default start, yet GJK's iteration count does not drop:
    contact with prediction 0 stops at the first separating axis (within 3% of
    plain), and closest points, which refine to convergence, only gain from
    the exact final direction (about 11% fewer iterations with it, measured on
    the oracle) while a direction a few degrees off costs iterations.  The test
    records both changes and checks that the results with the network's starts
    are bit for bit the oracle's given those starts."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    train = Q.DeviceBatch.from_host(W.mixed_convex(1 << 17, seed=45))
    held = W.mixed_convex(16384, seed=46)
    dh = Q.DeviceBatch.from_host(held)
    _, X = M.features(train)
    Y = M.labels(ctx, train)
    params, _ = M.train(X, Y, epochs=8, batch_size=4096, lr=3e-3, seed=0)
    d = M.infer(dh, params).cpu().numpy()

    def run(warm, query):
        ctx.set_warm_start(warm)
        if query == "closest":
            o = Q.closest_points_batch(ctx, dh, 0.1, with_iters=True)
        else:
            o = Q.contact_batch(ctx, dh, 0.0, with_iters=True)
        torch.cuda.synchronize()
        ctx.set_warm_start(N.WARM_NONE)
        return {k: (v.cpu().numpy() if v is not None else None) for k, v in o.items()}
    ctx.set_mlp_params(params)
    gjk = lambda o: (o["iters"].view(np.uint32) & 0xffff).astype(np.float64)
    plain_c, mlp_c = run(N.WARM_NONE, "contact"), run(N.WARM_MLP, "contact")
    plain_q, mlp_q = run(N.WARM_NONE, "closest"), run(N.WARM_MLP, "closest")
    contact_change = gjk(mlp_c).mean() / gjk(plain_c).mean() - 1.0
    closest_change = gjk(mlp_q).mean() / gjk(plain_q).mean() - 1.0
    print(f"GJK iterations with the learned start vs plain: contact {100 * contact_change:+.1f}%, "
          f"closest points {100 * closest_change:+.1f}%")
    assert abs(contact_change) < 0.03, contact_change
    assert np.isfinite(closest_change)
    # the closest points with the network's start equal the oracle given it
    r = O.query(held.with_init_dir(d), O.CLOSEST, O.MIXED, param=float(np.float32(0.1)), eps=-1.0, epa_tol=1e-6)
    assert np.array_equal(mlp_q["tag"], r.tag)
    assert np.array_equal(mlp_q["status"].view(np.uint32), r.status)
    assert np.array_equal(gjk(mlp_q).astype(np.uint32), r.counters[:, 0])
    m = r.tag == 1
    pts = np.concatenate([r.p1, r.p2], 1).astype(np.float32)
    assert np.array_equal(mlp_q["points"][m], pts[m])
