"""CUDA-graph replay and previous-frame direction reuse, against the oracle.

The reference's convex-polyhedron manifold generator keeps the direction of
the last GJK result and passes it as the next frame's init_dir
(convex_polyhedron_convex_polyhedron_manifold_generator.rs:96-145).  Here the
previous frame's out_dir is the next frame's init_dir; the oracle given the
same init_dir must agree bit for bit.  On coherent motion the reuse cuts the
GJK iterations of queries that need the exact closest features.
"""
import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _host(o):
    return {k: (None if v is None else v.cpu().numpy()) for k, v in o.items()}


def _check_contact(g, r):
    assert np.array_equal(g["status"].view(np.uint32), r.status)
    assert np.array_equal(g["has_contact"], r.tag)
    m = r.tag == 1
    c = g["contact"]
    want = np.concatenate([r.p1, r.p2, r.dir, r.value[:, None]], 1).astype(np.float32)
    assert np.array_equal(c[m], want[m])
    assert np.array_equal(g["dir"], r.dir.astype(np.float32))


def test_graph_replay_matches_direct_call(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_PRECISE, dispatch=N.DISPATCH_QUERY)
    b = W.mixed_convex(8192, seed=31)
    db = Q.DeviceBatch.from_host(b)
    want = _host(Q.contact_batch(ctx, db, 0.0, with_iters=True))
    g = Q.ContactGraph(ctx, db, 0.0, with_iters=True)
    for _ in range(2):
        got = _host(g.launch())
        torch.cuda.synchronize()
        for k in ("contact", "has_contact", "dir", "status", "iters"):
            assert np.array_equal(got[k], want[k]), k
    g.close()


def test_graph_sees_updated_poses(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    b0 = W.coherent_hull_pairs(4096, seed=32, pool=256)
    b1 = W.advance_frame(b0, np.random.default_rng(1))
    db = Q.DeviceBatch.from_host(b0)
    g = Q.ContactGraph(ctx, db, 0.0)
    db.m1.copy_(torch.from_numpy(b1.m1.astype(np.float32)))
    db.m2.copy_(torch.from_numpy(b1.m2.astype(np.float32)))
    got = _host(g.launch())
    torch.cuda.synchronize()
    r = O.query(b1, O.CONTACT, O.MIXED, eps=-1.0, epa_tol=1e-6)
    _check_contact(got, r)
    g.close()


def test_previous_frame_direction_reuse_bit_exact(ctx_factory):
    """Frame 0 plain, frames 1-2 replayed with out_dir == init_dir."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    rng = np.random.default_rng(2)
    frames = [W.coherent_hull_pairs(4096, seed=33, pool=256)]
    for _ in range(2):
        frames.append(W.advance_frame(frames[-1], rng))
    db = Q.DeviceBatch.from_host(frames[0])
    first = Q.contact_batch(ctx, db, 0.0)
    dirs = first["dir"].clone()
    prev = first["dir"].cpu().numpy()
    ctx.set_warm_start(N.WARM_INIT_DIR)
    dbw = db.with_init_dir(dirs)
    g = Q.ContactGraph(ctx, dbw, 0.0, reuse_dir=True)
    for f in frames[1:]:
        db.m1.copy_(torch.from_numpy(f.m1.astype(np.float32)))
        db.m2.copy_(torch.from_numpy(f.m2.astype(np.float32)))
        got = _host(g.launch())
        torch.cuda.synchronize()
        r = O.query(f.with_init_dir(prev), O.CONTACT, O.MIXED, eps=-1.0, epa_tol=1e-6)
        _check_contact(got, r)
        prev = got["dir"]
    g.close()


def test_previous_frame_reuse_cuts_closest_points_iterations(ctx_factory):
    """closest_points with prediction 1 needs the exact closest features, so
    the previous frame's direction saves GJK iterations (about 20% on coherent
    hull pairs); with prediction 0 a contact query stops at the first
    separating axis and reuse changes little (measured, not asserted beyond
    "no worse than 2%")."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    rng = np.random.default_rng(3)
    b0 = W.coherent_hull_pairs(16384, seed=34, pool=1024)
    b1 = W.advance_frame(b0, rng)
    r0 = O.query(b0, O.CLOSEST, O.MIXED, param=1.0, eps=-1.0, epa_tol=1e-6)
    d0 = r0.dir.astype(np.float32)
    plain = Q.closest_points_batch(ctx, Q.DeviceBatch.from_host(b1), 1.0, with_iters=True)
    ctx.set_warm_start(N.WARM_INIT_DIR)
    warm = Q.closest_points_batch(ctx, Q.DeviceBatch.from_host(b1.with_init_dir(d0)), 1.0, with_iters=True)
    torch.cuda.synchronize()
    rw = O.query(b1.with_init_dir(d0), O.CLOSEST, O.MIXED, param=1.0, eps=-1.0, epa_tol=1e-6)
    gw = _host(warm)
    assert np.array_equal(gw["tag"], rw.tag)
    assert np.array_equal(gw["iters"].view(np.uint32) & 0xffff, rw.counters[:, 0])
    ip = (plain["iters"].cpu().numpy().view(np.uint32) & 0xffff).astype(np.float64)
    iw = (gw["iters"].view(np.uint32) & 0xffff).astype(np.float64)
    assert iw.mean() < 0.9 * ip.mean(), (iw.mean(), ip.mean())
    # contact, prediction 0: reuse is about neutral
    d_c = Q.contact_batch(ctx, Q.DeviceBatch.from_host(b0), 0.0)["dir"]
    ctx.set_warm_start(N.WARM_NONE)
    cp = Q.contact_batch(ctx, Q.DeviceBatch.from_host(b1), 0.0, with_iters=True)
    ctx.set_warm_start(N.WARM_INIT_DIR)
    cw = Q.contact_batch(ctx, Q.DeviceBatch.from_host(b1).with_init_dir(d_c), 0.0, with_iters=True)
    ctx.set_warm_start(N.WARM_NONE)
    torch.cuda.synchronize()
    a = (cp["iters"].cpu().numpy().view(np.uint32) & 0xffff).mean()
    w = (cw["iters"].cpu().numpy().view(np.uint32) & 0xffff).mean()
    assert w <= 1.02 * a, (w, a)


def test_proximity_detector_sep_axis_cache_bit_exact(ctx_factory):
    """SupportMapSupportMapProximityDetector (support_map_support_map_proximity_detector.rs:32-60)
    keeps the returned separating axis for the next update, or None after an
    intersection; a batch expresses None as an all-zero init_dir entry."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE, warm_start=N.WARM_INIT_DIR)
    rng = np.random.default_rng(5)
    f = W.mixed_convex(4096, seed=35)
    cache = np.zeros((f.n_pairs, 3), np.float32)  # None for every pair at the first update
    margin = 0.05
    for _ in range(3):
        b = f.with_init_dir(cache)
        got = _host(Q.proximity_batch(ctx, Q.DeviceBatch.from_host(b), margin, with_iters=True))
        torch.cuda.synchronize()
        r = O.query(b, O.PROXIMITY, O.MIXED, param=margin, eps=-1.0, epa_tol=1e-6)
        assert np.array_equal(got["proximity"], r.tag)
        assert np.array_equal(got["dir"], r.dir.astype(np.float32))
        assert np.array_equal(got["iters"].view(np.uint32) & 0xffff, r.counters[:, 0])
        cache = np.where((got["proximity"] == 0)[:, None], 0.0, got["dir"]).astype(np.float32)
        f = W.advance_frame(f, rng)
