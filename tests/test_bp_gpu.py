"""GPU parity of the bounding volumes and the broad phase: ncg_aabb_batch
against the oracle's AABBs (bit-exact), and ncg_bp_update's pairs and
started / stopped events against the oracle's DBVTBroadPhase restatement
(identical sorted pair lists) over frames of motion, removals and additions."""
import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import shapes as S
from ncollide_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def gpu_aabbs(ctx, batch):
    db = Q.DeviceBatch.from_host(batch)
    out, st = Q.aabb_batch(ctx, db)
    torch.cuda.synchronize()
    return out.cpu().numpy(), st.cpu().numpy().view(np.uint32)


def same(a, b):
    return a.shape == b.shape and bool(((a == b) | (np.isnan(a) & np.isnan(b))).all())


def to_keys(p):
    p = np.asarray(p, np.int64).reshape(-1, 2)
    return (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)


def test_aabb_parity(ctx_factory):
    ctx = ctx_factory()
    b = W.scene_objects(20000, seed=31)
    bad = S.PairBatch(b.shapes, b.hull_points, b.m1, b.g1.copy(), b.m2, b.g2, scale=b.scale)
    bad.g1[11] = len(b.shapes) + 2
    got, st = gpu_aabbs(ctx, bad)
    want, wst = O.aabbs(bad)
    assert same(got, want)
    assert np.array_equal(st, wst) and st[11] == N.STATUS_BAD_INPUT
    # every box holds its shape's support points in the box's directions
    assert (got[:, :3] <= got[:, 3:]).all(where=~np.isnan(got[:, :3]))


@pytest.mark.parametrize("n", [0, 1, 2, 1000, 60000])
def test_bp_pairs_match_oracle(ctx_factory, n):
    ctx = ctx_factory()
    b = W.scene_objects(max(n, 1), seed=32 + n)
    boxes, _ = O.aabbs(b)
    boxes = boxes[:n]
    bp = Q.BroadPhase(ctx, 0.05)
    pairs, started, stopped = bp.update(torch.from_numpy(boxes))
    ob = O.BroadPhase(0.05)
    wp, ws, wt = ob.update(boxes)
    assert np.array_equal(to_keys(pairs.cpu().numpy()), wp)
    assert np.array_equal(to_keys(started.cpu().numpy()), ws)
    assert stopped.shape[0] == 0 and wt.size == 0
    bp.close()


def test_bp_degenerate_boxes(ctx_factory):
    """Identical boxes (equal Morton codes), a box overlapping everything,
    touching faces (closed intervals) and NaN boxes."""
    ctx = ctx_factory()
    rng = np.random.default_rng(5)
    same_box = np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (700, 1))
    small = rng.uniform(-20, 20, (3000, 3)).astype(np.float32)
    small = np.concatenate([small, small + 0.5], 1)
    giant = np.array([[-30, -30, -30, 30, 30, 30]], np.float32)
    touch = np.array([[5, 5, 5, 6, 6, 6], [6, 5, 5, 7, 6, 6]], np.float32)  # share the face x = 6
    nan = np.array([[np.nan, 0, 0, 1, 1, 1]], np.float32)
    boxes = np.concatenate([same_box, small, giant, touch, nan, same_box[:5] + 100])
    bp = Q.BroadPhase(ctx, 0.0)
    pairs, started, _ = bp.update(torch.from_numpy(boxes))
    wp, ws, _ = O.BroadPhase(0.0).update(boxes)
    assert np.array_equal(to_keys(pairs.cpu().numpy()), wp)
    assert np.array_equal(to_keys(started.cpu().numpy()), ws)
    i0 = len(same_box) + len(small) + 1
    assert ((np.uint64(i0) << np.uint64(32)) | np.uint64(i0 + 1)) in set(wp.tolist())
    bp.close()


def test_bp_frames_events(ctx_factory):
    """Frames of coherent motion with the stored-box rule, removals (NaN boxes)
    and added proxies: pairs, started and stopped equal the oracle's."""
    ctx = ctx_factory()
    b = W.scene_objects(30000, seed=33)
    rng = np.random.default_rng(7)
    bp = Q.BroadPhase(ctx, 0.1)
    ob = O.BroadPhase(0.1)
    n = 25000
    for frame in range(6):
        boxes, _ = gpu_aabbs(ctx, b)
        boxes = boxes[:n].copy()
        if frame == 3:
            boxes[rng.choice(n, 50, replace=False), 0] = np.nan  # removed proxies
        pairs, started, stopped = bp.update(torch.from_numpy(boxes))
        wp, ws, wt = ob.update(boxes)
        assert np.array_equal(to_keys(pairs.cpu().numpy()), wp), frame
        assert np.array_equal(to_keys(started.cpu().numpy()), ws), frame
        assert np.array_equal(to_keys(stopped.cpu().numpy()), wt), frame
        if frame > 0:
            assert ws.size + wt.size > 0
        b = W.advance_frame(b, rng, sigma_t=0.05, sigma_r=0.05)
        n = min(n + 1000, 30000)
    with pytest.raises(N.NcgError):
        bp.update(torch.from_numpy(boxes[:100]))  # the proxy count cannot shrink
    bp.close()
    with pytest.raises(N.NcgError):
        Q.BroadPhase(ctx, -1.0)


def test_scene_pipeline_contacts(ctx_factory):
    """AABBs -> broad phase -> gathered pairs -> query::contact, bit-exact
    against the oracle on the same pairs."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    ctx.set_dispatch(N.DISPATCH_QUERY)
    b = W.scene_objects(20000, seed=34, overlaps=8.0)
    objects = Q.DeviceBatch.from_host(b)
    boxes, _ = Q.aabb_batch(ctx, objects)
    bp = Q.BroadPhase(ctx, 0.0)
    pairs, _, _ = bp.update(boxes)
    db = Q.gather_pairs(ctx, objects, bp.pairs_u32)
    got = Q.contact_batch(ctx, db, 0.0, with_iters=True)
    torch.cuda.synchronize()
    p = pairs.cpu().numpy()
    assert p.shape[0] > 1000
    pb = S.PairBatch(b.shapes, b.hull_points, b.m1[p[:, 0]], p[:, 0].astype(np.uint32), b.m1[p[:, 1]],
                     p[:, 1].astype(np.uint32))
    assert np.array_equal(db.m1.cpu().numpy(), pb.m1) and np.array_equal(db.g2.cpu().numpy().view(np.uint32), pb.g2)
    r = O.query(pb, O.CONTACT_QUERY, O.MIXED, eps=-1.0, epa_tol=1e-6)
    assert np.array_equal(got["has_contact"].cpu().numpy(), r.tag)
    assert np.array_equal(got["status"].cpu().numpy().view(np.uint32), r.status)
    m = r.tag == 1
    c = got["contact"].cpu().numpy()
    want = np.concatenate([r.p1, r.p2, r.dir, r.value[:, None]], 1).astype(np.float32)
    assert np.array_equal(c[m], want[m])
    bp.close()
