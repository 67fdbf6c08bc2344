"""GPU parity of the time of impact: ncg_time_of_impact_batch through the C
ABI against the oracle's MIXED instantiation (f32 support points and ray
origin, f64-class ray parameter, bounds and simplex sub-solve), which follows
the kernel's arithmetic and evaluation order.  Expected: bit-exact TOI,
witnesses, normals, TOIStatus, Some/None, status bits and iteration counts.
"""
import json
import os

import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import shapes as S
from ncollide_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def _toi_batch(pairs):
    """A batch from (translation1, (kind, params), translation2, (kind, params))
    tuples under identity rotations."""
    shp = np.zeros(2 * len(pairs), S.SHAPE_DTYPE)
    m1 = np.zeros((len(pairs), 8), np.float32)
    m2 = np.zeros((len(pairs), 8), np.float32)
    for i, (t1, s1, t2, s2) in enumerate(pairs):
        for j, (t, sh, m) in enumerate(((t1, s1, m1), (t2, s2, m2))):
            shp[2 * i + j]["kind"] = sh[0]
            shp[2 * i + j]["p"] = list(sh[1]) + [0.0] * (4 - len(sh[1]))
            m[i, 3] = 1.0
            m[i, 4:7] = t
    g1 = np.arange(0, 2 * len(pairs), 2, dtype=np.uint32)
    return S.PairBatch(shp, np.zeros((1, 4), np.float32), m1, g1, m2, g1 + 1)


def gpu_toi(ctx, batch, v1, v2, max_toi=float("inf"), target=0.0):
    db = Q.DeviceBatch.from_host(batch)
    o = Q.time_of_impact_batch(ctx, db, torch.from_numpy(np.ascontiguousarray(v1, np.float32)).cuda(),
                               torch.from_numpy(np.ascontiguousarray(v2, np.float32)).cuda(), max_toi, target,
                               with_iters=True)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in o.items() if k != "_keep" and v is not None}


def check_parity(got, want):
    some = want["some"].astype(bool)
    assert np.array_equal(got["has_toi"].astype(bool), some)
    assert np.array_equal(got["status"].view(np.uint32), want["gjk_status"])
    assert np.array_equal(got["iters"].view(np.uint32), want["iters"])
    for k in ("witness1", "witness2", "normal1", "normal2"):
        w = want[k][some].astype(np.float32)
        g = got[k][some]
        bad = ~((g == w) | (np.isnan(g) & np.isnan(w))).all(1)
        assert not bad.any(), (k, np.nonzero(some)[0][bad][:5], g[bad][:3], w[bad][:3])
    assert np.array_equal(got["toi"][some], want["toi"][some].astype(np.float32))
    assert np.array_equal(got["toi_status"][some], want["status"][some])
    assert not got["has_toi"][~some].any()


@pytest.mark.parametrize("dispatch", [N.DISPATCH_SUPPORT_MAP, N.DISPATCH_QUERY])
@pytest.mark.parametrize("tol", [N.TOL_REFERENCE, N.TOL_PRECISE])
@pytest.mark.parametrize("target,max_toi", [(0.0, float("inf")), (0.05, float("inf")), (0.0, 0.75), (0.2, 1.5)])
def test_toi_parity_mixed(ctx_factory, dispatch, tol, target, max_toi):
    ctx = ctx_factory(tolerance=tol)
    ctx.set_dispatch(dispatch)
    b, v1, v2 = W.toi_sweeps(6000, seed=11)
    got = gpu_toi(ctx, b, v1, v2, max_toi, target)
    want = O.toi(b, v1, v2, O.MIXED, dispatch=dispatch, max_toi=max_toi, target_distance=float(np.float32(target)),
                 eps=0.0 if tol == N.TOL_REFERENCE else -1.0)
    assert 0.3 < want["some"].mean() < 0.95
    check_parity(got, want)


def test_toi_parity_balls_and_hulls(ctx_factory):
    ctx = ctx_factory()
    ctx.set_dispatch(N.DISPATCH_QUERY)
    b, v1, v2 = W.toi_sweeps(4000, seed=12, kinds=(W.BALL, W.CONVEX_HULL), hull_n=(4, 300))
    for target in (0.0, 0.1):
        check_parity(gpu_toi(ctx, b, v1, v2, target=target),
                     O.toi(b, v1, v2, O.MIXED, dispatch=1, target_distance=float(np.float32(target))))


def test_toi_known_answers(ctx_factory):
    ctx = ctx_factory()
    ctx.set_dispatch(N.DISPATCH_QUERY)
    k = GOLD["time_of_impact3_ball_cuboid"]
    ball, cub = (0, (k["ball"]["radius"],)), (1, tuple(k["cuboid"]["half_extents"]))
    b = _toi_batch([(cs["ball_translation"], ball, k["cuboid"]["translation"], cub) for cs in k["cases"]])
    v1 = np.array([cs["ball_vel"] for cs in k["cases"]], np.float32)
    v2 = np.array([cs["box_vel"] for cs in k["cases"]], np.float32)
    g = gpu_toi(ctx, b, v1, v2)
    assert list(g["has_toi"]) == [1, 1, 0]
    assert g["toi"][0] == 0.0 and g["toi_status"][0] == N.TOI_PENETRATING
    want = (np.sqrt(3.0) - 1.0) / np.linalg.norm(v1[1].astype(np.float64) - v2[1])
    assert abs(float(g["toi"][1]) - want) <= 1e-6 * want  # f32 output of the f64 known answer
    check_parity(g, O.toi(b, v1, v2, O.MIXED, dispatch=1))
    k = GOLD["ball_ball_toi"]
    ball = (0, (k["radius"],))
    b = _toi_batch([(k["m1_translation"], ball, k["m2_translation"], ball)])
    g = gpu_toi(ctx, b, np.array([k["vel1"]], np.float32), np.array([k["vel2"]], np.float32))
    assert g["has_toi"][0] == 1 and abs(float(g["toi"][0]) - k["toi"]) <= 1e-6
    k = GOLD["still_objects_toi"]
    c = (1, tuple(k["half_extents"]))
    b = _toi_batch([(k["m1_translation"], c, k["m2_translation"], c)] * len(k["cases"]))
    v1 = np.array([[0.0, cs["vel1_y"], 0.0] for cs in k["cases"]], np.float32)
    g = gpu_toi(ctx, b, v1, np.zeros_like(v1))
    assert [bool(x) for x in g["has_toi"]] == [cs["some"] for cs in k["cases"]]


def test_toi_edge_cases(ctx_factory):
    ctx = ctx_factory()
    b, v1, v2 = W.toi_sweeps(512, seed=13)
    # no relative motion: None for every pair (the ray has zero length)
    g = gpu_toi(ctx, b, v1, v1)
    assert not g["has_toi"].any() and not g["status"].any()
    # a bad shape index is reported, not trapped
    bad = S.PairBatch(b.shapes, b.hull_points, b.m1, b.g1.copy(), b.m2, b.g2, scale=b.scale)
    bad.g1[7] = len(b.shapes) + 3
    g = gpu_toi(ctx, bad, v1, v2)
    assert g["status"][7] == N.STATUS_BAD_INPUT and g["has_toi"][7] == 0
    check_parity(g, O.toi(bad, v1, v2, O.MIXED))
    # empty batch, and the argument checks of the reference's asserts
    empty = S.PairBatch(b.shapes, b.hull_points, b.m1[:0], b.g1[:0], b.m2[:0], b.g2[:0], scale=b.scale[:0])
    assert gpu_toi(ctx, empty, v1[:0], v2[:0])["has_toi"].size == 0
    db = Q.DeviceBatch.from_host(b)
    tv = torch.from_numpy(v1).cuda()
    for mt, td in ((-1.0, 0.0), (1.0, -0.5), (float("nan"), 0.0), (1.0, float("nan"))):
        with pytest.raises(N.NcgError):
            Q.time_of_impact_batch(ctx, db, tv, tv, mt, td)
