"""GPU parity of the support-map ray cast: ncg_ray_cast_batch through the C
ABI against the oracle's MIXED instantiation (f32 ray origin and support
points, f64-class ray parameter, bounds and simplex sub-solve).  Expected:
bit-exact hit flags, toi, normals, status bits and iteration counts."""
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


def gpu_rays(ctx, batch, rays, max_toi=float("inf"), solid=True):
    db = Q.DeviceBatch.from_host(batch)
    o = Q.ray_cast_batch(ctx, db, torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda(), max_toi, solid,
                         with_iters=True)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in o.items() if k != "_keep" and v is not None}


def check_parity(got, want):
    hit = want["hit"].astype(bool)
    assert np.array_equal(got["has_hit"].astype(bool), hit)
    assert np.array_equal(got["status"].view(np.uint32), want["status"])
    assert np.array_equal(got["iters"].view(np.uint32), want["iters"])
    assert np.array_equal(got["toi"][hit], want["toi"][hit].astype(np.float32))
    g, w = got["normal"][hit], want["normal"][hit].astype(np.float32)
    bad = ~((g == w) | (np.isnan(g) & np.isnan(w))).all(1)
    assert not bad.any(), (np.nonzero(hit)[0][bad][:5], g[bad][:3], w[bad][:3])


@pytest.mark.parametrize("tol", [N.TOL_REFERENCE, N.TOL_PRECISE])
@pytest.mark.parametrize("solid,max_toi", [(True, float("inf")), (False, float("inf")), (True, 1.25), (False, 0.5)])
def test_ray_parity_mixed(ctx_factory, tol, solid, max_toi):
    ctx = ctx_factory(tolerance=tol)
    b, rays = W.ray_casts(6000, seed=21)
    got = gpu_rays(ctx, b, rays, max_toi, solid)
    want = O.ray_cast(b, rays, O.MIXED, max_toi=max_toi, solid=solid, eps=0.0 if tol == N.TOL_REFERENCE else -1.0)
    assert 0.05 < want["hit"].mean() < 0.95
    check_parity(got, want)


def test_ray_known_answers(ctx_factory):
    ctx = ctx_factory()
    k = GOLD["solid_ray_cast3d"]
    shp = np.zeros(1, S.SHAPE_DTYPE)
    shp[0]["kind"] = 1
    shp[0]["p"] = k["half_extents"] + [0.0]
    m = np.zeros((1, 8), np.float32)
    m[0, 3] = 1.0
    b = S.PairBatch(shp, np.zeros((1, 4), np.float32), m, np.zeros(1, np.uint32), m, np.zeros(1, np.uint32))
    for cs in k["cases"]:
        rays = np.array([cs["origin"] + cs["dir"]], np.float32)
        g = gpu_rays(ctx, b, rays, solid=cs["solid"])
        if cs["toi"] is None:
            assert g["has_hit"][0] == 0
        else:
            assert g["has_hit"][0] == 1 and abs(float(g["toi"][0]) - cs["toi"]) <= 1e-6 * max(1.0, cs["toi"])
        check_parity(g, O.ray_cast(b, rays, O.MIXED, solid=cs["solid"]))


def test_ray_edge_cases(ctx_factory):
    ctx = ctx_factory()
    b, rays = W.ray_casts(512, seed=22)
    z = rays.copy()
    z[:, 3:] = 0.0  # zero direction: no hit
    g = gpu_rays(ctx, b, z)
    assert not g["has_hit"].any()
    bad = S.PairBatch(b.shapes, b.hull_points, b.m1, b.g1.copy(), b.m2, b.g2, scale=b.scale)
    bad.g1[5] = len(b.shapes) + 1
    g = gpu_rays(ctx, bad, rays)
    assert g["status"][5] == N.STATUS_BAD_INPUT and g["has_hit"][5] == 0
    check_parity(g, O.ray_cast(bad, rays, O.MIXED))
    db = Q.DeviceBatch.from_host(b)
    tr = torch.from_numpy(rays).cuda()
    for mt in (-1.0, float("nan")):
        with pytest.raises(N.NcgError):
            Q.ray_cast_batch(ctx, db, tr, mt)
