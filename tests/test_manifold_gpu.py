"""GPU parity of the contact manifolds: ncg_manifold_batch through the C ABI.
Its contact query equals the oracle's (bit-exact, as every contact query);
its manifolds equal the oracle's restatement of the generator's f32 manifold
step run on the same contacts: normals, point counts, points, depths and
feature ids bit-exact."""
import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run(ctx, b, prediction, a1, a2, topo=None):
    db = Q.DeviceBatch.from_host(b)
    o = Q.manifold_batch(ctx, db, prediction, a1, a2, topology=None if topo is None else topo.to_device())
    torch.cuda.synchronize()
    man = o["manifold"].cpu().numpy().view(O.MANIFOLD_DTYPE).reshape(-1)
    return o, man


def check(ctx, b, prediction, a1, a2, tol, topo=None):
    o, man = run(ctx, b, prediction, a1, a2, topo)
    eps, epa_tol = (0.0, 0.0) if tol == N.TOL_REFERENCE else (-1.0, 1e-6)
    r = O.query(b, O.CONTACT, O.MIXED, param=float(np.float32(prediction)), eps=eps, epa_tol=epa_tol)
    has = o["has_contact"].cpu().numpy()
    assert np.array_equal(has, r.tag)
    c = o["contact"].cpu().numpy()
    c9 = c[:, :9].copy()
    want, wst = O.manifold(b, c9, has, linear=prediction, angular1=a1, angular2=a2, topology=topo)
    st = o["status"].cpu().numpy().view(np.uint32)
    assert np.array_equal(st & (N.STATUS_NOT_POLYHEDRA | N.STATUS_MANIFOLD_FULL), wst)
    assert np.array_equal(man["n"], want["n"])
    assert np.array_equal(man["normal"][has == 1], want["normal"][has == 1])
    for k in range(O.MANIFOLD_MAX):
        m = man["n"] > k
        for f in ("world1", "world2", "depth", "feature1", "feature2"):
            assert np.array_equal(man["points"][f][m, k], want["points"][f][m, k]), (f, k)
    return man, want


@pytest.mark.parametrize("tol", [N.TOL_REFERENCE, N.TOL_PRECISE])
def test_manifold_stacks(ctx_factory, tol):
    ctx = ctx_factory(tolerance=tol)
    man, _ = check(ctx, W.cuboid_stacks(8000, seed=41), 0.1, 0.05, 0.05, tol)
    assert (man["n"] >= 4).mean() > 0.8


@pytest.mark.parametrize("prediction,angle", [(0.0, 0.0), (0.2, 0.1), (0.05, 0.5)])
def test_manifold_random_cuboids(ctx_factory, prediction, angle):
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    check(ctx, W.cuboid_pairs(8000, seed=42), prediction, angle, angle, N.TOL_PRECISE)


def test_manifold_mixed_kinds_and_warm_start(ctx_factory):
    """Non-Cuboid pairs get their single contact with NCG_STATUS_NOT_POLYHEDRA;
    with out_dir aliasing init_dir the next call starts from last_gjk_dir."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    b = W.mixed_convex(4000, seed=43, kinds=(W.BALL, W.CUBOID, W.CAPSULE))
    man, want = check(ctx, b, 0.05, 0.05, 0.05, N.TOL_PRECISE)
    k1 = b.shapes["kind"][b.g1]
    k2 = b.shapes["kind"][b.g2]
    other = (k1 != W.CUBOID) | (k2 != W.CUBOID)
    assert (man["n"][other] <= 1).all()
    db = Q.DeviceBatch.from_host(b)
    o1 = Q.manifold_batch(ctx, db, 0.05, 0.05, 0.05)
    ctx.set_warm_start(N.WARM_INIT_DIR)
    o2 = Q.manifold_batch(ctx, db.with_init_dir(o1["dir"].clone()), 0.05, 0.05, 0.05)
    ctx.set_warm_start(N.WARM_NONE)
    torch.cuda.synchronize()
    r = O.query(b.with_init_dir(o1["dir"].cpu().numpy()), O.CONTACT, O.MIXED, param=float(np.float32(0.05)),
                eps=-1.0, epa_tol=1e-6)
    assert np.array_equal(o2["has_contact"].cpu().numpy(), r.tag)


def test_manifold_bad_arguments(ctx_factory):
    ctx = ctx_factory()
    db = Q.DeviceBatch.from_host(W.cuboid_pairs(16, seed=1))
    for args in ((-1.0, 0.0, 0.0), (0.0, -0.1, 0.0), (0.0, 0.0, float("nan"))):
        with pytest.raises(N.NcgError):
            Q.manifold_batch(ctx, db, *args)


@pytest.mark.parametrize("prediction,angle,dmax", [(0.0, 0.0, 1.0), (0.1, 0.05, 1.0), (0.05, 0.3, 0.6)])
def test_manifold_convex_hull_pairs(ctx_factory, prediction, angle, dmax):
    """ConvexHull and Cuboid pairs with the hulls' face topology
    (ncg_manifold_batch_hulls): support faces and features of the hulls from
    their topology, clipped against each other and against cuboid faces, bit
    for bit the oracle's; pairs whose hull has no topology keep the single
    contact with NCG_STATUS_NOT_POLYHEDRA on both sides."""
    from ncollide_gb300 import hulls as H
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    b = W.hull_pairs_pooled(8192, seed=44, pool=512, dmax=dmax)
    topo = H.HostTopology(b)
    man, want = check(ctx, b, prediction, angle, angle, N.TOL_PRECISE, topo)
    k = b.shapes["kind"]
    hull_pair = (k[b.g1] == W.CONVEX_HULL) | (k[b.g2] == W.CONVEX_HULL)
    assert (man["n"][hull_pair] >= 2).sum() > 100  # polygonal contacts, not only single points
