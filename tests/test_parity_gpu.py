"""GPU parity: libncg.so through the C ABI against the oracle.

The oracle's MIXED instantiation computes the same arithmetic split as the
kernels (f32 support mapping and CSO points, f64 simplex sub-solve, f64 EPA
normals / distances / termination) with the same evaluation order and no
multiply-add contraction, so the expected result is BIT-EXACT: every output
float, tag, status bit and iteration count must be equal.
"""
import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import shapes as S
from ncollide_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DBL_EPS = float(np.finfo(np.float64).eps)


def oracle_mixed(batch, query, param, tol, policy=O.MIXED):
    # eps < 0 selects the oracle's PRECISE tolerance set (the kernels' NCG_TOL_PRECISE)
    eps, epa_tol = (0.0, 0.0) if tol == N.TOL_REFERENCE else (-1.0, 1e-6)
    return O.query(batch, query, policy, param=float(np.float32(param)), eps=eps, epa_tol=epa_tol)


def run_gpu(ctx, batch, query, param):
    db = Q.DeviceBatch.from_host(batch)
    if query in (O.CONTACT, O.CONTACT_QUERY):
        ctx.set_dispatch(N.DISPATCH_QUERY if query == O.CONTACT_QUERY else N.DISPATCH_SUPPORT_MAP)
        o = Q.contact_batch(ctx, db, prediction=param, with_iters=True)
    elif query == O.DISTANCE:
        o = Q.distance_batch(ctx, db, with_iters=True)
    elif query == O.PROXIMITY:
        o = Q.proximity_batch(ctx, db, margin=param, with_iters=True)
    else:
        o = Q.closest_points_batch(ctx, db, prediction=param, with_iters=True)
    torch.cuda.synchronize()
    return {k: (None if v is None else v.cpu().numpy()) for k, v in o.items()}


def f32(x):
    return np.asarray(x, np.float64).astype(np.float32)


def assert_same(name, got, want, batch):
    got, want = np.asarray(got), np.asarray(want)
    bad = got != want
    if got.ndim > 1:
        bad = bad.reshape(len(got), -1).any(1)
    # NaN == NaN counts as equal here (both sides produced the same NaN)
    if np.issubdtype(got.dtype, np.floating):
        nan_both = (np.isnan(got) & np.isnan(want))
        if got.ndim > 1:
            nan_both = nan_both.reshape(len(got), -1).all(1)
        bad &= ~nan_both
    if bad.any():
        idx = np.nonzero(bad)[0][:8]
        k1, k2 = batch.kinds()
        lines = [f"{name}: {bad.sum()} of {len(got)} pairs differ"]
        for i in idx:
            lines.append(f"  pair {i} kinds ({k1[i]},{k2[i]}): gpu={got[i]} oracle={want[i]}")
        raise AssertionError("\n".join(lines))


def check_query(ctx, batch, query, param, tol, policy=O.MIXED):
    """The kernels against the oracle instantiation `policy`: MIXED for the
    default arithmetic, F32 (the reference's f32 path) for NCG_ARITH_F32."""
    g = run_gpu(ctx, batch, query, param)
    r = oracle_mixed(batch, query, param, tol, policy)
    assert_same("status", g["status"].view(np.uint32), r.status, batch)
    it = g["iters"].view(np.uint32)
    assert_same("gjk iterations", it & 0xffff, np.minimum(r.counters[:, 0], 0xffff), batch)
    if query in (O.CONTACT, O.CONTACT_QUERY):
        assert_same("epa iterations", it >> 16, np.minimum(r.counters[:, 1], 0xffff), batch)
        assert_same("has_contact", g["has_contact"], r.tag, batch)
        m = r.tag == 1
        c = g["contact"]
        assert_same("world1", np.where(m[:, None], c[:, 0:3], 0), np.where(m[:, None], f32(r.p1), 0), batch)
        assert_same("world2", np.where(m[:, None], c[:, 3:6], 0), np.where(m[:, None], f32(r.p2), 0), batch)
        assert_same("normal", np.where(m[:, None], c[:, 6:9], 0), np.where(m[:, None], f32(r.dir), 0), batch)
        assert_same("depth", np.where(m, c[:, 9], 0), np.where(m, f32(r.value), 0), batch)
        assert_same("dir", g["dir"], f32(r.dir), batch)
    elif query == O.DISTANCE:
        assert_same("distance", g["distance"], f32(r.value), batch)
    elif query == O.PROXIMITY:
        assert_same("proximity", g["proximity"], r.tag, batch)
        assert_same("sep axis", g["dir"], f32(r.dir), batch)
    else:
        assert_same("closest tag", g["tag"], r.tag, batch)
        m = r.tag == 1
        pts = np.concatenate([f32(r.p1), f32(r.p2)], 1)
        assert_same("points", np.where(m[:, None], g["points"], 0), np.where(m[:, None], pts, 0), batch)
    return g, r


TOLS = [N.TOL_REFERENCE, N.TOL_PRECISE]


@pytest.mark.parametrize("tol", TOLS)
def test_cuboid_pairs_contact_bit_exact(ctx_factory, tol):
    ctx = ctx_factory(tolerance=tol)
    check_query(ctx, W.cuboid_pairs(8192, seed=0), O.CONTACT, 0.0, tol)


@pytest.mark.parametrize("tol", TOLS)
@pytest.mark.parametrize("query,param", [(O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 0.1),
                                         (O.CLOSEST, 0.5), (O.CONTACT, 0.25)])
def test_mixed_convex_bit_exact(ctx_factory, tol, query, param):
    ctx = ctx_factory(tolerance=tol)
    check_query(ctx, W.mixed_convex(8192, seed=11), query, param, tol)


@pytest.mark.parametrize("tol", TOLS)
@pytest.mark.parametrize("param", [0.0, 0.3])
def test_query_dispatch_bit_exact(ctx_factory, tol, param):
    # query::contact routing: Ball-Ball analytic, Ball-Cuboid/ConvexHull by point projection
    ctx = ctx_factory(tolerance=tol)
    check_query(ctx, W.mixed_convex(8192, seed=18), O.CONTACT_QUERY, param, tol)
    b = W.mixed_convex(4096, seed=19, kinds=(S.BALL, S.CUBOID, S.CONVEX_HULL))
    check_query(ctx, b, O.CONTACT_QUERY, param, tol)


def test_query_dispatch_contact_example(ctx_factory):
    pairs = [(S.isometry(t), S.Ball(1.0), S.isometry(), S.Cuboid((1, 1, 1))) for t in ((1, 1, 1), (2, 2, 2), (3, 3, 3))]
    pairs += [(S.isometry(), S.Cuboid((1, 1, 1)), S.isometry(t), S.Ball(1.0)) for t in ((1, 1, 1), (2, 2, 2), (3, 3, 3))]
    ctx = ctx_factory()
    g, _ = check_query(ctx, S.pack_pairs(pairs), O.CONTACT_QUERY, 1.0, N.TOL_REFERENCE)
    has, depth = g["has_contact"], g["contact"][:, 9]
    assert has[0] and depth[0] > 0 and has[1] and depth[1] < 0 and not has[2]   # examples/contact_query3d.rs
    assert has[3] and depth[3] > 0 and has[4] and depth[4] < 0 and not has[5]   # flipped


def test_epa_overflow_pass_is_exercised_and_exact(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_REFERENCE)
    b = W.mixed_convex(16384, seed=12)
    check_query(ctx, b, O.CONTACT, 0.0, N.TOL_REFERENCE)
    st = ctx.stats()
    assert st["n_epa"] > 0
    assert st["n_epa_overflow"] > 0  # the tail of curved pairs outgrows the shared store


def test_thin_shapes_bit_exact(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_REFERENCE)
    check_query(ctx, W.mixed_convex(4096, seed=13, thin=True), O.CONTACT, 0.0, N.TOL_REFERENCE)


@pytest.mark.parametrize("tol", TOLS)
def test_near_touching_thin_pairs_bit_exact(ctx_factory, tol):
    """The precision-stress inputs: thin shapes at signed gaps down to 1e-7."""
    import bench
    b, _ = bench.near_touching(W.mixed_convex(4096, seed=60, thin=True))
    ctx = ctx_factory(tolerance=tol)
    for q, p in ((O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 1e-6), (O.CONTACT_QUERY, 0.0)):
        check_query(ctx, b, q, p, tol)


def test_cylinders_bit_exact(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_REFERENCE)
    b = W.mixed_convex(4096, seed=14, kinds=(S.CYLINDER, S.CUBOID, S.CONVEX_HULL, S.BALL))
    for q, p in ((O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 0.05)):
        check_query(ctx, b, q, p, N.TOL_REFERENCE)


def _kat_batch():
    pairs = [
        (S.isometry((3.5, 0, 0)), S.Cuboid((2, 1, 1)), S.isometry(), S.Cuboid((2, 1, 1))),
        (S.isometry((0, 0.2, 0)), S.Cuboid((2, 1, 1)), S.isometry(), S.Cuboid((2, 1, 1))),
        (S.isometry((10.97, 0.925, 61.02)), S.Cylinder(0.925, 0.5), S.isometry((11.5, 0.75, 60.5)),
         S.Cuboid((0.05, 0.75, 0.5))),
        (S.isometry((0, 3, 0)), S.Ball(1.0), S.isometry(), S.Cuboid((1, 1, 1))),
        (S.isometry((0, 1, 0)), S.Ball(1.0), S.isometry(), S.Cuboid((1, 1, 1))),
        (S.isometry(), S.Cuboid((1, 1, 1)), S.isometry(), S.Cuboid((1, 1, 1))),
        (S.isometry(), S.Cuboid((0.5, 0.5, 0.1)), S.isometry((0, 1, 0)), S.Cuboid((0.5, 0.5, 0.1))),
    ]
    return S.pack_pairs(pairs)


@pytest.mark.parametrize("tol", TOLS)
def test_reference_known_answers_on_gpu(ctx_factory, tol):
    ctx = ctx_factory(tolerance=tol)
    b = _kat_batch()
    g, _ = check_query(ctx, b, O.CONTACT, 10.0, tol)
    # epa3.rs:14-15 — exact in f32 too for the 3.5 offset
    assert g["has_contact"][0] == 1 and g["contact"][0, 9] == 0.5
    assert list(g["contact"][0, 6:9]) == [-1.0, 0.0, 0.0]
    assert g["has_contact"][2] == 1  # cylinder_cuboid_contact.rs:21
    d, _ = check_query(ctx, b, O.DISTANCE, 0.0, tol)
    assert d["distance"][2] == 0.0
    assert abs(d["distance"][3] - 1.0) < 1e-4 and d["distance"][4] == 0.0
    p, _ = check_query(ctx, b, O.PROXIMITY, 0.1, tol)
    assert p["proximity"][2] == N.NCG_OK  # Intersecting == 0


def test_degenerate_hulls_bit_exact(ctx_factory):
    rng = np.random.default_rng(5)
    pairs = []
    for n in (1, 2, 3, 4, 5, 8, 33, 64):
        pts = rng.normal(size=(n, 3)).astype(np.float32) * 0.5
        if n >= 4:
            pts[1] = pts[0]  # duplicate vertex
        for _ in range(8):
            q = W.random_unit_quaternions(rng, 2)
            t = rng.uniform(-0.6, 0.6, 3)
            pairs.append((S.isometry((0, 0, 0), q[0]), S.ConvexHull(pts), S.isometry(t, q[1]),
                          S.Cuboid((0.3, 0.2, 0.4))))
            pairs.append((S.isometry((0, 0, 0), q[0]), S.ConvexHull(pts), S.isometry(t, q[1]), S.ConvexHull(pts)))
    b = S.pack_pairs(pairs)
    ctx = ctx_factory(tolerance=N.TOL_REFERENCE)
    for q, p in ((O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 0.1), (O.CLOSEST, 1.0)):
        check_query(ctx, b, q, p, N.TOL_REFERENCE)


def test_bad_inputs_flagged_not_trapped(ctx_factory):
    b = W.mixed_convex(256, seed=3)
    b.g2 = b.g2.copy()
    b.g2[7] = 10 ** 6                      # shape index out of range
    sh = b.shapes.copy()
    hulls = np.nonzero(sh["kind"] == S.CONVEX_HULL)[0]
    sh["hull_n"][hulls[0]] = 10 ** 8       # hull slice past the end of the points
    b.shapes = sh
    ctx = ctx_factory()
    g = run_gpu(ctx, b, O.CONTACT, 0.0)
    st = g["status"].view(np.uint32)
    assert st[7] & N.STATUS_BAD_INPUT
    owners = np.nonzero((b.g1 == hulls[0]) | (b.g2 == hulls[0]))[0]
    assert np.all(st[owners] & N.STATUS_BAD_INPUT)
    assert g["has_contact"][7] == 0


def test_empty_batch_and_negative_margin(ctx_factory):
    ctx = ctx_factory()
    b = W.mixed_convex(16, seed=4)
    db = Q.DeviceBatch.from_host(b.subset(np.arange(0)))
    out = Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    assert out["contact"].shape[0] == 0
    with pytest.raises(N.NcgError):
        Q.proximity_batch(ctx, Q.DeviceBatch.from_host(b), margin=-1.0)


def test_init_dir_warm_start_bit_exact(ctx_factory):
    ctx = ctx_factory(tolerance=N.TOL_REFERENCE, warm_start=N.WARM_INIT_DIR)
    b = W.mixed_convex(4096, seed=15)
    rng = np.random.default_rng(0)
    b = b.with_init_dir(W.random_unit_vectors(rng, b.n_pairs).astype(np.float32))
    for q, p in ((O.CONTACT, 0.0), (O.PROXIMITY, 0.1), (O.DISTANCE, 0.0)):
        check_query(ctx, b, q, p, N.TOL_REFERENCE)


def test_host_entry_points_match_device(ctx_factory):
    ctx = ctx_factory()
    b = W.mixed_convex(2048, seed=16)
    h = Q.contact_batch_host(ctx, b, 0.0)
    g = run_gpu(ctx, b, O.CONTACT, 0.0)
    assert np.array_equal(h["has_contact"], g["has_contact"])
    c = h["contact"]
    flat = np.concatenate([c["world1"], c["world2"], c["normal"], c["depth"][:, None]], 1)
    assert np.array_equal(flat[h["has_contact"] == 1], g["contact"][g["has_contact"] == 1])
    hd = Q.distance_batch_host(ctx, b)
    gd = run_gpu(ctx, b, O.DISTANCE, 0.0)
    assert np.array_equal(hd["distance"], gd["distance"])
    hp = Q.proximity_batch_host(ctx, b, 0.1)
    gp = run_gpu(ctx, b, O.PROXIMITY, 0.1)
    assert np.array_equal(hp["proximity"], gp["proximity"])


def test_repeated_calls_are_deterministic(ctx_factory):
    ctx = ctx_factory()
    db = Q.DeviceBatch.from_host(W.mixed_convex(8192, seed=17))
    a = Q.contact_batch(ctx, db, 0.0)
    b = Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    assert torch.equal(a["contact"], b["contact"]) and torch.equal(a["has_contact"], b["has_contact"])


@pytest.mark.parametrize("hull_warp", [1, 9])
@pytest.mark.parametrize("query,param", [(O.CONTACT_QUERY, 0.0), (O.DISTANCE, 0.0)])
def test_hull_gjk_warp_modes_bit_exact(ctx_factory, hull_warp, query, param):
    """ConvexHull GJK one warp per pair (all hull pairs, or those scanning >= 2^9
    points) gives the same results as one thread per pair."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    ctx.set_tuning(N.TUNE_HULL_GJK_WARP, hull_warp)
    try:
        check_query(ctx, W.mixed_convex(8192, seed=19), query, param, N.TOL_PRECISE)
    finally:
        ctx.set_tuning(N.TUNE_HULL_GJK_WARP, 0)


@pytest.mark.parametrize("epa_warp", [0, 2, 8, 10])
@pytest.mark.parametrize("tol", TOLS)
def test_hull_epa_warp_start_bit_exact(ctx_factory, epa_warp, tol):
    """EPA of ConvexHull pairs whose GJK ran one thread per pair, started in the
    warp stage for the hulls scanning >= 2^epa_warp points (2: every hull
    pair; 0: none, every EPA starts in the thread stage), gives the oracle's
    contacts bit for bit whichever stage it starts in."""
    ctx = ctx_factory(tolerance=tol)
    prev = ctx.tuning()["hull_epa_warp"]
    ctx.set_tuning(N.TUNE_HULL_EPA_WARP, epa_warp)
    try:
        check_query(ctx, W.mixed_convex(8192, seed=29), O.CONTACT_QUERY, 0.0, tol)
        check_query(ctx, W.mixed_convex(4096, seed=31, thin=True), O.CONTACT_QUERY, 0.0, tol)
        assert ctx.stats()["flags"] == 0
    finally:
        ctx.set_tuning(N.TUNE_HULL_EPA_WARP, prev)


@pytest.mark.parametrize("query,param", [(O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 0.1),
                                         (O.CLOSEST, 0.5)])
def test_hull_locality_sort_bit_exact(ctx_factory, query, param):
    """A batch that reuses its shapes (16,384 pairs over 1,024 shapes) is
    sorted with its ConvexHull pairs grouped by hull index range
    (NCG_TUNE_HULL_LOCALITY): the oracle's results bit for bit, and the same
    outputs with the grouping off."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE, dispatch="support_map")
    prev = ctx.tuning()["hull_locality"]
    b = W.mixed_convex_pooled(16384, seed=61, pool=1024)
    try:
        ctx.set_tuning(N.TUNE_HULL_LOCALITY, 1)
        g1, _ = check_query(ctx, b, query, param, N.TOL_PRECISE)
        ctx.set_tuning(N.TUNE_HULL_LOCALITY, 0)
        g0, _ = check_query(ctx, b, query, param, N.TOL_PRECISE)
        for k in g1:
            if g1[k] is not None:
                assert np.array_equal(g1[k].view(np.uint8), g0[k].view(np.uint8)), k
    finally:
        ctx.set_tuning(N.TUNE_HULL_LOCALITY, prev)


def _with_shared_hulls(batch, every=3):
    """Every `every`-th ConvexHull pair collides the first shape with itself
    (both shapes are the same slice of the point buffer)."""
    k1, _ = batch.kinds()
    g2 = batch.g2.copy()
    idx = np.nonzero(k1 == S.CONVEX_HULL)[0][::every]
    g2[idx] = batch.g1[idx]
    return S.PairBatch(batch.shapes, batch.hull_points, batch.m1, batch.g1, batch.m2, g2, None, None, dict(batch.meta))


@pytest.mark.parametrize("hull_warp,stage_min,stage_cap", [(1, 1, 1024), (1, 1, 64), (9, 256, 2048), (1, 8, 512)])
@pytest.mark.parametrize("query,param", [(O.CONTACT_QUERY, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 0.1)])
def test_hull_stage_bit_exact(ctx_factory, hull_warp, stage_min, stage_cap, query, param):
    """Warp-per-pair hull GJK with the pair's hull points staged in shared
    memory by bulk copies (all hull pairs or those from a point count on; a
    stage too small for some hulls; pairs whose two shapes are one hull) gives
    the oracle's results bit for bit, like the unstaged kernels."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE)
    ctx.set_tuning(N.TUNE_HULL_GJK_WARP, hull_warp)
    ctx.set_tuning(N.TUNE_HULL_STAGE_CAP, stage_cap)
    ctx.set_tuning(N.TUNE_HULL_STAGE_MIN, stage_min)
    try:
        b = _with_shared_hulls(W.mixed_convex(8192, seed=23))
        check_query(ctx, b, query, param, N.TOL_PRECISE)
        assert ctx.stats()["flags"] == 0
    finally:
        ctx.set_tuning(N.TUNE_HULL_STAGE_MIN, 0)
        ctx.set_tuning(N.TUNE_HULL_STAGE_CAP, 1024)
        ctx.set_tuning(N.TUNE_HULL_GJK_WARP, 0)


def test_hull_stage_tuning_rejects_bad_values(ctx_factory):
    ctx = ctx_factory()
    for key, v in ((N.TUNE_HULL_STAGE_CAP, 0), (N.TUNE_HULL_STAGE_CAP, 100), (N.TUNE_HULL_STAGE_CAP, 4096),
                   (N.TUNE_HULL_STAGE_MIN, -1), (N.TUNE_HULL_STAGE_MIN, 4096), (N.TUNE_HULL_EPA_WARP, 1),
                   (N.TUNE_HULL_EPA_WARP, -1), (N.TUNE_HULL_EPA_WARP, 99)):
        with pytest.raises(Exception):
            ctx.set_tuning(key, v)


@pytest.mark.parametrize("tol", TOLS)
def test_resumed_long_polytopes_bit_exact(ctx_factory, tol):
    """Deep, nearly concentric curved pairs (Ball, Capsule, Cone centres within
    5% of the summed radii): EPA refines a ring of equidistant faces for
    hundreds of steps, so most pairs outgrow the thread stage's store and the
    warp stage resumes them from the spilled polytope.  Bit-exact against the
    oracle, which never splits a run."""
    ctx = ctx_factory(tolerance=tol, dispatch="query")
    b = W.mixed_convex(2048, seed=71, kinds=(S.BALL, S.CAPSULE, S.CONE), dmax=0.05)
    g, r = check_query(ctx, b, O.CONTACT_QUERY, 0.0, tol)
    st = ctx.stats()
    assert st["n_epa_overflow"] > 100
    assert int(np.max(g["iters"].view(np.uint32) >> 16)) > 200  # long runs, resumed past the thread store


def test_host_entry_points_overlap_copies_correctly(ctx_factory):
    """The host entry points copy the hull points on a second stream while the
    analytic pairs run.  Two different hull-heavy batches in a row (the second
    one's hull points differ at the same offsets) must give exactly the
    device-resident results, for contact, distance and proximity."""
    ctx = ctx_factory(tolerance=N.TOL_PRECISE, dispatch="query")
    kinds = (S.CUBOID, S.CONVEX_HULL, S.BALL, S.CAPSULE)
    for seed in (81, 82):
        b = W.mixed_convex(4096, seed=seed, kinds=kinds)
        h = Q.contact_batch_host(ctx, b, 0.0)
        g = run_gpu(ctx, b, O.CONTACT_QUERY, 0.0)
        assert np.array_equal(h["has_contact"], g["has_contact"])
        c = h["contact"]
        flat = np.concatenate([c["world1"], c["world2"], c["normal"], c["depth"][:, None]], 1)
        assert np.array_equal(flat[h["has_contact"] == 1], g["contact"][g["has_contact"] == 1])
        assert np.array_equal(h["status"].view(np.uint32), g["status"].view(np.uint32))
        assert np.array_equal(Q.distance_batch_host(ctx, b)["distance"], run_gpu(ctx, b, O.DISTANCE, 0.0)["distance"])
        assert np.array_equal(Q.proximity_batch_host(ctx, b, 0.1)["proximity"],
                              run_gpu(ctx, b, O.PROXIMITY, 0.1)["proximity"])


@pytest.mark.parametrize("hull_warp", [0, 1])
def test_hull_with_nan_first_point_matches_serial_argmax(ctx_factory, hull_warp):
    """point_cloud_support_point starts from point 0's dot product and only
    replaces it by a larger one, so a NaN at point 0 makes it return 0 for
    every direction (no comparison with NaN is true).  The warp-parallel
    arg-max must do the same (its reduction ranks NaN below every number)."""
    rng = np.random.default_rng(91)
    pairs = []
    for k in range(96):
        n = int(rng.integers(40, 600))
        pts = rng.normal(size=(n, 3)).astype(np.float32) * 0.5
        if k % 3 == 0:
            pts[0] = np.nan
        elif k % 3 == 1:
            pts[0] = (np.inf, -np.inf, 0.0)   # NaN dot products for half of the directions
        q = W.random_unit_quaternions(rng, 2)
        t = rng.uniform(-0.8, 0.8, 3)
        other = S.ConvexHull(rng.normal(size=(64, 3)).astype(np.float32) * 0.4) if k % 2 else S.Cuboid((0.3, 0.2, 0.4))
        pairs.append((S.isometry((0, 0, 0), q[0]), S.ConvexHull(pts), S.isometry(t, q[1]), other))
    b = S.pack_pairs(pairs)
    ctx = ctx_factory(tolerance=N.TOL_REFERENCE)
    ctx.set_tuning(N.TUNE_HULL_GJK_WARP, hull_warp)
    try:
        # GJK-only queries: with a NaN or infinite support point the contact
        # query's EPA runs to its 10 000-iteration cap on every such pair
        for q, p in ((O.DISTANCE, 0.0), (O.PROXIMITY, 0.1), (O.CLOSEST, 1.0)):
            check_query(ctx, b, q, p, N.TOL_REFERENCE)
    finally:
        ctx.set_tuning(N.TUNE_HULL_GJK_WARP, 0)
