"""GPU parity of the f32 arithmetic (NCG_ARITH_F32) against the oracle's f32
instantiation, the reference's f32 path restated (f32 sub-solve and
constants, Rust BinaryHeap's order among equal EPA distances): every output
float, tag, status bit and GJK/EPA iteration count must be equal, bit for
bit.  This makes the contact classification equal the reference f32 path's
on every pair, the first half of the accuracy contract, in this arithmetic."""
import numpy as np
import pytest

from ncollide_gb300 import _native as N
from ncollide_gb300 import shapes as S
from ncollide_gb300 import workloads as W
from oracle import oracle as O
from test_parity_gpu import _kat_batch, check_query

pytestmark = pytest.mark.gpu

TOLS = [N.TOL_REFERENCE, N.TOL_PRECISE]


def f32_ctx(ctx_factory, tol, dispatch="support_map", **kw):
    return ctx_factory(tolerance=tol, dispatch=dispatch, arithmetic=N.ARITH_F32, **kw)


@pytest.mark.parametrize("tol", TOLS)
def test_f32_cuboid_pairs_bit_exact(ctx_factory, tol):
    ctx = f32_ctx(ctx_factory, tol, "query")
    check_query(ctx, W.cuboid_pairs(8192, seed=0), O.CONTACT_QUERY, 0.0, tol, O.F32)


@pytest.mark.parametrize("tol", TOLS)
@pytest.mark.parametrize("query,param", [(O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 0.1),
                                         (O.CLOSEST, 0.5), (O.CONTACT_QUERY, 0.0)])
def test_f32_mixed_convex_bit_exact(ctx_factory, tol, query, param):
    ctx = f32_ctx(ctx_factory, tol, "query" if query == O.CONTACT_QUERY else "support_map")
    check_query(ctx, W.mixed_convex(8192, seed=11), query, param, tol, O.F32)


@pytest.mark.parametrize("tol", TOLS)
def test_f32_precision_stress_bit_exact(ctx_factory, tol):
    """Thin shapes near touching: where the f32 path misclassifies ~15% of the
    pairs against f64, the f32 arithmetic reproduces it pair for pair."""
    import bench
    b, _ = bench.near_touching(W.mixed_convex(8192, seed=2, thin=True))
    ctx = f32_ctx(ctx_factory, tol)
    for q, p in ((O.CONTACT, 0.0), (O.DISTANCE, 0.0), (O.PROXIMITY, 1e-6)):
        check_query(ctx, b, q, p, tol, O.F32)


def test_f32_long_polytopes_bit_exact(ctx_factory):
    """Deep curved pairs: EPA runs past the thread store and the 1280-vertex
    store; the heap keeps the deleted faces' entries as Rust's does."""
    ctx = f32_ctx(ctx_factory, N.TOL_REFERENCE, "query")
    b = W.mixed_convex(2048, seed=71, kinds=(S.BALL, S.CAPSULE, S.CONE), dmax=0.05)
    g, _ = check_query(ctx, b, O.CONTACT_QUERY, 0.0, N.TOL_REFERENCE, O.F32)
    assert int(np.max(g["iters"].view(np.uint32) >> 16)) > 200


def test_f32_edge_cases_bit_exact(ctx_factory):
    ctx = f32_ctx(ctx_factory, N.TOL_REFERENCE)
    b = _kat_batch()
    g, _ = check_query(ctx, b, O.CONTACT, 10.0, N.TOL_REFERENCE, O.F32)
    assert g["has_contact"][0] == 1 and g["contact"][0, 9] == 0.5  # epa3.rs:14-15
    check_query(ctx, W.mixed_convex(4096, seed=14, kinds=(S.CYLINDER, S.CUBOID, S.CONVEX_HULL, S.BALL)),
                O.CONTACT, 0.0, N.TOL_REFERENCE, O.F32)
    check_query(ctx, W.mixed_convex(4096, seed=13, thin=True), O.CONTACT, 0.0, N.TOL_REFERENCE, O.F32)


def test_f32_init_dir_and_hull_warp_bit_exact(ctx_factory):
    ctx = f32_ctx(ctx_factory, N.TOL_REFERENCE, warm_start=N.WARM_INIT_DIR)
    b = W.mixed_convex(4096, seed=15)
    rng = np.random.default_rng(0)
    b = b.with_init_dir(W.random_unit_vectors(rng, b.n_pairs).astype(np.float32))
    for q, p in ((O.CONTACT, 0.0), (O.PROXIMITY, 0.1), (O.DISTANCE, 0.0)):
        check_query(ctx, b, q, p, N.TOL_REFERENCE, O.F32)
    ctx.set_tuning(N.TUNE_HULL_GJK_WARP, 1)
    try:
        check_query(ctx, W.mixed_convex(4096, seed=19), O.CONTACT, 0.0, N.TOL_REFERENCE, O.F32)
    finally:
        ctx.set_tuning(N.TUNE_HULL_GJK_WARP, 0)
    prev = ctx.tuning()["hull_epa_warp"]
    for ew in (0, 2):
        ctx.set_tuning(N.TUNE_HULL_EPA_WARP, ew)
        try:
            check_query(ctx, W.mixed_convex(4096, seed=21), O.CONTACT, 0.0, N.TOL_REFERENCE, O.F32)
        finally:
            ctx.set_tuning(N.TUNE_HULL_EPA_WARP, prev)
