"""The contact entry point that allocates nothing (ncg_contact_batch_noalloc).

It serves callers that cannot allocate device memory when they need contacts:
code recording a CUDA graph by stream capture without a graph memory pool,
real-time loops whose allocator is frozen after start-up, and host runtimes
that own every device allocation.  Its scratch is a fixed array inside the
library (at most NCG_NOALLOC_MAX_PAIRS pairs per call), shared by every call
on a device.  These tests call it through the C ABI and require its results to
equal those of the regular entry point, bit for bit (the same tolerance as the
other parity tests), on two consecutive calls — the second call runs on the
contents the first left in the shared array.  This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes
import time

import numpy as np
import pytest
import torch

from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import shapes as S
from ncollide_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(L, db, prediction, tol):
    n, dev = db.n_pairs, db.m1.device
    out = {"contact": torch.empty((n, 10), dtype=torch.float32, device=dev),
           "has_contact": torch.empty(n, dtype=torch.uint8, device=dev),
           "dir": torch.empty((n, 3), dtype=torch.float32, device=dev),
           "status": torch.empty(n, dtype=torch.int32, device=dev)}
    cb = db.c_struct()
    stream = torch.cuda.current_stream()
    rc = L.ncg_contact_batch_noalloc(ctypes.byref(cb), ctypes.c_float(prediction), int(tol),
                                     ctypes.c_void_p(out["contact"].data_ptr()),
                                     ctypes.c_void_p(out["has_contact"].data_ptr()),
                                     ctypes.c_void_p(out["dir"].data_ptr()),
                                     ctypes.c_void_p(out["status"].data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    return rc, out


@pytest.mark.parametrize("tol,seed,n", [(N.TOL_REFERENCE, 31, 8192), (N.TOL_PRECISE, 32, N.NOALLOC_MAX_PAIRS)])
def test_noalloc_equals_contact_batch_on_two_calls(tol, seed, n):
    L = N.load()
    b = W.mixed_convex(n, seed=seed)
    db = Q.DeviceBatch.from_host(b)
    ctx = Q.Context(0, tolerance=tol)
    ref = Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    ref = {k: v.cpu().numpy() for k, v in ref.items() if v is not None}
    ctx.close()
    has = ref["has_contact"] == 1
    for call in range(2):
        rc, out = _noalloc(L, db, 0.0, tol)
        assert rc == N.NCG_OK, L.ncg_last_error()
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in out.items()}
        assert np.array_equal(got["has_contact"], ref["has_contact"]), f"call {call}: has_contact differs"
        assert np.array_equal(got["contact"][has], ref["contact"][has]), f"call {call}: contacts differ"
        assert np.array_equal(got["dir"], ref["dir"]), f"call {call}: directions differ"
        assert np.array_equal(got["status"], ref["status"]), f"call {call}: status differs"


@pytest.mark.parametrize("tol", [N.TOL_REFERENCE, N.TOL_PRECISE])
def test_noalloc_deep_curved_pairs_through_every_store(tol):
    """Deep, nearly concentric Ball/Capsule/Cone pairs: EPA outgrows the
    thread store for most pairs, the 128-vertex store for hundreds and the
    1280-vertex store for some (over 4000 vertices for the deepest), so the
    restart from GJK's simplex and the single-warp slab both run.  The results
    must still equal the regular entry point's on two calls in a row."""
    L = N.load()
    b = W.mixed_convex(2048, seed=71, kinds=(S.BALL, S.CAPSULE, S.CONE), dmax=0.05)
    db = Q.DeviceBatch.from_host(b)
    ctx = Q.Context(0, tolerance=tol)
    ref = Q.contact_batch(ctx, db, 0.0, with_iters=True)
    torch.cuda.synchronize()
    ref = {k: v.cpu().numpy() for k, v in ref.items() if v is not None}
    ctx.close()
    epa_iters = ref["iters"].view(np.uint32) >> 16
    assert (epa_iters > 128).sum() > 100 and (epa_iters > 1280).sum() >= 5  # every store is reached
    has = ref["has_contact"] == 1
    for call in range(2):
        t0 = time.perf_counter()
        rc, out = _noalloc(L, db, 0.0, tol)
        assert rc == N.NCG_OK, L.ncg_last_error()
        torch.cuda.synchronize()
        print(f"no-allocation call {call}: {1e3 * (time.perf_counter() - t0):.1f} ms for {b.n_pairs} deep curved pairs "
              f"({int((epa_iters > 1280).sum())} beyond 1280 vertices)")
        got = {k: v.cpu().numpy() for k, v in out.items()}
        assert np.array_equal(got["has_contact"], ref["has_contact"]), f"call {call}: has_contact differs"
        assert np.array_equal(got["contact"][has], ref["contact"][has]), f"call {call}: contacts differ"
        assert np.array_equal(got["dir"], ref["dir"]), f"call {call}: directions differ"
        assert np.array_equal(got["status"], ref["status"]), f"call {call}: status differs"


def test_noalloc_rejects_batches_over_the_limit():
    L = N.load()
    b = W.cuboid_pairs(N.NOALLOC_MAX_PAIRS + 1, seed=33)
    db = Q.DeviceBatch.from_host(b)
    rc, _ = _noalloc(L, db, 0.0, N.TOL_REFERENCE)
    assert rc == N.NCG_EINVAL
    assert b"NCG_NOALLOC_MAX_PAIRS" in L.ncg_last_error()
