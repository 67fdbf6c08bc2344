"""The library's autotuner (ncg_autotune) on a GB300: it returns valid
values, leaves them set in the context, and the tuned context's results are
the untuned context's bit for bit (the autotuner itself checks every
candidate's outputs against the first's)."""
import numpy as np
import pytest
import torch

from ncollide_gb300 import query as Q
from ncollide_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("query,param", [("contact", 0.0), ("distance", 0.0), ("proximity", 0.1)])
def test_autotune_sets_fastest_and_keeps_results(ctx_factory, query, param):
    db = Q.DeviceBatch.from_host(W.mixed_convex(32768, seed=29))
    plain = ctx_factory(tolerance=1, dispatch="query")
    ref = {"contact": lambda c: Q.contact_batch(c, db, param),
           "distance": lambda c: Q.distance_batch(c, db),
           "proximity": lambda c: Q.proximity_batch(c, db, margin=param)}[query]
    want = ref(plain)
    tuned = ctx_factory(tolerance=1, dispatch="query")
    r = tuned.autotune(db, query, param, reps=1)
    assert r["ms"] > 0.0
    assert tuned.tuning() == r["values"]
    got = ref(tuned)
    torch.cuda.synchronize()
    for k, v in want.items():
        if v is not None:
            assert torch.equal(got[k], v), k
    # the chosen values are accepted again as they are
    other = ctx_factory(tolerance=1, dispatch="query")
    other.apply_tuning(r["values"])
    assert other.tuning() == r["values"]


def test_autotune_rejects_bad_arguments(ctx_factory):
    db = Q.DeviceBatch.from_host(W.mixed_convex(256, seed=30))
    ctx = ctx_factory()
    with pytest.raises(Exception):
        ctx.autotune(db, "proximity", -1.0)
    with pytest.raises(Exception):
        ctx.autotune(db, "contact", 0.0, reps=0)
