"""The accuracy contract (tests/contract.py) on the kernels' own outputs:
seeded samples of the three contact workloads (65,536 Cuboid pairs, the
1,048,576-pair mixed convex batch, the precision-stress batch of thin shapes
placed near touching), contact and distance through the C ABI in the PRECISE
tolerance set, against the reference's f32 path and the f64 oracle."""
import numpy as np
import pytest
import torch

import contract as C
from ncollide_gb300 import _native as N
from ncollide_gb300 import query as Q
from ncollide_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def cases():
    import bench
    stress, _ = bench.near_touching(W.mixed_convex(8192, seed=2, thin=True))
    return [("cuboid_pairs", W.cuboid_pairs(8192, seed=0), "query", False),
            ("mixed_convex", W.mixed_convex(8192, seed=1), "query", False),
            ("precision_stress", stress, "support_map", True)]


@pytest.mark.parametrize("name,batch,dispatch,stress", cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_contract_on_gpu(ctx_factory, name, batch, dispatch, stress):
    ctx = ctx_factory(tolerance=N.TOL_PRECISE, dispatch=dispatch)
    db = Q.DeviceBatch.from_host(batch)
    oc = Q.contact_batch(ctx, db, 0.0)
    od = Q.distance_batch(ctx, db)
    torch.cuda.synchronize()
    has = oc["has_contact"].cpu().numpy()
    contact = oc["contact"].cpu().numpy()
    dist = od["distance"].cpu().numpy()
    query = O.CONTACT_QUERY if dispatch == "query" else O.CONTACT
    counts = C.check_classification(has, batch, query, stress)
    report = C.check_accuracy(contact, has, dist, batch, query, stress)
    print(name, counts, report)
