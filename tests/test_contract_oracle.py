"""The accuracy contract (tests/contract.py) on the CPU, with the oracle's
mixed-precision instantiation standing in for the kernels (the GPU parity
tests require the kernels to equal it bit for bit; tests/test_contract_gpu.py
runs the same checks on the kernels' own outputs)."""
import numpy as np
import pytest

import contract as C
from ncollide_gb300 import workloads as W
from oracle import oracle as O


def mixed(batch, query):
    return O.query(batch, query, O.MIXED, param=0.0, eps=-1.0, epa_tol=1e-6)


def cases():
    import bench
    stress, _ = bench.near_touching(W.mixed_convex(4096, seed=2, thin=True))
    return [("cuboid_pairs", W.cuboid_pairs(4096, seed=0), O.CONTACT_QUERY, False),
            ("mixed_convex", W.mixed_convex(4096, seed=1), O.CONTACT_QUERY, False),
            ("precision_stress", stress, O.CONTACT, True)]


@pytest.mark.parametrize("name,batch,query,stress", cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_contract_with_oracle_mixed(name, batch, query, stress):
    r = mixed(batch, query)
    d = O.query(batch, O.DISTANCE, O.MIXED, eps=-1.0, epa_tol=1e-6)
    C.check_classification(r.tag, batch, query, stress)
    contact = np.concatenate([r.p1, r.p2, r.dir, r.value[:, None]], 1).astype(np.float32)
    C.check_accuracy(contact, r.tag, d.value.astype(np.float32), batch, query, stress)


def test_f32_reference_path_misses_the_contract_on_thin_shapes():
    """The reference's own f32 path (the oracle's f32 instantiation) is what
    the kernels cannot both equal and meet the contract with: on thin,
    near-touching shapes it misclassifies over 5% of the pairs outside the
    band against f64."""
    import bench
    b, _ = bench.near_touching(W.mixed_convex(2048, seed=2, thin=True))
    gap, r64, _ = C.signed_gap(b, O.CONTACT)
    r32 = O.query(b, O.CONTACT, O.F32, param=0.0)
    out = ~(np.abs(gap) <= C.BAND)
    assert ((r32.tag != r64.tag) & out).sum() > 0.05 * out.sum()
