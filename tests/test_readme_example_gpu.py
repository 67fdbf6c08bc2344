"""The Python example in README.md runs as written and its contacts equal the
oracle's (the default arithmetic, bit for bit)."""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_readme_python_example_runs():
    import torch
    from oracle import oracle as O
    text = open(os.path.join(ROOT, "README.md")).read()
    code = re.search(r"```python\n(.*?)```", text, re.S).group(1)
    env = {}
    exec(compile(code, "README.md", "exec"), env)
    torch.cuda.synchronize()
    out, host, man = env["out"], env["host"], env["man"]
    b = env["S"].pack_pairs(env["pairs"])
    r = O.query(b, O.CONTACT_QUERY, O.MIXED, param=0.0, eps=-1.0, epa_tol=1e-6)
    has = out["has_contact"].cpu().numpy()
    assert np.array_equal(has, r.tag)
    assert np.array_equal(host["has_contact"], has)
    c = out["contact"].cpu().numpy()
    want = np.concatenate([r.p1, r.p2, r.dir, r.value[:, None]], 1).astype(np.float32)
    m = has == 1
    assert np.array_equal(c[m], want[m])
    assert env["dist"].shape[0] == 2 and man["status"].shape[0] == 2
