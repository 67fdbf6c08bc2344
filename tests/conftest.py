import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx_factory():
    """Creates ncg contexts on cuda:0 (GPU tests only)."""
    from ncollide_gb300.query import Context
    made = []

    def make(**kw):
        c = Context(0, **kw)
        made.append(c)
        return c
    yield make
    for c in made:
        c.close()
