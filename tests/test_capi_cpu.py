"""CPU-side checks of the C ABI: the library builds, loads and exports every
symbol include/ncg.h declares; host-side argument validation needs no GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from ncollide_gb300 import _native as N
from ncollide_gb300 import shapes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "ncg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ncg_[a-z_0-9]+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for f in ("ncg_contact_batch", "ncg_distance_batch", "ncg_proximity_batch", "ncg_closest_points_batch",
              "ncg_ctx_create", "ncg_contact_batch_host"):
        assert f in names


def test_library_exports_every_declared_symbol():
    L = N.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert set(declared_functions()) <= set(N.EXPORTED) | {"ncg_last_error"}
    assert L.ncg_abi_version() == 3


def test_struct_layouts_match_header():
    assert S.SHAPE_DTYPE.itemsize == 32
    assert S.CONTACT_DTYPE.itemsize == 40
    assert ctypes.sizeof(N.NcgBatch) == 80
    assert ctypes.sizeof(N.NcgStats) == 56
    from oracle import oracle as O
    assert O.MANIFOLD_DTYPE.itemsize == 16 + 36 * N.MANIFOLD_MAX  # ncg_manifold


def test_invalid_arguments_rejected_without_gpu():
    L = N.load()
    # NULL context / batch: NCG_EINVAL before any CUDA call.
    assert L.ncg_contact_batch(None, None, 0.0, None, None, None, None, None, None) == N.NCG_EINVAL
    assert L.ncg_proximity_batch(None, None, ctypes.c_float(-1.0), None, None, None, None, None) == N.NCG_EINVAL
    assert L.ncg_ctx_set_tolerance(None, 0) == N.NCG_EINVAL
    f = ctypes.c_float
    # the reference's asserts become NCG_EINVAL: negative or NaN max_toi / target / margin / prediction
    assert L.ncg_time_of_impact_batch(None, None, None, None, f(-1.0), f(0.0), None, None, None, None,
                                      None) == N.NCG_EINVAL
    assert L.ncg_time_of_impact_batch(None, None, None, None, f(1.0), f(float("nan")), None, None, None, None,
                                      None) == N.NCG_EINVAL
    assert L.ncg_ray_cast_batch(None, None, None, f(-1.0), 1, None, None, None, None, None, None) == N.NCG_EINVAL
    assert L.ncg_manifold_batch(None, None, f(-0.1), f(0.0), f(0.0), None, None, None, None, None,
                                None) == N.NCG_EINVAL
    assert L.ncg_bp_create(None, f(0.1), None) == N.NCG_EINVAL
    assert L.ncg_bp_update(None, None, 0, None) == N.NCG_EINVAL
    assert L.ncg_aabb_batch(None, None, None, None, None) == N.NCG_EINVAL
    assert L.ncg_gather_pairs(None, None, None, None, 1, None, None, None, None, None) == N.NCG_EINVAL


def test_ctx_create_reports_missing_gpu():
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    L = N.load()
    p = ctypes.c_void_p()
    rc = L.ncg_ctx_create(ctypes.byref(p), 0)
    assert rc == N.NCG_ECUDA
    assert L.ncg_last_error()


def test_binding_abi_version_matches_header():
    src = open(os.path.join(ROOT, "include", "ncg.h")).read()
    m = re.search(r"#define NCG_ABI_VERSION (\d+)", src)
    assert m and int(m.group(1)) == N.ABI_VERSION == N.load().ncg_abi_version()
