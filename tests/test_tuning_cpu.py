"""Saved launch tuning (ncollide_gb300.tuning) and the autotuner's host-side
argument checks: no GPU needed."""
import ctypes
import json

from ncollide_gb300 import _native as N
from ncollide_gb300 import tuning as TU


def test_save_lookup_round_trip(tmp_path):
    p = str(tmp_path / "t.json")
    assert TU.lookup("NVIDIA GB300", 152, "w", path=p) is None
    TU.save("NVIDIA GB300", 152, "w", {"hull_gjk_warp": 9, "epa_blocks": 0}, ms=44.5, path=p)
    TU.save("NVIDIA GB300", 152, "other", {"hull_gjk_warp": 0}, path=p)
    assert TU.lookup("NVIDIA GB300", 152, "w", path=p) == {"hull_gjk_warp": 9, "epa_blocks": 0}
    assert TU.lookup("NVIDIA GB300", 148, "w", path=p) is None  # another SM count is another device
    data = json.load(open(p))
    assert len(data) == 2 and data["NVIDIA GB300|152|w"]["ms"] == 44.5


def test_committed_tuning_names_known_keys():
    from ncollide_gb300 import query as Q
    for entry in TU.load().values():
        assert set(entry["values"]) <= set(Q.TUNING_KEYS)


def test_autotune_rejects_bad_arguments_without_gpu():
    L = N.load()
    vals = (ctypes.c_int32 * N.N_TUNE)()
    ms = ctypes.c_float()
    assert L.ncg_autotune(None, None, 0, 0.0, 3, vals, ctypes.byref(ms), None) == N.NCG_EINVAL
    v = ctypes.c_int32()
    assert L.ncg_ctx_get_tuning(None, 0, ctypes.byref(v)) == N.NCG_EINVAL
