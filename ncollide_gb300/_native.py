"""ctypes binding of libncg.so (include/ncg.h).

The shared library is built in-tree (ncollide_gb300/_lib/libncg.so) by
ncollide_gb300.build.  There is no fallback: when the library is missing the
import of the query API raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB_PATH

ABI_VERSION = 3  # NCG_ABI_VERSION of include/ncg.h
NCG_OK, NCG_EINVAL, NCG_ECUDA, NCG_ENOMEM, NCG_ENOTBUILT, NCG_EINTERNAL = 0, -1, -2, -3, -4, -5
TOL_REFERENCE, TOL_PRECISE = 0, 1
ARITH_SPLIT, ARITH_F32 = 0, 1
WARM_NONE, WARM_INIT_DIR, WARM_MLP = 0, 1, 2

STATUS_GJK_MAX_ITER = 1 << 0
STATUS_EPA_FAILED = 1 << 1
STATUS_EPA_MAX_ITER = 1 << 2
STATUS_EPA_CAPACITY = 1 << 3
STATUS_EPA_NO_FACE = 1 << 4
STATUS_DEGENERATE = 1 << 5
STATUS_BAD_INPUT = 1 << 6

# Every symbol include/ncg.h declares.
EXPORTED = [
    "ncg_ctx_create", "ncg_ctx_destroy", "ncg_ctx_set_tolerance", "ncg_ctx_set_warm_start", "ncg_sync",
    "ncg_get_stats", "ncg_last_error", "ncg_abi_version", "ncg_contact_batch", "ncg_distance_batch",
    "ncg_proximity_batch", "ncg_closest_points_batch", "ncg_contact_batch_host", "ncg_distance_batch_host",
    "ncg_proximity_batch_host", "ncg_ctx_set_profiling", "ncg_get_stage_ms", "ncg_contact_batch_noalloc",
    "ncg_ctx_set_dispatch", "ncg_ctx_set_tuning", "ncg_contact_graph_create", "ncg_graph_launch",
    "ncg_graph_destroy", "ncg_mlp_n_params", "ncg_ctx_set_mlp_params", "ncg_mlp_features", "ncg_mlp_infer",
    "ncg_mlp_grad", "ncg_mlp_adam", "ncg_time_of_impact_batch",
    "ncg_ray_cast_batch", "ncg_aabb_batch", "ncg_bp_create", "ncg_bp_update", "ncg_bp_results",
    "ncg_bp_destroy", "ncg_bp_copy", "ncg_gather_pairs", "ncg_manifold_batch", "ncg_autotune",
    "ncg_ctx_get_tuning", "ncg_ctx_set_arithmetic", "ncg_hull_topology_build", "ncg_hull_topology_release",
    "ncg_manifold_batch_hulls",
]
MLP_N_INPUTS, MLP_N_PARAMS = 48, 23300
(TUNE_HULL_GJK_WARP, TUNE_GJK_BLOCKS, TUNE_EPA_BLOCKS, TUNE_L1_CARVEOUT, TUNE_HULL_STAGE_MIN, TUNE_HULL_STAGE_CAP,
 TUNE_HULL_EPA_WARP, TUNE_HULL_LOCALITY) = range(8)
N_TUNE = 8
QUERY_CONTACT, QUERY_DISTANCE, QUERY_PROXIMITY, QUERY_CLOSEST_POINTS = range(4)
DISPATCH_SUPPORT_MAP, DISPATCH_QUERY = 0, 1
TOI_OUT_OF_ITERATIONS, TOI_CONVERGED, TOI_FAILED, TOI_PENETRATING = range(4)
STATUS_UNSUPPORTED_FEATURE = 1 << 7
STATUS_EPA_PRECISION_LIMIT = 1 << 8
STATUS_NOT_POLYHEDRA = 1 << 9
STATUS_MANIFOLD_FULL = 1 << 10
POLY_MAX = 32
MANIFOLD_MAX = 16
NOALLOC_MAX_PAIRS = 32768
NOALLOC_SCRATCH_BYTES = 8420608
STAGES = ["classify", "gjk_thread", "gjk_warp", "epa_thread", "epa_warp", "epa_wide"]


class NcgBatch(ctypes.Structure):
    _fields_ = [("shapes", ctypes.c_void_p), ("hull_points", ctypes.c_void_p), ("n_shapes", ctypes.c_uint32),
                ("pad0", ctypes.c_uint32), ("n_hull_points", ctypes.c_uint64), ("m1", ctypes.c_void_p),
                ("g1", ctypes.c_void_p), ("m2", ctypes.c_void_p), ("g2", ctypes.c_void_p),
                ("n_pairs", ctypes.c_uint64), ("init_dir", ctypes.c_void_p)]


class NcgHullTopology(ctypes.Structure):
    _fields_ = [("n_shapes", ctypes.c_uint64), ("n_hull_points", ctypes.c_uint64), ("n_faces", ctypes.c_uint64),
                ("n_face_slots", ctypes.c_uint64), ("n_edges", ctypes.c_uint64), ("n_vertex_slots", ctypes.c_uint64),
                ("shape", ctypes.c_void_p), ("face_normal", ctypes.c_void_p), ("face_range", ctypes.c_void_p),
                ("face_vertex", ctypes.c_void_p), ("face_edge", ctypes.c_void_p), ("edge_vertex", ctypes.c_void_p),
                ("edge_dir", ctypes.c_void_p), ("vertex_range", ctypes.c_void_p), ("vertex_face", ctypes.c_void_p),
                ("vertex_edge", ctypes.c_void_p)]


class NcgStats(ctypes.Structure):
    _fields_ = [("n_pairs", ctypes.c_uint64), ("n_epa", ctypes.c_uint64), ("n_epa_overflow", ctypes.c_uint64),
                ("gjk_iters", ctypes.c_uint64), ("epa_iters", ctypes.c_uint64),
                ("kernels_launched", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("n_epa_thread", ctypes.c_uint64)]


class NcgError(RuntimeError):
    pass


_lib = None


def load(build_if_missing=True):
    """Loads libncg.so; builds it first when the sources are newer."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise NcgError(f"libncg.so is not built ({LIB_PATH}); run ncollide_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    L.ncg_abi_version.restype = ctypes.c_int
    if L.ncg_abi_version() != ABI_VERSION:
        raise NcgError(f"{LIB_PATH} has C ABI version {L.ncg_abi_version()}, this binding expects {ABI_VERSION}: "
                       "rebuild it (ncollide_gb300.build.build(force=True))")
    vp, i32, f32, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint32
    P = ctypes.POINTER
    L.ncg_ctx_create.argtypes = [P(vp), i32]
    L.ncg_ctx_destroy.argtypes = [vp]
    L.ncg_ctx_set_tolerance.argtypes = [vp, i32]
    L.ncg_ctx_set_arithmetic.argtypes = [vp, i32]
    L.ncg_ctx_set_warm_start.argtypes = [vp, i32]
    L.ncg_sync.argtypes = [vp, vp]
    L.ncg_get_stats.argtypes = [vp, P(NcgStats)]
    L.ncg_last_error.restype = ctypes.c_char_p
    L.ncg_contact_batch.argtypes = [vp, P(NcgBatch), f32, vp, vp, vp, vp, vp, vp]
    L.ncg_distance_batch.argtypes = [vp, P(NcgBatch), vp, vp, vp, vp]
    L.ncg_proximity_batch.argtypes = [vp, P(NcgBatch), f32, vp, vp, vp, vp, vp]
    L.ncg_closest_points_batch.argtypes = [vp, P(NcgBatch), f32, vp, vp, vp, vp, vp]
    L.ncg_contact_batch_host.argtypes = [vp, P(NcgBatch), f32, vp, vp, vp, vp]
    L.ncg_distance_batch_host.argtypes = [vp, P(NcgBatch), vp, vp]
    L.ncg_proximity_batch_host.argtypes = [vp, P(NcgBatch), f32, vp, vp, vp]
    L.ncg_ctx_set_profiling.argtypes = [vp, i32]
    L.ncg_ctx_set_dispatch.argtypes = [vp, i32]
    L.ncg_get_stage_ms.argtypes = [vp, vp, i32]
    L.ncg_contact_batch_noalloc.argtypes = [P(NcgBatch), f32, i32, vp, vp, vp, vp, vp]
    L.ncg_ctx_set_tuning.argtypes = [vp, i32, i32]
    L.ncg_ctx_get_tuning.argtypes = [vp, i32, P(i32)]
    L.ncg_autotune.argtypes = [vp, P(NcgBatch), i32, f32, i32, vp, P(f32), vp]
    L.ncg_time_of_impact_batch.argtypes = [vp, P(NcgBatch), vp, vp, f32, f32, vp, vp, vp, vp, vp]
    L.ncg_ray_cast_batch.argtypes = [vp, P(NcgBatch), vp, f32, i32, vp, vp, vp, vp, vp, vp]
    L.ncg_aabb_batch.argtypes = [vp, P(NcgBatch), vp, vp, vp]
    L.ncg_bp_create.argtypes = [vp, f32, P(vp)]
    L.ncg_bp_update.argtypes = [vp, vp, ctypes.c_uint32, vp]
    L.ncg_bp_results.argtypes = [vp, P(ctypes.c_uint64), P(ctypes.c_uint64), P(ctypes.c_uint64), P(vp), P(vp),
                                 P(vp)]
    L.ncg_bp_destroy.argtypes = [vp]
    L.ncg_bp_copy.argtypes = [vp, vp, vp, vp, vp]
    L.ncg_gather_pairs.argtypes = [vp, vp, vp, vp, ctypes.c_uint64, vp, vp, vp, vp, vp]
    L.ncg_manifold_batch.argtypes = [vp, P(NcgBatch), f32, f32, f32, vp, vp, vp, vp, vp, vp]
    L.ncg_manifold_batch_hulls.argtypes = [vp, P(NcgBatch), P(NcgHullTopology), f32, f32, f32, vp, vp, vp, vp, vp,
                                           vp]
    L.ncg_hull_topology_build.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_uint64, P(NcgHullTopology),
                                          P(ctypes.c_uint32)]
    L.ncg_hull_topology_release.argtypes = [P(NcgHullTopology)]
    L.ncg_contact_graph_create.argtypes = [vp, P(NcgBatch), f32, vp, vp, vp, vp, vp, P(vp)]
    L.ncg_graph_launch.argtypes = [vp, vp]
    L.ncg_graph_destroy.argtypes = [vp]
    L.ncg_mlp_n_params.argtypes = []
    L.ncg_ctx_set_mlp_params.argtypes = [vp, vp, i32]
    L.ncg_mlp_features.argtypes = [P(NcgBatch), vp, vp, vp]
    L.ncg_mlp_infer.argtypes = [P(NcgBatch), vp, vp, vp, vp, vp]
    L.ncg_mlp_grad.argtypes = [vp, vp, vp, ctypes.c_uint64, f32, vp, vp, vp, vp]
    L.ncg_mlp_adam.argtypes = [vp, vp, vp, vp, f32, f32, f32, f32, i32, vp]
    for name in EXPORTED:
        if name != "ncg_last_error":
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def check(rc, what="ncg call"):
    if rc != NCG_OK:
        msg = load().ncg_last_error()
        raise NcgError(f"{what} failed (rc={rc}): {msg.decode() if msg else ''}")
    return rc
