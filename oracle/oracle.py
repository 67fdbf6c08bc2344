"""ctypes front end of the oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker.  The oracle is the C++ restatement of
the reference path in ncg_oracle.hpp, built by oracle/Makefile into
oracle/_build/libncg_oracle.so.

Policies: F32 = reference f32 path, F64 = reference built with f64 (the FP64
error oracle), MIXED = f32 supports with the f64 sub-solve (the GPU split).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libncg_oracle.so")

F32, F64, MIXED = 0, 1, 2
CONTACT, DISTANCE, PROXIMITY, CLOSEST, CONTACT_QUERY = 0, 1, 2, 3, 4
GJK_INTERSECTION, GJK_CLOSEST_POINTS, GJK_PROXIMITY, GJK_NO_INTERSECTION = 0, 1, 2, 3

_lib = None


def build(force=False):
    """Compiles the oracle with the committed Makefile (g++ only)."""
    srcs = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "ncg_oracle.hpp", "ncg_oracle_toi.hpp",
                                            "ncg_oracle_bp.hpp", "ncg_oracle_manifold.hpp", "dw.hpp")]
    if not force and os.path.exists(LIB_PATH):
        if os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in srcs):
            return LIB_PATH
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, f64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
        L.ncgo_query.argtypes = [i32, i32, f64, f64, f64, i32, vp, u32, vp, u64, u64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.ncgo_query.restype = i32
        L.ncgo_query_f64in.argtypes = [i32, i32, f64, f64, f64, i32, vp, vp, vp, vp, u32, vp, u64, u64, vp, vp, vp, vp, vp,
                                       vp, vp, vp, vp]
        L.ncgo_query_f64in.restype = i32
        L.ncgo_simplex_kat.argtypes = [i32, vp, vp, vp, vp]
        L.ncgo_toi.argtypes = [i32, i32, f64, f64, f64, i32, vp, u32, vp, u64, u64, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                               vp]
        L.ncgo_toi.restype = i32
        L.ncgo_ray_cast.argtypes = [i32, f64, i32, f64, i32, vp, u32, vp, u64, u64, vp, vp, vp, vp, vp, vp, vp]
        L.ncgo_ray_cast.restype = i32
        L.ncgo_aabb.argtypes = [vp, u32, vp, u64, u64, vp, vp, vp, vp]
        L.ncgo_aabb.restype = i32
        L.ncgo_pairs.argtypes = [vp, u32, vp, u64]
        L.ncgo_pairs.restype = ctypes.c_int64
        L.ncgo_manifold.argtypes = [vp, u32, u64, vp, vp, vp, vp, vp, vp, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, vp, vp, i32, vp, u64, vp]
        L.ncgo_manifold.restype = i32
        L.ncgo_simplex_kat.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class Result(dict):
    """p1, p2, dir (float64 [N,3]), value (depth or distance), gjk_kind, tag,
    status, counters (uint32 [N,8]: gjk iters, epa iters, support calls,
    hull points scanned, faces created, EPA max vertices, EPA max faces,
    sub-solves)."""

    def __getattr__(self, k):
        return self[k]


def _unpack(out, tag, status, counters):
    return Result(p1=out[:, 0:3], p2=out[:, 3:6], dir=out[:, 6:9], value=out[:, 9],
                  gjk_kind=out[:, 10].astype(np.int32), tag=tag, status=status, counters=counters)


def query(batch, query=CONTACT, policy=F32, param=0.0, eps=0.0, threads=None, epa_tol=0.0):
    """Runs the oracle over a PairBatch (host arrays in the ncg_batch layout)."""
    L = lib()
    n = batch.n_pairs
    threads = threads if threads is not None else (os.cpu_count() or 1)
    out = np.zeros((n, 16), np.float64)
    tag = np.zeros(n, np.uint8)
    status = np.zeros(n, np.uint32)
    counters = np.zeros((n, 8), np.uint32)
    shapes = np.ascontiguousarray(batch.shapes)
    pts = np.ascontiguousarray(batch.hull_points, np.float32)
    m1 = np.ascontiguousarray(batch.m1, np.float32)
    m2 = np.ascontiguousarray(batch.m2, np.float32)
    g1 = np.ascontiguousarray(batch.g1, np.uint32)
    g2 = np.ascontiguousarray(batch.g2, np.uint32)
    init = None if batch.init_dir is None else np.ascontiguousarray(batch.init_dir, np.float32)
    rc = L.ncgo_query(policy, query, float(param), float(eps), float(epa_tol), int(threads), _p(shapes), len(shapes), _p(pts),
                      pts.shape[0], n, _p(m1), _p(g1), _p(m2), _p(g2), _p(init), _p(out), _p(tag), _p(status),
                      _p(counters))
    if rc != 0:
        raise ValueError(f"oracle rejected the call (rc={rc})")
    return _unpack(out, tag, status, counters)


def query_f64(pairs, query=CONTACT, policy=F64, param=0.0, eps=0.0, init_dirs=None, epa_tol=0.0):
    """Known-answer entry: pairs = [(pose8, (kind, params4, points or None), pose8, (...)), ...]
    with every number given in float64 (decimal literals the f32 layout cannot hold)."""
    L = lib()
    kinds, offs, cnts, params, pts, m1, m2 = [], [], [], [], [], [], []
    npts = 0
    for (a, sa, b, sb) in pairs:
        for s in (sa, sb):
            kind, prm, p = s
            kinds.append(kind)
            params.append(list(prm) + [0.0] * (4 - len(prm)))
            if p is not None:
                p4 = np.zeros((len(p), 4))
                p4[:, :3] = p
                pts.append(p4)
                offs.append(npts)
                cnts.append(len(p))
                npts += len(p)
            else:
                offs.append(0)
                cnts.append(0)
        m1.append(a)
        m2.append(b)
    n = len(pairs)
    kinds = np.asarray(kinds, np.int32)
    offs = np.asarray(offs, np.uint32)
    cnts = np.asarray(cnts, np.uint32)
    params = np.asarray(params, np.float64)
    pts = np.concatenate(pts) if pts else np.zeros((1, 4))
    m1 = np.asarray(m1, np.float64)
    m2 = np.asarray(m2, np.float64)
    g1 = np.arange(0, 2 * n, 2, dtype=np.uint32)
    g2 = np.arange(1, 2 * n, 2, dtype=np.uint32)
    init = None if init_dirs is None else np.ascontiguousarray(init_dirs, np.float64)
    out = np.zeros((n, 16))
    tag = np.zeros(n, np.uint8)
    status = np.zeros(n, np.uint32)
    counters = np.zeros((n, 8), np.uint32)
    rc = L.ncgo_query_f64in(policy, query, float(param), float(eps), float(epa_tol), 1, _p(kinds), _p(offs), _p(cnts), _p(params),
                            len(kinds), _p(pts), pts.shape[0], n, _p(m1), _p(g1), _p(m2), _p(g2), _p(init),
                            _p(out), _p(tag), _p(status), _p(counters))
    if rc != 0:
        raise ValueError(f"oracle rejected the call (rc={rc})")
    return _unpack(out, tag, status, counters)


def simplex_kat(points, policy=F32):
    """benches/query/algorithm.rs: reset(a); add_point(b, c, d); project."""
    L = lib()
    pts = np.ascontiguousarray(points, np.float64).reshape(4, 3)
    added = np.zeros(3, np.int32)
    proj = np.zeros(3)
    dim = np.zeros(1, np.int32)
    L.ncgo_simplex_kat(policy, _p(pts), _p(added), _p(proj), _p(dim))
    return added, proj, int(dim[0])


def pose8(translation=(0, 0, 0), quaternion=(0, 0, 0, 1)):
    return list(quaternion) + list(translation) + [0.0]


TOI_OUT_OF_ITERATIONS, TOI_CONVERGED, TOI_FAILED, TOI_PENETRATING = 0, 1, 2, 3


def toi(batch, vel1, vel2, policy=F32, dispatch=0, max_toi=float("inf"), target_distance=0.0, eps=0.0, threads=None):
    """Linear time of impact per pair (time_of_impact_support_map_support_map;
    dispatch=1: Ball-Ball pairs by time_of_impact_ball_ball).  Returns a dict
    with toi, witness1, witness2, normal1, normal2 (local frames), status
    (TOIStatus), some (tag), gjk_status, iters."""
    L = lib()
    n = batch.n_pairs
    threads = threads if threads is not None else (os.cpu_count() or 1)
    out = np.zeros((n, 16), np.float64)
    tag = np.zeros(n, np.uint8)
    status = np.zeros(n, np.uint32)
    counters = np.zeros((n, 8), np.uint32)
    shapes = np.ascontiguousarray(batch.shapes)
    pts = np.ascontiguousarray(batch.hull_points, np.float32)
    m1 = np.ascontiguousarray(batch.m1, np.float32)
    m2 = np.ascontiguousarray(batch.m2, np.float32)
    g1 = np.ascontiguousarray(batch.g1, np.uint32)
    g2 = np.ascontiguousarray(batch.g2, np.uint32)
    v1 = np.ascontiguousarray(vel1, np.float32).reshape(n, 3)
    v2 = np.ascontiguousarray(vel2, np.float32).reshape(n, 3)
    mt = float(np.finfo(np.float32).max) if not np.isfinite(max_toi) else float(max_toi)
    rc = L.ncgo_toi(policy, dispatch, mt, float(target_distance), float(eps), int(threads), _p(shapes), len(shapes),
                    _p(pts), pts.shape[0], n, _p(m1), _p(g1), _p(m2), _p(g2), _p(v1), _p(v2), _p(out), _p(tag),
                    _p(status), _p(counters))
    if rc != 0:
        raise ValueError(f"oracle rejected the call (rc={rc})")
    return {"toi": out[:, 0], "witness1": out[:, 1:4], "witness2": out[:, 4:7], "normal1": out[:, 7:10],
            "normal2": out[:, 10:13], "status": out[:, 13].astype(np.int32), "some": tag, "gjk_status": status,
            "iters": counters[:, 0]}



def ray_cast(batch, rays, policy=F32, max_toi=float("inf"), solid=True, eps=0.0, threads=None):
    """Ray casts on support maps (RayCast::toi_and_normal_with_ray via the GJK
    ray cast): ray i against shapes[g1[i]] at pose m1[i]; rays [N,6] = origin,
    dir (world).  Returns a dict with hit, toi, normal (world), status, iters."""
    L = lib()
    n = batch.n_pairs
    threads = threads if threads is not None else (os.cpu_count() or 1)
    out = np.zeros((n, 16), np.float64)
    tag = np.zeros(n, np.uint8)
    status = np.zeros(n, np.uint32)
    counters = np.zeros((n, 8), np.uint32)
    shapes = np.ascontiguousarray(batch.shapes)
    pts = np.ascontiguousarray(batch.hull_points, np.float32)
    m1 = np.ascontiguousarray(batch.m1, np.float32)
    g1 = np.ascontiguousarray(batch.g1, np.uint32)
    ry = np.ascontiguousarray(rays, np.float32).reshape(n, 6)
    mt = float(np.finfo(np.float32).max) if not np.isfinite(max_toi) else float(max_toi)
    rc = L.ncgo_ray_cast(policy, mt, int(bool(solid)), float(eps), int(threads), _p(shapes), len(shapes), _p(pts),
                         pts.shape[0], n, _p(m1), _p(g1), _p(ry), _p(out), _p(tag), _p(status), _p(counters))
    if rc != 0:
        raise ValueError(f"oracle rejected the call (rc={rc})")
    return {"hit": tag, "toi": out[:, 0], "normal": out[:, 1:4], "status": status, "iters": counters[:, 0]}


def aabbs(batch):
    """World AABBs [N,6] (mins, maxs) of shapes[g1[i]] at m1[i], and status."""
    L = lib()
    n = batch.n_pairs
    out = np.zeros((n, 6), np.float32)
    status = np.zeros(n, np.uint32)
    shapes = np.ascontiguousarray(batch.shapes)
    pts = np.ascontiguousarray(batch.hull_points, np.float32)
    m1 = np.ascontiguousarray(batch.m1, np.float32)
    g1 = np.ascontiguousarray(batch.g1, np.uint32)
    L.ncgo_aabb(_p(shapes), len(shapes), _p(pts), pts.shape[0], n, _p(m1), _p(g1), _p(out), _p(status))
    return out, status


def intersecting_pairs(boxes):
    """Sorted uint64 keys (lo << 32 | hi) of every intersecting pair of boxes [N,6]."""
    L = lib()
    b = np.ascontiguousarray(boxes, np.float32).reshape(-1, 6)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, np.uint64)
        k = L.ncgo_pairs(_p(b), b.shape[0], _p(out), cap)
        if k <= cap:
            return out[:k]
        cap = int(k)


class BroadPhase:
    """The pair set and events of DBVTBroadPhase.update (dbvt_broad_phase.rs:174-258):
    a proxy's stored box is replaced by new_box.loosened(margin) when the stored
    box does not contain the new one (deferred_set_bounding_volume, :322-347);
    the pairs are the intersecting pairs of the stored boxes; started / stopped
    are the pairs that entered / left the set.  A proxy whose box has a NaN
    bound has no pairs (removed)."""

    def __init__(self, margin):
        self.margin = np.float32(margin)
        self.stored = np.zeros((0, 6), np.float32)
        self.pairs = np.zeros(0, np.uint64)

    def update(self, boxes):
        b = np.asarray(boxes, np.float32).reshape(-1, 6)
        n_old = self.stored.shape[0]
        st = np.full((b.shape[0], 6), np.nan, np.float32)
        st[:n_old] = self.stored[:b.shape[0]]
        with np.errstate(invalid="ignore"):
            contains = (st[:, :3] <= b[:, :3]).all(1) & (st[:, 3:] >= b[:, 3:]).all(1)
        new = ~contains
        st[new, :3] = b[new, :3] + (-self.margin)
        st[new, 3:] = b[new, 3:] + self.margin
        self.stored = st
        pairs = intersecting_pairs(st)
        started = np.setdiff1d(pairs, self.pairs)
        stopped = np.setdiff1d(self.pairs, pairs)
        self.pairs = pairs
        return pairs, started, stopped


MANIFOLD_MAX = 16
MANIFOLD_DTYPE = np.dtype([("normal", np.float32, 3), ("n", np.uint32),
                           ("points", np.dtype([("world1", np.float32, 3), ("world2", np.float32, 3),
                                                ("depth", np.float32), ("feature1", np.uint32),
                                                ("feature2", np.uint32)]), MANIFOLD_MAX)])


def manifold(batch, contact9, has, linear=0.0, angular1=0.0, angular2=0.0, threads=None, topology=None):
    """Manifolds (MANIFOLD_DTYPE [N]) and status from each pair's contact query
    result: contact9 [N,9] = world1, world2, normal (float32), has [N].
    topology: the ConvexHull topology (an ncg_hull_topology of host arrays,
    ncollide_gb300.hulls.HostTopology) to treat ConvexHull shapes as
    polyhedra; None keeps their pairs to the single contact."""
    L = lib()
    n = batch.n_pairs
    out = np.zeros(n, MANIFOLD_DTYPE)
    status = np.zeros(n, np.uint32)
    shapes = np.ascontiguousarray(batch.shapes)
    m1 = np.ascontiguousarray(batch.m1, np.float32)
    m2 = np.ascontiguousarray(batch.m2, np.float32)
    g1 = np.ascontiguousarray(batch.g1, np.uint32)
    g2 = np.ascontiguousarray(batch.g2, np.uint32)
    c = np.ascontiguousarray(contact9, np.float32).reshape(n, 9)
    h = np.ascontiguousarray(has, np.uint8)
    threads = threads if threads is not None else (os.cpu_count() or 1)
    pts = np.ascontiguousarray(batch.hull_points, np.float32)
    L.ncgo_manifold(_p(shapes), len(shapes), n, _p(m1), _p(g1), _p(m2), _p(g2), _p(c), _p(h), float(linear),
                    float(angular1), float(angular2), _p(out), _p(status), int(threads), _p(pts), pts.shape[0],
                    None if topology is None else ctypes.addressof(topology.struct))
    return out, status