"""Batched queries: the drop-in for ncollide3d's support-map query functions.

    contact_batch        contact_support_map_support_map[_with_params]
                         (src/query/contact/contact_support_map_support_map.rs:9-88)
    distance_batch       distance_support_map_support_map[_with_params]
                         (src/query/distance/distance_support_map_support_map.rs:8-53)
    proximity_batch      proximity_support_map_support_map[_with_params]
                         (src/query/proximity/proximity_support_map_support_map.rs:10-75)
    closest_points_batch closest_points_support_map_support_map[_with_params]
                         (src/query/closest_points/closest_points_support_map_support_map.rs:9-67)

Each takes a Context and a DeviceBatch (pairs resident in device memory) and
returns device tensors; the work is queued on the current torch CUDA stream.
The *_host variants take a host PairBatch and copy in and out through the
library's synchronous host entry points.  PyTorch only supplies device memory
and streams; every computation runs in libncg.so.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .shapes import CONTACT_DTYPE, PairBatch

# Launch-tuning keys of ncg_ctx_set_tuning by name.
TUNING_KEYS = {"hull_gjk_warp": N.TUNE_HULL_GJK_WARP, "gjk_blocks": N.TUNE_GJK_BLOCKS,
               "epa_blocks": N.TUNE_EPA_BLOCKS, "l1_carveout": N.TUNE_L1_CARVEOUT,
               "hull_stage_min": N.TUNE_HULL_STAGE_MIN, "hull_stage_cap": N.TUNE_HULL_STAGE_CAP,
               "hull_epa_warp": N.TUNE_HULL_EPA_WARP, "hull_locality": N.TUNE_HULL_LOCALITY}


class Context:
    """Owns an ncg_ctx: scratch memory, EPA slabs and settings for one device."""

    def __init__(self, device=0, tolerance=N.TOL_REFERENCE, warm_start=N.WARM_NONE, dispatch=N.DISPATCH_SUPPORT_MAP,
                 arithmetic=N.ARITH_SPLIT):
        self._L = N.load()
        self._p = ctypes.c_void_p()
        if isinstance(device, torch.device):
            device = device.index or 0
        self.device = int(device)
        N.check(self._L.ncg_ctx_create(ctypes.byref(self._p), self.device), "ncg_ctx_create")
        self.set_tolerance(tolerance)
        self.set_warm_start(warm_start)
        self.set_dispatch(dispatch)
        self.set_arithmetic(arithmetic)

    @property
    def handle(self):
        return self._p

    def set_tolerance(self, mode):
        if isinstance(mode, str):
            mode = {"reference": N.TOL_REFERENCE, "precise": N.TOL_PRECISE}[mode]
        N.check(self._L.ncg_ctx_set_tolerance(self._p, int(mode)), "ncg_ctx_set_tolerance")
        self.tolerance = int(mode)

    def set_arithmetic(self, mode):
        """NCG_ARITH_SPLIT (f32 supports, double-word sub-solve; the default) or
        NCG_ARITH_F32 (the reference's f32 path bit for bit)."""
        if isinstance(mode, str):
            mode = {"split": N.ARITH_SPLIT, "f32": N.ARITH_F32}[mode]
        N.check(self._L.ncg_ctx_set_arithmetic(self._p, int(mode)), "ncg_ctx_set_arithmetic")
        self.arithmetic = int(mode)

    def set_dispatch(self, mode):
        """NCG_DISPATCH_SUPPORT_MAP (every pair by GJK/EPA) or NCG_DISPATCH_QUERY
        (query::contact's routing of Ball pairs)."""
        if isinstance(mode, str):
            mode = {"support_map": N.DISPATCH_SUPPORT_MAP, "query": N.DISPATCH_QUERY}[mode]
        N.check(self._L.ncg_ctx_set_dispatch(self._p, int(mode)), "ncg_ctx_set_dispatch")
        self.dispatch = int(mode)

    def set_tuning(self, key, value):
        """Launch tuning (ncg_ctx_set_tuning); results do not depend on it."""
        if isinstance(key, str):
            key = TUNING_KEYS[key]
        N.check(self._L.ncg_ctx_set_tuning(self._p, int(key), int(value)), "ncg_ctx_set_tuning")

    def tuning(self):
        """The context's launch tuning by key name (ncg_ctx_get_tuning)."""
        out = {}
        for name, key in TUNING_KEYS.items():
            v = ctypes.c_int32()
            N.check(self._L.ncg_ctx_get_tuning(self._p, int(key), ctypes.byref(v)), "ncg_ctx_get_tuning")
            out[name] = int(v.value)
        return out

    def apply_tuning(self, values):
        """Sets every key of a {name: value} mapping (e.g. a saved autotune result)."""
        for k, v in values.items():
            self.set_tuning(k, int(v))

    def autotune(self, batch, query="contact", param=0.0, reps=3, stream=None):
        """Runs the library's autotuner (ncg_autotune) on a device-resident
        batch and leaves the fastest launch tuning set in this context.
        Returns {"values": {name: value}, "ms": time of one call}."""
        q = {"contact": N.QUERY_CONTACT, "distance": N.QUERY_DISTANCE, "proximity": N.QUERY_PROXIMITY,
             "closest_points": N.QUERY_CLOSEST_POINTS}[query] if isinstance(query, str) else int(query)
        vals = (ctypes.c_int32 * N.N_TUNE)()
        ms = ctypes.c_float()
        st = stream if stream is not None else torch.cuda.current_stream(batch.m1.device)
        cb = batch.c_struct()
        N.check(self._L.ncg_autotune(self._p, ctypes.byref(cb), int(q), ctypes.c_float(param), int(reps), vals,
                                     ctypes.byref(ms), ctypes.c_void_p(st.cuda_stream)), "ncg_autotune")
        names = {v: k for k, v in TUNING_KEYS.items()}
        return {"values": {names[i]: int(vals[i]) for i in range(N.N_TUNE)}, "ms": float(ms.value)}

    def set_warm_start(self, mode):
        N.check(self._L.ncg_ctx_set_warm_start(self._p, int(mode)), "ncg_ctx_set_warm_start")
        self.warm_start = int(mode)

    def set_mlp_params(self, params):
        """Parameters of the learned warm start (NCG_MLP_N_PARAMS f32 values, host or device)."""
        if isinstance(params, torch.Tensor):
            t = params.detach().contiguous().float()
            N.check(self._L.ncg_ctx_set_mlp_params(self._p, ctypes.c_void_p(t.data_ptr()), int(t.numel())),
                    "ncg_ctx_set_mlp_params")
        else:
            a = np.ascontiguousarray(params, np.float32)
            N.check(self._L.ncg_ctx_set_mlp_params(self._p, ctypes.c_void_p(a.ctypes.data), int(a.size)),
                    "ncg_ctx_set_mlp_params")

    def set_profiling(self, on=True):
        """Records CUDA events between the library's kernel launches."""
        N.check(self._L.ncg_ctx_set_profiling(self._p, 1 if on else 0), "ncg_ctx_set_profiling")

    def stage_ms(self):
        """Per-kernel durations (ms) of the last call, keyed by stage name."""
        import numpy as _np
        buf = _np.zeros(len(N.STAGES), _np.float32)
        n = self._L.ncg_get_stage_ms(self._p, buf.ctypes.data, len(N.STAGES))
        if n < 0:
            N.check(n, "ncg_get_stage_ms")
        return {k: float(buf[i]) for i, k in enumerate(N.STAGES[:n])}

    def stats(self):
        s = N.NcgStats()
        N.check(self._L.ncg_get_stats(self._p, ctypes.byref(s)), "ncg_get_stats")
        return {k: int(getattr(s, k)) for k, _ in N.NcgStats._fields_ }

    def close(self):
        if self._p:
            self._L.ncg_ctx_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


@dataclass
class DeviceBatch:
    """A PairBatch resident in device memory (torch tensors, ncg_batch layout)."""
    shapes: torch.Tensor       # uint8 [S*32]
    hull_points: torch.Tensor  # float32 [P,4]
    m1: torch.Tensor           # float32 [N,8]
    g1: torch.Tensor           # int32 [N] (read as uint32)
    m2: torch.Tensor
    g2: torch.Tensor
    init_dir: torch.Tensor | None = None
    n_shapes: int = 0

    @property
    def n_pairs(self):
        return int(self.g1.shape[0])

    @classmethod
    def from_host(cls, b: PairBatch, device="cuda", non_blocking=False):
        def t(a, dt=None):
            x = torch.from_numpy(np.ascontiguousarray(a))
            if dt is not None:
                x = x.view(dt)
            return x.to(device, non_blocking=non_blocking)
        return cls(shapes=t(b.shapes.view(np.uint8)), hull_points=t(b.hull_points.astype(np.float32)),
                   m1=t(b.m1.astype(np.float32)), g1=t(b.g1.astype(np.uint32).view(np.int32)),
                   m2=t(b.m2.astype(np.float32)), g2=t(b.g2.astype(np.uint32).view(np.int32)),
                   init_dir=None if b.init_dir is None else t(b.init_dir.astype(np.float32)),
                   n_shapes=len(b.shapes))

    def with_init_dir(self, init_dir):
        return DeviceBatch(self.shapes, self.hull_points, self.m1, self.g1, self.m2, self.g2,
                           None if init_dir is None else init_dir.contiguous(), self.n_shapes)

    def c_struct(self):
        return N.NcgBatch(self.shapes.data_ptr(), self.hull_points.data_ptr(), self.n_shapes, 0,
                          int(self.hull_points.shape[0]), self.m1.data_ptr(), self.g1.data_ptr(),
                          self.m2.data_ptr(), self.g2.data_ptr(), self.n_pairs,
                          None if self.init_dir is None else self.init_dir.data_ptr())


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _empty(n, shape, dtype, device):
    return torch.empty((n,) + tuple(shape), dtype=dtype, device=device)


def contact_batch(ctx: Context, db: DeviceBatch, prediction=0.0, with_dir=True, with_iters=False, stream=None):
    """Returns dict: contact [N,10] (world1, world2, normal, depth), has_contact [N] uint8,
    dir [N,3] (the direction to pass back as init_dir), status [N] int32, iters [N] int32."""
    n, dev = db.n_pairs, db.m1.device
    out = {"contact": _empty(n, (10,), torch.float32, dev), "has_contact": _empty(n, (), torch.uint8, dev),
           "status": _empty(n, (), torch.int32, dev)}
    out["dir"] = _empty(n, (3,), torch.float32, dev) if with_dir else None
    out["iters"] = _empty(n, (), torch.int32, dev) if with_iters else None
    cb = db.c_struct()
    N.check(ctx._L.ncg_contact_batch(ctx.handle, ctypes.byref(cb), ctypes.c_float(prediction), _ptr(out["contact"]),
                                     _ptr(out["has_contact"]), _ptr(out["dir"]), _ptr(out["status"]),
                                     _ptr(out["iters"]), _stream(stream)), "ncg_contact_batch")
    return out


class ContactGraph:
    """One ncg_contact_batch call captured as a CUDA graph (ncg_contact_graph_create).

    `launch()` replays it on the batch's buffers as they are at replay time;
    the outputs live in `self.out`.  With `reuse_dir=True` the batch's init_dir
    buffer is also the out_dir buffer, so each replay starts GJK from the
    direction the previous replay returned (the reference's `last_gjk_dir`);
    the context must then have NCG_WARM_INIT_DIR set."""

    def __init__(self, ctx: Context, db: DeviceBatch, prediction=0.0, reuse_dir=False, with_iters=False):
        n, dev = db.n_pairs, db.m1.device
        self.ctx, self.db = ctx, db
        self.out = {"contact": _empty(n, (10,), torch.float32, dev), "has_contact": _empty(n, (), torch.uint8, dev),
                    "status": _empty(n, (), torch.int32, dev),
                    "iters": _empty(n, (), torch.int32, dev) if with_iters else None}
        if reuse_dir:
            if db.init_dir is None:
                raise ValueError("reuse_dir needs a batch with an init_dir buffer")
            self.out["dir"] = db.init_dir
        else:
            self.out["dir"] = _empty(n, (3,), torch.float32, dev)
        cb = db.c_struct()
        h = ctypes.c_void_p()
        o = self.out
        N.check(ctx._L.ncg_contact_graph_create(ctx.handle, ctypes.byref(cb), ctypes.c_float(prediction),
                                                _ptr(o["contact"]), _ptr(o["has_contact"]), _ptr(o["dir"]),
                                                _ptr(o["status"]), _ptr(o["iters"]), ctypes.byref(h)),
                "ncg_contact_graph_create")
        self._h = h

    def launch(self, stream=None):
        N.check(self.ctx._L.ncg_graph_launch(self._h, _stream(stream)), "ncg_graph_launch")
        return self.out

    def close(self):
        # a closed context has already destroyed its graphs
        if self._h and self.ctx._p:
            self.ctx._L.ncg_graph_destroy(self._h)
        self._h = None


def distance_batch(ctx: Context, db: DeviceBatch, with_iters=False, stream=None):
    n, dev = db.n_pairs, db.m1.device
    out = {"distance": _empty(n, (), torch.float32, dev), "status": _empty(n, (), torch.int32, dev),
           "iters": _empty(n, (), torch.int32, dev) if with_iters else None}
    cb = db.c_struct()
    N.check(ctx._L.ncg_distance_batch(ctx.handle, ctypes.byref(cb), _ptr(out["distance"]), _ptr(out["status"]),
                                      _ptr(out["iters"]), _stream(stream)), "ncg_distance_batch")
    return out


def proximity_batch(ctx: Context, db: DeviceBatch, margin=0.0, with_dir=True, with_iters=False, stream=None):
    n, dev = db.n_pairs, db.m1.device
    out = {"proximity": _empty(n, (), torch.uint8, dev), "status": _empty(n, (), torch.int32, dev),
           "dir": _empty(n, (3,), torch.float32, dev) if with_dir else None,
           "iters": _empty(n, (), torch.int32, dev) if with_iters else None}
    cb = db.c_struct()
    N.check(ctx._L.ncg_proximity_batch(ctx.handle, ctypes.byref(cb), ctypes.c_float(margin), _ptr(out["proximity"]),
                                       _ptr(out["dir"]), _ptr(out["status"]), _ptr(out["iters"]),
                                       _stream(stream)), "ncg_proximity_batch")
    return out


def closest_points_batch(ctx: Context, db: DeviceBatch, prediction=0.0, with_iters=False, stream=None):
    n, dev = db.n_pairs, db.m1.device
    out = {"tag": _empty(n, (), torch.uint8, dev), "points": _empty(n, (6,), torch.float32, dev),
           "status": _empty(n, (), torch.int32, dev),
           "iters": _empty(n, (), torch.int32, dev) if with_iters else None}
    cb = db.c_struct()
    N.check(ctx._L.ncg_closest_points_batch(ctx.handle, ctypes.byref(cb), ctypes.c_float(prediction),
                                            _ptr(out["tag"]), _ptr(out["points"]), _ptr(out["status"]),
                                            _ptr(out["iters"]), _stream(stream)), "ncg_closest_points_batch")
    return out


def time_of_impact_batch(ctx: Context, db: DeviceBatch, vel1, vel2, max_toi=float("inf"), target_distance=0.0,
                         with_iters=False, stream=None):
    """query::time_of_impact for every pair: vel1, vel2 [N,3] float32 device
    tensors (linear velocities).  Returns has_toi (1 = Some), toi, witness1,
    witness2, normal1, normal2 (local frames), toi_status (TOIStatus), status
    (NCG_STATUS_* bits) and, with with_iters, the ray-cast iterations."""
    n, dev = db.n_pairs, db.m1.device
    vel1 = vel1.to(dev, torch.float32).contiguous()
    vel2 = vel2.to(dev, torch.float32).contiguous()
    if n and (tuple(vel1.shape) != (n, 3) or tuple(vel2.shape) != (n, 3)):
        raise ValueError("vel1 and vel2 must be [n_pairs, 3]")
    rec = _empty(n, (14,), torch.float32, dev)
    has = _empty(n, (), torch.uint8, dev)
    status = _empty(n, (), torch.int32, dev)
    iters = _empty(n, (), torch.int32, dev) if with_iters else None
    cb = db.c_struct()
    N.check(ctx._L.ncg_time_of_impact_batch(ctx.handle, ctypes.byref(cb), _ptr(vel1), _ptr(vel2),
                                            ctypes.c_float(max_toi), ctypes.c_float(target_distance), _ptr(rec),
                                            _ptr(has), _ptr(status), _ptr(iters), _stream(stream)),
            "ncg_time_of_impact_batch")
    return {"has_toi": has, "toi": rec[:, 0], "witness1": rec[:, 1:4], "witness2": rec[:, 4:7],
            "normal1": rec[:, 7:10], "normal2": rec[:, 10:13], "toi_status": rec[:, 13].view(torch.int32),
            "status": status, "iters": iters, "_keep": (vel1, vel2)}


def ray_cast_batch(ctx: Context, db: DeviceBatch, rays, max_toi=float("inf"), solid=True, with_normal=True,
                   with_iters=False, stream=None):
    """RayCast::toi_and_normal_with_ray (GJK ray cast) for every ray: ray i
    against shape g1[i] at pose m1[i]; rays [N,6] float32 device tensor
    (origin, dir; world frame).  Returns has_hit, toi, normal (world), status
    and, with with_iters, the ray-cast iterations."""
    n, dev = db.n_pairs, db.m1.device
    rays = rays.to(dev, torch.float32).contiguous()
    if n and tuple(rays.shape) != (n, 6):
        raise ValueError("rays must be [n, 6]")
    out = {"has_hit": _empty(n, (), torch.uint8, dev), "toi": _empty(n, (), torch.float32, dev),
           "normal": _empty(n, (3,), torch.float32, dev) if with_normal else None,
           "status": _empty(n, (), torch.int32, dev),
           "iters": _empty(n, (), torch.int32, dev) if with_iters else None}
    cb = db.c_struct()
    N.check(ctx._L.ncg_ray_cast_batch(ctx.handle, ctypes.byref(cb), _ptr(rays), ctypes.c_float(max_toi),
                                      int(bool(solid)), _ptr(out["toi"]), _ptr(out["normal"]), _ptr(out["has_hit"]),
                                      _ptr(out["status"]), _ptr(out["iters"]), _stream(stream)),
            "ncg_ray_cast_batch")
    out["_keep"] = rays
    return out


def aabb_batch(ctx: Context, db: DeviceBatch, stream=None):
    """World AABBs [N,6] (mins, maxs) of shape g1[i] at pose m1[i], and status."""
    n, dev = db.n_pairs, db.m1.device
    out = _empty(n, (6,), torch.float32, dev)
    status = _empty(n, (), torch.int32, dev)
    cb = db.c_struct()
    N.check(ctx._L.ncg_aabb_batch(ctx.handle, ctypes.byref(cb), _ptr(out), _ptr(status), _stream(stream)),
            "ncg_aabb_batch")
    return out, status


class BroadPhase:
    """DBVTBroadPhase over proxies 0..n-1 on the device: update(boxes) stores
    each box (loosened by `margin` when it left its stored box) and returns
    (pairs, started, stopped) as int64 [k,2] device tensors sorted by
    (lower id, higher id)."""

    def __init__(self, ctx: Context, margin):
        self._L = ctx._L
        self._ctx = ctx
        self._p = ctypes.c_void_p()
        N.check(self._L.ncg_bp_create(ctx.handle, ctypes.c_float(margin), ctypes.byref(self._p)), "ncg_bp_create")
        self.device = torch.device("cuda", ctx.device)

    def update(self, boxes, stream=None):
        boxes = boxes.to(self.device, torch.float32).contiguous()
        n = boxes.shape[0]
        N.check(self._L.ncg_bp_update(self._p, _ptr(boxes) if n else None, n, _stream(stream)), "ncg_bp_update")
        counts = [ctypes.c_uint64() for _ in range(3)]
        ptrs = [ctypes.c_void_p() for _ in range(3)]
        N.check(self._L.ncg_bp_results(self._p, *[ctypes.byref(c) for c in counts], *[ctypes.byref(p) for p in ptrs]),
                "ncg_bp_results")
        bufs = [torch.empty((int(c.value), 2), dtype=torch.int32, device=self.device) for c in counts]
        N.check(self._L.ncg_bp_copy(self._p, *[_ptr(b) if b.numel() else None for b in bufs], _stream(stream)),
                "ncg_bp_copy")
        self.pairs_u32 = bufs[0]  # the pair list as stored (uint32 ids), for gather_pairs
        return tuple(b.to(torch.int64) & 0xffffffff for b in bufs)

    def close(self):
        if self._p:
            self._L.ncg_bp_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gather_pairs(ctx: Context, objects: DeviceBatch, pairs_u32, stream=None):
    """The narrow-phase DeviceBatch of a pair list: objects holds one proxy per
    entry (pose m1, shape id g1); pairs_u32 [k,2] int32 (uint32 ids)."""
    k, dev = int(pairs_u32.shape[0]), objects.m1.device
    pairs_u32 = pairs_u32.contiguous()
    m1 = torch.empty((k, 8), dtype=torch.float32, device=dev)
    m2 = torch.empty((k, 8), dtype=torch.float32, device=dev)
    g1 = torch.empty(k, dtype=torch.int32, device=dev)
    g2 = torch.empty(k, dtype=torch.int32, device=dev)
    N.check(ctx._L.ncg_gather_pairs(ctx.handle, _ptr(objects.m1), _ptr(objects.g1), _ptr(pairs_u32), k, _ptr(m1),
                                    _ptr(g1), _ptr(m2), _ptr(g2), _stream(stream)), "ncg_gather_pairs")
    return DeviceBatch(objects.shapes, objects.hull_points, m1, g1, m2, g2, None, objects.n_shapes)


def manifold_batch(ctx: Context, db: DeviceBatch, prediction=0.0, angular1=0.0, angular2=0.0, stream=None,
                   topology=None):
    """ConvexPolyhedronConvexPolyhedronManifoldGenerator::generate_contacts for
    every pair.  Returns the contact query's contact / has_contact / dir and
    manifold: uint8 [N, 16 + 16 * 36] device tensor in the ncg_manifold layout
    (normal[3] f32, n u32, 16 points of world1[3], world2[3], depth, feature1,
    feature2), and status.  topology: a hulls.DeviceTopology of the batch's
    shapes, to treat ConvexHull shapes as polyhedra (ncg_manifold_batch_hulls)."""
    n, dev = db.n_pairs, db.m1.device
    out = {"contact": _empty(n, (10,), torch.float32, dev), "has_contact": _empty(n, (), torch.uint8, dev),
           "dir": _empty(n, (3,), torch.float32, dev),
           "manifold": _empty(n, (16 + 36 * N.MANIFOLD_MAX,), torch.uint8, dev),
           "status": _empty(n, (), torch.int32, dev)}
    cb = db.c_struct()
    N.check(ctx._L.ncg_manifold_batch_hulls(ctx.handle, ctypes.byref(cb),
                                            None if topology is None else ctypes.byref(topology.struct),
                                            ctypes.c_float(prediction), ctypes.c_float(angular1),
                                            ctypes.c_float(angular2), _ptr(out["contact"]), _ptr(out["has_contact"]),
                                            _ptr(out["dir"]), _ptr(out["manifold"]), _ptr(out["status"]),
                                            _stream(stream)), "ncg_manifold_batch_hulls")
    return out


def _host_struct(b: PairBatch, keep):
    arrs = {"shapes": np.ascontiguousarray(b.shapes), "hull": np.ascontiguousarray(b.hull_points, np.float32),
            "m1": np.ascontiguousarray(b.m1, np.float32), "g1": np.ascontiguousarray(b.g1, np.uint32),
            "m2": np.ascontiguousarray(b.m2, np.float32), "g2": np.ascontiguousarray(b.g2, np.uint32),
            "init": None if b.init_dir is None else np.ascontiguousarray(b.init_dir, np.float32)}
    keep.append(arrs)
    p = lambda a: None if a is None else a.ctypes.data
    return N.NcgBatch(p(arrs["shapes"]), p(arrs["hull"]), len(b.shapes), 0, arrs["hull"].shape[0], p(arrs["m1"]),
                      p(arrs["g1"]), p(arrs["m2"]), p(arrs["g2"]), b.n_pairs, p(arrs["init"]))


def contact_batch_host(ctx: Context, b: PairBatch, prediction=0.0):
    """Host-memory contact query (copies inputs in and results out)."""
    keep = []
    cb = _host_struct(b, keep)
    n = b.n_pairs
    contact = np.zeros(n, CONTACT_DTYPE)
    has = np.zeros(n, np.uint8)
    d = np.zeros((n, 3), np.float32)
    st = np.zeros(n, np.uint32)
    N.check(ctx._L.ncg_contact_batch_host(ctx.handle, ctypes.byref(cb), ctypes.c_float(prediction),
                                          contact.ctypes.data, has.ctypes.data, d.ctypes.data, st.ctypes.data),
            "ncg_contact_batch_host")
    return {"contact": contact, "has_contact": has, "dir": d, "status": st}


def distance_batch_host(ctx: Context, b: PairBatch):
    keep = []
    cb = _host_struct(b, keep)
    n = b.n_pairs
    dist = np.zeros(n, np.float32)
    st = np.zeros(n, np.uint32)
    N.check(ctx._L.ncg_distance_batch_host(ctx.handle, ctypes.byref(cb), dist.ctypes.data, st.ctypes.data),
            "ncg_distance_batch_host")
    return {"distance": dist, "status": st}


def proximity_batch_host(ctx: Context, b: PairBatch, margin=0.0):
    keep = []
    cb = _host_struct(b, keep)
    n = b.n_pairs
    prox = np.zeros(n, np.uint8)
    d = np.zeros((n, 3), np.float32)
    st = np.zeros(n, np.uint32)
    N.check(ctx._L.ncg_proximity_batch_host(ctx.handle, ctypes.byref(cb), ctypes.c_float(margin), prox.ctypes.data,
                                            d.ctypes.data, st.ctypes.data), "ncg_proximity_batch_host")
    return {"proximity": prox, "dir": d, "status": st}
