"""ConvexHull face topology (ConvexHull::try_new, src/shape/convex.rs:88-328)
for the ConvexHull shapes of a batch, built once by the library on the host
(ncg_hull_topology_build) and kept as numpy arrays; `to_device` copies it for
ncg_manifold_batch_hulls."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .shapes import PairBatch

_ARRAYS = [  # field, dtype, columns, count field
    ("shape", np.uint32, 4, "n_shapes"), ("face_normal", np.float32, 4, "n_faces"),
    ("face_range", np.uint32, 2, "n_faces"), ("face_vertex", np.uint32, 1, "n_face_slots"),
    ("face_edge", np.uint32, 1, "n_face_slots"), ("edge_vertex", np.uint32, 2, "n_edges"),
    ("edge_dir", np.float32, 4, "n_edges"), ("vertex_range", np.uint32, 2, "n_hull_points"),
    ("vertex_face", np.uint32, 1, "n_vertex_slots"), ("vertex_edge", np.uint32, 1, "n_vertex_slots")]


class HostTopology:
    """The topology as numpy arrays, and an ncg_hull_topology struct over them."""

    def __init__(self, batch: PairBatch):
        L = N.load()
        raw = N.NcgHullTopology()
        failed = ctypes.c_uint32(0)
        shapes = np.ascontiguousarray(batch.shapes)
        pts = np.ascontiguousarray(batch.hull_points, np.float32)
        N.check(L.ncg_hull_topology_build(shapes.ctypes.data, len(shapes), pts.ctypes.data, pts.shape[0],
                                          ctypes.byref(raw), ctypes.byref(failed)), "ncg_hull_topology_build")
        self.counts = {k: int(getattr(raw, k)) for k in ("n_shapes", "n_hull_points", "n_faces", "n_face_slots",
                                                          "n_edges", "n_vertex_slots")}
        self.arrays = {}
        for name, dt, cols, cnt in _ARRAYS:
            n = self.counts[cnt] * cols
            ptr = getattr(raw, name)
            a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt))), (max(n, 1),))
            self.arrays[name] = a[:n].copy().reshape(-1, cols) if cols > 1 else a[:n].copy()
        L.ncg_hull_topology_release(ctypes.byref(raw))
        self.n_failed = int(failed.value)
        self.struct = self._struct(lambda a: a.ctypes.data if a.size else None)

    def _struct(self, ptr):
        s = N.NcgHullTopology(**self.counts)
        for name, _, _, _ in _ARRAYS:
            setattr(s, name, ptr(self.arrays[name]))
        return s

    def to_device(self, device="cuda"):
        return DeviceTopology(self, device)


class DeviceTopology:
    """The same arrays in device memory with their ncg_hull_topology struct."""

    def __init__(self, host: HostTopology, device="cuda"):
        self.tensors = {}
        for name, dt, _, _ in _ARRAYS:
            a = host.arrays[name]
            t = torch.from_numpy(np.ascontiguousarray(a.view(np.int32) if dt == np.uint32 else a))
            self.tensors[name] = t.to(device)
        self.counts = dict(host.counts)
        self.struct = N.NcgHullTopology(**self.counts)
        for name, _, _, _ in _ARRAYS:
            t = self.tensors[name]
            setattr(self.struct, name, t.data_ptr() if t.numel() else None)
