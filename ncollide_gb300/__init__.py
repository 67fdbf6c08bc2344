"""ncollide_gb300 — batched convex narrow phase (GJK + EPA) for GB300.

The drop-in boundary is the C ABI in include/ncg.h (libncg.so, built in-tree
by ncollide_gb300.build).  This package adds the Python host side: shape and
pose packing (shapes), seeded workloads (workloads) and the batched query
functions over device tensors (query).
"""
from .shapes import (BALL, CAPSULE, CONE, CONVEX_HULL, CUBOID, CYLINDER, Ball, Capsule, Cone, ConvexHull, Cuboid,
                     Cylinder, PairBatch, isometry, pack_pairs)

__all__ = ["BALL", "CUBOID", "CAPSULE", "CONE", "CYLINDER", "CONVEX_HULL", "Ball", "Cuboid", "Capsule", "Cone",
           "Cylinder", "ConvexHull", "PairBatch", "isometry", "pack_pairs"]
