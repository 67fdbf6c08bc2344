"""Shapes, isometries and the packed pair batch that crosses the C ABI.

The shape structs mirror ncollide3d's support-map shapes
(src/shape/{ball,cuboid,capsule,cone,cylinder,convex}.rs) and the packed
records mirror ``ncg_shape`` / ``ncg_pose`` in include/ncg.h: 32-byte shape
records, 32-byte poses (quaternion i j k w, translation, pad) and one flat
float4 array of hull points shared by all convex hulls.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BALL, CUBOID, CAPSULE, CONE, CYLINDER, CONVEX_HULL = 0, 1, 2, 3, 4, 5
KIND_NAMES = {BALL: "Ball", CUBOID: "Cuboid", CAPSULE: "Capsule", CONE: "Cone",
              CYLINDER: "Cylinder", CONVEX_HULL: "ConvexHull"}

SHAPE_DTYPE = np.dtype([("kind", "<u4"), ("hull_off", "<u4"), ("hull_n", "<u4"),
                        ("pad", "<u4"), ("p", "<f4", (4,))], align=True)
assert SHAPE_DTYPE.itemsize == 32
CONTACT_DTYPE = np.dtype([("world1", "<f4", (3,)), ("world2", "<f4", (3,)),
                          ("normal", "<f4", (3,)), ("depth", "<f4")])
assert CONTACT_DTYPE.itemsize == 40


@dataclass
class Ball:
    """ncollide3d::shape::Ball (src/shape/ball.rs)."""
    radius: float
    kind = BALL

    def params(self):
        return (self.radius, 0.0, 0.0, 0.0)

    def circumradius(self):
        return float(self.radius)


@dataclass
class Cuboid:
    """ncollide3d::shape::Cuboid (src/shape/cuboid.rs) given by its half extents."""
    half_extents: tuple
    kind = CUBOID

    def params(self):
        hx, hy, hz = self.half_extents
        return (hx, hy, hz, 0.0)

    def circumradius(self):
        return float(np.linalg.norm(self.half_extents))


@dataclass
class Capsule:
    """ncollide3d::shape::Capsule (src/shape/capsule.rs), axis y."""
    half_height: float
    radius: float
    kind = CAPSULE

    def params(self):
        return (self.half_height, self.radius, 0.0, 0.0)

    def circumradius(self):
        return float(self.half_height + self.radius)


@dataclass
class Cone:
    """ncollide3d::shape::Cone (src/shape/cone.rs), apex at +y."""
    half_height: float
    radius: float
    kind = CONE

    def params(self):
        return (self.half_height, self.radius, 0.0, 0.0)

    def circumradius(self):
        return float(np.hypot(self.half_height, self.radius))


@dataclass
class Cylinder:
    """ncollide3d::shape::Cylinder (src/shape/cylinder.rs), axis y."""
    half_height: float
    radius: float
    kind = CYLINDER

    def params(self):
        return (self.half_height, self.radius, 0.0, 0.0)

    def circumradius(self):
        return float(np.hypot(self.half_height, self.radius))


@dataclass
class ConvexHull:
    """ncollide3d::shape::ConvexHull (src/shape/convex.rs).

    Only the point set matters for the support map (convex.rs:418-423): the
    arg-max of <p, d> over the points equals the arg-max over the hull's
    vertices, so the sampled points are used as they are.
    """
    points: np.ndarray
    kind = CONVEX_HULL

    def params(self):
        return (0.0, 0.0, 0.0, 0.0)

    def circumradius(self):
        return float(np.sqrt((np.asarray(self.points, np.float64) ** 2).sum(1).max()))


def isometry(translation=(0.0, 0.0, 0.0), quaternion=(0.0, 0.0, 0.0, 1.0)):
    """Isometry3 packed as ncg_pose: (qi, qj, qk, qw, tx, ty, tz, 0)."""
    q = tuple(float(x) for x in quaternion)
    t = tuple(float(x) for x in translation)
    return np.array(q + t + (0.0,), dtype=np.float32)


@dataclass
class PairBatch:
    """A batch of pairs in the ncg_batch layout (host numpy arrays).

    shapes:      SHAPE_DTYPE records
    hull_points: float32 [P, 4]
    m1, m2:      float32 [N, 8] poses
    g1, g2:      uint32 [N] shape indices
    init_dir:    optional float32 [N, 3]
    scale:       float64 [N] length scale of each pair (sum of circumradii),
                 used to turn absolute errors into relative ones
    """
    shapes: np.ndarray
    hull_points: np.ndarray
    m1: np.ndarray
    g1: np.ndarray
    m2: np.ndarray
    g2: np.ndarray
    init_dir: np.ndarray | None = None
    scale: np.ndarray | None = None
    meta: dict = field(default_factory=dict)

    @property
    def n_pairs(self):
        return int(self.g1.shape[0])

    def subset(self, idx):
        idx = np.asarray(idx)
        return PairBatch(self.shapes, self.hull_points, self.m1[idx], self.g1[idx], self.m2[idx], self.g2[idx],
                         None if self.init_dir is None else self.init_dir[idx],
                         None if self.scale is None else self.scale[idx], dict(self.meta))

    def with_init_dir(self, init_dir):
        return PairBatch(self.shapes, self.hull_points, self.m1, self.g1, self.m2, self.g2,
                         None if init_dir is None else np.ascontiguousarray(init_dir, np.float32),
                         self.scale, dict(self.meta))

    def kinds(self):
        return self.shapes["kind"][self.g1], self.shapes["kind"][self.g2]

    def nbytes_inputs(self, include_hulls=True):
        b = self.m1.nbytes + self.m2.nbytes + self.g1.nbytes + self.g2.nbytes + self.shapes.nbytes
        if include_hulls:
            b += self.hull_points.nbytes
        if self.init_dir is not None:
            b += self.init_dir.nbytes
        return b


def pack_pairs(pairs):
    """Packs [(iso1, shape1, iso2, shape2), ...] with one shape record per use."""
    shapes, pts, m1, m2 = [], [], [], []
    n_pts = 0
    scale = []
    for (a, sa, b, sb) in pairs:
        for s in (sa, sb):
            rec = np.zeros((), SHAPE_DTYPE)
            rec["kind"] = s.kind
            rec["p"] = s.params()
            if s.kind == CONVEX_HULL:
                p = np.zeros((len(s.points), 4), np.float32)
                p[:, :3] = np.asarray(s.points, np.float32)
                rec["hull_off"] = n_pts
                rec["hull_n"] = len(p)
                pts.append(p)
                n_pts += len(p)
            shapes.append(rec)
        m1.append(np.asarray(a, np.float32))
        m2.append(np.asarray(b, np.float32))
        scale.append(sa.circumradius() + sb.circumradius())
    n = len(pairs)
    hull = np.concatenate(pts) if pts else np.zeros((1, 4), np.float32)
    return PairBatch(np.array(shapes, SHAPE_DTYPE), np.ascontiguousarray(hull),
                     np.ascontiguousarray(np.stack(m1)), np.arange(0, 2 * n, 2, dtype=np.uint32),
                     np.ascontiguousarray(np.stack(m2)), np.arange(1, 2 * n, 2, dtype=np.uint32),
                     scale=np.asarray(scale, np.float64))
