"""Seeded synthetic pair batches (the reference publishes no dataset).

Workloads, all f32:
  cuboid_pairs         65,536 Cuboid-Cuboid pairs (half extents U[0.1,1]^3)
  mixed_convex         1,048,576 pairs, kinds uniform over Ball, Cuboid,
                       Capsule, Cone, ConvexHull (n log-uniform in [8,1024],
                       ellipsoid samples with radial jitter U[0.95,1])
  precision_stress     the same mix with thin shapes and near-touching
                       placements (see ncollide_gb300.stress)
  coherent_hull_pairs  ConvexHull-ConvexHull pairs drawn from a pool of
                       shared hulls, moved by small steps frame to frame

Poses: rotations are normalised 4-D Gaussians, shape A's centre is uniform
in [-1,1]^3 and B's centre sits at d*(rA+rB) from A's along a uniform random
unit direction with d ~ U[0,1.2], r being each shape's circumradius, so
about half of the pairs intersect.
"""
from __future__ import annotations

import numpy as np

from .shapes import (BALL, CAPSULE, CONE, CONVEX_HULL, CUBOID, CYLINDER, SHAPE_DTYPE,
                     PairBatch)

MIXED_KINDS = (BALL, CUBOID, CAPSULE, CONE, CONVEX_HULL)


def random_unit_quaternions(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q  # (i, j, k, w)


def random_unit_vectors(rng, n):
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def log_uniform_int(rng, lo, hi, n):
    return np.clip(np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n))), lo, hi).astype(np.int64)


def _hull_points(rng, counts, semi_axes_lo=0.2, thin_axis=None, thin_scale=None):
    """Ellipsoid samples with radial jitter; one hull per entry of counts."""
    total = int(counts.sum())
    dirs = rng.standard_normal((total, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    dirs *= rng.uniform(0.95, 1.0, (total, 1))
    axes = rng.uniform(semi_axes_lo, 1.0, (len(counts), 3))
    if thin_axis is not None:
        axes[np.arange(len(counts)), thin_axis] *= thin_scale
    dirs *= np.repeat(axes, counts, axis=0)
    pts = np.zeros((total, 4), np.float32)
    pts[:, :3] = dirs
    return pts


def _circumradius(shapes, hull_points):
    kind = shapes["kind"]
    p = shapes["p"].astype(np.float64)
    r = np.zeros(len(shapes))
    r[kind == BALL] = p[kind == BALL, 0]
    m = kind == CUBOID
    r[m] = np.linalg.norm(p[m, :3], axis=1)
    m = kind == CAPSULE
    r[m] = p[m, 0] + p[m, 1]
    m = (kind == CONE) | (kind == CYLINDER)
    r[m] = np.hypot(p[m, 0], p[m, 1])
    hulls = np.nonzero(kind == CONVEX_HULL)[0]
    if len(hulls):
        sq = (hull_points[:, :3].astype(np.float64) ** 2).sum(1)
        off = shapes["hull_off"][hulls].astype(np.int64)
        cnt = shapes["hull_n"][hulls].astype(np.int64)
        # max over each contiguous slice
        order = np.argsort(off)
        starts = off[order]
        mx = np.maximum.reduceat(sq, starts) if len(starts) else np.zeros(0)
        # reduceat over sorted starts covers each hull's slice when slices tile the array
        rr = np.empty(len(hulls))
        rr[order] = np.sqrt(mx)
        assert np.all(cnt > 0)
        r[hulls] = rr
    return r


def random_shapes(rng, n, kinds=MIXED_KINDS, hull_n=(8, 1024), thin=False):
    """n shape records with kinds drawn uniformly from `kinds`."""
    kind = np.asarray(kinds, np.uint32)[rng.integers(0, len(kinds), n)]
    shapes = np.zeros(n, SHAPE_DTYPE)
    shapes["kind"] = kind
    p = np.zeros((n, 4), np.float64)
    m = kind == BALL
    p[m, 0] = rng.uniform(0.1, 1.0, m.sum())
    m = kind == CUBOID
    p[m, :3] = rng.uniform(0.1, 1.0, (m.sum(), 3))
    m = kind == CAPSULE
    p[m, 0] = rng.uniform(0.1, 1.0, m.sum())
    p[m, 1] = rng.uniform(0.05, 0.5, m.sum())
    m = (kind == CONE) | (kind == CYLINDER)
    p[m, 0] = rng.uniform(0.1, 1.0, m.sum())
    p[m, 1] = rng.uniform(0.1, 1.0, m.sum())
    hulls = np.nonzero(kind == CONVEX_HULL)[0]
    thin_axis = thin_scale = None
    if thin:
        s = np.exp(rng.uniform(np.log(1e-3), 0.0, n))
        ax = rng.integers(0, 3, n)
        m = kind == CUBOID
        p[m, ax[m]] *= s[m]
        m = (kind == CAPSULE) | (kind == CONE) | (kind == CYLINDER)
        # axis 0 -> half height, otherwise the radius
        p[m, np.where(ax[m] == 0, 0, 1)] *= s[m]
        thin_axis, thin_scale = ax[hulls], s[hulls]
    shapes["p"] = p.astype(np.float32)
    if len(hulls):
        counts = log_uniform_int(rng, hull_n[0], hull_n[1], len(hulls))
        pts = _hull_points(rng, counts, thin_axis=thin_axis, thin_scale=thin_scale)
        offs = np.concatenate([[0], np.cumsum(counts)[:-1]])
        shapes["hull_off"][hulls] = offs.astype(np.uint32)
        shapes["hull_n"][hulls] = counts.astype(np.uint32)
    else:
        pts = np.zeros((1, 4), np.float32)
    return shapes, pts


def _poses(rng, n, ra, rb, dmax=1.2):
    m1 = np.zeros((n, 8), np.float32)
    m2 = np.zeros((n, 8), np.float32)
    m1[:, :4] = random_unit_quaternions(rng, n)
    m2[:, :4] = random_unit_quaternions(rng, n)
    ta = rng.uniform(-1.0, 1.0, (n, 3))
    u = random_unit_vectors(rng, n)
    d = rng.uniform(0.0, dmax, (n, 1))
    m1[:, 4:7] = ta
    m2[:, 4:7] = ta + d * (ra + rb)[:, None] * u
    return m1, m2


def _pair_batch(shapes, pts, m1, m2, radii, meta):
    n = m1.shape[0]
    g1 = np.arange(0, 2 * n, 2, dtype=np.uint32)
    g2 = np.arange(1, 2 * n, 2, dtype=np.uint32)
    return PairBatch(shapes, np.ascontiguousarray(pts), m1, g1, m2, g2,
                     scale=radii[g1] + radii[g2], meta=meta)


def cuboid_pairs(n=65536, seed=0):
    """Cuboid-Cuboid pairs, half extents U[0.1,1]^3."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, 2 * n, kinds=(CUBOID,))
    radii = _circumradius(shapes, pts)
    m1, m2 = _poses(rng, n, radii[0::2], radii[1::2])
    return _pair_batch(shapes, pts, m1, m2, radii, {"workload": "cuboid_pairs", "n": n, "seed": seed})


def mixed_convex(n=1 << 20, seed=1, kinds=MIXED_KINDS, hull_n=(8, 1024), thin=False, dmax=1.2):
    """Mixed convex pairs with uneven costs (ConvexHull sizes 8..1024)."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, 2 * n, kinds=kinds, hull_n=hull_n, thin=thin)
    radii = _circumradius(shapes, pts)
    m1, m2 = _poses(rng, n, radii[0::2], radii[1::2], dmax=dmax)
    return _pair_batch(shapes, pts, m1, m2, radii,
                       {"workload": "mixed_convex", "n": n, "seed": seed, "thin": thin})


def mixed_convex_pooled(n=1 << 22, seed=3, pool=1 << 17, kinds=MIXED_KINDS, hull_n=(8, 1024)):
    """The mixed convex distribution over a pool of `pool` shared shapes: both
    shapes of a pair are drawn uniformly from the pool (so pair kinds stay
    uniform), poses as in mixed_convex.  Keeps multi-million-pair training and
    evaluation sets to a few hundred MB of hull points."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, pool, kinds=kinds, hull_n=hull_n)
    radii = _circumradius(shapes, pts)
    g1 = rng.integers(0, pool, n).astype(np.uint32)
    g2 = rng.integers(0, pool, n).astype(np.uint32)
    m1, m2 = _poses(rng, n, radii[g1], radii[g2])
    return PairBatch(shapes, pts, m1, g1, m2, g2, scale=radii[g1] + radii[g2],
                     meta={"workload": "mixed_convex_pooled", "n": n, "seed": seed, "pool": pool})


def coherent_hull_pairs(n=1 << 24, seed=5, pool=1 << 16, hull_n=(32, 1024)):
    """ConvexHull-ConvexHull pairs over a pool of `pool` shared hulls."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, pool, kinds=(CONVEX_HULL,), hull_n=hull_n)
    radii = _circumradius(shapes, pts)
    g1 = rng.integers(0, pool, n).astype(np.uint32)
    g2 = rng.integers(0, pool, n).astype(np.uint32)
    m1, m2 = _poses(rng, n, radii[g1], radii[g2])
    return PairBatch(shapes, pts, m1, g1, m2, g2, scale=radii[g1] + radii[g2],
                     meta={"workload": "coherent_hull_pairs", "n": n, "seed": seed, "pool": pool})


def _quat_mul(a, b):
    ai, aj, ak, aw = a[:, 0], a[:, 1], a[:, 2], a[:, 3]
    bi, bj, bk, bw = b[:, 0], b[:, 1], b[:, 2], b[:, 3]
    return np.stack([aw * bi + ai * bw + aj * bk - ak * bj,
                     aw * bj - ai * bk + aj * bw + ak * bi,
                     aw * bk + ai * bj - aj * bi + ak * bw,
                     aw * bw - ai * bi - aj * bj - ak * bk], axis=1)


def advance_frame(batch, rng, sigma_t=0.01, sigma_r=0.02):
    """One frame of coherent motion: every pose gets a translation step
    N(0, sigma_t^2) per axis and a rotation about a random axis by N(0, sigma_r^2)."""
    out = []
    for m in (batch.m1, batch.m2):
        n = m.shape[0]
        m = m.copy()
        ax = random_unit_vectors(rng, n)
        ang = rng.normal(0.0, sigma_r, n)
        dq = np.concatenate([ax * np.sin(ang / 2)[:, None], np.cos(ang / 2)[:, None]], axis=1)
        q = _quat_mul(dq, m[:, :4].astype(np.float64))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        m[:, :4] = q
        m[:, 4:7] += rng.normal(0.0, sigma_t, (n, 3))
        out.append(m)
    return PairBatch(batch.shapes, batch.hull_points, out[0], batch.g1, out[1], batch.g2,
                     batch.init_dir, batch.scale, dict(batch.meta))


def toi_sweeps(n=1 << 20, seed=7, kinds=MIXED_KINDS, hull_n=(8, 1024), dmax=3.0, cone_deg=30.0):
    """Linear sweeps for the time of impact: mixed convex pairs placed up to
    dmax times their summed circumradii apart, the first shape moving towards
    the second within a cone of half-angle cone_deg at speed U[0.5, 2] x the
    summed circumradii, the second drifting at a tenth of that.  Returns
    (batch, vel1 [n,3], vel2 [n,3])."""
    b = mixed_convex(n, seed=seed, kinds=kinds, hull_n=hull_n, dmax=dmax)
    b.meta.update({"workload": "toi_sweeps", "dmax": dmax, "cone_deg": cone_deg})
    rng = np.random.default_rng(seed + 7919)
    d = (b.m2[:, 4:7] - b.m1[:, 4:7]).astype(np.float64)
    dn = np.linalg.norm(d, axis=1, keepdims=True)
    d = np.where(dn > 0, d / np.maximum(dn, 1e-30), random_unit_vectors(rng, n))
    jitter = random_unit_vectors(rng, n)
    jitter -= (jitter * d).sum(1, keepdims=True) * d
    jn = np.linalg.norm(jitter, axis=1, keepdims=True)
    jitter = jitter / np.maximum(jn, 1e-30)
    ang = np.radians(cone_deg) * np.sqrt(rng.uniform(0.0, 1.0, (n, 1)))
    aim = d * np.cos(ang) + jitter * np.sin(ang)
    speed = rng.uniform(0.5, 2.0, (n, 1)) * b.scale[:, None]
    vel1 = (aim * speed).astype(np.float32)
    vel2 = (random_unit_vectors(rng, n) * speed * 0.1).astype(np.float32)
    return b, vel1, vel2


def ray_casts(n=1 << 20, seed=9, kinds=(BALL, CUBOID, CAPSULE, CONE, CYLINDER, CONVEX_HULL), hull_n=(8, 1024),
              inside=0.1, cone_deg=20.0):
    """Rays against single shapes: shape i at a random pose, the ray starting
    at 1.5 to 4 circumradii from its centre (a fraction `inside` of the rays
    start at the centre) and aimed at the centre within a cone of half-angle
    cone_deg; |dir| in [0.5, 2].  Returns (batch, rays [n,6]); the batch's m2/g2
    repeat m1/g1 and are unused."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, n, kinds=kinds, hull_n=hull_n)
    radii = _circumradius(shapes, pts)
    m1 = np.zeros((n, 8), np.float32)
    m1[:, :4] = random_unit_quaternions(rng, n)
    m1[:, 4:7] = rng.uniform(-1.0, 1.0, (n, 3))
    g1 = np.arange(n, dtype=np.uint32)
    u = random_unit_vectors(rng, n)
    dist = rng.uniform(1.5, 4.0, (n, 1)) * radii[:, None]
    dist[rng.uniform(0.0, 1.0, n) < inside] = 0.0
    origin = m1[:, 4:7].astype(np.float64) + u * dist
    jitter = random_unit_vectors(rng, n)
    jitter -= (jitter * u).sum(1, keepdims=True) * u
    jitter /= np.maximum(np.linalg.norm(jitter, axis=1, keepdims=True), 1e-30)
    ang = np.radians(cone_deg) * np.sqrt(rng.uniform(0.0, 1.0, (n, 1)))
    aim = -u * np.cos(ang) + jitter * np.sin(ang)
    rays = np.concatenate([origin, aim * rng.uniform(0.5, 2.0, (n, 1))], 1).astype(np.float32)
    b = PairBatch(shapes, np.ascontiguousarray(pts), m1, g1, m1.copy(), g1.copy(), scale=radii,
                  meta={"workload": "ray_casts", "n": n, "seed": seed})
    return b, rays


def scene_objects(n=1 << 20, seed=11, kinds=(BALL, CUBOID, CAPSULE, CONE, CYLINDER, CONVEX_HULL),
                  hull_n=(8, 256), overlaps=4.0):
    """A scene for the broad phase: n shapes with the mixed size distribution
    at uniform random poses in a cube sized so that an object's AABB meets
    about `overlaps` others.  Returns a batch whose pair i is object i alone
    (m1, g1 = its pose and shape; m2, g2 repeat them, unused)."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, n, kinds=kinds, hull_n=hull_n)
    radii = _circumradius(shapes, pts)
    # boxes of side ~2r: a pair overlaps when centres are within ~(r_a + r_b) per axis
    mean_side = float(np.mean(2.0 * radii))
    side = (n * (2.0 * mean_side) ** 3 / max(overlaps, 1e-6)) ** (1.0 / 3.0)
    m1 = np.zeros((n, 8), np.float32)
    m1[:, :4] = random_unit_quaternions(rng, n)
    m1[:, 4:7] = rng.uniform(-side / 2, side / 2, (n, 3))
    g1 = np.arange(n, dtype=np.uint32)
    return PairBatch(shapes, np.ascontiguousarray(pts), m1, g1, m1.copy(), g1.copy(), scale=radii,
                     meta={"workload": "scene_objects", "n": n, "seed": seed, "side": side})


def cuboid_stacks(n=1 << 18, seed=13, tilt_deg=5.0, gap=0.05):
    """Cuboid pairs resting on each other (the manifold generator's face-face
    case): B above A along A's y axis with a random yaw, a tilt up to tilt_deg
    and a vertical gap or penetration in [-gap, gap]; A at a random pose."""
    rng = np.random.default_rng(seed)
    shapes = np.zeros(2 * n, SHAPE_DTYPE)
    shapes["kind"] = CUBOID
    shapes["p"][:, :3] = rng.uniform(0.1, 1.0, (2 * n, 3))
    ha, hb = shapes["p"][0::2, :3].astype(np.float64), shapes["p"][1::2, :3].astype(np.float64)
    qa = random_unit_quaternions(rng, n).astype(np.float64)
    yaw = rng.uniform(-np.pi, np.pi, n)
    q_yaw = np.stack([np.zeros(n), np.sin(yaw / 2), np.zeros(n), np.cos(yaw / 2)], 1)
    ax = random_unit_vectors(rng, n)
    tilt = np.radians(tilt_deg) * rng.uniform(0.0, 1.0, n)
    q_tilt = np.concatenate([ax * np.sin(tilt / 2)[:, None], np.cos(tilt / 2)[:, None]], 1)
    qb_rel = _quat_mul(q_tilt, q_yaw)
    qb = _quat_mul(qa, qb_rel)
    qb /= np.linalg.norm(qb, axis=1, keepdims=True)
    up = _rotate(qa, np.tile([0.0, 1.0, 0.0], (n, 1)))
    slide = rng.uniform(-0.5, 0.5, (n, 2)) * np.minimum(ha[:, [0, 2]], hb[:, [0, 2]])
    side = _rotate(qa, np.stack([slide[:, 0], np.zeros(n), slide[:, 1]], 1))
    ta = rng.uniform(-1.0, 1.0, (n, 3))
    tb = ta + up * (ha[:, 1:2] + hb[:, 1:2] + rng.uniform(-gap, gap, (n, 1))) + side
    m1 = np.zeros((n, 8), np.float32)
    m2 = np.zeros((n, 8), np.float32)
    m1[:, :4], m1[:, 4:7] = qa, ta
    m2[:, :4], m2[:, 4:7] = qb, tb
    g1 = np.arange(0, 2 * n, 2, dtype=np.uint32)
    radii = np.linalg.norm(shapes["p"][:, :3], axis=1)
    return PairBatch(shapes, np.zeros((1, 4), np.float32), m1, g1, m2, g1 + 1, scale=radii[0::2] + radii[1::2],
                     meta={"workload": "cuboid_stacks", "n": n, "seed": seed})


def _rotate(q, v):
    qv = q[:, :3]
    t = 2.0 * np.cross(qv, v)
    return v + q[:, 3:4] * t + np.cross(qv, t)


def hull_pairs_pooled(n=1 << 18, seed=17, pool=4096, hull_n=(8, 256), kinds=(CUBOID, CONVEX_HULL), dmax=1.0):
    """ConvexHull and Cuboid pairs over a pool of shared shapes (the hulls'
    face topology is built once per pool shape): the manifold generator's
    polyhedron pairs, poses as in mixed_convex with d ~ U[0, dmax]."""
    rng = np.random.default_rng(seed)
    shapes, pts = random_shapes(rng, pool, kinds=kinds, hull_n=hull_n)
    radii = _circumradius(shapes, pts)
    g1 = rng.integers(0, pool, n).astype(np.uint32)
    g2 = rng.integers(0, pool, n).astype(np.uint32)
    m1, m2 = _poses(rng, n, radii[g1], radii[g2], dmax=dmax)
    return PairBatch(shapes, pts, m1, g1, m2, g2, scale=radii[g1] + radii[g2],
                     meta={"workload": "hull_pairs_pooled", "n": n, "seed": seed, "pool": pool})
