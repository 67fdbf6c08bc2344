// ncg_toi.cuh — device side of the linear time of impact: the GJK ray cast on
// the Minkowski difference of two support maps (optionally with the first
// shape dilated by the target distance) and the analytic Ball-Ball case.
//
// Same arithmetic split as the GJK loop (ncg_core.cuh): support points, the
// ray origin and the CSO points in f32; the simplex sub-solve, the ray
// parameter, the bounds and the search direction in double-word.
//
// Reference (ncollide 0.33):
//   src/query/algorithms/gjk.rs:196-345            directional_distance, minkowski_ray_cast
//   src/query/ray/ray_plane.rs:9-39                line_toi_with_plane, ray_toi_with_plane
//   src/query/algorithms/special_support_maps.rs:32-59   DilatedShape
//   src/shape/ball.rs:36-48, capsule.rs:72-84, support_map.rs:18-35   support_point_toward
//   src/query/time_of_impact/time_of_impact_support_map_support_map.rs:10-127
//   src/query/time_of_impact/time_of_impact_ball_ball.rs:9-62, src/query/ray/ray_ball.rs:77-121
//   src/query/time_of_impact/time_of_impact.rs:63-90 (Ball-Ball dispatch)
//   src/query/ray/ray_support_map.rs:14-56 and the RayCast impls :58-110,
//   src/query/algorithms/gjk.rs:180-194 (cast_ray)  ray casts on support maps
#pragma once

#include "ncg_core.cuh"

namespace ncg {

enum { TOI_OUT_OF_ITERATIONS = 0, TOI_CONVERGED = 1, TOI_FAILED = 2, TOI_PENETRATING = 3 };

struct ToiResult {
    bool some;
    real toi;
    vec3<float> w1, w2, n1, n2;  // the shapes' local frames
    int status;
};

// The first shape's support point: support_point(m, s, d), or with `toward`
// SupportMap::support_point_toward(m, s, d) for a unit d (Ball and Capsule
// use d as given; the other shapes go through local_support_point).  One
// inlined support switch serves both.
template <class Scan>
NCG_DEV vec3<float> support_point_ex(const Pose& m, const Shape& s, vec3<float> d, bool toward, const Scan& scan) {
    if (s.kind == KIND_CONSTANT_ORIGIN) return zero3<float>();
    if (s.kind == NCG_BALL) {
        vec3<float> u = toward ? d : d / vnorm(d);
        return m.t + u * s.p0;
    }
    vec3<float> l = qrot_inv(m.q, d);
    if (toward && s.kind == NCG_CAPSULE) {
        vec3<float> r{0.0f, copysignf(s.p0, l.y), 0.0f};
        return qrot(m.q, r + l * s.p1) + m.t;
    }
    return qrot(m.q, local_support(s, l, scan)) + m.t;
}

// CSOPoint::from_shapes with the first shape optionally a DilatedShape:
// its support point is support_point_toward(normalize(d)) + normalize(d) * r.
template <class Scan>
NCG_DEV CSO cso_dilated(const PairGeom& g, float radius, bool dilated, vec3<float> d, const Scan& scan) {
    vec3<float> u = d;
    if (dilated) u = d / vnorm(d);
    vec3<float> a = support_point_ex(g.m1, g.g1, u, dilated, scan);
    if (dilated) a = a + u * radius;
    vec3<float> b = support_point(g.m2, g.g2, -d, scan);
    return CSO{a - b, a, b};
}

// ray_toi_with_plane over line_toi_with_plane; relative_eq!(denom, 0) is |denom| <= eps.
NCG_DEV bool ray_toi_with_plane(vec3<real> center, vec3<real> normal, vec3<real> orig, vec3<real> dir, real eps,
                                real& t) {
    vec3<real> dpos = center - orig;
    real denom = dot(normal, dir);
    if (fabs(denom) <= eps) return false;
    real tt = dot(normal, dpos) / denom;
    if (tt >= real(0.0f)) {
        t = tt;
        return true;
    }
    return false;
}

struct RayHit {
    bool hit;
    real toi;
    vec3<real> normal;
};

// minkowski_ray_cast of the ray (origin0, ray_dir) against m1 * g1 - m2 * g2
// (None past max_toi).  `iters` counts loop entries.  The loop is
// rotated so that the support mapping and the simplex sub-solve each have a
// single call site (the first pass takes the reference's initial support
// point and simplex reset): inlined twice they overflow the instruction cache.
template <class Scan>
NCG_DEV RayHit minkowski_ray_cast(const PairGeom& g, float radius, bool dilated, vec3<float> origin0,
                                  vec3<real> ray_dir, real max_toi, Simplex& sx, const Tol& tol, const Scan& scan,
                                  uint32_t& iters, uint32_t& status, int max_iter) {
    RayHit out;
    out.hit = false;
    out.toi = real(0.0f);
    out.normal = zero3<real>();
    const real eps = from_host(tol.eps), eps_tol = from_host(tol.eps_tol), eps_rel = from_host(tol.eps_rel);
    const real ray_length = vnorm(ray_dir);
    if (ray_length <= eps) return out;
    real ltoi = real(0.0f);
    vec3<float> origin = origin0;
    const vec3<real> rdir = ray_dir / ray_length;
    vec3<real> dir = -rdir;
    vec3<real> ldir = dir;
    vec3<real> proj = zero3<real>();
    real max_bound = dw_max(), old_max_bound = dw_max();
    bool last_chance = false, first = true;
    int niter = 0;
    for (;;) {
        CSO c;
        if (!first && max_bound >= old_max_bound) {
            // upper-bound inconsistency: the projection itself is the support point
            last_chance = true;
            vec3<float> p = to_f(proj + to_r(origin));
            c = CSO{p, p, zero3<float>()};
        } else {
            c = cso_dilated(g, radius, dilated, to_f(dir), scan);
        }
        real min_bound = real(0.0f);
        if (!first) {
            if (last_chance && ltoi > real(0.0f)) { out.hit = true; out.toi = ltoi / ray_length; out.normal = ldir; return out; }
            real t;
            if (ray_toi_with_plane(to_r(c.p), dir, to_r(origin), rdir, eps, t)) {
                if (dot(dir, rdir) < real(0.0f) && t > real(0.0f)) {
                    // a new lower bound: the ray origin moves
                    ldir = dir;
                    ltoi = ltoi + t;
                    if (ltoi / ray_length > max_toi) return out;
                    const vec3<float> shift = to_f(rdir * t);
                    origin = origin + shift;
                    max_bound = dw_max();
                    for (int k = 0; k <= sx.dim; ++k) sx.v[k].p = sx.v[k].p - shift;
                    last_chance = false;
                }
            } else if (dot(dir, rdir) > eps_tol) {
                return out;  // the ray misses
            }
            if (last_chance) return out;
            min_bound = -dot(dir, to_r(c.p) - to_r(origin));
            if (min_bound != min_bound) status |= NCG_STATUS_BAD_INPUT;
            if (max_bound - min_bound <= eps_rel * max_bound) return out;
        }
        c.p = c.p - origin;
        if (first) sx.reset(c);
        else (void)sx.add_point(c, tol);
        proj = sx.project_origin_and_reduce(tol, status);
        if (!first) {
            if (sx.dim == 3) {
                if (min_bound >= eps_tol) return out;
                out.hit = true;
                out.toi = ltoi / ray_length;
                out.normal = ldir;
                return out;
            }
            niter += 1;
            if (niter == max_iter) {
                status |= NCG_STATUS_GJK_MAX_ITER;
                return out;
            }
        }
        first = false;
        iters++;
        old_max_bound = max_bound;
        vec3<real> u;
        real n;
        if (try_normalize(-proj, eps_tol, u, n)) { dir = u; max_bound = n; }
        else { out.hit = true; out.toi = ltoi / ray_length; out.normal = ldir; return out; }
    }
}

// time_of_impact_support_map_support_map.  max_toi and target_distance >= 0.
// With a dilated first shape and a toi of zero the result needs the closest
// points of the undilated shapes: `refine` is then set, `ref_dir` holds the
// world-space normal and toi_refine finishes the pair (a second pass, so that
// the GJK loop is not inlined next to the ray cast).
template <class Scan>
NCG_DEV ToiResult toi_support_map(const PairGeom& g, vec3<float> vel1, vec3<float> vel2, real max_toi, float target,
                                  const Tol& tol, const Scan& scan, uint32_t& iters, uint32_t& status, int max_iter,
                                  bool& refine, vec3<float>& ref_dir) {
    ToiResult o;
    o.some = false;
    o.toi = real(0.0f);
    o.w1 = o.w2 = o.n1 = o.n2 = zero3<float>();
    o.status = TOI_CONVERGED;
    refine = false;
    const vec3<float> dvel = vel2 - vel1;
    const bool dilated = target != 0.0f;
    Simplex sx;
    RayHit rc = minkowski_ray_cast(g, target, dilated, zero3<float>(), to_r(dvel), dw_max(), sx, tol, scan, iters,
                                   status, max_iter);
    if (!rc.hit) return o;
    // directional_distance: the witness points are the simplex's unless the toi is zero
    vec3<real> w1 = zero3<real>(), w2 = zero3<real>();
    if (!(rc.toi == real(0.0f))) gjk_result(sx, sx.dim == 3, w1, w2);
    if (rc.toi > max_toi) return o;
    o.some = true;
    o.toi = rc.toi;
    const vec3<float> nf = to_f(rc.normal);
    if (dilated && rc.toi == real(0.0f)) {
        refine = true;
        ref_dir = nf;
        return o;
    }
    o.n1 = qrot_inv(g.m1.q, nf);
    o.n2 = qrot_inv(g.m2.q, -nf);
    vec3<float> lw1 = qrot_inv(g.m1.q, to_f(w1) - g.m1.t);
    if (dilated) lw1 = lw1 - o.n1 * target;
    o.w1 = lw1;
    o.w2 = qrot_inv(g.m2.q, to_f(w2) - g.m2.t);
    o.status = dilated ? TOI_CONVERGED : (rc.toi == real(0.0f) ? TOI_PENETRATING : TOI_CONVERGED);
    return o;
}

// The zero-toi case of a dilated first shape: closest points of the undilated
// shapes within `target`, GJK started on the ray cast's normal nf (world
// frame).  The witness points of a zero toi are the origin.
template <class Scan>
NCG_DEV ToiResult toi_refine(const PairGeom& g, vec3<float> nf, float target, const Tol& tol, const Scan& scan,
                             uint32_t& iters, uint32_t& status, int max_iter) {
    ToiResult o;
    o.some = true;
    o.toi = real(0.0f);
    vec3<float> d;
    float dn;
    if (!try_normalize(nf, FLT_EPSILON, d, dn)) d = mk(1.0f, 0.0f, 0.0f);
    Simplex sx;
    sx.reset(cso_support(g, d, scan));
    GjkOut r = gjk(g, real(target), true, sx, tol, scan, iters, status, max_iter);
    const vec3<float> zf = zero3<float>();
    o.w2 = qrot_inv(g.m2.q, zf - g.m2.t);
    if (r.kind == GJK_CLOSEST_POINTS) {
        vec3<real> dp = r.p2 - r.p1;
        const vec3<float> nn = to_f(dp / vnorm(dp));
        o.n1 = qrot_inv(g.m1.q, nn);
        o.n2 = qrot_inv(g.m2.q, -nn);
        o.w1 = qrot_inv(g.m1.q, zf - g.m1.t);
        o.status = TOI_CONVERGED;
        return o;
    }
    o.n1 = qrot_inv(g.m1.q, nf);
    o.n2 = qrot_inv(g.m2.q, -nf);
    o.w1 = qrot_inv(g.m1.q, zf - g.m1.t) - o.n1 * target;
    o.status = r.kind == GJK_INTERSECTION ? TOI_PENETRATING : TOI_CONVERGED;
    return o;
}

// ray_toi_with_ball (solid, ray origin 0): 0 miss, 1 hit, 2 origin inside.
NCG_DEV int ray_toi_with_ball(vec3<real> center, real radius, vec3<real> dir, real& t) {
    const vec3<real> dcenter = -center;
    const real a = norm_sq(dir);
    const real b = dot(dcenter, dir);
    const real c = norm_sq(dcenter) - radius * radius;
    if (a == real(0.0f)) {
        if (c > real(0.0f)) return 0;
        t = real(0.0f);
        return 2;
    }
    if (c > real(0.0f) && b > real(0.0f)) return 0;
    const real delta = b * b - a * c;
    if (delta < real(0.0f)) return 0;
    const real tt = (-b - sqrt(delta)) / a;
    if (tt <= real(0.0f)) {
        t = real(0.0f);
        return 2;
    }
    t = tt;
    return 1;
}

// time_of_impact_ball_ball on the balls' centres, then the dispatcher's
// rotation of witnesses and normals into the balls' frames.
NCG_DEV ToiResult toi_ball_ball(const Pose& m1, vec3<float> vel1, float r1, const Pose& m2, vec3<float> vel2,
                                float r2, real max_toi, float target) {
    ToiResult o;
    o.some = false;
    o.toi = real(0.0f);
    o.w1 = o.w2 = o.n1 = o.n2 = zero3<float>();
    o.status = TOI_CONVERGED;
    const vec3<real> vel = to_r(vel1) - to_r(vel2);
    const real rsum = real(r1) + real(r2);
    const real radius = rsum + real(target);
    const vec3<real> center = to_r(m1.t) - to_r(m2.t);
    const vec3<real> dir = -vel;
    real toi;
    const int hit = ray_toi_with_ball(center, radius, dir, toi);
    if (!hit) return o;
    if (toi > max_toi) return o;
    o.some = true;
    o.toi = toi;
    const vec3<real> dpt = dir * toi - center;
    vec3<real> n1, n2, w1, w2;
    if (radius == real(0.0f)) {
        n1 = n2 = mk(real(1.0f), real(0.0f), real(0.0f));
        w1 = w2 = zero3<real>();
    } else {
        n1 = dpt / radius;
        n2 = -n1;
        w1 = n1 * real(r1);
        w2 = n2 * real(r2);
    }
    o.status = (hit == 2 && norm_sq(center) < rsum * rsum) ? TOI_PENETRATING : TOI_CONVERGED;
    o.w1 = qrot_inv(m1.q, to_f(w1));
    o.w2 = qrot_inv(m2.q, to_f(w2));
    o.n1 = qrot_inv(m1.q, to_f(n1));
    o.n2 = qrot_inv(m2.q, to_f(n2));
    return o;
}

// RayCast::toi_and_normal_with_ray of a support-map shape: the ray in the
// shape's local frame, gjk::cast_ray against (identity, g) - (identity,
// ConstantOrigin); with solid false and the origin inside, a second cast
// backwards from beyond the shape (the support distance along the ray +
// 0.001).  The normal is rotated back into the world frame.
struct RayResult {
    bool hit;
    real toi;
    vec3<float> normal;
};

template <class Scan>
NCG_DEV RayResult ray_cast_support_map(const Pose& m, const Shape& s, vec3<float> ro, vec3<float> rd, real max_toi,
                                       bool solid, const Tol& tol, const Scan& scan, uint32_t& iters,
                                       uint32_t& status, int max_iter) {
    RayResult o;
    o.hit = false;
    o.toi = real(0.0f);
    o.normal = zero3<float>();
    PairGeom g;
    g.m1 = Pose{make_float4(0.0f, 0.0f, 0.0f, 1.0f), zero3<float>()};
    g.g1 = s;
    g.m2 = g.m1;
    g.g2 = Shape{KIND_CONSTANT_ORIGIN, 0, 0, 0.0f, 0.0f, 0.0f};
    const vec3<float> lo = qrot_inv(m.q, ro - m.t);
    const vec3<float> ld = qrot_inv(m.q, rd);
    Simplex sx;
    // at most two casts; the second starts beyond the shape, looking back
    vec3<float> origin = lo, dir = ld;
    real cast_max = max_toi;
    float shift = 0.0f;
    for (int pass = 0; pass < 2; ++pass) {
        RayHit rc = minkowski_ray_cast(g, 0.0f, false, origin, to_r(dir), cast_max, sx, tol, scan, iters, status,
                                       max_iter);
        if (!rc.hit) return o;
        if (pass == 1) {
            const real toi = real(shift) - rc.toi;
            if (!(toi <= max_toi)) return o;
            o.hit = true;
            o.toi = toi;
            o.normal = qrot(m.q, to_f(rc.normal));
            return o;
        }
        if (solid || !(rc.toi == real(0.0f))) {
            o.hit = true;
            o.toi = rc.toi;
            o.normal = qrot(m.q, to_f(rc.normal));
            return o;
        }
        // the ray starts inside the shape
        const vec3<float> ndir = ld / vnorm(ld);
        const vec3<float> supp = support_point(g.m1, s, ndir, scan);
        const float eps = 0.001f;
        shift = dot(supp - lo, ndir) + eps;
        origin = lo + ndir * shift;
        dir = -ld;
        cast_max = real(shift + eps);
    }
    return o;
}

}  // namespace ncg
