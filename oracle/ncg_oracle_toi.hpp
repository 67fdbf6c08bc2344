// ncg_oracle_toi.hpp — TEST INFRASTRUCTURE ONLY: CPU restatement of the
// reference's linear time of impact for support-map shapes (the GJK ray cast
// on the Minkowski difference), with the same arithmetic templates as
// ncg_oracle.hpp: N for support points and their translations, S for the
// ray-cast bookkeeping and the simplex sub-solve.
//
// Reference (ncollide 0.33):
//   src/query/algorithms/gjk.rs:196-345            directional_distance, minkowski_ray_cast
//   src/query/ray/ray_plane.rs:9-39                line_toi_with_plane, ray_toi_with_plane
//   src/query/algorithms/special_support_maps.rs:32-59   DilatedShape
//   src/shape/ball.rs:36-48, capsule.rs:72-84, support_map.rs:18-35   support_point_toward
//   src/query/time_of_impact/time_of_impact_support_map_support_map.rs:10-127
//   src/query/time_of_impact/time_of_impact_ball_ball.rs:9-62, query/ray/ray_ball.rs:77-121
//   src/query/time_of_impact/time_of_impact.rs:63-90 (Ball-Ball dispatch)
//   src/query/ray/ray_support_map.rs:14-56 and the RayCast impls :58-110,
//   src/query/algorithms/gjk.rs:180-194 (cast_ray)  ray casts on support maps
#pragma once

#include "ncg_oracle.hpp"

namespace ncgo {

enum TOIStatusCode { TOI_OUT_OF_ITERATIONS = 0, TOI_CONVERGED = 1, TOI_FAILED = 2, TOI_PENETRATING = 3 };

template <class S> struct TOIOut {
    bool some = false;
    S toi = S(0);
    V3<S> w1, w2, n1, n2;  // local frames of the shapes
    int status = TOI_CONVERGED;
};

// SupportMap::support_point_toward with a unit direction: Ball (ball.rs:36-38)
// and Capsule (capsule.rs:79-84) use it without normalising again; the other
// shapes fall back on local_support_point (support_map.rs:18-20, 32-35).
template <class N> inline V3<N> support_point_toward(const Iso<N>& m, const Shape<N>& s, V3<N> u, Counters* c) {
    if (c) c->support_calls++;
    if (s.kind == CONSTANT_ORIGIN) return zero3<N>();
    if (s.kind == BALL) return m.t + u * s.p0;
    V3<N> local = inverse_transform_vector(m, u);
    if (s.kind == CAPSULE) {
        V3<N> res{N(0), std::copysign(s.p0, local.y), N(0)};
        return transform_point(m, res + local * s.p1);
    }
    return transform_point(m, local_support_point(s, local, c));
}

// CSOPoint::from_shapes with g1 optionally dilated by `radius`
// (DilatedShape::support_point: support_point_toward(m, normalize(dir)) + u r).
template <class N>
inline CSOPoint<N> cso_dilated(const Iso<N>& m1, const Shape<N>& g1, N radius, bool dilated, const Iso<N>& m2,
                               const Shape<N>& g2, V3<N> dir, Counters* c) {
    V3<N> sp1;
    if (dilated) {
        V3<N> u = dir / norm(dir);
        sp1 = support_point_toward(m1, g1, u, c) + u * radius;
    } else {
        sp1 = support_point(m1, g1, dir, c);
    }
    V3<N> sp2 = support_point(m2, g2, -dir, c);
    return CSOPoint<N>{sp1 - sp2, sp1, sp2};
}

// ray_toi_with_plane (ray_plane.rs:27-39) over line_toi_with_plane (:9-23);
// relative_eq!(denom, 0) is |denom| <= eps.
template <class S> inline bool ray_toi_with_plane(V3<S> center, V3<S> normal, V3<S> orig, V3<S> dir, S eps, S* t) {
    V3<S> dpos = center - orig;
    S denom = dot(normal, dir);
    if ((denom < S(0) ? -denom : denom) <= eps) return false;
    S tt = dot(normal, dpos) / denom;
    if (tt >= S(0)) {
        *t = tt;
        return true;
    }
    return false;
}

template <class S> struct RayCastOut {
    bool hit = false;
    S toi = S(0);
    V3<S> normal;
};

// minkowski_ray_cast (gjk.rs:226-345) of the ray (ray_origin, ray_dir) against
// m1 * g1 - m2 * g2.  The ray origin and the simplex points move in N (the
// CSO point arithmetic); the bounds, the ray parameter and the direction in S.
template <class N, class S>
RayCastOut<S> minkowski_ray_cast(const Iso<N>& m1, const Shape<N>& g1, N radius, bool dilated, const Iso<N>& m2,
                                 const Shape<N>& g2, V3<N> ray_origin, V3<S> ray_dir, S max_toi,
                                 VoronoiSimplex<N, S>& simplex, const Tol<S>& tol, Counters* cnt) {
    RayCastOut<S> out;
    const S ray_length = norm(ray_dir);
    if (ray_length <= tol.eps) return out;  // relative_eq!(ray_length, 0) (a norm is >= 0)
    S ltoi = S(0);
    V3<N> origin = ray_origin;
    const V3<S> rdir = ray_dir / ray_length;
    V3<S> dir = -rdir;
    V3<S> ldir = dir;
    CSOPoint<N> sp = cso_dilated(m1, g1, radius, dilated, m2, g2, cvt<N>(dir), cnt);
    sp.point = sp.point - origin;
    simplex.reset(sp);
    V3<S> proj = simplex.project_origin_and_reduce(tol, cnt);
    S max_bound = std::numeric_limits<S>::max();
    bool last_chance = false;
    int niter = 0;
    for (;;) {
        if (cnt) cnt->gjk_iters++;
        const S old_max_bound = max_bound;
        {
            V3<S> u;
            S n;
            if (try_normalize(-proj, tol.eps_tol, &u, &n)) { dir = u; max_bound = n; }
            else { out.hit = true; out.toi = ltoi / ray_length; out.normal = ldir; return out; }
        }
        CSOPoint<N> support;
        if (max_bound >= old_max_bound) {
            // upper-bound inconsistency: the projection is the support point (CSOPoint::single_point)
            last_chance = true;
            V3<N> p = cvt<N>(proj + cvt<S>(origin));
            support = CSOPoint<N>{p, p, zero3<N>()};
        } else {
            support = cso_dilated(m1, g1, radius, dilated, m2, g2, cvt<N>(dir), cnt);
        }
        if (last_chance && ltoi > S(0)) { out.hit = true; out.toi = ltoi / ray_length; out.normal = ldir; return out; }
        S t;
        if (ray_toi_with_plane(cvt<S>(support.point), dir, cvt<S>(origin), rdir, tol.eps, &t)) {
            if (dot(dir, rdir) < S(0) && t > S(0)) {
                // new lower bound: move the origin
                ldir = dir;
                ltoi = ltoi + t;
                if (ltoi / ray_length > max_toi) return out;
                const V3<N> shift = cvt<N>(rdir * t);
                origin = origin + shift;
                max_bound = std::numeric_limits<S>::max();
                for (int i = 0; i <= simplex.dim; ++i) simplex.vertices[i].point = simplex.vertices[i].point - shift;
                last_chance = false;
            }
        } else if (dot(dir, rdir) > tol.eps_tol) {
            return out;  // miss
        }
        if (last_chance) return out;
        const S min_bound = -dot(dir, cvt<S>(support.point) - cvt<S>(origin));
        if (min_bound != min_bound) { if (cnt) cnt->status |= ST_BAD_INPUT; }  // assert at :324
        if (max_bound - min_bound <= tol.eps_rel * max_bound) return out;
        support.point = support.point - origin;
        (void)simplex.add_point(support, tol);
        proj = simplex.project_origin_and_reduce(tol, cnt);
        if (simplex.dim == 3) {
            if (min_bound >= tol.eps_tol) return out;
            out.hit = true;
            out.toi = ltoi / ray_length;
            out.normal = ldir;
            return out;
        }
        niter += 1;
        if (niter == 10000) { if (cnt) cnt->status |= ST_GJK_MAX_ITER; return out; }
    }
}

// time_of_impact_support_map_support_map (time_of_impact_support_map_support_map.rs:10-127).
// The local-frame outputs are computed in N from the S results.
template <class N, class S>
TOIOut<S> toi_support_map(const Iso<N>& m1, V3<N> vel1, const Shape<N>& g1, const Iso<N>& m2, V3<N> vel2,
                          const Shape<N>& g2, S max_toi, N target_distance, const Tol<S>& tol, Counters* cnt) {
    TOIOut<S> o;
    const V3<N> dvel = vel2 - vel1;
    const bool dilated = target_distance != N(0);
    VoronoiSimplex<N, S> simplex;
    RayCastOut<S> rc = minkowski_ray_cast(m1, g1, target_distance, dilated, m2, g2, zero3<N>(), cvt<S>(dvel),
                                          std::numeric_limits<S>::max(), simplex, tol, cnt);
    if (!rc.hit) return o;
    // directional_distance (gjk.rs:196-224): witnesses unless the toi is zero
    V3<S> w1 = zero3<S>(), w2 = zero3<S>();
    if (!(rc.toi == S(0))) gjk_result(simplex, simplex.dim == 3, &w1, &w2);
    if (rc.toi > max_toi) return o;
    o.some = true;
    o.toi = rc.toi;
    V3<S> normal = rc.normal;
    int status = TOI_CONVERGED;
    if (dilated && rc.toi == S(0)) {
        // closest points of the undilated shapes within target_distance, from the normal
        V3<N> nd = cvt<N>(normal);
        QueryOut<S> cp = closest_points<N, S>(m1, g1, m2, g2, S(target_distance), &nd, tol, cnt);
        if (cp.gjk_kind == GJK_CLOSEST_POINTS) {
            V3<S> d = cp.p2 - cp.p1;
            V3<S> nn = d / norm(d);
            const V3<N> nN = cvt<N>(nn);
            o.n1 = cvt<S>(inverse_transform_vector(m1, nN));
            o.n2 = cvt<S>(inverse_transform_vector(m2, -nN));
            o.w1 = cvt<S>(inverse_transform_vector(m1, cvt<N>(w1) - m1.t));
            o.w2 = cvt<S>(inverse_transform_vector(m2, cvt<N>(w2) - m2.t));
            o.status = TOI_CONVERGED;
            return o;
        }
        if (cp.gjk_kind == GJK_INTERSECTION) status = TOI_PENETRATING;
    } else if (!dilated) {
        status = rc.toi == S(0) ? TOI_PENETRATING : TOI_CONVERGED;
    }
    const V3<N> nN = cvt<N>(normal);
    const V3<N> n1 = inverse_transform_vector(m1, nN);
    o.n1 = cvt<S>(n1);
    o.n2 = cvt<S>(inverse_transform_vector(m2, -nN));
    V3<N> lw1 = inverse_transform_vector(m1, cvt<N>(w1) - m1.t);
    if (dilated) lw1 = lw1 - n1 * target_distance;
    o.w1 = cvt<S>(lw1);
    o.w2 = cvt<S>(inverse_transform_vector(m2, cvt<N>(w2) - m2.t));
    o.status = status;
    return o;
}

// ray_toi_with_ball (ray_ball.rs:77-121), solid, ray origin at 0.
template <class S> inline int ray_toi_with_ball(V3<S> center, S radius, V3<S> dir, S* t) {
    using std::sqrt;
    const V3<S> dcenter = -center;
    const S a = norm_sq(dir);
    const S b = dot(dcenter, dir);
    const S c = norm_sq(dcenter) - radius * radius;
    if (a == S(0)) {
        if (c > S(0)) return 0;
        *t = S(0);
        return 2;  // inside
    }
    if (c > S(0) && b > S(0)) return 0;
    const S delta = b * b - a * c;
    if (delta < S(0)) return 0;
    const S tt = (-b - sqrt(delta)) / a;
    if (tt <= S(0)) {
        *t = S(0);
        return 2;
    }
    *t = tt;
    return 1;
}

// time_of_impact_ball_ball (time_of_impact_ball_ball.rs:9-62) in S, and the
// dispatcher's rotation of the results into the balls' frames
// (time_of_impact.rs:63-90).
template <class N, class S>
TOIOut<S> toi_ball_ball(const Iso<N>& m1, V3<N> vel1, N r1, const Iso<N>& m2, V3<N> vel2, N r2, S max_toi,
                        N target_distance) {
    TOIOut<S> o;
    const V3<S> vel = cvt<S>(vel1) - cvt<S>(vel2);
    const S rsum = S(r1) + S(r2);
    const S radius = rsum + S(target_distance);
    const V3<S> center = cvt<S>(m1.t) - cvt<S>(m2.t);
    const V3<S> dir = -vel;
    S toi;
    const int hit = ray_toi_with_ball(center, radius, dir, &toi);
    if (!hit) return o;
    if (toi > max_toi) return o;
    o.some = true;
    o.toi = toi;
    const V3<S> dpt = dir * toi - center;
    V3<S> n1, n2, w1, w2;
    if (radius == S(0)) {
        n1 = n2 = v3<S>(S(1), S(0), S(0));
        w1 = w2 = zero3<S>();
    } else {
        n1 = dpt / radius;
        n2 = -n1;
        w1 = n1 * S(r1);
        w2 = n2 * S(r2);
    }
    o.status = (hit == 2 && norm_sq(center) < rsum * rsum) ? TOI_PENETRATING : TOI_CONVERGED;
    o.w1 = cvt<S>(inverse_transform_vector(m1, cvt<N>(w1)));
    o.w2 = cvt<S>(inverse_transform_vector(m2, cvt<N>(w2)));
    o.n1 = cvt<S>(inverse_transform_vector(m1, cvt<N>(n1)));
    o.n2 = cvt<S>(inverse_transform_vector(m2, cvt<N>(n2)));
    return o;
}

template <class S> struct RayOut {
    bool hit = false;
    S toi = S(0);
    V3<S> normal;  // world frame
};

// RayCast::toi_and_normal_with_ray of a support-map shape (the impls of
// ray_support_map.rs:58-110): the ray in the shape's local frame,
// ray_intersection_with_support_map_with_params (:14-56) = gjk::cast_ray
// (gjk.rs:180-194), i.e. the ray cast against (identity, g) - (identity,
// ConstantOrigin); with solid = false and the origin inside the shape, a
// second cast backwards from beyond the shape (shift = the support distance
// along the ray + 0.001).  The normal is rotated back into the world frame.
// The ray parameters are in S, the ray origin and the shift in N.
template <class N, class S>
RayOut<S> ray_cast_support_map(const Iso<N>& m, const Shape<N>& g, V3<N> ray_origin, V3<N> ray_dir, S max_toi,
                               bool solid, const Tol<S>& tol, Counters* cnt) {
    RayOut<S> o;
    const Iso<N> id{Quat<N>{N(0), N(0), N(0), N(1)}, zero3<N>()};
    Shape<N> origin{};
    origin.kind = CONSTANT_ORIGIN;
    const V3<N> lo = inverse_transform_vector(m, ray_origin - m.t);
    const V3<N> ld = inverse_transform_vector(m, ray_dir);
    VoronoiSimplex<N, S> simplex;
    RayCastOut<S> rc = minkowski_ray_cast(id, g, N(0), false, id, origin, lo, cvt<S>(ld), max_toi, simplex, tol, cnt);
    if (!rc.hit) return o;
    S toi = rc.toi;
    V3<S> normal = rc.normal;
    if (!solid && toi == S(0)) {
        // the ray starts inside the shape
        const V3<N> ndir = ld / norm(ld);
        const V3<N> supp = support_point(id, g, ndir, cnt);
        const N eps = N(0.001);
        const N shift = dot(supp - lo, ndir) + eps;
        const V3<N> no = lo + ndir * shift;
        RayCastOut<S> rc2 =
            minkowski_ray_cast(id, g, N(0), false, id, origin, no, cvt<S>(-ld), S(shift + eps), simplex, tol, cnt);
        if (!rc2.hit) return o;
        toi = S(shift) - rc2.toi;
        if (!(toi <= max_toi)) return o;
        normal = rc2.normal;
    }
    o.hit = true;
    o.toi = toi;
    o.normal = cvt<S>(rotate(m.q, cvt<N>(normal)));
    return o;
}

}  // namespace ncgo
