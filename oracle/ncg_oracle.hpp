// ncg_oracle.hpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of ncollide3d 0.33's convex narrow phase: support maps,
// CSOPoint, VoronoiSimplex with the segment/triangle/tetrahedron Voronoi
// projections, gjk::closest_points, 3-D EPA, and the contact / distance /
// proximity / closest_points wrappers for support-map pairs.  It is used only
// by the test-suite, by the smoke check and by the CPU-baseline leg of the
// benchmark, as the checker.  The GPU library never includes or links it.
//
// Templates:  N = arithmetic of support mapping and CSO points,
//             S = arithmetic of the simplex sub-solve, EPA face normals and
//                 the termination tests.
//   <float, float>   = the reference f32 path,
//   <double, double> = the reference built with f64 (the FP64 error oracle),
//   <float, dw>      = the mixed split that the GPU kernels compute (dw =
//                      double-word float-float arithmetic, dw.hpp).
// Build with -ffp-contract=off: the reference (Rust) never fuses mul+add.
//
// Parity pins: the known-answer tests of the reference (tests/geometry/epa3.rs,
// tests/geometry/cylinder_cuboid_contact.rs, examples/{distance,proximity}_query3d.rs,
// benches/query/algorithm.rs) run against this file in tests/test_oracle_kat.py.
// nalgebra 0.30 (third-party, not vendored) supplies the vector/quaternion
// arithmetic; it is restated from its published formulas below, so bit-level
// agreement with nalgebra's rounding is unpinned.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#include "dw.hpp"

namespace ncgo {

// ---------------------------------------------------------------- vectors
template <class T> struct V3 {
    T x, y, z;
};
template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
// nalgebra's 3-row dot: (a0*b0 + a1*b1) + a2*b2.
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T norm_sq(V3<T> a) { return dot(a, a); }
template <class T> inline T norm(V3<T> a) {
    using std::sqrt;
    return sqrt(norm_sq(a));
}
template <class T, class U> inline V3<T> cvt(V3<U> a) { return {T(a.x), T(a.y), T(a.z)}; }
template <class T> inline V3<T> zero3() { return {T(0), T(0), T(0)}; }

// Unit::try_new_and_get (nalgebra): None when |v| <= min_norm, else (v/|v|, |v|).
template <class T> inline bool try_normalize(V3<T> v, T min_norm, V3<T>* out, T* n_out) {
    T n = norm(v);
    if (n <= min_norm) return false;
    *out = v / n;
    if (n_out) *n_out = n;
    return true;
}

template <class T> struct Quat {
    T i, j, k, w;
};
// UnitQuaternion * Vector3 (nalgebra): t = 2 (q.v x v); v' = t*w + q.v x t + v.
template <class T> inline V3<T> rotate(const Quat<T>& q, V3<T> v) {
    V3<T> qv{q.i, q.j, q.k};
    V3<T> t = cross(qv, v) * T(2);
    V3<T> c = cross(qv, t);
    return (t * q.w + c) + v;
}
template <class T> inline V3<T> inv_rotate(const Quat<T>& q, V3<T> v) {
    Quat<T> c{-q.i, -q.j, -q.k, q.w};
    return rotate(c, v);
}

template <class T> struct Iso {
    Quat<T> q;
    V3<T> t;
};
template <class T> inline V3<T> transform_point(const Iso<T>& m, V3<T> p) { return rotate(m.q, p) + m.t; }
template <class T> inline V3<T> inverse_transform_vector(const Iso<T>& m, V3<T> v) { return inv_rotate(m.q, v); }

// ---------------------------------------------------------------- shapes
enum Kind { BALL = 0, CUBOID = 1, CAPSULE = 2, CONE = 3, CYLINDER = 4, CONVEX_HULL = 5, CONSTANT_ORIGIN = 7 };

template <class N> struct Shape {
    int kind;
    N p0, p1, p2;
    const float* pts4 = nullptr;  // hull points, 4 floats per point (f32 storage)
    const double* pts4d = nullptr; // hull points in f64 storage (known-answer inputs)
    uint32_t n = 0;
    inline V3<N> point(uint32_t i) const {
        if (pts4d) return {N(pts4d[4 * i]), N(pts4d[4 * i + 1]), N(pts4d[4 * i + 2])};
        return {N(pts4[4 * i]), N(pts4[4 * i + 1]), N(pts4[4 * i + 2])};
    }
};

struct Counters {
    uint32_t gjk_iters = 0;
    uint32_t epa_iters = 0;
    uint32_t support_calls = 0;
    uint32_t hull_points_scanned = 0;
    uint32_t subsolve[4] = {0, 0, 0, 0};
    uint32_t faces_created = 0;
    uint32_t epa_max_vertices = 0;
    uint32_t epa_max_faces = 0;
    uint32_t epa_exit = 0;  // EPA exit taken, one of EpaExit
    uint32_t status = 0;
};

// Which return of EPA::closest_points was taken (epa3.rs line numbers).
enum EpaExit : uint32_t {
    EXIT_NONE = 0,
    EXIT_DIM0 = 1,          // :243-246
    EXIT_CONVERGED = 2,     // :351-355
    EXIT_NUMERIC = 3,       // :397-402 (new face closer than the popped one)
    EXIT_HEAP_EMPTY = 4,    // :427-429
    EXIT_FAILED = 5,        // None: :278-293, :369-372, :404, :409-413, :421-424
    EXIT_PRECISION = 7,     // PRECISE set: a None of the expansion loop, answered with the best face
};

enum StatusBits : uint32_t {
    ST_GJK_MAX_ITER = 1u << 0,
    ST_EPA_FAILED = 1u << 1,
    ST_EPA_MAX_ITER = 1u << 2,
    ST_EPA_CAPACITY = 1u << 3,
    ST_EPA_NO_FACE = 1u << 4,
    ST_DEGENERATE = 1u << 5,
    ST_BAD_INPUT = 1u << 6,
    ST_UNSUPPORTED_FEATURE = 1u << 7,
    ST_EPA_PRECISION_LIMIT = 1u << 8,
};

// src/utils/point_cloud_support_point.rs:6-33 — first maximum wins.
template <class N> inline uint32_t point_cloud_support_point_id(V3<N> dir, const Shape<N>& s, Counters* c) {
    uint32_t best = 0;
    N best_dot = dot(s.point(0), dir);
    for (uint32_t i = 1; i < s.n; ++i) {
        N d = dot(s.point(i), dir);
        if (d > best_dot) {
            best_dot = d;
            best = i;
        }
    }
    if (c) c->hull_points_scanned += s.n;
    return best;
}

// Local support functions: ball.rs:45-48, cuboid.rs:135-146, capsule.rs:72-84,
// cone.rs:45-67, cylinder.rs:47-63, convex.rs:418-423.
template <class N> inline V3<N> local_support_point(const Shape<N>& s, V3<N> dir, Counters* c) {
    switch (s.kind) {
    case BALL: {
        V3<N> d = dir / norm(dir);
        return d * s.p0;
    }
    case CUBOID:
        return {std::copysign(s.p0, dir.x), std::copysign(s.p1, dir.y), std::copysign(s.p2, dir.z)};
    case CAPSULE: {
        V3<N> d = dir / norm(dir);
        V3<N> res{N(0), std::copysign(s.p0, d.y), N(0)};
        return res + d * s.p1;
    }
    case CONE: {
        V3<N> v{dir.x, N(0), dir.z};
        N n = norm(v);
        v = v / n;
        if (n == N(0)) {
            return {N(0), std::copysign(s.p0, dir.y), N(0)};
        }
        v = v * s.p1;
        v.y = -s.p0;
        if (dot(dir, v) < dir.y * s.p0) return {N(0), s.p0, N(0)};
        return v;
    }
    case CYLINDER: {
        V3<N> v{dir.x, N(0), dir.z};
        N n = norm(v);
        v = v / n;
        if (n == N(0)) v = zero3<N>();
        else v = v * s.p1;
        v.y = std::copysign(s.p0, dir.y);
        return v;
    }
    case CONSTANT_ORIGIN:
        return zero3<N>();
    case CONVEX_HULL:
    default:
        return s.point(point_cloud_support_point_id(dir, s, c));
    }
}

// SupportMap::support_point (support_map.rs:25-28); Ball overrides it (ball.rs:31-39).
template <class N> inline V3<N> support_point(const Iso<N>& m, const Shape<N>& s, V3<N> dir, Counters* c) {
    if (c) c->support_calls++;
    if (s.kind == CONSTANT_ORIGIN) return zero3<N>();  // special_support_maps.rs:9-30
    if (s.kind == BALL) {
        V3<N> d = dir / norm(dir);
        return m.t + d * s.p0;
    }
    V3<N> local = inverse_transform_vector(m, dir);
    return transform_point(m, local_support_point(s, local, c));
}

// cso_point.rs:14-22, 66-81.
template <class N> struct CSOPoint {
    V3<N> point, orig1, orig2;
};
template <class N>
inline CSOPoint<N> cso_from_shapes(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2,
                                   V3<N> dir, Counters* c) {
    V3<N> sp1 = support_point(m1, g1, dir, c);
    V3<N> sp2 = support_point(m2, g2, -dir, c);
    return CSOPoint<N>{sp1 - sp2, sp1, sp2};
}

// Tolerances: gjk.rs:26-29 (eps_tol = 10 eps), gjk.rs:92 (eps_rel = sqrt),
// epa3.rs:231-232 (100 eps), utils/triangle.rs:94-101 ((100 eps)^2).
template <class S> struct Tol {
    S eps, eps_tol, eps_rel, epa_eps_tol, affine_eps;
    S add_tol;  // VoronoiSimplex::add_point's degeneracy threshold (gjk::eps_tol in the reference)
    // PRECISE set only: when the expansion loop would return None (a new face
    // with the origin more than eps_tol outside it, or no new face), EPA
    // answers with the best face found so far instead.
    bool best_on_failure = false;
    Tol() {}
    // In S arithmetic, as the reference computes them for N = S.
    // epa_tol > 0 replaces EPA's termination threshold (100 eps) only.
    explicit Tol(S e, S epa_tol = S(0)) {
        using std::sqrt;
        eps = e;
        eps_tol = e * S(10.0);
        eps_rel = sqrt(eps_tol);
        epa_eps_tol = epa_tol > S(0) ? epa_tol : e * S(100.0);
        S t = e * S(100.0);
        affine_eps = t * t;
        add_tol = eps_tol;
    }
};
template <class S> inline Tol<S> make_tol(double e, double epa_tol) { return Tol<S>(S(e), S(epa_tol)); }
// The double-word split computes its constants in f64 and rounds them to
// double-word (the kernels' host code does the same).
template <> inline Tol<dw> make_tol<dw>(double e, double epa_tol) {
    Tol<dw> t;
    t.eps = dw::from_double(e);
    t.eps_tol = dw::from_double(e * 10.0);
    t.eps_rel = dw::from_double(std::sqrt(e * 10.0));
    t.epa_eps_tol = dw::from_double(epa_tol > 0 ? epa_tol : e * 100.0);
    double a = e * 100.0;
    t.affine_eps = dw::from_double(a * a);
    t.add_tol = t.eps_tol;
    return t;
}
// The kernels' PRECISE tolerance set: the tests that classify (origin on the
// simplex, origin inside the tetrahedron, EPA face checks and visibility) keep
// the f32 machine epsilon, the noise floor of f32 support points; the tests
// that decide how far GJK refines (add_point's degeneracy threshold and the
// relative gap sqrt(10 eps)) use f64::EPSILON as the reference built with f64.
template <class S> inline Tol<S> make_tol_precise(double epa_tol) {
    Tol<S> t = make_tol<S>((double)FLT_EPSILON, epa_tol);
    t.eps_rel = S(std::sqrt(10.0 * (double)DBL_EPSILON));
    t.add_tol = S(10.0 * (double)DBL_EPSILON);
    t.best_on_failure = true;
    return t;
}
template <> inline Tol<dw> make_tol_precise<dw>(double epa_tol) {
    Tol<dw> t = make_tol<dw>((double)FLT_EPSILON, epa_tol);
    t.eps_rel = dw::from_double(std::sqrt(10.0 * (double)DBL_EPSILON));
    t.add_tol = dw::from_double(10.0 * (double)DBL_EPSILON);
    t.best_on_failure = true;
    return t;
}


// ------------------------------------------------- point projections (solid)
enum LocKind { ON_VERTEX, ON_EDGE, ON_FACE, ON_SOLID };
template <class S> struct Loc {
    LocKind kind;
    int i;        // vertex / edge / face index
    S b[3];       // barycentric coordinates
};

// point_segment.rs:52-91 with m = identity and pt = origin.
template <class S> inline V3<S> project_origin_segment(V3<S> a, V3<S> b, Loc<S>* loc) {
    V3<S> p = zero3<S>();
    V3<S> ab = b - a;
    V3<S> ap = p - a;
    S ab_ap = dot(ab, ap);
    S sqnab = norm_sq(ab);
    if (ab_ap <= S(0)) {
        *loc = {ON_VERTEX, 0, {S(1), S(0), S(0)}};
        return a;
    } else if (ab_ap >= sqnab) {
        *loc = {ON_VERTEX, 1, {S(1), S(0), S(0)}};
        return b;
    }
    S u = ab_ap / sqnab;
    *loc = {ON_EDGE, 0, {S(1) - u, u, S(0)}};
    return a + ab * u;
}

// point_triangle.rs:61-309 with m = identity, pt = origin and solid = true.
template <class S> inline V3<S> project_origin_triangle(V3<S> a, V3<S> b, V3<S> c, Loc<S>* loc) {
    V3<S> p = zero3<S>();
    V3<S> ab = b - a, ac = c - a, ap = p - a;
    S ab_ap = dot(ab, ap), ac_ap = dot(ac, ap);
    if (ab_ap <= S(0) && ac_ap <= S(0)) {
        *loc = {ON_VERTEX, 0, {S(1), S(0), S(0)}};
        return a;
    }
    V3<S> bp = p - b;
    S ab_bp = dot(ab, bp), ac_bp = dot(ac, bp);
    if (ab_bp >= S(0) && ac_bp <= ab_bp) {
        *loc = {ON_VERTEX, 1, {S(1), S(0), S(0)}};
        return b;
    }
    V3<S> cp = p - c;
    S ab_cp = dot(ab, cp), ac_cp = dot(ac, cp);
    if (ac_cp >= S(0) && ab_cp <= ac_cp) {
        *loc = {ON_VERTEX, 2, {S(1), S(0), S(0)}};
        return c;
    }
    V3<S> bc = c - b;
    // stable_check_edges_voronoi, 3-D branch (:158-191), no improved_fixed_point_support.
    V3<S> n = cross(ab, ac);
    S vc = dot(n, cross(ab, ap));
    if (vc < S(0) && ab_ap >= S(0) && ab_bp <= S(0)) {
        S v = ab_ap / norm_sq(ab);
        *loc = {ON_EDGE, 0, {S(1) - v, v, S(0)}};
        return a + ab * v;
    }
    S vb = -dot(n, cross(ac, cp));
    if (vb < S(0) && ac_ap >= S(0) && ac_cp <= S(0)) {
        S w = ac_ap / norm_sq(ac);
        *loc = {ON_EDGE, 2, {S(1) - w, w, S(0)}};
        return a + ac * w;
    }
    S va = dot(n, cross(bc, bp));
    if (va < S(0) && ac_bp - ab_bp >= S(0) && ab_cp - ac_cp >= S(0)) {
        S w = dot(bc, bp) / norm_sq(bc);
        *loc = {ON_EDGE, 1, {S(1) - w, w, S(0)}};
        return b + bc * w;
    }
    int clockwise = dot(n, ap) >= S(0) ? 0 : 1;
    if (va + vb + vc != S(0)) {
        S denom = S(1) / (va + vb + vc);
        S v = vb * denom;
        S w = vc * denom;
        *loc = {ON_FACE, clockwise, {S(1) - v - w, v, w}};
        return (a + ab * v) + ac * w;
    }
    *loc = {ON_SOLID, 0, {S(0), S(0), S(0)}};
    return p;
}

// point_tetrahedron.rs:35-353 with m = identity, pt = origin, solid = true.
template <class S> struct TetraEdge {
    S d1, d2;
    bool hit;
    V3<S> proj;
    S b[2];
};
template <class S>
inline TetraEdge<S> tetra_check_edge(V3<S> a, V3<S> nabc, V3<S> nabd, V3<S> ap, V3<S> ab, S ap_ab, S bp_ab) {
    TetraEdge<S> r;
    S ab_ab = ap_ab - bp_ab;
    V3<S> ap_x_ab = cross(ap, ab);
    r.d1 = dot(ap_x_ab, nabc);
    r.d2 = dot(ap_x_ab, nabd);
    r.hit = false;
    if (ab_ab != S(0) && r.d1 >= S(0) && r.d2 >= S(0) && ap_ab >= S(0) && ap_ab <= ab_ab) {
        S u = ap_ab / ab_ab;
        r.b[0] = S(1) - u;
        r.b[1] = u;
        r.proj = a + ab * u;
        r.hit = true;
    }
    return r;
}
template <class S>
inline bool tetra_check_face(V3<S> a, V3<S> b, V3<S> c, V3<S> ap, V3<S> bp, V3<S> cp, V3<S> ab, V3<S> ac, V3<S> ad,
                             S dabc, S dbca, S dacb, S eps, V3<S>* proj, S bc_out[3], uint32_t* status) {
    if (dabc < S(0) && dbca < S(0) && dacb < S(0)) {
        V3<S> n = cross(ab, ac);
        if (dot(n, ad) * dot(n, ap) < S(0)) {
            V3<S> normal;
            if (!try_normalize(n, eps, &normal, (S*)nullptr)) return false;  // the `?` at :289
            S vc = dot(normal, cross(ap, bp));
            S va = dot(normal, cross(bp, cp));
            S vb = dot(normal, cross(cp, ap));
            S denom = va + vb + vc;
            if (denom == S(0)) *status |= ST_DEGENERATE;  // assert!(denom != 0) at :295
            S inv = S(1) / denom;
            bc_out[0] = va * inv;
            bc_out[1] = vb * inv;
            bc_out[2] = vc * inv;
            *proj = (a * bc_out[0] + b * bc_out[1]) + c * bc_out[2];
            return true;
        }
    }
    return false;
}
template <class S>
inline V3<S> project_origin_tetrahedron(V3<S> a, V3<S> b, V3<S> c, V3<S> d, S eps, Loc<S>* loc, uint32_t* status) {
    V3<S> p = zero3<S>();
    V3<S> ab = b - a, ac = c - a, ad = d - a, ap = p - a;
    S ap_ab = dot(ap, ab), ap_ac = dot(ap, ac), ap_ad = dot(ap, ad);
    if (ap_ab <= S(0) && ap_ac <= S(0) && ap_ad <= S(0)) {
        *loc = {ON_VERTEX, 0, {S(1), S(0), S(0)}};
        return a;
    }
    V3<S> bc = c - b, bd = d - b, bp = p - b;
    S bp_bc = dot(bp, bc), bp_bd = dot(bp, bd), bp_ab = dot(bp, ab);
    if (bp_bc <= S(0) && bp_bd <= S(0) && bp_ab >= S(0)) {
        *loc = {ON_VERTEX, 1, {S(1), S(0), S(0)}};
        return b;
    }
    V3<S> cd = d - c, cp = p - c;
    S cp_ac = dot(cp, ac), cp_bc = dot(cp, bc), cp_cd = dot(cp, cd);
    if (cp_cd <= S(0) && cp_bc >= S(0) && cp_ac >= S(0)) {
        *loc = {ON_VERTEX, 2, {S(1), S(0), S(0)}};
        return c;
    }
    V3<S> dp = p - d;
    S dp_cd = dot(dp, cd), dp_bd = dot(dp, bd), dp_ad = dot(dp, ad);
    if (dp_ad >= S(0) && dp_bd >= S(0) && dp_cd >= S(0)) {
        *loc = {ON_VERTEX, 3, {S(1), S(0), S(0)}};
        return d;
    }
    V3<S> nabc = cross(ab, ac), nabd = cross(ab, ad);
    TetraEdge<S> e0 = tetra_check_edge(a, nabc, nabd, ap, ab, ap_ab, bp_ab);
    if (e0.hit) { *loc = {ON_EDGE, 0, {e0.b[0], e0.b[1], S(0)}}; return e0.proj; }
    S dabc = e0.d1, dabd = e0.d2;
    V3<S> nacd = cross(ac, ad);
    TetraEdge<S> e1 = tetra_check_edge(a, nacd, -nabc, ap, ac, ap_ac, cp_ac);
    if (e1.hit) { *loc = {ON_EDGE, 1, {e1.b[0], e1.b[1], S(0)}}; return e1.proj; }
    S dacd = e1.d1, dacb = e1.d2;
    TetraEdge<S> e2 = tetra_check_edge(a, -nabd, -nacd, ap, ad, ap_ad, dp_ad);
    if (e2.hit) { *loc = {ON_EDGE, 2, {e2.b[0], e2.b[1], S(0)}}; return e2.proj; }
    S dadb = e2.d1, dadc = e2.d2;
    V3<S> nbcd = cross(bc, bd);
    TetraEdge<S> e3 = tetra_check_edge(b, nabc, nbcd, bp, bc, bp_bc, cp_bc);
    if (e3.hit) { *loc = {ON_EDGE, 3, {e3.b[0], e3.b[1], S(0)}}; return e3.proj; }
    S dbca = e3.d1, dbcd = e3.d2;
    TetraEdge<S> e4 = tetra_check_edge(b, -nbcd, nabd, bp, bd, bp_bd, dp_bd);
    if (e4.hit) { *loc = {ON_EDGE, 4, {e4.b[0], e4.b[1], S(0)}}; return e4.proj; }
    S dbdc = e4.d1, dbda = e4.d2;
    TetraEdge<S> e5 = tetra_check_edge(c, nacd, nbcd, cp, cd, cp_cd, dp_cd);
    if (e5.hit) { *loc = {ON_EDGE, 5, {e5.b[0], e5.b[1], S(0)}}; return e5.proj; }
    S dcda = e5.d1, dcdb = e5.d2;

    V3<S> proj;
    S bc3[3];
    if (tetra_check_face(a, b, c, ap, bp, cp, ab, ac, ad, dabc, dbca, dacb, eps, &proj, bc3, status)) {
        *loc = {ON_FACE, 0, {bc3[0], bc3[1], bc3[2]}};
        return proj;
    }
    if (tetra_check_face(a, b, d, ap, bp, dp, ab, ad, ac, dadb, dabd, dbda, eps, &proj, bc3, status)) {
        *loc = {ON_FACE, 1, {bc3[0], bc3[1], bc3[2]}};
        return proj;
    }
    if (tetra_check_face(a, c, d, ap, cp, dp, ac, ad, ab, dacd, dcda, dadc, eps, &proj, bc3, status)) {
        *loc = {ON_FACE, 2, {bc3[0], bc3[1], bc3[2]}};
        return proj;
    }
    if (tetra_check_face(b, c, d, bp, cp, dp, bc, bd, -ab, dbcd, dcdb, dbdc, eps, &proj, bc3, status)) {
        *loc = {ON_FACE, 3, {bc3[0], bc3[1], bc3[2]}};
        return proj;
    }
    *loc = {ON_SOLID, 0, {S(0), S(0), S(0)}};
    return p;
}

// ------------------------------------------------------ VoronoiSimplex
// voronoi_simplex3.rs:12-280.
template <class N, class S> struct VoronoiSimplex {
    int prev_vertices[4] = {0, 1, 2, 3};
    S prev_proj[3] = {S(0), S(0), S(0)};
    int prev_dim = 0;
    CSOPoint<N> vertices[4];
    S proj[3] = {S(0), S(0), S(0)};
    int dim = 0;

    VoronoiSimplex() {
        for (auto& v : vertices) v = CSOPoint<N>{zero3<N>(), zero3<N>(), zero3<N>()};
    }
    void swap(int i1, int i2) {
        std::swap(vertices[i1], vertices[i2]);
        std::swap(prev_vertices[i1], prev_vertices[i2]);
    }
    void reset(const CSOPoint<N>& pt) {
        dim = 0;
        prev_dim = 0;
        vertices[0] = pt;
    }
    V3<S> pt(int i) const { return cvt<S>(vertices[i].point); }

    bool add_point(const CSOPoint<N>& p, const Tol<S>& tol) {
        prev_dim = dim;
        for (int i = 0; i < 3; ++i) prev_proj[i] = proj[i];
        for (int i = 0; i < 4; ++i) prev_vertices[i] = i;
        V3<S> ps = cvt<S>(p.point);
        if (dim == 0) {
            if (norm_sq(pt(0) - ps) < tol.add_tol) return false;
        } else if (dim == 1) {
            V3<S> ab = pt(1) - pt(0);
            V3<S> ac = ps - pt(0);
            if (norm_sq(cross(ab, ac)) < tol.add_tol) return false;
        } else {  // dim == 2
            V3<S> ab = pt(1) - pt(0);
            V3<S> ac = pt(2) - pt(0);
            V3<S> ap = ps - pt(0);
            V3<S> c = cross(ab, ac);
            V3<S> n = c / norm(c);
            using std::fabs;
            if (fabs(dot(n, ap)) < tol.add_tol) return false;
        }
        dim += 1;
        vertices[dim] = p;
        return true;
    }

    V3<S> project_origin_and_reduce(const Tol<S>& tol, Counters* cnt) {
        if (cnt) cnt->subsolve[dim]++;
        if (dim == 0) {
            proj[0] = S(1);
            return pt(0);
        } else if (dim == 1) {
            Loc<S> loc;
            V3<S> r = project_origin_segment(pt(0), pt(1), &loc);
            if (loc.kind == ON_VERTEX && loc.i == 0) {
                proj[0] = S(1);
                dim = 0;
            } else if (loc.kind == ON_VERTEX) {
                swap(0, 1);
                proj[0] = S(1);
                dim = 0;
            } else {
                proj[0] = loc.b[0];
                proj[1] = loc.b[1];
            }
            return r;
        } else if (dim == 2) {
            Loc<S> loc;
            V3<S> r = project_origin_triangle(pt(0), pt(1), pt(2), &loc);
            if (loc.kind == ON_VERTEX) {
                swap(0, loc.i);
                proj[0] = S(1);
                dim = 0;
            } else if (loc.kind == ON_EDGE) {
                if (loc.i == 0) {
                    proj[0] = loc.b[0];
                    proj[1] = loc.b[1];
                } else if (loc.i == 1) {
                    swap(0, 2);
                    proj[0] = loc.b[1];
                    proj[1] = loc.b[0];
                } else {
                    swap(1, 2);
                    proj[0] = loc.b[0];
                    proj[1] = loc.b[1];
                }
                dim = 1;
            } else if (loc.kind == ON_FACE) {
                proj[0] = loc.b[0];
                proj[1] = loc.b[1];
                proj[2] = loc.b[2];
            }
            // ON_SOLID: nothing changes (voronoi_simplex3.rs:181).
            return r;
        } else {
            Loc<S> loc;
            uint32_t st = 0;
            V3<S> r = project_origin_tetrahedron(pt(0), pt(1), pt(2), pt(3), tol.eps, &loc, &st);
            if (cnt) cnt->status |= st;
            if (loc.kind == ON_VERTEX) {
                swap(0, loc.i);
                proj[0] = S(1);
                dim = 0;
            } else if (loc.kind == ON_EDGE) {
                switch (loc.i) {
                case 0: break;
                case 1: swap(1, 2); break;
                case 2: swap(1, 3); break;
                case 3: swap(0, 2); break;
                case 4: swap(0, 3); break;
                case 5: swap(0, 2); swap(1, 3); break;
                }
                if (loc.i == 3 || loc.i == 4) {
                    proj[0] = loc.b[1];
                    proj[1] = loc.b[0];
                } else {
                    proj[0] = loc.b[0];
                    proj[1] = loc.b[1];
                }
                dim = 1;
            } else if (loc.kind == ON_FACE) {
                switch (loc.i) {
                case 0:
                    proj[0] = loc.b[0]; proj[1] = loc.b[1]; proj[2] = loc.b[2];
                    break;
                case 1:
                    vertices[2] = vertices[3];
                    proj[0] = loc.b[0]; proj[1] = loc.b[1]; proj[2] = loc.b[2];
                    break;
                case 2:
                    vertices[1] = vertices[3];
                    proj[0] = loc.b[0]; proj[1] = loc.b[2]; proj[2] = loc.b[1];
                    break;
                case 3:
                    vertices[0] = vertices[3];
                    proj[0] = loc.b[2]; proj[1] = loc.b[0]; proj[2] = loc.b[1];
                    break;
                }
                dim = 2;
            }
            return r;
        }
    }
};

// --------------------------------------------------------------- GJK
enum GJKKind { GJK_INTERSECTION = 0, GJK_CLOSEST_POINTS = 1, GJK_PROXIMITY = 2, GJK_NO_INTERSECTION = 3 };
template <class S> struct GJKResult {
    GJKKind kind;
    V3<S> p1, p2, dir;
};

// gjk.rs:367-388.
template <class N, class S> inline void gjk_result(const VoronoiSimplex<N, S>& s, bool prev, V3<S>* p1, V3<S>* p2) {
    V3<S> r1 = zero3<S>(), r2 = zero3<S>();
    if (prev) {
        for (int i = 0; i < s.prev_dim + 1; ++i) {
            S c = s.prev_proj[i];
            const CSOPoint<N>& p = s.vertices[s.prev_vertices[i]];
            r1 = r1 + cvt<S>(p.orig1) * c;
            r2 = r2 + cvt<S>(p.orig2) * c;
        }
    } else {
        for (int i = 0; i < s.dim + 1; ++i) {
            S c = s.proj[i];
            const CSOPoint<N>& p = s.vertices[i];
            r1 = r1 + cvt<S>(p.orig1) * c;
            r2 = r2 + cvt<S>(p.orig2) * c;
        }
    }
    *p1 = r1;
    *p2 = r2;
}

// gjk.rs:76-177.
template <class N, class S>
GJKResult<S> gjk_closest_points(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2, S max_dist,
                                bool exact_dist, VoronoiSimplex<N, S>& simplex, const Tol<S>& tol, Counters* cnt,
                                int max_iter = 10000) {
    GJKResult<S> res;
    V3<S> proj = simplex.project_origin_and_reduce(tol, cnt);
    V3<S> old_dir;
    {
        V3<S> u;
        if (try_normalize(proj, S(0), &u, (S*)nullptr)) old_dir = -u;
        else { res.kind = GJK_INTERSECTION; return res; }
    }
    S max_bound = std::numeric_limits<S>::max();
    V3<S> dir;
    int niter = 0;
    for (;;) {
        if (cnt) cnt->gjk_iters++;
        S old_max_bound = max_bound;
        {
            V3<S> u;
            S n;
            if (try_normalize(-proj, tol.eps_tol, &u, &n)) { dir = u; max_bound = n; }
            else { res.kind = GJK_INTERSECTION; return res; }
        }
        if (max_bound >= old_max_bound) {
            if (exact_dist) {
                gjk_result(simplex, true, &res.p1, &res.p2);
                res.kind = GJK_CLOSEST_POINTS; res.dir = old_dir; return res;
            }
            res.kind = GJK_PROXIMITY; res.dir = old_dir; return res;
        }
        CSOPoint<N> cso = cso_from_shapes(m1, g1, m2, g2, cvt<N>(dir), cnt);
        S min_bound = -dot(dir, cvt<S>(cso.point));
        if (min_bound != min_bound) { if (cnt) cnt->status |= ST_BAD_INPUT; }  // assert at :132
        if (min_bound > max_dist) {
            res.kind = GJK_NO_INTERSECTION; res.dir = dir; return res;
        } else if (!exact_dist && min_bound > S(0) && max_bound <= max_dist) {
            res.kind = GJK_PROXIMITY; res.dir = old_dir; return res;
        } else if (max_bound - min_bound <= tol.eps_rel * max_bound) {
            if (exact_dist) {
                gjk_result(simplex, false, &res.p1, &res.p2);
                res.kind = GJK_CLOSEST_POINTS; res.dir = dir; return res;
            }
            res.kind = GJK_PROXIMITY; res.dir = dir; return res;
        }
        if (!simplex.add_point(cso, tol)) {
            if (exact_dist) {
                gjk_result(simplex, false, &res.p1, &res.p2);
                res.kind = GJK_CLOSEST_POINTS; res.dir = dir; return res;
            }
            res.kind = GJK_PROXIMITY; res.dir = dir; return res;
        }
        old_dir = dir;
        proj = simplex.project_origin_and_reduce(tol, cnt);
        if (simplex.dim == 3) {
            if (min_bound >= tol.eps_tol) {
                if (exact_dist) {
                    gjk_result(simplex, true, &res.p1, &res.p2);
                    res.kind = GJK_CLOSEST_POINTS; res.dir = old_dir; return res;
                }
                res.kind = GJK_PROXIMITY; res.dir = old_dir; return res;
            }
            res.kind = GJK_INTERSECTION; return res;
        }
        niter += 1;
        if (niter == max_iter) {
            if (cnt) cnt->status |= ST_GJK_MAX_ITER;
            res.kind = GJK_NO_INTERSECTION; res.dir = v3<S>(S(1), S(0), S(0)); return res;
        }
    }
}

// --------------------------------------------------------------- EPA
// epa3.rs:13-49: FaceId ordered by neg_dist (max-heap => smallest distance first).
template <class S> struct FaceId {
    size_t id;
    S neg_dist;
};
template <class S> inline bool face_le(const FaceId<S>& a, const FaceId<S>& b) {
    // PartialOrd::le through partial_cmp: false when either is NaN.
    return a.neg_dist <= b.neg_dist;
}

// Restatement of Rust std's BinaryHeap (push = sift_up; pop = swap the last
// element to the root, sift_down_to_bottom, then sift_up), so that the pop
// order of equal keys matches the reference exactly.
template <class S> struct RustBinaryHeap {
    std::vector<FaceId<S>> data;
    void clear() { data.clear(); }
    size_t size() const { return data.size(); }
    void sift_up(size_t start, size_t pos) {
        FaceId<S> elt = data[pos];
        while (pos > start) {
            size_t parent = (pos - 1) / 2;
            if (face_le(elt, data[parent])) break;
            data[pos] = data[parent];
            pos = parent;
        }
        data[pos] = elt;
    }
    void sift_down_to_bottom(size_t pos) {
        size_t end = data.size();
        size_t start = pos;
        FaceId<S> elt = data[pos];
        size_t child = 2 * pos + 1;
        while (end >= 2 && child <= end - 2) {
            child += face_le(data[child], data[child + 1]) ? 1 : 0;
            data[pos] = data[child];
            pos = child;
            child = 2 * pos + 1;
        }
        if (child == end - 1) {
            data[pos] = data[child];
            pos = child;
        }
        data[pos] = elt;
        sift_up(start, pos);
    }
    void push(FaceId<S> f) {
        size_t old_len = data.size();
        data.push_back(f);
        sift_up(0, old_len);
    }
    bool pop(FaceId<S>* out) {
        if (data.empty()) return false;
        FaceId<S> item = data.back();
        data.pop_back();
        if (!data.empty()) {
            std::swap(item, data[0]);
            sift_down_to_bottom(0);
        }
        *out = item;
        return true;
    }
};

// Priority queue with a strict total order: larger neg_dist first, then the
// earlier push (FIFO among equal keys).  The pop order is then a function of
// the set of entries alone, whatever the container; the kernels use this order
// (their heap recycles face slots and purges deleted entries).  Equal keys are
// the only case where it differs from Rust's BinaryHeap, whose tie order is an
// implementation detail of the Rust version.
template <class S> struct SeqHeap {
    struct E {
        size_t id;
        S neg_dist;
        uint64_t seq;
    };
    std::vector<E> data;
    uint64_t next_seq = 0;
    static bool before(const E& a, const E& b) {  // a pops before b
        if (a.neg_dist > b.neg_dist) return true;
        if (b.neg_dist > a.neg_dist) return false;
        return a.seq < b.seq;
    }
    void clear() { data.clear(); next_seq = 0; }
    size_t size() const { return data.size(); }
    void push(FaceId<S> f) { data.push_back(E{f.id, f.neg_dist, next_seq++}); }
    size_t best() const {
        size_t b = 0;
        for (size_t i = 1; i < data.size(); ++i)
            if (before(data[i], data[b])) b = i;
        return b;
    }
    FaceId<S> top() const { return FaceId<S>{data[best()].id, data[best()].neg_dist}; }
    bool pop(FaceId<S>* out) {
        if (data.empty()) return false;
        size_t b = best();
        *out = FaceId<S>{data[b].id, data[b].neg_dist};
        data.erase(data.begin() + (long)b);
        return true;
    }
};
template <class S> inline FaceId<S> heap_top(const RustBinaryHeap<S>& h) { return h.data[0]; }
template <class S> inline FaceId<S> heap_top(const SeqHeap<S>& h) { return h.top(); }

// The reference instantiations (N == S) keep Rust's heap; the kernels' split uses SeqHeap.
template <class N, class S> struct HeapFor { using type = SeqHeap<S>; };
template <class T> struct HeapFor<T, T> { using type = RustBinaryHeap<T>; };

// The polytope's expansion (triangle projection, visibility) runs in N; the
// face normal is computed in S and stored in N; distances, heap keys and the
// termination test are in S.  With N = S this is the reference's EPA exactly.
template <class N> struct Face {
    size_t pts[3];
    size_t adj[3];
    V3<N> normal;
    N bcoords[3];
    bool deleted;
};

template <class N, class S> struct EPA {
    std::vector<CSOPoint<N>> vertices;
    std::vector<Face<N>> faces;
    std::vector<std::pair<size_t, size_t>> silhouette;  // (face_id, opp_pt_id)
    typename HeapFor<N, S>::type heap;
    const Tol<S>* tol = nullptr;

    V3<S> vp(size_t i) const { return cvt<S>(vertices[i].point); }
    V3<N> vn(size_t i) const { return vertices[i].point; }
    V3<S> fnormal(size_t f) const { return cvt<S>(faces[f].normal); }

    // epa3.rs:63-94 (ccw_face_normal: utils/ccw_face_normal.rs:21-27).
    Face<N> face_with_proj(const N b[3], size_t p0, size_t p1, size_t p2, size_t a0, size_t a1, size_t a2) {
        Face<N> f;
        f.pts[0] = p0; f.pts[1] = p1; f.pts[2] = p2;
        f.adj[0] = a0; f.adj[1] = a1; f.adj[2] = a2;
        V3<S> ab = vp(p1) - vp(p0), ac = vp(p2) - vp(p0);
        // The cross product in S; its normalisation in N (the result is stored
        // in N).  With N = S this is ccw_face_normal exactly.
        V3<N> n;
        if (!try_normalize(cvt<N>(cross(ab, ac)), N(tol->eps), &n, (N*)nullptr)) n = zero3<N>();
        f.normal = n;
        f.bcoords[0] = b[0]; f.bcoords[1] = b[1]; f.bcoords[2] = b[2];
        f.deleted = false;
        return f;
    }
    // epa3.rs:96-115 (the projected point itself is never used).
    Face<N> face_new(size_t p0, size_t p1, size_t p2, size_t a0, size_t a1, size_t a2, bool* inside) {
        Loc<N> loc;
        (void)project_origin_triangle(vn(p0), vn(p1), vn(p2), &loc);
        if (loc.kind == ON_FACE) {
            *inside = true;
            return face_with_proj(loc.b, p0, p1, p2, a0, a1, a2);
        }
        *inside = false;
        N z[3] = {N(0), N(0), N(0)};
        return face_with_proj(z, p0, p1, p2, a0, a1, a2);
    }
    // epa3.rs:117-126.
    void face_closest_points(const Face<N>& f, V3<S>* p1, V3<S>* p2) const {
        S b0 = S(f.bcoords[0]), b1 = S(f.bcoords[1]), b2 = S(f.bcoords[2]);
        *p1 = (cvt<S>(vertices[f.pts[0]].orig1) * b0 + cvt<S>(vertices[f.pts[1]].orig1) * b1) +
              cvt<S>(vertices[f.pts[2]].orig1) * b2;
        *p2 = (cvt<S>(vertices[f.pts[0]].orig2) * b0 + cvt<S>(vertices[f.pts[1]].orig2) * b1) +
              cvt<S>(vertices[f.pts[2]].orig2) * b2;
    }
    static size_t next_ccw_pt_id(const Face<N>& f, size_t id) {
        if (f.pts[0] == id) return 1;
        if (f.pts[1] == id) return 2;
        return 0;
    }
    // epa3.rs:143-156 and utils/triangle.rs:85-102.
    bool can_be_seen_by(const Face<N>& f, size_t point, size_t opp) const {
        V3<N> p0 = vn(f.pts[opp]);
        V3<N> p1 = vn(f.pts[(opp + 1) % 3]);
        V3<N> p2 = vn(f.pts[(opp + 2) % 3]);
        V3<N> pt = vn(point);
        if (dot(pt - p0, f.normal) >= -N(tol->eps_tol)) return true;
        // relative_eq!(|p1p2 x p1p3|^2, 0, epsilon = (100 eps)^2)
        N x = norm_sq(cross(p2 - p1, pt - p1));
        return x == N(0) || std::fabs(x) <= N(tol->affine_eps);
    }
    // epa3.rs:432-454.
    void compute_silhouette(size_t point, size_t id, size_t opp) {
        if (!faces[id].deleted) {
            if (!can_be_seen_by(faces[id], point, opp)) {
                silhouette.push_back({id, opp});
            } else {
                faces[id].deleted = true;
                size_t adj_pt_id1 = (opp + 2) % 3;
                size_t adj_pt_id2 = opp;
                size_t adj1 = faces[id].adj[adj_pt_id1];
                size_t adj2 = faces[id].adj[adj_pt_id2];
                size_t o1 = next_ccw_pt_id(faces[adj1], faces[id].pts[adj_pt_id1]);
                size_t o2 = next_ccw_pt_id(faces[adj2], faces[id].pts[adj_pt_id2]);
                compute_silhouette(point, adj1, o1);
                compute_silhouette(point, adj2, o2);
            }
        }
    }

    // epa3.rs:219-430.  Returns false for None.
    bool closest_points(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2,
                        const VoronoiSimplex<N, S>& simplex, const Tol<S>& t, V3<S>* out_p1, V3<S>* out_p2,
                        V3<S>* out_n, Counters* cnt, int max_iter = 10000) {
        tol = &t;
        vertices.clear();
        faces.clear();
        heap.clear();
        silhouette.clear();
        for (int i = 0; i < simplex.dim + 1; ++i) vertices.push_back(simplex.vertices[i]);

        if (simplex.dim == 0) {
            *out_p1 = zero3<S>();
            *out_p2 = zero3<S>();
            *out_n = v3<S>(S(0), S(1), S(0));
            if (cnt) cnt->epa_exit = EXIT_DIM0;
            return true;
        } else if (simplex.dim == 3) {
            V3<S> dp1 = vp(1) - vp(0), dp2 = vp(2) - vp(0), dp3 = vp(3) - vp(0);
            if (dot(cross(dp1, dp2), dp3) > S(0)) std::swap(vertices[1], vertices[2]);
            bool in1, in2, in3, in4;
            faces.push_back(face_new(0, 1, 2, 3, 1, 2, &in1));
            faces.push_back(face_new(1, 3, 2, 3, 2, 0, &in2));
            faces.push_back(face_new(0, 2, 3, 0, 1, 3, &in3));
            faces.push_back(face_new(0, 3, 1, 2, 1, 0, &in4));
            if (cnt) cnt->faces_created += 4;
            bool ins[4] = {in1, in2, in3, in4};
            for (size_t k = 0; k < 4; ++k) {
                if (ins[k]) {
                    S dist = dot(fnormal(k), vp(k));
                    if (-dist > t.eps_tol) { if (cnt) cnt->status |= ST_EPA_FAILED; return false; }
                    heap.push(FaceId<S>{k, -dist});
                }
            }
        } else {
            if (simplex.dim == 1) {
                // nalgebra orthonormal_subspace_basis(&[dpt]) for 3-D; the
                // closure returns false after the first basis vector a x dpt.
                V3<S> dpt = vp(1) - vp(0);
                V3<S> a;
                using std::fabs;
                if (fabs(dpt.x) > fabs(dpt.y)) a = v3<S>(dpt.z, S(0), -dpt.x);
                else a = v3<S>(S(0), -dpt.z, dpt.y);
                a = a / norm(a);
                V3<S> dir = cross(a, dpt);
                vertices.push_back(cso_from_shapes(m1, g1, m2, g2, cvt<N>(dir), cnt));
            }
            bool in1, in2;
            faces.push_back(face_new(0, 1, 2, 1, 1, 1, &in1));
            faces.push_back(face_new(0, 2, 1, 0, 0, 0, &in2));
            if (cnt) cnt->faces_created += 2;
            heap.push(FaceId<S>{0, S(0)});
            heap.push(FaceId<S>{1, S(0)});
        }

        if (heap.size() == 0) {  // heap.peek().unwrap() panics at epa3.rs:325
            if (cnt) cnt->status |= ST_EPA_NO_FACE;
            return false;
        }
        int niter = 0;
        S max_dist = std::numeric_limits<S>::max();
        FaceId<S> best_face_id = heap_top(heap);

        FaceId<S> face_id;
        while (heap.pop(&face_id)) {
            Face<N> face = faces[face_id.id];
            if (face.deleted) continue;
            if (cnt) cnt->epa_iters++;
            CSOPoint<N> cso = cso_from_shapes(m1, g1, m2, g2, cvt<N>(face.normal), cnt);
            size_t support_point_id = vertices.size();
            vertices.push_back(cso);
            S candidate_max_dist = dot(cvt<S>(cso.point), cvt<S>(face.normal));
            if (candidate_max_dist < max_dist) {
                best_face_id = face_id;
                max_dist = candidate_max_dist;
            }
            S curr_dist = -face_id.neg_dist;
            if (max_dist - curr_dist < t.epa_eps_tol) {
                const Face<N>& bf = faces[best_face_id.id];
                face_closest_points(bf, out_p1, out_p2);
                *out_n = cvt<S>(bf.normal);
                if (cnt) cnt->epa_exit = EXIT_CONVERGED;
                track(cnt);
                return true;
            }
            faces[face_id.id].deleted = true;
            size_t o1 = next_ccw_pt_id(faces[face.adj[0]], face.pts[0]);
            size_t o2 = next_ccw_pt_id(faces[face.adj[1]], face.pts[1]);
            size_t o3 = next_ccw_pt_id(faces[face.adj[2]], face.pts[2]);
            compute_silhouette(support_point_id, face.adj[0], o1);
            compute_silhouette(support_point_id, face.adj[1], o2);
            compute_silhouette(support_point_id, face.adj[2], o3);

            size_t first_new_face_id = faces.size();
            if (silhouette.empty()) {
                if (t.best_on_failure) return best_face(best_face_id, out_p1, out_p2, out_n, cnt);
                if (cnt) cnt->status |= ST_EPA_FAILED;
                track(cnt);
                return false;
            }
            for (const auto& edge : silhouette) {
                if (!faces[edge.first].deleted) {
                    size_t new_face_id = faces.size();
                    size_t pt_id1 = faces[edge.first].pts[(edge.second + 2) % 3];
                    size_t pt_id2 = faces[edge.first].pts[(edge.second + 1) % 3];
                    bool inside;
                    Face<N> nf = face_new(pt_id1, pt_id2, support_point_id, edge.first, new_face_id + 1,
                                          new_face_id - 1, &inside);
                    faces[edge.first].adj[(edge.second + 1) % 3] = new_face_id;
                    faces.push_back(nf);
                    if (cnt) cnt->faces_created++;
                    if (inside) {
                        S dist = dot(fnormal(new_face_id), vp(faces[new_face_id].pts[0]));
                        if (dist < curr_dist) {
                            face_closest_points(face, out_p1, out_p2);
                            *out_n = cvt<S>(face.normal);
                            if (cnt) cnt->epa_exit = EXIT_NUMERIC;
                            track(cnt);
                            return true;
                        }
                        if (-dist > t.eps_tol) {
                            if (t.best_on_failure) return best_face(best_face_id, out_p1, out_p2, out_n, cnt);
                            if (cnt) cnt->status |= ST_EPA_FAILED;
                            track(cnt);
                            return false;
                        }
                        heap.push(FaceId<S>{new_face_id, -dist});
                    }
                }
            }
            if (first_new_face_id == faces.size()) {
                if (t.best_on_failure) return best_face(best_face_id, out_p1, out_p2, out_n, cnt);
                if (cnt) cnt->status |= ST_EPA_FAILED;
                track(cnt);
                return false;
            }
            faces[first_new_face_id].adj[2] = faces.size() - 1;
            faces.back().adj[1] = first_new_face_id;
            silhouette.clear();
            niter += 1;
            if (niter > max_iter) {
                if (cnt) cnt->status |= ST_EPA_MAX_ITER;
                track(cnt);
                return false;
            }
        }
        const Face<N>& bf = faces[best_face_id.id];
        face_closest_points(bf, out_p1, out_p2);
        *out_n = cvt<S>(bf.normal);
        if (cnt) cnt->epa_exit = EXIT_HEAP_EMPTY;
        track(cnt);
        return true;
    }
    // The PRECISE set's answer to a failed expansion step.
    bool best_face(const FaceId<S>& best, V3<S>* out_p1, V3<S>* out_p2, V3<S>* out_n, Counters* cnt) {
        const Face<N>& bf = faces[best.id];
        face_closest_points(bf, out_p1, out_p2);
        *out_n = cvt<S>(bf.normal);
        if (cnt) {
            cnt->status |= ST_EPA_PRECISION_LIMIT;
            cnt->epa_exit = EXIT_PRECISION;
        }
        track(cnt);
        return true;
    }
    void track(Counters* cnt) const {
        if (!cnt) return;
        if (cnt->epa_exit == EXIT_NONE) cnt->epa_exit = EXIT_FAILED;
        cnt->epa_max_vertices = std::max<uint32_t>(cnt->epa_max_vertices, (uint32_t)vertices.size());
        cnt->epa_max_faces = std::max<uint32_t>(cnt->epa_max_faces, (uint32_t)faces.size());
    }
};

// --------------------------------------------------------------- queries
template <class S> struct QueryOut {
    V3<S> p1, p2, dir;
    S value;     // depth (contact) or distance
    int tag;     // contact: 1 = Some; proximity: Proximity; closest: ClosestPoints tag
    int gjk_kind;
};

// contact_support_map_support_map_with_params (contact_support_map_support_map.rs:38-88)
// + Contact::new_wo_depth (contact.rs:43-46).
template <class N, class S>
QueryOut<S> contact(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2, S prediction,
                    const V3<N>* init_dir, const Tol<S>& tol, Counters* cnt) {
    QueryOut<S> o{};
    V3<N> dir;
    if (init_dir) dir = *init_dir;
    else if (!try_normalize(m2.t - m1.t, std::numeric_limits<N>::epsilon(), &dir, (N*)nullptr)) dir = v3<N>(N(1), N(0), N(0));
    VoronoiSimplex<N, S> simplex;
    simplex.reset(cso_from_shapes(m1, g1, m2, g2, dir, cnt));
    GJKResult<S> r = gjk_closest_points(m1, g1, m2, g2, prediction, true, simplex, tol, cnt);
    o.gjk_kind = r.kind;
    if (r.kind == GJK_INTERSECTION) {
        EPA<N, S> epa;
        V3<S> p1, p2, n;
        if (epa.closest_points(m1, g1, m2, g2, simplex, tol, &p1, &p2, &n, cnt)) {
            r.kind = GJK_CLOSEST_POINTS;
            r.p1 = p1; r.p2 = p2; r.dir = n;
        } else {
            r.kind = GJK_NO_INTERSECTION;
            r.dir = v3<S>(S(1), S(0), S(0));
        }
    }
    if (r.kind == GJK_CLOSEST_POINTS) {
        o.tag = 1;
        o.p1 = r.p1; o.p2 = r.p2; o.dir = r.dir;
        o.value = -dot(r.dir, r.p2 - r.p1);
    } else {
        o.tag = 0;
        o.dir = r.dir;
    }
    return o;
}

// distance_support_map_support_map_with_params (distance_support_map_support_map.rs:25-53).
template <class N, class S>
QueryOut<S> distance(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2,
                     const V3<N>* init_dir, const Tol<S>& tol, Counters* cnt) {
    QueryOut<S> o{};
    V3<N> d0 = init_dir ? *init_dir : (m1.t - m2.t);
    V3<N> dir;
    if (!try_normalize(d0, std::numeric_limits<N>::epsilon(), &dir, (N*)nullptr)) dir = v3<N>(N(1), N(0), N(0));
    VoronoiSimplex<N, S> simplex;
    simplex.reset(cso_from_shapes(m1, g1, m2, g2, dir, cnt));
    GJKResult<S> r = gjk_closest_points(m1, g1, m2, g2, std::numeric_limits<S>::max(), true, simplex, tol, cnt);
    o.gjk_kind = r.kind;
    if (r.kind == GJK_CLOSEST_POINTS) {
        o.value = norm(r.p2 - r.p1);
        o.p1 = r.p1; o.p2 = r.p2; o.dir = r.dir;
    } else {
        o.value = S(0);
    }
    return o;
}

// proximity_support_map_support_map_with_params (proximity_support_map_support_map.rs:37-75).
template <class N, class S>
QueryOut<S> proximity(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2, S margin,
                      const V3<N>* init_dir, const Tol<S>& tol, Counters* cnt) {
    QueryOut<S> o{};
    V3<N> dir;
    if (init_dir) dir = *init_dir;
    else if (!try_normalize(m2.t - m1.t, std::numeric_limits<N>::epsilon(), &dir, (N*)nullptr)) dir = v3<N>(N(1), N(0), N(0));
    VoronoiSimplex<N, S> simplex;
    simplex.reset(cso_from_shapes(m1, g1, m2, g2, dir, cnt));
    GJKResult<S> r = gjk_closest_points(m1, g1, m2, g2, margin, false, simplex, tol, cnt);
    o.gjk_kind = r.kind;
    if (r.kind == GJK_INTERSECTION) { o.tag = 0; o.dir = cvt<S>(dir); }
    else if (r.kind == GJK_PROXIMITY) { o.tag = 1; o.dir = r.dir; }
    else { o.tag = 2; o.dir = r.dir; }
    return o;
}

// closest_points_support_map_support_map_with_params (closest_points_support_map_support_map.rs:40-67).
template <class N, class S>
QueryOut<S> closest_points(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2, S prediction,
                           const V3<N>* init_dir, const Tol<S>& tol, Counters* cnt) {
    QueryOut<S> o{};
    V3<N> d0 = init_dir ? *init_dir : (m1.t - m2.t);
    V3<N> dir;
    if (!try_normalize(d0, std::numeric_limits<N>::epsilon(), &dir, (N*)nullptr)) dir = v3<N>(N(1), N(0), N(0));
    VoronoiSimplex<N, S> simplex;
    simplex.reset(cso_from_shapes(m1, g1, m2, g2, dir, cnt));
    GJKResult<S> r = gjk_closest_points(m1, g1, m2, g2, prediction, true, simplex, tol, cnt);
    o.gjk_kind = r.kind;
    if (r.kind == GJK_CLOSEST_POINTS) { o.tag = 1; o.p1 = r.p1; o.p2 = r.p2; o.dir = r.dir; }
    else if (r.kind == GJK_NO_INTERSECTION) { o.tag = 2; }
    else { o.tag = 0; }
    return o;
}

}  // namespace ncgo

namespace ncgo {

// ---------------------------------------------------- query::contact dispatch
// contact_shape_shape.rs:10-47 for the shapes of this library: Ball-Ball is
// analytic, Ball against a ConvexPolyhedron with PointQuery (Cuboid,
// ConvexHull) goes through point projection, every other pair (Capsule, Cone,
// Cylinder included) through contact_support_map_support_map.

// contact_ball_ball.rs:8-38 (Contact::new with the explicit depth).
template <class N, class S>
QueryOut<S> contact_ball_ball(V3<N> c1, N r1, V3<N> c2, N r2, S prediction) {
    QueryOut<S> o{};
    V3<S> a = cvt<S>(c1), b = cvt<S>(c2);
    V3<S> delta = b - a;
    S d2 = norm_sq(delta);
    S sum = S(r1) + S(r2);
    S se = sum + prediction;
    o.gjk_kind = -1;
    if (d2 < se * se) {
        using std::sqrt;
        V3<S> n = d2 != S(0) ? delta / norm(delta) : v3<S>(S(1), S(0), S(0));
        o.tag = 1;
        o.p1 = a + n * S(r1);
        o.p2 = b + n * (-S(r2));
        o.dir = n;
        o.value = sum - sqrt(d2);
    } else {
        o.tag = 0;
        o.dir = zero3<S>();
    }
    return o;
}

// Cuboid features (FeatureId): faces 0..5, edges, vertices.
enum FeatKind { F_UNKNOWN = 0, F_FACE = 1, F_EDGE = 2, F_VERTEX = 3 };

// point_aabb.rs:9-135 for the cuboid [-h, h] (solid = false), in N.
template <class N>
void aabb_project_with_feature(const Iso<N>& m, V3<N> h, V3<N> pt, bool* inside, V3<N>* proj, int* fkind,
                               int* fid) {
    V3<N> mins = zero3<N>() - h, maxs = zero3<N>() + h;
    V3<N> ls = inv_rotate(m.q, pt - m.t);  // Isometry::inverse_transform_point
    V3<N> mins_pt = mins - ls, pt_maxs = ls - maxs;
    auto sup0 = [](N x) { return x > N(0) ? x : N(0); };  // Vector::sup with zero
    N mp[3] = {mins_pt.x, mins_pt.y, mins_pt.z}, pm[3] = {pt_maxs.x, pt_maxs.y, pt_maxs.z};
    N shift[3] = {sup0(mp[0]) - sup0(pm[0]), sup0(mp[1]) - sup0(pm[1]), sup0(mp[2]) - sup0(pm[2])};
    bool in = shift[0] == N(0) && shift[1] == N(0) && shift[2] == N(0);
    if (in) {
        N best = -std::numeric_limits<N>::max();
        bool is_mins = false;
        int best_id = 0;
        for (int i = 0; i < 3; ++i) {
            if (mp[i] < pm[i]) {
                if (pm[i] > best) { best_id = i; is_mins = false; best = pm[i]; }
            } else if (mp[i] > best) {
                best_id = i; is_mins = true; best = mp[i];
            }
        }
        shift[0] = shift[1] = shift[2] = N(0);
        shift[best_id] = is_mins ? best : -best;
    }
    V3<N> lp{ls.x + shift[0], ls.y + shift[1], ls.z + shift[2]};
    *inside = in;
    *proj = transform_point(m, lp);
    N l[3] = {lp.x, lp.y, lp.z}, mx[3] = {maxs.x, maxs.y, maxs.z}, mn[3] = {mins.x, mins.y, mins.z};
    int nzero = 0, last_zero = 0, last_nonzero = 0;
    for (int i = 0; i < 3; ++i) {
        if (shift[i] == N(0)) { nzero++; last_zero = i; }
        else last_nonzero = i;
    }
    N eps = std::numeric_limits<N>::epsilon();
    N center[3] = {(mn[0] + mx[0]) * N(0.5), (mn[1] + mx[1]) * N(0.5), (mn[2] + mx[2]) * N(0.5)};
    if (nzero == 3) {
        for (int i = 0; i < 3; ++i) {
            if (l[i] > mx[i] - eps) { *fkind = F_FACE; *fid = i; return; }
            if (l[i] <= mn[i] + eps) { *fkind = F_FACE; *fid = i + 3; return; }
        }
        *fkind = F_UNKNOWN; *fid = 0;
    } else if (nzero == 2) {
        *fkind = F_FACE;
        *fid = l[last_nonzero] < center[last_nonzero] ? last_nonzero + 3 : last_nonzero;
    } else {
        int id = 0;
        for (int i = 0; i < 3; ++i)
            if (l[i] < center[i]) id |= 1 << i;
        if (nzero == 0) { *fkind = F_VERTEX; *fid = id; }
        else { *fkind = F_EDGE; *fid = (id << 2) | last_zero; }
    }
}

// cuboid.rs feature_normal (3-D), in the cuboid's local frame.
template <class N> V3<N> cuboid_feature_normal(int kind, int id) {
    N c[3] = {N(0), N(0), N(0)};
    if (kind == F_FACE) {
        if (id < 3) c[id] = N(1);
        else c[id - 3] = N(-1);
        return {c[0], c[1], c[2]};
    }
    if (kind == F_EDGE) {
        int edge = id & 3, f1 = (edge + 1) % 3, f2 = (edge + 2) % 3, signs = id >> 2;
        c[f1] = (signs & (1 << f1)) ? N(-1) : N(1);
        c[f2] = (signs & (1 << f2)) ? N(-1) : N(1);
    } else {
        for (int i = 0; i < 3; ++i) c[i] = (id & (1 << i)) ? N(-1) : N(1);
    }
    V3<N> v{c[0], c[1], c[2]};
    return v / norm(v);
}

// point_support_map.rs:15-53 (solid = false): GJK projection of the origin on
// the shape translated by -point, EPA when the point is inside.
template <class N, class S>
bool point_projection_on_support_map(const Iso<N>& m2, const Shape<N>& g, V3<N> point, const Tol<S>& tol,
                                     Counters* cnt, V3<S>* proj) {
    Iso<N> m{m2.q, (zero3<N>() - point) + m2.t};
    Iso<N> id{Quat<N>{N(0), N(0), N(0), N(1)}, zero3<N>()};
    Shape<N> origin{};
    origin.kind = CONSTANT_ORIGIN;
    V3<N> dir;
    if (!try_normalize(-m.t, std::numeric_limits<N>::epsilon(), &dir, (N*)nullptr)) dir = v3<N>(N(1), N(0), N(0));
    VoronoiSimplex<N, S> simplex;
    simplex.reset(cso_from_shapes(m, g, id, origin, dir, cnt));
    GJKResult<S> r = gjk_closest_points(m, g, id, origin, std::numeric_limits<S>::max(), true, simplex, tol, cnt);
    if (r.kind == GJK_CLOSEST_POINTS) {
        *proj = r.p1 + cvt<S>(point);
        return false;
    }
    if (r.kind != GJK_INTERSECTION && cnt) cnt->status |= ST_GJK_MAX_ITER;  // unreachable!() in gjk.rs:57
    EPA<N, S> epa;
    V3<S> p1, p2, n;
    if (r.kind == GJK_INTERSECTION && epa.closest_points(m, g, id, origin, simplex, tol, &p1, &p2, &n, cnt)) {
        *proj = p1 + cvt<S>(point);
        return true;
    }
    *proj = cvt<S>(point);
    return true;
}

// contact_ball_convex_polyhedron.rs:11-58 (and the flip of :65-77).
template <class N, class S>
QueryOut<S> contact_ball_polyhedron(V3<N> c, N r, const Iso<N>& m2, const Shape<N>& g2, S prediction,
                                    const Tol<S>& tol, Counters* cnt, bool flip) {
    QueryOut<S> o{};
    o.gjk_kind = -1;
    bool inside;
    V3<S> world2;
    int fkind = F_UNKNOWN, fid = 0;
    if (g2.kind == CUBOID) {
        V3<N> pr;
        aabb_project_with_feature(m2, v3<N>(g2.p0, g2.p1, g2.p2), c, &inside, &pr, &fkind, &fid);
        world2 = cvt<S>(pr);
    } else {
        inside = point_projection_on_support_map(m2, g2, c, tol, cnt, &world2);
    }
    V3<S> cs = cvt<S>(c);
    V3<S> dpt = world2 - cs;
    V3<S> dir, normal;
    S dist, depth;
    if (try_normalize(dpt, S(std::numeric_limits<N>::epsilon()), &dir, &dist)) {
        if (inside) { depth = dist + S(r); normal = -dir; }
        else { depth = -dist + S(r); normal = dir; }
    } else {
        // ConvexHull::project_point_with_feature needs the hull's face topology,
        // which this library does not build: the ball centre on the hull's
        // surface is reported as unsupported.
        if (g2.kind != CUBOID) { if (cnt) cnt->status |= ST_UNSUPPORTED_FEATURE; fkind = F_UNKNOWN; }
        if (fkind == F_UNKNOWN) { o.tag = 0; o.dir = zero3<S>(); return o; }
        depth = S(r);
        normal = -cvt<S>(cuboid_feature_normal<N>(fkind, fid));  // local normal, as the reference does
    }
    if (depth >= -prediction) {
        V3<S> world1 = cs + normal * S(r);
        o.tag = 1;
        o.value = depth;
        if (flip) { o.p1 = world2; o.p2 = world1; o.dir = -normal; }
        else { o.p1 = world1; o.p2 = world2; o.dir = normal; }
        return o;
    }
    o.tag = 0;
    o.dir = zero3<S>();
    return o;
}

template <class N, class S>
QueryOut<S> contact_query(const Iso<N>& m1, const Shape<N>& g1, const Iso<N>& m2, const Shape<N>& g2, S prediction,
                          const V3<N>* init_dir, const Tol<S>& tol, Counters* cnt) {
    bool b1 = g1.kind == BALL, b2 = g2.kind == BALL;
    bool p1 = g1.kind == CUBOID || g1.kind == CONVEX_HULL, p2 = g2.kind == CUBOID || g2.kind == CONVEX_HULL;
    if (b1 && b2) return contact_ball_ball<N, S>(m1.t, g1.p0, m2.t, g2.p0, prediction);
    if (b1 && p2) return contact_ball_polyhedron<N, S>(m1.t, g1.p0, m2, g2, prediction, tol, cnt, false);
    if (p1 && b2) return contact_ball_polyhedron<N, S>(m2.t, g2.p0, m1, g1, prediction, tol, cnt, true);
    return contact<N, S>(m1, g1, m2, g2, prediction, init_dir, tol, cnt);
}

}  // namespace ncgo
