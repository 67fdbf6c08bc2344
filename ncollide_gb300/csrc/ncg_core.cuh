// ncg_core.cuh — device side of the batched narrow phase: vector math, the
// support maps, CSO points, the Voronoi simplex and the GJK loop.
//
// Arithmetic split: support mapping and CSO points in f32; the simplex
// sub-solve (segment / triangle / tetrahedron Voronoi projection), GJK's bound
// tests and the search direction in double-word arithmetic (`real`, see
// ncg_dw.cuh), which gives FP64-class precision on the FP32 pipes.  The library
// is compiled with -fmad=false and every expression keeps the reference's
// evaluation order, so a pair's result is a deterministic function of its
// inputs (no contraction, IEEE division and square root).
//
// Reference (ncollide 0.33): src/shape/support_map.rs:25-28,
// src/shape/{ball,cuboid,capsule,cone,cylinder}.rs, src/shape/convex.rs:418-423,
// src/utils/point_cloud_support_point.rs:6-33, src/query/algorithms/cso_point.rs:66-81,
// src/query/algorithms/voronoi_simplex3.rs:42-280, src/query/point/point_segment.rs:52-91,
// src/query/point/point_triangle.rs:61-309, src/query/point/point_tetrahedron.rs:35-353,
// src/query/algorithms/gjk.rs:76-177,367-388.
#pragma once

#include <cstdint>
#include <cfloat>

#include "../../include/ncg.h"

#define NCG_DEV __device__ __forceinline__
// Large double-word sub-solvers are kept out of line: inlined at every call
// site they overflow the instruction cache (warps of a thread-per-pair kernel
// sit in different sub-solver branches at the same time).
#define NCG_OUTLINE static __device__ __noinline__

#include "ncg_dw.cuh"

namespace ncg {

// The arithmetic of the sub-solve, GJK's bounds and EPA's distances: double-word
// (FP64-class on the FP32 pipes) by default; plain f32, the reference's own f32
// path, in the translation units built with NCG_REAL_F32.  The stage kernels
// and launchers of a translation unit live in namespace NCG_ARITH_NS (dwa or
// f32a), so that one library holds both builds of the GJK and EPA stages.
#ifdef NCG_REAL_F32
using real = f32r;
#define NCG_ARITH_NS f32a
#else
using real = dw;
#define NCG_ARITH_NS dwa
#endif
// A host-computed constant (split into two floats) in `real`.
NCG_DEV real from_host(dw_host x) { return real(x.h, x.l); }
NCG_DEV real dw_max() { return real(FLT_MAX); }

// ------------------------------------------------------------------ vectors
template <class T> struct vec3 {
    T x, y, z;
};
template <class T> NCG_DEV vec3<T> mk(T x, T y, T z) { return vec3<T>{x, y, z}; }
template <class T> NCG_DEV vec3<T> operator+(vec3<T> a, vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> NCG_DEV vec3<T> operator-(vec3<T> a, vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> NCG_DEV vec3<T> operator-(vec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> NCG_DEV vec3<T> operator*(vec3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> NCG_DEV vec3<T> operator/(vec3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> NCG_DEV T dot(vec3<T> a, vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> NCG_DEV vec3<T> cross(vec3<T> a, vec3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> NCG_DEV T norm_sq(vec3<T> a) { return dot(a, a); }
NCG_DEV float vnorm(vec3<float> a) { return __fsqrt_rn(norm_sq(a)); }
NCG_DEV real vnorm(vec3<real> a) { return sqrt(norm_sq(a)); }
NCG_DEV vec3<real> to_r(vec3<float> a) { return {real(a.x), real(a.y), real(a.z)}; }
NCG_DEV vec3<float> to_f(vec3<real> a) { return {a.x.h, a.y.h, a.z.h}; }
template <class T> NCG_DEV vec3<T> zero3() { return {T(0), T(0), T(0)}; }

// Unit::try_new_and_get: None when |v| <= min_norm.
template <class T> NCG_DEV bool try_normalize(vec3<T> v, T min_norm, vec3<T>& out, T& n) {
    n = vnorm(v);
    if (n <= min_norm) return false;
    out = v / n;
    return true;
}

// UnitQuaternion * Vector3: t = 2 (q.v x v); v' = (t*w + q.v x t) + v.
NCG_DEV vec3<float> qrot(float4 q, vec3<float> v) {
    vec3<float> qv{q.x, q.y, q.z};
    vec3<float> t = cross(qv, v) * 2.0f;
    vec3<float> c = cross(qv, t);
    return (t * q.w + c) + v;
}
NCG_DEV vec3<float> qrot_inv(float4 q, vec3<float> v) { return qrot(make_float4(-q.x, -q.y, -q.z, q.w), v); }

struct Pose {
    float4 q;
    vec3<float> t;
};
NCG_DEV Pose load_pose(const ncg_pose* p) {
    const float4* f = reinterpret_cast<const float4*>(p);
    float4 a = __ldg(f), b = __ldg(f + 1);
    return Pose{a, {b.x, b.y, b.z}};
}

struct Shape {
    uint32_t kind, off, n;
    float p0, p1, p2;
};
// Internal shape kind: ConstantOrigin (special_support_maps.rs:7-30), whose
// support point is the origin whatever the pose (point projection).
constexpr uint32_t KIND_CONSTANT_ORIGIN = 7;

// Validates and loads a shape record; returns false on a bad index or hull slice.
NCG_DEV bool load_shape(const ncg_batch& b, uint32_t id, Shape& s) {
    if (id >= b.n_shapes) return false;
    const uint4* r = reinterpret_cast<const uint4*>(b.shapes + id);
    uint4 h = __ldg(r);
    float4 p = __ldg(reinterpret_cast<const float4*>(r + 1));
    s.kind = h.x;
    s.off = h.y;
    s.n = h.z;
    s.p0 = p.x;
    s.p1 = p.y;
    s.p2 = p.z;
    if (s.kind > NCG_CONVEX_HULL) return false;
    if (s.kind == NCG_CONVEX_HULL && (s.n == 0 || (uint64_t)s.off + s.n > b.n_hull_points)) return false;
    return true;
}

// ------------------------------------------------------------------ hull scans
// point_cloud_support_point: arg-max of <p, d>, the first maximum wins.
struct ThreadScan {
    const float4* pts;
    NCG_DEV uint32_t argmax(const Shape& s, vec3<float> d) const {
        const float4* p = pts + s.off;
        float4 v = __ldg(p);
        float best = dot(vec3<float>{v.x, v.y, v.z}, d);
        uint32_t bi = 0;
        for (uint32_t i = 1; i < s.n; ++i) {
            v = __ldg(p + i);
            float x = dot(vec3<float>{v.x, v.y, v.z}, d);
            if (x > best) {
                best = x;
                bi = i;
            }
        }
        return bi;
    }
};

// Butterfly reduction of the lanes' (dot, index) keys, larger dot then smaller
// index, so that every lane gets the first maximum.  The serial scan starts
// from point 0's dot and keeps it when that dot is NaN (no comparison with a
// NaN is true): lane 0 reports that case (nan0) and the result is then 0.
NCG_DEV uint32_t warp_argmax_finish(float best, uint32_t bi, bool nan0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float ob = __shfl_xor_sync(0xffffffffu, best, o);
        uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        bool take = ob > best || (ob == best && oi < bi);
        if (take) {
            best = ob;
            bi = oi;
        }
    }
    return __shfl_sync(0xffffffffu, (int)nan0, 0) ? 0u : bi;
}

// All 32 lanes of a warp call argmax with the same arguments; lane l scans
// points l, l+32, ... (one coalesced 128-bit load per lane per step), then a
// butterfly reduction keeps (larger dot, smaller index) so every lane gets
// the first maximum, as the serial scan would.
struct WarpScan {
    const float4* pts;
    NCG_DEV uint32_t argmax(const Shape& s, vec3<float> d) const {
        const unsigned lane = threadIdx.x & 31u;
        const float4* p = pts + s.off;
        // Key (dot, index) ordered by larger dot then smaller index; NaN dots
        // rank as -inf so that every lane pair agrees (a strict total order).
        float best = -INFINITY;
        uint32_t bi = 0xffffffffu;
        bool nan0 = false;
        for (uint32_t i = lane; i < s.n; i += 32) {
            float4 v = __ldg(p + i);
            float x = dot(vec3<float>{v.x, v.y, v.z}, d);
            if (i == 0) nan0 = x != x;
            x = (x != x) ? -INFINITY : x;
            if (bi == 0xffffffffu || x > best) {
                best = x;
                bi = i;
            }
        }
        return warp_argmax_finish(best, bi, nan0);
    }
};

// WarpScan for a pair whose ConvexHull points (one or two slices of the flat
// point buffer) sit in the warp's shared-memory stage, copied there by the
// bulk-copy engine: up to two staged slices, identified by their first point
// and count; every other shape is scanned from global memory.  The points
// and the order of comparisons are those of WarpScan, so the arg-max is the
// same whichever memory the points come from.
struct StagedWarpScan {
    const float4* pts;
    uint32_t sbase;                // shared-memory address of the warp's stage
    uint32_t off[2], n[2], at[2];  // staged slice: first point, count (0: none), index in the stage
    NCG_DEV uint32_t argmax(const Shape& s, vec3<float> d) const {
        const int k = (n[0] != 0 && s.off == off[0] && s.n == n[0])   ? 0
                      : (n[1] != 0 && s.off == off[1] && s.n == n[1]) ? 1
                                                                       : -1;
        if (k < 0) return WarpScan{pts}.argmax(s, d);
        const unsigned lane = threadIdx.x & 31u;
        const uint32_t base = sbase + 16u * at[k];
        float best = -INFINITY;
        uint32_t bi = 0xffffffffu;
        bool nan0 = false;
        for (uint32_t i = lane; i < s.n; i += 32) {
            float4 v;
            // volatile: the stage is written by the async proxy; these reads
            // stay after the barrier wait that made it visible
            asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                         : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                         : "r"(base + 16u * i));
            float x = dot(vec3<float>{v.x, v.y, v.z}, d);
            if (i == 0) nan0 = x != x;
            x = (x != x) ? -INFINITY : x;
            if (bi == 0xffffffffu || x > best) {
                best = x;
                bi = i;
            }
        }
        return warp_argmax_finish(best, bi, nan0);
    }
};

// Local support functions.
template <class Scan> NCG_DEV vec3<float> local_support(const Shape& s, vec3<float> d, const Scan& scan) {
    switch (s.kind) {
    case NCG_BALL: {
        vec3<float> u = d / vnorm(d);
        return u * s.p0;
    }
    case NCG_CUBOID:
        return {copysignf(s.p0, d.x), copysignf(s.p1, d.y), copysignf(s.p2, d.z)};
    case NCG_CAPSULE: {
        vec3<float> u = d / vnorm(d);
        vec3<float> r{0.0f, copysignf(s.p0, u.y), 0.0f};
        return r + u * s.p1;
    }
    case NCG_CONE: {
        vec3<float> v{d.x, 0.0f, d.z};
        float n = vnorm(v);
        v = v / n;
        if (n == 0.0f) return {0.0f, copysignf(s.p0, d.y), 0.0f};
        v = v * s.p1;
        v.y = -s.p0;
        if (dot(d, v) < d.y * s.p0) return {0.0f, s.p0, 0.0f};
        return v;
    }
    case KIND_CONSTANT_ORIGIN:
        return zero3<float>();
    case NCG_CYLINDER: {
        vec3<float> v{d.x, 0.0f, d.z};
        float n = vnorm(v);
        v = v / n;
        if (n == 0.0f) v = zero3<float>();
        else v = v * s.p1;
        v.y = copysignf(s.p0, d.y);
        return v;
    }
    default: {
        uint32_t i = scan.argmax(s, d);
        float4 v = __ldg(scan.pts + s.off + i);
        return {v.x, v.y, v.z};
    }
    }
}

// World-space support point (Ball overrides the default transform).
template <class Scan>
NCG_DEV vec3<float> support_point(const Pose& m, const Shape& s, vec3<float> d, const Scan& scan) {
    if (s.kind == KIND_CONSTANT_ORIGIN) return zero3<float>();
    if (s.kind == NCG_BALL) {
        vec3<float> u = d / vnorm(d);
        return m.t + u * s.p0;
    }
    vec3<float> l = qrot_inv(m.q, d);
    return qrot(m.q, local_support(s, l, scan)) + m.t;
}

struct CSO {
    vec3<float> p, o1, o2;
};

struct PairGeom {
    Pose m1, m2;
    Shape g1, g2;
};

template <class Scan> NCG_DEV CSO cso_support(const PairGeom& g, vec3<float> d, const Scan& scan) {
    vec3<float> a = support_point(g.m1, g.g1, d, scan);
    vec3<float> b = support_point(g.m2, g.g2, -d, scan);
    return CSO{a - b, a, b};
}

// ------------------------------------------------------------------ tolerances
// gjk.rs:26-29, :92; epa3.rs:231-232; utils/triangle.rs:94-101.  Computed on
// the host in f64 from the chosen epsilon and split into double-words.
struct Tol {
    dw_host eps, eps_tol, eps_rel, epa_eps_tol, affine_eps;
    dw_host add_tol;                // VoronoiSimplex::add_point's degeneracy threshold
    float eps_tol_f, affine_eps_f;  // the same thresholds for the f32 EPA visibility test
    float init_eps;                 // f32::EPSILON: Unit::try_new on the initial direction
    int best_on_failure;            // PRECISE: a failed EPA expansion answers with the best face so far
};

// ------------------------------------------------------------------ projections
enum { LOC_VERTEX = 0, LOC_EDGE = 1, LOC_FACE = 2, LOC_SOLID = 3 };
template <class T> struct Loc {
    int kind, i;
    T b0, b1, b2;
};

template <class T> NCG_DEV vec3<T> proj_segment(vec3<T> a, vec3<T> b, Loc<T>& loc) {
    vec3<T> p = zero3<T>();
    vec3<T> ab = b - a, ap = p - a;
    T ab_ap = dot(ab, ap), sqnab = norm_sq(ab);
    if (ab_ap <= T(0.0f)) {
        loc = Loc<T>{LOC_VERTEX, 0, T(1.0f), T(0.0f), T(0.0f)};
        return a;
    } else if (ab_ap >= sqnab) {
        loc = Loc<T>{LOC_VERTEX, 1, T(1.0f), T(0.0f), T(0.0f)};
        return b;
    }
    T u = ab_ap / sqnab;
    loc = Loc<T>{LOC_EDGE, 0, T(1.0f) - u, u, T(0.0f)};
    return a + ab * u;
}

template <class T> NCG_DEV vec3<T> proj_triangle(vec3<T> a, vec3<T> b, vec3<T> c, Loc<T>& loc) {
    vec3<T> p = zero3<T>();
    vec3<T> ab = b - a, ac = c - a, ap = p - a;
    T ab_ap = dot(ab, ap), ac_ap = dot(ac, ap);
    if (ab_ap <= T(0.0f) && ac_ap <= T(0.0f)) {
        loc = Loc<T>{LOC_VERTEX, 0, T(1.0f), T(0.0f), T(0.0f)};
        return a;
    }
    vec3<T> bp = p - b;
    T ab_bp = dot(ab, bp), ac_bp = dot(ac, bp);
    if (ab_bp >= T(0.0f) && ac_bp <= ab_bp) {
        loc = Loc<T>{LOC_VERTEX, 1, T(1.0f), T(0.0f), T(0.0f)};
        return b;
    }
    vec3<T> cp = p - c;
    T ab_cp = dot(ab, cp), ac_cp = dot(ac, cp);
    if (ac_cp >= T(0.0f) && ab_cp <= ac_cp) {
        loc = Loc<T>{LOC_VERTEX, 2, T(1.0f), T(0.0f), T(0.0f)};
        return c;
    }
    vec3<T> bc = c - b;
    vec3<T> n = cross(ab, ac);
    T vc = dot(n, cross(ab, ap));
    if (vc < T(0.0f) && ab_ap >= T(0.0f) && ab_bp <= T(0.0f)) {
        T v = ab_ap / norm_sq(ab);
        loc = Loc<T>{LOC_EDGE, 0, T(1.0f) - v, v, T(0.0f)};
        return a + ab * v;
    }
    T vb = -dot(n, cross(ac, cp));
    if (vb < T(0.0f) && ac_ap >= T(0.0f) && ac_cp <= T(0.0f)) {
        T w = ac_ap / norm_sq(ac);
        loc = Loc<T>{LOC_EDGE, 2, T(1.0f) - w, w, T(0.0f)};
        return a + ac * w;
    }
    T va = dot(n, cross(bc, bp));
    if (va < T(0.0f) && ac_bp - ab_bp >= T(0.0f) && ab_cp - ac_cp >= T(0.0f)) {
        T w = dot(bc, bp) / norm_sq(bc);
        loc = Loc<T>{LOC_EDGE, 1, T(1.0f) - w, w, T(0.0f)};
        return b + bc * w;
    }
    int cw = dot(n, ap) >= T(0.0f) ? 0 : 1;
    if (va + vb + vc != T(0.0f)) {
        T denom = T(1.0f) / (va + vb + vc);
        T v = vb * denom, w = vc * denom;
        loc = Loc<T>{LOC_FACE, cw, T(1.0f) - v - w, v, w};
        return (a + ab * v) + ac * w;
    }
    loc = Loc<T>{LOC_SOLID, 0, T(0.0f), T(0.0f), T(0.0f)};
    return p;
}

struct EdgeTest {
    real d1, d2;
    bool hit;
    real u;
};
NCG_OUTLINE EdgeTest tet_edge(vec3<real> nabc, vec3<real> nabd, vec3<real> ap, vec3<real> ab, real ap_ab, real bp_ab) {
    EdgeTest r;
    real ab_ab = ap_ab - bp_ab;
    vec3<real> x = cross(ap, ab);
    r.d1 = dot(x, nabc);
    r.d2 = dot(x, nabd);
    r.hit = ab_ab != real(0.0f) && r.d1 >= real(0.0f) && r.d2 >= real(0.0f) && ap_ab >= real(0.0f) && ap_ab <= ab_ab;
    r.u = r.hit ? ap_ab / ab_ab : real(0.0f);
    return r;
}
NCG_OUTLINE bool tet_face(vec3<real> a, vec3<real> b, vec3<real> c, vec3<real> ap, vec3<real> bp, vec3<real> cp,
                      vec3<real> ab, vec3<real> ac, vec3<real> ad, real dabc, real dbca, real dacb, real eps,
                      vec3<real>& proj, real bc[3], uint32_t& status) {
    if (dabc < real(0.0f) && dbca < real(0.0f) && dacb < real(0.0f)) {
        vec3<real> n = cross(ab, ac);
        if (dot(n, ad) * dot(n, ap) < real(0.0f)) {
            vec3<real> nn;
            real len;
            if (!try_normalize(n, eps, nn, len)) return false;
            real vc = dot(nn, cross(ap, bp));
            real va = dot(nn, cross(bp, cp));
            real vb = dot(nn, cross(cp, ap));
            real denom = va + vb + vc;
            if (denom == real(0.0f)) status |= NCG_STATUS_DEGENERATE;
            real inv = real(1.0f) / denom;
            bc[0] = va * inv;
            bc[1] = vb * inv;
            bc[2] = vc * inv;
            proj = (a * bc[0] + b * bc[1]) + c * bc[2];
            return true;
        }
    }
    return false;
}
NCG_DEV vec3<real> proj_tetrahedron(vec3<real> a, vec3<real> b, vec3<real> c, vec3<real> d, real eps,
                                    Loc<real>& loc, uint32_t& status) {
    vec3<real> p = zero3<real>();
    vec3<real> ab = b - a, ac = c - a, ad = d - a, ap = p - a;
    real ap_ab = dot(ap, ab), ap_ac = dot(ap, ac), ap_ad = dot(ap, ad);
    if (ap_ab <= real(0.0f) && ap_ac <= real(0.0f) && ap_ad <= real(0.0f)) {
        loc = Loc<real>{LOC_VERTEX, 0, real(1.0f), real(0.0f), real(0.0f)};
        return a;
    }
    vec3<real> bc = c - b, bd = d - b, bp = p - b;
    real bp_bc = dot(bp, bc), bp_bd = dot(bp, bd), bp_ab = dot(bp, ab);
    if (bp_bc <= real(0.0f) && bp_bd <= real(0.0f) && bp_ab >= real(0.0f)) {
        loc = Loc<real>{LOC_VERTEX, 1, real(1.0f), real(0.0f), real(0.0f)};
        return b;
    }
    vec3<real> cd = d - c, cp = p - c;
    real cp_ac = dot(cp, ac), cp_bc = dot(cp, bc), cp_cd = dot(cp, cd);
    if (cp_cd <= real(0.0f) && cp_bc >= real(0.0f) && cp_ac >= real(0.0f)) {
        loc = Loc<real>{LOC_VERTEX, 2, real(1.0f), real(0.0f), real(0.0f)};
        return c;
    }
    vec3<real> dp = p - d;
    real dp_cd = dot(dp, cd), dp_bd = dot(dp, bd), dp_ad = dot(dp, ad);
    if (dp_ad >= real(0.0f) && dp_bd >= real(0.0f) && dp_cd >= real(0.0f)) {
        loc = Loc<real>{LOC_VERTEX, 3, real(1.0f), real(0.0f), real(0.0f)};
        return d;
    }
    vec3<real> nabc = cross(ab, ac), nabd = cross(ab, ad);
    EdgeTest e = tet_edge(nabc, nabd, ap, ab, ap_ab, bp_ab);
    if (e.hit) { loc = Loc<real>{LOC_EDGE, 0, real(1.0f) - e.u, e.u, real(0.0f)}; return a + ab * e.u; }
    real dabc = e.d1, dabd = e.d2;
    vec3<real> nacd = cross(ac, ad);
    e = tet_edge(nacd, -nabc, ap, ac, ap_ac, cp_ac);
    if (e.hit) { loc = Loc<real>{LOC_EDGE, 1, real(1.0f) - e.u, e.u, real(0.0f)}; return a + ac * e.u; }
    real dacd = e.d1, dacb = e.d2;
    e = tet_edge(-nabd, -nacd, ap, ad, ap_ad, dp_ad);
    if (e.hit) { loc = Loc<real>{LOC_EDGE, 2, real(1.0f) - e.u, e.u, real(0.0f)}; return a + ad * e.u; }
    real dadb = e.d1, dadc = e.d2;
    vec3<real> nbcd = cross(bc, bd);
    e = tet_edge(nabc, nbcd, bp, bc, bp_bc, cp_bc);
    if (e.hit) { loc = Loc<real>{LOC_EDGE, 3, real(1.0f) - e.u, e.u, real(0.0f)}; return b + bc * e.u; }
    real dbca = e.d1, dbcd = e.d2;
    e = tet_edge(-nbcd, nabd, bp, bd, bp_bd, dp_bd);
    if (e.hit) { loc = Loc<real>{LOC_EDGE, 4, real(1.0f) - e.u, e.u, real(0.0f)}; return b + bd * e.u; }
    real dbdc = e.d1, dbda = e.d2;
    e = tet_edge(nacd, nbcd, cp, cd, cp_cd, dp_cd);
    if (e.hit) { loc = Loc<real>{LOC_EDGE, 5, real(1.0f) - e.u, e.u, real(0.0f)}; return c + cd * e.u; }
    real dcda = e.d1, dcdb = e.d2;

    vec3<real> pr;
    real bw[3];
    if (tet_face(a, b, c, ap, bp, cp, ab, ac, ad, dabc, dbca, dacb, eps, pr, bw, status)) {
        loc = Loc<real>{LOC_FACE, 0, bw[0], bw[1], bw[2]};
        return pr;
    }
    if (tet_face(a, b, d, ap, bp, dp, ab, ad, ac, dadb, dabd, dbda, eps, pr, bw, status)) {
        loc = Loc<real>{LOC_FACE, 1, bw[0], bw[1], bw[2]};
        return pr;
    }
    if (tet_face(a, c, d, ap, cp, dp, ac, ad, ab, dacd, dcda, dadc, eps, pr, bw, status)) {
        loc = Loc<real>{LOC_FACE, 2, bw[0], bw[1], bw[2]};
        return pr;
    }
    if (tet_face(b, c, d, bp, cp, dp, bc, bd, -ab, dbcd, dcdb, dbdc, eps, pr, bw, status)) {
        loc = Loc<real>{LOC_FACE, 3, bw[0], bw[1], bw[2]};
        return pr;
    }
    loc = Loc<real>{LOC_SOLID, 0, real(0.0f), real(0.0f), real(0.0f)};
    return p;
}

// ------------------------------------------------------------------ simplex
struct Simplex {
    CSO v[4];
    real proj[3];
    real prev_proj[3];
    int prev_v[4];
    int dim, prev_dim;

    NCG_DEV vec3<real> pt(int i) const { return to_r(v[i].p); }
    NCG_DEV void swap(int i, int j) {
        CSO t = v[i];
        v[i] = v[j];
        v[j] = t;
        int k = prev_v[i];
        prev_v[i] = prev_v[j];
        prev_v[j] = k;
    }
    NCG_DEV void reset(const CSO& c) {
        dim = 0;
        prev_dim = 0;
        v[0] = c;
        prev_v[0] = 0; prev_v[1] = 1; prev_v[2] = 2; prev_v[3] = 3;
        proj[0] = proj[1] = proj[2] = real(0.0f);
        prev_proj[0] = prev_proj[1] = prev_proj[2] = real(0.0f);
    }
    NCG_DEV bool add_point(const CSO& c, const Tol& tol) {
        prev_dim = dim;
        prev_proj[0] = proj[0];
        prev_proj[1] = proj[1];
        prev_proj[2] = proj[2];
        prev_v[0] = 0; prev_v[1] = 1; prev_v[2] = 2; prev_v[3] = 3;
        vec3<real> ps = to_r(c.p);
        if (dim == 0) {
            if (norm_sq(pt(0) - ps) < from_host(tol.add_tol)) return false;
        } else if (dim == 1) {
            vec3<real> ab = pt(1) - pt(0), ac = ps - pt(0);
            if (norm_sq(cross(ab, ac)) < from_host(tol.add_tol)) return false;
        } else {
            vec3<real> ab = pt(1) - pt(0), ac = pt(2) - pt(0), ap = ps - pt(0);
            vec3<real> cr = cross(ab, ac);
            vec3<real> n = cr / vnorm(cr);
            if (fabs(dot(n, ap)) < from_host(tol.add_tol)) return false;
        }
        dim += 1;
        v[dim] = c;
        return true;
    }
    NCG_DEV vec3<real> project_origin_and_reduce(const Tol& tol, uint32_t& status) {
        if (dim == 0) {
            proj[0] = real(1.0f);
            return pt(0);
        } else if (dim == 1) {
            Loc<real> loc;
            vec3<real> r = proj_segment(pt(0), pt(1), loc);
            if (loc.kind == LOC_VERTEX && loc.i == 0) {
                proj[0] = real(1.0f);
                dim = 0;
            } else if (loc.kind == LOC_VERTEX) {
                swap(0, 1);
                proj[0] = real(1.0f);
                dim = 0;
            } else {
                proj[0] = loc.b0;
                proj[1] = loc.b1;
            }
            return r;
        } else if (dim == 2) {
            Loc<real> loc;
            vec3<real> r = proj_triangle(pt(0), pt(1), pt(2), loc);
            if (loc.kind == LOC_VERTEX) {
                swap(0, loc.i);
                proj[0] = real(1.0f);
                dim = 0;
            } else if (loc.kind == LOC_EDGE) {
                if (loc.i == 0) {
                    proj[0] = loc.b0;
                    proj[1] = loc.b1;
                } else if (loc.i == 1) {
                    swap(0, 2);
                    proj[0] = loc.b1;
                    proj[1] = loc.b0;
                } else {
                    swap(1, 2);
                    proj[0] = loc.b0;
                    proj[1] = loc.b1;
                }
                dim = 1;
            } else if (loc.kind == LOC_FACE) {
                proj[0] = loc.b0;
                proj[1] = loc.b1;
                proj[2] = loc.b2;
            }
            return r;
        }
        Loc<real> loc;
        vec3<real> r = proj_tetrahedron(pt(0), pt(1), pt(2), pt(3), from_host(tol.eps), loc, status);
        if (loc.kind == LOC_VERTEX) {
            swap(0, loc.i);
            proj[0] = real(1.0f);
            dim = 0;
        } else if (loc.kind == LOC_EDGE) {
            switch (loc.i) {
            case 1: swap(1, 2); break;
            case 2: swap(1, 3); break;
            case 3: swap(0, 2); break;
            case 4: swap(0, 3); break;
            case 5: swap(0, 2); swap(1, 3); break;
            default: break;
            }
            if (loc.i == 3 || loc.i == 4) {
                proj[0] = loc.b1;
                proj[1] = loc.b0;
            } else {
                proj[0] = loc.b0;
                proj[1] = loc.b1;
            }
            dim = 1;
        } else if (loc.kind == LOC_FACE) {
            if (loc.i == 0) {
                proj[0] = loc.b0; proj[1] = loc.b1; proj[2] = loc.b2;
            } else if (loc.i == 1) {
                v[2] = v[3];
                proj[0] = loc.b0; proj[1] = loc.b1; proj[2] = loc.b2;
            } else if (loc.i == 2) {
                v[1] = v[3];
                proj[0] = loc.b0; proj[1] = loc.b2; proj[2] = loc.b1;
            } else {
                v[0] = v[3];
                proj[0] = loc.b2; proj[1] = loc.b0; proj[2] = loc.b1;
            }
            dim = 2;
        }
        return r;
    }
};

// ------------------------------------------------------------------ GJK
enum { GJK_INTERSECTION = 0, GJK_CLOSEST_POINTS = 1, GJK_PROXIMITY = 2, GJK_NO_INTERSECTION = 3 };
struct GjkOut {
    int kind;
    vec3<real> p1, p2, dir;
};

NCG_DEV void gjk_result(const Simplex& s, bool prev, vec3<real>& p1, vec3<real>& p2) {
    vec3<real> r1 = zero3<real>(), r2 = zero3<real>();
    if (prev) {
        for (int i = 0; i < s.prev_dim + 1; ++i) {
            real c = s.prev_proj[i];
            const CSO& p = s.v[s.prev_v[i]];
            r1 = r1 + to_r(p.o1) * c;
            r2 = r2 + to_r(p.o2) * c;
        }
    } else {
        for (int i = 0; i < s.dim + 1; ++i) {
            real c = s.proj[i];
            const CSO& p = s.v[i];
            r1 = r1 + to_r(p.o1) * c;
            r2 = r2 + to_r(p.o2) * c;
        }
    }
    p1 = r1;
    p2 = r2;
}

// gjk::closest_points.  `iters` counts loop entries (one CSO support each).
template <class Scan>
NCG_DEV GjkOut gjk(const PairGeom& g, real max_dist, bool exact, Simplex& s, const Tol& tol, const Scan& scan,
                   uint32_t& iters, uint32_t& status, int max_iter) {
    GjkOut r;
    r.p1 = r.p2 = r.dir = zero3<real>();
    vec3<real> proj = s.project_origin_and_reduce(tol, status);
    vec3<real> old_dir, dir;
    {
        vec3<real> u;
        real n;
        if (try_normalize(proj, real(0.0f), u, n)) old_dir = -u;
        else { r.kind = GJK_INTERSECTION; return r; }
    }
    real max_bound = dw_max();
    const real eps_tol = from_host(tol.eps_tol), eps_rel = from_host(tol.eps_rel);
    int niter = 0;
    for (;;) {
        iters++;
        real old_max_bound = max_bound;
        {
            vec3<real> u;
            real n;
            if (try_normalize(-proj, eps_tol, u, n)) { dir = u; max_bound = n; }
            else { r.kind = GJK_INTERSECTION; return r; }
        }
        if (max_bound >= old_max_bound) {
            if (exact) { gjk_result(s, true, r.p1, r.p2); r.kind = GJK_CLOSEST_POINTS; }
            else r.kind = GJK_PROXIMITY;
            r.dir = old_dir;
            return r;
        }
        CSO c = cso_support(g, to_f(dir), scan);
        real min_bound = -dot(dir, to_r(c.p));
        if (min_bound != min_bound) status |= NCG_STATUS_BAD_INPUT;
        if (min_bound > max_dist) {
            r.kind = GJK_NO_INTERSECTION; r.dir = dir; return r;
        } else if (!exact && min_bound > real(0.0f) && max_bound <= max_dist) {
            r.kind = GJK_PROXIMITY; r.dir = old_dir; return r;
        } else if (max_bound - min_bound <= eps_rel * max_bound) {
            if (exact) { gjk_result(s, false, r.p1, r.p2); r.kind = GJK_CLOSEST_POINTS; }
            else r.kind = GJK_PROXIMITY;
            r.dir = dir;
            return r;
        }
        if (!s.add_point(c, tol)) {
            if (exact) { gjk_result(s, false, r.p1, r.p2); r.kind = GJK_CLOSEST_POINTS; }
            else r.kind = GJK_PROXIMITY;
            r.dir = dir;
            return r;
        }
        old_dir = dir;
        proj = s.project_origin_and_reduce(tol, status);
        if (s.dim == 3) {
            if (min_bound >= eps_tol) {
                if (exact) { gjk_result(s, true, r.p1, r.p2); r.kind = GJK_CLOSEST_POINTS; }
                else r.kind = GJK_PROXIMITY;
                r.dir = old_dir;
                return r;
            }
            r.kind = GJK_INTERSECTION;
            return r;
        }
        niter += 1;
        if (niter == max_iter) {
            status |= NCG_STATUS_GJK_MAX_ITER;
            r.kind = GJK_NO_INTERSECTION;
            r.dir = mk(real(1.0f), real(0.0f), real(0.0f));
            return r;
        }
    }
}

}  // namespace ncg
