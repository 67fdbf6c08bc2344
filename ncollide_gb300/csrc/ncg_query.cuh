// ncg_query.cuh — query::contact's routing for Ball pairs
// (src/query/contact/contact_shape_shape.rs:10-47):
//   Ball-Ball            contact_ball_ball           (contact_ball_ball.rs:8-38)
//   Ball-Cuboid          contact_ball_convex_polyhedron with the cuboid's AABB
//                        point projection and features (point_aabb.rs:9-135,
//                        cuboid.rs feature_normal)
//   Ball-ConvexHull      contact_ball_convex_polyhedron with GJK/EPA point
//                        projection (point_support_map.rs:15-53)
// The ball contact and the AABB projection run in f32 (the reference's f32
// arithmetic); the point projection on a hull uses the GJK/EPA split and the
// assembly of the contact runs in double-word.
#pragma once

#include "ncg_core.cuh"

namespace ncg {

struct QContact {
    int tag;
    vec3<real> p1, p2, n;
    real depth;
    uint32_t status;
};

// contact_ball_ball.rs:8-38.
NCG_DEV QContact contact_ball_ball(vec3<float> c1, float r1, vec3<float> c2, float r2, real prediction) {
    QContact o;
    o.status = 0;
    vec3<real> a = to_r(c1), b = to_r(c2);
    vec3<real> delta = b - a;
    real d2 = norm_sq(delta);
    real sum = real(r1) + real(r2);
    real se = sum + prediction;
    if (d2 < se * se) {
        vec3<real> n = d2 != real(0.0f) ? delta / vnorm(delta) : mk(real(1.0f), real(0.0f), real(0.0f));
        o.tag = 1;
        o.p1 = a + n * real(r1);
        o.p2 = b + n * (-real(r2));
        o.n = n;
        o.depth = sum - sqrt(d2);
    } else {
        o.tag = 0;
        o.p1 = o.p2 = o.n = zero3<real>();
        o.depth = real(0.0f);
    }
    return o;
}

enum { F_UNKNOWN = 0, F_FACE = 1, F_EDGE = 2, F_VERTEX = 3 };

NCG_DEV float fsel(const float* a, int i) { return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]); }

// AABB [-h, h] projection with feature (solid = false), in f32.
NCG_DEV void aabb_project_with_feature(const Pose& m, vec3<float> h, vec3<float> pt, bool& inside,
                                       vec3<float>& proj, int& fkind, int& fid) {
    vec3<float> mins = zero3<float>() - h, maxs = zero3<float>() + h;
    vec3<float> ls = qrot_inv(m.q, pt - m.t);
    vec3<float> mp3 = mins - ls, pm3 = ls - maxs;
    float mp[3] = {mp3.x, mp3.y, mp3.z}, pm[3] = {pm3.x, pm3.y, pm3.z};
    float sh[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float a = mp[i] > 0.0f ? mp[i] : 0.0f;
        float b = pm[i] > 0.0f ? pm[i] : 0.0f;
        sh[i] = a - b;
    }
    bool in = sh[0] == 0.0f && sh[1] == 0.0f && sh[2] == 0.0f;
    if (in) {
        float best = -FLT_MAX;
        bool is_mins = false;
        int best_id = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (mp[i] < pm[i]) {
                if (pm[i] > best) { best_id = i; is_mins = false; best = pm[i]; }
            } else if (mp[i] > best) {
                best_id = i; is_mins = true; best = mp[i];
            }
        }
        float v = is_mins ? best : -best;
        sh[0] = best_id == 0 ? v : 0.0f;
        sh[1] = best_id == 1 ? v : 0.0f;
        sh[2] = best_id == 2 ? v : 0.0f;
    }
    vec3<float> lp{ls.x + sh[0], ls.y + sh[1], ls.z + sh[2]};
    inside = in;
    proj = qrot(m.q, lp) + m.t;
    float l[3] = {lp.x, lp.y, lp.z}, mx[3] = {maxs.x, maxs.y, maxs.z}, mn[3] = {mins.x, mins.y, mins.z};
    int nzero = 0, last_zero = 0, last_nonzero = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (sh[i] == 0.0f) { nzero++; last_zero = i; }
        else last_nonzero = i;
    }
    const float eps = FLT_EPSILON;
    float center[3] = {(mn[0] + mx[0]) * 0.5f, (mn[1] + mx[1]) * 0.5f, (mn[2] + mx[2]) * 0.5f};
    fkind = F_UNKNOWN;
    fid = 0;
    if (nzero == 3) {
        for (int i = 0; i < 3; ++i) {
            if (l[i] > mx[i] - eps) { fkind = F_FACE; fid = i; return; }
            if (l[i] <= mn[i] + eps) { fkind = F_FACE; fid = i + 3; return; }
        }
    } else if (nzero == 2) {
        fkind = F_FACE;
        fid = fsel(l, last_nonzero) < fsel(center, last_nonzero) ? last_nonzero + 3 : last_nonzero;
    } else {
        int id = 0;
        for (int i = 0; i < 3; ++i)
            if (l[i] < center[i]) id |= 1 << i;
        if (nzero == 0) { fkind = F_VERTEX; fid = id; }
        else { fkind = F_EDGE; fid = (id << 2) | last_zero; }
    }
}

// cuboid.rs feature_normal (3-D), in the cuboid's local frame.
NCG_DEV vec3<float> cuboid_feature_normal(int kind, int id) {
    float c[3] = {0.0f, 0.0f, 0.0f};
    if (kind == F_FACE) {
        float v = id < 3 ? 1.0f : -1.0f;
        int k = id < 3 ? id : id - 3;
        return {k == 0 ? v : 0.0f, k == 1 ? v : 0.0f, k == 2 ? v : 0.0f};
    }
    if (kind == F_EDGE) {
        int edge = id & 3, f1 = (edge + 1) % 3, f2 = (edge + 2) % 3, signs = id >> 2;
        float s1 = (signs & (1 << f1)) ? -1.0f : 1.0f, s2 = (signs & (1 << f2)) ? -1.0f : 1.0f;
        c[0] = f1 == 0 ? s1 : (f2 == 0 ? s2 : 0.0f);
        c[1] = f1 == 1 ? s1 : (f2 == 1 ? s2 : 0.0f);
        c[2] = f1 == 2 ? s1 : (f2 == 2 ? s2 : 0.0f);
    } else {
        c[0] = (id & 1) ? -1.0f : 1.0f;
        c[1] = (id & 2) ? -1.0f : 1.0f;
        c[2] = (id & 4) ? -1.0f : 1.0f;
    }
    vec3<float> v{c[0], c[1], c[2]};
    return v / vnorm(v);
}

// contact_ball_convex_polyhedron.rs:28-58 from the projection of the ball's
// centre; `flip` gives contact_convex_polyhedron_ball (:65-77).
NCG_DEV QContact ball_polyhedron_assemble(vec3<float> c, float r, bool inside, vec3<real> world2, int fkind,
                                          int fid, bool is_cuboid, real prediction, bool flip) {
    QContact o;
    o.status = 0;
    o.tag = 0;
    o.p1 = o.p2 = o.n = zero3<real>();
    o.depth = real(0.0f);
    vec3<real> cs = to_r(c);
    vec3<real> dpt = world2 - cs;
    vec3<real> dir, normal;
    real dist, depth;
    if (try_normalize(dpt, real(FLT_EPSILON), dir, dist)) {
        if (inside) { depth = dist + real(r); normal = -dir; }
        else { depth = -dist + real(r); normal = dir; }
    } else {
        if (!is_cuboid) { o.status |= NCG_STATUS_UNSUPPORTED_FEATURE; fkind = F_UNKNOWN; }
        if (fkind == F_UNKNOWN) return o;
        depth = real(r);
        normal = -to_r(cuboid_feature_normal(fkind, fid));
    }
    if (depth >= -prediction) {
        vec3<real> world1 = cs + normal * real(r);
        o.tag = 1;
        o.depth = depth;
        if (flip) { o.p1 = world2; o.p2 = world1; o.n = -normal; }
        else { o.p1 = world1; o.p2 = world2; o.n = normal; }
    }
    return o;
}

// The geometry of point_projection_on_support_map: the hull translated by
// -point against ConstantOrigin under the identity.
NCG_DEV PairGeom projection_geom(const Pose& hull_pose, const Shape& hull, vec3<float> point) {
    PairGeom g;
    g.m1 = Pose{hull_pose.q, (zero3<float>() - point) + hull_pose.t};
    g.g1 = hull;
    g.m2 = Pose{make_float4(0.0f, 0.0f, 0.0f, 1.0f), zero3<float>()};
    g.g2 = Shape{KIND_CONSTANT_ORIGIN, 0, 0, 0.0f, 0.0f, 0.0f};
    return g;
}

}  // namespace ncg
