// ncg_oracle_manifold.hpp — TEST INFRASTRUCTURE ONLY: CPU restatement (f32)
// of the contact-manifold step of ConvexPolyhedronConvexPolyhedronManifoldGenerator
// for pairs of Cuboid and ConvexHull shapes: from the GJK/EPA contact, the
// support features of both shapes toward the normal (a ConvexHull's over the
// face topology the library builds, src/shape/convex.rs:383-546), their
// polygonal clipping, and the contacts the generator pushes into the manifold.
//
// Reference (ncollide 0.33):
//   src/pipeline/narrow_phase/contact_generator/convex_polyhedron_convex_polyhedron_manifold_generator.rs:84-176
//   src/shape/cuboid.rs:148-405          vertex, edge, face, support_face_toward, support_feature_toward
//   src/shape/convex_polygonal_feature3.rs:90-400   transform_by, recompute_edge_normals, clip, edge,
//                                                   add_contact_to_manifold (feature checks)
//   src/utils/point_in_poly2d.rs:5-26, src/query/ray/ray_plane.rs:9-23 (line_toi_with_plane)
//   src/query/closest_points/closest_points_segment_segment.rs:44-141 (nD, with locations)
//   src/query/contact/contact.rs:43-46 (Contact::new_wo_depth)
// Third-party arithmetic restated from the published definitions: nalgebra
// 0.30's Vector3::orthonormal_subspace_basis (as in the EPA restatement),
// approx 0.5's relative_eq! / ulps_eq! defaults (epsilon = f32::EPSILON,
// max_relative = f32::EPSILON, max_ulps = 4) and Rust's f32::signum.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/ncg.h"
#include "ncg_oracle.hpp"

namespace ncgo {

enum { FEAT_UNKNOWN = 0, FEAT_VERTEX = 1, FEAT_EDGE = 2, FEAT_FACE = 3 };
inline uint32_t feat(int kind, uint32_t id) { return ((uint32_t)kind << 28) | id; }

constexpr int MANIFOLD_MAX = 16;
constexpr int POLY_MAX = 32;

struct ManifoldPoint {
    V3<float> w1, w2;
    float depth;
    uint32_t f1, f2;
};

struct PolyFeature {
    int nv = 0;
    V3<float> v[POLY_MAX];
    uint32_t vid[POLY_MAX];
    int ne = 0;  // edge feature ids pushed
    uint32_t eid[POLY_MAX];
    int nn = 0;  // edge normals pushed
    V3<float> en[POLY_MAX];
    bool has_normal = false;
    V3<float> normal;
    uint32_t feature = feat(FEAT_UNKNOWN, 0);

    void push(V3<float> p, uint32_t id) {
        v[nv] = p;
        vid[nv] = id;
        ++nv;
    }
    int nedges() const { return nv == 1 ? 0 : (nv == 2 ? 1 : nv); }
};

// Rust's f32::signum (NaN stays NaN).
inline float signum(float x) { return x != x ? x : std::copysign(1.0f, x); }

inline float comp(const V3<float>& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
inline void set_comp(V3<float>& v, int i, float x) { (i == 0 ? v.x : (i == 1 ? v.y : v.z)) = x; }

// Cuboid::face (cuboid.rs:185-277, 3-D branch) in the local frame.
inline void cuboid_face(const V3<float>& h, uint32_t i, PolyFeature& out) {
    out = PolyFeature();
    uint32_t i1;
    float sign;
    if (i < 3) { i1 = i; sign = 1.0f; }
    else { i1 = i - 3; sign = -1.0f; }
    const uint32_t i2 = (i1 + 1) % 3, i3 = (i1 + 2) % 3;
    const uint32_t edge_i2 = sign > 0.0f ? i2 : i3, edge_i3 = sign > 0.0f ? i3 : i2;
    const uint32_t mask_i2 = ~(1u << edge_i2), mask_i3 = ~(1u << edge_i3);
    V3<float> vertex = h;
    set_comp(vertex, i1, comp(vertex, i1) * sign);
    const uint32_t sbit = sign < 0.0f ? 1u : 0u, msbit = sign < 0.0f ? 0u : 1u;
    uint32_t vertex_id = sbit << i1;
    out.push(vertex, feat(FEAT_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(FEAT_EDGE, edge_i2 | ((vertex_id & mask_i2) << 2));
    set_comp(vertex, i2, -sign * comp(h, i2));
    set_comp(vertex, i3, sign * comp(h, i3));
    vertex_id |= msbit << i2 | sbit << i3;
    out.push(vertex, feat(FEAT_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(FEAT_EDGE, edge_i3 | ((vertex_id & mask_i3) << 2));
    set_comp(vertex, i2, -comp(h, i2));
    set_comp(vertex, i3, -comp(h, i3));
    vertex_id |= 1u << i2 | 1u << i3;
    out.push(vertex, feat(FEAT_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(FEAT_EDGE, edge_i2 | ((vertex_id & mask_i2) << 2));
    set_comp(vertex, i2, sign * comp(h, i2));
    set_comp(vertex, i3, -sign * comp(h, i3));
    vertex_id = sbit << i1 | sbit << i2 | msbit << i3;
    out.push(vertex, feat(FEAT_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(FEAT_EDGE, edge_i3 | ((vertex_id & mask_i3) << 2));
    V3<float> normal{0.0f, 0.0f, 0.0f};
    set_comp(normal, i1, sign);
    out.has_normal = true;
    out.normal = normal;
    out.feature = feat(FEAT_FACE, sign > 0.0f ? i1 : i1 + 3);
    // recompute_edge_normals (convex_polygonal_feature3.rs:162-176)
    out.nn = 0;
    for (int a = 0; a < out.nv; ++a) {
        const int b = (a + 1) % out.nv;
        const V3<float> sn = cross(out.v[b] - out.v[a], out.normal);
        V3<float> u;
        if (try_normalize(sn, std::numeric_limits<float>::epsilon(), &u, (float*)nullptr)) out.en[out.nn++] = u;
        else out.en[out.nn++] = zero3<float>();
    }
}

// ConvexPolygonalFeature::transform_by.
inline void transform_by(PolyFeature& f, const Iso<float>& m) {
    for (int k = 0; k < f.nv; ++k) f.v[k] = transform_point(m, f.v[k]);
    for (int k = 0; k < f.nn; ++k) f.en[k] = rotate(m.q, f.en[k]);
    if (f.has_normal) f.normal = rotate(m.q, f.normal);
}

// Cuboid::support_face_toward (cuboid.rs:279-307).
inline void cuboid_support_face_toward(const Iso<float>& m, const V3<float>& h, const V3<float>& dir,
                                       PolyFeature& out) {
    const V3<float> l = inverse_transform_vector(m, dir);
    int iamax = 0;
    float amax = std::fabs(l.x);
    for (int i = 1; i < 3; ++i) {
        const float c = std::fabs(comp(l, i));
        if (c > amax) { amax = c; iamax = i; }
    }
    cuboid_face(h, comp(l, iamax) > 0.0f ? (uint32_t)iamax : (uint32_t)iamax + 3, out);
    transform_by(out, m);
}

// Cuboid::support_feature_toward (cuboid.rs:309-405, 3-D branch) with the
// cosine and sine of the angular tolerance.
inline void cuboid_support_feature_toward(const Iso<float>& m, const V3<float>& h, const V3<float>& dir, float cang,
                                          float sang, PolyFeature& out) {
    const V3<float> l = inverse_transform_vector(m, dir);
    V3<float> sp = h;
    out = PolyFeature();
    uint32_t spid = 0;
    for (int i1 = 0; i1 < 3; ++i1) {
        const float sign = signum(comp(l, i1));
        if (sign * comp(l, i1) >= cang) {
            cuboid_face(h, sign > 0.0f ? (uint32_t)i1 : (uint32_t)i1 + 3, out);
            transform_by(out, m);
            return;
        } else if (sign < 0.0f) {
            set_comp(sp, i1, comp(sp, i1) * sign);
            spid |= 1u << i1;
        }
    }
    for (int i = 0; i < 3; ++i) {
        const float sign = signum(comp(l, i));
        if (sign * comp(l, i) <= sang) {
            set_comp(sp, i, -comp(h, i));
            const V3<float> p1 = sp;
            set_comp(sp, i, comp(h, i));
            const V3<float> p2 = sp;
            const uint32_t p2_id = spid & ~(1u << i);
            out.push(transform_point(m, p1), feat(FEAT_VERTEX, spid | (1u << i)));
            out.push(transform_point(m, p2), feat(FEAT_VERTEX, p2_id));
            const uint32_t edge_id = feat(FEAT_EDGE, (uint32_t)i | (p2_id << 2));
            out.eid[out.ne++] = edge_id;
            out.feature = edge_id;
            return;
        }
    }
    out.push(transform_point(m, sp), feat(FEAT_VERTEX, spid));
    out.feature = feat(FEAT_VERTEX, spid);
}

struct V2 {
    float x, y;
};

inline bool point_in_poly2d(V2 pt, const V2* poly, int n) {
    if (n == 0) return false;
    float sign = 0.0f;
    for (int i1 = 0; i1 < n; ++i1) {
        const int i2 = (i1 + 1) % n;
        const V2 sd{poly[i2].x - poly[i1].x, poly[i2].y - poly[i1].y};
        const V2 dp{pt.x - poly[i1].x, pt.y - poly[i1].y};
        const float perp = dp.x * sd.y - dp.y * sd.x;
        if (sign == 0.0f) sign = perp;
        else if (sign * perp < 0.0f) return false;
    }
    return true;
}

// approx::ulps_eq! for f32 with the default epsilon and max_ulps = 4.
inline bool ulps_eq_f32(float a, float b) {
    if (std::fabs(a - b) <= std::numeric_limits<float>::epsilon()) return true;
    if (signum(a) != signum(b)) return false;
    uint32_t ia, ib;
    std::memcpy(&ia, &a, 4);
    std::memcpy(&ib, &b, 4);
    return (ia <= ib ? ib - ia : ia - ib) <= 4u;
}

inline float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// closest_points_segment_segment_with_locations_nD (2-D): true when both
// closest points are inside their segments (OnEdge), with their barycentric
// second coordinates s and t.
inline bool segment_segment_on_edges(V2 a0, V2 a1, V2 b0, V2 b1, float* s_out, float* t_out) {
    const float eps = std::numeric_limits<float>::epsilon();
    const V2 d1{a1.x - a0.x, a1.y - a0.y}, d2{b1.x - b0.x, b1.y - b0.y}, r{a0.x - b0.x, a0.y - b0.y};
    const float a = d1.x * d1.x + d1.y * d1.y;
    const float e = d2.x * d2.x + d2.y * d2.y;
    const float f = d2.x * r.x + d2.y * r.y;
    float s, t;
    if (a <= eps && e <= eps) {
        s = 0.0f;
        t = 0.0f;
    } else if (a <= eps) {
        s = 0.0f;
        t = clamp01(f / e);
    } else {
        const float c = d1.x * r.x + d1.y * r.y;
        if (e <= eps) {
            t = 0.0f;
            s = clamp01(-c / a);
        } else {
            const float b = d1.x * d2.x + d1.y * d2.y;
            const float ae = a * e, bb = b * b;
            const float denom = ae - bb;
            const bool parallel = denom <= eps || ulps_eq_f32(ae, bb);
            s = parallel ? 0.0f : clamp01((b * f - c * e) / denom);
            t = (b * s + f) / e;
            if (t < 0.0f) {
                t = 0.0f;
                s = clamp01(-c / a);
            } else if (t > 1.0f) {
                t = 1.0f;
                s = clamp01((b - c) / a);
            }
        }
    }
    *s_out = s;
    *t_out = t;
    return s != 0.0f && s != 1.0f && t != 0.0f && t != 1.0f;
}

// Contact::new_wo_depth's depth.
inline float depth_wo(const V3<float>& w1, const V3<float>& w2, const V3<float>& n) { return -dot(n, w2 - w1); }

// line_toi_with_plane; relative_eq!(denom, 0) is |denom| <= f32::EPSILON.
inline bool line_toi_with_plane_f(V3<float> c, V3<float> n, V3<float> o, V3<float> d, float* t) {
    const V3<float> dpos = c - o;
    const float denom = dot(n, d);
    if (std::fabs(denom) <= std::numeric_limits<float>::epsilon()) return false;
    *t = dot(n, dpos) / denom;
    return true;
}

// ConvexPolygonalFeature::clip (convex_polygonal_feature3.rs:217-339).
inline int clip(const PolyFeature& f1, const PolyFeature& f2, const V3<float>& normal, float linear,
                ManifoldPoint* out, int n_out, bool* full = nullptr) {
    if (f1.nv <= 2 && f2.nv <= 2) return n_out;
    // nalgebra 0.30 orthonormal_subspace_basis of the normal: a, then a x normal first
    V3<float> a;
    if (std::fabs(normal.x) > std::fabs(normal.y)) a = v3<float>(normal.z, 0.0f, -normal.x);
    else a = v3<float>(0.0f, -normal.z, normal.y);
    a = a / norm(a);
    const V3<float> basis0 = cross(a, normal), basis1 = a;
    const V3<float> ref = f1.v[0];
    V2 p1[POLY_MAX], p2[POLY_MAX];
    for (int k = 0; k < f1.nv; ++k) {
        const V3<float> d = f1.v[k] - ref;
        p1[k] = V2{dot(basis0, d), dot(basis1, d)};
    }
    for (int k = 0; k < f2.nv; ++k) {
        const V3<float> d = f2.v[k] - ref;
        p2[k] = V2{dot(basis0, d), dot(basis1, d)};
    }
    auto emit = [&](V3<float> w1, V3<float> w2, uint32_t a1, uint32_t a2) {
        const float depth = depth_wo(w1, w2, normal);
        if (-depth <= linear && n_out >= MANIFOLD_MAX && full) *full = true;
        if (-depth <= linear && n_out < MANIFOLD_MAX) out[n_out++] = ManifoldPoint{w1, w2, depth, a1, a2};
    };
    if (f2.nv > 2) {
        for (int i = 0; i < f1.nv; ++i) {
            if (!point_in_poly2d(p1[i], p2, f2.nv)) continue;
            const V3<float> origin = (ref + basis0 * p1[i].x) + basis1 * p1[i].y;
            float toi2;
            if (line_toi_with_plane_f(f2.v[0], f2.normal, origin, normal, &toi2))
                emit(f1.v[i], origin + normal * toi2, f1.vid[i], f2.feature);
        }
    }
    if (f1.nv > 2) {
        for (int i = 0; i < f2.nv; ++i) {
            if (!point_in_poly2d(p2[i], p1, f1.nv)) continue;
            const V3<float> origin = (ref + basis0 * p2[i].x) + basis1 * p2[i].y;
            float toi1;
            if (line_toi_with_plane_f(f1.v[0], f1.normal, origin, normal, &toi1))
                emit(origin + normal * toi1, f2.v[i], f1.feature, f2.vid[i]);
        }
    }
    const int ne1 = f1.nedges(), ne2 = f2.nedges();
    for (int i1 = 0; i1 < ne1; ++i1) {
        const int j1 = (i1 + 1) % f1.nv;
        for (int i2 = 0; i2 < ne2; ++i2) {
            const int j2 = (i2 + 1) % f2.nv;
            float s, t;
            if (!segment_segment_on_edges(p1[i1], p1[j1], p2[i2], p2[j2], &s, &t)) continue;
            // Segment::point_at(OnEdge([1 - s, s]))
            const V3<float> w1 = f1.v[i1] * (1.0f - s) + f1.v[j1] * s;
            const V3<float> w2 = f2.v[i2] * (1.0f - t) + f2.v[j2] * t;
            emit(w1, w2, f1.eid[i1], f2.eid[i2]);
        }
    }
    return n_out;
}

// Segment::direction of the edge with id `e` of the feature is Some
// (add_contact_to_manifold drops contacts on zero-length edges).
inline bool edge_has_direction(const PolyFeature& f, uint32_t e) {
    for (int i = 0; i < f.nv && i < f.ne; ++i) {
        if (f.eid[i] != e) continue;
        const V3<float> d = f.v[(i + 1) % f.nv] - f.v[i];
        return norm(d) > std::numeric_limits<float>::epsilon();
    }
    return false;  // edge() returned None: the reference panics ("Invalid edge id.")
}
inline bool feature_accepted(const PolyFeature& f, uint32_t id) {
    const uint32_t kind = id >> 28;
    if (kind == FEAT_UNKNOWN) return false;
    if (kind == FEAT_EDGE) return edge_has_direction(f, id);
    return true;
}

// generate_contacts after the contact query: (w1, w2, normal) of the
// GJK/EPA ClosestPoints result; returns the number of contacts pushed.
inline int cuboid_manifold(const Iso<float>& m1, const V3<float>& h1, const Iso<float>& m2, const V3<float>& h2,
                           V3<float> w1, V3<float> w2, V3<float> normal, float linear, float cang1, float sang1,
                           float cang2, float sang2, ManifoldPoint* out) {
    PolyFeature f1, f2;
    const float depth = depth_wo(w1, w2, normal);
    if (depth > 0.0f) {
        cuboid_support_face_toward(m1, h1, normal, f1);
        cuboid_support_face_toward(m2, h2, -normal, f2);
    } else {
        cuboid_support_feature_toward(m1, h1, normal, cang1, sang1, f1);
        cuboid_support_feature_toward(m2, h2, -normal, cang2, sang2, f2);
    }
    ManifoldPoint tmp[MANIFOLD_MAX];
    int n = clip(f1, f2, normal, linear, tmp, 0);
    if (n == 0) tmp[n++] = ManifoldPoint{w1, w2, depth, f1.feature, f2.feature};
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (feature_accepted(f1, tmp[i].f1) && feature_accepted(f2, tmp[i].f2)) out[k++] = tmp[i];
    return k;
}

// ---- ConvexHull as a polyhedron over its topology (ncg_hull_topology, host
// arrays): ConvexHull::face, support_face_toward, support_feature_toward with
// support_feature_id_toward_eps (convex.rs:383-416, 453-470, 502-546).
struct HullView {
    const ncg_hull_topology* t;
    const float* pts;  // the batch's hull points, 4 floats each
    uint32_t off, n, sid;
    V3<float> point(uint32_t i) const {
        const float* q = pts + 4 * ((size_t)off + i);
        return {q[0], q[1], q[2]};
    }
    V3<float> face_normal(uint32_t f) const { return {t->face_normal[4 * f], t->face_normal[4 * f + 1], t->face_normal[4 * f + 2]}; }
};

inline bool hull_face(const HullView& h, uint32_t face, PolyFeature& out) {
    out = PolyFeature();
    const uint32_t f = h.t->shape[4 * h.sid] + face;
    const uint32_t first = h.t->face_range[2 * f], count = h.t->face_range[2 * f + 1];
    if (count > (uint32_t)POLY_MAX) return false;
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t vid = h.t->face_vertex[i];
        out.push(h.point(vid), feat(FEAT_VERTEX, vid));
        out.eid[out.ne++] = feat(FEAT_EDGE, h.t->face_edge[i]);
    }
    out.has_normal = true;
    out.normal = h.face_normal(f);
    out.feature = feat(FEAT_FACE, face);
    out.nn = 0;
    for (int a = 0; a < out.nv; ++a) {
        const int b = (a + 1) % out.nv;
        const V3<float> sn = cross(out.v[b] - out.v[a], out.normal);
        V3<float> u;
        if (try_normalize(sn, std::numeric_limits<float>::epsilon(), &u, (float*)nullptr)) out.en[out.nn++] = u;
        else out.en[out.nn++] = zero3<float>();
    }
    return true;
}

inline bool hull_support_face_toward(const HullView& h, const Iso<float>& m, const V3<float>& dir, PolyFeature& out) {
    const V3<float> l = inverse_transform_vector(m, dir);
    const uint32_t f0 = h.t->shape[4 * h.sid], nf = h.t->shape[4 * h.sid + 1];
    uint32_t best = 0;
    float max_dot = dot(h.face_normal(f0), l);
    for (uint32_t i = 1; i < nf; ++i) {
        const float d = dot(h.face_normal(f0 + i), l);
        if (d > max_dot) { max_dot = d; best = i; }
    }
    if (!hull_face(h, best, out)) return false;
    transform_by(out, m);
    return true;
}

inline bool hull_support_feature_toward(const HullView& h, const Iso<float>& m, const V3<float>& dir, float cang,
                                        float sang, PolyFeature& out) {
    out = PolyFeature();
    const V3<float> l = inverse_transform_vector(m, dir);
    // point_cloud_support_point_id: the first maximum
    uint32_t sp = 0;
    float best = dot(h.point(0), l);
    for (uint32_t i = 1; i < h.n; ++i) {
        const float d = dot(h.point(i), l);
        if (d > best) { best = d; sp = i; }
    }
    const uint32_t f0 = h.t->shape[4 * h.sid], e0 = h.t->shape[4 * h.sid + 2];
    const size_t vr = 2 * ((size_t)h.off + sp);
    const uint32_t first = h.t->vertex_range[vr], count = h.t->vertex_range[vr + 1];
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t face = h.t->vertex_face[i];
        if (dot(h.face_normal(f0 + face), l) >= cang) {
            if (!hull_face(h, face, out)) return false;
            transform_by(out, m);
            return true;
        }
    }
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t edge = h.t->vertex_edge[i];
        const float* d4 = h.t->edge_dir + 4 * ((size_t)e0 + edge);
        if (std::fabs(dot(V3<float>{d4[0], d4[1], d4[2]}, l)) <= sang) {
            const uint32_t v1 = h.t->edge_vertex[2 * ((size_t)e0 + edge)], v2 = h.t->edge_vertex[2 * ((size_t)e0 + edge) + 1];
            out.push(h.point(v1), feat(FEAT_VERTEX, v1));
            out.push(h.point(v2), feat(FEAT_VERTEX, v2));
            out.feature = feat(FEAT_EDGE, edge);
            out.eid[out.ne++] = out.feature;
            transform_by(out, m);
            return true;
        }
    }
    out.push(h.point(sp), feat(FEAT_VERTEX, sp));
    out.feature = feat(FEAT_VERTEX, sp);
    transform_by(out, m);
    return true;
}

// A Cuboid (h) or ConvexHull (hv) side of a pair.
struct PolySide {
    bool hull;
    V3<float> h;
    HullView hv;
};
inline bool side_face_toward(const PolySide& s, const Iso<float>& m, const V3<float>& dir, PolyFeature& out) {
    if (!s.hull) { cuboid_support_face_toward(m, s.h, dir, out); return true; }
    return hull_support_face_toward(s.hv, m, dir, out);
}
inline bool side_feature_toward(const PolySide& s, const Iso<float>& m, const V3<float>& dir, float cang, float sang,
                                PolyFeature& out) {
    if (!s.hull) { cuboid_support_feature_toward(m, s.h, dir, cang, sang, out); return true; }
    return hull_support_feature_toward(s.hv, m, dir, cang, sang, out);
}

// generate_contacts for a pair of polyhedra; -1 when a face does not fit a
// PolyFeature (the caller falls back to the single contact).
inline int poly_manifold(const Iso<float>& m1, const PolySide& a, const Iso<float>& m2, const PolySide& b, V3<float> w1,
                         V3<float> w2, V3<float> normal, float linear, float cang1, float sang1, float cang2,
                         float sang2, ManifoldPoint* out, bool* full) {
    PolyFeature f1, f2;
    const float depth = depth_wo(w1, w2, normal);
    bool ok;
    if (depth > 0.0f) ok = side_face_toward(a, m1, normal, f1) && side_face_toward(b, m2, -normal, f2);
    else ok = side_feature_toward(a, m1, normal, cang1, sang1, f1) && side_feature_toward(b, m2, -normal, cang2, sang2, f2);
    if (!ok) return -1;
    ManifoldPoint tmp[MANIFOLD_MAX];
    int n = clip(f1, f2, normal, linear, tmp, 0, full);
    if (n == 0) tmp[n++] = ManifoldPoint{w1, w2, depth, f1.feature, f2.feature};
    int k = 0;
    for (int i = 0; i < n; ++i)
        if (feature_accepted(f1, tmp[i].f1) && feature_accepted(f2, tmp[i].f2)) out[k++] = tmp[i];
    return k;
}

}  // namespace ncgo
