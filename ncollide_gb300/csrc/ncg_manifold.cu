// ncg_manifold.cu — the contact-manifold step of
// ConvexPolyhedronConvexPolyhedronManifoldGenerator::generate_contacts
// (convex_polyhedron_convex_polyhedron_manifold_generator.rs:84-176) for pairs
// of Cuboid and ConvexHull shapes, one thread per pair, in f32 as the
// reference computes it: from the GJK/EPA contact, the support faces
// (penetrating) or the support features within the angular tolerances
// (separated) of both shapes (cuboid.rs:148-405; for a ConvexHull convex.rs:
// 383-546 over its face topology, built by ncg_hull.cpp), their polygonal
// clipping (convex_polygonal_feature3.rs:217-339) and the feature checks of
// add_contact_to_manifold (:341-400).
#include <cuda_runtime.h>

#include <cfloat>
#include <string>

#include "../../include/ncg.h"
#include "ncg_core.cuh"
#include "ncg_manifold.h"
#include "ncg_mlp.h"

namespace ncg {
namespace {

NCG_DEV uint32_t feat(uint32_t kind, uint32_t id) { return (kind << 28) | id; }

// A ConvexPolygonalFeature of at most NCG_POLY_MAX vertices.
struct Poly {
    int nv, ne, nn;
    vec3<float> v[NCG_POLY_MAX];
    uint32_t vid[NCG_POLY_MAX], eid[NCG_POLY_MAX];
    vec3<float> en[NCG_POLY_MAX];
    bool has_normal;
    vec3<float> normal;
    uint32_t feature;
    NCG_DEV void clear() {
        nv = ne = nn = 0;
        has_normal = false;
        normal = zero3<float>();
        feature = feat(NCG_FEATURE_UNKNOWN, 0);
    }
    NCG_DEV void push(vec3<float> p, uint32_t id) {
        v[nv] = p;
        vid[nv] = id;
        ++nv;
    }
    NCG_DEV int nedges() const { return nv == 1 ? 0 : (nv == 2 ? 1 : nv); }
};

NCG_DEV float comp(const vec3<float>& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
NCG_DEV void set_comp(vec3<float>& v, int i, float x) {
    if (i == 0) v.x = x;
    else if (i == 1) v.y = x;
    else v.z = x;
}
// Rust's f32::signum.
NCG_DEV float signum(float x) { return x != x ? x : copysignf(1.0f, x); }
NCG_DEV vec3<float> xform(const Pose& m, vec3<float> p) { return qrot(m.q, p) + m.t; }

// Cuboid::face (3-D) in the local frame, with its edge normals.
NCG_DEV void cuboid_face(vec3<float> h, uint32_t i, Poly& out) {
    out.clear();
    const uint32_t i1 = i < 3 ? i : i - 3;
    const float sign = i < 3 ? 1.0f : -1.0f;
    const uint32_t i2 = (i1 + 1) % 3, i3 = (i1 + 2) % 3;
    const uint32_t edge_i2 = sign > 0.0f ? i2 : i3, edge_i3 = sign > 0.0f ? i3 : i2;
    const uint32_t mask_i2 = ~(1u << edge_i2), mask_i3 = ~(1u << edge_i3);
    vec3<float> vertex = h;
    set_comp(vertex, i1, comp(vertex, i1) * sign);
    const uint32_t sbit = sign < 0.0f ? 1u : 0u, msbit = sign < 0.0f ? 0u : 1u;
    uint32_t vertex_id = sbit << i1;
    out.push(vertex, feat(NCG_FEATURE_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(NCG_FEATURE_EDGE, edge_i2 | ((vertex_id & mask_i2) << 2));
    set_comp(vertex, i2, -sign * comp(h, i2));
    set_comp(vertex, i3, sign * comp(h, i3));
    vertex_id |= msbit << i2 | sbit << i3;
    out.push(vertex, feat(NCG_FEATURE_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(NCG_FEATURE_EDGE, edge_i3 | ((vertex_id & mask_i3) << 2));
    set_comp(vertex, i2, -comp(h, i2));
    set_comp(vertex, i3, -comp(h, i3));
    vertex_id |= 1u << i2 | 1u << i3;
    out.push(vertex, feat(NCG_FEATURE_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(NCG_FEATURE_EDGE, edge_i2 | ((vertex_id & mask_i2) << 2));
    set_comp(vertex, i2, sign * comp(h, i2));
    set_comp(vertex, i3, -sign * comp(h, i3));
    vertex_id = sbit << i1 | sbit << i2 | msbit << i3;
    out.push(vertex, feat(NCG_FEATURE_VERTEX, vertex_id));
    out.eid[out.ne++] = feat(NCG_FEATURE_EDGE, edge_i3 | ((vertex_id & mask_i3) << 2));
    vec3<float> normal = zero3<float>();
    set_comp(normal, i1, sign);
    out.has_normal = true;
    out.normal = normal;
    out.feature = feat(NCG_FEATURE_FACE, sign > 0.0f ? i1 : i1 + 3);
    for (int a = 0; a < out.nv; ++a) {
        const int b = (a + 1) % out.nv;
        const vec3<float> sn = cross(out.v[b] - out.v[a], out.normal);
        vec3<float> u;
        float n;
        out.en[out.nn++] = try_normalize(sn, FLT_EPSILON, u, n) ? u : zero3<float>();
    }
}

// recompute_edge_normals (convex_polygonal_feature3.rs:162-176).
NCG_DEV void edge_normals(Poly& out) {
    out.nn = 0;
    for (int a = 0; a < out.nv; ++a) {
        const int b = (a + 1) % out.nv;
        const vec3<float> sn = cross(out.v[b] - out.v[a], out.normal);
        vec3<float> u;
        float n;
        out.en[out.nn++] = try_normalize(sn, FLT_EPSILON, u, n) ? u : zero3<float>();
    }
}

NCG_DEV void transform_by(Poly& f, const Pose& m) {
    for (int k = 0; k < f.nv; ++k) f.v[k] = xform(m, f.v[k]);
    for (int k = 0; k < f.nn; ++k) f.en[k] = qrot(m.q, f.en[k]);
    if (f.has_normal) f.normal = qrot(m.q, f.normal);
}

NCG_DEV void support_face_toward(const Pose& m, vec3<float> h, vec3<float> dir, Poly& out) {
    const vec3<float> l = qrot_inv(m.q, dir);
    int iamax = 0;
    float amax = fabsf(l.x);
    for (int i = 1; i < 3; ++i) {
        const float c = fabsf(comp(l, i));
        if (c > amax) {
            amax = c;
            iamax = i;
        }
    }
    cuboid_face(h, comp(l, iamax) > 0.0f ? (uint32_t)iamax : (uint32_t)iamax + 3, out);
    transform_by(out, m);
}

NCG_DEV void support_feature_toward(const Pose& m, vec3<float> h, vec3<float> dir, float cang, float sang, Poly& out) {
    const vec3<float> l = qrot_inv(m.q, dir);
    vec3<float> sp = h;
    out.clear();
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
            const vec3<float> p1 = sp;
            set_comp(sp, i, comp(h, i));
            const vec3<float> p2 = sp;
            const uint32_t p2_id = spid & ~(1u << i);
            out.push(xform(m, p1), feat(NCG_FEATURE_VERTEX, spid | (1u << i)));
            out.push(xform(m, p2), feat(NCG_FEATURE_VERTEX, p2_id));
            const uint32_t edge_id = feat(NCG_FEATURE_EDGE, (uint32_t)i | (p2_id << 2));
            out.eid[out.ne++] = edge_id;
            out.feature = edge_id;
            return;
        }
    }
    out.push(xform(m, sp), feat(NCG_FEATURE_VERTEX, spid));
    out.feature = feat(NCG_FEATURE_VERTEX, spid);
}

// ---- ConvexHull as a polyhedron (convex.rs:383-546) over its topology
NCG_DEV vec3<float> f3(float4 a) { return {a.x, a.y, a.z}; }
NCG_DEV vec3<float> hull_point(const ncg_batch& b, const Shape& s, uint32_t i) {
    return f3(__ldg(reinterpret_cast<const float4*>(b.hull_points) + s.off + i));
}
NCG_DEV vec3<float> hull_face_normal(const HullTopo& t, uint32_t f) {
    return f3(__ldg(reinterpret_cast<const float4*>(t.face_normal) + f));
}

// ConvexHull::face (convex.rs:453-470) in the local frame; false when the face
// has more vertices than a Poly holds.
NCG_DEV bool hull_face(const ncg_batch& b, const HullTopo& t, const Shape& s, uint32_t sid, uint32_t face, Poly& out) {
    out.clear();
    const uint32_t f = t.shape[4 * sid] + face;
    const uint32_t first = t.face_range[2 * f], count = t.face_range[2 * f + 1];
    if (count > NCG_POLY_MAX) return false;
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t vid = t.face_vertex[i];
        out.push(hull_point(b, s, vid), feat(NCG_FEATURE_VERTEX, vid));
        out.eid[out.ne++] = feat(NCG_FEATURE_EDGE, t.face_edge[i]);
    }
    out.normal = hull_face_normal(t, f);
    out.has_normal = true;
    out.feature = feat(NCG_FEATURE_FACE, face);
    edge_normals(out);
    return true;
}

// ConvexHull::support_face_toward (convex.rs:502-523): the face whose normal
// has the largest dot product with the direction (the first on ties).
NCG_DEV bool hull_support_face_toward(const ncg_batch& b, const HullTopo& t, const Shape& s, uint32_t sid,
                                      const Pose& m, vec3<float> dir, Poly& out) {
    const vec3<float> l = qrot_inv(m.q, dir);
    const uint32_t f0 = t.shape[4 * sid], nf = t.shape[4 * sid + 1];
    uint32_t best = 0;
    float max_dot = dot(hull_face_normal(t, f0), l);
    for (uint32_t i = 1; i < nf; ++i) {
        const float d = dot(hull_face_normal(t, f0 + i), l);
        if (d > max_dot) {
            max_dot = d;
            best = i;
        }
    }
    if (!hull_face(b, t, s, sid, best, out)) return false;
    transform_by(out, m);
    return true;
}

// ConvexHull::support_feature_toward (convex.rs:525-546) with
// support_feature_id_toward_eps (:383-416): the support point's first
// adjacent face whose normal is within the angle of the direction, else its
// first adjacent edge within the angle of orthogonal to it, else the vertex.
NCG_DEV bool hull_support_feature_toward(const ncg_batch& b, const HullTopo& t, const Shape& s, uint32_t sid,
                                         const Pose& m, vec3<float> dir, float cang, float sang, Poly& out) {
    out.clear();
    const vec3<float> l = qrot_inv(m.q, dir);
    const uint32_t sp = ThreadScan{reinterpret_cast<const float4*>(b.hull_points)}.argmax(s, l);
    const uint32_t f0 = t.shape[4 * sid], e0 = t.shape[4 * sid + 2];
    const size_t vr = 2 * ((size_t)s.off + sp);
    const uint32_t first = t.vertex_range[vr], count = t.vertex_range[vr + 1];
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t face = t.vertex_face[i];
        if (dot(hull_face_normal(t, f0 + face), l) >= cang) {
            if (!hull_face(b, t, s, sid, face, out)) return false;
            transform_by(out, m);
            return true;
        }
    }
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t edge = t.vertex_edge[i];
        const vec3<float> ed = f3(__ldg(reinterpret_cast<const float4*>(t.edge_dir) + e0 + edge));
        if (fabsf(dot(ed, l)) <= sang) {
            const uint32_t v1 = t.edge_vertex[2 * (e0 + edge)], v2 = t.edge_vertex[2 * (e0 + edge) + 1];
            out.push(hull_point(b, s, v1), feat(NCG_FEATURE_VERTEX, v1));
            out.push(hull_point(b, s, v2), feat(NCG_FEATURE_VERTEX, v2));
            out.feature = feat(NCG_FEATURE_EDGE, edge);
            out.eid[out.ne++] = out.feature;
            transform_by(out, m);
            return true;
        }
    }
    out.push(hull_point(b, s, sp), feat(NCG_FEATURE_VERTEX, sp));
    out.feature = feat(NCG_FEATURE_VERTEX, sp);
    transform_by(out, m);
    return true;
}

struct P2 {
    float x, y;
};

NCG_DEV bool point_in_poly2d(P2 pt, const P2* poly, int n) {
    if (n == 0) return false;
    float sign = 0.0f;
    for (int i1 = 0; i1 < n; ++i1) {
        const int i2 = (i1 + 1) % n;
        const P2 sd{poly[i2].x - poly[i1].x, poly[i2].y - poly[i1].y};
        const P2 dp{pt.x - poly[i1].x, pt.y - poly[i1].y};
        const float perp = dp.x * sd.y - dp.y * sd.x;
        if (sign == 0.0f) sign = perp;
        else if (sign * perp < 0.0f) return false;
    }
    return true;
}

// approx's ulps_eq! for f32 (epsilon f32::EPSILON, max_ulps 4).
NCG_DEV bool ulps_eq_f32(float a, float b) {
    if (fabsf(a - b) <= FLT_EPSILON) return true;
    if (signum(a) != signum(b)) return false;
    const uint32_t ia = __float_as_uint(a), ib = __float_as_uint(b);
    return (ia <= ib ? ib - ia : ia - ib) <= 4u;
}
NCG_DEV float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// closest_points_segment_segment_with_locations_nD (2-D): both closest points
// strictly inside their segments.
NCG_DEV bool seg_seg_on_edges(P2 a0, P2 a1, P2 b0, P2 b1, float& s, float& t) {
    const float eps = FLT_EPSILON;
    const P2 d1{a1.x - a0.x, a1.y - a0.y}, d2{b1.x - b0.x, b1.y - b0.y}, r{a0.x - b0.x, a0.y - b0.y};
    const float a = d1.x * d1.x + d1.y * d1.y;
    const float e = d2.x * d2.x + d2.y * d2.y;
    const float f = d2.x * r.x + d2.y * r.y;
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
    return s != 0.0f && s != 1.0f && t != 0.0f && t != 1.0f;
}

NCG_DEV float depth_wo(vec3<float> w1, vec3<float> w2, vec3<float> n) { return -dot(n, w2 - w1); }

NCG_DEV bool line_toi_with_plane(vec3<float> c, vec3<float> n, vec3<float> o, vec3<float> d, float& t) {
    const vec3<float> dpos = c - o;
    const float denom = dot(n, d);
    if (fabsf(denom) <= FLT_EPSILON) return false;
    t = dot(n, dpos) / denom;
    return true;
}

struct Out {
    ncg_manifold_point* pts;
    int n;
    bool full;
    NCG_DEV void emit(vec3<float> w1, vec3<float> w2, vec3<float> normal, float linear, uint32_t f1, uint32_t f2) {
        const float depth = depth_wo(w1, w2, normal);
        if (-depth <= linear && n >= NCG_MANIFOLD_MAX) full = true;
        if (-depth <= linear && n < NCG_MANIFOLD_MAX) {
            ncg_manifold_point& p = pts[n++];
            p.world1[0] = w1.x; p.world1[1] = w1.y; p.world1[2] = w1.z;
            p.world2[0] = w2.x; p.world2[1] = w2.y; p.world2[2] = w2.z;
            p.depth = depth;
            p.feature1 = f1;
            p.feature2 = f2;
        }
    }
};

NCG_DEV void clip(const Poly& f1, const Poly& f2, vec3<float> normal, float linear, Out& o) {
    if (f1.nv <= 2 && f2.nv <= 2) return;
    vec3<float> a = fabsf(normal.x) > fabsf(normal.y) ? vec3<float>{normal.z, 0.0f, -normal.x}
                                                     : vec3<float>{0.0f, -normal.z, normal.y};
    a = a / vnorm(a);
    const vec3<float> b0 = cross(a, normal), b1 = a;
    const vec3<float> ref = f1.v[0];
    P2 p1[NCG_POLY_MAX], p2[NCG_POLY_MAX];
    for (int k = 0; k < f1.nv; ++k) {
        const vec3<float> d = f1.v[k] - ref;
        p1[k] = P2{dot(b0, d), dot(b1, d)};
    }
    for (int k = 0; k < f2.nv; ++k) {
        const vec3<float> d = f2.v[k] - ref;
        p2[k] = P2{dot(b0, d), dot(b1, d)};
    }
    if (f2.nv > 2) {
        for (int i = 0; i < f1.nv; ++i) {
            if (!point_in_poly2d(p1[i], p2, f2.nv)) continue;
            const vec3<float> origin = (ref + b0 * p1[i].x) + b1 * p1[i].y;
            float toi2;
            if (line_toi_with_plane(f2.v[0], f2.normal, origin, normal, toi2))
                o.emit(f1.v[i], origin + normal * toi2, normal, linear, f1.vid[i], f2.feature);
        }
    }
    if (f1.nv > 2) {
        for (int i = 0; i < f2.nv; ++i) {
            if (!point_in_poly2d(p2[i], p1, f1.nv)) continue;
            const vec3<float> origin = (ref + b0 * p2[i].x) + b1 * p2[i].y;
            float toi1;
            if (line_toi_with_plane(f1.v[0], f1.normal, origin, normal, toi1))
                o.emit(origin + normal * toi1, f2.v[i], normal, linear, f1.feature, f2.vid[i]);
        }
    }
    const int ne1 = f1.nedges(), ne2 = f2.nedges();
    for (int i1 = 0; i1 < ne1; ++i1) {
        const int j1 = (i1 + 1) % f1.nv;
        for (int i2 = 0; i2 < ne2; ++i2) {
            const int j2 = (i2 + 1) % f2.nv;
            float s, t;
            if (!seg_seg_on_edges(p1[i1], p1[j1], p2[i2], p2[j2], s, t)) continue;
            const vec3<float> w1 = f1.v[i1] * (1.0f - s) + f1.v[j1] * s;
            const vec3<float> w2 = f2.v[i2] * (1.0f - t) + f2.v[j2] * t;
            o.emit(w1, w2, normal, linear, f1.eid[i1], f2.eid[i2]);
        }
    }
}

NCG_DEV bool feature_accepted(const Poly& f, uint32_t id) {
    const uint32_t kind = id >> 28;
    if (kind == NCG_FEATURE_UNKNOWN) return false;
    if (kind != NCG_FEATURE_EDGE) return true;
    for (int i = 0; i < f.nv && i < f.ne; ++i) {
        if (f.eid[i] != id) continue;
        return vnorm(f.v[(i + 1) % f.nv] - f.v[i]) > FLT_EPSILON;
    }
    return false;
}

// A shape's support face / feature toward a direction: Cuboid, or ConvexHull
// with its topology (false: no topology, or a face too large for a Poly).
NCG_DEV bool is_polyhedron(const Shape& s, uint32_t sid, const HullTopo& t) {
    if (s.kind == NCG_CUBOID) return true;
    return s.kind == NCG_CONVEX_HULL && t.shape != nullptr && t.shape[4 * sid + 1] > 0;
}
NCG_DEV bool face_toward(const ncg_batch& b, const HullTopo& t, const Shape& s, uint32_t sid, const Pose& m,
                         vec3<float> dir, Poly& out) {
    if (s.kind == NCG_CUBOID) {
        support_face_toward(m, vec3<float>{s.p0, s.p1, s.p2}, dir, out);
        return true;
    }
    return hull_support_face_toward(b, t, s, sid, m, dir, out);
}
NCG_DEV bool feature_toward(const ncg_batch& b, const HullTopo& t, const Shape& s, uint32_t sid, const Pose& m,
                            vec3<float> dir, float cang, float sang, Poly& out) {
    if (s.kind == NCG_CUBOID) {
        support_feature_toward(m, vec3<float>{s.p0, s.p1, s.p2}, dir, cang, sang, out);
        return true;
    }
    return hull_support_feature_toward(b, t, s, sid, m, dir, cang, sang, out);
}

__global__ void __launch_bounds__(128) k_manifold(ncg_batch b, const ncg_contact* contact, const uint8_t* has,
                                                  ManifoldParams mp, HullTopo topo, ncg_manifold* out,
                                                  uint32_t* status) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_pairs; i += stride) {
        ncg_manifold& o = out[i];
        if (!has[i]) {
            o.normal[0] = o.normal[1] = o.normal[2] = 0.0f;
            o.n = 0;
            continue;
        }
        const ncg_contact c = contact[i];
        const vec3<float> w1{c.world1[0], c.world1[1], c.world1[2]};
        const vec3<float> w2{c.world2[0], c.world2[1], c.world2[2]};
        const vec3<float> nn{c.normal[0], c.normal[1], c.normal[2]};
        o.normal[0] = nn.x;
        o.normal[1] = nn.y;
        o.normal[2] = nn.z;
        Shape s1, s2;
        const uint32_t id1 = b.g1[i], id2 = b.g2[i];
        const bool poly = load_shape(b, id1, s1) && load_shape(b, id2, s2) && is_polyhedron(s1, id1, topo) &&
                          is_polyhedron(s2, id2, topo);
        const Pose m1 = load_pose(b.m1 + i), m2 = load_pose(b.m2 + i);
        Poly f1, f2;
        const float depth = depth_wo(w1, w2, nn);
        bool ok = poly;
        if (ok) {
            if (depth > 0.0f) {
                ok = face_toward(b, topo, s1, id1, m1, nn, f1) && face_toward(b, topo, s2, id2, m2, -nn, f2);
            } else {
                ok = feature_toward(b, topo, s1, id1, m1, nn, mp.cang1, mp.sang1, f1) &&
                     feature_toward(b, topo, s2, id2, m2, -nn, mp.cang2, mp.sang2, f2);
            }
        }
        if (!ok) {
            ncg_manifold_point& p = o.points[0];
            p.world1[0] = w1.x; p.world1[1] = w1.y; p.world1[2] = w1.z;
            p.world2[0] = w2.x; p.world2[1] = w2.y; p.world2[2] = w2.z;
            p.depth = depth_wo(w1, w2, nn);
            p.feature1 = p.feature2 = 0u;
            o.n = 1;
            status[i] |= NCG_STATUS_NOT_POLYHEDRA;
            continue;
        }
        ncg_manifold_point tmp[NCG_MANIFOLD_MAX];
        Out t{tmp, 0, false};
        clip(f1, f2, nn, mp.linear, t);
        if (t.full) status[i] |= NCG_STATUS_MANIFOLD_FULL;
        if (t.n == 0) {
            ncg_manifold_point& p = tmp[t.n++];
            p.world1[0] = w1.x; p.world1[1] = w1.y; p.world1[2] = w1.z;
            p.world2[0] = w2.x; p.world2[1] = w2.y; p.world2[2] = w2.z;
            p.depth = depth;
            p.feature1 = f1.feature;
            p.feature2 = f2.feature;
        }
        int k = 0;
        for (int j = 0; j < t.n; ++j)
            if (feature_accepted(f1, tmp[j].feature1) && feature_accepted(f2, tmp[j].feature2)) o.points[k++] = tmp[j];
        o.n = (uint32_t)k;
    }
}

}  // namespace

int manifold_launch(const ncg_batch& b, const ncg_contact* contact, const uint8_t* has, const ManifoldParams& mp,
                    const HullTopo& topo, ncg_manifold* out, uint32_t* status, int num_sms, cudaStream_t st) {
    const uint64_t need = (b.n_pairs + 127) / 128;
    const uint64_t cap = (uint64_t)num_sms * 8;
    k_manifold<<<(unsigned)(need < cap ? need : cap), 128, 0, st>>>(b, contact, has, mp, topo, out, status);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("k_manifold launch: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    return NCG_OK;
}

}  // namespace ncg
