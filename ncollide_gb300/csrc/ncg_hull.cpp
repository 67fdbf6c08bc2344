// ncg_hull.cpp — face topology of ConvexHull shapes, built once on the host
// (the shape set-up of ConvexHull::try_new, not part of a query).
//
// 1. The convex hull of a shape's points as a triangle mesh: an incremental
//    hull in f64 (the initial tetrahedron of extreme points, then every point
//    outside the current hull replaces the faces it sees by the fan from the
//    horizon), triangles counter-clockwise seen from outside.  The points stay
//    where they are (the hull's support map scans all of them), so point ids
//    are the shape's own.
// 2. ConvexHull::try_new (src/shape/convex.rs:88-328) on those points and
//    triangles, in f32 as the reference computes it: edges from the triangles'
//    sides (a sorted pair per edge), each with its unit direction
//    (Unit::try_new, None when |d| <= f32::EPSILON), triangle normals
//    (ccw_face_normal), edges between triangles whose normals differ by less
//    than sqrt(f32::EPSILON) deleted, polygonal faces extracted by following
//    the contours of the remaining edges, the faces and edges around each
//    vertex, and the Euler characteristic check.
// A hull whose points are degenerate (fewer than four, coplanar, collinear)
// or that fails a check of try_new gets no topology (its manifold falls back
// to the single contact of the contact query).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/ncg.h"

namespace ncg {
void set_last_error(const std::string& msg);
}

namespace {

// ---------------------------------------------------------------- 1. the hull
struct D3 {
    double x, y, z;
};
inline D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dotd(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 crossd(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double lend(D3 a) { return std::sqrt(dotd(a, a)); }

struct Tri {
    uint32_t v[3];
    D3 n;      // unit outward normal
    double d;  // n . v0
    bool alive;
};

inline uint64_t dkey(uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; }

// Triangles (counter-clockwise from outside) of the convex hull of p; false
// for degenerate input or an inconsistent mesh.
bool hull_triangles(const std::vector<D3>& p, std::vector<uint32_t>& out) {
    const uint32_t n = (uint32_t)p.size();
    out.clear();
    if (n < 4) return false;
    double scale = 0.0;
    for (const D3& q : p) scale = std::fmax(scale, std::fmax(std::fabs(q.x), std::fmax(std::fabs(q.y), std::fabs(q.z))));
    if (!(scale > 0.0) || !std::isfinite(scale)) return false;
    const double eps = 1e-10 * scale;
    // initial tetrahedron of extreme points
    uint32_t i0 = 0;
    for (uint32_t i = 1; i < n; ++i)
        if (p[i].x < p[i0].x) i0 = i;
    uint32_t i1 = i0;
    double best = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const double d = lend(sub(p[i], p[i0]));
        if (d > best) { best = d; i1 = i; }
    }
    if (best <= eps) return false;
    const D3 u = sub(p[i1], p[i0]);
    uint32_t i2 = i0;
    best = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const double d = lend(crossd(u, sub(p[i], p[i0]))) / lend(u);
        if (d > best) { best = d; i2 = i; }
    }
    if (best <= eps) return false;
    D3 pn = crossd(u, sub(p[i2], p[i0]));
    const double ln = lend(pn);
    pn = {pn.x / ln, pn.y / ln, pn.z / ln};
    uint32_t i3 = i0;
    best = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const double d = std::fabs(dotd(pn, sub(p[i], p[i0])));
        if (d > best) { best = d; i3 = i; }
    }
    if (best <= eps) return false;

    std::vector<Tri> tris;
    std::unordered_map<uint64_t, uint32_t> edge;  // directed edge a->b -> the triangle holding it
    auto add = [&](uint32_t a, uint32_t b, uint32_t c) -> bool {
        D3 nn = crossd(sub(p[b], p[a]), sub(p[c], p[a]));
        const double l = lend(nn);
        if (!(l > 0.0)) return false;
        nn = {nn.x / l, nn.y / l, nn.z / l};
        const uint32_t id = (uint32_t)tris.size();
        tris.push_back(Tri{{a, b, c}, nn, dotd(nn, p[a]), true});
        for (int k = 0; k < 3; ++k) {
            const uint64_t key = dkey(tris[id].v[k], tris[id].v[(k + 1) % 3]);
            if (edge.count(key)) return false;  // not a 2-manifold: give up
            edge[key] = id;
        }
        return true;
    };
    auto kill = [&](uint32_t id) {
        tris[id].alive = false;
        for (int k = 0; k < 3; ++k) edge.erase(dkey(tris[id].v[k], tris[id].v[(k + 1) % 3]));
    };
    // the tetrahedron, oriented outward
    const bool below = dotd(pn, sub(p[i3], p[i0])) < 0.0;
    const bool ok = below ? (add(i0, i1, i2) && add(i0, i3, i1) && add(i1, i3, i2) && add(i0, i2, i3))
                          : (add(i0, i2, i1) && add(i0, i1, i3) && add(i1, i2, i3) && add(i0, i3, i2));
    if (!ok) return false;
    std::vector<uint32_t> vis, horizon;
    std::vector<char> seen;
    for (uint32_t k = 0; k < n; ++k) {
        if (k == i0 || k == i1 || k == i2 || k == i3) continue;
        vis.clear();
        for (uint32_t t = 0; t < tris.size(); ++t)
            if (tris[t].alive && dotd(tris[t].n, p[k]) - tris[t].d > eps) vis.push_back(t);
        if (vis.empty()) continue;
        seen.assign(tris.size(), 0);
        for (uint32_t t : vis) seen[t] = 1;
        horizon.clear();
        for (uint32_t t : vis)
            for (int e = 0; e < 3; ++e) {
                const uint32_t a = tris[t].v[e], b = tris[t].v[(e + 1) % 3];
                auto it = edge.find(dkey(b, a));
                if (it == edge.end()) return false;
                if (!seen[it->second]) { horizon.push_back(a); horizon.push_back(b); }
            }
        for (uint32_t t : vis) kill(t);
        for (size_t h = 0; h < horizon.size(); h += 2)
            if (!add(horizon[h], horizon[h + 1], k)) return false;
    }
    for (const Tri& t : tris)
        if (t.alive) {
            out.push_back(t.v[0]);
            out.push_back(t.v[1]);
            out.push_back(t.v[2]);
        }
    return !out.empty();
}

// ---------------------------------------------------------------- 2. try_new
struct F3 {
    float x, y, z;
};
inline F3 fsub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 fcross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// Unit::try_new as restated for the whole path: None when |v| <= min_norm.
inline bool funit(F3 v, float min_norm, F3& out) {
    const float n = std::sqrt(fdot(v, v));
    if (n <= min_norm) return false;
    out = {v.x / n, v.y / n, v.z / n};
    return true;
}

struct HEdge {
    uint32_t v[2], f[2];
    F3 dir;
    bool deleted;
};
struct HTri {
    uint32_t v[3], e[3];
    F3 normal;
    int64_t parent;
};
struct HFace {
    uint32_t first, count;
    F3 normal;
};

struct Topo {
    std::vector<HFace> faces;
    std::vector<HEdge> edges;
    std::vector<uint32_t> fv, fe;                  // vertices / edges adjacent to faces
    std::vector<uint32_t> vfirst, vcount, vf, ve;  // per point: the faces / edges around it
};

// ConvexHull::try_new(points, indices) — convex.rs:88-328.
bool try_new(const std::vector<F3>& pts, const std::vector<uint32_t>& idx, Topo& o) {
    const float eps = std::sqrt(FLT_EPSILON);
    std::vector<HTri> tris;
    std::unordered_map<uint64_t, uint32_t> edge_map;  // SortedPair -> edge
    o = Topo();
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const uint32_t face_id = (uint32_t)tris.size();
        HTri tri;
        for (int i1 = 0; i1 < 3; ++i1) {
            const int i2 = (i1 + 1) % 3;
            const uint32_t a = idx[t + i1], b = idx[t + i2];
            const uint64_t key = a < b ? dkey(a, b) : dkey(b, a);
            auto it = edge_map.find(key);
            if (it != edge_map.end()) {
                tri.e[i1] = it->second;
                o.edges[it->second].f[1] = face_id;
            } else {
                F3 dir;
                if (!funit(fsub(pts[b], pts[a]), FLT_EPSILON, dir)) return false;
                tri.e[i1] = (uint32_t)o.edges.size();
                edge_map[key] = tri.e[i1];
                o.edges.push_back(HEdge{{a, b}, {face_id, 0}, dir, false});
            }
        }
        tri.v[0] = idx[t];
        tri.v[1] = idx[t + 1];
        tri.v[2] = idx[t + 2];
        // ccw_face_normal
        if (!funit(fcross(fsub(pts[tri.v[1]], pts[tri.v[0]]), fsub(pts[tri.v[2]], pts[tri.v[0]])), FLT_EPSILON,
                   tri.normal))
            return false;
        tri.parent = -1;
        tris.push_back(tri);
    }
    // edges between (nearly) coplanar triangles are deleted
    uint32_t num_valid_edges = 0;
    for (HEdge& e : o.edges) {
        if (fdot(tris[e.f[0]].normal, tris[e.f[1]].normal) > 1.0f - eps) e.deleted = true;
        else ++num_valid_edges;
    }
    // faces, by following contours
    auto next_edge_id = [&](const HTri& t, uint32_t id) -> int {
        for (int i = 0; i < 3; ++i)
            if (t.e[i] == id) return (i + 1) % 3;
        return -1;
    };
    for (size_t i = 0; i < tris.size(); ++i) {
        if (tris[i].parent >= 0) continue;
        for (int j1 = 0; j1 < 3; ++j1) {
            if (o.edges[tris[i].e[j1]].deleted) continue;
            const uint32_t new_face_id = (uint32_t)o.faces.size();
            HFace nf{(uint32_t)o.fe.size(), 1, tris[i].normal};
            o.fe.push_back(tris[i].e[j1]);
            o.fv.push_back(tris[i].v[j1]);
            const int j2 = (j1 + 1) % 3;
            const uint32_t start_vertex = tris[i].v[j1];
            size_t curr_triangle = i;
            int curr_edge_id = j2;
            size_t guard = 0;
            while (tris[curr_triangle].v[curr_edge_id] != start_vertex) {
                if (++guard > 4 * (o.edges.size() + 4)) return false;  // a contour that never closes
                const uint32_t curr_edge = tris[curr_triangle].e[curr_edge_id];
                const uint32_t curr_vertex = tris[curr_triangle].v[curr_edge_id];
                tris[curr_triangle].parent = new_face_id;
                if (!o.edges[curr_edge].deleted) {
                    o.fe.push_back(curr_edge);
                    o.fv.push_back(curr_vertex);
                    nf.count += 1;
                    curr_edge_id = (curr_edge_id + 1) % 3;
                } else {
                    const HEdge& ce = o.edges[curr_edge];
                    curr_triangle = ce.f[0] == curr_triangle ? ce.f[1] : ce.f[0];
                    curr_edge_id = next_edge_id(tris[curr_triangle], curr_edge);
                    if (curr_edge_id < 0 || tris[curr_triangle].v[curr_edge_id] != curr_vertex) return false;
                }
            }
            if (nf.count > 2) o.faces.push_back(nf);
            break;
        }
    }
    for (HEdge& e : o.edges) {
        if (tris[e.f[0]].parent >= 0) e.f[0] = (uint32_t)tris[e.f[0]].parent;
        if (tris[e.f[1]].parent >= 0) e.f[1] = (uint32_t)tris[e.f[1]].parent;
    }
    // the faces and edges around each vertex
    const size_t np = pts.size();
    o.vfirst.assign(np, 0);
    o.vcount.assign(np, 0);
    for (const HFace& f : o.faces)
        for (uint32_t k = f.first; k < f.first + f.count; ++k) o.vcount[o.fv[k]] += 1;
    uint32_t total = 0;
    for (size_t v = 0; v < np; ++v) {
        o.vfirst[v] = total;
        total += o.vcount[v];
    }
    o.vf.assign(total, 0);
    o.ve.assign(total, 0);
    std::fill(o.vcount.begin(), o.vcount.end(), 0u);
    for (uint32_t face_id = 0; face_id < o.faces.size(); ++face_id) {
        const HFace& f = o.faces[face_id];
        for (uint32_t k = f.first; k < f.first + f.count; ++k) {
            const uint32_t v = o.fv[k];
            o.vf[o.vfirst[v] + o.vcount[v]] = face_id;
            o.ve[o.vfirst[v] + o.vcount[v]] = o.fe[k];
            o.vcount[v] += 1;
        }
    }
    size_t num_valid_vertices = 0;
    for (size_t v = 0; v < np; ++v)
        if (o.vcount[v] != 0) ++num_valid_vertices;
    return num_valid_vertices + o.faces.size() - num_valid_edges == 2;
}

template <class T> T* dup(const std::vector<T>& v) {
    T* p = (T*)std::malloc(sizeof(T) * (v.empty() ? 1 : v.size()));
    if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
}

}  // namespace

extern "C" {

int ncg_hull_topology_build(const ncg_shape* shapes, uint32_t n_shapes, const float* hull_points,
                            uint64_t n_hull_points, ncg_hull_topology* out, uint32_t* n_failed) {
    if (!shapes || !out || (n_hull_points && !hull_points)) {
        ncg::set_last_error("ncg_hull_topology_build: null argument");
        return NCG_EINVAL;
    }
    std::memset(out, 0, sizeof(*out));
    std::vector<uint32_t> shape(4 * (size_t)n_shapes, 0u);
    std::vector<float> face_normal, edge_dir;
    std::vector<uint32_t> face_range, face_vertex, face_edge, edge_vertex, vertex_face, vertex_edge;
    std::vector<uint32_t> vertex_range(2 * (size_t)n_hull_points, 0u);
    uint32_t failed = 0;
    std::vector<D3> pd;
    std::vector<F3> pf;
    std::vector<uint32_t> tri;
    Topo t;
    for (uint32_t s = 0; s < n_shapes; ++s) {
        const ncg_shape& sh = shapes[s];
        if (sh.kind != NCG_CONVEX_HULL) continue;
        if ((uint64_t)sh.hull_off + sh.hull_n > n_hull_points) {
            ncg::set_last_error("ncg_hull_topology_build: hull slice past the end of the points");
            return NCG_EINVAL;
        }
        pd.resize(sh.hull_n);
        pf.resize(sh.hull_n);
        for (uint32_t i = 0; i < sh.hull_n; ++i) {
            const float* q = hull_points + 4 * ((size_t)sh.hull_off + i);
            pf[i] = F3{q[0], q[1], q[2]};
            pd[i] = D3{q[0], q[1], q[2]};
        }
        if (!hull_triangles(pd, tri) || !try_new(pf, tri, t)) {
            ++failed;
            continue;
        }
        shape[4 * (size_t)s + 0] = (uint32_t)(face_range.size() / 2);
        shape[4 * (size_t)s + 1] = (uint32_t)t.faces.size();
        shape[4 * (size_t)s + 2] = (uint32_t)(edge_vertex.size() / 2);
        shape[4 * (size_t)s + 3] = (uint32_t)t.edges.size();
        const uint32_t fslot0 = (uint32_t)face_vertex.size();
        for (const HFace& f : t.faces) {
            face_normal.insert(face_normal.end(), {f.normal.x, f.normal.y, f.normal.z, 0.0f});
            face_range.push_back(fslot0 + f.first);
            face_range.push_back(f.count);
        }
        face_vertex.insert(face_vertex.end(), t.fv.begin(), t.fv.end());
        face_edge.insert(face_edge.end(), t.fe.begin(), t.fe.end());
        for (const HEdge& e : t.edges) {
            edge_vertex.push_back(e.v[0]);
            edge_vertex.push_back(e.v[1]);
            edge_dir.insert(edge_dir.end(), {e.dir.x, e.dir.y, e.dir.z, 0.0f});
        }
        const uint32_t vslot0 = (uint32_t)vertex_face.size();
        for (uint32_t i = 0; i < sh.hull_n; ++i) {
            vertex_range[2 * ((size_t)sh.hull_off + i)] = vslot0 + t.vfirst[i];
            vertex_range[2 * ((size_t)sh.hull_off + i) + 1] = t.vcount[i];
        }
        vertex_face.insert(vertex_face.end(), t.vf.begin(), t.vf.end());
        vertex_edge.insert(vertex_edge.end(), t.ve.begin(), t.ve.end());
    }
    out->n_shapes = n_shapes;
    out->n_hull_points = n_hull_points;
    out->n_faces = face_range.size() / 2;
    out->n_face_slots = face_vertex.size();
    out->n_edges = edge_vertex.size() / 2;
    out->n_vertex_slots = vertex_face.size();
    out->shape = dup(shape);
    out->face_normal = dup(face_normal);
    out->face_range = dup(face_range);
    out->face_vertex = dup(face_vertex);
    out->face_edge = dup(face_edge);
    out->edge_vertex = dup(edge_vertex);
    out->edge_dir = dup(edge_dir);
    out->vertex_range = dup(vertex_range);
    out->vertex_face = dup(vertex_face);
    out->vertex_edge = dup(vertex_edge);
    if (n_failed) *n_failed = failed;
    return NCG_OK;
}

int ncg_hull_topology_release(ncg_hull_topology* t) {
    if (!t) return NCG_EINVAL;
    const void* ptrs[] = {t->shape, t->face_normal, t->face_range, t->face_vertex, t->face_edge,
                          t->edge_vertex, t->edge_dir, t->vertex_range, t->vertex_face, t->vertex_edge};
    for (const void* p : ptrs) std::free(const_cast<void*>(p));
    std::memset(t, 0, sizeof(*t));
    return NCG_OK;
}

}  // extern "C"
