// oracle_capi.cpp — TEST INFRASTRUCTURE ONLY: extern "C" batch driver of the
// oracle (ncg_oracle.hpp) for ctypes.  Reads the same packed inputs as the GPU
// library (include/ncg.h) and runs the reference algorithm per pair on
// std::threads (one static contiguous chunk of pairs per thread).
#include <cstring>
#include <thread>
#include <vector>

#include "../include/ncg.h"
#include "ncg_oracle.hpp"
#include "ncg_oracle_toi.hpp"
#include "ncg_oracle_bp.hpp"
#include "ncg_oracle_manifold.hpp"

using namespace ncgo;

namespace {

enum Policy { POLICY_F32 = 0, POLICY_F64 = 1, POLICY_MIXED = 2 };
enum Query { Q_CONTACT = 0, Q_DISTANCE = 1, Q_PROXIMITY = 2, Q_CLOSEST = 3, Q_CONTACT_QUERY = 4 };

// Inputs either in the library's f32 layout or as f64 arrays (known-answer tests
// use decimal literals that f32 cannot hold; the f64 oracle must see them exactly).
struct InF32 {
    const ncg_shape* shapes;
    uint32_t n_shapes;
    const float* pts;
    uint64_t n_pts;
    const ncg_pose* m1;
    const uint32_t* g1;
    const ncg_pose* m2;
    const uint32_t* g2;
    const float* init_dir;
};
struct InF64 {
    const int32_t* kinds;
    const uint32_t* hull_off;
    const uint32_t* hull_n;
    const double* params;  // 4 per shape
    uint32_t n_shapes;
    const double* pts;     // 4 per point
    uint64_t n_pts;
    const double* m1;      // 8 per pair: qi qj qk qw tx ty tz pad
    const uint32_t* g1;
    const double* m2;
    const uint32_t* g2;
    const double* init_dir;
};

template <class N> bool load_shape(const InF32& in, uint32_t id, Shape<N>* s) {
    if (id >= in.n_shapes) return false;
    const ncg_shape& r = in.shapes[id];
    s->kind = (int)r.kind;
    s->p0 = N(r.p[0]);
    s->p1 = N(r.p[1]);
    s->p2 = N(r.p[2]);
    s->pts4 = nullptr;
    s->pts4d = nullptr;
    s->n = 0;
    if (r.kind > NCG_CONVEX_HULL) return false;
    if (r.kind == NCG_CONVEX_HULL) {
        if (r.hull_n == 0 || (uint64_t)r.hull_off + r.hull_n > in.n_pts) return false;
        s->pts4 = in.pts + 4 * (uint64_t)r.hull_off;
        s->n = r.hull_n;
    }
    return true;
}
template <class N> bool load_shape(const InF64& in, uint32_t id, Shape<N>* s) {
    if (id >= in.n_shapes) return false;
    s->kind = in.kinds[id];
    s->p0 = N(in.params[4 * id]);
    s->p1 = N(in.params[4 * id + 1]);
    s->p2 = N(in.params[4 * id + 2]);
    s->pts4 = nullptr;
    s->pts4d = nullptr;
    s->n = 0;
    if (s->kind < 0 || s->kind > NCG_CONVEX_HULL) return false;
    if (s->kind == NCG_CONVEX_HULL) {
        if (in.hull_n[id] == 0 || (uint64_t)in.hull_off[id] + in.hull_n[id] > in.n_pts) return false;
        s->pts4d = in.pts + 4 * (uint64_t)in.hull_off[id];
        s->n = in.hull_n[id];
    }
    return true;
}
template <class N> Iso<N> load_pose(const ncg_pose& p) {
    return Iso<N>{Quat<N>{N(p.q[0]), N(p.q[1]), N(p.q[2]), N(p.q[3])}, V3<N>{N(p.t[0]), N(p.t[1]), N(p.t[2])}};
}
template <class N> Iso<N> load_pose(const double* p) {
    return Iso<N>{Quat<N>{N(p[0]), N(p[1]), N(p[2]), N(p[3])}, V3<N>{N(p[4]), N(p[5]), N(p[6])}};
}
template <class N> Iso<N> pose1(const InF32& in, uint64_t i) { return load_pose<N>(in.m1[i]); }
template <class N> Iso<N> pose2(const InF32& in, uint64_t i) { return load_pose<N>(in.m2[i]); }
template <class N> Iso<N> pose1(const InF64& in, uint64_t i) { return load_pose<N>(in.m1 + 8 * i); }
template <class N> Iso<N> pose2(const InF64& in, uint64_t i) { return load_pose<N>(in.m2 + 8 * i); }
// An all-zero init_dir entry means "no init_dir" (the reference's None): no
// unit vector is zero, so this extends the reference's inputs without changing
// any of them (a cached direction a proximity detector has dropped).
template <class N> bool init_dir(const InF32& in, uint64_t i, V3<N>* d) {
    if (!in.init_dir) return false;
    if (in.init_dir[3 * i] == 0.0f && in.init_dir[3 * i + 1] == 0.0f && in.init_dir[3 * i + 2] == 0.0f) return false;
    *d = V3<N>{N(in.init_dir[3 * i]), N(in.init_dir[3 * i + 1]), N(in.init_dir[3 * i + 2])};
    return true;
}
template <class N> bool init_dir(const InF64& in, uint64_t i, V3<N>* d) {
    if (!in.init_dir) return false;
    if (in.init_dir[3 * i] == 0.0 && in.init_dir[3 * i + 1] == 0.0 && in.init_dir[3 * i + 2] == 0.0) return false;
    *d = V3<N>{N(in.init_dir[3 * i]), N(in.init_dir[3 * i + 1]), N(in.init_dir[3 * i + 2])};
    return true;
}

struct Outs {
    double* out16;
    uint8_t* tag;
    uint32_t* status;
    uint32_t* counters8;
};

template <class N, class S, class In>
void run_range(const In& in, int query, S param, const Tol<S>& tol, uint64_t lo, uint64_t hi, const Outs& o) {
    for (uint64_t i = lo; i < hi; ++i) {
        Counters cnt;
        Shape<N> s1, s2;
        QueryOut<S> r{};
        bool ok = load_shape<N>(in, in.g1[i], &s1) && load_shape<N>(in, in.g2[i], &s2);
        if (!ok) {
            cnt.status |= ST_BAD_INPUT;
        } else {
            Iso<N> m1 = pose1<N>(in, i), m2 = pose2<N>(in, i);
            V3<N> d;
            const V3<N>* dp = init_dir<N>(in, i, &d) ? &d : nullptr;
            switch (query) {
            case Q_CONTACT: r = contact<N, S>(m1, s1, m2, s2, param, dp, tol, &cnt); break;
            case Q_DISTANCE: r = distance<N, S>(m1, s1, m2, s2, dp, tol, &cnt); break;
            case Q_PROXIMITY: r = proximity<N, S>(m1, s1, m2, s2, param, dp, tol, &cnt); break;
            case Q_CONTACT_QUERY: r = contact_query<N, S>(m1, s1, m2, s2, param, dp, tol, &cnt); break;
            default: r = closest_points<N, S>(m1, s1, m2, s2, param, dp, tol, &cnt); break;
            }
        }
        if (o.out16) {
            double* w = o.out16 + 16 * i;
            // double-word values are reported by their high word (the f32
            // the kernels write out)
            w[0] = double(r.p1.x); w[1] = double(r.p1.y); w[2] = double(r.p1.z);
            w[3] = double(r.p2.x); w[4] = double(r.p2.y); w[5] = double(r.p2.z);
            w[6] = double(r.dir.x); w[7] = double(r.dir.y); w[8] = double(r.dir.z);
            w[9] = double(r.value);
            w[10] = r.gjk_kind;
            for (int k = 11; k < 16; ++k) w[k] = 0.0;
        }
        if (o.tag) o.tag[i] = (uint8_t)r.tag;
        if (o.status) o.status[i] = cnt.status;
        if (o.counters8) {
            uint32_t* c = o.counters8 + 8 * i;
            c[0] = cnt.gjk_iters;
            c[1] = cnt.epa_iters;
            c[2] = cnt.support_calls;
            c[3] = cnt.hull_points_scanned;
            c[4] = cnt.faces_created;
            c[5] = cnt.epa_max_vertices;
            c[6] = cnt.epa_max_faces;
            c[7] = (cnt.subsolve[0] + cnt.subsolve[1] + cnt.subsolve[2] + cnt.subsolve[3]) | (cnt.epa_exit << 24);
        }
    }
}

template <class N, class S, class In>
int run(const In& in, uint64_t n_pairs, int query, double param, double eps, double epa_tol, int n_threads,
        const Outs& o) {
    // eps < 0 selects the PRECISE tolerance set (make_tol_precise).
    double e = eps > 0 ? eps : (double)std::numeric_limits<N>::epsilon();
    Tol<S> tol = eps < 0 ? make_tol_precise<S>(epa_tol > 0 ? epa_tol : 0.0) : make_tol<S>(e, epa_tol > 0 ? epa_tol : 0.0);
    S p = S(param);
    if (n_threads <= 1 || n_pairs < 64) {
        run_range<N, S>(in, query, p, tol, 0, n_pairs, o);
        return 0;
    }
    std::vector<std::thread> th;
    uint64_t chunk = (n_pairs + n_threads - 1) / n_threads;
    for (int t = 0; t < n_threads; ++t) {
        uint64_t lo = t * chunk, hi = std::min<uint64_t>(n_pairs, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([&, lo, hi] { run_range<N, S>(in, query, p, tol, lo, hi, o); });
    }
    for (auto& x : th) x.join();
    return 0;
}

template <class In>
int dispatch(int policy, const In& in, uint64_t n, int query, double param, double eps, double epa_tol, int nt,
             const Outs& o) {
    if (query == Q_PROXIMITY && param < 0) return NCG_EINVAL;
    switch (policy) {
    case POLICY_F32: return run<float, float>(in, n, query, param, eps, epa_tol, nt, o);
    case POLICY_F64: return run<double, double>(in, n, query, param, eps, epa_tol, nt, o);
    case POLICY_MIXED: return run<float, dw>(in, n, query, param, eps, epa_tol, nt, o);
    default: return NCG_EINVAL;
    }
}

template <class N, class S>
void toi_range(const InF32& in, const float* vel1, const float* vel2, int dispatch, S max_toi, N target,
               const Tol<S>& tol, uint64_t lo, uint64_t hi, const Outs& o) {
    for (uint64_t i = lo; i < hi; ++i) {
        Counters cnt;
        Shape<N> s1, s2;
        TOIOut<S> r;
        bool ok = load_shape<N>(in, in.g1[i], &s1) && load_shape<N>(in, in.g2[i], &s2);
        if (!ok) {
            cnt.status |= ST_BAD_INPUT;
        } else {
            Iso<N> m1 = pose1<N>(in, i), m2 = pose2<N>(in, i);
            V3<N> v1{N(vel1[3 * i]), N(vel1[3 * i + 1]), N(vel1[3 * i + 2])};
            V3<N> v2{N(vel2[3 * i]), N(vel2[3 * i + 1]), N(vel2[3 * i + 2])};
            if (dispatch == 1 && s1.kind == BALL && s2.kind == BALL)
                r = toi_ball_ball<N, S>(m1, v1, s1.p0, m2, v2, s2.p0, max_toi, target);
            else
                r = toi_support_map<N, S>(m1, v1, s1, m2, v2, s2, max_toi, target, tol, &cnt);
        }
        if (o.out16) {
            double* w = o.out16 + 16 * i;
            w[0] = double(r.toi);
            const V3<S>* v[4] = {&r.w1, &r.w2, &r.n1, &r.n2};
            for (int k = 0; k < 4; ++k) {
                w[1 + 3 * k] = double(v[k]->x);
                w[2 + 3 * k] = double(v[k]->y);
                w[3 + 3 * k] = double(v[k]->z);
            }
            w[13] = r.status;
            w[14] = w[15] = 0.0;
        }
        if (o.tag) o.tag[i] = r.some ? 1 : 0;
        if (o.status) o.status[i] = cnt.status;
        if (o.counters8) {
            uint32_t* c = o.counters8 + 8 * i;
            for (int k = 0; k < 8; ++k) c[k] = 0;
            c[0] = cnt.gjk_iters;
            c[2] = cnt.support_calls;
            c[3] = cnt.hull_points_scanned;
        }
    }
}

template <class N, class S>
int toi_run(const InF32& in, const float* vel1, const float* vel2, uint64_t n, int dispatch, double max_toi,
            double target, double eps, int nt, const Outs& o) {
    double e = eps > 0 ? eps : (double)std::numeric_limits<N>::epsilon();
    Tol<S> tol = eps < 0 ? make_tol_precise<S>(0.0) : make_tol<S>(e, 0.0);
    S mt = max_toi >= (double)std::numeric_limits<float>::max() ? std::numeric_limits<S>::max() : S(max_toi);
    N tg = N(target);
    if (nt <= 1 || n < 64) {
        toi_range<N, S>(in, vel1, vel2, dispatch, mt, tg, tol, 0, n, o);
        return 0;
    }
    std::vector<std::thread> th;
    uint64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        uint64_t lo = t * chunk, hi = std::min<uint64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([&, lo, hi] { toi_range<N, S>(in, vel1, vel2, dispatch, mt, tg, tol, lo, hi, o); });
    }
    for (auto& x : th) x.join();
    return 0;
}

template <class N, class S>
void ray_range(const InF32& in, const float* rays, S max_toi, bool solid, const Tol<S>& tol, uint64_t lo, uint64_t hi,
               const Outs& o) {
    for (uint64_t i = lo; i < hi; ++i) {
        Counters cnt;
        Shape<N> s1;
        RayOut<S> r;
        if (!load_shape<N>(in, in.g1[i], &s1)) {
            cnt.status |= ST_BAD_INPUT;
        } else {
            const Iso<N> m = pose1<N>(in, i);
            const float* ry = rays + 6 * i;
            r = ray_cast_support_map<N, S>(m, s1, V3<N>{N(ry[0]), N(ry[1]), N(ry[2])},
                                           V3<N>{N(ry[3]), N(ry[4]), N(ry[5])}, max_toi, solid, tol, &cnt);
        }
        if (o.out16) {
            double* w = o.out16 + 16 * i;
            for (int k = 0; k < 16; ++k) w[k] = 0.0;
            if (r.hit) {
                w[0] = double(r.toi);
                w[1] = double(r.normal.x);
                w[2] = double(r.normal.y);
                w[3] = double(r.normal.z);
            }
        }
        if (o.tag) o.tag[i] = r.hit ? 1 : 0;
        if (o.status) o.status[i] = cnt.status;
        if (o.counters8) {
            uint32_t* c = o.counters8 + 8 * i;
            for (int k = 0; k < 8; ++k) c[k] = 0;
            c[0] = cnt.gjk_iters;
            c[2] = cnt.support_calls;
            c[3] = cnt.hull_points_scanned;
        }
    }
}

template <class N, class S>
int ray_run(const InF32& in, const float* rays, uint64_t n, double max_toi, int solid, double eps, int nt,
            const Outs& o) {
    double e = eps > 0 ? eps : (double)std::numeric_limits<N>::epsilon();
    Tol<S> tol = eps < 0 ? make_tol_precise<S>(0.0) : make_tol<S>(e, 0.0);
    S mt = max_toi >= (double)std::numeric_limits<float>::max() ? std::numeric_limits<S>::max() : S(max_toi);
    if (nt <= 1 || n < 64) {
        ray_range<N, S>(in, rays, mt, solid != 0, tol, 0, n, o);
        return 0;
    }
    std::vector<std::thread> th;
    uint64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        uint64_t lo = t * chunk, hi = std::min<uint64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([&, lo, hi] { ray_range<N, S>(in, rays, mt, solid != 0, tol, lo, hi, o); });
    }
    for (auto& x : th) x.join();
    return 0;
}

}  // namespace

extern "C" {

// Ray casts on support maps (RayCast::toi_and_normal_with_ray through
// ray_intersection_with_support_map_with_params): ray i hits the shape
// shapes[g1[i]] at pose m1[i]; rays: origin[3], dir[3] per ray (world).
// out16: toi, normal[3] (world); tag 1 = hit.  counters8[0] = ray-cast
// iterations (both casts when solid = 0 and the origin is inside).
int ncgo_ray_cast(int policy, double max_toi, int solid, double eps, int n_threads, const ncg_shape* shapes,
                  uint32_t n_shapes, const float* hull_points, uint64_t n_hull_points, uint64_t n_rays,
                  const ncg_pose* m1, const uint32_t* g1, const float* rays, double* out16, uint8_t* tag,
                  uint32_t* status, uint32_t* counters8) {
    if (!(max_toi >= 0.0)) return NCG_EINVAL;
    InF32 in{shapes, n_shapes, hull_points, n_hull_points, m1, g1, nullptr, nullptr, nullptr};
    Outs o{out16, tag, status, counters8};
    switch (policy) {
    case POLICY_F32: return ray_run<float, float>(in, rays, n_rays, max_toi, solid, eps, n_threads, o);
    case POLICY_F64: return ray_run<double, double>(in, rays, n_rays, max_toi, solid, eps, n_threads, o);
    case POLICY_MIXED: return ray_run<float, dw>(in, rays, n_rays, max_toi, solid, eps, n_threads, o);
    default: return NCG_EINVAL;
    }
}

// World AABBs of shapes[g1[i]] at m1[i] (HasBoundingVolume<AABB>::bounding_volume):
// out6 = mins[3], maxs[3] per entry; status ST_BAD_INPUT (and NaN boxes) for a bad shape.
int ncgo_aabb(const ncg_shape* shapes, uint32_t n_shapes, const float* hull_points, uint64_t n_hull_points,
              uint64_t n, const ncg_pose* m1, const uint32_t* g1, float* out6, uint32_t* status) {
    InF32 in{shapes, n_shapes, hull_points, n_hull_points, m1, g1, nullptr, nullptr, nullptr};
    for (uint64_t i = 0; i < n; ++i) {
        Shape<float> s;
        float* o = out6 + 6 * i;
        if (!load_shape<float>(in, in.g1[i], &s)) {
            for (int k = 0; k < 6; ++k) o[k] = std::numeric_limits<float>::quiet_NaN();
            if (status) status[i] = ST_BAD_INPUT;
            continue;
        }
        const AABB b = shape_aabb(pose1<float>(in, i), s);
        for (int d = 0; d < 3; ++d) {
            o[d] = b.mins[d];
            o[3 + d] = b.maxs[d];
        }
        if (status) status[i] = 0;
    }
    return 0;
}

// The sorted intersecting pairs (lo << 32 | hi) of n boxes (6 floats each);
// writes at most cap of them and returns how many there are.
int64_t ncgo_pairs(const float* boxes6, uint32_t n, uint64_t* out, uint64_t cap) {
    std::vector<AABB> b(n);
    for (uint32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            b[i].mins[d] = boxes6[6 * i + d];
            b[i].maxs[d] = boxes6[6 * i + 3 + d];
        }
    const std::vector<uint64_t> p = intersecting_pairs(b.data(), n);
    for (uint64_t k = 0; k < p.size() && k < cap; ++k) out[k] = p[k];
    return (int64_t)p.size();
}

// The manifold step of ConvexPolyhedronConvexPolyhedronManifoldGenerator from
// each pair's contact query result: contact9 = world1, world2, normal (f32),
// has = the query returned ClosestPoints.  out: ncg_manifold per pair; one
// static chunk of pairs per thread.
int ncgo_manifold(const ncg_shape* shapes, uint32_t n_shapes, uint64_t n, const ncg_pose* m1, const uint32_t* g1,
                  const ncg_pose* m2, const uint32_t* g2, const float* contact9, const uint8_t* has, float linear,
                  float angular1, float angular2, ncg_manifold* out, uint32_t* status, int n_threads,
                  const float* hull_points, uint64_t n_hull_points, const ncg_hull_topology* topo) {
    InF32 in{shapes, n_shapes, nullptr, 0, m1, g1, m2, g2, nullptr};
    const float cang1 = std::cos(angular1), sang1 = std::sin(angular1);
    const float cang2 = std::cos(angular2), sang2 = std::sin(angular2);
    // a Cuboid, or a ConvexHull with a topology, is a polyhedron
    auto side = [&](uint32_t id, PolySide& ps) -> bool {
        if (id >= n_shapes) return false;
        const ncg_shape& sh = shapes[id];
        if (sh.kind == NCG_CUBOID) {
            ps.hull = false;
            ps.h = V3<float>{sh.p[0], sh.p[1], sh.p[2]};
            return true;
        }
        if (sh.kind != NCG_CONVEX_HULL || !topo || !hull_points || id >= topo->n_shapes ||
            (uint64_t)sh.hull_off + sh.hull_n > n_hull_points || topo->shape[4 * (size_t)id + 1] == 0)
            return false;
        ps.hull = true;
        ps.hv = HullView{topo, hull_points, sh.hull_off, sh.hull_n, id};
        return true;
    };
    auto range = [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
        ncg_manifold& o = out[i];
        std::memset(&o, 0, sizeof(o));
        status[i] = 0;
        const float* c = contact9 + 9 * i;
        const V3<float> w1{c[0], c[1], c[2]}, w2{c[3], c[4], c[5]}, nn{c[6], c[7], c[8]};
        if (!has[i]) continue;
        o.normal[0] = nn.x;
        o.normal[1] = nn.y;
        o.normal[2] = nn.z;
        PolySide a, b;
        ManifoldPoint pts[MANIFOLD_MAX];
        int k = -1;
        bool full = false;
        if (side(g1[i], a) && side(g2[i], b))
            k = poly_manifold(pose1<float>(in, i), a, pose2<float>(in, i), b, w1, w2, nn, linear, cang1, sang1, cang2,
                              sang2, pts, &full);
        if (k < 0) {
            pts[0] = ManifoldPoint{w1, w2, depth_wo(w1, w2, nn), 0u, 0u};
            k = 1;
            status[i] = NCG_STATUS_NOT_POLYHEDRA;
        }
        if (full) status[i] |= NCG_STATUS_MANIFOLD_FULL;
        o.n = (uint32_t)k;
        for (int j = 0; j < k; ++j) {
            ncg_manifold_point& p = o.points[j];
            p.world1[0] = pts[j].w1.x; p.world1[1] = pts[j].w1.y; p.world1[2] = pts[j].w1.z;
            p.world2[0] = pts[j].w2.x; p.world2[1] = pts[j].w2.y; p.world2[2] = pts[j].w2.z;
            p.depth = pts[j].depth;
            p.feature1 = pts[j].f1;
            p.feature2 = pts[j].f2;
        }
    }
    };
    if (n_threads <= 1 || n < 1024) {
        range(0, n);
        return 0;
    }
    std::vector<std::thread> th;
    const uint64_t chunk = (n + n_threads - 1) / n_threads;
    for (int t = 0; t < n_threads; ++t) {
        const uint64_t lo = t * chunk, hi = std::min<uint64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back(range, lo, hi);
    }
    for (auto& x : th) x.join();
    return 0;
}

// Linear time of impact (time_of_impact_support_map_support_map; with
// dispatch 1 Ball-Ball pairs take time_of_impact_ball_ball as
// query::time_of_impact does).  vel1, vel2: 3 floats per pair.  max_toi at or
// above FLT_MAX means unbounded.  out16: toi, witness1[3], witness2[3],
// normal1[3], normal2[3] (local frames), TOIStatus; tag 1 = Some.
// counters8[0] = ray-cast iterations.
int ncgo_toi(int policy, int dispatch, double max_toi, double target_distance, double eps, int n_threads,
             const ncg_shape* shapes, uint32_t n_shapes, const float* hull_points, uint64_t n_hull_points,
             uint64_t n_pairs, const ncg_pose* m1, const uint32_t* g1, const ncg_pose* m2, const uint32_t* g2,
             const float* vel1, const float* vel2, double* out16, uint8_t* tag, uint32_t* status,
             uint32_t* counters8) {
    if (!(target_distance >= 0.0) || !(max_toi >= 0.0)) return NCG_EINVAL;
    InF32 in{shapes, n_shapes, hull_points, n_hull_points, m1, g1, m2, g2, nullptr};
    Outs o{out16, tag, status, counters8};
    switch (policy) {
    case POLICY_F32: return toi_run<float, float>(in, vel1, vel2, n_pairs, dispatch, max_toi, target_distance, eps, n_threads, o);
    case POLICY_F64: return toi_run<double, double>(in, vel1, vel2, n_pairs, dispatch, max_toi, target_distance, eps, n_threads, o);
    case POLICY_MIXED: return toi_run<float, dw>(in, vel1, vel2, n_pairs, dispatch, max_toi, target_distance, eps, n_threads, o);
    default: return NCG_EINVAL;
    }
}

// policy: 0 = reference f32, 1 = reference f64, 2 = f32 supports + double-word sub-solve.
// query:  0 = contact (support-map pairs), 1 = distance, 2 = proximity,
//         3 = closest_points, 4 = contact with query::contact's dispatch.
// eps == 0 selects the machine epsilon of the policy's N (the reference's
// default_epsilon); eps > 0 replaces it in every tolerance; eps < 0 selects
// the PRECISE set (f32 zero tests, f64 relative GJK convergence).
// epa_tol > 0 replaces EPA's termination threshold (100 eps) alone.
// out16: per pair p1[3] p2[3] dir[3] value gjk_kind, padded to 16 doubles.
// counters8: gjk iters, epa iters, support calls, hull points scanned,
//            faces created, EPA max vertices, EPA max faces,
//            sub-solves | (EPA exit << 24).
int ncgo_query(int policy, int query, double param, double eps, double epa_tol, int n_threads, const ncg_shape* shapes,
               uint32_t n_shapes, const float* hull_points, uint64_t n_hull_points, uint64_t n_pairs,
               const ncg_pose* m1, const uint32_t* g1, const ncg_pose* m2, const uint32_t* g2,
               const float* init_dir, double* out16, uint8_t* tag, uint32_t* status, uint32_t* counters8) {
    InF32 in{shapes, n_shapes, hull_points, n_hull_points, m1, g1, m2, g2, init_dir};
    Outs o{out16, tag, status, counters8};
    return dispatch(policy, in, n_pairs, query, param, eps, epa_tol, n_threads, o);
}

int ncgo_query_f64in(int policy, int query, double param, double eps, double epa_tol, int n_threads, const int32_t* kinds,
                     const uint32_t* hull_off, const uint32_t* hull_n, const double* params, uint32_t n_shapes,
                     const double* hull_points, uint64_t n_hull_points, uint64_t n_pairs, const double* m1,
                     const uint32_t* g1, const double* m2, const uint32_t* g2, const double* init_dir,
                     double* out16, uint8_t* tag, uint32_t* status, uint32_t* counters8) {
    InF64 in{kinds, hull_off, hull_n, params, n_shapes, hull_points, n_hull_points, m1, g1, m2, g2, init_dir};
    Outs o{out16, tag, status, counters8};
    return dispatch(policy, in, n_pairs, query, param, eps, epa_tol, n_threads, o);
}

// benches/query/algorithm.rs:5-23: reset(a), add_point(b, c, d), project.
// pts: 4 points x 3 doubles.  added[3] receives add_point's results.
int ncgo_simplex_kat(int policy, const double* pts, int* added, double* proj, int* dim_out) {
    auto go = [&](auto tag_n) {
        using N = decltype(tag_n);
        using S = N;
        Tol<S> tol(std::numeric_limits<S>::epsilon());
        CSOPoint<N> c[4];
        for (int i = 0; i < 4; ++i) {
            V3<N> p{N(pts[3 * i]), N(pts[3 * i + 1]), N(pts[3 * i + 2])};
            c[i] = CSOPoint<N>{p, p, zero3<N>()};  // CSOPoint::single_point
        }
        VoronoiSimplex<N, S> s;
        s.reset(c[0]);
        for (int i = 1; i < 4; ++i) added[i - 1] = s.add_point(c[i], tol) ? 1 : 0;
        V3<S> r = s.project_origin_and_reduce(tol, nullptr);
        proj[0] = r.x; proj[1] = r.y; proj[2] = r.z;
        *dim_out = s.dim;
    };
    if (policy == POLICY_F64) go(double(0));
    else go(float(0));
    return 0;
}

int ncgo_abi_version(void) { return NCG_ABI_VERSION; }

}  // extern "C"
