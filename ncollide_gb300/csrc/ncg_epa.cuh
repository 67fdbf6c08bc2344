// ncg_epa.cuh — warp-cooperative 3-D EPA (src/query/algorithms/epa3.rs:171-454).
//
// One warp expands one polytope.  The polytope (CSO vertices, faces,
// adjacency, deleted flags), the face heap and the silhouette live in a
// bounded store: a slice of shared memory for the first pass, a slab of global
// memory for the pairs whose polytope outgrew the shared one.
//
// Arithmetic: the expansion (Face::new's projection of the origin, the
// visibility test of the silhouette) runs in f32; each face normal is
// computed in double-word from the f32 vertices and stored rounded to f32;
// face distances, heap keys and the termination tests are double-word.
//
// Work split inside the warp:
//   * support point along the popped face's normal: every lane (hull arg-max
//     is warp-parallel, analytic maps are computed redundantly);
//   * the new faces of one expansion step: one lane per silhouette edge;
//   * heap push/pop, the silhouette flood fill and the ordered post-pass over
//     the new faces: lane 0, because their order decides which face the
//     reference pops next.  The heap is a restatement of Rust's BinaryHeap
//     (push = sift_up; pop = move last to root, sift_down_to_bottom, sift_up)
//     so that equal keys pop in the reference's order.
#pragma once

#include "ncg_core.cuh"

namespace ncg {

enum EpaExit : int {
    EPA_OK_DIM0 = 1,
    EPA_OK_CONVERGED = 2,
    EPA_OK_NUMERIC = 3,
    EPA_OK_HEAP_EMPTY = 4,
    EPA_NONE = 5,        // EPA returned None
    EPA_OVERFLOW = 6,    // store capacity exceeded (result not valid)
};

// Pointers into one warp's store.  Capacities: VC vertices, FC faces (also the
// heap capacity, each face is pushed at most once), SC silhouette edges, TC
// flood-fill stack entries.  All indices fit in 16 bits.
struct EpaStore {
    float* v;         // [9][VC]: point xyz, orig1 xyz, orig2 xyz
    float* fn;        // [3][FC] face normals
    float* hkey;      // [2][FC] heap keys (neg_dist), double-word hi / lo
    float* sdist;     // [2][SC] distance of the face built on silhouette edge k
    uint16_t* fpts;   // [3][FC]
    uint16_t* fadj;   // [3][FC]
    uint16_t* hid;    // [FC]
    uint16_t* sface;  // [SC]
    uint16_t* tface;  // [TC]
    uint8_t* fdel;    // [FC]
    uint8_t* sopp;    // [SC]
    uint8_t* topp;    // [TC]
    uint8_t* sflag;   // [SC] bit0 = face built, bit1 = origin projects inside
    int VC, FC, SC, TC;

    // Bytes needed for one store (each array padded to 16 bytes).
    static constexpr __host__ __device__ size_t r16(size_t b) { return (b + 15) & ~size_t(15); }
    static constexpr __host__ __device__ size_t bytes(int VC, int FC, int SC, int TC) {
        return r16(9 * 4 * (size_t)VC) + r16(3 * 4 * (size_t)FC) + r16(8 * (size_t)FC) + r16(8 * (size_t)SC) +
               r16(3 * 2 * (size_t)FC) + r16(3 * 2 * (size_t)FC) + r16(2 * (size_t)FC) + r16(2 * (size_t)SC) +
               r16(2 * (size_t)TC) + r16((size_t)FC) + r16((size_t)SC) + r16((size_t)TC) + r16((size_t)SC);
    }
    NCG_DEV void carve(char* base, int vc, int fc, int sc, int tc) {
        VC = vc; FC = fc; SC = sc; TC = tc;
        auto r = [](size_t b) { return (b + 15) & ~size_t(15); };
        char* p = base;
        v = (float*)p; p += r(9 * 4 * (size_t)VC);
        fn = (float*)p; p += r(3 * 4 * (size_t)FC);
        hkey = (float*)p; p += r(8 * (size_t)FC);
        sdist = (float*)p; p += r(8 * (size_t)SC);
        fpts = (uint16_t*)p; p += r(3 * 2 * (size_t)FC);
        fadj = (uint16_t*)p; p += r(3 * 2 * (size_t)FC);
        hid = (uint16_t*)p; p += r(2 * (size_t)FC);
        sface = (uint16_t*)p; p += r(2 * (size_t)SC);
        tface = (uint16_t*)p; p += r(2 * (size_t)TC);
        fdel = (uint8_t*)p; p += r((size_t)FC);
        sopp = (uint8_t*)p; p += r((size_t)SC);
        topp = (uint8_t*)p; p += r((size_t)TC);
        sflag = (uint8_t*)p;
    }

    NCG_DEV vec3<float> vf(int i) const { return {v[i], v[VC + i], v[2 * VC + i]}; }
    NCG_DEV vec3<real> vp(int i) const { return to_r(vf(i)); }
    NCG_DEV vec3<real> vo1(int i) const { return {real(v[3 * VC + i]), real(v[4 * VC + i]), real(v[5 * VC + i])}; }
    NCG_DEV vec3<real> vo2(int i) const { return {real(v[6 * VC + i]), real(v[7 * VC + i]), real(v[8 * VC + i])}; }
    NCG_DEV void put_vertex(int i, const CSO& c) {
        v[i] = c.p.x; v[VC + i] = c.p.y; v[2 * VC + i] = c.p.z;
        v[3 * VC + i] = c.o1.x; v[4 * VC + i] = c.o1.y; v[5 * VC + i] = c.o1.z;
        v[6 * VC + i] = c.o2.x; v[7 * VC + i] = c.o2.y; v[8 * VC + i] = c.o2.z;
    }
    NCG_DEV CSO get_vertex(int i) const {
        return CSO{{v[i], v[VC + i], v[2 * VC + i]}, {v[3 * VC + i], v[4 * VC + i], v[5 * VC + i]},
                   {v[6 * VC + i], v[7 * VC + i], v[8 * VC + i]}};
    }
    NCG_DEV int pt(int f, int k) const { return fpts[k * FC + f]; }
    NCG_DEV int adj(int f, int k) const { return fadj[k * FC + f]; }
    NCG_DEV void set_adj(int f, int k, int a) { fadj[k * FC + f] = (uint16_t)a; }
    NCG_DEV vec3<float> normalf(int f) const { return {fn[f], fn[FC + f], fn[2 * FC + f]}; }
    NCG_DEV vec3<real> normal(int f) const { return to_r(normalf(f)); }
    NCG_DEV real key(int h) const { return real(hkey[h], hkey[FC + h]); }

    // Face::new (epa3.rs:96-115) + ccw_face_normal (utils/ccw_face_normal.rs:21-27).
    // Writes face f; returns whether the origin projects inside; dist = n . pts[0].
    NCG_DEV bool build_face(int f, int p0, int p1, int p2, int a0, int a1, int a2, real eps, real& dist) {
        vec3<float> Af = vf(p0), Bf = vf(p1), Cf = vf(p2);
        Loc<float> loc;
        (void)proj_triangle(Af, Bf, Cf, loc);
        vec3<real> A = to_r(Af);
        vec3<real> u;
        real len;
        vec3<float> n;
        if (try_normalize(cross(to_r(Bf) - A, to_r(Cf) - A), eps, u, len)) n = to_f(u);
        else n = zero3<float>();
        fpts[f] = (uint16_t)p0; fpts[FC + f] = (uint16_t)p1; fpts[2 * FC + f] = (uint16_t)p2;
        fadj[f] = (uint16_t)a0; fadj[FC + f] = (uint16_t)a1; fadj[2 * FC + f] = (uint16_t)a2;
        fn[f] = n.x; fn[FC + f] = n.y; fn[2 * FC + f] = n.z;
        fdel[f] = 0;
        dist = dot(to_r(n), A);
        return loc.kind == LOC_FACE;
    }
    // Face::closest_points with the barycentric coordinates Face::new stored
    // (recomputed: the projection is a pure function of the three vertices).
    NCG_DEV void face_points(int f, vec3<real>& p1, vec3<real>& p2) const {
        int a = pt(f, 0), b = pt(f, 1), c = pt(f, 2);
        Loc<float> loc;
        (void)proj_triangle(vf(a), vf(b), vf(c), loc);
        real b0(0.0f), b1(0.0f), b2(0.0f);
        if (loc.kind == LOC_FACE) { b0 = real(loc.b0); b1 = real(loc.b1); b2 = real(loc.b2); }
        p1 = (vo1(a) * b0 + vo1(b) * b1) + vo1(c) * b2;
        p2 = (vo2(a) * b0 + vo2(b) * b1) + vo2(c) * b2;
    }
    NCG_DEV int next_ccw(int f, int id) const {
        if (pt(f, 0) == id) return 1;
        if (pt(f, 1) == id) return 2;
        return 0;
    }
    // epa3.rs:143-156 and utils/triangle.rs:85-102 (f32).
    NCG_DEV bool seen_by(int f, int point, int opp, const Tol& tol) const {
        vec3<float> p0 = vf(pt(f, opp)), p1 = vf(pt(f, (opp + 1) % 3)), p2 = vf(pt(f, (opp + 2) % 3));
        vec3<float> q = vf(point);
        if (dot(q - p0, normalf(f)) >= -tol.eps_tol_f) return true;
        float x = norm_sq(cross(p2 - p1, q - p1));
        return x == 0.0f || fabsf(x) <= tol.affine_eps_f;
    }

    // ---- Rust BinaryHeap<FaceId> (max-heap on neg_dist) — lane 0 only.
    NCG_DEV void hput(int pos, int id, real k) {
        hkey[pos] = k.h;
        hkey[FC + pos] = k.l;
        hid[pos] = (uint16_t)id;
    }
    NCG_DEV void hmove(int dst, int src) {
        hkey[dst] = hkey[src];
        hkey[FC + dst] = hkey[FC + src];
        hid[dst] = hid[src];
    }
    NCG_DEV void heap_sift_up(int start, int pos, int id, real k) {
        while (pos > start) {
            int parent = (pos - 1) / 2;
            if (k <= key(parent)) break;
            hmove(pos, parent);
            pos = parent;
        }
        hput(pos, id, k);
    }
    NCG_DEV void heap_push(int& size, int id, real k) {
        int pos = size++;
        heap_sift_up(0, pos, id, k);
    }
    NCG_DEV bool heap_pop(int& size, int& id, real& k) {
        if (size == 0) return false;
        size--;
        int lid = hid[size];
        real lkey = key(size);
        if (size == 0) {
            id = lid;
            k = lkey;
            return true;
        }
        id = hid[0];
        k = key(0);
        // sift_down_to_bottom(0) with the former last element in the hole.
        int end = size, pos = 0, child = 1;
        while (end >= 2 && child <= end - 2) {
            child += (key(child) <= key(child + 1)) ? 1 : 0;
            hmove(pos, child);
            pos = child;
            child = 2 * pos + 1;
        }
        if (child == end - 1) {
            hmove(pos, child);
            pos = child;
        }
        heap_sift_up(0, pos, lid, lkey);
        return true;
    }
};

struct EpaResult {
    int exit;
    vec3<real> p1, p2, n;
    uint32_t iters;
    uint32_t status;
};

NCG_DEV int bcast(int x) { return __shfl_sync(0xffffffffu, x, 0); }
NCG_DEV real bcastr(real x) {
    return real(__shfl_sync(0xffffffffu, x.h, 0), __shfl_sync(0xffffffffu, x.l, 0));
}

// EPA::closest_points.  Called by all 32 lanes of a warp with identical
// arguments; every lane returns the same result.
template <class Scan>
NCG_DEV EpaResult epa_warp(const PairGeom& g, int dim, const CSO* sv, const Tol& tol, const Scan& scan, EpaStore& st,
                           int max_iter) {
    const int lane = threadIdx.x & 31;
    EpaResult res;
    res.exit = EPA_NONE;
    res.p1 = res.p2 = res.n = zero3<real>();
    res.iters = 0;
    res.status = 0;

    if (dim == 0) {
        res.n = mk(real(0.0f), real(1.0f), real(0.0f));
        res.exit = EPA_OK_DIM0;
        return res;
    }
    int nv = dim + 1, nf = 0, hsize = 0;
    const real eps = from_host(tol.eps), eps_tol = from_host(tol.eps_tol), epa_tol = from_host(tol.epa_eps_tol);
    if (lane == 0)
        for (int i = 0; i < nv; ++i) st.put_vertex(i, sv[i]);
    __syncwarp();

    if (dim == 3) {
        vec3<real> v0 = st.vp(0);
        vec3<real> dp1 = st.vp(1) - v0, dp2 = st.vp(2) - v0, dp3 = st.vp(3) - v0;
        __syncwarp();
        if (dot(cross(dp1, dp2), dp3) > real(0.0f)) {
            if (lane == 0) {
                CSO a = st.get_vertex(1), b = st.get_vertex(2);
                st.put_vertex(1, b);
                st.put_vertex(2, a);
            }
            __syncwarp();
        }
        // Faces [0,1,2] [1,3,2] [0,2,3] [0,3,1], adjacency per epa3.rs:256-264; lanes 0..3.
        const int P[4][3] = {{0, 1, 2}, {1, 3, 2}, {0, 2, 3}, {0, 3, 1}};
        const int A[4][3] = {{3, 1, 2}, {3, 2, 0}, {0, 1, 3}, {2, 1, 0}};
        real d;
        bool inside = false;
        if (lane < 4) inside = st.build_face(lane, P[lane][0], P[lane][1], P[lane][2], A[lane][0], A[lane][1],
                                             A[lane][2], eps, d);
        unsigned ins = __ballot_sync(0xffffffffu, inside);
        __syncwarp();
        int fail = 0;
        if (lane == 0) {
            for (int k = 0; k < 4; ++k) {
                if (!(ins >> k & 1u)) continue;
                // dist_k = normal_k . vertices[k] (epa3.rs:277,282,287,292)
                real dk = dot(st.normal(k), st.vp(k));
                if (-dk > eps_tol) { fail = 1; break; }
                st.heap_push(hsize, k, -dk);
            }
        }
        (void)d;
        fail = bcast(fail);
        hsize = bcast(hsize);
        nf = 4;
        if (fail) { res.exit = EPA_NONE; res.status |= NCG_STATUS_EPA_FAILED; return res; }
    } else {
        if (dim == 1) {
            vec3<real> dpt = st.vp(1) - st.vp(0);
            vec3<real> a = fabs(dpt.x) > fabs(dpt.y) ? mk(dpt.z, real(0.0f), -dpt.x) : mk(real(0.0f), -dpt.z, dpt.y);
            a = a / vnorm(a);
            vec3<real> dir = cross(a, dpt);
            CSO c = cso_support(g, to_f(dir), scan);
            if (lane == 0) st.put_vertex(2, c);
            nv = 3;
            __syncwarp();
        }
        real d;
        if (lane == 0) (void)st.build_face(0, 0, 1, 2, 1, 1, 1, eps, d);
        if (lane == 1) (void)st.build_face(1, 0, 2, 1, 0, 0, 0, eps, d);
        __syncwarp();
        if (lane == 0) {
            st.heap_push(hsize, 0, real(0.0f));
            st.heap_push(hsize, 1, real(0.0f));
        }
        hsize = 2;
        nf = 2;
        __syncwarp();
    }
    if (hsize == 0) {  // the reference panics on heap.peek().unwrap()
        res.exit = EPA_NONE;
        res.status |= NCG_STATUS_EPA_NO_FACE;
        return res;
    }
    int best = bcast(lane == 0 ? (int)st.hid[0] : 0);
    real max_dist = dw_max();
    int niter = 0;

    for (;;) {
        // ---- pop the closest non-deleted face (lane 0)
        int fid = -1;
        real key(0.0f);
        if (lane == 0) {
            int id;
            real k;
            while (st.heap_pop(hsize, id, k)) {
                if (!st.fdel[id]) { fid = id; key = k; break; }
            }
        }
        fid = bcast(fid);
        key = bcastr(key);
        hsize = bcast(hsize);
        if (fid < 0) {
            st.face_points(best, res.p1, res.p2);
            res.n = st.normal(best);
            res.exit = EPA_OK_HEAP_EMPTY;
            return res;
        }
        res.iters++;
        vec3<float> fnf = st.normalf(fid);
        vec3<real> fnrm = to_r(fnf);
        CSO c = cso_support(g, fnf, scan);
        if (nv >= st.VC) { res.exit = EPA_OVERFLOW; return res; }
        const int sup = nv++;
        if (lane == 0) st.put_vertex(sup, c);
        real cand = dot(to_r(c.p), fnrm);
        if (cand < max_dist) {
            best = fid;
            max_dist = cand;
        }
        real curr = -key;
        __syncwarp();
        if (max_dist - curr < epa_tol) {
            st.face_points(best, res.p1, res.p2);
            res.n = st.normal(best);
            res.exit = EPA_OK_CONVERGED;
            return res;
        }

        // ---- silhouette flood fill (lane 0), recursion order kept with a stack
        int nsil = 0, ovf = 0;
        if (lane == 0) {
            st.fdel[fid] = 1;
            int a0 = st.adj(fid, 0), a1 = st.adj(fid, 1), a2 = st.adj(fid, 2);
            int o0 = st.next_ccw(a0, st.pt(fid, 0));
            int o1 = st.next_ccw(a1, st.pt(fid, 1));
            int o2 = st.next_ccw(a2, st.pt(fid, 2));
            int top = 0;
            if (st.TC < 3) ovf = 1;
            else {
                st.tface[top] = (uint16_t)a2; st.topp[top++] = (uint8_t)o2;
                st.tface[top] = (uint16_t)a1; st.topp[top++] = (uint8_t)o1;
                st.tface[top] = (uint16_t)a0; st.topp[top++] = (uint8_t)o0;
            }
            while (top > 0 && !ovf) {
                --top;
                int id = st.tface[top], opp = st.topp[top];
                if (st.fdel[id]) continue;
                if (!st.seen_by(id, sup, opp, tol)) {
                    if (nsil >= st.SC) { ovf = 1; break; }
                    st.sface[nsil] = (uint16_t)id;
                    st.sopp[nsil] = (uint8_t)opp;
                    nsil++;
                } else {
                    st.fdel[id] = 1;
                    int k1 = (opp + 2) % 3, k2 = opp;
                    int b1 = st.adj(id, k1), b2 = st.adj(id, k2);
                    int q1 = st.next_ccw(b1, st.pt(id, k1));
                    int q2 = st.next_ccw(b2, st.pt(id, k2));
                    if (top + 2 > st.TC) { ovf = 1; break; }
                    st.tface[top] = (uint16_t)b2; st.topp[top++] = (uint8_t)q2;
                    st.tface[top] = (uint16_t)b1; st.topp[top++] = (uint8_t)q1;
                }
            }
        }
        nsil = bcast(nsil);
        ovf = bcast(ovf);
        __syncwarp();
        if (ovf) { res.exit = EPA_OVERFLOW; return res; }
        if (nsil == 0) {
            res.exit = EPA_NONE;
            res.status |= NCG_STATUS_EPA_FAILED;
            return res;
        }

        // ---- new faces, one lane per surviving silhouette edge
        const int first_new = nf;
        int built = 0;
        for (int base = 0; base < nsil; base += 32) {
            int k = base + lane;
            bool live = false;
            int sf = 0, so = 0;
            if (k < nsil) {
                sf = st.sface[k];
                so = st.sopp[k];
                live = !st.fdel[sf];
            }
            unsigned m = __ballot_sync(0xffffffffu, live);
            int rank = __popc(m & ((1u << lane) - 1u));
            int id = first_new + built + rank;
            if (first_new + built + __popc(m) > st.FC) { ovf = 1; }
            if (live && !ovf) {
                int q1 = st.pt(sf, (so + 2) % 3), q2 = st.pt(sf, (so + 1) % 3);
                real dist;
                bool in = st.build_face(id, q1, q2, sup, sf, id + 1, id - 1, eps, dist);
                st.sdist[k] = dist.h;
                st.sdist[st.SC + k] = dist.l;
                st.sflag[k] = (uint8_t)(1 | (in ? 2 : 0));
            } else if (k < nsil) {
                st.sflag[k] = 0;
            }
            built += __popc(m);
        }
        __syncwarp();
        if (ovf) { res.exit = EPA_OVERFLOW; return res; }

        // ---- ordered post-pass (lane 0): adjacency, checks, heap pushes
        int outcome = 0;  // 0 continue, 1 numeric return, 2 None
        if (lane == 0) {
            int id = first_new;
            for (int k = 0; k < nsil; ++k) {
                uint8_t fl = st.sflag[k];
                if (!(fl & 1)) continue;
                int sf = st.sface[k], so = st.sopp[k];
                st.set_adj(sf, (so + 1) % 3, id);
                if (fl & 2) {
                    real dist(st.sdist[k], st.sdist[st.SC + k]);
                    if (dist < curr) { outcome = 1; break; }
                    if (-dist > eps_tol) { outcome = 2; break; }
                    st.heap_push(hsize, id, -dist);
                }
                id++;
            }
        }
        outcome = bcast(outcome);
        hsize = bcast(hsize);
        __syncwarp();
        if (outcome == 1) {
            st.face_points(fid, res.p1, res.p2);
            res.n = fnrm;
            res.exit = EPA_OK_NUMERIC;
            return res;
        }
        if (outcome == 2 || built == 0) {
            res.exit = EPA_NONE;
            res.status |= NCG_STATUS_EPA_FAILED;
            return res;
        }
        nf = first_new + built;
        if (lane == 0) {
            st.set_adj(first_new, 2, nf - 1);
            st.set_adj(nf - 1, 1, first_new);
        }
        __syncwarp();
        niter += 1;
        if (niter > max_iter) {
            res.exit = EPA_NONE;
            res.status |= NCG_STATUS_EPA_MAX_ITER;
            return res;
        }
    }
}

}  // namespace ncg
