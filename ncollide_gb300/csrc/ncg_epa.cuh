// ncg_epa.cuh — warp-cooperative 3-D EPA (src/query/algorithms/epa3.rs:171-454).
//
// The algorithm is written once for two execution policies:
//   ThreadExec  one thread expands one polytope held in its local memory (a
//               warp runs 32 independent pairs and thousands of threads hide
//               the latency); used for small polytopes.
//   WarpExec    one warp expands one polytope held in shared memory (tiers A
//               and B) or a global-memory slab (tier C); used for ConvexHull
//               pairs (warp-parallel support scans) and for polytopes that
//               outgrow a thread's store.
//
// Layout (one store is contiguous, so a thread's records share cache sectors):
//   vertex  float4 (x, y, z, 0); the two support points behind each vertex
//           (witness data, read only at the end) in a separate 6 x f32 record
//   face    float4 (normal xyz, p0 | p1 << 16) then uint4 (p2 | gen << 16,
//           adj0, adj1, adj2): one 32-byte record
//   heap    float4 (key hi, key lo, push sequence, face reference)
// A face reference is slot | gen << 16.  Deleting a face bumps its slot's
// generation and frees the slot, so every reference taken before the deletion
// (adjacency, heap entries, flood-fill stack) reads as deleted, exactly like
// the reference's `deleted` flag, and the store only needs room for the live
// faces (about twice the vertices) instead of every face ever created.  A
// slot is reused at most once per iteration, so with at most 10 000
// iterations its 16-bit generation never wraps.
//
// Priority order: larger neg_dist first, then the earlier push.  With this
// strict total order the pop sequence depends only on the set of entries, not
// on how the heap is arranged, so the entries of deleted faces can be dropped
// whenever the heap fills up.  Equal keys (the only case where this differs
// from Rust's BinaryHeap) pop first-in first-out.  The f32 build
// (NCG_REAL_F32) keeps Rust's BinaryHeap instead, deleted entries included.
//
// Arithmetic: the expansion (Face::new's projection of the origin, the
// visibility test of the silhouette) runs in f32; each face normal is the
// double-word cross product of exact double-word edge vectors, normalised in
// f32 and stored in f32; face distances, queue keys and the termination tests
// are double-word (all f32 in the f32 build: `real`).
//
// Work split inside a warp (WarpExec): the support point along the popped
// face's normal uses every lane (the hull arg-max is warp-parallel); the faces
// of one expansion step are built one lane per silhouette edge; heap
// operations, the silhouette flood fill and the ordered post-pass run on lane
// 0 because their order decides the result.
#pragma once

#include "ncg_core.cuh"

#ifndef NCG_EPA_HEAP_ARITY
#define NCG_EPA_HEAP_ARITY 2
#endif

namespace ncg {

enum EpaExit : int {
    EPA_OK_DIM0 = 1,
    EPA_OK_CONVERGED = 2,
    EPA_OK_NUMERIC = 3,
    EPA_OK_HEAP_EMPTY = 4,
    EPA_NONE = 5,        // EPA returned None
    EPA_OVERFLOW = 6,    // no room for the next support point, stopped between two steps (resumable)
    EPA_OK_PRECISION = 7,  // PRECISE set: a failed expansion step answered with the best face
    EPA_OVERFLOW_MID = 8,  // a silhouette, stack, slot or heap limit hit inside a step: the store is
                           // left half-updated, so a larger store restarts from GJK's simplex
};
NCG_DEV bool epa_overflow(int e) { return e == EPA_OVERFLOW || e == EPA_OVERFLOW_MID; }
NCG_DEV bool epa_ok(int e) { return (e >= EPA_OK_DIM0 && e <= EPA_OK_HEAP_EMPTY) || e == EPA_OK_PRECISION; }

NCG_DEV uint32_t mkref(int slot, uint32_t gen) { return (uint32_t)slot | (gen << 16); }
NCG_DEV int rslot(uint32_t r) { return (int)(r & 0xffffu); }

struct EpaStore {
    float4* vpt;      // [VC]
    float* vo;        // [VC][6] orig1 xyz, orig2 xyz
    float4* face;     // [FC][2] float4 (normal xyz, pts p0 | p1 << 16), uint4 (p2 | gen << 16, adj0..2)
    float4* heap;     // [HC] key hi, key lo, seq, ref
    uint32_t* freel;  // [FC] free slots (stack)
    uint32_t* sref;   // [SC] silhouette face references
    uint32_t* snew;   // [SC] reference of the face built on edge k
    uint32_t* snext;  // [SC] reference of the next live edge's new face
    uint32_t* sprev;  // [SC] reference of the previous live edge's new face
    float2* sdist;    // [SC] distance of the new face (double-word)
    uint8_t* sopp;    // [SC]
    uint8_t* sflag;   // [SC] bit0 live edge, bit1 origin projects inside
    uint32_t* tref;   // [TC] flood-fill stack: references
    uint8_t* topp;    // [TC] flood-fill stack: opposite vertex
    int VC, FC, SC, TC;
    int HC;  // heap entries: FC, or more for the f32 build's largest store (its heap keeps deleted faces)

    static constexpr __host__ __device__ size_t r16(size_t b) { return (b + 15) & ~size_t(15); }
    // Bytes of one store.
    static constexpr __host__ __device__ size_t bytes(int VC, int FC, int SC, int TC, int HC) {
        return r16(16 * (size_t)VC) + r16(32 * (size_t)FC) + r16(16 * (size_t)HC) +
               r16(4 * (size_t)FC) + 4 * r16(4 * (size_t)SC) + r16(8 * (size_t)SC) + 2 * r16((size_t)SC) +
               r16(4 * (size_t)TC) + r16((size_t)TC) + r16(24 * (size_t)VC);
    }

    NCG_DEV void carve(char* base, int vc, int fc, int sc, int tc, int hc) {
        VC = vc; FC = fc; SC = sc; TC = tc; HC = hc;
        char* p = base;
        vpt = (float4*)p; p += r16(16 * (size_t)VC);
        face = (float4*)p; p += r16(32 * (size_t)FC);
        heap = (float4*)p; p += r16(16 * (size_t)HC);
        freel = (uint32_t*)p; p += r16(4 * (size_t)FC);
        sref = (uint32_t*)p; p += r16(4 * (size_t)SC);
        snew = (uint32_t*)p; p += r16(4 * (size_t)SC);
        snext = (uint32_t*)p; p += r16(4 * (size_t)SC);
        sprev = (uint32_t*)p; p += r16(4 * (size_t)SC);
        sdist = (float2*)p; p += r16(8 * (size_t)SC);
        sopp = (uint8_t*)p; p += r16((size_t)SC);
        sflag = (uint8_t*)p; p += r16((size_t)SC);
        tref = (uint32_t*)p; p += r16(4 * (size_t)TC);
        topp = (uint8_t*)p; p += r16((size_t)TC);
        vo = (float*)p;
    }

    NCG_DEV vec3<float> vf(int i) const {
        float4 v = vpt[i];
        return {v.x, v.y, v.z};
    }
    // A face's two 16-byte halves are adjacent (one 32-byte sector).
    NCG_DEV float4& FA(int f) const { return face[2 * f]; }
    NCG_DEV uint4& FB(int f) const { return reinterpret_cast<uint4*>(face)[2 * f + 1]; }
    NCG_DEV vec3<real> vo1(int i) const { return {real(vo[6 * i]), real(vo[6 * i + 1]), real(vo[6 * i + 2])}; }
    NCG_DEV vec3<real> vo2(int i) const { return {real(vo[6 * i + 3]), real(vo[6 * i + 4]), real(vo[6 * i + 5])}; }
    NCG_DEV void put_vertex(int i, const CSO& c) {
        vpt[i] = make_float4(c.p.x, c.p.y, c.p.z, 0.0f);
        float* w = vo + 6 * i;
        w[0] = c.o1.x; w[1] = c.o1.y; w[2] = c.o1.z;
        w[3] = c.o2.x; w[4] = c.o2.y; w[5] = c.o2.z;
    }
    NCG_DEV CSO get_vertex(int i) const {
        const float* w = vo + 6 * i;
        return CSO{vf(i), {w[0], w[1], w[2]}, {w[3], w[4], w[5]}};
    }
    NCG_DEV uint32_t gen(int f) const { return FB(f).x >> 16; }
    NCG_DEV bool live(uint32_t ref) const { return gen(rslot(ref)) == (ref >> 16); }
    NCG_DEV void pts(int f, int& a, int& b, int& c) const {
        uint32_t ab = __float_as_uint(FA(f).w);
        a = (int)(ab & 0xffffu);
        b = (int)(ab >> 16);
        c = (int)(FB(f).x & 0xffffu);
    }
    NCG_DEV int pt(int f, int k) const {
        int a, b, c;
        pts(f, a, b, c);
        return k == 0 ? a : (k == 1 ? b : c);
    }
    NCG_DEV uint32_t adj(int f, int k) const {
        uint4 b = FB(f);
        return k == 0 ? b.y : (k == 1 ? b.z : b.w);
    }
    NCG_DEV void set_adj(int f, int k, uint32_t r) {
        if (k == 0) FB(f).y = r;
        else if (k == 1) FB(f).z = r;
        else FB(f).w = r;
    }
    NCG_DEV vec3<float> normalf(int f) const {
        float4 a = FA(f);
        return {a.x, a.y, a.z};
    }
    NCG_DEV vec3<real> normal(int f) const { return to_r(normalf(f)); }
    // Deletes a face: bumps its slot's generation (all references go stale) and frees the slot.
    NCG_DEV void kill(int f, int& nfree) {
        FB(f).x += 1u << 16;
        freel[nfree++] = (uint32_t)f;
    }

    // Face::new (epa3.rs:96-115) + ccw_face_normal (utils/ccw_face_normal.rs:21-27).
    // Writes face f (generation g); returns whether the origin projects inside;
    // dist = n . pts[0].
    __device__ __noinline__ bool build_face(int f, uint32_t g, int p0, int p1, int p2, uint32_t a0, uint32_t a1,
                                            uint32_t a2, float eps, real& dist) {
        vec3<float> Af = vf(p0), Bf = vf(p1), Cf = vf(p2);
        Loc<float> loc;
        (void)proj_triangle(Af, Bf, Cf, loc);
        vec3<real> A = to_r(Af);
        vec3<float> n;
        float len;
        if (!try_normalize(to_f(cross(to_r(Bf) - A, to_r(Cf) - A)), eps, n, len)) n = zero3<float>();
        FA(f) = make_float4(n.x, n.y, n.z, __uint_as_float((uint32_t)p0 | ((uint32_t)p1 << 16)));
        FB(f) = make_uint4((uint32_t)p2 | (g << 16), a0, a1, a2);
        dist = dot(to_r(n), A);
        return loc.kind == LOC_FACE;
    }
    // Face::closest_points: the barycentric coordinates Face::new stored are
    // recomputed from the three vertices (a pure function of them).
    __device__ __noinline__ void face_points(int a, int b, int c, vec3<real>& p1, vec3<real>& p2) const {
        Loc<float> loc;
        (void)proj_triangle(vf(a), vf(b), vf(c), loc);
        real b0(0.0f), b1(0.0f), b2(0.0f);
        if (loc.kind == LOC_FACE) { b0 = real(loc.b0); b1 = real(loc.b1); b2 = real(loc.b2); }
        p1 = (vo1(a) * b0 + vo1(b) * b1) + vo1(c) * b2;
        p2 = (vo2(a) * b0 + vo2(b) * b1) + vo2(c) * b2;
    }
    NCG_DEV int next_ccw(int f, int id) const {
        int a, b, c;
        pts(f, a, b, c);
        if (a == id) return 1;
        if (b == id) return 2;
        return 0;
    }
    // epa3.rs:143-156 and utils/triangle.rs:85-102 (f32).
    NCG_DEV bool seen_by(int f, int point, int opp, const Tol& tol) const {
        int a, b, c;
        pts(f, a, b, c);
        int i0 = opp == 0 ? a : (opp == 1 ? b : c);
        int i1 = opp == 0 ? b : (opp == 1 ? c : a);
        int i2 = opp == 0 ? c : (opp == 1 ? a : b);
        vec3<float> p0 = vf(i0), p1 = vf(i1), p2 = vf(i2);
        vec3<float> x = vf(point);
        if (dot(x - p0, normalf(f)) >= -tol.eps_tol_f) return true;
        float s = norm_sq(cross(p2 - p1, x - p1));
        return s == 0.0f || fabsf(s) <= tol.affine_eps_f;
    }

#ifndef NCG_REAL_F32
    // ---- d-ary heap on (neg_dist, earlier push) — one thread only.  With a
    // strict total order the pop sequence does not depend on the arity
    // (NCG_EPA_HEAP_ARITY; 4- and 8-ary heaps measured no faster than binary:
    // the heap is not what bounds an EPA iteration).
    static constexpr int HA = NCG_EPA_HEAP_ARITY;
    NCG_DEV static bool before(float4 a, float4 b) {
        real ka(a.x, a.y), kb(b.x, b.y);
        if (ka > kb) return true;
        if (kb > ka) return false;
        return __float_as_uint(a.z) < __float_as_uint(b.z);
    }
    NCG_DEV void sift_up(int pos, float4 e) {
        while (pos > 0) {
            int parent = (pos - 1) / HA;
            float4 p = heap[parent];
            if (!before(e, p)) break;
            heap[pos] = p;
            pos = parent;
        }
        heap[pos] = e;
    }
    NCG_DEV void sift_down(int pos, int size, float4 e) {
        for (;;) {
            const int c0 = HA * pos + 1;
            if (c0 >= size) break;
            int c = c0;
            float4 ce = heap[c0];
#pragma unroll
            for (int k = 1; k < HA; ++k) {
                if (c0 + k < size) {
                    float4 ck = heap[c0 + k];
                    if (before(ck, ce)) { ce = ck; c = c0 + k; }
                }
            }
            if (!before(ce, e)) break;
            heap[pos] = ce;
            pos = c;
        }
        heap[pos] = e;
    }
    // Drops the entries of deleted faces (the pop order does not change).
    NCG_DEV void purge(int& size) {
        int j = 0;
        for (int i = 0; i < size; ++i) {
            float4 e = heap[i];
            if (live(__float_as_uint(e.w))) heap[j++] = e;
        }
        size = j;
        for (int i = (size - 2) / HA; i >= 0; --i) sift_down(i, size, heap[i]);
    }
    // Returns false when the heap is full even after purging.
    NCG_DEV bool push(int& size, uint32_t& seq, uint32_t ref, real key) {
        if (size >= HC) {
            purge(size);
            if (size >= HC) return false;
        }
        float4 e = make_float4(key.h, key.l, __uint_as_float(seq++), __uint_as_float(ref));
        sift_up(size++, e);
        return true;
    }
    // Pops the first live entry (returned whole in *popped); false when none is left.
    NCG_DEV bool pop_live(int& size, int& fid, real& key, float4& popped) {
        while (size > 0) {
            float4 e = heap[0];
            size--;
            if (size > 0) sift_down(0, size, heap[size]);
            uint32_t r = __float_as_uint(e.w);
            if (live(r)) {
                fid = rslot(r);
                key = real(e.x, e.y);
                popped = e;
                return true;
            }
        }
        return false;
    }
#else
    // ---- Rust's BinaryHeap on neg_dist alone (the reference f32 path): push
    // sifts up while the entry is greater than its parent; pop moves the last
    // entry to the root, sifts that hole to the bottom along the greater child
    // (the right one on ties) and back up (alloc/collections/binary_heap).  The
    // order among equal distances then follows the reference exactly, which
    // needs the deleted faces' entries kept as the reference keeps them: a
    // full heap is an overflow, never purged.
    NCG_DEV static bool le(float4 a, float4 b) { return a.x <= b.x; }  // PartialOrd::le (false with NaN)
    NCG_DEV void sift_up_from(int pos, float4 e) {
        while (pos > 0) {
            const int parent = (pos - 1) / 2;
            const float4 p = heap[parent];
            if (le(e, p)) break;
            heap[pos] = p;
            pos = parent;
        }
        heap[pos] = e;
    }
    NCG_DEV bool push(int& size, uint32_t& seq, uint32_t ref, real key) {
        if (size >= HC) return false;
        float4 e = make_float4(key.h, 0.0f, __uint_as_float(seq++), __uint_as_float(ref));
        sift_up_from(size++, e);
        return true;
    }
    NCG_DEV float4 pop_one(int& size) {
        float4 item = heap[--size];
        if (size > 0) {
            const float4 top = heap[0];
            int pos = 0, child = 1;
            while (size >= 2 && child <= size - 2) {
                child += le(heap[child], heap[child + 1]) ? 1 : 0;
                heap[pos] = heap[child];
                pos = child;
                child = 2 * pos + 1;
            }
            if (child == size - 1) {
                heap[pos] = heap[child];
                pos = child;
            }
            sift_up_from(pos, item);
            item = top;
        }
        return item;
    }
    NCG_DEV bool pop_live(int& size, int& fid, real& key, float4& popped) {
        while (size > 0) {
            const float4 e = pop_one(size);
            const uint32_t r = __float_as_uint(e.w);
            if (live(r)) {
                fid = rslot(r);
                key = real(e.x, e.y);
                popped = e;
                return true;
            }
        }
        return false;
    }
#endif
#ifndef NCG_REAL_F32
    // Puts a popped entry back unchanged (same key and push sequence, so the
    // pop order is as if it had never left).
    NCG_DEV void repush(int& size, float4 e) { sift_up(size++, e); }
#endif
};

// Execution policies.
struct WarpExec {
    static constexpr int W = 32;
    NCG_DEV static int lane() { return threadIdx.x & 31; }
    NCG_DEV static void sync() { __syncwarp(); }
    NCG_DEV static int bcast(int x) { return __shfl_sync(0xffffffffu, x, 0); }
    NCG_DEV static uint32_t bcast(uint32_t x) { return __shfl_sync(0xffffffffu, x, 0); }
    NCG_DEV static real bcast(real x) {
        return real(__shfl_sync(0xffffffffu, x.h, 0), __shfl_sync(0xffffffffu, x.l, 0));
    }
};
struct ThreadExec {
    static constexpr int W = 1;
    NCG_DEV static int lane() { return 0; }
    NCG_DEV static void sync() {}
    NCG_DEV static int bcast(int x) { return x; }
    NCG_DEV static uint32_t bcast(uint32_t x) { return x; }
    NCG_DEV static real bcast(real x) { return x; }
};

struct EpaResult {
    int exit;
    vec3<real> p1, p2, n;
    uint32_t iters;
    uint32_t status;
};

// The state EPA keeps from one expansion step to the next (the store holds
// the polytope): counts of vertices, fresh and free face slots, heap size and
// push sequence, the best face so far and its support distance, and the result.
struct EpaState {
    int nv, nfresh, nfree, hsize, niter;
    uint32_t seq;
    int b0, b1, b2;
    vec3<float> bn;
    real max_dist;
    EpaResult res;
};

// EPA::closest_points (epa3.rs:219-430) in two parts: epa_begin builds the
// initial polytope from GJK's simplex (epa3.rs:219-321); epa_step runs one
// iteration of the expansion loop (epa3.rs:323-428).  Each returns true when
// EPA has finished, with the result in S.res.  With WarpExec all 32 lanes of a
// warp call them with identical arguments and every lane gets the same state;
// with ThreadExec one thread runs them alone.  Between two steps the state and
// the store are all there is, which lets a larger store resume a run
// (epa_spill, epa_resume) and lets a thread interleave steps of several pairs.
template <class E, class Scan>
NCG_DEV bool epa_begin(const PairGeom& g, int dim, const CSO* sv, const Tol& tol, const Scan& scan, EpaStore& st,
                       EpaState& S) {
    const int lane = E::lane();
    EpaResult& res = S.res;
    res.exit = EPA_NONE;
    res.p1 = res.p2 = res.n = zero3<real>();
    res.iters = 0;
    res.status = 0;
    if (dim == 0) {
        res.n = mk(real(0.0f), real(1.0f), real(0.0f));
        res.exit = EPA_OK_DIM0;
        return true;
    }
    const real eps_tol = from_host(tol.eps_tol);
    const float eps = tol.eps.h;
    int nv = dim + 1, nfresh = 0, nfree = 0, hsize = 0;
    uint32_t seq = 0;
    if (lane == 0)
        for (int i = 0; i < nv; ++i) st.put_vertex(i, sv[i]);
    E::sync();

    if (dim == 3) {
        vec3<real> v0 = to_r(st.vf(0));
        vec3<real> dp1 = to_r(st.vf(1)) - v0, dp2 = to_r(st.vf(2)) - v0, dp3 = to_r(st.vf(3)) - v0;
        E::sync();
        if (dot(cross(dp1, dp2), dp3) > real(0.0f)) {
            if (lane == 0) {
                CSO a = st.get_vertex(1), b = st.get_vertex(2);
                st.put_vertex(1, b);
                st.put_vertex(2, a);
            }
            E::sync();
        }
        // Faces [0,1,2] [1,3,2] [0,2,3] [0,3,1], adjacency per epa3.rs:256-264; lanes 0..3.
        const int P[4][3] = {{0, 1, 2}, {1, 3, 2}, {0, 2, 3}, {0, 3, 1}};
        const int A[4][3] = {{3, 1, 2}, {3, 2, 0}, {0, 1, 3}, {2, 1, 0}};
        real d;
        unsigned ins = 0;
        for (int k = lane; k < 4; k += E::W)
            if (st.build_face(k, 0, P[k][0], P[k][1], P[k][2], mkref(A[k][0], 0), mkref(A[k][1], 0),
                              mkref(A[k][2], 0), eps, d))
                ins |= 1u << k;
        if (E::W > 1) ins = __reduce_or_sync(0xffffffffu, ins);
        E::sync();
        int fail = 0;
        if (lane == 0) {
            for (int k = 0; k < 4; ++k) {
                if (!(ins >> k & 1u)) continue;
                // dist_k = normal_k . vertices[k] (epa3.rs:277,282,287,292)
                real dk = dot(st.normal(k), to_r(st.vf(k)));
                if (-dk > eps_tol) { fail = 1; break; }
                st.push(hsize, seq, mkref(k, 0), -dk);
            }
        }
        fail = E::bcast(fail);
        hsize = E::bcast(hsize);
        seq = E::bcast(seq);
        nfresh = 4;
        if (fail) { res.status |= NCG_STATUS_EPA_FAILED; return true; }
    } else {
        if (dim == 1) {
            vec3<real> dpt = to_r(st.vf(1)) - to_r(st.vf(0));
            vec3<real> a = fabs(dpt.x) > fabs(dpt.y) ? mk(dpt.z, real(0.0f), -dpt.x) : mk(real(0.0f), -dpt.z, dpt.y);
            a = a / vnorm(a);
            vec3<real> dir = cross(a, dpt);
            CSO c = cso_support(g, to_f(dir), scan);
            if (lane == 0) st.put_vertex(2, c);
            nv = 3;
            E::sync();
        }
        real d;
        if (lane == 0) (void)st.build_face(0, 0, 0, 1, 2, mkref(1, 0), mkref(1, 0), mkref(1, 0), eps, d);
        if (lane == (E::W > 1 ? 1 : 0))
            (void)st.build_face(1, 0, 0, 2, 1, mkref(0, 0), mkref(0, 0), mkref(0, 0), eps, d);
        E::sync();
        if (lane == 0) {
            st.push(hsize, seq, mkref(0, 0), real(0.0f));
            st.push(hsize, seq, mkref(1, 0), real(0.0f));
        }
        hsize = 2;
        seq = 2;
        nfresh = 2;
        E::sync();
    }
    if (hsize == 0) {  // the reference panics on heap.peek().unwrap()
        res.status |= NCG_STATUS_EPA_NO_FACE;
        return true;
    }
    // best face (its points and normal are kept: its slot may be recycled)
    int bslot = rslot(__float_as_uint(st.heap[0].w));
    st.pts(bslot, S.b0, S.b1, S.b2);
    S.bn = st.normalf(bslot);
    S.max_dist = dw_max();
    S.niter = 0;
    S.nv = nv;
    S.nfresh = nfresh;
    S.nfree = nfree;
    S.hsize = hsize;
    S.seq = seq;
    return false;
}

template <class E, class Scan>
NCG_DEV bool epa_step(const PairGeom& g, const Tol& tol, const Scan& scan, EpaStore& st, EpaState& S, int max_iter) {
    const int lane = E::lane();
    EpaResult& res = S.res;
    const real eps_tol = from_host(tol.eps_tol), epa_tol = from_host(tol.epa_eps_tol);
    const float eps = tol.eps.h;
    int& nv = S.nv;
    int& nfresh = S.nfresh;
    int& nfree = S.nfree;
    int& hsize = S.hsize;
    uint32_t& seq = S.seq;
    int& b0 = S.b0;
    int& b1 = S.b1;
    int& b2 = S.b2;
    vec3<float>& bn = S.bn;
    real& max_dist = S.max_dist;
    int& niter = S.niter;
    {
        // ---- pop the closest live face (lane 0)
        int fid = -1;
        real key(0.0f);
        float4 popped = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#ifdef NCG_REAL_F32
        // Rust's heap cannot take a popped entry back unchanged: stop before
        // the pop when no room is left for this iteration's support point
        if (nv >= st.VC) {
            res.exit = EPA_OVERFLOW;
            return true;
        }
#endif
        if (lane == 0) {
            if (!st.pop_live(hsize, fid, key, popped)) fid = -1;
        }
        fid = E::bcast(fid);
        key = E::bcast(key);
        hsize = E::bcast(hsize);
        E::sync();
        if (fid < 0) {
            st.face_points(b0, b1, b2, res.p1, res.p2);
            res.n = to_r(bn);
            res.exit = EPA_OK_HEAP_EMPTY;
            return true;
        }
#ifndef NCG_REAL_F32
        if (nv >= st.VC) {
            // no room for this iteration's support point: put the face back and
            // stop between two iterations, so that a larger store can resume
            // from this state (epa_spill / epa_resume) with the same result
            if (lane == 0) st.repush(hsize, popped);
            hsize = E::bcast(hsize);
            E::sync();
            res.exit = EPA_OVERFLOW;
            return true;
        }
#endif
        res.iters++;
        int f0, f1, f2;
        st.pts(fid, f0, f1, f2);
        vec3<float> fnf = st.normalf(fid);
        vec3<real> fnrm = to_r(fnf);
        CSO c = cso_support(g, fnf, scan);
        const int sup = nv++;
        if (lane == 0) st.put_vertex(sup, c);
        real cand = dot(to_r(c.p), fnrm);
        if (cand < max_dist) {
            b0 = f0; b1 = f1; b2 = f2;
            bn = fnf;
            max_dist = cand;
        }
        real curr = -key;
        E::sync();
        if (max_dist - curr < epa_tol) {
            st.face_points(b0, b1, b2, res.p1, res.p2);
            res.n = to_r(bn);
            res.exit = EPA_OK_CONVERGED;
            return true;
        }

        // ---- silhouette flood fill (lane 0), recursion order kept with a stack
        int nsil = 0, ovf = 0;
        if (lane == 0) {
            uint32_t a0 = st.adj(fid, 0), a1 = st.adj(fid, 1), a2 = st.adj(fid, 2);
            int o0 = st.next_ccw(rslot(a0), f0);
            int o1 = st.next_ccw(rslot(a1), f1);
            int o2 = st.next_ccw(rslot(a2), f2);
            st.kill(fid, nfree);
            int top = 0;
            if (st.TC < 3) ovf = 1;
            else {
                st.tref[top] = a2; st.topp[top++] = (uint8_t)o2;
                st.tref[top] = a1; st.topp[top++] = (uint8_t)o1;
                st.tref[top] = a0; st.topp[top++] = (uint8_t)o0;
            }
            while (top > 0 && !ovf) {
                --top;
                uint32_t r = st.tref[top];
                int opp = st.topp[top];
                if (!st.live(r)) continue;
                int id = rslot(r);
                if (!st.seen_by(id, sup, opp, tol)) {
                    if (nsil >= st.SC) { ovf = 1; break; }
                    st.sref[nsil] = r;
                    st.sopp[nsil] = (uint8_t)opp;
                    nsil++;
                } else {
                    int k1 = (opp + 2) % 3, k2 = opp;
                    uint32_t r1 = st.adj(id, k1), r2 = st.adj(id, k2);
                    int q1 = st.next_ccw(rslot(r1), st.pt(id, k1));
                    int q2 = st.next_ccw(rslot(r2), st.pt(id, k2));
                    st.kill(id, nfree);
                    if (top + 2 > st.TC) { ovf = 1; break; }
                    st.tref[top] = r2; st.topp[top++] = (uint8_t)q2;
                    st.tref[top] = r1; st.topp[top++] = (uint8_t)q1;
                }
            }
        }
        nsil = E::bcast(nsil);
        ovf = E::bcast(ovf);
        nfree = E::bcast(nfree);
        E::sync();
        if (ovf) { res.exit = EPA_OVERFLOW_MID; return true; }
        if (nsil == 0) {
            if (tol.best_on_failure) {
                st.face_points(b0, b1, b2, res.p1, res.p2);
                res.n = to_r(bn);
                res.exit = EPA_OK_PRECISION;
                res.status |= NCG_STATUS_EPA_PRECISION_LIMIT;
                return true;
            }
            res.status |= NCG_STATUS_EPA_FAILED;
            return true;
        }

        // ---- which silhouette edges still border a live face (after the whole fill)
        for (int k = lane; k < nsil; k += E::W) st.sflag[k] = st.live(st.sref[k]) ? 1 : 0;
        E::sync();
        // ---- slots for the new faces, in silhouette order (lane 0)
        int built = 0;
        if (lane == 0) {
            int first = -1, prev = -1;
            for (int k = 0; k < nsil; ++k) {
                if (!(st.sflag[k] & 1)) continue;
                int slot;
                uint32_t gg;
                if (nfree > 0) { slot = (int)st.freel[--nfree]; gg = st.gen(slot); }
                else if (nfresh < st.FC) { slot = nfresh++; gg = 0; }
                else { ovf = 1; break; }
                uint32_t r = mkref(slot, gg);
                st.snew[k] = r;
                if (prev >= 0) { st.snext[prev] = r; st.sprev[k] = st.snew[prev]; }
                if (first < 0) first = k;
                prev = k;
                built++;
            }
            if (!ovf && built > 0) {  // close the ring (epa3.rs:415-416)
                st.snext[prev] = st.snew[first];
                st.sprev[first] = st.snew[prev];
            }
        }
        ovf = E::bcast(ovf);
        built = E::bcast(built);
        nfree = E::bcast(nfree);
        nfresh = E::bcast(nfresh);
        E::sync();
        if (ovf) { res.exit = EPA_OVERFLOW_MID; return true; }
        if (built == 0) {  // epa3.rs:409-413
            if (tol.best_on_failure) {
                st.face_points(b0, b1, b2, res.p1, res.p2);
                res.n = to_r(bn);
                res.exit = EPA_OK_PRECISION;
                res.status |= NCG_STATUS_EPA_PRECISION_LIMIT;
                return true;
            }
            res.status |= NCG_STATUS_EPA_FAILED;
            return true;
        }
        // ---- build the new faces, one lane per live edge
        for (int k = lane; k < nsil; k += E::W) {
            if (!(st.sflag[k] & 1)) continue;
            uint32_t sr = st.sref[k];
            int sf = rslot(sr), so = st.sopp[k];
            int q1 = st.pt(sf, (so + 2) % 3), q2 = st.pt(sf, (so + 1) % 3);
            uint32_t r = st.snew[k];
            real dist;
            bool in = st.build_face(rslot(r), r >> 16, q1, q2, sup, sr, st.snext[k], st.sprev[k], eps, dist);
            st.sdist[k] = make_float2(dist.h, dist.l);
            st.sflag[k] = (uint8_t)(1 | (in ? 2 : 0));
        }
        E::sync();

        // ---- ordered post-pass (lane 0): adjacency, checks, heap pushes
        int outcome = 0;  // 0 continue, 1 numeric return, 2 None, 3 overflow
        if (lane == 0) {
            for (int k = 0; k < nsil; ++k) {
                uint8_t fl = st.sflag[k];
                if (!(fl & 1)) continue;
                int sf = rslot(st.sref[k]), so = st.sopp[k];
                st.set_adj(sf, (so + 1) % 3, st.snew[k]);
                if (fl & 2) {
                    real dist(st.sdist[k].x, st.sdist[k].y);
                    if (dist < curr) { outcome = 1; break; }
                    if (-dist > eps_tol) { outcome = 2; break; }
                    if (!st.push(hsize, seq, st.snew[k], -dist)) { outcome = 3; break; }
                }
            }
        }
        outcome = E::bcast(outcome);
        hsize = E::bcast(hsize);
        seq = E::bcast(seq);
        E::sync();
        if (outcome == 1) {
            st.face_points(f0, f1, f2, res.p1, res.p2);
            res.n = fnrm;
            res.exit = EPA_OK_NUMERIC;
            return true;
        }
        if (outcome == 2) {
            if (tol.best_on_failure) {
                st.face_points(b0, b1, b2, res.p1, res.p2);
                res.n = to_r(bn);
                res.exit = EPA_OK_PRECISION;
                res.status |= NCG_STATUS_EPA_PRECISION_LIMIT;
                return true;
            }
            res.status |= NCG_STATUS_EPA_FAILED;
            return true;
        }
        if (outcome == 3) { res.exit = EPA_OVERFLOW_MID; return true; }
        niter += 1;
        if (niter > max_iter) {
            res.status |= NCG_STATUS_EPA_MAX_ITER;
            return true;
        }
    }
    return false;
}

// A polytope between two expansion steps, copied out of a store: a 64-byte
// header (the EpaState scalars), then the used parts of the store's vertex,
// witness, face, heap and free-list arrays, each at the offset it would have
// for a store of capacities (VC, FC) whose heap holds FC entries.  Slots, generations, heap entries and
// push sequences are copied unchanged, so a store with at least those
// capacities continues exactly where this one stopped.
struct EpaSpill {
    static constexpr __host__ __device__ size_t bytes(int VC, int FC) {
        return 64 + 16 * (size_t)VC + 24 * (size_t)VC + 32 * (size_t)FC + 16 * (size_t)FC + 4 * (size_t)FC;
    }
    NCG_DEV static float4* vpt(char* r) { return (float4*)(r + 64); }
    NCG_DEV static float* vo(char* r, int VC) { return (float*)(r + 64 + 16 * (size_t)VC); }
    NCG_DEV static float4* face(char* r, int VC) { return (float4*)(r + 64 + 40 * (size_t)VC); }
    NCG_DEV static float4* heap(char* r, int VC, int FC) { return (float4*)(r + 64 + 40 * (size_t)VC + 32 * (size_t)FC); }
    NCG_DEV static uint32_t* freel(char* r, int VC, int FC) {
        return (uint32_t*)(r + 64 + 40 * (size_t)VC + 48 * (size_t)FC);
    }
};

// Writes store `st` and state S (between two steps) to spill record r, laid
// out for capacities (VC, FC) of the source store.  With WarpExec the lanes
// share the copy.
template <class E>
NCG_DEV void epa_spill(const EpaStore& st, const EpaState& S, char* r) {
    const int lane = E::lane();
    if (lane == 0) {
        int4* h = (int4*)r;
        h[0] = make_int4(S.nv, S.nfresh, S.nfree, S.hsize);
        h[1] = make_int4(S.niter, (int)S.seq, S.b0, S.b1);
        h[2] = make_int4(S.b2, __float_as_int(S.bn.x), __float_as_int(S.bn.y), __float_as_int(S.bn.z));
        h[3] = make_int4(__float_as_int(S.max_dist.h), __float_as_int(S.max_dist.l), (int)S.res.iters,
                         (int)S.res.status);
    }
    float4* vp = EpaSpill::vpt(r);
    float* vo = EpaSpill::vo(r, st.VC);
    float4* fa = EpaSpill::face(r, st.VC);
    float4* hp = EpaSpill::heap(r, st.VC, st.FC);
    uint32_t* fl = EpaSpill::freel(r, st.VC, st.FC);
    for (int i = lane; i < S.nv; i += E::W) vp[i] = st.vpt[i];
    for (int i = lane; i < 6 * S.nv; i += E::W) vo[i] = st.vo[i];
    for (int i = lane; i < 2 * S.nfresh; i += E::W) fa[i] = st.face[i];
    for (int i = lane; i < S.hsize; i += E::W) hp[i] = st.heap[i];
    for (int i = lane; i < S.nfree; i += E::W) fl[i] = st.freel[i];
    E::sync();
}

// Loads spill record r (written from a store of capacities VC, FC) into store
// `st` and state S; false when `st` is smaller than the source store.
template <class E>
NCG_DEV bool epa_resume(const char* rc, int VC, int FC, EpaStore& st, EpaState& S) {
    if (st.VC < VC || st.FC < FC || st.HC < FC) return false;
    char* r = const_cast<char*>(rc);
    const int lane = E::lane();
    const int4* h = (const int4*)r;
    const int4 h0 = h[0], h1 = h[1], h2 = h[2], h3 = h[3];
    S.nv = h0.x; S.nfresh = h0.y; S.nfree = h0.z; S.hsize = h0.w;
    S.niter = h1.x; S.seq = (uint32_t)h1.y; S.b0 = h1.z; S.b1 = h1.w;
    S.b2 = h2.x;
    S.bn = mk(__int_as_float(h2.y), __int_as_float(h2.z), __int_as_float(h2.w));
    S.max_dist = real(__int_as_float(h3.x), __int_as_float(h3.y));
    S.res.exit = EPA_NONE;
    S.res.p1 = S.res.p2 = S.res.n = zero3<real>();
    S.res.iters = (uint32_t)h3.z;
    S.res.status = (uint32_t)h3.w;
    const float4* vp = EpaSpill::vpt(r);
    const float* vo = EpaSpill::vo(r, VC);
    const float4* fa = EpaSpill::face(r, VC);
    const float4* hp = EpaSpill::heap(r, VC, FC);
    const uint32_t* fl = EpaSpill::freel(r, VC, FC);
    for (int i = lane; i < S.nv; i += E::W) st.vpt[i] = vp[i];
    for (int i = lane; i < 6 * S.nv; i += E::W) st.vo[i] = vo[i];
    for (int i = lane; i < 2 * S.nfresh; i += E::W) st.face[i] = fa[i];
    for (int i = lane; i < S.hsize; i += E::W) st.heap[i] = hp[i];
    for (int i = lane; i < S.nfree; i += E::W) st.freel[i] = fl[i];
    E::sync();
    return true;
}

// EPA::closest_points from GJK's final simplex to the end.
template <class E, class Scan>
NCG_DEV EpaResult epa_run(const PairGeom& g, int dim, const CSO* sv, const Tol& tol, const Scan& scan, EpaStore& st,
                          int max_iter) {
    EpaState S;
    if (epa_begin<E>(g, dim, sv, tol, scan, st, S)) return S.res;
    while (!epa_step<E>(g, tol, scan, st, S, max_iter)) {
    }
    return S.res;
}

}  // namespace ncg
