// ncg_epa_stages.cu — the EPA stages of a batched contact query: the thread
// stage (one thread per pair, the polytope in local memory) and the warp
// stages (one warp per pair, the polytope in shared memory or a global slab),
// with their host-side launchers.
//
// This file is compiled twice into the library: as is (namespace dwa, the
// double-word sub-solve) and through ncg_epa_stages_f32.cu with NCG_REAL_F32
// (namespace f32a, the reference's f32 path with its heap order).
#include <cuda_runtime.h>

#include <cstring>

#include "ncg_pipeline.cuh"

namespace ncg {
namespace NCG_ARITH_NS {
namespace {

// Writes a contact finished by EPA.
NCG_DEV void write_epa(const Outputs& o, const EpaItem& it, const EpaResult& r, uint32_t extra_status) {
    const uint32_t i = it.pair;
    ncg_contact c;
    memset(&c, 0, sizeof(c));
    uint8_t tag = 0;
    vec3<real> dir = mk(real(1.0f), real(0.0f), real(0.0f));
    if (epa_ok(r.exit)) {
        tag = 1;
        wr3(c.world1, r.p1);
        wr3(c.world2, r.p2);
        wr3(c.normal, r.n);
        c.depth = (-dot(r.n, r.p2 - r.p1)).h;
        dir = r.n;
    }
    o.contact[i] = c;
    o.tag[i] = tag;
    if (o.dir) wr3(o.dir + 3 * (size_t)i, dir);
    o.status[i] = it.status | r.status | extra_status;
    if (o.iters) o.iters[i] = pack_iters(it.gjk_iters, r.iters);
}

NCG_DEV PairGeom load_geom(const ncg_batch& b, uint32_t i) {
    PairGeom g;
    load_shape(b, b.g1[i], g.g1);
    load_shape(b, b.g2[i], g.g2);
    g.m1 = load_pose(b.m1 + i);
    g.m2 = load_pose(b.m2 + i);
    return g;
}

// The geometry an EPA work item runs on (mode 1: the translated hull against
// ConstantOrigin).
NCG_DEV PairGeom item_geom(const ncg_batch& b, const EpaItem& it) {
    PairGeom g = load_geom(b, it.pair);
    if (it.mode == 0) return g;
    const Pose& pb = it.flip ? g.m2 : g.m1;
    const Pose& pp = it.flip ? g.m1 : g.m2;
    const Shape& sp = it.flip ? g.g1 : g.g2;
    return projection_geom(pp, sp, pb.t);
}

// Finishes an EPA work item: a contact (mode 0) or the ball-hull contact from
// the EPA projection of the ball's centre (mode 1).
NCG_DEV void finish_epa(const ncg_batch& b, const QueryParams& qp, const Outputs& o, const EpaItem& it,
                        const EpaResult& r, uint32_t extra_status) {
    if (it.mode == 0) {
        write_epa(o, it, r, extra_status);
        return;
    }
    PairGeom g = load_geom(b, it.pair);
    const Pose& pb = it.flip ? g.m2 : g.m1;
    const Shape& sb = it.flip ? g.g2 : g.g1;
    const bool ok = epa_ok(r.exit);
    vec3<real> w2 = ok ? r.p1 + to_r(pb.t) : to_r(pb.t);
    QContact q = ball_polyhedron_assemble(pb.t, sb.p0, true, w2, F_UNKNOWN, 0, false, from_host(qp.param), it.flip != 0);
    write_qcontact(o, it.pair, q, it.status | r.status | extra_status, pack_iters(it.gjk_iters, r.iters));
}

NCG_DEV void load_simplex(const EpaItem& it, CSO* sv) {
    for (int k = 0; k <= it.dim; ++k) {
        const float* w = it.v[k];
        sv[k] = CSO{{w[0], w[1], w[2]}, {w[3], w[4], w[5]}, {w[6], w[7], w[8]}};
    }
}

// A warp EPA stage: one warp per pair (one warp per block), the polytope in
// dynamic shared memory or in a global-memory slab per block.  It drains queue
// q_in, then q_in2 (when >= 0); a pair whose polytope outgrows the store is
// queued on q_out and re-run there from GJK's simplex, or, when q_out < 0,
// ends with NCG_STATUS_EPA_CAPACITY.  One kernel serves every stage (runtime
// capacities) to keep the code footprint small.

#ifndef NCG_EPA_WARP_MIN_BLOCKS
#define NCG_EPA_WARP_MIN_BLOCKS 1
#endif
__global__ void __launch_bounds__(32, NCG_EPA_WARP_MIN_BLOCKS) k_epa(ncg_batch b, QueryParams qp, Outputs o, Scratch s, TierCaps tc) {
    extern __shared__ __align__(16) char smem[];
    const unsigned lane = threadIdx.x & 31u;
    EpaStore st;
    if (tc.slab < 0) {
        st.carve(smem, tc.VC, tc.FC, tc.SC, tc.TC, tc.HC);
    } else {
        if (blockIdx.x >= (unsigned)s.n_slabs[tc.slab]) return;
        st.carve(s.slabs[tc.slab] + (size_t)blockIdx.x * s.slab_bytes[tc.slab], tc.VC, tc.FC, tc.SC, tc.TC, tc.HC);
    }
    WarpScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    unsigned long long acc = 0;
    int q = tc.q_in;
    unsigned long long n = *(volatile unsigned long long*)&s.ctr->epa_count[q];
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(&s.ctr->epa_next[q], 1ull);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= n) {
            if (q == tc.q_in && tc.q_in2 >= 0) {
                q = tc.q_in2;
                n = *(volatile unsigned long long*)&s.ctr->epa_count[q];
                continue;
            }
            break;
        }
        const uint32_t item = s.queue[q][k];
        const EpaItem& it = s.items[item];
        PairGeom g = item_geom(b, it);
        EpaState S;
        bool done;
        if (it.spilled && epa_resume<WarpExec>(s.spill + (size_t)s.spill_of[item] * s.spill_bytes, EpaTier<0>::VC,
                                                EpaTier<0>::FC, st, S)) {
            // the thread stage's polytope: continue where it stopped
            done = false;
        } else {
            CSO sv[4];
            load_simplex(it, sv);
            done = epa_begin<WarpExec>(g, it.dim, sv, qp.tol, scan, st, S);
        }
        while (!done) done = epa_step<WarpExec>(g, qp.tol, scan, st, S, qp.epa_max_iter);
        const EpaResult& r = S.res;
        if (epa_overflow(r.exit) && tc.q_out >= 0) {
            if (lane == 0) {
                unsigned long long pos = atomicAdd(&s.ctr->epa_count[tc.q_out], 1ull);
                s.queue[tc.q_out][pos] = item;
            }
        } else {
            acc += r.iters;
            if (lane == 0) {
                if (epa_overflow(r.exit)) {
                    EpaResult none = r;
                    none.exit = EPA_NONE;
                    finish_epa(b, qp, o, it, none, NCG_STATUS_EPA_CAPACITY);
                } else {
                    finish_epa(b, qp, o, it, r, 0);
                }
            }
        }
        __syncwarp();
    }
    if (lane == 0 && acc) atomicAdd(&s.ctr->epa_iters, acc);
}
// The thread stage's scheduler: each thread takes the next EPA item from the
// queue as soon as its current one finishes (a pair needs 1 to ~60 steps
// here); with a fixed item per lane and round, the lanes whose pairs finished
// early would idle until the round's longest pair was done.
NCG_DEV void epa_thread_finish(const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s,
                               uint32_t item, const EpaResult& r, unsigned long long& acc, const EpaStore& st,
                               const EpaState& S) {
    EpaItem& it = s.items[item];
    if (epa_overflow(r.exit)) {
        // keep the polytope (when a spill record is free and the store
        // stopped between two steps) so that the warp stage resumes it
        // instead of repeating these iterations
        if (s.spill && r.exit == EPA_OVERFLOW) {
            const unsigned long long rec = atomicAdd(&s.ctr->spill_next, 1ull);
            if (rec < s.spill_cap) {
                epa_spill<ThreadExec>(st, S, s.spill + (size_t)rec * s.spill_bytes);
                s.spill_of[item] = (uint32_t)rec;
                it.spilled = 1;
            }
        }
        // pairs of two curved shapes (their polytopes grow longest) go first;
        // the shape kinds are re-read here (rare path) rather than kept live
        const uint32_t k1 = s.bucket_kind1(b, it.pair), k2 = s.bucket_kind2(b, it.pair);
        const bool curved = k1 != NCG_CUBOID && k1 != NCG_CONVEX_HULL && k2 != NCG_CUBOID && k2 != NCG_CONVEX_HULL;
        const int qo = curved ? Q_WARP_LONG : Q_WARP;
        unsigned long long pos = atomicAdd(&s.ctr->epa_count[qo], 1ull);
        s.queue[qo][pos] = item;
    } else {
        acc += r.iters;
        finish_epa(b, qp, o, it, r, 0);
    }
}

// Takes the next thread-stage queue entry: one atomic per group of lanes
// asking together, which get consecutive entries (pairs of one kind, adjacent).
NCG_DEV unsigned long long epa_thread_fetch(const Scratch& s, int q) {
    const unsigned m = __activemask();
    const int lead = __ffs(m) - 1;
    const unsigned rank = __popc(m & ((1u << (threadIdx.x & 31u)) - 1u));
    unsigned long long base = 0;
    if ((int)(threadIdx.x & 31u) == lead) base = atomicAdd(&s.ctr->epa_next[q], (unsigned long long)__popc(m));
    base = __shfl_sync(m, base, lead);
    return base + rank;
}

// Thread-stage scheduling (compile-time): 0 runs each item to its end, then
// takes the next (default); 1 advances every thread's pair by one expansion
// step per pass of one loop, taking a new item as soon as a pair ends (the
// lanes stay on the same step of the loop body whatever pairs they hold).
// Both take items dynamically; 1 measured 12% slower on mixed pairs and 11%
// on short cuboid pairs (a larger loop body around the step).
#ifndef NCG_EPA_THREAD_SCHED
#define NCG_EPA_THREAD_SCHED 0
#endif

NCG_DEV void epa_thread_loop(const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s,
                             EpaStore& st, int q) {
    const unsigned long long n = *(volatile unsigned long long*)&s.ctr->epa_count[q];
    ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    unsigned long long acc = 0;
    EpaState S;
    PairGeom g;
    uint32_t item = 0;
#if NCG_EPA_THREAD_SCHED == 0
    for (;;) {
        const unsigned long long k = epa_thread_fetch(s, q);
        if (k >= n) break;
        item = s.queue[q][k];
        const EpaItem& it = s.items[item];
        g = item_geom(b, it);
        CSO sv[4];
        load_simplex(it, sv);
        bool done = epa_begin<ThreadExec>(g, it.dim, sv, qp.tol, scan, st, S);
        while (!done) done = epa_step<ThreadExec>(g, qp.tol, scan, st, S, qp.epa_max_iter);
        epa_thread_finish(b, qp, o, s, item, S.res, acc, st, S);
    }
#else
    bool active = false;
    for (;;) {
        // take items until one needs expansion steps (or the queue is empty)
        while (!active) {
            const unsigned long long k = epa_thread_fetch(s, q);
            if (k >= n) break;
            item = s.queue[q][k];
            const EpaItem& it = s.items[item];
            g = item_geom(b, it);
            CSO sv[4];
            load_simplex(it, sv);
            if (epa_begin<ThreadExec>(g, it.dim, sv, qp.tol, scan, st, S))
                epa_thread_finish(b, qp, o, s, item, S.res, acc, st, S);
            else
                active = true;
        }
        if (!active) break;
        if (epa_step<ThreadExec>(g, qp.tol, scan, st, S, qp.epa_max_iter)) {
            epa_thread_finish(b, qp, o, s, item, S.res, acc, st, S);
            active = false;
        }
    }
#endif
    warp_add(&s.ctr->epa_iters, acc);
}


// Thread stage: one thread per pair, the polytope in the thread's local
// memory (L1 write-back; a per-thread global slab measured 17% slower, its
// stores write through to L2).  A pair that outgrows it goes to warp tier A.
constexpr size_t THREAD_STORE_BYTES =
    EpaStore::bytes(EpaTier<0>::VC, EpaTier<0>::FC, EpaTier<0>::SC, EpaTier<0>::TC, EpaTier<0>::HC);
__global__ void __launch_bounds__(128, NCG_EPA_THREAD_MIN_BLOCKS)
k_epa_thread(ncg_batch b, QueryParams qp, Outputs o, Scratch s, int q) {
    __align__(16) char buf[THREAD_STORE_BYTES];
    EpaStore st;
    st.carve(buf, EpaTier<0>::VC, EpaTier<0>::FC, EpaTier<0>::SC, EpaTier<0>::TC, EpaTier<0>::HC);
    epa_thread_loop(b, qp, o, s, st, q);
}



}  // namespace

void epa_launch_thread(int grid, const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s,
                       int q, cudaStream_t st) {
    k_epa_thread<<<grid, 128, 0, st>>>(b, qp, o, s, q);
}

void epa_launch_warp(int grid, size_t smem, const ncg_batch& b, const QueryParams& qp, const Outputs& o,
                     const Scratch& s, TierCaps tc, cudaStream_t st) {
    k_epa<<<grid, 32, smem, st>>>(b, qp, o, s, tc);
}

void epa_occupancy(int* occ_thread, int* occ_global, int occ_smem[2]) {
    cudaFuncSetAttribute(k_epa, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tier_bytes<2>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ_thread, k_epa_thread, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ_global, k_epa, 32, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_smem[0], k_epa, 32, tier_bytes<1>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_smem[1], k_epa, 32, tier_bytes<2>());
}

cudaError_t epa_set_carveout(int pct) {
    return cudaFuncSetAttribute(k_epa_thread, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

}  // namespace NCG_ARITH_NS
}  // namespace ncg
