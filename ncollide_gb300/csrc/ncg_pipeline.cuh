// ncg_pipeline.cuh — types and output writers shared by the GJK stage
// (ncg_gjk.cu) and the EPA stages and host code (ncg_kernels.cu) of one
// batched query, and the GJK stage's host-side launchers.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

#include "ncg_core.cuh"
#include "ncg_epa.cuh"
#include "ncg_query.cuh"
#include "ncg_sort.cuh"

namespace ncg {

enum QueryKind { Q_CONTACT = 0, Q_DISTANCE = 1, Q_PROXIMITY = 2, Q_CLOSEST = 3 };

struct Outputs {
    ncg_contact* contact;
    uint8_t* tag;
    float* dir;
    float* value;
    float* points;
    uint32_t* status;
    uint32_t* iters;
};

struct QueryParams {
    int query;
    int dispatch;  // ncg_dispatch (contact only)
    int use_init_dir;
    int gjk_max_iter;
    int epa_max_iter;
    dw_host param;  // prediction / margin
    Tol tol;
};

// EPA work item: the pair and GJK's final simplex (dim + 1 CSO points).
// `mode` 0: contact_support_map_support_map; 1: point projection of a ball's
// centre on a ConvexHull (query::contact dispatch), `flip` when the ball is
// the second shape.
// `spilled` 1: the thread stage's polytope was kept when the pair outgrew it,
// in spill record Scratch::spill_of[item]; 0: the next stage starts from the
// simplex.
struct __align__(16) EpaItem {
    uint32_t pair;
    uint32_t gjk_iters;
    uint32_t status;
    uint8_t dim, mode, flip, spilled;
    float v[4][9];
};

// EPA queues: 0 the thread stage; 1 and 2 the first warp stage (1: pairs of two
// curved shapes, whose polytopes grow longest, drained first; 2: the rest);
// 3 the later warp stage; 4 the thread stage's ConvexHull pairs (a query
// runs the thread stage over queue 0 before the ConvexHull GJK, then over
// queue 4) or, in the no-allocation path, the last warp stage.
constexpr int N_EPA_QUEUES = 5;
// Sort keys of the query pipeline: the analytic kind pairs, then each
// ConvexHull size bucket split into HULL_SUB sub-buckets by the index range of
// the pair's first ConvexHull shape, so that pairs sharing hulls run close
// together (their points stay in L1 and L2) when a batch reuses its shapes.
// Measured on 4,194,304 ConvexHull pairs over 65,536 hulls: contact 265.7 ms
// ungrouped, 243.8 / 241.5 / 237.7 ms with 64 / 512 / 4096 sub-buckets.
#ifndef NCG_HULL_SUB
#define NCG_HULL_SUB 4096
#endif
constexpr int HULL_SUB = NCG_HULL_SUB;
static_assert(HULL_SUB >= 1 && HULL_SUB <= 65536, "sub-buckets are stored in 16 bits");
constexpr int N_SORT_KEYS = NB_ANALYTIC + NB_HULL * HULL_SUB;
constexpr int Q_WARP_LONG = 1, Q_WARP = 2, Q_THREAD_HULL = 4;

struct DevCounters {
    unsigned long long n_analytic, n_hull;
    unsigned long long hull_next;
    unsigned long long gjk_next[2];  // next entry of the thread GJK kernels' lists (dynamic fetch)
    unsigned long long n_items;       // EPA work items written
    unsigned long long epa_count[N_EPA_QUEUES];  // items per queue
    unsigned long long epa_next[N_EPA_QUEUES];
    unsigned long long gjk_iters, epa_iters;
    uint32_t bucket_n[NB], bucket_fill[NB];
    uint32_t mlp_err;  // bit 0: a learned warm-start tensor-core wait timed out
    uint32_t stage_err;  // bit 0: a hull-stage bulk-copy wait timed out (the pair read global memory)
    unsigned long long spill_next;  // spill records taken
    // the sort keys' counts, fill positions and first slots (device only:
    // the host copies the counters up to key_n)
    uint32_t key_n[N_SORT_KEYS], key_fill[N_SORT_KEYS], key_base[N_SORT_KEYS];
};
constexpr size_t CTR_SLOT = (sizeof(DevCounters) + 4095) / 4096 * 4096;
static_assert(sizeof(DevCounters) <= CTR_SLOT, "counters must fit their slot");
constexpr size_t CTR_HOST_BYTES = offsetof(DevCounters, key_n);

struct Scratch {
    // Shape kinds of a pair's two shapes (validated by k_classify).
    NCG_DEV uint32_t bucket_kind1(const ncg_batch& b, uint32_t i) const { return __ldg(&b.shapes[b.g1[i]].kind); }
    NCG_DEV uint32_t bucket_kind2(const ncg_batch& b, uint32_t i) const { return __ldg(&b.shapes[b.g2[i]].kind); }
    uint8_t* bucket;  // per pair: its cost bucket, NO_BUCKET for bad input
    uint16_t* sub;    // per ConvexHull pair: its locality sub-bucket
    uint32_t loc_shift;  // sub-bucket = first hull shape index >> loc_shift (capped); >= 32: one sub-bucket
    uint32_t* sorted;  // pair indices by bucket: analytic pairs, then hull pairs
    uint32_t* queue[N_EPA_QUEUES];  // item indices per EPA stage
    EpaItem* items;
    DevCounters* ctr;
    char* slabs[2];  // global EPA stores of the warp stages that use them, one per block
    size_t slab_bytes[2];
    int n_slabs[2];
    char* spill;          // spill records of the thread stage (nullptr: none)
    uint32_t* spill_of;   // per EPA item: its spill record (valid when the item is `spilled`)
    size_t spill_bytes;   // bytes per record
    uint32_t spill_cap;   // records
};

NCG_DEV uint32_t pack_iters(uint32_t g, uint32_t e) { return (g > 0xffffu ? 0xffffu : g) | ((e > 0xffffu ? 0xffffu : e) << 16); }

// Results leave the device as the high word of each double-word.
NCG_DEV void wr3(float* p, vec3<real> v) {
    p[0] = v.x.h;
    p[1] = v.y.h;
    p[2] = v.z.h;
}

// Writes the outputs of a finished pair (every query except an EPA-bound contact).
NCG_DEV void write_outputs(const QueryParams& qp, const Outputs& o, uint32_t i, const GjkOut& r,
                           vec3<float> init_dir, uint32_t status, uint32_t iters) {
    switch (qp.query) {
    case Q_CONTACT: {
        ncg_contact c;
        memset(&c, 0, sizeof(c));
        uint8_t tag = 0;
        if (r.kind == GJK_CLOSEST_POINTS) {
            tag = 1;
            wr3(c.world1, r.p1);
            wr3(c.world2, r.p2);
            wr3(c.normal, r.dir);
            c.depth = (-dot(r.dir, r.p2 - r.p1)).h;
        }
        o.contact[i] = c;
        o.tag[i] = tag;
        if (o.dir) wr3(o.dir + 3 * (size_t)i, r.dir);
        break;
    }
    case Q_DISTANCE:
        o.value[i] = r.kind == GJK_CLOSEST_POINTS ? vnorm(r.p2 - r.p1).h : 0.0f;
        break;
    case Q_PROXIMITY: {
        uint8_t t = r.kind == GJK_INTERSECTION ? NCG_INTERSECTING
                    : r.kind == GJK_PROXIMITY  ? NCG_WITHIN_MARGIN
                                               : NCG_DISJOINT;
        o.tag[i] = t;
        if (o.dir) {
            float* d = o.dir + 3 * (size_t)i;
            if (r.kind == GJK_INTERSECTION) { d[0] = init_dir.x; d[1] = init_dir.y; d[2] = init_dir.z; }
            else wr3(d, r.dir);
        }
        break;
    }
    default: {
        uint8_t t = r.kind == GJK_CLOSEST_POINTS ? NCG_CP_WITHIN_MARGIN
                    : r.kind == GJK_NO_INTERSECTION ? NCG_CP_DISJOINT
                                                    : NCG_CP_INTERSECTING;
        o.tag[i] = t;
        if (o.points) {
            float* p = o.points + 6 * (size_t)i;
            if (t == NCG_CP_WITHIN_MARGIN) { wr3(p, r.p1); wr3(p + 3, r.p2); }
            else { for (int k = 0; k < 6; ++k) p[k] = 0.0f; }
        }
        break;
    }
    }
    o.status[i] = status;
    if (o.iters) o.iters[i] = iters;
}

// Writes a contact of the query::contact routes (explicit depth; the normal as
// the returned direction, zeros when there is no contact).
NCG_DEV void write_qcontact(const Outputs& o, uint32_t i, const QContact& q, uint32_t status, uint32_t iters) {
    ncg_contact c;
    memset(&c, 0, sizeof(c));
    if (q.tag) {
        wr3(c.world1, q.p1);
        wr3(c.world2, q.p2);
        wr3(c.normal, q.n);
        c.depth = q.depth.h;
    }
    o.contact[i] = c;
    o.tag[i] = (uint8_t)q.tag;
    if (o.dir) wr3(o.dir + 3 * (size_t)i, q.n);
    o.status[i] = status | q.status;
    if (o.iters) o.iters[i] = iters;
}

// A pair with an invalid shape index or hull slice: no contact, distance 0,
// Disjoint, and NCG_STATUS_BAD_INPUT (the reference would index out of bounds).
NCG_DEV void write_bad(const QueryParams& qp, const Outputs& o, uint32_t i) {
    GjkOut r;
    r.kind = GJK_NO_INTERSECTION;
    r.p1 = r.p2 = r.dir = zero3<real>();
    write_outputs(qp, o, i, r, zero3<float>(), NCG_STATUS_BAD_INPUT, 0);
}

NCG_DEV void warp_add(unsigned long long* dst, unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31u) == 0 && v) atomicAdd(dst, v);
}

// ---- EPA store capacities ------------------------------------------------------
// EPA store capacities: vertices, live face slots (about twice the vertices),
// silhouette edges, flood-fill stack.  Store 0 is the per-thread store, 1-4
// the warp stores (shared memory or one global slab per block).
template <int T> struct EpaTier;
// Compile-time tuning: the thread stage's capacity and its minimum resident
// blocks per SM (which caps its registers).
#ifndef NCG_EPA_THREAD_VC
#define NCG_EPA_THREAD_VC 64
#endif
#ifndef NCG_EPA_THREAD_MIN_BLOCKS
#define NCG_EPA_THREAD_MIN_BLOCKS 4
#endif
template <> struct EpaTier<0> {
    static constexpr int VC = NCG_EPA_THREAD_VC, FC = 2 * VC + 16, SC = VC < 64 ? 32 : VC / 2, TC = 2 * VC, HC = FC;
};
// 1: shared-memory warp store (the no-allocation path); 2: the warp stage's
// global slabs; 3: the wide stage (one global slab per SM).
template <> struct EpaTier<1> { static constexpr int VC = 128, FC = 2 * 128 + 64, SC = 64, TC = 256, HC = FC; };
template <> struct EpaTier<2> { static constexpr int VC = 1280, FC = 2 * 1280 + 64, SC = 512, TC = 2048, HC = FC; };
// The wide stage's heap holds 64Ki entries: the f32 build keeps every deleted
// face's entry, as Rust's heap does (a 10 000-step run creates ~50 000 faces).
template <> struct EpaTier<3> {
    static constexpr int VC = 10240, FC = 2 * 10240 + 64, SC = 4096, TC = 16384, HC = 65536;
};
static_assert(EpaTier<0>::HC == EpaTier<0>::FC, "spill records lay the heap out with FC entries");
static_assert(EpaTier<3>::FC < 65536 && EpaTier<3>::VC < 65536, "16-bit face and vertex indices");
// Warps per SM of the warp stage (registers allow 12 at 168 per thread).
#ifndef NCG_WARP_STAGE_PER_SM
#define NCG_WARP_STAGE_PER_SM 12
#endif
constexpr int WARP_STAGE_MAX_PER_SM = NCG_WARP_STAGE_PER_SM;
template <int T> constexpr size_t tier_bytes() {
    return EpaStore::bytes(EpaTier<T>::VC, EpaTier<T>::FC, EpaTier<T>::SC, EpaTier<T>::TC, EpaTier<T>::HC);
}


// A warp EPA stage's queues and store: it drains queue q_in, then q_in2 (when
// >= 0); a pair whose polytope outgrows the store is queued on q_out and
// continues there, or, when q_out < 0, ends with NCG_STATUS_EPA_CAPACITY.
struct TierCaps {
    int q_in, q_in2, q_out;
    int slab;  // -1: shared memory; else index into Scratch::slabs
    int VC, FC, SC, TC, HC;
};
template <int T> TierCaps caps(int q_in, int q_in2, int q_out, int slab) {
    return TierCaps{q_in, q_in2, q_out, slab, EpaTier<T>::VC, EpaTier<T>::FC, EpaTier<T>::SC, EpaTier<T>::TC,
                    EpaTier<T>::HC};
}
// Bytes of a thread-stage spill record (the thread store's polytope).
constexpr size_t SPILL_BYTES = (EpaSpill::bytes(EpaTier<0>::VC, EpaTier<0>::FC) + 255) & ~size_t(255);

// ---- the stage launchers ------------------------------------------------------
// The GJK stage (ncg_gjk.cu) and the EPA stages (ncg_epa_stages.cu) are each
// built twice: in namespace dwa with the double-word sub-solve (the default
// arithmetic) and in namespace f32a with the reference's f32 path throughout
// (NCG_ARITH_F32).  Both builds share these declarations.
#define NCG_STAGE_API                                                                                              \
    /* Validates the pairs, writes the outputs of bad ones and counting-sorts */                                  \
    /* the rest into s.sorted (k_classify, k_bucket): two launches over n pairs. */                               \
    void gjk_launch_sort(const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s,           \
                         cudaStream_t st);                                                                         \
    /* One thread per pair over list 0 (analytic pairs) or 1 (the ConvexHull pairs */                             \
    /* after the first `warp_buckets` hull buckets); EPA work items go to */                                      \
    /* thread-stage queue `epa_queue`, those of the hull buckets before */                                        \
    /* `epa_warp_buckets` to the warp stage. */                                                                   \
    void gjk_launch_thread(int grid, const ncg_batch& b, const QueryParams& qp, const Outputs& o,                 \
                           const Scratch& s, int list, int warp_buckets, int epa_queue, int epa_warp_buckets,     \
                           cudaStream_t st);                                                                       \
    /* One warp per pair over the ConvexHull pairs of the first `warp_buckets` */                                 \
    /* hull buckets (the largest hulls); with stage_min > 0, pairs whose hulls */                                 \
    /* hold at least stage_min points are staged in shared memory (stage_cap */                                   \
    /* points per warp) by bulk copies. */                                                                         \
    void gjk_launch_warp(int grid, const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s, \
                         int warp_buckets, uint32_t stage_min, uint32_t stage_cap, cudaStream_t st);               \
    /* Dynamic shared memory of a staged warp-GJK block (4 warps of stage_cap points). */                        \
    size_t gjk_warp_stage_bytes(uint32_t stage_cap);                                                               \
    /* Allows the staged kernel that much shared memory and returns its resident */                              \
    /* blocks per SM (0 if it cannot run). */                                                                      \
    int gjk_warp_stage_occupancy(uint32_t stage_cap);                                                              \
    /* Resident 128-thread blocks per SM of the thread and warp GJK kernels. */                                  \
    void gjk_occupancy(int* occ_thread, int* occ_warp);                                                            \
    /* Shared-memory carveout preference of the thread GJK kernel. */                                            \
    cudaError_t gjk_set_carveout(int pct);                                                                         \
    /* The thread EPA stage over queue q (one thread per pair, 128-thread blocks). */                            \
    void epa_launch_thread(int grid, const ncg_batch& b, const QueryParams& qp, const Outputs& o,                 \
                           const Scratch& s, int q, cudaStream_t st);                                              \
    /* A warp EPA stage (one warp per block); smem > 0 holds the store in */                                     \
    /* dynamic shared memory (tc.slab < 0). */                                                                     \
    void epa_launch_warp(int grid, size_t smem, const ncg_batch& b, const QueryParams& qp, const Outputs& o,      \
                         const Scratch& s, TierCaps tc, cudaStream_t st);                                          \
    /* Resident blocks per SM of the EPA kernels: the thread stage, a warp stage */                              \
    /* on global slabs, and with the stores of EpaTier<1> / <2> in shared memory */                              \
    /* (allows the warp kernel that much shared memory). */                                                        \
    void epa_occupancy(int* occ_thread, int* occ_global, int occ_smem[2]);                                         \
    /* Shared-memory carveout preference of the thread EPA kernel. */                                            \
    cudaError_t epa_set_carveout(int pct);

namespace dwa {
NCG_STAGE_API
}  // namespace dwa
namespace f32a {
NCG_STAGE_API
}  // namespace f32a

}  // namespace ncg
