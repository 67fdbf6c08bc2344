// ncg_gjk.cu — the GJK stage of a batched query: classification and the
// counting sort by cost bucket, then GJK one thread per pair (analytic list,
// and the ConvexHull list by default) or one warp per pair (ConvexHull list).
// Pairs whose contact needs EPA leave their final simplex in the EPA queue.
// Compiled twice into the library: as is (namespace dwa, the double-word
// sub-solve) and through ncg_gjk_f32.cu with NCG_REAL_F32 (namespace f32a,
// the reference's f32 path).
//
// The double-word sum, quotient and square root are kept out of line in this
// translation unit: the GJK loop is bound by instruction fetch (its warps sit
// in different sub-solver branches), and one shared copy of each operation
// roughly halves its time.  The EPA stages (ncg_kernels.cu) keep them inline.
#define NCG_DW_OUTLINE 1

#include <cuda_runtime.h>

#include "ncg_pipeline.cuh"
#include "ncg_tc.cuh"

#ifndef NCG_GJK_THREAD_MIN_BLOCKS
#define NCG_GJK_THREAD_MIN_BLOCKS 4
#endif
// Minimum resident 128-thread blocks per SM of the warp-per-pair GJK kernel
// (1: no register cap).
#ifndef NCG_GJK_WARP_MIN_BLOCKS
#define NCG_GJK_WARP_MIN_BLOCKS 1
#endif

namespace ncg {
namespace NCG_ARITH_NS {
namespace {

// First search direction of each *_with_params wrapper.  An all-zero
// init_dir entry means None (no unit vector is zero): the default is used.
NCG_DEV vec3<float> initial_dir(const QueryParams& qp, const ncg_batch& b, uint32_t i, const PairGeom& g) {
    vec3<float> d;
    float n;
    vec3<float> given{0.0f, 0.0f, 0.0f};
    bool has = false;
    if (qp.use_init_dir && b.init_dir) {
        const float* p = b.init_dir + 3 * (size_t)i;
        given = {p[0], p[1], p[2]};
        has = !(given.x == 0.0f && given.y == 0.0f && given.z == 0.0f);
    }
    if (qp.query == Q_CONTACT || qp.query == Q_PROXIMITY) {
        if (has) return given;
        if (try_normalize(g.m2.t - g.m1.t, qp.tol.init_eps, d, n)) return d;
        return {1.0f, 0.0f, 0.0f};
    }
    vec3<float> d0 = has ? given : g.m1.t - g.m2.t;
    if (try_normalize(d0, qp.tol.init_eps, d, n)) return d;
    return {1.0f, 0.0f, 0.0f};
}

// Runs one pair through GJK; writes its outputs or its EPA work item.
// All lanes of a warp call this with the same pair when Scan is WarpScan.
// epa_queue: the EPA stage the pair starts in (0 = thread stage, 1 = warp tier A).
// Writes an EPA work item (GJK's final simplex) and queues it for `queue`.
NCG_DEV void enqueue_epa(const Scratch& s, uint32_t i, int queue, const Simplex& sx, uint32_t iters, uint32_t status,
                         int mode, bool flip) {
    unsigned long long slot = atomicAdd(&s.ctr->n_items, 1ull);
    unsigned long long pos = atomicAdd(&s.ctr->epa_count[queue], 1ull);
    s.queue[queue][pos] = (uint32_t)slot;
    EpaItem& it = s.items[slot];
    it.pair = i;
    it.gjk_iters = iters;
    it.status = status;
    it.dim = (uint8_t)sx.dim;
    it.mode = (uint8_t)mode;
    it.flip = flip ? 1 : 0;
    it.spilled = 0;
    for (int k = 0; k <= sx.dim; ++k) {
        const CSO& c = sx.v[k];
        float* w = it.v[k];
        w[0] = c.p.x; w[1] = c.p.y; w[2] = c.p.z;
        w[3] = c.o1.x; w[4] = c.o1.y; w[5] = c.o1.z;
        w[6] = c.o2.x; w[7] = c.o2.y; w[8] = c.o2.z;
    }
}

// Runs one pair through GJK; writes its outputs or its EPA work item.
// All lanes of a warp call this with the same pair when Scan is WarpScan.
// epa_queue: the EPA stage the pair starts in (0 = thread stage, 1 = warp tier A).
// Both GJK routes (the pair itself, or the point projection of a ball's centre
// on a ConvexHull) share one inlined GJK loop to keep the kernel's code small.
template <class Scan>
NCG_DEV void gjk_pair(const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s, uint32_t i,
                      const Scan& scan, bool writer, unsigned long long& iter_acc, int epa_queue) {
    PairGeom g;
    load_shape(b, b.g1[i], g.g1);
    load_shape(b, b.g2[i], g.g2);
    g.m1 = load_pose(b.m1 + i);
    g.m2 = load_pose(b.m2 + i);
    int mode = 0;  // 0: GJK on the pair; 1: point projection of a ball's centre on a hull
    bool flip = false;
    const real pred = from_host(qp.param);
    vec3<float> d;
    real max_dist;
    bool exact;
    if (qp.query == Q_CONTACT && qp.dispatch == NCG_DISPATCH_QUERY) {
        const bool b1 = g.g1.kind == NCG_BALL, b2 = g.g2.kind == NCG_BALL;
        const bool p1 = g.g1.kind == NCG_CUBOID || g.g1.kind == NCG_CONVEX_HULL;
        const bool p2 = g.g2.kind == NCG_CUBOID || g.g2.kind == NCG_CONVEX_HULL;
        if (b1 && b2) {
            QContact q = contact_ball_ball(g.m1.t, g.g1.p0, g.m2.t, g.g2.p0, pred);
            if (writer) write_qcontact(o, i, q, 0, 0);
            return;
        }
        if ((b1 && p2) || (p1 && b2)) {
            flip = !b1;
            const Pose& pb = flip ? g.m2 : g.m1;
            const Shape& sb = flip ? g.g2 : g.g1;
            const Pose& pp = flip ? g.m1 : g.m2;
            const Shape& sp = flip ? g.g1 : g.g2;
            if (sp.kind == NCG_CUBOID) {
                bool inside;
                vec3<float> pr;
                int fk, fi;
                aabb_project_with_feature(pp, mk(sp.p0, sp.p1, sp.p2), pb.t, inside, pr, fk, fi);
                QContact q = ball_polyhedron_assemble(pb.t, sb.p0, inside, to_r(pr), fk, fi, true, pred, flip);
                if (writer) write_qcontact(o, i, q, 0, 0);
                return;
            }
            // point_projection_on_support_map: GJK on the translated hull
            mode = 1;
        }
    }
    PairGeom gg = g;
    if (mode == 1) {
        gg = projection_geom(flip ? g.m1 : g.m2, flip ? g.g1 : g.g2, flip ? g.m2.t : g.m1.t);
        float dn;
        if (!try_normalize(-gg.m1.t, FLT_EPSILON, d, dn)) d = mk(1.0f, 0.0f, 0.0f);
        max_dist = dw_max();
        exact = true;
    } else {
        d = initial_dir(qp, b, i, g);
        max_dist = qp.query == Q_DISTANCE ? dw_max() : pred;
        exact = qp.query != Q_PROXIMITY;
    }
    Simplex sx;
    sx.reset(cso_support(gg, d, scan));
    uint32_t iters = 0, status = 0;
    GjkOut r = gjk(gg, max_dist, exact, sx, qp.tol, scan, iters, status, qp.gjk_max_iter);
    iter_acc += iters;
    if (qp.query == Q_CONTACT && r.kind == GJK_INTERSECTION) {
        if (writer) enqueue_epa(s, i, epa_queue, sx, iters, status, mode, flip);
        return;
    }
    if (mode == 1) {
        const Pose& pb = flip ? g.m2 : g.m1;
        const Shape& sb = flip ? g.g2 : g.g1;
        bool inside = r.kind != GJK_CLOSEST_POINTS;  // the iteration cap: unreachable!() in gjk.rs:57
        vec3<real> w2 = inside ? to_r(pb.t) : r.p1 + to_r(pb.t);
        QContact q = ball_polyhedron_assemble(pb.t, sb.p0, inside, w2, F_UNKNOWN, 0, false, pred, flip);
        if (writer) write_qcontact(o, i, q, status, pack_iters(iters, 0));
        return;
    }
    if (writer) write_outputs(qp, o, i, r, d, status, pack_iters(iters, 0));
}

// The sort key of a valid pair: its analytic kind pair, or its ConvexHull
// size bucket's locality sub-bucket.
NCG_DEV int sort_key(int bucket, uint32_t sub) {
    return bucket < NB_ANALYTIC ? bucket : NB_ANALYTIC + (bucket - NB_ANALYTIC) * HULL_SUB + (int)sub;
}

// Validates every pair, writes the outputs of bad ones and counts the buckets
// and the sort keys.
__global__ void k_classify(ncg_batch b, QueryParams qp, Outputs o, Scratch s) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1, sk = 0;
    if (i < b.n_pairs) {
        Shape a, c;
        bool ok = load_shape(b, b.g1[i], a) && load_shape(b, b.g2[i], c);
        if (!ok) write_bad(qp, o, (uint32_t)i);
        else key = pair_bucket(a, c);
        s.bucket[i] = key < 0 ? NO_BUCKET : (uint8_t)key;
        if (key >= NB_ANALYTIC) {
            const uint32_t g = a.kind == NCG_CONVEX_HULL ? b.g1[i] : b.g2[i];
            const uint32_t sub = s.loc_shift >= 32 ? 0u : min(g >> s.loc_shift, (uint32_t)HULL_SUB - 1u);
            s.sub[i] = (uint16_t)sub;
            sk = sort_key(key, sub);
        } else if (key >= 0) {
            sk = key;
        }
    }
    (void)bucket_slot(s.ctr->bucket_n, key < 0 ? 0 : key, key >= 0);
    (void)bucket_slot(s.ctr->key_n, sk, key >= 0);
}

// First slot of every sort key (one block: an exclusive scan of the counts)
// and the lengths of the analytic and ConvexHull lists.
__global__ void __launch_bounds__(1024) k_sort_base(Scratch s) {
    __shared__ uint32_t part[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    constexpr int PER = (N_SORT_KEYS + 1023) / 1024;
    uint32_t v[PER], sum = 0;
    for (int j = 0; j < PER; ++j) {
        const int k = t * PER + j;
        v[j] = k < N_SORT_KEYS ? s.ctr->key_n[k] : 0u;
        sum += v[j];
    }
    uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) part[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t p = part[lane], q = p;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, q, o);
            if (lane >= o) q += y;
        }
        part[lane] = q - p;  // exclusive over warps
    }
    __syncthreads();
    uint32_t base = part[w] + incl - sum;
    for (int j = 0; j < PER; ++j) {
        const int k = t * PER + j;
        if (k < N_SORT_KEYS) s.ctr->key_base[k] = base;
        base += v[j];
    }
    if (t == 0) {
        unsigned long long na = 0, nh = 0;
        for (int k = 0; k < NB; ++k) (k < NB_ANALYTIC ? na : nh) += s.ctr->bucket_n[k];
        s.ctr->n_analytic = na;
        s.ctr->n_hull = nh;
    }
}

// Scatters the pairs into `sorted` by sort key: analytic kind pairs, then
// ConvexHull size buckets largest first, each by locality sub-bucket.  The
// order inside a key is arbitrary: every pair's result depends on the pair
// alone.
__global__ void k_bucket(ncg_batch b, Scratch s) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int key = i < b.n_pairs ? (int)s.bucket[i] : (int)NO_BUCKET;
    const bool active = key != NO_BUCKET;
    const int sk = active ? sort_key(key, key >= NB_ANALYTIC ? s.sub[i] : 0u) : 0;
    const uint32_t slot = bucket_slot(s.ctr->key_fill, sk, active);
    if (active) s.sorted[s.ctr->key_base[sk] + slot] = (uint32_t)i;
}

// Hull pairs in the first `warp_buckets` ConvexHull buckets (the largest
// hulls) run one warp per pair; the rest of the hull list one thread per pair.
NCG_DEV unsigned long long hull_warp_count(const Scratch& s, int warp_buckets) {
    unsigned long long n = 0;
    for (int k = 0; k < warp_buckets && k < NB_HULL; ++k) n += *(volatile uint32_t*)&s.ctr->bucket_n[NB_ANALYTIC + k];
    return n;
}

// Thread GJK scheduling (compile-time): 0 gives each thread the pairs
// start, start + grid, ... of its list; 1 (default) lets each thread take the
// next pair of the list when its pair ends (one atomic per group of lanes
// asking together, consecutive pairs to a group): analytic GJK 17% and hull
// GJK 6% faster on the mixed convex workload.
#ifndef NCG_GJK_THREAD_SCHED
#define NCG_GJK_THREAD_SCHED 1
#endif

// One thread per pair over a pair list (list 0: analytic pairs, list 1:
// ConvexHull pairs after the warp kernel's, whose points the thread scans
// itself); EPA starts in the thread stage, queue `epa_queue`, except for the
// hull pairs of buckets [warp_buckets, epa_warp_buckets) (the largest hulls
// after the warp kernel's), whose EPA starts in the warp stage (queue Q_WARP):
// a thread-per-pair EPA scans their hulls serially at every support point.
__global__ void __launch_bounds__(128, NCG_GJK_THREAD_MIN_BLOCKS)
k_gjk_thread(ncg_batch b, QueryParams qp, Outputs o, Scratch s, int list, int warp_buckets, int epa_queue,
             int epa_warp_buckets) {
    const unsigned long long na = *(volatile unsigned long long*)&s.ctr->n_analytic;
    const unsigned long long nw = list == 0 ? 0ull : hull_warp_count(s, warp_buckets);
    const unsigned long long nbig = list == 0 ? 0ull : hull_warp_count(s, epa_warp_buckets) - nw;
    const unsigned long long n = list == 0 ? na : *(volatile unsigned long long*)&s.ctr->n_hull - nw;
    const uint32_t* ids = list == 0 ? s.sorted : s.sorted + na + nw;
    ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    unsigned long long acc = 0;
#if NCG_GJK_THREAD_SCHED == 1
    for (;;) {
        const unsigned m = __activemask();
        const int lead = __ffs(m) - 1;
        const unsigned rank = __popc(m & ((1u << (threadIdx.x & 31u)) - 1u));
        unsigned long long base = 0;
        if ((int)(threadIdx.x & 31u) == lead) base = atomicAdd(&s.ctr->gjk_next[list & 1], (unsigned long long)__popc(m));
        base = __shfl_sync(m, base, lead);
        const unsigned long long k = base + rank;
        if (k >= n) break;
        gjk_pair(b, qp, o, s, ids[k], scan, true, acc, k < nbig ? Q_WARP : epa_queue);
    }
#else
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long start = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long rounds = (n + stride - 1) / stride;
    for (unsigned long long r = 0; r < rounds; ++r) {
        unsigned long long k = start + r * stride;
        if (k < n) gjk_pair(b, qp, o, s, ids[k], scan, true, acc, k < nbig ? Q_WARP : epa_queue);
    }
#endif
    warp_add(&s.ctr->gjk_iters, acc);
}

// Plans the shared-memory stage of pair i: its ConvexHull slices (one when
// both shapes are the same slice) if they hold at least `stage_min` points
// together; the first shape's slice, then the second's, each if it still fits
// in `cap` points.  Every lane computes the same plan.
NCG_DEV void plan_stage(const ncg_batch& b, uint32_t i, uint32_t stage_min, uint32_t cap, StagedWarpScan& sc) {
    sc.n[0] = sc.n[1] = 0;
    Shape a, c;
    const bool oka = load_shape(b, b.g1[i], a), okc = load_shape(b, b.g2[i], c);
    uint32_t na = (oka && a.kind == NCG_CONVEX_HULL) ? a.n : 0u;
    uint32_t nc = (okc && c.kind == NCG_CONVEX_HULL) ? c.n : 0u;
    if (na && nc && a.off == c.off && a.n == c.n) nc = 0;
    if (na + nc < stage_min) return;
    uint32_t used = 0;
    int k = 0;
    if (na && na <= cap) {
        sc.off[k] = a.off; sc.n[k] = na; sc.at[k] = 0; used = na; ++k;
    }
    if (nc && used + nc <= cap) {
        sc.off[k] = c.off; sc.n[k] = nc; sc.at[k] = used;
    }
}

// One warp per pair over the ConvexHull pairs of the first `warp_buckets`
// buckets, drained from a shared counter.  With STAGE, a pair whose hulls
// hold at least `stage_min` points first has them copied into its warp's
// shared-memory stage (`stage_cap` points per warp) by the bulk-copy engine
// (cp.async.bulk completing on an mbarrier), and its scans read shared memory
// instead of global memory.  On the mixed convex workload the stage costs more
// than it saves (every pair waits for its whole copy before its first scan,
// and a GJK run makes only a few scans, which L1 serves; a 2048-point stage
// also leaves one block per SM instead of two): off by default, a tuning key
// for the autotuner.  Every wait is bounded; a timeout sets
// ctr->stage_err and the kernel reads global memory from then on.
template <bool STAGE>
__global__ void __launch_bounds__(128, NCG_GJK_WARP_MIN_BLOCKS)
k_gjk_warp(ncg_batch b, QueryParams qp, Outputs o, Scratch s, int warp_buckets, uint32_t stage_min,
           uint32_t stage_cap) {
    extern __shared__ __align__(128) float4 stage[];  // [4 warps][stage_cap]
    __shared__ __align__(8) uint64_t bar[4];
    const unsigned long long n = hull_warp_count(s, warp_buckets);
    const uint32_t* ids = s.sorted + *(volatile unsigned long long*)&s.ctr->n_analytic;
    const float4* pts = reinterpret_cast<const float4*>(b.hull_points);
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    bool staging = STAGE && stage_min > 0 && stage_cap > 0 && (reinterpret_cast<uintptr_t>(pts) & 15u) == 0;
    uint32_t parity = 0;
    if (STAGE) {
        if (lane == 0) tc::mbar_init(&bar[w], 1);
        __syncwarp();
    }
    const uint32_t sbase = STAGE ? tc::smem_u32(stage + (size_t)w * stage_cap) : 0u;
    unsigned long long acc = 0;
    for (;;) {
        unsigned long long k = 0;
        if (lane == 0) k = atomicAdd(&s.ctr->hull_next, 1ull);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= n) break;
        const uint32_t i = ids[k];
        unsigned long long a = 0;
        if constexpr (STAGE) {
            StagedWarpScan scan{pts, sbase, {0u, 0u}, {0u, 0u}, {0u, 0u}};
            if (staging) {
                plan_stage(b, i, stage_min, stage_cap, scan);
                const uint32_t bytes = 16u * (scan.n[0] + scan.n[1]);
                if (bytes) {
                    __syncwarp();  // every lane has finished reading the previous pair's stage
                    if (lane == 0) {
                        tc::fence_async_smem();  // those reads come before the copy's writes
                        tc::mbar_arrive_expect_tx(&bar[w], bytes);
                        tc::bulk_g2s(sbase + 16u * scan.at[0], pts + scan.off[0], 16u * scan.n[0], &bar[w]);
                        if (scan.n[1]) tc::bulk_g2s(sbase + 16u * scan.at[1], pts + scan.off[1], 16u * scan.n[1], &bar[w]);
                    }
                    bool ok = tc::mbar_wait(&bar[w], parity, &s.ctr->stage_err);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok) {
                        // give the copies in flight a second bounded wait, then stop staging
                        (void)tc::mbar_wait(&bar[w], parity, &s.ctr->stage_err);
                        staging = false;
                        scan.n[0] = scan.n[1] = 0;
                    }
                    parity ^= 1u;
                }
            }
            gjk_pair(b, qp, o, s, i, scan, lane == 0, a, Q_WARP);
        } else {
            WarpScan scan{pts};
            gjk_pair(b, qp, o, s, i, scan, lane == 0, a, Q_WARP);
        }
        if (lane == 0) acc += a;
    }
    warp_add(&s.ctr->gjk_iters, acc);
}

}  // namespace

void gjk_launch_sort(const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s, cudaStream_t st) {
    const unsigned n = (unsigned)b.n_pairs;
    k_classify<<<(n + 255) / 256, 256, 0, st>>>(b, qp, o, s);
    k_sort_base<<<1, 1024, 0, st>>>(s);
    k_bucket<<<(n + 255) / 256, 256, 0, st>>>(b, s);
}

void gjk_launch_thread(int grid, const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s,
                       int list, int warp_buckets, int epa_queue, int epa_warp_buckets, cudaStream_t st) {
    k_gjk_thread<<<grid, 128, 0, st>>>(b, qp, o, s, list, warp_buckets, epa_queue,
                                       epa_warp_buckets > warp_buckets ? epa_warp_buckets : warp_buckets);
}

void gjk_launch_warp(int grid, const ncg_batch& b, const QueryParams& qp, const Outputs& o, const Scratch& s,
                     int warp_buckets, uint32_t stage_min, uint32_t stage_cap, cudaStream_t st) {
    if (stage_min > 0 && stage_cap > 0)
        k_gjk_warp<true><<<grid, 128, gjk_warp_stage_bytes(stage_cap), st>>>(b, qp, o, s, warp_buckets, stage_min,
                                                                             stage_cap);
    else
        k_gjk_warp<false><<<grid, 128, 0, st>>>(b, qp, o, s, warp_buckets, 0u, 0u);
}

size_t gjk_warp_stage_bytes(uint32_t stage_cap) { return 4u * 16u * (size_t)stage_cap; }

void gjk_occupancy(int* occ_thread, int* occ_warp) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ_thread, k_gjk_thread, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ_warp, k_gjk_warp<false>, 128, 0);
}

int gjk_warp_stage_occupancy(uint32_t stage_cap) {
    // the attribute is per function: allow the largest stage so that contexts
    // with different stage sizes can share the device
    if (cudaFuncSetAttribute(k_gjk_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gjk_warp_stage_bytes(2048)) != cudaSuccess)
        return 0;
    const size_t bytes = gjk_warp_stage_bytes(stage_cap);
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gjk_warp<true>, 128, bytes) != cudaSuccess) return 0;
    return occ;
}

cudaError_t gjk_set_carveout(int pct) {
    return cudaFuncSetAttribute(k_gjk_thread, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

}  // namespace NCG_ARITH_NS
}  // namespace ncg
