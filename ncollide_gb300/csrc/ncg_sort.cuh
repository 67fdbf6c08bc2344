// ncg_sort.cuh — counting sort of pairs into cost buckets, shared by the
// query pipeline and the time of impact.
//
// Pairs are sorted before the GJK-type loops so that the threads of a warp run
// pairs of one shape-kind combination (analytic pairs) or of similar hull
// sizes (ConvexHull pairs): the hull arg-max scans of a warp then take about
// the same time.  Buckets 0-24: analytic kind pairs (k1 * 5 + k2, k1 <= k2);
// 25-36: ConvexHull pairs by floor(log2(points scanned)), largest first.
#pragma once

#include "ncg_core.cuh"

namespace ncg {

constexpr int NB_ANALYTIC = 25;
constexpr int NB_HULL = 12;
constexpr int NB = NB_ANALYTIC + NB_HULL;
constexpr uint8_t NO_BUCKET = 0xff;

NCG_DEV int pair_bucket(const Shape& a, const Shape& c) {
    if (a.kind == NCG_CONVEX_HULL || c.kind == NCG_CONVEX_HULL) {
        uint32_t n = (a.kind == NCG_CONVEX_HULL ? a.n : 0u) + (c.kind == NCG_CONVEX_HULL ? c.n : 0u);
        int lg = 31 - __clz(n);  // n >= 1: load_shape rejects empty hulls
        lg = lg < 3 ? 3 : (lg > 3 + NB_HULL - 1 ? 3 + NB_HULL - 1 : lg);
        return NB_ANALYTIC + (3 + NB_HULL - 1 - lg);
    }
    uint32_t k1 = a.kind < c.kind ? a.kind : c.kind, k2 = a.kind < c.kind ? c.kind : a.kind;
    return (int)(k1 * 5u + k2);
}

// Warp-aggregated add to a per-bucket counter; returns this thread's slot.
// Every lane of the warp calls it.
NCG_DEV uint32_t bucket_slot(uint32_t* ctr, int key, bool active) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned act = __ballot_sync(0xffffffffu, active);
    uint32_t slot = 0;
    if (active) {
        const unsigned peers = __match_any_sync(act, key);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&ctr[key], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        slot = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    }
    return slot;
}

// Body of the scatter kernel (one thread per pair, after bucket_n holds the
// bucket sizes): writes the pair indices into `sorted` bucket by bucket and
// the lengths of the analytic and ConvexHull lists.  The order inside a
// bucket is arbitrary: every pair's result depends on the pair alone.
NCG_DEV void scatter_by_bucket(uint64_t n_pairs, const uint8_t* bucket, const uint32_t* bucket_n,
                               uint32_t* bucket_fill, uint32_t* sorted, unsigned long long* n_analytic,
                               unsigned long long* n_hull) {
    __shared__ uint32_t base[NB];
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int k = 0; k < NB; ++k) {
            base[k] = acc;
            acc += bucket_n[k];
            if (k == NB_ANALYTIC - 1 && blockIdx.x == 0) *n_analytic = acc;
        }
        if (blockIdx.x == 0) *n_hull = acc - base[NB_ANALYTIC];
    }
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int key = i < n_pairs ? (int)bucket[i] : (int)NO_BUCKET;
    const bool active = key != NO_BUCKET;
    const uint32_t slot = bucket_slot(bucket_fill, active ? key : 0, active);
    if (active) sorted[base[key] + slot] = (uint32_t)i;
}

}  // namespace ncg
