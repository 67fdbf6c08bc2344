// ncg_toi.cu — batched linear time of impact: query::time_of_impact for the
// support-map shapes of this library (time_of_impact.rs:63-90), one thread per
// pair.  The arithmetic is in ncg_toi.cuh.  As in the GJK stage, the
// double-word sum, quotient and square root are kept out of line (the loop is
// bound by instruction fetch).
#define NCG_DW_OUTLINE 1

#include <cuda_runtime.h>

#include <cfloat>
#include <string>

#include "ncg_mlp.h"
#include "ncg_sort.cuh"
#include "ncg_toi.cuh"
#include "ncg_toi.h"

#ifndef NCG_TOI_MIN_BLOCKS
#define NCG_TOI_MIN_BLOCKS 4
#endif

namespace ncg {
namespace {

struct ToiArgs {
    const float* vel1;
    const float* vel2;
    dw_host max_toi;
    float target;
    int dispatch;
    int max_iter;
    ncg_toi* out;
    uint8_t* has;
    uint32_t* status;
    uint32_t* iters;
};

struct ToiCounters {
    uint32_t bucket_n[NB], bucket_fill[NB];
    unsigned long long n_analytic, n_hull;
    unsigned long long n_refine;  // pairs queued for toi_refine
};

// A pair queued for the closest-points refinement.
struct RefineItem {
    uint32_t pair, iters, status;
    float dir[3];
};
static_assert(sizeof(ToiCounters) <= 512, "TOI counters must fit their slot");

NCG_DEV void write_toi(const ToiArgs& a, uint64_t i, const ToiResult& r, uint32_t status, uint32_t iters) {
    ncg_toi& o = a.out[i];
    if (r.some) {
        o.toi = float(r.toi);
        o.witness1[0] = r.w1.x; o.witness1[1] = r.w1.y; o.witness1[2] = r.w1.z;
        o.witness2[0] = r.w2.x; o.witness2[1] = r.w2.y; o.witness2[2] = r.w2.z;
        o.normal1[0] = r.n1.x; o.normal1[1] = r.n1.y; o.normal1[2] = r.n1.z;
        o.normal2[0] = r.n2.x; o.normal2[1] = r.n2.y; o.normal2[2] = r.n2.z;
        o.status = (uint32_t)r.status;
    } else {
        o = ncg_toi{};
    }
    a.has[i] = r.some ? 1 : 0;
    a.status[i] = status;
    if (a.iters) a.iters[i] = iters;
}

// Validates every pair, writes the outputs of bad ones and counts the buckets.
__global__ void k_toi_classify(ncg_batch b, ToiArgs a, uint8_t* bucket, ToiCounters* ctr) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < b.n_pairs) {
        Shape s1, s2;
        if (load_shape(b, b.g1[i], s1) && load_shape(b, b.g2[i], s2)) {
            key = pair_bucket(s1, s2);
        } else {
            ToiResult r;
            r.some = false;
            write_toi(a, i, r, NCG_STATUS_BAD_INPUT, 0);
        }
        bucket[i] = key < 0 ? NO_BUCKET : (uint8_t)key;
    }
    (void)bucket_slot(ctr->bucket_n, key < 0 ? 0 : key, key >= 0);
}

__global__ void k_toi_bucket(ncg_batch b, const uint8_t* bucket, uint32_t* sorted, ToiCounters* ctr) {
    scatter_by_bucket(b.n_pairs, bucket, ctr->bucket_n, ctr->bucket_fill, sorted, &ctr->n_analytic, &ctr->n_hull);
}

// One thread per pair over the sorted pairs: the ConvexHull list first
// (largest hulls first), then the analytic list, so that the longest pairs
// start earliest.
__global__ void __launch_bounds__(128, NCG_TOI_MIN_BLOCKS)
k_toi(ncg_batch b, Tol tol, ToiArgs a, const uint32_t* sorted, ToiCounters* ctr, RefineItem* refine_items,
      unsigned long long* iter_sum) {
    const ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    const unsigned long long na = *(volatile const unsigned long long*)&ctr->n_analytic;
    const unsigned long long nh = *(volatile const unsigned long long*)&ctr->n_hull;
    const unsigned long long n = na + nh;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const uint32_t i = sorted[k < nh ? na + k : k - nh];
        uint32_t status = 0, iters = 0;
        ToiResult r;
        PairGeom g;
        load_shape(b, b.g1[i], g.g1);
        load_shape(b, b.g2[i], g.g2);
        g.m1 = load_pose(b.m1 + i);
        g.m2 = load_pose(b.m2 + i);
        const float* p = a.vel1 + 3 * (size_t)i;
        const float* q = a.vel2 + 3 * (size_t)i;
        const vec3<float> v1{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
        const vec3<float> v2{__ldg(q), __ldg(q + 1), __ldg(q + 2)};
        const real max_toi = from_host(a.max_toi);
        bool refine = false;
        vec3<float> rdir;
        if (a.dispatch == NCG_DISPATCH_QUERY && g.g1.kind == NCG_BALL && g.g2.kind == NCG_BALL)
            r = toi_ball_ball(g.m1, v1, g.g1.p0, g.m2, v2, g.g2.p0, max_toi, a.target);
        else
            r = toi_support_map(g, v1, v2, max_toi, a.target, tol, scan, iters, status, a.max_iter, refine, rdir);
        if (refine) {
            const unsigned long long slot = atomicAdd(&ctr->n_refine, 1ull);
            RefineItem& it = refine_items[slot];
            it.pair = i;
            it.iters = iters;
            it.status = status;
            it.dir[0] = rdir.x;
            it.dir[1] = rdir.y;
            it.dir[2] = rdir.z;
        } else {
            write_toi(a, i, r, status, iters);
        }
        acc += iters;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0 && acc) atomicAdd(iter_sum, acc);
}

// The closest-points refinement of the queued zero-toi pairs (dilated first
// shape), one thread per pair.
__global__ void __launch_bounds__(128, NCG_TOI_MIN_BLOCKS)
k_toi_refine(ncg_batch b, Tol tol, ToiArgs a, const ToiCounters* ctr, const RefineItem* items,
             unsigned long long* iter_sum) {
    const ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    const unsigned long long n = *(volatile const unsigned long long*)&ctr->n_refine;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const RefineItem it = items[k];
        const uint32_t i = it.pair;
        PairGeom g;
        load_shape(b, b.g1[i], g.g1);
        load_shape(b, b.g2[i], g.g2);
        g.m1 = load_pose(b.m1 + i);
        g.m2 = load_pose(b.m2 + i);
        uint32_t iters = it.iters, status = it.status;
        const ToiResult r = toi_refine(g, vec3<float>{it.dir[0], it.dir[1], it.dir[2]}, a.target, tol, scan, iters,
                                       status, a.max_iter);
        write_toi(a, i, r, status, iters);
        acc += iters - it.iters;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0 && acc) atomicAdd(iter_sum, acc);
}

struct RayArgs {
    const float* rays;  // origin[3], dir[3] per ray (world)
    dw_host max_toi;
    int solid;
    int max_iter;
    float* toi;
    float* normal;  // nullable
    uint8_t* hit;
    uint32_t* status;
    uint32_t* iters;  // nullable
};

NCG_DEV void write_ray(const RayArgs& a, uint64_t i, const RayResult& r, uint32_t status, uint32_t iters) {
    a.toi[i] = r.hit ? float(r.toi) : 0.0f;
    if (a.normal) {
        float* n = a.normal + 3 * i;
        n[0] = r.normal.x;
        n[1] = r.normal.y;
        n[2] = r.normal.z;
    }
    a.hit[i] = r.hit ? 1 : 0;
    a.status[i] = status;
    if (a.iters) a.iters[i] = iters;
}

// Validates every ray's shape, writes the outputs of bad ones and counts the
// buckets (the shape's kind, or its hull size).
__global__ void k_ray_classify(ncg_batch b, RayArgs a, uint8_t* bucket, ToiCounters* ctr) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < b.n_pairs) {
        Shape s1;
        if (load_shape(b, b.g1[i], s1)) {
            const Shape ball{NCG_BALL, 0, 0, 0.0f, 0.0f, 0.0f};
            key = pair_bucket(ball, s1);
        } else {
            RayResult r;
            r.hit = false;
            r.normal = zero3<float>();
            write_ray(a, i, r, NCG_STATUS_BAD_INPUT, 0);
        }
        bucket[i] = key < 0 ? NO_BUCKET : (uint8_t)key;
    }
    (void)bucket_slot(ctr->bucket_n, key < 0 ? 0 : key, key >= 0);
}

// One thread per ray over the sorted rays (ConvexHull shapes first).
__global__ void __launch_bounds__(128, NCG_TOI_MIN_BLOCKS)
k_ray(ncg_batch b, Tol tol, RayArgs a, const uint32_t* sorted, const ToiCounters* ctr, unsigned long long* iter_sum) {
    const ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    const unsigned long long na = *(volatile const unsigned long long*)&ctr->n_analytic;
    const unsigned long long nh = *(volatile const unsigned long long*)&ctr->n_hull;
    const unsigned long long n = na + nh;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const uint32_t i = sorted[k < nh ? na + k : k - nh];
        Shape s1;
        load_shape(b, b.g1[i], s1);
        const Pose m = load_pose(b.m1 + i);
        const float* r6 = a.rays + 6 * (size_t)i;
        const vec3<float> ro{__ldg(r6), __ldg(r6 + 1), __ldg(r6 + 2)};
        const vec3<float> rd{__ldg(r6 + 3), __ldg(r6 + 4), __ldg(r6 + 5)};
        uint32_t status = 0, iters = 0;
        const RayResult r = ray_cast_support_map(m, s1, ro, rd, from_host(a.max_toi), a.solid != 0, tol, scan, iters,
                                                 status, a.max_iter);
        write_ray(a, i, r, status, iters);
        acc += iters;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0 && acc) atomicAdd(iter_sum, acc);
}

}  // namespace

int toi_launch(const ncg_batch& b, const Tol& tol, int dispatch, const float* vel1, const float* vel2,
               float max_toi, float target_distance, ncg_toi* out, uint8_t* has_toi, uint32_t* status,
               uint32_t* iters, const ToiScratch& scratch, int num_sms, cudaStream_t st, uint32_t* launches) {
    ToiArgs a;
    a.vel1 = vel1;
    a.vel2 = vel2;
    a.max_toi = max_toi >= FLT_MAX ? dw_host{FLT_MAX, 0.0f} : dw_split((double)max_toi);
    a.target = target_distance;
    a.dispatch = dispatch;
    a.max_iter = 10000;
    a.out = out;
    a.has = has_toi;
    a.status = status;
    a.iters = iters;
    ToiCounters* ctr = static_cast<ToiCounters*>(scratch.ctr);
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(ToiCounters), st);
    if (e != cudaSuccess) {
        set_last_error(std::string("memset TOI counters: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    const unsigned blocks = (unsigned)((b.n_pairs + 255) / 256);
    k_toi_classify<<<blocks, 256, 0, st>>>(b, a, scratch.bucket, ctr);
    k_toi_bucket<<<blocks, 256, 0, st>>>(b, scratch.bucket, scratch.sorted, ctr);
    const uint64_t need = (b.n_pairs + 127) / 128;
    const uint64_t cap = (uint64_t)num_sms * NCG_TOI_MIN_BLOCKS;
    RefineItem* items = reinterpret_cast<RefineItem*>(scratch.refine);
    k_toi<<<(unsigned)(need < cap ? need : cap), 128, 0, st>>>(b, tol, a, scratch.sorted, ctr, items,
                                                               scratch.iter_sum);
    *launches += 3;
    if (target_distance != 0.0f) {
        k_toi_refine<<<(unsigned)cap, 128, 0, st>>>(b, tol, a, ctr, items, scratch.iter_sum);
        *launches += 1;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("TOI kernel launch: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    return NCG_OK;
}

int ray_launch(const ncg_batch& b, const Tol& tol, const float* rays, float max_toi, int solid, float* out_toi,
               float* out_normal, uint8_t* hit, uint32_t* status, uint32_t* iters, const ToiScratch& scratch,
               int num_sms, cudaStream_t st, uint32_t* launches) {
    RayArgs a;
    a.rays = rays;
    a.max_toi = max_toi >= FLT_MAX ? dw_host{FLT_MAX, 0.0f} : dw_split((double)max_toi);
    a.solid = solid;
    a.max_iter = 10000;
    a.toi = out_toi;
    a.normal = out_normal;
    a.hit = hit;
    a.status = status;
    a.iters = iters;
    ToiCounters* ctr = static_cast<ToiCounters*>(scratch.ctr);
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(ToiCounters), st);
    if (e != cudaSuccess) {
        set_last_error(std::string("memset ray counters: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    const unsigned blocks = (unsigned)((b.n_pairs + 255) / 256);
    k_ray_classify<<<blocks, 256, 0, st>>>(b, a, scratch.bucket, ctr);
    k_toi_bucket<<<blocks, 256, 0, st>>>(b, scratch.bucket, scratch.sorted, ctr);
    const uint64_t need = (b.n_pairs + 127) / 128;
    const uint64_t cap = (uint64_t)num_sms * NCG_TOI_MIN_BLOCKS;
    k_ray<<<(unsigned)(need < cap ? need : cap), 128, 0, st>>>(b, tol, a, scratch.sorted, ctr, scratch.iter_sum);
    *launches += 3;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("ray-cast kernel launch: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    return NCG_OK;
}

}  // namespace ncg
