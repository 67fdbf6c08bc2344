// ncg_bp.cu — bounding volumes and the broad phase on the GPU.
//
//   ncg_aabb_batch      HasBoundingVolume<AABB>::bounding_volume of every
//                       (pose, shape): Ball centre -+ r, Cuboid |R| h,
//                       Capsule/Cone/Cylinder support points along -+e_d,
//                       ConvexHull min/max of the transformed points.
//   ncg_bp_update       DBVTBroadPhase::update (dbvt_broad_phase.rs:174-258):
//                       stored boxes are replaced by new.loosened(margin) when
//                       they do not contain the new box; the pair set is every
//                       intersecting pair of stored boxes; started / stopped
//                       are the pairs that entered / left it.
//
// The reference keeps two dynamic AABB trees and re-inserts moved leaves one
// by one.  On the GPU the tree is rebuilt for every update instead: a linear
// BVH over the valid boxes (Karras, "Maximizing parallelism in the
// construction of BVHs, octrees, and k-d trees", HPG 2012: Morton codes of the
// box centres, a stable LSD radix sort, the radix tree from longest common
// prefixes, a bottom-up refit), then one thread per leaf walks the tree with
// its box and reports the leaves after it that its box intersects.  The pair
// set equals the reference's (both are exactly the intersecting pairs of the
// stored boxes; box tests are comparisons, so no rounding enters); pairs and
// events are returned sorted by (lower id, higher id).
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <string>

#include "../../include/ncg.h"
#include "ncg_core.cuh"
#include "ncg_mlp.h"
#include "ncg_bp.h"

namespace ncg {
namespace {

// ------------------------------------------------------------------ AABBs
// UnitQuaternion::to_rotation_matrix (nalgebra), row-major.
NCG_DEV void rotation_matrix(float4 q, float r[3][3]) {
    const float i = q.x, j = q.y, k = q.z, w = q.w;
    const float ww = w * w, ii = i * i, jj = j * j, kk = k * k;
    const float ij = i * j * 2.0f, wk = w * k * 2.0f, wj = w * j * 2.0f, ik = i * k * 2.0f, jk = j * k * 2.0f,
                wi = w * i * 2.0f;
    r[0][0] = ww + ii - jj - kk; r[0][1] = ij - wk;           r[0][2] = wj + ik;
    r[1][0] = wk + ij;           r[1][1] = ww - ii + jj - kk; r[1][2] = jk - wi;
    r[2][0] = ik - wj;           r[2][1] = wi + jk;           r[2][2] = ww - ii - jj + kk;
}

__global__ void k_aabb(ncg_batch b, float* out, uint32_t* status) {
    const ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_pairs; i += stride) {
        Shape s;
        float mn[3], mx[3];
        uint32_t st = 0;
        if (!load_shape(b, b.g1[i], s)) {
            for (int d = 0; d < 3; ++d) mn[d] = mx[d] = __int_as_float(0x7fc00000);
            st = NCG_STATUS_BAD_INPUT;
        } else {
            const Pose m = load_pose(b.m1 + i);
            const float t[3] = {m.t.x, m.t.y, m.t.z};
            if (s.kind == NCG_BALL) {
                for (int d = 0; d < 3; ++d) {
                    mn[d] = t[d] + -s.p0;
                    mx[d] = t[d] + s.p0;
                }
            } else if (s.kind == NCG_CUBOID) {
                float r[3][3];
                rotation_matrix(m.q, r);
                const float h[3] = {s.p0, s.p1, s.p2};
                for (int d = 0; d < 3; ++d) {
                    const float he = (fabsf(r[d][0]) * h[0] + fabsf(r[d][1]) * h[1]) + fabsf(r[d][2]) * h[2];
                    mn[d] = t[d] - he;
                    mx[d] = t[d] + he;
                }
            } else if (s.kind == NCG_CONVEX_HULL) {
                const float4* p = scan.pts + s.off;
                for (uint32_t k = 0; k < s.n; ++k) {
                    const float4 v = __ldg(p + k);
                    const vec3<float> w = qrot(m.q, vec3<float>{v.x, v.y, v.z}) + m.t;
                    const float c[3] = {w.x, w.y, w.z};
                    for (int d = 0; d < 3; ++d) {
                        if (k == 0 || c[d] < mn[d]) mn[d] = c[d];
                        if (k == 0 || c[d] > mx[d]) mx[d] = c[d];
                    }
                }
            } else {
                for (int d = 0; d < 3; ++d) {
                    vec3<float> e{d == 0 ? 1.0f : 0.0f, d == 1 ? 1.0f : 0.0f, d == 2 ? 1.0f : 0.0f};
                    const vec3<float> hi = support_point(m, s, e, scan);
                    e = vec3<float>{d == 0 ? -1.0f : 0.0f, d == 1 ? -1.0f : 0.0f, d == 2 ? -1.0f : 0.0f};
                    const vec3<float> lo = support_point(m, s, e, scan);
                    mx[d] = d == 0 ? hi.x : (d == 1 ? hi.y : hi.z);
                    mn[d] = d == 0 ? lo.x : (d == 1 ? lo.y : lo.z);
                }
            }
        }
        float* o = out + 6 * i;
        o[0] = mn[0]; o[1] = mn[1]; o[2] = mn[2];
        o[3] = mx[0]; o[4] = mx[1]; o[5] = mx[2];
        if (status) status[i] = st;
    }
}

// ------------------------------------------------------------------ scan
constexpr int SCAN_BLOCK = 1024;

// Exclusive scan of each 1024-element block; block totals to sums.
__global__ void k_scan_block(const uint32_t* in, uint32_t* out, uint32_t* sums, uint32_t n) {
    __shared__ uint32_t warp_tot[32];
    const uint32_t i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (unsigned)o) t += y;
        }
        warp_tot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = w > 0 ? warp_tot[w - 1] : 0u;
    if (i < n) out[i] = before + x - v;
    if (threadIdx.x == SCAN_BLOCK - 1 && sums) sums[blockIdx.x] = warp_tot[31];
}

__global__ void k_scan_add(uint32_t* out, const uint32_t* offsets, uint32_t n) {
    const uint32_t i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += offsets[blockIdx.x];
}

// Exclusive scan of n <= 2^30 values (in and out may alias); tmp holds
// 2 * ceil(n / 1024) + 2 * ceil(n / 2^20) + 2 words.
void exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, cudaStream_t st) {
    if (n == 0) return;
    const uint32_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    if (nb == 1) {
        k_scan_block<<<1, SCAN_BLOCK, 0, st>>>(in, out, nullptr, n);
        return;
    }
    uint32_t* sums = tmp;
    uint32_t* sums_scanned = tmp + nb;
    k_scan_block<<<nb, SCAN_BLOCK, 0, st>>>(in, out, sums, n);
    exclusive_scan(sums, sums_scanned, nb, tmp + 2 * nb, st);
    k_scan_add<<<nb, SCAN_BLOCK, 0, st>>>(out, sums_scanned, n);
}

// ------------------------------------------------------------------ radix sort
// Stable LSD radix sort of (key, value) pairs by 8-bit digits.
constexpr int RS_THREADS = 256, RS_ITEMS = 8, RS_TILE = RS_THREADS * RS_ITEMS;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t* hist,
                                                        uint32_t n_tiles) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        const uint32_t i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Scatters one tile in index order: within a round of 256 keys a key's rank is
// its lane's rank among equal digits of its warp plus the counts of the warps
// before it; rounds follow each other, so equal digits keep their order.
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t* keys, const uint32_t* vals,
                                                           uint32_t* keys_out, uint32_t* vals_out, uint32_t n,
                                                           int shift, const uint32_t* offs, uint32_t n_tiles) {
    __shared__ uint32_t warp_cnt[RS_THREADS / 32][256];
    __shared__ uint32_t running[256];
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    running[threadIdx.x] = offs[threadIdx.x * n_tiles + blockIdx.x];
    const uint32_t base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        for (int k = 0; k < RS_THREADS / 32; ++k) warp_cnt[k][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t i = base + r * RS_THREADS + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys[i] : 0u;
        const uint32_t d = valid ? (key >> shift) & 255u : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) warp_cnt[w][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = running[d] + rank;
            for (unsigned k = 0; k < w; ++k) pos += warp_cnt[k][d];
            keys_out[pos] = key;
            vals_out[pos] = vals[i];
        }
        __syncthreads();
        uint32_t tot = 0;
        for (int k = 0; k < RS_THREADS / 32; ++k) tot += warp_cnt[k][threadIdx.x];
        running[threadIdx.x] += tot;
        __syncthreads();
    }
}

// Sorts n (key, value) pairs by the low `bits` bits of the keys; the result
// is in (keys, vals).  tmp: see RadixTmp.
struct RadixTmp {
    uint32_t* keys2;
    uint32_t* vals2;
    uint32_t* hist;      // 256 * ceil(n / RS_TILE)
    uint32_t* scan_tmp;  // exclusive_scan's tmp for 256 * ceil(n / RS_TILE) values
};
void radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, const RadixTmp& t, cudaStream_t st) {
    if (n <= 1) return;
    const uint32_t n_tiles = (n + RS_TILE - 1) / RS_TILE;
    uint32_t *ka = keys, *va = vals, *kb = t.keys2, *vb = t.vals2;
    int passes = (bits + 7) / 8;
    if (passes & 1) passes += 1;  // an even number of passes leaves the result in (keys, vals)
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_rs_hist<<<n_tiles, RS_THREADS, 0, st>>>(ka, n, shift, t.hist, n_tiles);
        exclusive_scan(t.hist, t.hist, 256 * n_tiles, t.scan_tmp, st);
        k_rs_scatter<<<n_tiles, RS_THREADS, 0, st>>>(ka, va, kb, vb, n, shift, t.hist, n_tiles);
        uint32_t* x = ka; ka = kb; kb = x;
        x = va; va = vb; vb = x;
    }
}

// ------------------------------------------------------------------ LBVH
struct Box {
    float mn[3], mx[3];
};
NCG_DEV Box load_box(const float* b6) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.mn[d] = b6[d];
        b.mx[d] = b6[3 + d];
    }
    return b;
}
NCG_DEV bool overlap(const Box& a, const Box& b) {
    return a.mn[0] <= b.mx[0] && a.mx[0] >= b.mn[0] && a.mn[1] <= b.mx[1] && a.mx[1] >= b.mn[1] &&
           a.mn[2] <= b.mx[2] && a.mx[2] >= b.mn[2];
}

struct BpCounters {
    uint32_t bounds[6];  // order-preserving uint encodings: min centre xyz, max centre xyz
    uint32_t n_valid;
    uint32_t overflow;   // 1: a traversal stack ran out (depth <= 62: not expected); 2: malformed tree
    unsigned long long n_pairs, n_started, n_stopped;
};

NCG_DEV uint32_t f2u(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
NCG_DEV float u2f(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

// Stored-box update: replaced by new.loosened(margin) unless it contains the
// new box (the first update stores every box).  Marks valid boxes (no NaN).
__global__ void k_bp_store(const float* boxes, float* stored, uint32_t n, uint32_t n_old, float margin,
                           uint32_t* valid, BpCounters* ctr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Box nb = load_box(boxes + 6 * (size_t)i);
    Box s = i < n_old ? load_box(stored + 6 * (size_t)i) : Box{};
    bool contains = i < n_old;
    for (int d = 0; d < 3 && contains; ++d) contains = s.mn[d] <= nb.mn[d] && s.mx[d] >= nb.mx[d];
    if (!contains) {
        for (int d = 0; d < 3; ++d) {
            s.mn[d] = nb.mn[d] + -margin;
            s.mx[d] = nb.mx[d] + margin;
        }
        float* o = stored + 6 * (size_t)i;
        for (int d = 0; d < 3; ++d) {
            o[d] = s.mn[d];
            o[3 + d] = s.mx[d];
        }
    }
    bool ok = true;
    for (int d = 0; d < 3; ++d) ok = ok && s.mn[d] == s.mn[d] && s.mx[d] == s.mx[d];
    valid[i] = ok ? 1u : 0u;
    if (ok) {
        for (int d = 0; d < 3; ++d) {
            const float c = 0.5f * s.mn[d] + 0.5f * s.mx[d];
            atomicMin(&ctr->bounds[d], f2u(c));
            atomicMax(&ctr->bounds[3 + d], f2u(c));
        }
    }
}

// Compacts the valid boxes (ids, boxes) and computes their 30-bit Morton codes.
__global__ void k_bp_morton(const float* stored, const uint32_t* valid, const uint32_t* pos, uint32_t n,
                            const BpCounters* ctr, uint32_t* codes, uint32_t* ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !valid[i]) return;
    const Box s = load_box(stored + 6 * (size_t)i);
    uint32_t code = 0;
    for (int d = 0; d < 3; ++d) {
        const float lo = u2f(ctr->bounds[d]), hi = u2f(ctr->bounds[3 + d]);
        const float c = 0.5f * s.mn[d] + 0.5f * s.mx[d];
        const float ext = hi - lo;
        float u = ext > 0.0f ? (c - lo) / ext : 0.0f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        uint32_t q = (uint32_t)(u * 1023.0f);
        // spread 10 bits to every third bit
        q = (q | (q << 16)) & 0x030000FFu;
        q = (q | (q << 8)) & 0x0300F00Fu;
        q = (q | (q << 4)) & 0x030C30C3u;
        q = (q | (q << 2)) & 0x09249249u;
        code |= q << (2 - d);
    }
    const uint32_t k = pos[i];
    codes[k] = code;
    ids[k] = i;
}

// Node layout: internal nodes 0 .. m-2, leaves m-1 .. 2m-2 (leaf k = sorted
// position k).  child[2 * node] / child[2 * node + 1]; parent per node; the
// last leaf (sorted position) each internal node covers; boxes per node.
struct Tree {
    uint32_t* child;
    uint32_t* parent;
    uint32_t* last;
    float* box;  // 6 floats per node
    uint32_t* flag;
};

NCG_DEV int lcp(const uint32_t* codes, uint32_t m, int i, int j) {
    if (j < 0 || j >= (int)m) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Karras 2012, Figure 4: the range and the split of internal node i.
__global__ void k_bp_build(const uint32_t* codes, uint32_t m, Tree t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)m - 1) return;
    const int d = (lcp(codes, m, i, i + 1) - lcp(codes, m, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = lcp(codes, m, i, i - d);
    int lmax = 2;
    while (lcp(codes, m, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int s = lmax >> 1; s >= 1; s >>= 1)
        if (lcp(codes, m, i, i + (l + s) * d) > dmin) l += s;
    const int j = i + l * d;
    const int dnode = lcp(codes, m, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        const int step = (l + div - 1) / div;
        if (lcp(codes, m, i, i + (s + step) * d) > dnode) s += step;
        if (step <= 1) break;
    }
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    const uint32_t left = (lo == gamma) ? (m - 1 + gamma) : (uint32_t)gamma;
    const uint32_t right = (hi == gamma + 1) ? (m - 1 + gamma + 1) : (uint32_t)(gamma + 1);
    t.child[2 * i] = left;
    t.child[2 * i + 1] = right;
    t.parent[left] = i;
    t.parent[right] = i;
    t.last[i] = hi;
}

// Leaves' boxes, then the bottom-up refit: the second child to arrive at a
// node writes the node's box (the union of its children's) and goes on.
__global__ void k_bp_refit(const float* stored, const uint32_t* ids, uint32_t m, Tree t) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const uint32_t leaf = m - 1 + k;
    const float* src = stored + 6 * (size_t)ids[k];
    float* dst = t.box + 6 * (size_t)leaf;
    for (int c = 0; c < 6; ++c) dst[c] = src[c];
    if (m == 1) return;
    uint32_t node = t.parent[leaf];
    for (int depth = 0; depth < 64; ++depth) {
        __threadfence();
        if (atomicAdd(&t.flag[node], 1u) == 0u) return;  // the other child is not done yet
        __threadfence();
        const float* a = t.box + 6 * (size_t)t.child[2 * node];
        const float* b = t.box + 6 * (size_t)t.child[2 * node + 1];
        float* o = t.box + 6 * (size_t)node;
        for (int c = 0; c < 3; ++c) {
            const float x = __ldcg(a + c), y = __ldcg(b + c);
            o[c] = x < y ? x : y;
            const float u = __ldcg(a + 3 + c), v = __ldcg(b + 3 + c);
            o[3 + c] = u > v ? u : v;
        }
        if (node == 0) return;
        node = t.parent[node];
    }
}

// One thread per leaf k: every leaf after k (sorted position) whose box the
// leaf's box intersects, appended as (lower id, higher id).
__global__ void __launch_bounds__(128) k_bp_traverse(const uint32_t* ids, uint32_t m, Tree t, uint2* pairs,
                                                     unsigned long long cap, BpCounters* ctr) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m || m < 2) return;
    const Box q = load_box(t.box + 6 * (size_t)(m - 1 + k));
    const uint32_t qid = ids[k];
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = 0;
    // a tree of m leaves has m - 1 internal nodes: more pops mean a malformed tree
    for (uint32_t pops = 0; sp > 0; ++pops) {
        if (pops >= m) {
            atomicOr(&ctr->overflow, 2u);
            break;
        }
        const uint32_t node = stack[--sp];
        for (int c = 0; c < 2; ++c) {
            const uint32_t ch = t.child[2 * node + c];
            if (ch >= m - 1) {
                const uint32_t kk = ch - (m - 1);
                if (kk <= k) continue;
                if (!overlap(q, load_box(t.box + 6 * (size_t)ch))) continue;
                const uint32_t oid = ids[kk];
                const unsigned long long slot = atomicAdd(&ctr->n_pairs, 1ull);
                if (slot < cap) pairs[slot] = make_uint2(qid < oid ? qid : oid, qid < oid ? oid : qid);
            } else {
                if (t.last[ch] <= k) continue;
                if (!overlap(q, load_box(t.box + 6 * (size_t)ch))) continue;
                if (sp < 64) stack[sp++] = ch;
                else atomicOr(&ctr->overflow, 1u);
            }
        }
    }
}

__global__ void k_split(const uint2* pairs, uint32_t n, uint32_t* lo, uint32_t* hi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lo[i] = pairs[i].x;
    hi[i] = pairs[i].y;
}
__global__ void k_join(const uint32_t* lo, const uint32_t* hi, uint32_t n, uint2* pairs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pairs[i] = make_uint2(lo[i], hi[i]);
}

NCG_DEV bool pair_less(uint2 a, uint2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
NCG_DEV bool contains_pair(const uint2* set, uint32_t n, uint2 p) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pair_less(set[mid], p)) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && set[lo].x == p.x && set[lo].y == p.y;
}
// flag[i] = 1 when a[i] is not in b.
__global__ void k_not_in(const uint2* a, uint32_t na, const uint2* b, uint32_t nb, uint32_t* flag) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= na) return;
    flag[i] = contains_pair(b, nb, a[i]) ? 0u : 1u;
}
__global__ void k_compact(const uint2* a, uint32_t na, const uint32_t* flag, const uint32_t* pos, uint2* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= na || !flag[i]) return;
    out[pos[i]] = a[i];
}

// Narrow-phase batch of the broad phase's pairs: pair k = (proxy a, proxy b).
__global__ void k_gather_pairs(const ncg_pose* poses, const uint32_t* shape_ids, const uint2* pairs, uint64_t n,
                               ncg_pose* m1, uint32_t* g1, ncg_pose* m2, uint32_t* g2) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const uint2 p = pairs[k];
        const float4* a = reinterpret_cast<const float4*>(poses + p.x);
        const float4* b = reinterpret_cast<const float4*>(poses + p.y);
        float4* o1 = reinterpret_cast<float4*>(m1 + k);
        float4* o2 = reinterpret_cast<float4*>(m2 + k);
        o1[0] = __ldg(a);
        o1[1] = __ldg(a + 1);
        o2[0] = __ldg(b);
        o2[1] = __ldg(b + 1);
        g1[k] = __ldg(shape_ids + p.x);
        g2[k] = __ldg(shape_ids + p.y);
    }
}

}  // namespace

// ------------------------------------------------------------------ host side
int gather_launch(const ncg_pose* poses, const uint32_t* shape_ids, const uint32_t* pairs, uint64_t n, ncg_pose* m1,
                  uint32_t* g1, ncg_pose* m2, uint32_t* g2, int num_sms, cudaStream_t st) {
    if (n == 0) return NCG_OK;
    const uint64_t need = (n + 255) / 256;
    const uint64_t cap = (uint64_t)num_sms * 8;
    k_gather_pairs<<<(unsigned)(need < cap ? need : cap), 256, 0, st>>>(
        poses, shape_ids, reinterpret_cast<const uint2*>(pairs), n, m1, g1, m2, g2);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("k_gather_pairs launch: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    return NCG_OK;
}

int aabb_launch(const ncg_batch& b, float* out, uint32_t* status, int num_sms, cudaStream_t st) {
    const uint64_t need = (b.n_pairs + 127) / 128;
    const uint64_t cap = (uint64_t)num_sms * 16;
    k_aabb<<<(unsigned)(need < cap ? need : cap), 128, 0, st>>>(b, out, status);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("k_aabb launch: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    return NCG_OK;
}

namespace {
bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}
template <class T> bool grow(T*& p, size_t& cap, size_t need, const char* what) {
    if (need <= cap && p) return true;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t c = need < 1024 ? 1024 : need + need / 4;
    if (!ok(cudaMalloc(&p, c * sizeof(T)), what)) return false;
    cap = c;
    return true;
}
}  // namespace

struct BroadPhaseState {
    int device = 0;
    float margin = 0.0f;
    uint32_t n = 0;  // proxies stored
    float* stored = nullptr;
    size_t stored_cap = 0;
    // per-proxy work arrays
    uint32_t *valid = nullptr, *pos = nullptr, *codes = nullptr, *ids = nullptr, *codes2 = nullptr, *ids2 = nullptr;
    size_t proxy_cap = 0;
    uint32_t* tmp = nullptr;  // histograms and scan scratch
    size_t tmp_cap = 0;
    // tree
    uint32_t *child = nullptr, *parent = nullptr, *last = nullptr, *flag = nullptr;
    float* box = nullptr;
    size_t node_cap = 0;
    // pairs: current, previous, events, sort buffers
    uint2 *pairs = nullptr, *prev = nullptr, *started = nullptr, *stopped = nullptr;
    size_t pairs_cap = 0, prev_cap = 0, started_cap = 0, stopped_cap = 0;
    uint32_t *plo = nullptr, *phi = nullptr, *plo2 = nullptr, *phi2 = nullptr, *pflag = nullptr, *ppos = nullptr;
    size_t pwork_cap = 0;
    uint64_t n_pairs = 0, n_prev = 0, n_started = 0, n_stopped = 0;
    BpCounters* ctr = nullptr;
    BpCounters* host_ctr = nullptr;
};

namespace {
size_t scan_tmp_words(size_t n) {
    size_t w = 2;
    while (n > 1) {
        const size_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
        w += 2 * nb;
        n = nb;
    }
    return w;
}
size_t radix_tmp_words(size_t n) {
    const size_t tiles = (n + RS_TILE - 1) / RS_TILE;
    return 256 * tiles + scan_tmp_words(256 * tiles);
}
}  // namespace

int bp_create(float margin, int device, BroadPhaseState** out) {
    BroadPhaseState* s = new BroadPhaseState();
    s->device = device;
    s->margin = margin;
    if (!ok(cudaMalloc(&s->ctr, sizeof(BpCounters)), "cudaMalloc(bp counters)") ||
        !ok(cudaMallocHost(&s->host_ctr, sizeof(BpCounters)), "cudaMallocHost(bp counters)")) {
        bp_destroy(s);
        return NCG_ENOMEM;
    }
    *out = s;
    return NCG_OK;
}

void bp_destroy(BroadPhaseState* s) {
    if (!s) return;
    void* dev[] = {s->stored, s->valid, s->pos, s->codes, s->ids, s->codes2, s->ids2, s->tmp, s->child, s->parent,
                   s->last, s->flag, s->box, s->pairs, s->prev, s->started, s->stopped, s->plo, s->phi, s->plo2,
                   s->phi2, s->pflag, s->ppos, s->ctr};
    for (void* p : dev)
        if (p) cudaFree(p);
    if (s->host_ctr) cudaFreeHost(s->host_ctr);
    delete s;
}

int bp_update(BroadPhaseState* s, const float* boxes, uint32_t n, cudaStream_t st) {
    if (n < s->n) {
        set_last_error("ncg_bp_update: the proxy count cannot shrink (give removed proxies NaN boxes)");
        return NCG_EINVAL;
    }
    if (!ok(cudaSetDevice(s->device), "cudaSetDevice")) return NCG_ECUDA;
    // buffers sized by the proxy count
    if (!grow(s->stored, s->stored_cap, 6 * (size_t)n, "cudaMalloc(bp stored)")) return NCG_ENOMEM;
    if (s->proxy_cap < n) {
        uint32_t** arrs[] = {&s->valid, &s->pos, &s->codes, &s->ids, &s->codes2, &s->ids2};
        size_t c = 0;
        for (uint32_t** a : arrs) {
            c = s->proxy_cap;
            if (!grow(*a, c, n, "cudaMalloc(bp proxies)")) return NCG_ENOMEM;
        }
        s->proxy_cap = c;
        if (!grow(s->box, s->node_cap, 6 * (2 * (size_t)n), "cudaMalloc(bp tree boxes)")) return NCG_ENOMEM;
        uint32_t** tr[] = {&s->child, &s->parent, &s->last, &s->flag};
        for (uint32_t** a : tr) {
            size_t cc = 0;
            if (*a) cudaFree(*a);
            *a = nullptr;
            if (!grow(*a, cc, 2 * (size_t)n + 2, "cudaMalloc(bp tree)")) return NCG_ENOMEM;
        }
    }
    const size_t need_tmp = radix_tmp_words(n) + scan_tmp_words(n) + 16;
    if (!grow(s->tmp, s->tmp_cap, need_tmp, "cudaMalloc(bp scratch)")) return NCG_ENOMEM;

    // stored boxes, validity, centre bounds
    BpCounters init{};
    for (int d = 0; d < 3; ++d) {
        init.bounds[d] = 0xffffffffu;
        init.bounds[3 + d] = 0u;
    }
    if (!ok(cudaMemcpyAsync(s->ctr, &init, sizeof(BpCounters), cudaMemcpyHostToDevice, st), "bp counters")) return NCG_ECUDA;
    const unsigned blocks = (n + 255) / 256;
    if (n > 0) k_bp_store<<<blocks, 256, 0, st>>>(boxes, s->stored, n, s->n, s->margin, s->valid, s->ctr);
    s->n = n;
    // compaction of the valid boxes and Morton codes
    exclusive_scan(s->valid, s->pos, n, s->tmp, st);
    if (n > 0) k_bp_morton<<<blocks, 256, 0, st>>>(s->stored, s->valid, s->pos, n, s->ctr, s->codes, s->ids);
    // the number of valid boxes: last position + last flag
    uint32_t m = 0;
    if (n > 0) {
        uint32_t lastpos = 0, lastvalid = 0;
        if (!ok(cudaMemcpyAsync(&lastpos, s->pos + n - 1, 4, cudaMemcpyDeviceToHost, st), "bp count") ||
            !ok(cudaMemcpyAsync(&lastvalid, s->valid + n - 1, 4, cudaMemcpyDeviceToHost, st), "bp count") ||
            !ok(cudaStreamSynchronize(st), "bp sync"))
            return NCG_ECUDA;
        m = lastpos + lastvalid;
    }
    // sort by Morton code, build, refit
    RadixTmp rt{s->codes2, s->ids2, s->tmp, s->tmp + 256 * ((m + RS_TILE - 1) / RS_TILE)};
    radix_sort(s->codes, s->ids, m, 30, rt, st);
    Tree t{s->child, s->parent, s->last, s->box, s->flag};
    if (m > 1) {
        if (!ok(cudaMemsetAsync(s->flag, 0, 4 * (size_t)m, st), "bp flags")) return NCG_ECUDA;
        k_bp_build<<<(m - 1 + 255) / 256, 256, 0, st>>>(s->codes, m, t);
    }
    if (m > 0) k_bp_refit<<<(m + 255) / 256, 256, 0, st>>>(s->stored, s->ids, m, t);
    // traversal; rerun with a larger buffer when the pairs did not fit
    // previous pairs are kept for the events
    uint2* x = s->prev; s->prev = s->pairs; s->pairs = x;
    size_t xc = s->prev_cap; s->prev_cap = s->pairs_cap; s->pairs_cap = xc;
    s->n_prev = s->n_pairs;
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (!grow(s->pairs, s->pairs_cap, s->pairs_cap > 0 ? s->pairs_cap : 4 * (size_t)n + 1024,
                  "cudaMalloc(bp pairs)"))
            return NCG_ENOMEM;
        if (!ok(cudaMemsetAsync(&s->ctr->n_pairs, 0, 8, st), "bp pair count")) return NCG_ECUDA;
        if (m > 1)
            k_bp_traverse<<<(m + 127) / 128, 128, 0, st>>>(s->ids, m, t, s->pairs, s->pairs_cap, s->ctr);
        if (!ok(cudaMemcpyAsync(s->host_ctr, s->ctr, sizeof(BpCounters), cudaMemcpyDeviceToHost, st), "bp counters") ||
            !ok(cudaStreamSynchronize(st), "bp sync"))
            return NCG_ECUDA;
        if (s->host_ctr->n_pairs <= s->pairs_cap) break;
        const size_t need = s->host_ctr->n_pairs;
        cudaFree(s->pairs);
        s->pairs = nullptr;
        s->pairs_cap = 0;
        if (!grow(s->pairs, s->pairs_cap, need, "cudaMalloc(bp pairs)")) return NCG_ENOMEM;
    }
    if (s->host_ctr->overflow) {
        set_last_error("ncg_bp_update: tree traversal out of bounds");
        return NCG_ECUDA;
    }
    const uint64_t np = s->host_ctr->n_pairs;
    if (np > 0xffffffffull / 2) {
        set_last_error("ncg_bp_update: more than 2^31 pairs");
        return NCG_EINVAL;
    }
    s->n_pairs = np;
    // canonical order: stable sort by the higher id, then by the lower id
    const uint32_t npi = (uint32_t)np;
    const size_t nwork = np > s->n_prev ? np : s->n_prev;
    if (s->pwork_cap < nwork) {
        uint32_t** arrs[] = {&s->plo, &s->phi, &s->plo2, &s->phi2, &s->pflag, &s->ppos};
        size_t c = 0;
        for (uint32_t** a : arrs) {
            c = s->pwork_cap;
            if (!grow(*a, c, nwork, "cudaMalloc(bp pair work)")) return NCG_ENOMEM;
        }
        s->pwork_cap = c;
    }
    const size_t need_tmp2 = radix_tmp_words(nwork) + scan_tmp_words(nwork) + 16;
    if (!grow(s->tmp, s->tmp_cap, need_tmp2, "cudaMalloc(bp scratch)")) return NCG_ENOMEM;
    int id_bits = 1;
    while (id_bits < 32 && (1ull << id_bits) < n) ++id_bits;
    if (npi > 0) {
        const unsigned pb = (npi + 255) / 256;
        k_split<<<pb, 256, 0, st>>>(s->pairs, npi, s->plo, s->phi);
        RadixTmp r1{s->plo2, s->phi2, s->tmp, s->tmp + 256 * ((npi + RS_TILE - 1) / RS_TILE)};
        radix_sort(s->phi, s->plo, npi, id_bits, r1, st);   // by higher id
        radix_sort(s->plo, s->phi, npi, id_bits, r1, st);   // then stably by lower id
        k_join<<<pb, 256, 0, st>>>(s->plo, s->phi, npi, s->pairs);
    }
    // events: started = pairs not in prev, stopped = prev not in pairs
    const uint32_t npv = (uint32_t)s->n_prev;
    if (!grow(s->started, s->started_cap, np + 1, "cudaMalloc(bp started)") ||
        !grow(s->stopped, s->stopped_cap, (size_t)npv + 1, "cudaMalloc(bp stopped)"))
        return NCG_ENOMEM;
    uint32_t counts[4] = {0, 0, 0, 0};
    if (npi > 0) {
        const unsigned pb = (npi + 255) / 256;
        k_not_in<<<pb, 256, 0, st>>>(s->pairs, npi, s->prev, npv, s->pflag);
        exclusive_scan(s->pflag, s->ppos, npi, s->tmp, st);
        k_compact<<<pb, 256, 0, st>>>(s->pairs, npi, s->pflag, s->ppos, s->started);
        cudaMemcpyAsync(&counts[0], s->ppos + npi - 1, 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&counts[1], s->pflag + npi - 1, 4, cudaMemcpyDeviceToHost, st);
        if (!ok(cudaStreamSynchronize(st), "bp sync")) return NCG_ECUDA;
    }
    if (npv > 0) {
        const unsigned pb = (npv + 255) / 256;
        k_not_in<<<pb, 256, 0, st>>>(s->prev, npv, s->pairs, npi, s->pflag);
        exclusive_scan(s->pflag, s->ppos, npv, s->tmp, st);
        k_compact<<<pb, 256, 0, st>>>(s->prev, npv, s->pflag, s->ppos, s->stopped);
        cudaMemcpyAsync(&counts[2], s->ppos + npv - 1, 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&counts[3], s->pflag + npv - 1, 4, cudaMemcpyDeviceToHost, st);
    }
    if (!ok(cudaGetLastError(), "bp kernels") || !ok(cudaStreamSynchronize(st), "bp sync")) return NCG_ECUDA;
    s->n_started = npi > 0 ? counts[0] + counts[1] : 0;
    s->n_stopped = npv > 0 ? counts[2] + counts[3] : 0;
    return NCG_OK;
}

void bp_results(const BroadPhaseState* s, uint64_t* n_pairs, uint64_t* n_started, uint64_t* n_stopped,
                const uint32_t** pairs, const uint32_t** started, const uint32_t** stopped) {
    if (n_pairs) *n_pairs = s->n_pairs;
    if (n_started) *n_started = s->n_started;
    if (n_stopped) *n_stopped = s->n_stopped;
    if (pairs) *pairs = reinterpret_cast<const uint32_t*>(s->pairs);
    if (started) *started = reinterpret_cast<const uint32_t*>(s->started);
    if (stopped) *stopped = reinterpret_cast<const uint32_t*>(s->stopped);
}

}  // namespace ncg
