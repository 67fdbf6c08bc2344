// ncg_mlp.cu — the learned warm start: a small MLP that predicts GJK's first
// search direction (and the sign of the separation) from a pair's relative
// pose and two shape descriptors, with its inference and training kernels on
// the tensor cores (tcgen05, bf16 operands, f32 accumulators in TMEM).
//
// Network: x (39 features, padded to 48) -> 128 (GELU) -> 128 (GELU) -> 4
// (direction xyz in the first shape's frame, separation logit).  Parameters
// are kept in f32 (the optimiser's master copy) and rounded to bf16 when a
// CTA stages them in shared memory; every product accumulates in f32.
//
// The network only picks the init_dir of contact_support_map_support_map_with_params
// (src/query/contact/contact_support_map_support_map.rs:38-57); GJK and EPA
// then run to their own termination, so a prediction can change the
// iteration count, never the kind of answer.  A prediction that is not a
// finite non-zero vector is replaced by the reference's default direction.
//
// Features of a pair (A = first shape, B = second):
//   0-2   R_A^T (t_B - t_A) / (r_A + r_B)      (r = circumradius)
//   3-6   q_A^-1 q_B, sign chosen so that w >= 0
//   7-22  descriptor of A, 23-38 descriptor of B:
//         one-hot kind (6), extents (3: the shape's parameters, or a hull's
//         local AABB half-extents), square roots of the hull's point
//         covariance eigenvalues (3, descending), log2(points) / 10,
//         circumradius, 0, 0
//   39-47 zero
//
// Kernels: k_shape_desc (one warp per shape), k_mlp_infer (features ->
// three layers -> world-space unit direction, persistent over 128-pair
// tiles), k_mlp_train_tile (forward, loss, backward and per-tile parameter
// gradients of one 128-sample tile), k_mlp_reduce (sums the tile gradients in
// a fixed order) and k_mlp_adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/ncg.h"
#include "ncg_core.cuh"
#include "ncg_mlp.h"
#include "ncg_tc.cuh"

namespace ncg {
namespace mlp {

constexpr int NF = 39, K1 = 48, HID = 128, NO = 4, N3 = 16, TILE = 128, DESC = 16;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + HID * K1;
constexpr int OFF_W2 = OFF_B1 + HID;
constexpr int OFF_B2 = OFF_W2 + HID * HID;
constexpr int OFF_W3 = OFF_B2 + HID;
constexpr int OFF_B3 = OFF_W3 + NO * HID;
constexpr int N_PARAMS = OFF_B3 + NO;  // 23300
constexpr int PARTIAL = N_PARAMS + 4;  // + loss, direction loss, logit loss, pad
static_assert(N_PARAMS == NCG_MLP_N_PARAMS, "parameter count");
static_assert(K1 == NCG_MLP_N_INPUTS, "input width");

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ---------------------------------------------------------------- descriptors
// Eigenvalues of a symmetric 3x3 matrix, descending (trigonometric solution,
// f32: descriptors are network inputs, not geometry).
__device__ void sym3_eig(float a00, float a01, float a02, float a11, float a12, float a22, float e[3]) {
    const float p1 = a01 * a01 + a02 * a02 + a12 * a12;
    const float q = (a00 + a11 + a22) * (1.0f / 3.0f);
    const float p2 = (a00 - q) * (a00 - q) + (a11 - q) * (a11 - q) + (a22 - q) * (a22 - q) + 2.0f * p1;
    if (!(p2 > 1e-30f)) { e[0] = e[1] = e[2] = q; return; }
    const float p = sqrtf(p2 * (1.0f / 6.0f));
    const float ip = 1.0f / p;
    const float b00 = (a00 - q) * ip, b11 = (a11 - q) * ip, b22 = (a22 - q) * ip;
    const float b01 = a01 * ip, b02 = a02 * ip, b12 = a12 * ip;
    float r = 0.5f * (b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02));
    r = fminf(fmaxf(r, -1.0f), 1.0f);
    const float phi = acosf(r) * (1.0f / 3.0f);
    e[0] = q + 2.0f * p * cosf(phi);
    e[2] = q + 2.0f * p * cosf(phi + 2.09439510f);
    e[1] = 3.0f * q - e[0] - e[2];
}

__global__ void k_shape_desc(ncg_batch b, float* desc) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t sid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (sid >= b.n_shapes) return;
    Shape s;
    float d[DESC];
    for (int i = 0; i < DESC; ++i) d[i] = 0.0f;
    if (!load_shape(b, (uint32_t)sid, s)) {
        if (lane < DESC) desc[sid * DESC + lane] = 0.0f;
        return;
    }
    d[s.kind] = 1.0f;
    if (s.kind != NCG_CONVEX_HULL) {
        d[6] = s.p0; d[7] = s.p1; d[8] = s.p2;
        float r;
        switch (s.kind) {
        case NCG_BALL: r = s.p0; break;
        case NCG_CUBOID: r = sqrtf(s.p0 * s.p0 + s.p1 * s.p1 + s.p2 * s.p2); break;
        case NCG_CAPSULE: r = s.p0 + s.p1; break;
        default: r = sqrtf(s.p0 * s.p0 + s.p1 * s.p1); break;  // cone, cylinder
        }
        d[13] = r;
    } else {
        const float4* pts = reinterpret_cast<const float4*>(b.hull_points) + s.off;
        float mx = 0.0f, my = 0.0f, mz = 0.0f, r2 = 0.0f;
        float sx = 0, sy = 0, sz = 0, sxx = 0, sxy = 0, sxz = 0, syy = 0, syz = 0, szz = 0;
        for (uint32_t i = lane; i < s.n; i += 32) {
            float4 p = __ldg(pts + i);
            mx = fmaxf(mx, fabsf(p.x)); my = fmaxf(my, fabsf(p.y)); mz = fmaxf(mz, fabsf(p.z));
            r2 = fmaxf(r2, p.x * p.x + p.y * p.y + p.z * p.z);
            sx += p.x; sy += p.y; sz += p.z;
            sxx += p.x * p.x; sxy += p.x * p.y; sxz += p.x * p.z;
            syy += p.y * p.y; syz += p.y * p.z; szz += p.z * p.z;
        }
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
            mz = fmaxf(mz, __shfl_xor_sync(0xffffffffu, mz, o));
            r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, o));
            sx += __shfl_xor_sync(0xffffffffu, sx, o); sy += __shfl_xor_sync(0xffffffffu, sy, o);
            sz += __shfl_xor_sync(0xffffffffu, sz, o); sxx += __shfl_xor_sync(0xffffffffu, sxx, o);
            sxy += __shfl_xor_sync(0xffffffffu, sxy, o); sxz += __shfl_xor_sync(0xffffffffu, sxz, o);
            syy += __shfl_xor_sync(0xffffffffu, syy, o); syz += __shfl_xor_sync(0xffffffffu, syz, o);
            szz += __shfl_xor_sync(0xffffffffu, szz, o);
        }
        const float inv = 1.0f / (float)s.n;
        const float cx = sx * inv, cy = sy * inv, cz = sz * inv;
        float e[3];
        sym3_eig(sxx * inv - cx * cx, sxy * inv - cx * cy, sxz * inv - cx * cz, syy * inv - cy * cy,
                 syz * inv - cy * cz, szz * inv - cz * cz, e);
        d[6] = mx; d[7] = my; d[8] = mz;
        d[9] = sqrtf(fmaxf(e[0], 0.0f));
        d[10] = sqrtf(fmaxf(e[1], 0.0f));
        d[11] = sqrtf(fmaxf(e[2], 0.0f));
        d[12] = log2f((float)s.n) * 0.1f;
        d[13] = sqrtf(r2);
    }
    // one lane per descriptor entry (coalesced 64-byte store)
    float v = 0.0f;
#pragma unroll
    for (int i = 0; i < DESC; ++i) v = (int)lane == i ? d[i] : v;
    if (lane < DESC) desc[sid * DESC + lane] = v;
}

// Features of pair i (K1 floats, zero padded) and the pose of A; false for a
// pair with an invalid shape index.
__device__ bool pair_features(const ncg_batch& b, const float* desc, uint64_t i, float* x, Pose& pa) {
    for (int k = 0; k < K1; ++k) x[k] = 0.0f;
    const uint32_t ga = b.g1[i], gb = b.g2[i];
    pa = load_pose(b.m1 + i);
    const Pose pb = load_pose(b.m2 + i);
    if (ga >= b.n_shapes || gb >= b.n_shapes) return false;
    const float* da = desc + (uint64_t)ga * DESC;
    const float* db = desc + (uint64_t)gb * DESC;
    float ra = da[13], rb = db[13];
    float sc = ra + rb;
    sc = sc > 1e-6f ? sc : 1.0f;
    vec3<float> t = qrot_inv(pa.q, pb.t - pa.t);
    x[0] = t.x / sc; x[1] = t.y / sc; x[2] = t.z / sc;
    // q_A^-1 q_B
    const float ai = -pa.q.x, aj = -pa.q.y, ak = -pa.q.z, aw = pa.q.w;
    const float bi = pb.q.x, bj = pb.q.y, bk = pb.q.z, bw = pb.q.w;
    float qi = aw * bi + ai * bw + aj * bk - ak * bj;
    float qj = aw * bj - ai * bk + aj * bw + ak * bi;
    float qk = aw * bk + ai * bj - aj * bi + ak * bw;
    float qw = aw * bw - ai * bi - aj * bj - ak * bk;
    if (qw < 0.0f) { qi = -qi; qj = -qj; qk = -qk; qw = -qw; }
    x[3] = qi; x[4] = qj; x[5] = qk; x[6] = qw;
    for (int k = 0; k < DESC; ++k) { x[7 + k] = da[k]; x[23 + k] = db[k]; }
    return true;
}

__global__ void k_features(ncg_batch b, const float* desc, float* X) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n_pairs) return;
    float x[K1];
    Pose pa;
    pair_features(b, desc, i, x, pa);
    for (int k = 0; k < K1; ++k) X[i * K1 + k] = x[k];
}

// ---------------------------------------------------------------- smem staging
// Row `r` of a K-major tile: columns k0..k0+7 from v (one 16-byte store).
__device__ __forceinline__ void put8(uint8_t* tile, int r, int k0, int K, const float* v) {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]), p1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]), p3 = __floats2bfloat162_rn(v[6], v[7]);
    uint4 u;
    u.x = *reinterpret_cast<uint32_t*>(&p0);
    u.y = *reinterpret_cast<uint32_t*>(&p1);
    u.z = *reinterpret_cast<uint32_t*>(&p2);
    u.w = *reinterpret_cast<uint32_t*>(&p3);
    *reinterpret_cast<uint4*>(tile + tc::kmaj(r, k0, K)) = u;
}
__device__ __forceinline__ void put1(uint8_t* tile, int r, int k, int K, float v) {
    *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmaj(r, k, K)) = __float2bfloat16_rn(v);
}

// Stages the parameters as bf16 K-major operands.  `rows x K` tile t holds
// element (r, k) = W[src(r, k)]; zero where the source is out of range.
__device__ void stage_weights(const float* P, uint8_t* sW1, uint8_t* sW2, uint8_t* sW3, uint8_t* sW3T,
                              uint8_t* sW2T) {
    for (int e = threadIdx.x; e < HID * K1; e += blockDim.x) {
        int r = e / K1, k = e % K1;
        put1(sW1, r, k, K1, P[OFF_W1 + r * K1 + k]);
    }
    for (int e = threadIdx.x; e < HID * HID; e += blockDim.x) {
        int r = e / HID, k = e % HID;
        float w = P[OFF_W2 + r * HID + k];
        put1(sW2, r, k, HID, w);
        if (sW2T) put1(sW2T, k, r, HID, w);
    }
    for (int e = threadIdx.x; e < N3 * HID; e += blockDim.x) {
        int r = e / HID, k = e % HID;
        float w = r < NO ? P[OFF_W3 + r * HID + k] : 0.0f;
        put1(sW3, r, k, HID, w);
        if (sW3T) put1(sW3T, k, r, N3, w);
    }
}

// Column sums of a 128 x 32 block held one row per thread (thread = row):
// out[c] for c < n_out gets the sum over the 128 rows in a fixed order.
// Every thread of the CTA must call it.
__device__ void colsum32(const float* v, float* red /*[4][32]*/, float* out, int n_out) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    float mine = 0.0f;
#pragma unroll
    for (int c = 0; c < 32; ++c) {
        float s = v[c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((int)lane == c) mine = s;
    }
    red[warp * 32 + lane] = mine;
    __syncthreads();
    if ((int)threadIdx.x < n_out) {
        float s = ((red[threadIdx.x] + red[32 + threadIdx.x]) + red[64 + threadIdx.x]) + red[96 + threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

// ---------------------------------------------------------------- inference
struct InferSmem {
    static constexpr size_t W1 = 0, W2 = W1 + HID * K1 * 2, W3 = W2 + HID * HID * 2, X = W3 + N3 * HID * 2,
                            A = X + TILE * K1 * 2, BIAS = A + TILE * HID * 2, BAR = BIAS + (2 * HID + N3) * 4,
                            TSLOT = BAR + 8, BYTES = TSLOT + 8;
};
// Two CTAs fit on an SM (shared memory and 2 x 256 TMEM columns).
static_assert(2 * InferSmem::BYTES <= 228 * 1024 - 2 * 1024, "two inference CTAs per SM");

// Persistent over 128-pair tiles: features -> three layers -> init_dir (world,
// unit).  128 threads: thread t owns row t of a tile (TMEM lane t).
__global__ void __launch_bounds__(128, 2) k_mlp_infer(ncg_batch b, const float* P, const float* desc, float* init_dir,
                                                      uint32_t* err) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t *sW1 = sm + InferSmem::W1, *sW2 = sm + InferSmem::W2, *sW3 = sm + InferSmem::W3;
    uint8_t *sX = sm + InferSmem::X, *sA = sm + InferSmem::A;
    float* bias = reinterpret_cast<float*>(sm + InferSmem::BIAS);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + InferSmem::BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + InferSmem::TSLOT);
    const int t = threadIdx.x, warp = t >> 5;

    stage_weights(P, sW1, sW2, sW3, nullptr, nullptr);
    for (int e = t; e < HID; e += blockDim.x) { bias[e] = P[OFF_B1 + e]; bias[HID + e] = P[OFF_B2 + e]; }
    if (t < N3) bias[2 * HID + t] = t < NO ? P[OFF_B3 + t] : 0.0f;
    if (t == 0) tc::mbar_init(bar, 1);
    if (warp == 0) tc::tmem_alloc(tslot, 256);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    const uint32_t D1 = tbase, D2 = tbase + 128, D3 = tbase;
    uint32_t phase = 0;
    bool ok = true;
    const uint64_t n_tiles = (b.n_pairs + TILE - 1) / TILE;

    for (uint64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const uint64_t i = tile * TILE + t;
        float x[K1];
        Pose pa;
        pa.q = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        pa.t = zero3<float>();
        if (i < b.n_pairs) pair_features(b, desc, i, x, pa);
        else for (int k = 0; k < K1; ++k) x[k] = 0.0f;
        for (int k = 0; k < K1; k += 8) put8(sX, t, k, K1, x + k);
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        // layer 1
        if (t == 0) {
            tc::fence_after_sync();
            tc::mma_tile(D1, tc::smem_u32(sX), tc::smem_u32(sW1), TILE, HID, K1, false);
            tc::commit(bar);
        }
        ok = __syncthreads_and(tc::mbar_wait(bar, phase, err)) != 0;
        phase ^= 1u;
        tc::fence_after_sync();
        if (!ok) break;
        for (int c = 0; c < HID; c += 32) {
            float v[32];
            tc::tmem_ld32(D1 + lane_off + c, v);
            for (int j = 0; j < 32; ++j) v[j] = gelu(v[j] + bias[c + j]);
            for (int j = 0; j < 32; j += 8) put8(sA, t, c + j, HID, v + j);
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        // layer 2
        if (t == 0) {
            tc::fence_after_sync();
            tc::mma_tile(D2, tc::smem_u32(sA), tc::smem_u32(sW2), TILE, HID, HID, false);
            tc::commit(bar);
        }
        ok = __syncthreads_and(tc::mbar_wait(bar, phase, err)) != 0;
        phase ^= 1u;
        tc::fence_after_sync();
        if (!ok) break;
        for (int c = 0; c < HID; c += 32) {
            float v[32];
            tc::tmem_ld32(D2 + lane_off + c, v);
            for (int j = 0; j < 32; ++j) v[j] = gelu(v[j] + bias[HID + c + j]);
            for (int j = 0; j < 32; j += 8) put8(sA, t, c + j, HID, v + j);  // H2 over H1 (layer 2 done)
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        // layer 3 (overwrites D1's first 16 columns, consumed above)
        if (t == 0) {
            tc::fence_after_sync();
            tc::mma_tile(D3, tc::smem_u32(sA), tc::smem_u32(sW3), TILE, N3, HID, false);
            tc::commit(bar);
        }
        ok = __syncthreads_and(tc::mbar_wait(bar, phase, err)) != 0;
        phase ^= 1u;
        tc::fence_after_sync();
        if (!ok) break;
        float y[16];
        tc::tmem_ld16(D3 + lane_off, y);
        if (i < b.n_pairs) {
            vec3<float> u{y[0] + bias[2 * HID], y[1] + bias[2 * HID + 1], y[2] + bias[2 * HID + 2]};
            vec3<float> w = qrot(pa.q, u);
            float n = sqrtf(w.x * w.x + w.y * w.y + w.z * w.z);
            vec3<float> d;
            if (n > 1e-12f && isfinite(n)) {
                d = {w.x / n, w.y / n, w.z / n};
            } else {  // the reference's default: normalize(t2 - t1), else +x
                const Pose pb = load_pose(b.m2 + i);
                vec3<float> dd = pb.t - pa.t;
                float m = sqrtf(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
                d = m > FLT_EPSILON ? vec3<float>{dd.x / m, dd.y / m, dd.z / m} : vec3<float>{1.0f, 0.0f, 0.0f};
            }
            init_dir[3 * i] = d.x;
            init_dir[3 * i + 1] = d.y;
            init_dir[3 * i + 2] = d.z;
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

// ---------------------------------------------------------------- training
struct TrainSmem {
    static constexpr size_t W1 = 0, W2 = W1 + HID * K1 * 2, W3 = W2 + HID * HID * 2, W3T = W3 + N3 * HID * 2,
                            W2T = W3T + HID * N3 * 2, X = W2T + HID * HID * 2, XT = X + TILE * K1 * 2,
                            A = XT + K1 * TILE * 2, H1T = A + TILE * HID * 2, B = H1T + HID * TILE * 2,
                            DY = B + HID * TILE * 2, DYT = DY + TILE * N3 * 2, RED = DYT + N3 * TILE * 2,
                            BIAS = RED + 4 * 32 * 4, BAR = BIAS + (2 * HID + N3) * 4, TSLOT = BAR + 8,
                            BYTES = TSLOT + 8;
};
static_assert(TrainSmem::BYTES <= 232448, "training tile must fit in shared memory");

// One 128-sample tile: forward, loss, backward; writes the tile's parameter
// gradients (and loss sums) to partial[tile * PARTIAL ...].  Rows past n are
// padding and contribute nothing.  labels: [n][4] = direction (A's frame,
// unit) xyz, intersecting (0/1).  Gradients are of the mean loss over
// `n_mean` samples.
__global__ void __launch_bounds__(128, 1) k_mlp_train_tile(const float* P, const float* X, const float* labels,
                                                           uint64_t n, float inv_n, float logit_weight,
                                                           float* partial, uint32_t* err) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t *sW1 = sm + TrainSmem::W1, *sW2 = sm + TrainSmem::W2, *sW3 = sm + TrainSmem::W3;
    uint8_t *sW3T = sm + TrainSmem::W3T, *sW2T = sm + TrainSmem::W2T, *sX = sm + TrainSmem::X;
    uint8_t *sXT = sm + TrainSmem::XT, *sA = sm + TrainSmem::A, *sH1T = sm + TrainSmem::H1T;
    uint8_t *sB = sm + TrainSmem::B, *sDY = sm + TrainSmem::DY, *sDYT = sm + TrainSmem::DYT;
    float* red = reinterpret_cast<float*>(sm + TrainSmem::RED);
    float* bias = reinterpret_cast<float*>(sm + TrainSmem::BIAS);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + TrainSmem::BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + TrainSmem::TSLOT);
    const int t = threadIdx.x, warp = t >> 5;
    const uint64_t tile = blockIdx.x;
    const uint64_t row = tile * TILE + t;
    const bool valid = row < n;
    float* out = partial + tile * PARTIAL;

    stage_weights(P, sW1, sW2, sW3, sW3T, sW2T);
    for (int e = t; e < HID; e += blockDim.x) { bias[e] = P[OFF_B1 + e]; bias[HID + e] = P[OFF_B2 + e]; }
    if (t < N3) bias[2 * HID + t] = t < NO ? P[OFF_B3 + t] : 0.0f;
    float x[K1];
    for (int k = 0; k < K1; ++k) x[k] = valid ? X[row * K1 + k] : 0.0f;
    for (int k = 0; k < K1; k += 8) put8(sX, t, k, K1, x + k);
    for (int k = 0; k < K1; ++k) put1(sXT, k, t, TILE, x[k]);
    if (t == 0) tc::mbar_init(bar, 1);
    if (warp == 0) tc::tmem_alloc(tslot, 512);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tb = *tslot;
    const uint32_t lo = (uint32_t)(warp * 32) << 16;
    // TMEM columns: [0,128) z1 then dW1; [128,256) z2 then dW2; [256,384) dH2
    // then dH1; [384,400) y then dW3^T.
    const uint32_t C_Z1 = tb, C_Z2 = tb + 128, C_DH = tb + 256, C_Y = tb + 384;
    uint32_t ph = 0;
    bool ok = true;
    auto sync_mma = [&]() {  // all threads: make smem writes visible, then order against the MMA issue
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
    };
    auto wait_mma = [&]() -> bool {  // CTA-uniform result
        bool r = tc::mbar_wait(bar, ph, err);
        ph ^= 1u;
        tc::fence_after_sync();
        return __syncthreads_and(r) != 0;
    };

    // ---- forward, layer 1: z1 = X W1^T
    if (t == 0) {
        tc::fence_after_sync();
        tc::mma_tile(C_Z1, tc::smem_u32(sX), tc::smem_u32(sW1), TILE, HID, K1, false);
        tc::commit(bar);
    }
    ok = wait_mma();
    if (ok) {
        for (int c = 0; c < HID; c += 32) {
            float v[32];
            tc::tmem_ld32(C_Z1 + lo + c, v);
            for (int j = 0; j < 32; ++j) v[j] = gelu(v[j] + bias[c + j]);
            for (int j = 0; j < 32; j += 8) put8(sA, t, c + j, HID, v + j);
            for (int j = 0; j < 32; ++j) put1(sH1T, c + j, t, TILE, v[j]);
        }
    }
    sync_mma();
    // ---- layer 2: z2 = H1 W2^T
    if (ok && t == 0) {
        tc::fence_after_sync();
        tc::mma_tile(C_Z2, tc::smem_u32(sA), tc::smem_u32(sW2), TILE, HID, HID, false);
        tc::commit(bar);
    }
    if (ok) ok = wait_mma();
    if (ok) {
        for (int c = 0; c < HID; c += 32) {
            float v[32];
            tc::tmem_ld32(C_Z2 + lo + c, v);
            for (int j = 0; j < 32; ++j) v[j] = gelu(v[j] + bias[HID + c + j]);
            for (int j = 0; j < 32; j += 8) put8(sA, t, c + j, HID, v + j);  // H2 (H1 consumed)
            for (int j = 0; j < 32; ++j) put1(sB, c + j, t, TILE, v[j]);     // H2^T
        }
    }
    sync_mma();
    // ---- layer 3: y = H2 W3^T
    if (ok && t == 0) {
        tc::fence_after_sync();
        tc::mma_tile(C_Y, tc::smem_u32(sA), tc::smem_u32(sW3), TILE, N3, HID, false);
        tc::commit(bar);
    }
    if (ok) ok = wait_mma();
    // ---- loss and dY
    float dy[N3], lsum[32];
    for (int j = 0; j < N3; ++j) dy[j] = 0.0f;
    for (int j = 0; j < 32; ++j) lsum[j] = 0.0f;
    if (ok) {
        float y[16];
        tc::tmem_ld16(C_Y + lo, y);
        if (valid) {
            const float* lab = labels + row * 4;
            float u0 = y[0] + bias[2 * HID], u1 = y[1] + bias[2 * HID + 1], u2 = y[2] + bias[2 * HID + 2];
            float s = y[3] + bias[2 * HID + 3];
            float nu = sqrtf(u0 * u0 + u1 * u1 + u2 * u2 + 1e-12f);
            float d0 = u0 / nu, d1 = u1 / nu, d2 = u2 / nu;
            float c = d0 * lab[0] + d1 * lab[1] + d2 * lab[2];
            dy[0] = -(lab[0] - c * d0) / nu * inv_n;
            dy[1] = -(lab[1] - c * d1) / nu * inv_n;
            dy[2] = -(lab[2] - c * d2) / nu * inv_n;
            float z = lab[3];
            float sig = 1.0f / (1.0f + expf(-s));
            dy[3] = logit_weight * (sig - z) * inv_n;
            float sp = fmaxf(s, 0.0f) + log1pf(expf(-fabsf(s)));  // softplus(s)
            lsum[1] = (1.0f - c) * inv_n;
            lsum[2] = (sp - z * s) * inv_n;
            lsum[0] = lsum[1] + logit_weight * lsum[2];
        }
    }
    // dY (A: rows = samples, K = 16 outputs) and dY^T (B: rows = outputs, K = samples)
    for (int j = 0; j < N3; j += 8) put8(sDY, t, j, N3, dy + j);
    for (int j = 0; j < N3; ++j) put1(sDYT, j, t, TILE, dy[j]);
    colsum32(lsum, red, out + N_PARAMS, 3);  // loss, direction loss, logit loss
    {                                          // db3 = column sums of dY (first 4 columns)
        float v[32];
        for (int j = 0; j < 32; ++j) v[j] = j < NO ? dy[j] : 0.0f;
        colsum32(v, red, out + OFF_B3, NO);
    }
    sync_mma();
    // ---- dH2 = dY W3 ; dW3^T = H2^T dY
    if (ok && t == 0) {
        tc::fence_after_sync();
        tc::mma_tile(C_DH, tc::smem_u32(sDY), tc::smem_u32(sW3T), TILE, HID, N3, false);
        tc::mma_tile(C_Y, tc::smem_u32(sB), tc::smem_u32(sDYT), HID, N3, TILE, false);
        tc::commit(bar);
    }
    if (ok) ok = wait_mma();
    if (ok) {
        float w3[16];
        tc::tmem_ld16(C_Y + lo, w3);  // row t = hidden unit i, columns = outputs o
        for (int o = 0; o < NO; ++o) out[OFF_W3 + o * HID + t] = w3[o];
        for (int c = 0; c < HID; c += 32) {
            float g[32], z[32];
            tc::tmem_ld32(C_DH + lo + c, g);
            tc::tmem_ld32(C_Z2 + lo + c, z);
            for (int j = 0; j < 32; ++j) g[j] = valid ? g[j] * gelu_d(z[j] + bias[HID + c + j]) : 0.0f;
            for (int j = 0; j < 32; j += 8) put8(sA, t, c + j, HID, g + j);  // dZ2 (H2 consumed)
            for (int j = 0; j < 32; ++j) put1(sB, c + j, t, TILE, g[j]);     // dZ2^T (H2^T consumed)
            colsum32(g, red, out + OFF_B2 + c, 32);                           // db2
        }
    }
    sync_mma();
    // ---- dH1 = dZ2 W2 ; dW2 = dZ2^T H1
    if (ok && t == 0) {
        tc::fence_after_sync();
        tc::mma_tile(C_DH, tc::smem_u32(sA), tc::smem_u32(sW2T), TILE, HID, HID, false);
        tc::mma_tile(C_Z2, tc::smem_u32(sB), tc::smem_u32(sH1T), HID, HID, TILE, false);
        tc::commit(bar);
    }
    if (ok) ok = wait_mma();
    if (ok) {
        for (int c = 0; c < HID; c += 32) {
            float w[32];
            tc::tmem_ld32(C_Z2 + lo + c, w);  // dW2 row o = t, columns i
            for (int j = 0; j < 32; ++j) out[OFF_W2 + t * HID + c + j] = w[j];
        }
        for (int c = 0; c < HID; c += 32) {
            float g[32], z[32];
            tc::tmem_ld32(C_DH + lo + c, g);
            tc::tmem_ld32(C_Z1 + lo + c, z);
            for (int j = 0; j < 32; ++j) g[j] = valid ? g[j] * gelu_d(z[j] + bias[c + j]) : 0.0f;
            for (int j = 0; j < 32; ++j) put1(sA, c + j, t, TILE, g[j]);  // dZ1^T (dZ2 consumed)
            colsum32(g, red, out + OFF_B1 + c, 32);                      // db1
        }
    }
    sync_mma();
    // ---- dW1 = dZ1^T X
    if (ok && t == 0) {
        tc::fence_after_sync();
        tc::mma_tile(C_Z1, tc::smem_u32(sA), tc::smem_u32(sXT), HID, K1, TILE, false);
        tc::commit(bar);
    }
    if (ok) ok = wait_mma();
    if (ok) {
        float w[32];
        tc::tmem_ld32(C_Z1 + lo, w);
        for (int j = 0; j < 32; ++j) out[OFF_W1 + t * K1 + j] = w[j];
        float w2[16];
        tc::tmem_ld16(C_Z1 + lo + 32, w2);
        for (int j = 0; j < 16; ++j) out[OFF_W1 + t * K1 + 32 + j] = j + 32 < NF ? w2[j] : 0.0f;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tb, 512);
}

// grad[p] = sum over tiles of partial[tile][p], tiles in order.
__global__ void k_mlp_reduce(const float* partial, uint64_t tiles, float* grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= PARTIAL) return;
    float s = 0.0f;
    for (uint64_t k = 0; k < tiles; ++k) s += partial[k * PARTIAL + p];
    grad[p] = s;
}

__global__ void k_mlp_adam(float* P, float* m, float* v, const float* g, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N_PARAMS) return;
    const float gi = g[p];
    const float mi = b1 * m[p] + (1.0f - b1) * gi;
    const float vi = b2 * v[p] + (1.0f - b2) * gi * gi;
    m[p] = mi;
    v[p] = vi;
    P[p] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

}  // namespace mlp

// ---------------------------------------------------------------- internal API
int mlp_shape_desc(const ncg_batch& b, float* desc, cudaStream_t st) {
    if (b.n_shapes == 0) return NCG_OK;
    const uint64_t threads = (uint64_t)b.n_shapes * 32;
    mlp::k_shape_desc<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(b, desc);
    return mlp::ok(cudaGetLastError(), "k_shape_desc") ? NCG_OK : NCG_ECUDA;
}

int mlp_prepare() {
    bool a = mlp::ok(cudaFuncSetAttribute(mlp::k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)mlp::InferSmem::BYTES),
                     "k_mlp_infer attribute");
    bool b = mlp::ok(cudaFuncSetAttribute(mlp::k_mlp_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)mlp::TrainSmem::BYTES),
                     "k_mlp_train_tile attribute");
    return a && b ? NCG_OK : NCG_ECUDA;
}

int mlp_infer(const ncg_batch& b, const float* params, const float* desc, float* init_dir, uint32_t* err, int num_sms,
              cudaStream_t st) {
    const uint64_t tiles = (b.n_pairs + mlp::TILE - 1) / mlp::TILE;
    const uint64_t ctas = 2ull * (uint64_t)num_sms;
    const unsigned grid = (unsigned)(tiles < ctas ? tiles : ctas);
    if (grid == 0) return NCG_OK;
    mlp::k_mlp_infer<<<grid, 128, mlp::InferSmem::BYTES, st>>>(b, params, desc, init_dir, err);
    return mlp::ok(cudaGetLastError(), "k_mlp_infer") ? NCG_OK : NCG_ECUDA;
}

}  // namespace ncg

// ---------------------------------------------------------------- C ABI
extern "C" {

int ncg_mlp_n_params(void) { return ncg::mlp::N_PARAMS; }

int ncg_mlp_features(const ncg_batch* b, float* desc, float* X, void* stream) {
    if (!b || !desc || !X) return NCG_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ncg::mlp_shape_desc(*b, desc, st);
    if (rc) return rc;
    if (b->n_pairs == 0) return NCG_OK;
    ncg::mlp::k_features<<<(unsigned)((b->n_pairs + 127) / 128), 128, 0, st>>>(*b, desc, X);
    return ncg::mlp::ok(cudaGetLastError(), "k_features") ? NCG_OK : NCG_ECUDA;
}

int ncg_mlp_infer(const ncg_batch* b, const float* params, float* desc, float* init_dir, uint32_t* err,
                  void* stream) {
    if (!b || !params || !desc || !init_dir || !err) return NCG_EINVAL;
    int dev = 0, sms = 0;
    if (!ncg::mlp::ok(cudaGetDevice(&dev), "cudaGetDevice")) return NCG_ECUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ncg::mlp_prepare();
    if (rc) return rc;
    rc = ncg::mlp_shape_desc(*b, desc, st);
    if (rc) return rc;
    return ncg::mlp_infer(*b, params, desc, init_dir, err, sms, st);
}

int ncg_mlp_grad(const float* params, const float* X, const float* labels, uint64_t n, float logit_weight,
                 float* partial, float* grad, uint32_t* err, void* stream) {
    if (!params || !X || !labels || !partial || !grad || !err || n == 0) return NCG_EINVAL;
    int rc = ncg::mlp_prepare();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t tiles = (n + ncg::mlp::TILE - 1) / ncg::mlp::TILE;
    ncg::mlp::k_mlp_train_tile<<<(unsigned)tiles, 128, ncg::mlp::TrainSmem::BYTES, st>>>(
        params, X, labels, n, 1.0f / (float)n, logit_weight, partial, err);
    ncg::mlp::k_mlp_reduce<<<(ncg::mlp::PARTIAL + 255) / 256, 256, 0, st>>>(partial, tiles, grad);
    return ncg::mlp::ok(cudaGetLastError(), "k_mlp_train_tile") ? NCG_OK : NCG_ECUDA;
}

int ncg_mlp_adam(float* params, float* m, float* v, const float* grad, float lr, float beta1, float beta2, float eps,
                 int step, void* stream) {
    if (!params || !m || !v || !grad || step < 1) return NCG_EINVAL;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    ncg::mlp::k_mlp_adam<<<(ncg::mlp::N_PARAMS + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, m, v, grad, lr,
                                                                                           beta1, beta2, eps, c1, c2);
    return ncg::mlp::ok(cudaGetLastError(), "k_mlp_adam") ? NCG_OK : NCG_ECUDA;
}

}  // extern "C"
