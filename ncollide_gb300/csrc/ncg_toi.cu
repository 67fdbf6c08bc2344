// ncg_toi.cu — batched linear time of impact: query::time_of_impact for the
// support-map shapes of this library (time_of_impact.rs:63-90), one thread per
// pair.  The arithmetic is in ncg_toi.cuh.
#include <cuda_runtime.h>

#include <cfloat>
#include <string>

#include "ncg_mlp.h"
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

__global__ void __launch_bounds__(128, NCG_TOI_MIN_BLOCKS) k_toi(ncg_batch b, Tol tol, ToiArgs a) {
    const ThreadScan scan{reinterpret_cast<const float4*>(b.hull_points)};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_pairs; i += stride) {
        uint32_t status = 0, iters = 0;
        ToiResult r;
        r.some = false;
        PairGeom g;
        const bool ok = load_shape(b, b.g1[i], g.g1) && load_shape(b, b.g2[i], g.g2);
        if (!ok) {
            status = NCG_STATUS_BAD_INPUT;
        } else {
            g.m1 = load_pose(b.m1 + i);
            g.m2 = load_pose(b.m2 + i);
            const float* p = a.vel1 + 3 * i;
            const float* q = a.vel2 + 3 * i;
            const vec3<float> v1{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
            const vec3<float> v2{__ldg(q), __ldg(q + 1), __ldg(q + 2)};
            const real max_toi = from_host(a.max_toi);
            if (a.dispatch == NCG_DISPATCH_QUERY && g.g1.kind == NCG_BALL && g.g2.kind == NCG_BALL)
                r = toi_ball_ball(g.m1, v1, g.g1.p0, g.m2, v2, g.g2.p0, max_toi, a.target);
            else
                r = toi_support_map(g, v1, v2, max_toi, a.target, tol, scan, iters, status, a.max_iter);
        }
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
}

}  // namespace

int toi_launch(const ncg_batch& b, const Tol& tol, int dispatch, const float* vel1, const float* vel2,
               float max_toi, float target_distance, ncg_toi* out, uint8_t* has_toi, uint32_t* status,
               uint32_t* iters, int num_sms, cudaStream_t st) {
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
    const uint64_t blocks = (b.n_pairs + 127) / 128;
    const uint64_t cap = (uint64_t)num_sms * NCG_TOI_MIN_BLOCKS * 8;
    k_toi<<<(unsigned)(blocks < cap ? blocks : cap), 128, 0, st>>>(b, tol, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("k_toi launch: ") + cudaGetErrorString(e));
        return NCG_ECUDA;
    }
    return NCG_OK;
}

}  // namespace ncg
