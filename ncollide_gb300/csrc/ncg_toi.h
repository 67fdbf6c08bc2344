// ncg_toi.h — internal interface between the C ABI (ncg_kernels.cu) and the
// time-of-impact and ray-cast kernels (ncg_toi.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/ncg.h"

namespace ncg {

struct Tol;

// Device scratch of one call: a bucket byte and a sorted index per pair, 512
// bytes of counters, 24 bytes per pair for the refinement queue (16-byte
// aligned), and the 64-bit sum of the iteration counts (added to).
struct ToiScratch {
    uint8_t* bucket;
    uint32_t* sorted;
    void* ctr;
    void* refine;
    unsigned long long* iter_sum;
};

// Launches the time-of-impact kernels over every pair of the batch (arguments
// validated by the caller): classification, the counting sort by cost bucket,
// then one thread per pair over the sorted list.  Adds the number of launches
// to *launches.  Returns NCG_OK or NCG_ECUDA.
int toi_launch(const ncg_batch& b, const Tol& tol, int dispatch, const float* vel1, const float* vel2,
               float max_toi, float target_distance, ncg_toi* out, uint8_t* has_toi, uint32_t* status,
               uint32_t* iters, const ToiScratch& scratch, int num_sms, cudaStream_t st, uint32_t* launches);

// Launches the ray-cast kernels over every ray of the batch (ray i against
// shapes[g1[i]] at m1[i]; m2, g2 unused; arguments validated by the caller).
int ray_launch(const ncg_batch& b, const Tol& tol, const float* rays, float max_toi, int solid, float* out_toi,
               float* out_normal, uint8_t* hit, uint32_t* status, uint32_t* iters, const ToiScratch& scratch,
               int num_sms, cudaStream_t st, uint32_t* launches);

}  // namespace ncg
