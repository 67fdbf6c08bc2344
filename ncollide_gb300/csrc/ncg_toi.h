// ncg_toi.h — internal interface between the C ABI (ncg_kernels.cu) and the
// time-of-impact kernel (ncg_toi.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/ncg.h"

namespace ncg {

struct Tol;

// Launches the time-of-impact kernel over every pair of the batch (arguments
// validated by the caller).  Returns NCG_OK or NCG_ECUDA.
int toi_launch(const ncg_batch& b, const Tol& tol, int dispatch, const float* vel1, const float* vel2,
               float max_toi, float target_distance, ncg_toi* out, uint8_t* has_toi, uint32_t* status,
               uint32_t* iters, int num_sms, cudaStream_t st);

}  // namespace ncg
