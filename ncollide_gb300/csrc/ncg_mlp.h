// ncg_mlp.h — internal interface between the query pipeline (ncg_kernels.cu)
// and the learned warm start (ncg_mlp.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/ncg.h"

namespace ncg {

// Records the message ncg_last_error() returns on this thread.
void set_last_error(const std::string& msg);

// Sets the network kernels' shared-memory limits on the current device (call
// outside stream capture).
int mlp_prepare();

// Per-shape descriptors (16 floats per shape) of the batch's shape table.
int mlp_shape_desc(const ncg_batch& b, float* desc, cudaStream_t st);

// The network's GJK start direction (world frame, unit) for every pair of
// the batch, from `params` (NCG_MLP_N_PARAMS floats) and the descriptors.
// A timeout of a tensor-core wait sets *err.
int mlp_infer(const ncg_batch& b, const float* params, const float* desc, float* init_dir, uint32_t* err,
              int num_sms, cudaStream_t st);

}  // namespace ncg
