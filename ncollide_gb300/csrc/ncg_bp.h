// ncg_bp.h — internal interface between the C ABI (ncg_kernels.cu) and the
// bounding-volume and broad-phase kernels (ncg_bp.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/ncg.h"

namespace ncg {

struct BroadPhaseState;

// World AABBs (mins[3], maxs[3]) of shapes[g1[i]] at m1[i] for every entry of
// the batch; a bad shape gets NaN bounds and NCG_STATUS_BAD_INPUT.
int aabb_launch(const ncg_batch& b, float* out, uint32_t* status, int num_sms, cudaStream_t st);

// m1/g1/m2/g2 of pair k = (pairs[2k], pairs[2k+1]) from the proxies' poses and shape ids.
int gather_launch(const ncg_pose* poses, const uint32_t* shape_ids, const uint32_t* pairs, uint64_t n, ncg_pose* m1,
                  uint32_t* g1, ncg_pose* m2, uint32_t* g2, int num_sms, cudaStream_t st);

int bp_create(float margin, int device, BroadPhaseState** out);
void bp_destroy(BroadPhaseState* s);
// Stores the boxes (loosened where they left their stored box), rebuilds the
// tree, finds the pairs and the events; synchronises the stream.
int bp_update(BroadPhaseState* s, const float* boxes, uint32_t n, cudaStream_t st);
void bp_results(const BroadPhaseState* s, uint64_t* n_pairs, uint64_t* n_started, uint64_t* n_stopped,
                const uint32_t** pairs, const uint32_t** started, const uint32_t** stopped);

}  // namespace ncg
