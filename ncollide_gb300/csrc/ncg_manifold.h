// ncg_manifold.h — internal interface between the C ABI (ncg_kernels.cu) and
// the contact-manifold kernel (ncg_manifold.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/ncg.h"

namespace ncg {

// ContactPrediction: the linear margin and the cosines / sines of the two
// angular tolerances (computed on the host, as the reference's f32 cos / sin).
struct ManifoldParams {
    float linear, cang1, sang1, cang2, sang2;
};

// Manifolds of every pair from the contact query's outputs; ORs
// NCG_STATUS_NOT_POLYHEDRA into status for pairs that are not two Cuboids.
int manifold_launch(const ncg_batch& b, const ncg_contact* contact, const uint8_t* has, const ManifoldParams& mp,
                    ncg_manifold* out, uint32_t* status, int num_sms, cudaStream_t st);

}  // namespace ncg
