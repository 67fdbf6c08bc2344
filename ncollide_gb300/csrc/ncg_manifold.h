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

// The device arrays of an ncg_hull_topology (shape == nullptr: no ConvexHull
// topology, ConvexHull pairs keep their single contact).
struct HullTopo {
    const uint32_t* shape;
    const float* face_normal;
    const uint32_t* face_range;
    const uint32_t* face_vertex;
    const uint32_t* face_edge;
    const uint32_t* edge_vertex;
    const float* edge_dir;
    const uint32_t* vertex_range;
    const uint32_t* vertex_face;
    const uint32_t* vertex_edge;
};

// Manifolds of every pair from the contact query's outputs; ORs
// NCG_STATUS_NOT_POLYHEDRA into status for pairs that are not two polyhedra
// (Cuboid, or ConvexHull with a topology).
int manifold_launch(const ncg_batch& b, const ncg_contact* contact, const uint8_t* has, const ManifoldParams& mp,
                    const HullTopo& topo, ncg_manifold* out, uint32_t* status, int num_sms, cudaStream_t st);

}  // namespace ncg
