// ncg_oracle_bp.hpp — TEST INFRASTRUCTURE ONLY: CPU restatement of the
// bounding volumes of the support-map shapes and of the pair set the DBVT
// broad phase maintains.
//
// Reference (ncollide 0.33):
//   src/bounding_volume/aabb_ball.rs:7-13, 23-28       ball_aabb: centre -+ radius
//   src/bounding_volume/aabb_cuboid.rs:8-13            |R| h about the translation
//   src/bounding_volume/aabb_support_map.rs            Capsule, Cone, Cylinder: support_map_aabb
//   src/bounding_volume/aabb_utils.rs:8-31             support_map_aabb (support points along +-e_d)
//   src/bounding_volume/aabb_utils.rs:55-74            point_cloud_aabb (ConvexHull, aabb_convex.rs)
//   src/bounding_volume/aabb.rs:156-195                intersects, contains, loosened
//   src/pipeline/broad_phase/dbvt_broad_phase.rs:174-258, 322-347   update, deferred_set_bounding_volume
// The rotation matrix of a unit quaternion is nalgebra's to_rotation_matrix
// (nalgebra 0.30, not vendored), restated from the published formula
// (ww + ii - jj - kk, 2(ij - wk), 2(wj + ik); ...); its bit-level agreement
// with nalgebra is unpinned, like the quaternion rotation of the query path.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "ncg_oracle.hpp"

namespace ncgo {

struct AABB {
    float mins[3], maxs[3];
};

// UnitQuaternion::to_rotation_matrix, row-major.
inline void rotation_matrix(const Quat<float>& q, float r[3][3]) {
    const float i = q.i, j = q.j, k = q.k, w = q.w;
    const float ww = w * w, ii = i * i, jj = j * j, kk = k * k;
    const float ij = i * j * 2.0f, wk = w * k * 2.0f, wj = w * j * 2.0f, ik = i * k * 2.0f, jk = j * k * 2.0f,
                wi = w * i * 2.0f;
    r[0][0] = ww + ii - jj - kk; r[0][1] = ij - wk;           r[0][2] = wj + ik;
    r[1][0] = wk + ij;           r[1][1] = ww - ii + jj - kk; r[1][2] = jk - wi;
    r[2][0] = ik - wj;           r[2][1] = wi + jk;           r[2][2] = ww - ii - jj + kk;
}

// HasBoundingVolume<AABB>::bounding_volume of each support-map shape at pose m.
inline AABB shape_aabb(const Iso<float>& m, const Shape<float>& s) {
    AABB b;
    const float t[3] = {m.t.x, m.t.y, m.t.z};
    if (s.kind == BALL) {
        for (int d = 0; d < 3; ++d) {
            b.mins[d] = t[d] + -s.p0;
            b.maxs[d] = t[d] + s.p0;
        }
    } else if (s.kind == CUBOID) {
        float r[3][3];
        rotation_matrix(m.q, r);
        const float h[3] = {s.p0, s.p1, s.p2};
        for (int d = 0; d < 3; ++d) {
            const float he = (std::fabs(r[d][0]) * h[0] + std::fabs(r[d][1]) * h[1]) + std::fabs(r[d][2]) * h[2];
            b.mins[d] = t[d] - he;
            b.maxs[d] = t[d] + he;
        }
    } else if (s.kind == CONVEX_HULL) {
        for (uint32_t p = 0; p < s.n; ++p) {
            const V3<float> w = transform_point(m, s.point(p));
            const float v[3] = {w.x, w.y, w.z};
            for (int d = 0; d < 3; ++d) {
                if (p == 0 || v[d] < b.mins[d]) b.mins[d] = v[d];
                if (p == 0 || v[d] > b.maxs[d]) b.maxs[d] = v[d];
            }
        }
    } else {
        for (int d = 0; d < 3; ++d) {
            V3<float> e{0.0f, 0.0f, 0.0f};
            (&e.x)[d] = 1.0f;
            const V3<float> hi = support_point(m, s, e, nullptr);
            (&e.x)[d] = -1.0f;
            const V3<float> lo = support_point(m, s, e, nullptr);
            b.maxs[d] = (&hi.x)[d];
            b.mins[d] = (&lo.x)[d];
        }
    }
    return b;
}

// AABB::intersects (closed intervals; false when a bound is NaN).
inline bool intersects(const AABB& a, const AABB& b) {
    for (int d = 0; d < 3; ++d)
        if (!(a.mins[d] <= b.maxs[d] && a.maxs[d] >= b.mins[d])) return false;
    return true;
}

// Every unordered pair (i < j) of intersecting boxes, sorted: sort and sweep
// along x (the pair set equals the DBVT's: both report exactly the
// intersecting pairs of the stored boxes).
inline std::vector<uint64_t> intersecting_pairs(const AABB* boxes, uint32_t n) {
    std::vector<uint32_t> order;
    for (uint32_t i = 0; i < n; ++i)
        if (boxes[i].mins[0] == boxes[i].mins[0]) order.push_back(i);  // NaN boxes never intersect
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return boxes[a].mins[0] < boxes[b].mins[0] || (boxes[a].mins[0] == boxes[b].mins[0] && a < b);
    });
    std::vector<uint64_t> out;
    for (size_t a = 0; a < order.size(); ++a) {
        const AABB& A = boxes[order[a]];
        for (size_t c = a + 1; c < order.size(); ++c) {
            const AABB& C = boxes[order[c]];
            if (!(C.mins[0] <= A.maxs[0])) break;
            if (intersects(A, C)) {
                const uint32_t lo = std::min(order[a], order[c]), hi = std::max(order[a], order[c]);
                out.push_back(((uint64_t)lo << 32) | hi);
            }
        }
    }
    std::sort(out.begin(), out.end());
    return out;
}

}  // namespace ncgo
