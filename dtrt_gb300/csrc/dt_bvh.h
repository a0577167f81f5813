// dtrt_gb300 — host BVH builder (binned SAH, 2-wide nodes, leaves of <= 8 triangles).
// Replaces the Embree scene build of the reference (src/scene.cpp:17-43).
#pragma once
#include <cstdint>
#include <vector>

#include "dt_scene.h"

namespace dt {

struct BvhBuildOut {
    std::vector<BvhNode> nodes;
    std::vector<float4> leaf_tris;  // 3 per triangle: (v0, id) (e1, 0) (e2, 0)
    int max_depth = 0;
};

// tri_verts: [num_tris][3] vertex positions (xyz). Triangle ids are their index.
void build_bvh(const std::vector<float> &tri_verts, int num_tris, BvhBuildOut &out);

}  // namespace dt
