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

// Refit a tree from build_bvh to new positions of the same triangles: the topology and
// the leaf order stay, every child box and leaf triangle is recomputed bottom-up. Nodes
// are in depth-first pre-order (a child's index is above its parent's), so one reverse
// sweep visits every child before its parent. Refitting to the positions a tree was built
// from reproduces it bit for bit.
void refit_bvh(const std::vector<float> &tri_verts, BvhBuildOut &tree);

// Surface-area cost of a tree relative to its root box: the sum over inner nodes of
// area(node) plus, over leaves, triangles x area(leaf), all divided by area(root). A refit
// tree whose cost grows well past its cost at build time traverses slowly and is rebuilt.
double bvh_sah_cost(const BvhBuildOut &tree);

}  // namespace dt
