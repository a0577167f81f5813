// dtrt_gb300 — host BVH builder (binned SAH, 2-wide nodes, leaves of <= 8 triangles).
// Replaces the Embree scene build of the reference (src/scene.cpp:17-43).
#pragma once
#include <cstdint>
#include <string>
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

// A tree built on the device (dt_bvh_build.cu): device allocations owned by the caller.
struct DeviceBvh {
    BvhNode *nodes = nullptr;
    float4 *leaf_tris = nullptr;
    int num_nodes = 0;
    size_t leaf_tris_bytes = 0;
    int max_depth = 0;  // of the uncollapsed binary tree (bounds the traversal stack)
};

// Linear BVH of the triangles on the current device, in the layout build_bvh writes
// (2-wide nodes, leaves of <= 4 triangles, (v0, id) (e1) (e2) records in leaf order).
// Returns 0 on success; 1 for fewer than two triangles; 2 on a CUDA error (message in
// err); 3 when the tree is deeper than the traversal stack allows (nothing allocated:
// build on the host instead).
int build_bvh_device(const std::vector<float> &tri_verts, int num_tris, DeviceBvh &out, std::string &err);

// Stable sort of n (key, value) pairs by the low `bits` bits of the key on stream st (8-bit
// LSD passes of the BVH build's radix sort). keys2 / vals2 hold n entries, hist
// radix_hist_entries(n). Returns the values in key order: vals after an even number of
// passes, vals2 after an odd one.
size_t radix_hist_entries(long long n);
// kernel launches of one radix_sort_bits call (4 per pass)
int radix_sort_launches(int bits);
int *radix_sort_bits(unsigned *keys, int *vals, unsigned *keys2, int *vals2, unsigned *hist, int n, int bits,
                     cudaStream_t st);

}  // namespace dt
