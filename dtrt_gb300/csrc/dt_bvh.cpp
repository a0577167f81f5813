// dtrt_gb300 — binned-SAH BVH build on the host (see dt_bvh.h).
#include "dt_bvh.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace dt {
namespace {

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const float *p) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
    }
    void grow(const Box &b) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
    }
    float area() const {
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = std::max(0.f, hi[a] - lo[a]);
        return 2.f * (d[0] * d[1] + d[0] * d[2] + d[1] * d[2]);
    }
};

// child code of a leaf: ~((first triangle << 3) | (count - 1))
inline void leaf_range(int code, int &base, int &count) {
    const int v = ~code;
    base = v >> 3;
    count = (v & 7) + 1;
}

struct Builder {
    const std::vector<float> &tv;
    std::vector<int> order;
    std::vector<Box> tbox;
    std::vector<float> cen;  // 3 per triangle
    BvhBuildOut &out;
    static constexpr int kBins = 16, kLeafMax = 8, kLeafPref = 4, kDepthCap = kStackDepth - 2;

    Builder(const std::vector<float> &t, int n, BvhBuildOut &o) : tv(t), order(n), tbox(n), cen(3 * n), out(o) {
        for (int i = 0; i < n; ++i) {
            order[i] = i;
            for (int k = 0; k < 3; ++k) tbox[i].grow(&tv[9 * i + 3 * k]);
            for (int a = 0; a < 3; ++a) cen[3 * i + a] = 0.5f * (tbox[i].lo[a] + tbox[i].hi[a]);
        }
    }

    int make_leaf(int first, int count) {
        const int base = (int)out.leaf_tris.size() / 3;
        for (int i = first; i < first + count; ++i) {
            const int t = order[i];
            const float *v = &tv[9 * t];
            float4 a = make_float4(v[0], v[1], v[2], 0.f);
            int tid = t;
            std::memcpy(&a.w, &tid, 4);
            out.leaf_tris.push_back(a);
            out.leaf_tris.push_back(make_float4(v[3] - v[0], v[4] - v[1], v[5] - v[2], 0.f));
            out.leaf_tris.push_back(make_float4(v[6] - v[0], v[7] - v[1], v[8] - v[2], 0.f));
        }
        return ~((base << 3) | (count - 1));
    }

    // returns the child code of the subtree over order[first, first+count) and its box
    int build(int first, int count, int depth, Box &box) {
        box = Box();
        Box cb;
        for (int i = first; i < first + count; ++i) {
            box.grow(tbox[order[i]]);
            cb.grow(&cen[3 * order[i]]);
        }
        out.max_depth = std::max(out.max_depth, depth);
        if (count <= kLeafPref || (depth >= kDepthCap && count <= kLeafMax)) return make_leaf(first, count);
        // binned SAH over the centroid bounds: one pass bins all three axes
        int best_axis = -1, best_split = -1;
        float best_cost = FLT_MAX;
        Box bins[3][kBins];
        int counts[3][kBins] = {{0}};
        float kb[3];
        bool axis_ok[3];
        for (int a = 0; a < 3; ++a) {
            const float ext = cb.hi[a] - cb.lo[a];
            axis_ok[a] = ext > 0.f;
            kb[a] = axis_ok[a] ? kBins / ext : 0.f;
        }
        for (int i = first; i < first + count; ++i) {
            const int t = order[i];
            const Box &tb = tbox[t];
            const float *c = &cen[3 * t];
            for (int a = 0; a < 3; ++a) {
                if (!axis_ok[a]) continue;
                const int b = std::min(kBins - 1, (int)((c[a] - cb.lo[a]) * kb[a]));
                counts[a][b]++;
                bins[a][b].grow(tb);
            }
        }
        for (int a = 0; a < 3; ++a) {
            if (!axis_ok[a]) continue;
            const Box *bb = bins[a];
            const int *bc = counts[a];
            Box lb[kBins], rb[kBins];
            int lc[kBins], rc[kBins];
            Box acc;
            int n = 0;
            for (int b = 0; b < kBins; ++b) { acc.grow(bb[b]); n += bc[b]; lb[b] = acc; lc[b] = n; }
            acc = Box();
            n = 0;
            for (int b = kBins - 1; b >= 0; --b) { acc.grow(bb[b]); n += bc[b]; rb[b] = acc; rc[b] = n; }
            for (int s = 0; s < kBins - 1; ++s) {
                if (lc[s] == 0 || rc[s + 1] == 0) continue;
                const float cost = lc[s] * lb[s].area() + rc[s + 1] * rb[s + 1].area();
                if (cost < best_cost) { best_cost = cost; best_axis = a; best_split = s; }
            }
        }
        int mid;
        if (best_axis >= 0) {
            const float leaf_cost = count * box.area();
            if (count <= kLeafMax && best_cost >= leaf_cost) return make_leaf(first, count);
            const float k = kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
            auto it = std::partition(order.begin() + first, order.begin() + first + count, [&](int t) {
                return std::min(kBins - 1, (int)((cen[3 * t + best_axis] - cb.lo[best_axis]) * k)) <= best_split;
            });
            mid = (int)(it - order.begin());
        } else {
            mid = first;  // all centroids coincide
        }
        if (mid == first || mid == first + count) {
            if (count <= kLeafMax) return make_leaf(first, count);
            mid = first + count / 2;  // median split of coincident centroids
        }
        const int idx = (int)out.nodes.size();
        out.nodes.push_back(BvhNode());
        Box lbx, rbx;
        const int lcode = build(first, mid - first, depth + 1, lbx);
        const int rcode = build(mid, first + count - mid, depth + 1, rbx);
        BvhNode &nd = out.nodes[idx];
        nd.x = make_float4(lbx.lo[0], lbx.hi[0], rbx.lo[0], rbx.hi[0]);
        nd.y = make_float4(lbx.lo[1], lbx.hi[1], rbx.lo[1], rbx.hi[1]);
        nd.z = make_float4(lbx.lo[2], lbx.hi[2], rbx.lo[2], rbx.hi[2]);
        nd.child = make_int4(lcode, rcode, 0, 0);
        return idx;
    }
};

}  // namespace

void build_bvh(const std::vector<float> &tri_verts, int num_tris, BvhBuildOut &out) {
    out.nodes.clear();
    out.leaf_tris.clear();
    out.max_depth = 0;
    if (num_tris <= 0) return;
    Builder b(tri_verts, num_tris, out);
    Box box;
    const int code = b.build(0, num_tris, 1, box);
    if (code < 0) {
        // the whole scene is one leaf: a root whose two children are that leaf (a
        // duplicate test of the same triangles cannot change the closest hit)
        BvhNode nd;
        nd.x = make_float4(box.lo[0], box.hi[0], box.lo[0], box.hi[0]);
        nd.y = make_float4(box.lo[1], box.hi[1], box.lo[1], box.hi[1]);
        nd.z = make_float4(box.lo[2], box.hi[2], box.lo[2], box.hi[2]);
        nd.child = make_int4(code, code, 0, 0);
        out.nodes.insert(out.nodes.begin(), nd);
    }
}

void refit_bvh(const std::vector<float> &tri_verts, BvhBuildOut &tree) {
    const int n = (int)tree.nodes.size();
    std::vector<Box> nbox(n);
    for (int i = n - 1; i >= 0; --i) {
        BvhNode &nd = tree.nodes[i];
        const int codes[2] = {nd.child.x, nd.child.y};
        Box cb[2];
        for (int c = 0; c < 2; ++c) {
            if (codes[c] >= 0) {
                cb[c] = nbox[codes[c]];
                continue;
            }
            int base, count;
            leaf_range(codes[c], base, count);
            for (int k = base; k < base + count; ++k) {
                float4 &a = tree.leaf_tris[3 * (size_t)k];
                int t;
                std::memcpy(&t, &a.w, 4);
                const float *v = &tri_verts[9 * (size_t)t];
                for (int q = 0; q < 3; ++q) cb[c].grow(v + 3 * q);
                a.x = v[0]; a.y = v[1]; a.z = v[2];
                tree.leaf_tris[3 * (size_t)k + 1] = make_float4(v[3] - v[0], v[4] - v[1], v[5] - v[2], 0.f);
                tree.leaf_tris[3 * (size_t)k + 2] = make_float4(v[6] - v[0], v[7] - v[1], v[8] - v[2], 0.f);
            }
        }
        nd.x = make_float4(cb[0].lo[0], cb[0].hi[0], cb[1].lo[0], cb[1].hi[0]);
        nd.y = make_float4(cb[0].lo[1], cb[0].hi[1], cb[1].lo[1], cb[1].hi[1]);
        nd.z = make_float4(cb[0].lo[2], cb[0].hi[2], cb[1].lo[2], cb[1].hi[2]);
        nbox[i] = cb[0];
        nbox[i].grow(cb[1]);
    }
}

double bvh_sah_cost(const BvhBuildOut &tree) {
    if (tree.nodes.empty()) return 0.0;
    double inner = 0.0, leaves = 0.0, root = 0.0;
    for (size_t i = 0; i < tree.nodes.size(); ++i) {
        const BvhNode &nd = tree.nodes[i];
        Box cb[2];
        const float lo[2][3] = {{nd.x.x, nd.y.x, nd.z.x}, {nd.x.z, nd.y.z, nd.z.z}};
        const float hi[2][3] = {{nd.x.y, nd.y.y, nd.z.y}, {nd.x.w, nd.y.w, nd.z.w}};
        Box u;
        for (int c = 0; c < 2; ++c) {
            cb[c].grow(lo[c]);
            cb[c].grow(hi[c]);
            u.grow(cb[c]);
        }
        const double a = u.area();
        if (i == 0) root = a;
        inner += a;
        const int codes[2] = {nd.child.x, nd.child.y};
        for (int c = 0; c < 2; ++c)
            if (codes[c] < 0) {
                int base, count;
                leaf_range(codes[c], base, count);
                leaves += (double)count * cb[c].area();
            }
    }
    return root > 0.0 ? (inner + leaves) / root : 0.0;
}

}  // namespace dt
