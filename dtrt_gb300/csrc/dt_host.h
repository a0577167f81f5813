// dtrt_gb300 — host-side scene object and the per-width render entry points.
#pragma once
#include <string>
#include <vector>

#include "../../include/dtrt_gb300.h"
#include "dt_bvh.h"
#include "dt_kernels.cuh"

namespace dt {

void set_last_error(const std::string &msg);

// Device buffers reused across renders of one scene, grown on demand.
struct Scratch {
    double *acc1 = nullptr, *acc2 = nullptr;
    size_t acc1_n = 0, acc2_n = 0;
    float *out = nullptr;
    size_t out_n = 0;
    void *qe = nullptr, *ql = nullptr, *qli = nullptr;
    size_t qe_bytes = 0, ql_bytes = 0, qli_bytes = 0;
    unsigned long long *counts = nullptr;  // [0] edge recs, [1] lins recs, [2] li tasks, [8..] counters
    unsigned int *err = nullptr;
    // adjoint render: dL/dI staging, density gradient, FP64 image accumulator, image staging
    float *adj_dimg = nullptr, *adj_grad = nullptr, *adj_out = nullptr;
    double *adj_img = nullptr;
    size_t adj_dimg_n = 0, adj_grad_n = 0, adj_out_n = 0, adj_img_n = 0;
    // wavefront schedules: path states and vertex inputs, four path-index queues, per-level counts
    void *cam_state = nullptr, *cam_q = nullptr, *cam_cnt = nullptr;
    size_t cam_state_bytes = 0, cam_q_bytes = 0, cam_cnt_bytes = 0;
    // sort of the Li sub-path pairs: keys, values, their double buffers and digit counts
    void *li_sort = nullptr;
    size_t li_sort_bytes = 0;

};

bool ensure_buffer(void **ptr, size_t *have, size_t need);

// Buffers of the Li pair sort for queues of li_cap tasks (li_cap / 2 pairs): false (and
// the allocation error cleared) when the device has no room, the Li kernels then read the
// queue in order.
inline bool ensure_li_sort(Scratch &sb, uint64_t li_cap) {
    const long long cap = (long long)(li_cap / 2);
    if (ensure_buffer(&sb.li_sort, &sb.li_sort_bytes, (size_t)cap * 16 + radix_hist_entries(cap) * 4)) return true;
    cudaGetLastError();
    return false;
}

// The n queued Li tasks' pairs (slots 2m, 2m + 1) in key order (k_li_keys) on stream st;
// nullptr when n is odd or holds one pair (the queue is then read in order). Adds the
// kernels it launches to `launches`.
template <class Task>
const int *sort_li_pairs(const DevScene &sc, const Task *tasks, long long n, Scratch &sb, uint64_t li_cap,
                         cudaStream_t st, uint64_t &launches) {
    const long long np = n / 2, cap = (long long)(li_cap / 2);
    if ((n & 1) || np < 2 || np > cap) return nullptr;
    unsigned *keys = (unsigned *)sb.li_sort, *keys2 = keys + cap;
    int *vals = (int *)(keys2 + cap), *vals2 = vals + cap;
    unsigned *hist = (unsigned *)(vals2 + cap);
    k_li_keys<Task><<<(unsigned)((np + 255) / 256), 256, 0, st>>>(sc, tasks, np, keys, vals);
    launches += 1 + radix_sort_launches(kLiSortKeyBits);
    return radix_sort_bits(keys, vals, keys2, vals2, hist, (int)np, kLiSortKeyBits, st);
}

// The primary-edge samples [rp.prim_begin, + rp.prim_count) in key order (k_primary_keys),
// in the Li sort's buffers (a chunk holds at most li_cap / 2 samples); nullptr for one.
// Adds the kernels it launches to `launches`.
inline const int *sort_primary_samples(const RenderParams &rp, Scratch &sb, uint64_t li_cap, cudaStream_t st,
                                       uint64_t &launches) {
    const long long cap = (long long)(li_cap / 2);
    if (rp.prim_count < 2 || rp.prim_count > cap) return nullptr;
    unsigned *keys = (unsigned *)sb.li_sort, *keys2 = keys + cap;
    int *vals = (int *)(keys2 + cap), *vals2 = vals + cap;
    unsigned *hist = (unsigned *)(vals2 + cap);
    k_primary_keys<<<(unsigned)((rp.prim_count + 255) / 256), 256, 0, st>>>(rp, keys, vals);
    launches += 1 + radix_sort_launches(20);
    return radix_sort_bits(keys, vals, keys2, vals2, hist, (int)rp.prim_count, 20, st);
}


// Connectivity kept from the last build, so that a rebuild from a description with the
// same triangles (an optimisation step that moves vertices) skips the edge search and
// refits the BVH instead of building it again.
struct SceneTopology {
    bool valid = false;
    std::vector<int> shape_nv, shape_nt;
    std::vector<int> indices;                // every shape's triangles, shape-local vertex ids
    std::vector<int4> adj;                   // per shape: (a, b, f0, f1 or -1), shape-local, sorted by (a, b)
    std::vector<int> adj_off;                // num_shapes + 1 offsets into adj
    std::vector<int> media_type, media_res;  // per medium: type; density resolution (3 ints)
    BvhBuildOut bvh;                         // the tree as last built or refit (host builds)
    double sah_build = 0.0;                  // its surface-area cost right after the last full build
};

// Process-wide choice of the BVH builder for scenes created or updated afterwards.
int bvh_builder_setting();

}  // namespace dt

struct dtrt_scene {
    int nder = 0;
    int device = 0;
    dt::DevScene dev{};
    std::vector<void *> allocs;       // scene-lifetime device allocations, one per upload (null: empty)
    std::vector<size_t> alloc_bytes;  // byte size of each entry of allocs
    dt::Scratch scratch;
    bool counters = false;
    uint64_t queue_cap = 0;  // 0: automatic
    int camera_schedule = 0;  // DTRT_CAMERA_AUTO / _MEGAKERNEL / _WAVEFRONT
    dtrt_render_stats last{};
    int num_shapes = 0;
    std::vector<float> shape_edge_len;  // per shape total edge length (for re-weighting)
    std::vector<int> shape_skip;        // null-BSDF shapes without emitter
    std::vector<dt::DevMedium> media_host;  // host copy of the device media array
    std::vector<void *> dgrid_bufs;         // per medium: per-voxel derivative directions (owned)
    long long density_voxels = 0;           // voxels of all heterogeneous media (adjoint gradient length)
    dt::SceneTopology topo;
    dtrt_bvh_info bvh_info{};               // how the current tree was made
};

namespace dt {
template <int N>
int render_n(dtrt_scene *s, const dtrt_render_options *o, float *out, int out_on_device, cudaStream_t stream);
int render_adjoint(dtrt_scene *s, const dtrt_render_options *o, const float *d_image, float *image, float *d_density,
                   int on_device, cudaStream_t stream);
cudaError_t launch_adjoint(const DevScene &sc, const RenderParams &rp, const float *dimg, float *grad, double *img_acc,
                           unsigned long long *ctr, long long stride, cudaStream_t st);
// Device workspace of the wavefront density replay: path states, vertex inputs, four path-index queues,
// pass-A values and event values for `cap` paths, level counts of both passes.
struct AdjWave {
    void *states = nullptr, *vins = nullptr;
    int *q = nullptr;
    float3 *tots = nullptr, *ev = nullptr;
    unsigned long long *cnt = nullptr;
    long long cap = 0;
    int levels = 0;
    static size_t bytes(long long cap, int levels);
    void carve(void *base, long long cap, int levels);  // lay the arrays out in one allocation
};
cudaError_t launch_adjoint_wave(const DevScene &sc, const RenderParams &range, const float *dimg, float *grad,
                                double *img_acc, unsigned long long *ctr, const AdjWave &w, int sms, cudaStream_t st,
                                uint64_t *launches);
int render_vertex_adjoint(dtrt_scene *s, const dtrt_render_options *o, const float *d_image, float *image,
                          float *d_vertices, int on_device, cudaStream_t stream);
template <int N>
int render_n_noalloc(dtrt_scene *s, const dtrt_render_options *o, float *out, int out_on_device, cudaStream_t stream,
                     unsigned char *scratch, size_t scratch_bytes);
}  // namespace dt
