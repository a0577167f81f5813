// dtrt_gb300 — host orchestration of the vertex-position adjoint (dt_vadjoint.cuh).
//
// Per batch of camera paths: k_vadj_camera (value + frame-factor passes, edge records),
// [k_vadj_edge -> k_vadj_li]* in chunks, then k_vadj_chain (x0 gradient slots -> vertices).
// Primary edges: [k_vadj_primary -> k_vadj_li]*. The batch size bounds both the record
// queue (one record per path level) and the x0 slot buffer (3 floats per path level).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "dt_host.h"
#include "dt_vadjoint.cuh"

namespace dt {

#define DT_VCK(call)                                                                 \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return DTRT_ERR_CUDA;                                                    \
        }                                                                            \
    } while (0)

int vadjoint_supported(const dtrt_scene *s) {
    const DevScene &d = s->dev;
    if (d.num_media > 0) {
        set_last_error("the vertex-position adjoint needs a scene without participating media");
        return DTRT_ERR_UNSUPPORTED;
    }
    std::vector<DevShape> shapes(d.num_shapes);
    std::vector<DevEmitter> ems(d.num_emitters);
    if (cudaMemcpy(shapes.data(), d.shapes, sizeof(DevShape) * shapes.size(), cudaMemcpyDeviceToHost) != cudaSuccess ||
        (!ems.empty() && cudaMemcpy(ems.data(), d.emitters, sizeof(DevEmitter) * ems.size(), cudaMemcpyDeviceToHost) !=
                             cudaSuccess)) {
        set_last_error("vertex adjoint: scene readback failed");
        return DTRT_ERR_CUDA;
    }
    for (const DevShape &sh : shapes)
        if (sh.has_normals) {
            set_last_error("the vertex-position adjoint does not cover shapes with vertex normals");
            return DTRT_ERR_UNSUPPORTED;
        }
    for (const DevEmitter &e : ems)
        if (e.type != EMITTER_AREA) {
            set_last_error("the vertex-position adjoint covers AreaLight emitters only");
            return DTRT_ERR_UNSUPPORTED;
        }
    return DTRT_OK;
}

int render_vertex_adjoint(dtrt_scene *s, const dtrt_render_options *o, const float *d_image, float *image,
                          float *d_vertices, int on_device, cudaStream_t st) {
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    int rc = vadjoint_supported(s);
    if (rc) return rc;
    if (o->max_bounces < 0 || o->max_bounces + 1 > kVMaxLevels) {
        set_last_error("the vertex-position adjoint needs 0 <= max_bounces < 32");
        return DTRT_ERR_UNSUPPORTED;
    }
    DevScene sc = s->dev;
    Scratch &sb = s->scratch;
    const DevCamera &cam = sc.cam;
    const bool cropped = cam.crop_w > 0 && cam.crop_h > 0;
    RenderParams rp{};
    rp.seed = o->seed;
    rp.spp = o->spp;
    rp.max_bounces = o->max_bounces;
    rp.sppse = std::max(0, o->sppse);
    rp.inv_sppse = rp.sppse > 0 ? 1.0 / rp.sppse : 0.0;
    rp.mode = o->mode >= 0 ? o->mode : MODE_ALL;
    rp.jitter = o->sppe >= 0 ? 1 : 0;
    rp.ddist = o->ddist_coeff;
    rp.inv_spp = o->spp > 0 ? 1.0f / (float)o->spp : 0.f;
    rp.out_w = cropped ? cam.crop_w : cam.width;
    rp.out_h = cropped ? cam.crop_h : cam.height;
    rp.crop_x = cropped ? cam.crop_x : 0;
    rp.crop_y = cropped ? cam.crop_y : 0;
    rp.npix = rp.out_w * rp.out_h;
    const size_t npix = (size_t)rp.npix;
    // values only: no velocity inputs (the adjoint replaces the derivative slots)
    sc.vert_der = nullptr;
    sc.face_n_der = nullptr;
    sc.normal_der = nullptr;
    std::memset(sc.cam.d_cpos, 0, sizeof(sc.cam.d_cpos));
    std::memset(sc.cam.d_cframe, 0, sizeof(sc.cam.d_cframe));
    if (!sb.err) DT_VCK(cudaMalloc(&sb.err, sizeof(unsigned int)));
    if (!sb.counts) DT_VCK(cudaMalloc(&sb.counts, kCountSlots * sizeof(unsigned long long)));
    sc.error_flags = sb.err;
    DT_VCK(cudaMemsetAsync(sb.err, 0, sizeof(unsigned int), st));
    DT_VCK(cudaMemsetAsync(sb.counts, 0, kCountSlots * sizeof(unsigned long long), st));
    unsigned long long *ctr = s->counters ? sb.counts + 8 : nullptr;
    // ---------------------------------------------------------------- buffers
    const float *dimg = d_image;
    if (!on_device) {
        if (!ensure_buffer((void **)&sb.adj_dimg, &sb.adj_dimg_n, npix * 3 * 4)) return DTRT_ERR_CUDA;
        DT_VCK(cudaMemcpyAsync(sb.adj_dimg, d_image, npix * 3 * 4, cudaMemcpyHostToDevice, st));
        dimg = sb.adj_dimg;
    }
    const size_t nv3 = (size_t)sc.num_verts * 3;
    float *grad = d_vertices;
    if (!on_device) {
        if (!ensure_buffer((void **)&sb.adj_grad, &sb.adj_grad_n, std::max<size_t>(nv3, 1) * 4)) return DTRT_ERR_CUDA;
        grad = sb.adj_grad;
    }
    if (nv3) DT_VCK(cudaMemsetAsync(grad, 0, nv3 * 4, st));
    double *img_acc = nullptr;
    if (image) {
        if (!ensure_buffer((void **)&sb.adj_img, &sb.adj_img_n, npix * 3 * 8)) return DTRT_ERR_CUDA;
        img_acc = sb.adj_img;
        DT_VCK(cudaMemsetAsync(img_acc, 0, npix * 3 * 8, st));
    }
    const int levels = o->max_bounces + 1;
    const uint64_t li_cap = s->queue_cap ? s->queue_cap : (uint64_t)24 << 20;
    const uint64_t rec_cap = s->queue_cap ? s->queue_cap : (uint64_t)8 << 20;
    if (!ensure_buffer(&sb.qli, &sb.qli_bytes, li_cap * sizeof(VLiTask)) ||
        !ensure_buffer(&sb.qe, &sb.qe_bytes, rec_cap * sizeof(VEdgeRec)))
        return DTRT_ERR_CUDA;
    const long long total = (long long)npix * std::max(0, o->spp);
    long long B = std::max<long long>(128, (long long)(rec_cap / (uint64_t)levels));
    B = std::min<long long>(B, std::max<long long>(total, 1));
    float *xadj = nullptr;  // x0 gradient slots of one batch (held in the Lins queue buffer)
    if (!ensure_buffer(&sb.ql, &sb.ql_bytes, (size_t)B * levels * 3 * 4)) return DTRT_ERR_CUDA;
    xadj = (float *)sb.ql;
    Queue qe{sb.qe, sb.counts + 0, rec_cap}, qli{sb.qli, sb.counts + 2, li_cap};
    cudaEvent_t e0, e1;
    DT_VCK(cudaEventCreate(&e0));
    DT_VCK(cudaEventCreate(&e1));
    uint64_t launches = 0, tot_edge = 0, tot_li = 0, batches = 0;
    auto blocks = [](long long n) { return (unsigned)((n + kBlock - 1) / kBlock); };
    unsigned long long hcnt[3];
    auto read_counts = [&]() -> int {
        DT_VCK(cudaMemcpyAsync(hcnt, sb.counts, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        DT_VCK(cudaStreamSynchronize(st));
        return DTRT_OK;
    };
    const bool li_sorted = sc.num_nodes > 0 && ensure_li_sort(sb, li_cap);  // pairs by origin and direction
    auto drain_li = [&]() -> int {
        int r = read_counts();
        if (r) return r;
        const unsigned long long n = std::min<unsigned long long>(hcnt[2], li_cap);
        tot_li += n;
        if (n) {
            const int *perm =
                li_sorted ? sort_li_pairs(sc, (const VLiTask *)qli.data, (long long)n, sb, li_cap, st, launches)
                          : nullptr;
            k_vadj_li<<<blocks((long long)n), kBlock, 0, st>>>(sc, rp, qli, (long long)n, dimg, grad, xadj, perm,
                                                               ctr);
            ++launches;
            DT_VCK(cudaGetLastError());
        }
        DT_VCK(cudaMemsetAsync(sb.counts + 2, 0, sizeof(unsigned long long), st));
        return DTRT_OK;
    };
    DT_VCK(cudaEventRecord(e0, st));
    const long long per_chunk = std::max<long long>(1, (long long)(li_cap / (uint64_t)std::max(1, 2 * rp.sppse)));
    for (long long b0 = 0; b0 < total; b0 += B) {
        ++batches;
        rp.path_begin = b0;
        rp.path_count = std::min(B, total - b0);
        DT_VCK(cudaMemsetAsync(sb.counts, 0, 3 * sizeof(unsigned long long), st));
        DT_VCK(cudaMemsetAsync(xadj, 0, (size_t)rp.path_count * levels * 3 * 4, st));
        k_vadj_camera<<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, dimg, grad, qe, img_acc, levels, ctr);
        ++launches;
        DT_VCK(cudaGetLastError());
        if ((rc = read_counts())) return rc;
        const unsigned long long ne = std::min<unsigned long long>(hcnt[0], rec_cap);
        tot_edge += ne;
        for (unsigned long long r0 = 0; r0 < ne && rp.sppse > 0; r0 += per_chunk) {
            const long long cnt = (long long)std::min<unsigned long long>(per_chunk, ne - r0);
            k_vadj_edge<<<blocks(cnt * rp.sppse), kBlock, 0, st>>>(sc, rp, qe, (long long)r0, cnt, qli, ctr);
            ++launches;
            DT_VCK(cudaGetLastError());
            if ((rc = drain_li())) return rc;
        }
        if (ne > 0) {
            k_vadj_chain<<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, grad, xadj, levels, ctr);
            ++launches;
            DT_VCK(cudaGetLastError());
        }
    }
    uint64_t prim_samples = 0;
    if (o->sppe > 0 && sc.num_pedges > 0) {
        const long long nblock = (long long)std::ceil(sc.pedge_sum * o->sppe / 128.0);
        const long long ns = nblock * 128;
        prim_samples = (uint64_t)ns;
        rp.prim_weight = sc.pedge_sum / (double)ns;
        const long long chunk = std::max<long long>(1, (long long)(li_cap / 2));
        for (long long k0 = 0; k0 < ns; k0 += chunk) {
            rp.prim_begin = k0;
            rp.prim_count = std::min(chunk, ns - k0);
            const int *perm = li_sorted ? sort_primary_samples(rp, sb, li_cap, st, launches) : nullptr;
            k_vadj_primary<<<blocks(rp.prim_count), kBlock, 0, st>>>(sc, rp, qli, perm, ctr);
            ++launches;
            DT_VCK(cudaGetLastError());
            if ((rc = drain_li())) return rc;
        }
    }
    DT_VCK(cudaEventRecord(e1, st));
    if (image) {
        float *dst = image;
        if (!on_device) {
            if (!ensure_buffer((void **)&sb.adj_out, &sb.adj_out_n, npix * 3 * 4)) return DTRT_ERR_CUDA;
            dst = sb.adj_out;
        }
        k_adjoint_image<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(rp.npix, img_acc, dst);
        ++launches;
        DT_VCK(cudaGetLastError());
        if (!on_device) DT_VCK(cudaMemcpyAsync(image, sb.adj_out, npix * 3 * 4, cudaMemcpyDeviceToHost, st));
    }
    if (!on_device && nv3) DT_VCK(cudaMemcpyAsync(d_vertices, grad, nv3 * 4, cudaMemcpyDeviceToHost, st));
    unsigned int herr = 0;
    DT_VCK(cudaMemcpyAsync(&herr, sb.err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    DT_VCK(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dtrt_render_stats &ls = s->last;
    std::memset(&ls, 0, sizeof(ls));
    ls.camera_paths = (uint64_t)total;
    ls.edge_records = tot_edge;
    ls.li_tasks = tot_li;
    ls.primary_edge_samples = prim_samples;
    ls.batches = batches;
    ls.kernel_launches = launches;
    ls.ms_camera = ms;
    ls.ms_total = std::chrono::duration<double, std::milli>(clk::now() - t_start).count();
    if (herr & ERR_QUEUE) {
        set_last_error("work queue overflow (capacity below one camera path's worst case)");
        return DTRT_ERR_OVERFLOW;
    }
    if (herr & ERR_STACK) {
        set_last_error("BVH traversal stack overflow");
        return DTRT_ERR_INVALID;
    }
    if (herr & ERR_TRACK_CAP) {
        set_last_error("a delta/ratio tracking loop hit its iteration cap");
        return DTRT_ERR_STEP_CAP;
    }
    return DTRT_OK;
}

}  // namespace dt
