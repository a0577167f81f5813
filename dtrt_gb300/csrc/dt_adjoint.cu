// dtrt_gb300 — host orchestration of the reverse-mode density adjoint (k_adjoint).
//
// The replay runs with derivative width 1 whatever the scene's nder: the adjoint needs the
// path values only, and the per-voxel gradient replaces the derivative slots. The scene
// copy given to the kernel drops every velocity input so the dual slot stays zero and the
// no-derivative fast paths apply; values and random decisions are those of dtrt_render_fwd.
#include <algorithm>
#include <chrono>
#include <cstring>

#include "dt_adjoint.cuh"
#include "dt_host.h"

namespace dt {

#define DT_ACK(call)                                                                 \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return DTRT_ERR_CUDA;                                                    \
        }                                                                            \
    } while (0)

// one replay launch (shared with the batch schedules, so every caller runs this unit's
// compilation of the kernel)
cudaError_t launch_adjoint(const DevScene &sc, const RenderParams &rp, const float *dimg, float *grad, double *img_acc,
                           unsigned long long *ctr, long long stride, cudaStream_t st) {
    const long long n = (rp.path_count + stride - 1) / stride;
    if (n <= 0) return cudaSuccess;
    k_adjoint<1><<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, st>>>(sc, rp, dimg, grad, img_acc, ctr, stride);
    return cudaGetLastError();
}

size_t AdjWave::bytes(long long cap, int levels) {
    return (size_t)cap * (sizeof(AdjState<1>) + sizeof(VertexIn<1>) + 4 * sizeof(int) + sizeof(float3) +
                          kReplayEvents * sizeof(float3)) +
           (size_t)6 * (levels + 1) * sizeof(unsigned long long) + 2048;  // + 256-byte alignment of 6 arrays
}

void AdjWave::carve(void *base, long long capacity, int lv) {
    char *p = (char *)base;
    auto take = [&](size_t n) {
        void *r = p;
        p += (n + 255) & ~(size_t)255;
        return r;
    };
    cap = capacity;
    levels = lv;
    states = take((size_t)cap * sizeof(AdjState<1>));
    vins = take((size_t)cap * sizeof(VertexIn<1>));
    q = (int *)take((size_t)4 * cap * sizeof(int));
    tots = (float3 *)take((size_t)cap * sizeof(float3));
    ev = (float3 *)take((size_t)cap * kReplayEvents * sizeof(float3));
    cnt = (unsigned long long *)take((size_t)6 * (levels + 1) * sizeof(unsigned long long));
}

// Wavefront replay of paths [rp.path_begin, +rp.path_count) in chunks of the workspace's
// capacity: pass A (values, image) then, with a gradient, pass B (scatter); each pass is
// a start launch, one launch per vertex level over the live paths, (A) a totals launch.
cudaError_t launch_adjoint_wave(const DevScene &sc, const RenderParams &range, const float *dimg, float *grad,
                                double *img_acc, unsigned long long *ctr, const AdjWave &w, int sms, cudaStream_t st,
                                uint64_t *launches) {
    const int levels = range.max_bounces + 1;
    if (levels > w.levels) return cudaErrorInvalidValue;
    auto blocks = [](long long n) { return (unsigned)((n + kBlock - 1) / kBlock); };
    AdjState<1> *states = (AdjState<1> *)w.states;
    VertexIn<1> *vins = (VertexIn<1> *)w.vins;
    int *qa = w.q, *qb = qa + w.cap, *qv = qb + w.cap, *qs = qv + w.cap;
    const bool pass_b = grad != nullptr && dimg != nullptr;
    RenderParams rp = range;
    for (long long b0 = 0; b0 < range.path_count; b0 += w.cap) {
        rp.path_begin = range.path_begin + b0;
        rp.path_count = std::min(w.cap, range.path_count - b0);
        const unsigned gw = std::min<unsigned>(blocks(rp.path_count), (unsigned)std::max(1, sms) * 16u);
        cudaError_t e = cudaMemsetAsync(w.cnt, 0, (size_t)6 * (levels + 1) * sizeof(unsigned long long), st);
        if (e != cudaSuccess) return e;
        for (int pass = 0; pass < (pass_b ? 2 : 1); ++pass) {
            const bool b = pass == 1;
            // counts of this pass per level [0, levels]: volume vertices, interface vertices
            // pushed from the front and from the back of their queue (3 (levels + 1) per pass)
            unsigned long long *vc = w.cnt + pass * 3 * (levels + 1), *sc_ = vc + (levels + 1);
            const QueueEnds qx{w.cap, levels + 1};
            // volume / interface queues of level L: (qa, qb) for even L, (qv, qs) for odd L
            k_adj_start<1><<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, states, vins, qa, vc, qv, vc + 1, qs,
                                                                    sc_ + 1, dimg, grad, w.tots, w.ev, qx, b, ctr);
            for (int L = 0; L < levels; ++L) {
                int *qvl = (L & 1) ? qv : qa, *qsl = (L & 1) ? qs : qb;
                int *qvn = (L & 1) ? qa : qv, *qsn = (L & 1) ? qb : qs;
                k_adj_vertex<1, true><<<gw, kBlock, 0, st>>>(sc, rp, states, vins, qvl, vc + L, qvn, vc + L + 1, qsn,
                                                            sc_ + L + 1, dimg, grad, w.tots, w.ev, qx, b, ctr);
                if (L > 0)  // level 0's interface vertices ran in k_adj_start
                    k_adj_vertex<1, false><<<gw, kBlock, 0, st>>>(sc, rp, states, vins, qsl, sc_ + L, qvn, vc + L + 1,
                                                                 qsn, sc_ + L + 1, dimg, grad, w.tots, w.ev, qx, b,
                                                                 ctr);
            }
            if (pass == 0) k_adj_totals<1><<<blocks(rp.path_count), kBlock, 0, st>>>(rp, states, w.tots, img_acc);
            if (launches) *launches += 2 * levels + (pass == 0 ? 1 : 0);  // start, 2 per level (1 at level 0), totals in pass A
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int render_adjoint(dtrt_scene *s, const dtrt_render_options *o, const float *d_image, float *image, float *d_density,
                   int on_device, cudaStream_t st) {
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    DevScene sc = s->dev;
    Scratch &sb = s->scratch;
    const DevCamera &cam = sc.cam;
    const bool cropped = cam.crop_w > 0 && cam.crop_h > 0;
    if (o->max_bounces < 0) {
        set_last_error("max_bounces must be >= 0");
        return DTRT_ERR_INVALID;
    }
    RenderParams rp{};
    rp.seed = o->seed;
    rp.spp = o->spp;
    rp.max_bounces = o->max_bounces;
    rp.sppse = 0;  // boundary terms carry no density derivative
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
    // values only: no velocity inputs
    sc.vert_der = nullptr;
    sc.face_n_der = nullptr;
    sc.normal_der = nullptr;
    sc.moving_geometry = 0;
    std::memset(sc.cam.d_cpos, 0, sizeof(sc.cam.d_cpos));
    std::memset(sc.cam.d_cframe, 0, sizeof(sc.cam.d_cframe));
    if (!sb.err) DT_ACK(cudaMalloc(&sb.err, sizeof(unsigned int)));
    if (!sb.counts) DT_ACK(cudaMalloc(&sb.counts, kCountSlots * sizeof(unsigned long long)));
    sc.error_flags = sb.err;
    DT_ACK(cudaMemsetAsync(sb.err, 0, sizeof(unsigned int), st));
    DT_ACK(cudaMemsetAsync(sb.counts, 0, kCountSlots * sizeof(unsigned long long), st));
    unsigned long long *ctr = s->counters ? sb.counts + 8 : nullptr;
    // ---------------------------------------------------------------- inputs and outputs
    const float *dimg = nullptr;
    if (d_image) {
        if (on_device) {
            dimg = d_image;
        } else {
            if (!ensure_buffer((void **)&sb.adj_dimg, &sb.adj_dimg_n, npix * 3 * 4)) return DTRT_ERR_CUDA;
            DT_ACK(cudaMemcpyAsync(sb.adj_dimg, d_image, npix * 3 * 4, cudaMemcpyHostToDevice, st));
            dimg = sb.adj_dimg;
        }
    }
    const size_t nvox = (size_t)s->density_voxels;
    float *grad = nullptr;
    if (d_density && nvox > 0) {
        if (on_device) {
            grad = d_density;
        } else {
            if (!ensure_buffer((void **)&sb.adj_grad, &sb.adj_grad_n, nvox * 4)) return DTRT_ERR_CUDA;
            grad = sb.adj_grad;
        }
        DT_ACK(cudaMemsetAsync(grad, 0, nvox * 4, st));
    }
    double *img_acc = nullptr;
    if (image) {
        if (!ensure_buffer((void **)&sb.adj_img, &sb.adj_img_n, npix * 3 * 8)) return DTRT_ERR_CUDA;
        img_acc = sb.adj_img;
        DT_ACK(cudaMemsetAsync(img_acc, 0, npix * 3 * 8, st));
    }
    // ---------------------------------------------------------------- replay
    cudaEvent_t e0, e1;
    DT_ACK(cudaEventCreate(&e0));
    DT_ACK(cudaEventCreate(&e1));
    const long long total = (long long)npix * std::max(0, o->spp);
    uint64_t launches = 0;
    float ms_replay = 0.f;
    DT_ACK(cudaEventRecord(e0, st));
    // schedule: the wavefront (pass A and pass B each one launch per vertex over the live
    // paths) for large renders, as dtrt_render_fwd's camera schedule
    const long long B = 1ll << 24;  // paths per megakernel launch
    bool wavefront = s->camera_schedule == DTRT_CAMERA_WAVEFRONT ||
                     (s->camera_schedule == DTRT_CAMERA_AUTO && total >= kWavefrontMinPaths);
    AdjWave w{};
    if (wavefront) {
        const long long cap = std::min<long long>(1ll << 22, std::max<long long>(total, 1));
        if (ensure_buffer(&sb.cam_state, &sb.cam_state_bytes, AdjWave::bytes(cap, o->max_bounces + 1))) {
            w.carve(sb.cam_state, cap, o->max_bounces + 1);
        } else {
            if (s->camera_schedule == DTRT_CAMERA_WAVEFRONT) return DTRT_ERR_CUDA;
            cudaGetLastError();  // AUTO: no room for the path states, run the megakernel
            wavefront = false;
        }
    }
    if (wavefront) {
        int sms = 0;
        DT_ACK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
        rp.path_begin = 0;
        rp.path_count = total;
        DT_ACK(launch_adjoint_wave(sc, rp, dimg, grad, img_acc, ctr, w, sms, st, &launches));
    } else {
        for (long long b0 = 0; b0 < total; b0 += B) {
            rp.path_begin = b0;
            rp.path_count = std::min(B, total - b0);
            DT_ACK(launch_adjoint(sc, rp, dimg, grad, img_acc, ctr, 1, st));
            ++launches;
        }
    }
    DT_ACK(cudaEventRecord(e1, st));
    if (image) {
        float *dst = image;
        if (!on_device) {
            if (!ensure_buffer((void **)&sb.adj_out, &sb.adj_out_n, npix * 3 * 4)) return DTRT_ERR_CUDA;
            dst = sb.adj_out;
        }
        k_adjoint_image<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(rp.npix, img_acc, dst);
        ++launches;
        DT_ACK(cudaGetLastError());
        if (!on_device) DT_ACK(cudaMemcpyAsync(image, sb.adj_out, npix * 3 * 4, cudaMemcpyDeviceToHost, st));
    }
    if (grad && !on_device) DT_ACK(cudaMemcpyAsync(d_density, grad, nvox * 4, cudaMemcpyDeviceToHost, st));
    unsigned int herr = 0;
    unsigned long long hc[CT_NUM] = {0};
    DT_ACK(cudaMemcpyAsync(&herr, sb.err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    if (ctr) DT_ACK(cudaMemcpyAsync(hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, st));
    DT_ACK(cudaStreamSynchronize(st));
    cudaEventElapsedTime(&ms_replay, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dtrt_render_stats &ls = s->last;
    std::memset(&ls, 0, sizeof(ls));
    ls.camera_paths = (uint64_t)total;
    ls.kernel_launches = launches;
    ls.batches = (uint64_t)((total + (wavefront ? w.cap : B) - 1) / std::max<long long>(1, wavefront ? w.cap : B));
    ls.counters_enabled = ctr != nullptr;
    ls.camera_schedule = wavefront ? DTRT_CAMERA_WAVEFRONT : DTRT_CAMERA_MEGAKERNEL;
    ls.k_rays[0] = ls.rays = hc[0];
    ls.k_node_visits[0] = ls.node_visits = hc[1];
    ls.k_tri_tests[0] = ls.tri_tests = hc[2];
    ls.k_grid_lookups[0] = ls.grid_lookups = hc[3];
    ls.k_light_samples[0] = ls.light_samples = hc[4];
    ls.ms_camera = ms_replay;
    ls.ms_total = std::chrono::duration<double, std::milli>(clk::now() - t_start).count();
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
