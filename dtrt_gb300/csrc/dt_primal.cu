// dtrt_gb300 — primal volumetric path tracer (VolPathTracer, no derivatives).
//
// VolPathTracer::render (src/integrator/volpath.cpp:105-140) traces `spp` jittered
// primary rays per pixel through VolPathTracer::radiance (volpath.cpp:10-103), which is
// the non-AD Li loop also used by the edge terms (li_path / li_step). Here: no dual
// numbers, no queues; per-path PCG32 streams (RndSampler(seed, path index)), FP64 pixel
// accumulation in path order, and the reference's unconditional write. Two schedules with
// identical results: one thread per path (k_primal) or a wavefront of li_step launches.
#include <algorithm>
#include <chrono>
#include <cstring>

#include "dt_host.h"
#include "dt_kernels.cuh"

namespace dt {

__global__ void __launch_bounds__(kBlock) k_primal(DevScene sc, RenderParams rp, double *img_acc,
                                                   unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < rp.path_count;
    const long long g = rp.path_begin + (active ? gi : 0);
    const int pixel = (int)(g / rp.spp);
    Ctr c;
    float3 L = mk(0.f, 0.f, 0.f);
    if (active) {
        const int ix = rp.crop_x + pixel % rp.out_w, iy = rp.crop_y + pixel / rp.out_w;
        Rng rng;
        rng.init(rp.seed, (uint64_t)g);
        const double jx = rng.next1d(), jy = rng.next1d();  // samplePrimaryRay(ix, iy, next2D())
        float3 o, d;
        camera_ray(sc.cam, ix + jx, iy + jy, o, d);
        L = li_path(sc, stack, rng, o, d, rp.max_bounces, sc.cam.med_id, true, c, false) * rp.inv_spp;
    }
    const unsigned full = 0xffffffffu;
    const int p0 = __shfl_sync(full, pixel, 0);
    const bool uniform = __all_sync(full, active && pixel == p0);
    float v[3] = {L.x, L.y, L.z};
    if (uniform)
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(full, v[k], off);
    if (active && (!uniform || (threadIdx.x & 31) == 0))
        for (int k = 0; k < 3; ++k)
            if (v[k] != 0.f) atomicAdd(img_acc + (size_t)pixel * 3 + k, (double)v[k]);
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// Wavefront schedule of the primal render (as the forward camera stage): the path state
// (LiState) between vertices in HBM, one launch per vertex over the compacted live paths,
// each path's radiance kept per path and summed per pixel in path order.
__global__ void __launch_bounds__(kBlock) k_primal_start(DevScene sc, RenderParams rp, LiState *states, float3 *rets,
                                                         int *q_out, unsigned long long *cnt_out,
                                                         unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    bool live = false;
    if (gi < rp.path_count) {
        const long long g = rp.path_begin + gi;
        const int pixel = (int)(g / rp.spp);
        const int ix = rp.crop_x + pixel % rp.out_w, iy = rp.crop_y + pixel / rp.out_w;
        LiState st;
        st.rng.init(rp.seed, (uint64_t)g);
        const double jx = st.rng.next1d(), jy = st.rng.next1d();
        float3 o, d;
        camera_ray(sc.cam, ix + jx, iy + jy, o, d);
        live = li_start(sc, stack, st, o, d, rp.max_bounces, sc.cam.med_id, true, c, false);
        if (live) states[gi] = st;
        rets[gi] = mk(0.f, 0.f, 0.f);
    }
    push_path(q_out, cnt_out, (int)gi, live);
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

__global__ void __launch_bounds__(kBlock) k_primal_level(DevScene sc, RenderParams rp, LiState *states, float3 *rets,
                                                         const int *q_in, const unsigned long long *cnt_in, int *q_out,
                                                         unsigned long long *cnt_out, unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long n = (long long)*cnt_in;
    Ctr c;
    for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < n; i += (long long)gridDim.x * kBlock) {
        const int id = q_in[i];
        LiState st = states[id];
        const bool alive = li_step(sc, stack, st, c);
        if (alive) states[id] = st;
        else rets[id] = st.ret;
        push_path(q_out, cnt_out, id, alive);
    }
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

__global__ void __launch_bounds__(kBlock) k_primal_accum(RenderParams rp, const float3 *rets, double *img_acc) {
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < rp.path_count;
    const int pixel = (int)((rp.path_begin + (active ? gi : 0)) / rp.spp);
    const float3 L = active ? rets[gi] * rp.inv_spp : mk(0.f, 0.f, 0.f);
    const unsigned full = 0xffffffffu;
    const int p0 = __shfl_sync(full, pixel, 0);
    const bool uniform = __all_sync(full, active && pixel == p0);
    float v[3] = {L.x, L.y, L.z};
    if (uniform)
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(full, v[k], off);
    if (active && (!uniform || (threadIdx.x & 31) == 0))
        for (int k = 0; k < 3; ++k)
            if (v[k] != 0.f) atomicAdd(img_acc + (size_t)pixel * 3 + k, (double)v[k]);
}

__global__ void k_primal_image(int npix, const double *acc, float *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    for (int k = 0; k < 3; ++k) out[(size_t)p * 3 + k] = (float)acc[(size_t)p * 3 + k];  // volpath.cpp:134-136
}

#define DT_PCK(call)                                                                 \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return DTRT_ERR_CUDA;                                                    \
        }                                                                            \
    } while (0)

int render_primal(dtrt_scene *s, const dtrt_render_options *o, float *out, int out_on_device, cudaStream_t st) {
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    DevScene sc = s->dev;
    Scratch &sb = s->scratch;
    const DevCamera &cam = sc.cam;
    const bool cropped = cam.crop_w > 0 && cam.crop_h > 0;
    if (o->max_bounces < 0 || o->spp < 0) {
        set_last_error("spp and max_bounces must be >= 0");
        return DTRT_ERR_INVALID;
    }
    RenderParams rp{};
    rp.seed = o->seed;
    rp.spp = o->spp;
    rp.max_bounces = o->max_bounces;
    rp.inv_spp = o->spp > 0 ? 1.0f / (float)o->spp : 0.f;
    rp.out_w = cropped ? cam.crop_w : cam.width;
    rp.out_h = cropped ? cam.crop_h : cam.height;
    rp.crop_x = cropped ? cam.crop_x : 0;
    rp.crop_y = cropped ? cam.crop_y : 0;
    rp.npix = rp.out_w * rp.out_h;
    const size_t npix = (size_t)rp.npix;
    if (!sb.err) DT_PCK(cudaMalloc(&sb.err, sizeof(unsigned int)));
    if (!sb.counts) DT_PCK(cudaMalloc(&sb.counts, kCountSlots * sizeof(unsigned long long)));
    sc.error_flags = sb.err;
    DT_PCK(cudaMemsetAsync(sb.err, 0, sizeof(unsigned int), st));
    DT_PCK(cudaMemsetAsync(sb.counts, 0, kCountSlots * sizeof(unsigned long long), st));
    unsigned long long *ctr = s->counters ? sb.counts + 8 : nullptr;
    if (!ensure_buffer((void **)&sb.adj_img, &sb.adj_img_n, npix * 3 * 8)) return DTRT_ERR_CUDA;
    DT_PCK(cudaMemsetAsync(sb.adj_img, 0, npix * 3 * 8, st));
    cudaEvent_t e0, e1;
    DT_PCK(cudaEventCreate(&e0));
    DT_PCK(cudaEventCreate(&e1));
    const long long total = (long long)npix * o->spp;
    long long B = 1ll << 26;  // paths per megakernel launch
    uint64_t launches = 0;
    // schedule: AUTO runs the wavefront for large renders of scenes with grid media, whose
    // paths differ most in length (C1 primal 42.1 -> 19.0 ms); on surface scenes the paths
    // are short and the megakernel measured faster (C2 2.7 against 3.3 ms)
    bool wavefront = s->camera_schedule == DTRT_CAMERA_WAVEFRONT ||
                     (s->camera_schedule == DTRT_CAMERA_AUTO && total >= kWavefrontMinPaths && sc.has_grid_media);
    const int levels = o->max_bounces + 2;  // li_step runs at most max_bounces + 1 vertices
    LiState *states = nullptr;
    float3 *rets = nullptr;
    int *qa = nullptr, *qb = nullptr;
    unsigned long long *lcnt = nullptr;
    if (wavefront) {
        B = std::min<long long>(1ll << 22, std::max<long long>(total, 1));
        const size_t sbytes = ((size_t)B * sizeof(LiState) + 255) & ~(size_t)255;
        if (ensure_buffer(&sb.cam_state, &sb.cam_state_bytes, sbytes + (size_t)B * sizeof(float3)) &&
            ensure_buffer(&sb.cam_q, &sb.cam_q_bytes, (size_t)2 * B * sizeof(int)) &&
            ensure_buffer(&sb.cam_cnt, &sb.cam_cnt_bytes, (size_t)(levels + 1) * sizeof(unsigned long long))) {
            states = (LiState *)sb.cam_state;
            rets = (float3 *)((char *)sb.cam_state + sbytes);
            qa = (int *)sb.cam_q;
            qb = qa + B;
            lcnt = (unsigned long long *)sb.cam_cnt;
        } else {
            if (s->camera_schedule == DTRT_CAMERA_WAVEFRONT) return DTRT_ERR_CUDA;
            cudaGetLastError();  // AUTO: no room for the path states, run the megakernel
            wavefront = false;
            B = 1ll << 26;
        }
    }
    int sms = 0;
    DT_PCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
    auto blocks = [](long long n) { return (unsigned)((n + kBlock - 1) / kBlock); };
    DT_PCK(cudaEventRecord(e0, st));
    for (long long b0 = 0; b0 < total; b0 += B) {
        rp.path_begin = b0;
        rp.path_count = std::min(B, total - b0);
        if (!wavefront) {
            k_primal<<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, sb.adj_img, ctr);
            ++launches;
            DT_PCK(cudaGetLastError());
            continue;
        }
        const unsigned gw = std::min<unsigned>(blocks(rp.path_count), (unsigned)std::max(1, sms) * 16u);
        DT_PCK(cudaMemsetAsync(lcnt, 0, (size_t)(levels + 1) * sizeof(unsigned long long), st));
        k_primal_start<<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, states, rets, qa, lcnt, ctr);
        for (int L = 0; L < levels; ++L)
            k_primal_level<<<gw, kBlock, 0, st>>>(sc, rp, states, rets, (L & 1) ? qb : qa, lcnt + L, (L & 1) ? qa : qb,
                                                  lcnt + L + 1, ctr);
        k_primal_accum<<<blocks(rp.path_count), kBlock, 0, st>>>(rp, rets, sb.adj_img);
        launches += levels + 2;
        DT_PCK(cudaGetLastError());
    }
    DT_PCK(cudaEventRecord(e1, st));
    float *dst = out;
    if (!out_on_device) {
        if (!ensure_buffer((void **)&sb.adj_out, &sb.adj_out_n, npix * 3 * 4)) return DTRT_ERR_CUDA;
        dst = sb.adj_out;
    }
    k_primal_image<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(rp.npix, sb.adj_img, dst);
    ++launches;
    DT_PCK(cudaGetLastError());
    if (!out_on_device) DT_PCK(cudaMemcpyAsync(out, sb.adj_out, npix * 3 * 4, cudaMemcpyDeviceToHost, st));
    unsigned int herr = 0;
    unsigned long long hc[CT_NUM] = {0};
    DT_PCK(cudaMemcpyAsync(&herr, sb.err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    if (ctr) DT_PCK(cudaMemcpyAsync(hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, st));
    DT_PCK(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dtrt_render_stats &ls = s->last;
    std::memset(&ls, 0, sizeof(ls));
    ls.camera_paths = (uint64_t)total;
    ls.kernel_launches = launches;
    ls.batches = (uint64_t)((total + B - 1) / B);
    ls.counters_enabled = ctr != nullptr;
    ls.camera_schedule = wavefront ? DTRT_CAMERA_WAVEFRONT : DTRT_CAMERA_MEGAKERNEL;
    ls.k_rays[0] = ls.rays = hc[0];
    ls.k_node_visits[0] = ls.node_visits = hc[1];
    ls.k_tri_tests[0] = ls.tri_tests = hc[2];
    ls.k_grid_lookups[0] = ls.grid_lookups = hc[3];
    ls.k_light_samples[0] = ls.light_samples = hc[4];
    ls.ms_camera = ms;
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

extern "C" int dtrt_render_primal(dtrt_scene *scene, const dtrt_render_options *opts, float *out, int out_on_device,
                                  void *stream) {
    if (!scene || !opts || !out) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    return dt::render_primal(scene, opts, out, out_on_device, (cudaStream_t)stream);
}
