// dtrt_gb300 — render orchestration for one derivative width (instantiated per N).
//
// IntegratorAD::render (integratorAD.cpp:19-166) as batches of camera paths:
//   for each batch:   k_camera -> [k_edge -> k_li]* (chunked) -> k_lins
//   primary edges:    [k_primary -> k_li]* (chunked)
//   k_finalize
// Queue capacities bound device memory; the worst case per camera path (one edge or
// Lins record per bounce, two Li tasks per edge sample) sizes the batches so that a
// push can only overflow when a caller forces a capacity below one path's worst case.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "dt_host.h"

namespace dt {

#define DT_CK(call)                                                                  \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return DTRT_ERR_CUDA;                                                    \
        }                                                                            \
    } while (0)

template <int N>
int render_n(dtrt_scene *s, const dtrt_render_options *o, float *out, int out_on_device, cudaStream_t st) {
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
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
    if (o->max_bounces < 0) {
        set_last_error("max_bounces must be >= 0");
        return DTRT_ERR_INVALID;
    }
    const size_t npix = (size_t)rp.npix;
    // ---------------------------------------------------------------- buffers
    const size_t acc1_n = (N + 1) * npix * 3, acc2_n = (size_t)N * npix * 3, out_n = (N + 1) * npix * 3;
    if (!ensure_buffer((void **)&sb.acc1, &sb.acc1_n, acc1_n * 8) || !ensure_buffer((void **)&sb.acc2, &sb.acc2_n, acc2_n * 8))
        return DTRT_ERR_CUDA;
    if (!out_on_device && !ensure_buffer((void **)&sb.out, &sb.out_n, out_n * 4)) return DTRT_ERR_CUDA;
    const uint64_t li_cap = s->queue_cap ? s->queue_cap : (uint64_t)24 << 20;
    // 16 Mi records bound a camera batch at 16Mi/(max_bounces+1) paths (1.5 M at depth 10):
    // few launches, so the partial last wave of each batch costs little
    const uint64_t rec_cap = s->queue_cap ? s->queue_cap : (uint64_t)16 << 20;
    if (!ensure_buffer(&sb.qli, &sb.qli_bytes, li_cap * sizeof(LiTask<N>)) ||
        !ensure_buffer(&sb.qe, &sb.qe_bytes, rec_cap * sizeof(EdgeRec<N>)) ||
        !ensure_buffer(&sb.ql, &sb.ql_bytes, rec_cap * sizeof(LinsRec<N>)))
        return DTRT_ERR_CUDA;
    if (!sb.counts) DT_CK(cudaMalloc(&sb.counts, kCountSlots * sizeof(unsigned long long)));
    if (!sb.err) DT_CK(cudaMalloc(&sb.err, sizeof(unsigned int)));
    sc.error_flags = sb.err;
    DT_CK(cudaMemsetAsync(sb.acc1, 0, acc1_n * 8, st));
    DT_CK(cudaMemsetAsync(sb.acc2, 0, acc2_n * 8, st));
    DT_CK(cudaMemsetAsync(sb.counts, 0, kCountSlots * sizeof(unsigned long long), st));
    DT_CK(cudaMemsetAsync(sb.err, 0, sizeof(unsigned int), st));
    unsigned long long *ctr = s->counters ? sb.counts + 8 : nullptr;
    Queue qe{sb.qe, sb.counts + 0, rec_cap}, ql{sb.ql, sb.counts + 1, rec_cap}, qli{sb.qli, sb.counts + 2, li_cap};

    cudaEvent_t e0, e1;
    DT_CK(cudaEventCreate(&e0));
    DT_CK(cudaEventCreate(&e1));
    double ms_camera = 0, ms_edge = 0, ms_li = 0, ms_primary = 0;
    uint64_t launches = 0;
    auto timed = [&](double &acc, auto &&launch) -> int {
        ++launches;
        cudaEventRecord(e0, st);
        launch();
        cudaEventRecord(e1, st);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) {
            set_last_error(std::string("kernel launch: ") + cudaGetErrorString(err));
            return DTRT_ERR_CUDA;
        }
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        acc += ms;
        return DTRT_OK;
    };
    unsigned long long hcnt[3];
    auto read_counts = [&]() -> int {
        DT_CK(cudaMemcpyAsync(hcnt, sb.counts, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        DT_CK(cudaStreamSynchronize(st));
        return DTRT_OK;
    };
    auto blocks = [](long long n) { return (unsigned)((n + kBlock - 1) / kBlock); };
    uint64_t tot_edge = 0, tot_lins = 0, tot_li = 0, batches = 0;
    uint64_t state_traffic = 0;  // wavefront path-state bytes read + written (counted when counters are on)
    bool used_wavefront = false;
    int rc = DTRT_OK;
    // Li sub-path pairs sorted by origin and direction before k_li (needs a tree)
    const bool li_sorted = sc.num_nodes > 0 && ensure_li_sort(sb, li_cap);
    // Li tasks are drained chunk by chunk so that the queue never exceeds li_cap
    auto drain_li = [&]() -> int {
        if ((rc = read_counts())) return rc;
        const unsigned long long n = std::min<unsigned long long>(hcnt[2], li_cap);
        tot_li += n;
        if (n)
            if ((rc = timed(ms_li, [&] {
                     const int *perm = li_sorted ? sort_li_pairs(sc, (const LiTask<N> *)qli.data, (long long)n, sb,
                                                                 li_cap, st, launches)
                                                 : nullptr;
                     k_li<N><<<blocks(n), kBlock, 0, st>>>(sc, rp, qli, 0, n, sb.acc1, sb.acc2, perm, ctr);
                 })))
                return rc;
        DT_CK(cudaMemsetAsync(sb.counts + 2, 0, sizeof(unsigned long long), st));
        return DTRT_OK;
    };

    // ---------------------------------------------------------------- pass 1
    const long long total = (long long)npix * std::max(0, o->spp);
    if (total > 0) {
        const long long unit = std::max<long long>(128, (long long)rp.spp % 32 == 0 ? std::max(rp.spp, 128) : 128);
        long long B = (long long)(rec_cap / (uint64_t)std::max(1, o->max_bounces + 1));
        B = std::max<long long>(unit, (B / unit) * unit);
        const long long per_chunk = std::max<long long>(1, (long long)(li_cap / (uint64_t)std::max(1, 2 * rp.sppse)));
        // camera schedule: the wavefront keeps CamState and VertexIn per path of a batch in device memory
        const long long Bw = std::min<long long>(B, total);
        const int levels = o->max_bounces + 1;  // a continuing vertex always spends one bounce
        bool wavefront = s->camera_schedule == DTRT_CAMERA_WAVEFRONT ||
                         (s->camera_schedule == DTRT_CAMERA_AUTO && Bw >= kWavefrontMinPaths);
        const size_t state_bytes = ((size_t)Bw * sizeof(CamState<N>) + 255) & ~(size_t)255;
        if (wavefront && !(ensure_buffer(&sb.cam_state, &sb.cam_state_bytes, state_bytes + (size_t)Bw * sizeof(VertexIn<N>)) &&
                           ensure_buffer(&sb.cam_q, &sb.cam_q_bytes, (size_t)4 * Bw * sizeof(int)) &&
                           ensure_buffer(&sb.cam_cnt, &sb.cam_cnt_bytes, (size_t)3 * (levels + 1) * sizeof(unsigned long long)))) {
            if (s->camera_schedule == DTRT_CAMERA_WAVEFRONT) return DTRT_ERR_CUDA;
            cudaGetLastError();  // AUTO: no room for the path states, run the megakernel
            wavefront = false;
        }
        int sms = 0;
        DT_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
        used_wavefront = wavefront;
        CamState<N> *states = (CamState<N> *)sb.cam_state;
        VertexIn<N> *vins = (VertexIn<N> *)((char *)sb.cam_state + state_bytes);
        int *qa = (int *)sb.cam_q, *qb = qa + Bw, *qv = qb + Bw, *qs = qv + Bw;
        // volume and interface vertices queued per level [0, levels] (interface: pushed from the
        // front of the queue, scnt, and from its back, sbk)
        unsigned long long *vcnt = (unsigned long long *)sb.cam_cnt, *scnt = vcnt + (levels + 1),
                           *sbk = scnt + (levels + 1);
        for (long long b0 = 0; b0 < total; b0 += B) {
            ++batches;
            rp.path_begin = b0;
            rp.path_count = std::min(B, total - b0);
            DT_CK(cudaMemsetAsync(sb.counts, 0, 3 * sizeof(unsigned long long), st));
            if (wavefront) {
                // grid-stride launches of a few waves: late levels hold few live paths
                const unsigned gw = std::min<unsigned>(blocks(rp.path_count), (unsigned)std::max(1, sms) * 16u);
                if ((rc = timed(ms_camera, [&] {
                         cudaMemsetAsync(vcnt, 0, (size_t)3 * (levels + 1) * sizeof(unsigned long long), st);
                         // volume / interface queues of level L: (qa, qb) for even L, (qv, qs) for odd L
                         k_cam_start<N><<<blocks(rp.path_count), kBlock, 0, st>>>(
                             sc, rp, states, vins, qa, vcnt, qv, vcnt + 1, qs, scnt + 1, sbk + 1, Bw, qe, ql, ctr);
                         for (int L = 0; L < levels; ++L) {
                             int *qvl = (L & 1) ? qv : qa, *qsl = (L & 1) ? qs : qb;
                             int *qvn = (L & 1) ? qa : qv, *qsn = (L & 1) ? qb : qs;
                             k_cam_vertex<N, true><<<gw, kBlock, 0, st>>>(sc, rp, states, vins, qvl, vcnt + L, nullptr,
                                                                          qvn, vcnt + L + 1, qsn, scnt + L + 1,
                                                                          sbk + L + 1, Bw, qe, ql, ctr);
                             if (L > 0)  // level 0's interface vertices ran in k_cam_start
                                 k_cam_vertex<N, false><<<gw, kBlock, 0, st>>>(sc, rp, states, vins, qsl, scnt + L,
                                                                               sbk + L, qvn, vcnt + L + 1, qsn,
                                                                               scnt + L + 1, sbk + L + 1, Bw, qe, ql,
                                                                               ctr);
                         }
                         k_cam_accum<N><<<blocks(rp.path_count), kBlock, 0, st>>>(rp, states, sb.acc1);
                     })))
                    return rc;
                launches += 2 * levels + 1;  // start, 2 per level (1 at level 0), accumulation
                if (ctr) {
                    // every launched vertex reads and writes its path's state and vertex inputs;
                    // the start writes them once per path, the accumulation reads the sums
                    std::vector<unsigned long long> lc((size_t)3 * (levels + 1));
                    DT_CK(cudaMemcpyAsync(lc.data(), vcnt, lc.size() * sizeof(unsigned long long),
                                          cudaMemcpyDeviceToHost, st));
                    DT_CK(cudaStreamSynchronize(st));
                    // each queued vertex's state and inputs are written once and read once (a
                    // volume vertex's without the hit record); an ended path writes its sums,
                    // which k_cam_accum reads
                    const uint64_t sv = sizeof(CamState<N>) + sizeof(VertexIn<N>), si = sizeof(ItsAD<N>);
                    uint64_t vol = 0, itf = 0;
                    for (int L = 0; L < levels; ++L) {
                        vol += lc[L];
                        itf += L > 0 ? lc[levels + 1 + L] + lc[2 * (levels + 1) + L] : 0;
                    }
                    state_traffic += 2 * ((sv - si) * vol + sv * itf) + 2 * sizeof(DV<N>) * (uint64_t)rp.path_count;
                }
            } else if ((rc = timed(ms_camera, [&] {
                            k_camera<N><<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, qe, ql, sb.acc1, ctr);
                        }))) {
                return rc;
            }
            if ((rc = read_counts())) return rc;
            const unsigned long long ne = std::min<unsigned long long>(hcnt[0], rec_cap);
            const unsigned long long nl = std::min<unsigned long long>(hcnt[1], rec_cap);
            tot_edge += ne;
            tot_lins += nl;
            for (unsigned long long r0 = 0; r0 < ne && rp.sppse > 0; r0 += per_chunk) {
                const long long cnt = (long long)std::min<unsigned long long>(per_chunk, ne - r0);
                if ((rc = timed(ms_edge, [&] {
                         k_edge<N><<<blocks(cnt * rp.sppse), kBlock, 0, st>>>(sc, rp, qe, (long long)r0, cnt, qli, ctr);
                     })))
                    return rc;
                if ((rc = drain_li())) return rc;
            }
            if (nl)
                if ((rc = timed(ms_li, [&] { k_lins<N><<<blocks(nl), kBlock, 0, st>>>(sc, rp, ql, nl, sb.acc1, ctr); })))
                    return rc;
        }
    }
    // ---------------------------------------------------------------- pass 2: primary edges
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
            if ((rc = timed(ms_primary, [&] {
                     const int *perm = li_sorted ? sort_primary_samples(rp, sb, li_cap, st, launches) : nullptr;
                     k_primary<N><<<blocks(rp.prim_count), kBlock, 0, st>>>(sc, rp, qli, perm, ctr);
                 })))
                return rc;
            if ((rc = drain_li())) return rc;
        }
    }
    // ---------------------------------------------------------------- finalize
    float *dst = out_on_device ? out : sb.out;
    k_finalize<N><<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(rp, sb.acc1, sb.acc2, dst);
    ++launches;
    DT_CK(cudaGetLastError());
    if (!out_on_device) DT_CK(cudaMemcpyAsync(out, sb.out, out_n * 4, cudaMemcpyDeviceToHost, st));
    unsigned int herr = 0;
    unsigned long long hc[CT_NUM] = {0};
    DT_CK(cudaMemcpyAsync(&herr, sb.err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    if (ctr) DT_CK(cudaMemcpyAsync(hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, st));
    DT_CK(cudaStreamSynchronize(st));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dtrt_render_stats &ls = s->last;
    std::memset(&ls, 0, sizeof(ls));
    ls.camera_paths = (uint64_t)total;
    ls.edge_records = tot_edge;
    ls.lins_records = tot_lins;
    ls.li_tasks = tot_li;
    ls.primary_edge_samples = prim_samples;
    ls.batches = batches;
    ls.kernel_launches = launches;
    ls.counters_enabled = ctr != nullptr;
    ls.camera_schedule = used_wavefront ? DTRT_CAMERA_WAVEFRONT : DTRT_CAMERA_MEGAKERNEL;
    for (int k = 0; k < 5; ++k) {
        const unsigned long long *h = hc + kCtrPerKernel * k;
        ls.k_rays[k] = h[0];
        ls.k_node_visits[k] = h[1];
        ls.k_tri_tests[k] = h[2];
        ls.k_grid_lookups[k] = h[3];
        ls.k_light_samples[k] = h[4];
        ls.rays += h[0];
        ls.node_visits += h[1];
        ls.tri_tests += h[2];
        ls.grid_lookups += h[3];
        ls.light_samples += h[4];
    }
    ls.camera_state_bytes = state_traffic;
    ls.edge_samples = ctr ? hc[CT_EDGE_SAMPLES] : tot_edge * (uint64_t)rp.sppse;
    ls.ms_camera = ms_camera;
    ls.ms_edge = ms_edge;
    ls.ms_li = ms_li;
    ls.ms_primary = ms_primary;
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

namespace dt {

// ====================================================================== no-allocation render
// Same work as render_n, on caller-provided scratch (the static array of dt_noalloc.cu):
// fixed small queue capacities, no cudaMalloc / cudaFree / event creation.
constexpr uint64_t kNoallocLiCap = 16384, kNoallocRecCap = 4096;

constexpr size_t noalloc_round(size_t b) { return (b + 255) & ~(size_t)255; }
// Bytes the carve below takes at its largest: DTRT_NOALLOC_MAX_PIXELS pixels with a host
// output (staging copy) and the three queues at their fixed capacities.
template <int N>
constexpr size_t noalloc_worst_case_bytes() {
    return noalloc_round((size_t)(N + 1) * DTRT_NOALLOC_MAX_PIXELS * 3 * 8) +
           noalloc_round((size_t)N * DTRT_NOALLOC_MAX_PIXELS * 3 * 8) +
           noalloc_round((size_t)(N + 1) * DTRT_NOALLOC_MAX_PIXELS * 3 * 4) + noalloc_round(32 * 8) +
           noalloc_round(sizeof(unsigned int)) + noalloc_round(kNoallocLiCap * sizeof(LiTask<N>)) +
           noalloc_round(kNoallocRecCap * sizeof(EdgeRec<N>)) + noalloc_round(kNoallocRecCap * sizeof(LinsRec<N>));
}

template <int N>
int render_n_noalloc(dtrt_scene *s, const dtrt_render_options *o, float *out, int out_on_device, cudaStream_t st,
                     unsigned char *scratch, size_t scratch_bytes) {
    static_assert(noalloc_worst_case_bytes<N>() <= DTRT_NOALLOC_SCRATCH_BYTES,
                  "the no-allocation scratch array cannot hold the largest allowed render");
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    DevScene sc = s->dev;
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
    if (npix > DTRT_NOALLOC_MAX_PIXELS) {
        set_last_error("dtrt_render_fwd_noalloc: image has " + std::to_string(npix) + " pixels, the maximum is " +
                       std::to_string(DTRT_NOALLOC_MAX_PIXELS));
        return DTRT_ERR_INVALID;
    }
    if (o->max_bounces < 0 || o->max_bounces > 31 || rp.sppse > (int)(kNoallocLiCap / 2)) {
        set_last_error("dtrt_render_fwd_noalloc: needs 0 <= max_bounces <= 31 and sppse <= 8192");
        return DTRT_ERR_INVALID;
    }
    // carve the scratch array (256-byte aligned pieces)
    size_t off = 0;
    auto take = [&](size_t bytes) -> unsigned char * {
        unsigned char *p = scratch + off;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    const size_t acc1_n = (N + 1) * npix * 3, acc2_n = (size_t)N * npix * 3, out_n = (N + 1) * npix * 3;
    double *acc1 = (double *)take(acc1_n * 8);
    double *acc2 = (double *)take(acc2_n * 8);
    float *stage = out_on_device ? nullptr : (float *)take(out_n * 4);
    unsigned long long *counts = (unsigned long long *)take(32 * sizeof(unsigned long long));
    unsigned int *err = (unsigned int *)take(sizeof(unsigned int));
    void *qli_p = take(kNoallocLiCap * sizeof(LiTask<N>));
    void *qe_p = take(kNoallocRecCap * sizeof(EdgeRec<N>));
    void *ql_p = take(kNoallocRecCap * sizeof(LinsRec<N>));
    if (off > scratch_bytes) {
        set_last_error("dtrt_render_fwd_noalloc: scratch array too small for this image");
        return DTRT_ERR_INVALID;
    }
    sc.error_flags = err;
    DT_CK(cudaMemsetAsync(acc1, 0, acc1_n * 8, st));
    DT_CK(cudaMemsetAsync(acc2, 0, acc2_n * 8, st));
    DT_CK(cudaMemsetAsync(counts, 0, 32 * sizeof(unsigned long long), st));
    DT_CK(cudaMemsetAsync(err, 0, sizeof(unsigned int), st));
    Queue qe{qe_p, counts + 0, kNoallocRecCap}, ql{ql_p, counts + 1, kNoallocRecCap}, qli{qli_p, counts + 2, kNoallocLiCap};
    unsigned long long hcnt[3];
    uint64_t launches = 0, batches = 0, tot_edge = 0, tot_lins = 0, tot_li = 0;
    auto read_counts = [&]() -> int {
        DT_CK(cudaMemcpyAsync(hcnt, counts, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        DT_CK(cudaStreamSynchronize(st));
        return DTRT_OK;
    };
    auto launched = [&]() -> int {
        ++launches;
        DT_CK(cudaGetLastError());
        return DTRT_OK;
    };
    auto blocks = [](long long n) { return (unsigned)((n + kBlock - 1) / kBlock); };
    int rc = DTRT_OK;
    auto drain_li = [&]() -> int {
        if ((rc = read_counts())) return rc;
        const unsigned long long n = std::min<unsigned long long>(hcnt[2], kNoallocLiCap);
        tot_li += n;
        if (n) {
            k_li<N><<<blocks(n), kBlock, 0, st>>>(sc, rp, qli, 0, n, acc1, acc2, nullptr, nullptr);
            if ((rc = launched())) return rc;
        }
        DT_CK(cudaMemsetAsync(counts + 2, 0, sizeof(unsigned long long), st));
        return DTRT_OK;
    };
    const long long total = (long long)npix * std::max(0, o->spp);
    if (total > 0) {
        // 128-path units keep every warp inside one pixel whenever spp is a multiple of 32
        const long long unit = 128;
        long long B = (long long)(kNoallocRecCap / (uint64_t)(o->max_bounces + 1));
        B = std::max<long long>(unit, (B / unit) * unit);
        const long long per_chunk = std::max<long long>(1, (long long)(kNoallocLiCap / (uint64_t)std::max(1, 2 * rp.sppse)));
        for (long long b0 = 0; b0 < total; b0 += B) {
            ++batches;
            rp.path_begin = b0;
            rp.path_count = std::min(B, total - b0);
            DT_CK(cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), st));
            k_camera<N><<<blocks(rp.path_count), kBlock, 0, st>>>(sc, rp, qe, ql, acc1, nullptr);
            if ((rc = launched())) return rc;
            if ((rc = read_counts())) return rc;
            const unsigned long long ne = std::min<unsigned long long>(hcnt[0], kNoallocRecCap);
            const unsigned long long nl = std::min<unsigned long long>(hcnt[1], kNoallocRecCap);
            tot_edge += ne;
            tot_lins += nl;
            for (unsigned long long r0 = 0; r0 < ne && rp.sppse > 0; r0 += per_chunk) {
                const long long cnt = (long long)std::min<unsigned long long>(per_chunk, ne - r0);
                k_edge<N><<<blocks(cnt * rp.sppse), kBlock, 0, st>>>(sc, rp, qe, (long long)r0, cnt, qli, nullptr);
                if ((rc = launched())) return rc;
                if ((rc = drain_li())) return rc;
            }
            if (nl) {
                k_lins<N><<<blocks(nl), kBlock, 0, st>>>(sc, rp, ql, nl, acc1, nullptr);
                if ((rc = launched())) return rc;
            }
        }
    }
    uint64_t prim_samples = 0;
    if (o->sppe > 0 && sc.num_pedges > 0) {
        const long long nblock = (long long)std::ceil(sc.pedge_sum * o->sppe / 128.0);
        const long long ns = nblock * 128;
        prim_samples = (uint64_t)ns;
        rp.prim_weight = sc.pedge_sum / (double)ns;
        const long long chunk = (long long)(kNoallocLiCap / 2);
        for (long long k0 = 0; k0 < ns; k0 += chunk) {
            rp.prim_begin = k0;
            rp.prim_count = std::min(chunk, ns - k0);
            k_primary<N><<<blocks(rp.prim_count), kBlock, 0, st>>>(sc, rp, qli, nullptr, nullptr);
            if ((rc = launched())) return rc;
            if ((rc = drain_li())) return rc;
        }
    }
    float *dst = out_on_device ? out : stage;
    k_finalize<N><<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(rp, acc1, acc2, dst);
    if ((rc = launched())) return rc;
    if (!out_on_device) DT_CK(cudaMemcpyAsync(out, stage, out_n * 4, cudaMemcpyDeviceToHost, st));
    unsigned int herr = 0;
    DT_CK(cudaMemcpyAsync(&herr, err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    DT_CK(cudaStreamSynchronize(st));
    dtrt_render_stats &ls = s->last;
    std::memset(&ls, 0, sizeof(ls));
    ls.camera_paths = (uint64_t)total;
    ls.edge_records = tot_edge;
    ls.lins_records = tot_lins;
    ls.li_tasks = tot_li;
    ls.primary_edge_samples = prim_samples;
    ls.batches = batches;
    ls.kernel_launches = launches;
    ls.edge_samples = tot_edge * (uint64_t)rp.sppse;
    ls.camera_schedule = DTRT_CAMERA_MEGAKERNEL;
    ls.ms_total = std::chrono::duration<double, std::milli>(clk::now() - t_start).count();
    if (herr & ERR_QUEUE) {
        set_last_error("work queue overflow");
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
