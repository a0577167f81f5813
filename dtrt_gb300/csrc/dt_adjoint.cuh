// dtrt_gb300 — reverse-mode adjoint of the interior term by path replay.
//
// Scope: the gradient of <dL/dI, I> with respect to the density voxels of every
// heterogeneous medium. The reference has no reverse mode; its forward-mode estimator
// (volpathAD.cpp:145-620) is the thing differentiated, and this kernel computes the exact
// transpose of that estimator's per-voxel directional derivative, path by path:
//
//   Density enters a camera path only through log-derivative factors:
//     * distance sampling (heterogeneous.cpp:40-75) multiplies the throughput of every
//       later event by (sigma_t(p) / sigma_t(p).val) * (1, -int dsigma_t): log-derivative
//       d density(p) / density(p) - integral, or just -integral when no scatter happens;
//     * the transmittance of a NEE or emitter-hit segment (heterogeneous.cpp:113-118)
//       multiplies only that event's contribution: log-derivative -integral.
//   The integral is the 10-sample stratified estimate of intSigT (heterogeneous.cpp:121-141).
//
// So d(path)/d(density) = sum over factors of (log-derivative) * (radiance the factor
// multiplies). Each thread runs its camera path twice from the same RNG seed:
//   pass A: the path value, i.e. the sum of its event contributions (the image);
//   pass B: the same path again; before each distance-sampling factor the suffix radiance
//           (pass-A total minus what pass B has accumulated so far) is known, so every
//           density lookup feeding that factor scatters dot(dL/dI, suffix)/spp times its
//           coefficient into the 8 voxels it read. A NEE or emitter-hit event is first
//           evaluated for its value, then re-run from the saved RNG state with the weight
//           dot(dL/dI, event)/spp, which replays the identical random decisions.
// No path state is stored. Boundary terms (edges, Lins, primary edges) depend on moving
// geometry only and carry no density derivative, so the replay does not spawn them.
#pragma once
#include "dt_kernels.cuh"

namespace dt {

// One camera path of k_camera's loop, value-only, with adjoint scattering in pass B.
// Must consume the RNG exactly like k_camera: every branch below mirrors it.
// Event values of pass A kept for pass B (per thread): pass B then runs each NEE or
// emitter-hit query once, with the weight known beforehand. Events past the capacity use
// the rewind of the RNG state instead.
constexpr int kReplayEvents = 40;

// State of one replayed camera path between vertices (wavefront schedule: in HBM).
template <int N>
struct alignas(16) AdjState {
    Rng rng;
    RayAD<N> ray;
    ItsAD<N> its;
    float3 P, acc;
    int med, depth, mode, level, ne;  // ne: event index, in path order (identical in both passes)
};

template <int N>
DT_D bool replay_start(const DevScene &sc, const RenderParams &rp, int *stack, long long g, AdjState<N> &st, Ctr &c) {
    const int pixel = (int)(g / rp.spp);
    const int ix = rp.crop_x + pixel % rp.out_w, iy = rp.crop_y + pixel / rp.out_w;
    st.rng.init(rp.seed, (uint64_t)g);
    double jx = 0.5, jy = 0.5;
    if (rp.jitter) {
        jx = st.rng.next1d();
        jy = st.rng.next1d();
    }
    st.ray = camera_ray_ad<N>(sc.cam, ix + jx, iy + jy);
    st.its = ItsAD<N>();
    st.med = sc.cam.med_id;
    st.depth = rp.max_bounces;
    st.mode = rp.mode;
    st.level = 0;
    st.ne = 0;
    st.P = mk(1.f, 1.f, 1.f);
    st.acc = mk(0.f, 0.f, 0.f);
    return ray_intersect_ad<N>(sc, stack, st.ray, false, st.its, c);
}

// One vertex of the replayed path (camera_step's branches, values only). Pass B scatters
// dot(dL/dI, suffix)/spp into the voxels behind every distance-sampling factor and each
// NEE / emitter-hit event's own weight; ev holds pass A's event values. In three parts as
// the camera vertex: replay_decide (random numbers, distance sampling with its scatter),
// then replay_volume or replay_surface.
template <int N>
DT_D int replay_decide(const DevScene &sc, const RenderParams &rp, bool pass_b, float3 total, float3 gpix, AdjCtx &adj,
                       Ctr &c, AdjState<N> &st, VertexIn<N> &vin) {
    Rng &rng = st.rng;
    const float r1a = rng.next1(), r1b = rng.next1();
    vin.r2[0] = rng.next1(); vin.r2[1] = rng.next1(); vin.r2[2] = rng.next1(); vin.r2[3] = rng.next1();
    vin.r3a = rng.next1(); vin.r3b = rng.next1(); vin.r3c = rng.next1();
    vin.thr = DV<N>(mk(1.f, 1.f, 1.f));
    vin.dir_in = st.ray.d.val();
    if (pass_b) adj.w = dot(gpix, total - st.acc) * rp.inv_spp;  // suffix radiance of this factor
    if (st.med >= 0 && sample_distance_ad<N>(sc, sc.media[st.med], st.ray, st.its.t, r1a, r1b, rng, vin.thr, c,
                                             pass_b ? &adj : nullptr))
        return (st.depth == 0 || vin.thr.is_zero()) ? 0 : 1;
    return (!st.its.valid() || vin.thr.is_zero()) ? 0 : 2;
}

template <int N>
DT_D bool replay_volume(const DevScene &sc, const RenderParams &rp, int *stack, bool pass_b, float3 gpix, AdjCtx &adj,
                        Ctr &c, float3 *ev, AdjState<N> &st, const VertexIn<N> &vin) {
    Rng &rng = st.rng;
    RayAD<N> &ray = st.ray;
    ItsAD<N> &its = st.its;
    float3 &P = st.P, &acc = st.acc;
    int &med = st.med, &depth = st.depth, &mode = st.mode, &ne = st.ne;
    const float3 zero = mk(0.f, 0.f, 0.f);
    const AdjCtx *hook = pass_b ? &adj : nullptr;
    const float *r2 = vin.r2;
    const float r3a = vin.r3a, r3b = vin.r3b;
    const DV<N> &thr = vin.thr;
    const float3 dir_in = vin.dir_in;
    bool alive = false;
    // ------------------------------------------------ volumetric vertex
    const DevPhase &ph = sc.phases[sc.media[med].phase_id];
    const float3 Q = cmul(P, thr.val());
    DV<N> wo;
    float pdf_nee;
    if (mode & MODE_VOLUME_MAIN) {
        const int k = ne++;
        if (pass_b && k < kReplayEvents) {
            const float3 e = ev[k];
            adj.w = dot(gpix, e) * rp.inv_spp;
            nee_point_ad<N>(sc, stack, ray.o, r2, rng, med, depth - 1, wo, pdf_nee, c,
                            is_zero3(e, 0.f) ? nullptr : hook);
            acc = acc + e;
        } else {
            const Rng saved = rng;
            DV<N> v = nee_point_ad<N>(sc, stack, ray.o, r2, rng, med, depth - 1, wo, pdf_nee, c);
            float3 e = zero;
            if (!v.is_zero()) {
                const Df<N> pv = phase_eval_ad<N>(ph, -ray.d, wo);
                if (pv.v > kEps)
                    e = cmul(Q, v.val()) * (pv.v * mis_weight(pdf_nee, phase_eval(ph, -dir_in, wo.val())));
            }
            if (pass_b && !is_zero3(e, 0.f)) {
                const Rng after = rng;
                rng = saved;
                adj.w = dot(gpix, e) * rp.inv_spp;
                DV<N> wo2;
                float pdf2;
                nee_point_ad<N>(sc, stack, ray.o, r2, rng, med, depth - 1, wo2, pdf2, c, hook);
                rng = after;
            }
            if (!pass_b && k < kReplayEvents) ev[k] = e;
            acc = acc + e;
        }
    }
    const Df<N> pvs = phase_sample_ad<N>(ph, -ray.d, r3a, r3b, wo);
    if (pvs.v > kEps) {
        const float3 thr1 = thr.val() * pvs.v;
        ray.d = wo;
        ItsAD<N> its1;
        const int k = ne++;
        if (pass_b && k < kReplayEvents) {
            const float3 e = ev[k];
            adj.w = dot(gpix, e) * rp.inv_spp;
            look_for_emitter_ad<N>(sc, stack, ray, false, rng, med, depth - 1, its1, pdf_nee, nullptr, nullptr,
                                   c, is_zero3(e, 0.f) ? nullptr : hook);
            acc = acc + e;
        } else {
            const Rng saved = rng;
            DV<N> att = look_for_emitter_ad<N>(sc, stack, ray, false, rng, med, depth - 1, its1, pdf_nee,
                                               nullptr, nullptr, c);
            float3 e = zero;
            if (!att.is_zero() && (mode & MODE_VOLUME_MAIN))
                e = cmul(cmul(P, thr1), att.val()) * mis_weight(phase_eval(ph, -wo.val(), wo.val()), pdf_nee);
            if (pass_b && !is_zero3(e, 0.f)) {
                const Rng after = rng;
                rng = saved;
                adj.w = dot(gpix, e) * rp.inv_spp;
                ItsAD<N> its2;
                float pdf2;
                look_for_emitter_ad<N>(sc, stack, ray, false, rng, med, depth - 1, its2, pdf2, nullptr, nullptr,
                                       c, hook);
                rng = after;
            }
            if (!pass_b && k < kReplayEvents) ev[k] = e;
            acc = acc + e;
        }
        its = its1;
        P = cmul(P, thr1);
        depth -= 1;
        mode &= ~MODE_EMISSION;
        alive = true;
    }
    return alive;
}

template <int N>
DT_D bool replay_surface(const DevScene &sc, const RenderParams &rp, int *stack, bool pass_b, float3 gpix,
                         AdjCtx &adj, Ctr &c, float3 *ev, AdjState<N> &st, const VertexIn<N> &vin) {
    Rng &rng = st.rng;
    RayAD<N> &ray = st.ray;
    ItsAD<N> &its = st.its;
    float3 &P = st.P, &acc = st.acc;
    int &med = st.med, &depth = st.depth, &mode = st.mode, &ne = st.ne;
    const float3 zero = mk(0.f, 0.f, 0.f);
    const AdjCtx *hook = pass_b ? &adj : nullptr;
    const float *r2 = vin.r2;
    const float r3a = vin.r3a, r3b = vin.r3b, r3c = vin.r3c;
    const DV<N> &thr = vin.thr;
    const float3 dir_in = vin.dir_in;
    bool alive = false;
    // ---------------------------------------------------- interface vertex
    const DevShape &sh = sc.shapes[its.shape];
    if (is_transition(sh) && target_medium(sc, its.shape, its.ng, -dir_in) != med) return false;
    const float3 Q = cmul(P, thr.val());
    if (sh.light_id >= 0 && (mode & MODE_EMISSION)) acc = acc + cmul(Q, le_ad<N>(sc, its, -ray.d).val());
    if (depth == 0) return false;
    const DevBsdf &b = sc.bsdfs[sh.bsdf_id];
    const bool is_null = b.type == BSDF_NULL;
    const FrameAD<N> fr = its.frame();
    const Its its0 = its.plain();
    DV<N> wo;
    float pdf_nee;
    if (!is_null && (mode & MODE_SURFACE_MAIN)) {
        const int k = ne++;
        if (pass_b && k < kReplayEvents) {
            const float3 e = ev[k];
            adj.w = dot(gpix, e) * rp.inv_spp;
            nee_surface_ad<N>(sc, stack, its, fr, r2, rng, med, depth - 1, wo, pdf_nee, c,
                              is_zero3(e, 0.f) ? nullptr : hook, &b);
            acc = acc + e;
        } else {
            const Rng saved = rng;
            DV<N> v = nee_surface_ad<N>(sc, stack, its, fr, r2, rng, med, depth - 1, wo, pdf_nee, c, nullptr, &b);
            float3 e = zero;
            if (!v.is_zero()) {
                const DV<N> bv = bsdf_eval_ad<N>(b, its.wi, wo);
                const float bp = bsdf_pdf(b, its0.wi, wo.val());
                e = cmul(cmul(Q, v.val()), bv.val()) * mis_weight(pdf_nee, bp);
            }
            if (pass_b && !is_zero3(e, 0.f)) {
                const Rng after = rng;
                rng = saved;
                adj.w = dot(gpix, e) * rp.inv_spp;
                DV<N> wo2;
                float pdf2;
                nee_surface_ad<N>(sc, stack, its, fr, r2, rng, med, depth - 1, wo2, pdf2, c, hook, &b);
                rng = after;
            }
            if (!pass_b && k < kReplayEvents) ev[k] = e;
            acc = acc + e;
        }
    }
    float bpdf, beta;
    const DV<N> bw = bsdf_sample_ad<N>(b, its, fr, its0, r3a, r3b, r3c, wo, bpdf, beta);
    if (!bw.is_zero()) {
        wo = fr.to_world(wo);
        if (!is_null) wo = zero_grad(wo);
        ray.o = its.p;
        ray.d = wo;
        const int med1 = is_transition(sh) ? target_medium(sc, its.shape, its.ng, wo.val()) : med;
        float3 thr1 = thr.val();
        ItsAD<N> its1;
        if (is_null) {
            ray_intersect_ad<N>(sc, stack, ray, true, its1, c);
        } else {
            thr1 = cmul(thr1, bw.val());
            const int k = ne++;
            if (pass_b && k < kReplayEvents) {
                const float3 e = ev[k];
                adj.w = dot(gpix, e) * rp.inv_spp;
                look_for_emitter_ad<N>(sc, stack, ray, true, rng, med1, depth - 1, its1, pdf_nee, nullptr, nullptr,
                                       c, is_zero3(e, 0.f) ? nullptr : hook);
                acc = acc + e;
            } else {
                const Rng saved = rng;
                DV<N> att = look_for_emitter_ad<N>(sc, stack, ray, true, rng, med1, depth - 1, its1, pdf_nee,
                                                   nullptr, nullptr, c);
                float3 e = zero;
                if (!att.is_zero() && (mode & MODE_SURFACE_MAIN))
                    e = cmul(cmul(P, thr1), att.val()) * mis_weight(bpdf, pdf_nee);
                if (pass_b && !is_zero3(e, 0.f)) {
                    const Rng after = rng;
                    rng = saved;
                    adj.w = dot(gpix, e) * rp.inv_spp;
                    ItsAD<N> its2;
                    float pdf2;
                    look_for_emitter_ad<N>(sc, stack, ray, true, rng, med1, depth - 1, its2, pdf2, nullptr,
                                           nullptr, c, hook);
                    rng = after;
                }
                if (!pass_b && k < kReplayEvents) ev[k] = e;
                acc = acc + e;
            }
            mode &= ~MODE_EMISSION;
        }
        its = its1;
        P = cmul(P, thr1);
        med = med1;
        depth -= 1;
        alive = true;
    }
    return alive;
}

template <int N>
DT_D bool replay_step(const DevScene &sc, const RenderParams &rp, int *stack, bool pass_b, float3 total, float3 gpix,
                      AdjCtx &adj, Ctr &c, float3 *ev, AdjState<N> &st) {
    VertexIn<N> vin;
    const int kind = replay_decide<N>(sc, rp, pass_b, total, gpix, adj, c, st, vin);
    if (kind == 1) return replay_volume<N>(sc, rp, stack, pass_b, gpix, adj, c, ev, st, vin);
    if (kind == 2) return replay_surface<N>(sc, rp, stack, pass_b, gpix, adj, c, ev, st, vin);
    return false;
}

template <int N>
DT_D float3 replay_path(const DevScene &sc, const RenderParams &rp, int *stack, long long g, bool pass_b, float3 total,
                        float3 gpix, AdjCtx &adj, Ctr &c, float3 *ev) {
    AdjState<N> st;
    bool alive = replay_start<N>(sc, rp, stack, g, st, c);
    while (alive && st.mode != 0) {
        alive = replay_step<N>(sc, rp, stack, pass_b, total, gpix, adj, c, ev, st);
        ++st.level;
    }
    return st.acc;
}

// One camera path (index gi of the launch's range): pass A (value), then pass B (scatter)
// when the path and its pixel's dL/dI are non-zero. img_acc (optional) receives the image,
// FP64 [npix][3]. Contains warp collectives: all 32 lanes of a warp must call it together.
template <int N>
DT_D void adjoint_one(const DevScene &sc, const RenderParams &rp, int *stack, long long gi, const float *dimg,
                      float *grad, double *img_acc, Ctr &c, long long stride = 1) {
    // stride > 1 (autotuning samples): path gi*stride of the range
    const bool active = gi * stride < rp.path_count;
    const long long g = rp.path_begin + (active ? gi * stride : 0);
    const int pixel = (int)(g / rp.spp);
    AdjCtx adj{grad, 0.f};
    float3 ev[kReplayEvents];
    float3 total = mk(0.f, 0.f, 0.f);
    if (active) {
        total = replay_path<N>(sc, rp, stack, g, false, total, total, adj, c, ev);
        if (grad != nullptr && dimg != nullptr && !is_zero3(total, 0.f)) {
            const float3 gp = mk(__ldg(dimg + 3 * (size_t)pixel), __ldg(dimg + 3 * (size_t)pixel + 1),
                                 __ldg(dimg + 3 * (size_t)pixel + 2));
            if (!is_zero3(gp, 0.f)) replay_path<N>(sc, rp, stack, g, true, total, gp, adj, c, ev);
        }
    }
    if (img_acc != nullptr) {
        const unsigned full = 0xffffffffu;
        const int p0 = __shfl_sync(full, pixel, 0);
        const bool uniform = __all_sync(full, active && pixel == p0);
        float v[3] = {total.x * rp.inv_spp, total.y * rp.inv_spp, total.z * rp.inv_spp};
        if (uniform)
            for (int k = 0; k < 3; ++k)
                for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(full, v[k], off);
        if (active && (!uniform || (threadIdx.x & 31) == 0))
            for (int k = 0; k < 3; ++k)
                if (v[k] != 0.f) atomicAdd(img_acc + (size_t)pixel * 3 + k, (double)v[k]);
    }
}

// One thread per camera path of one scene.
template <int N>
__global__ void __launch_bounds__(kBlock) k_adjoint(DevScene sc, RenderParams rp, const float *dimg, float *grad,
                                                    double *img_acc, unsigned long long *ctr, long long stride = 1) {
    __shared__ int s_stack[kStackDepth * kBlock];
    Ctr c;
    adjoint_one<N>(sc, rp, s_stack + threadIdx.x, (long long)blockIdx.x * kBlock + threadIdx.x, dimg, grad, img_acc, c,
                   stride);
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// Wavefront schedule of the replay: pass A and pass B each run one launch per path
// vertex over the paths still alive (compacted path-index queues, as the camera stage).
DT_D float3 pixel_dldi(const RenderParams &rp, const float *dimg, long long g) {
    const int pixel = (int)(g / rp.spp);
    return mk(__ldg(dimg + 3 * (size_t)pixel), __ldg(dimg + 3 * (size_t)pixel + 1), __ldg(dimg + 3 * (size_t)pixel + 2));
}

// After a vertex of level L of one pass: a continuing path runs level L+1's random numbers
// and distance sampling (with pass B's scatter of its factor) and is queued as a volume or
// interface vertex of L+1 (as camera_next).
template <int N>
DT_D void replay_next(const DevScene &sc, const RenderParams &rp, AdjState<N> &st, bool alive, bool pass_b,
                      float3 total, float3 gp, AdjCtx &adj, VertexIn<N> *vins, int id, int *qv,
                      unsigned long long *cnt_v, int *qs, unsigned long long *cnt_s, const QueueEnds &qx, Ctr &c) {
    int kind = 0;
    if (alive && st.mode != 0) {
        VertexIn<N> vin;
        kind = replay_decide<N>(sc, rp, pass_b, total, gp, adj, c, st, vin);
        if (kind) vins[id] = vin;
    }
    // interface vertices from both ends of their queue by BSDF class, as camera_next
    const bool back = kind == 2 && interface_back(sc, st.its.shape);
    push_path(qv, cnt_v, id, kind == 1);
    push_path(qs, cnt_s, id, kind == 2 && !back);
    push_path_back(qs, qx.cap, cnt_s + qx.back, id, back);
}

// Path start and level 0 of one pass, as k_cam_start: an interface vertex runs here and
// the path goes on to level 1's distance sampling, a volume vertex is queued for level 0.
// Pass B starts only paths with a value whose pixel has a non-zero dL/dI.
template <int N>
__global__ void __launch_bounds__(kBlock) k_adj_start(DevScene sc, RenderParams rp, AdjState<N> *states,
                                                      VertexIn<N> *vins, int *qv0, unsigned long long *cnt_v0,
                                                      int *qv1, unsigned long long *cnt_v1, int *qs1,
                                                      unsigned long long *cnt_s1, const float *dimg, float *grad,
                                                      const float3 *totals, float3 *evbuf, QueueEnds qx, bool pass_b,
                                                      unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    int kind = 0;
    bool next = false, run = false;
    AdjState<N> st;
    const float3 zero = mk(0.f, 0.f, 0.f);
    float3 total = zero, gp = zero;
    AdjCtx adj{grad, 0.f};
    if (gi < rp.path_count) {
        const long long g = rp.path_begin + gi;
        if (pass_b) {
            total = totals[gi];
            gp = pixel_dldi(rp, dimg, g);
        }
        run = !pass_b || (!is_zero3(total, 0.f) && !is_zero3(gp, 0.f));
        if (run && replay_start<N>(sc, rp, stack, g, st, c) && st.mode != 0) {
            VertexIn<N> vin;
            kind = replay_decide<N>(sc, rp, pass_b, total, gp, adj, c, st, vin);
            if (kind == 1) vins[gi] = vin;
            if (kind == 2) {
                next = replay_surface<N>(sc, rp, stack, pass_b, gp, adj, c, evbuf + (size_t)gi * kReplayEvents, st, vin);
                ++st.level;
            }
        }
    }
    push_path(qv0, cnt_v0, (int)gi, kind == 1);
    replay_next<N>(sc, rp, st, next, pass_b, total, gp, adj, vins, (int)gi, qv1, cnt_v1, qs1, cnt_s1, qx, c);
    if (run) states[gi] = st;
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// Vertex level of one pass: the volume (kVolume) or interface vertices, each continuing path
// then running level L+1's distance sampling (replay_next).
template <int N, bool kVolume>
__global__ void __launch_bounds__(kBlock) k_adj_vertex(DevScene sc, RenderParams rp, AdjState<N> *states,
                                                       VertexIn<N> *vins, const int *q_in,
                                                       const unsigned long long *cnt_in, int *qv_next,
                                                       unsigned long long *cnt_v_next, int *qs_next,
                                                       unsigned long long *cnt_s_next, const float *dimg, float *grad,
                                                       const float3 *totals, float3 *evbuf, QueueEnds qx, bool pass_b,
                                                       unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long nf = (long long)*cnt_in, n = nf + (kVolume ? 0 : (long long)cnt_in[qx.back]);
    Ctr c;
    for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < n; i += (long long)gridDim.x * kBlock) {
        const int id = i < nf ? q_in[i] : q_in[qx.cap - 1 - (i - nf)];
        AdjState<N> st = states[id];
        const VertexIn<N> vin = vins[id];
        const float3 zero = mk(0.f, 0.f, 0.f);
        const float3 total = pass_b ? totals[id] : zero, gp = pass_b ? pixel_dldi(rp, dimg, rp.path_begin + id) : zero;
        AdjCtx adj{grad, 0.f};
        float3 *ev = evbuf + (size_t)id * kReplayEvents;
        const bool alive = kVolume ? replay_volume<N>(sc, rp, stack, pass_b, gp, adj, c, ev, st, vin)
                                   : replay_surface<N>(sc, rp, stack, pass_b, gp, adj, c, ev, st, vin);
        ++st.level;
        replay_next<N>(sc, rp, st, alive, pass_b, total, gp, adj, vins, id, qv_next, cnt_v_next, qs_next, cnt_s_next,
                       qx, c);
        states[id] = st;
    }
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// after pass A: each path's value (pass B's suffix base) and the image sum in path order
template <int N>
__global__ void __launch_bounds__(kBlock) k_adj_totals(RenderParams rp, const AdjState<N> *states, float3 *totals,
                                                       double *img_acc) {
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < rp.path_count;
    const long long g = rp.path_begin + (active ? gi : 0);
    const int pixel = (int)(g / rp.spp);
    float3 total = mk(0.f, 0.f, 0.f);
    if (active) {
        total = states[gi].acc;
        totals[gi] = total;
    }
    if (img_acc != nullptr) {
        const unsigned full = 0xffffffffu;
        const int p0 = __shfl_sync(full, pixel, 0);
        const bool uniform = __all_sync(full, active && pixel == p0);
        float v[3] = {total.x * rp.inv_spp, total.y * rp.inv_spp, total.z * rp.inv_spp};
        if (uniform)
            for (int k = 0; k < 3; ++k)
                for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(full, v[k], off);
        if (active && (!uniform || (threadIdx.x & 31) == 0))
            for (int k = 0; k < 3; ++k)
                if (v[k] != 0.f) atomicAdd(img_acc + (size_t)pixel * 3 + k, (double)v[k]);
    }
}

// Image write rule of integratorAD.cpp:59-87 (a pixel is written only if non-negative).
static __global__ void k_adjoint_image(int npix, const double *acc, float *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const double *a = acc + (size_t)p * 3;
    const bool nonneg = a[0] >= 0.0 && a[1] >= 0.0 && a[2] >= 0.0;
    for (int c = 0; c < 3; ++c) out[(size_t)p * 3 + c] = nonneg ? (float)a[c] : 0.f;
}

// ====================================================================== batched wavefront
// The replay of many scenes as one wavefront (batch schedule of dt_batch.cu): the camera
// paths of all items are numbered item after item (gbeg[i]: the first global path of the
// i-th item of `order`), a workspace of `count` consecutive global paths runs pass A and
// pass B as above, and every level launch covers the live paths of all items at once. A
// thread finds its path's item by binary search over gbeg and reads that item's scene and
// parameters from global memory. With stride > 1 (tuning), global path k of an item is
// its path k * stride.
struct BatchItemDev {
    DevScene sc;
    RenderParams rp;
    const float *dimg;
    float *grad;
    double *img_acc;
};

struct BatchWave {
    const BatchItemDev *items;
    const long long *gbeg;  // n + 1 entries
    const int *order;
    int n;
    long long begin, count;  // global paths of this workspace: [begin, begin + count)
    long long stride;
};

// item of workspace slot i and its local path index
DT_D const BatchItemDev &batch_item(const BatchWave &bw, long long i, long long &g) {
    const long long G = bw.begin + i;
    int lo = 0, hi = bw.n - 1;  // largest position with gbeg <= G
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bw.gbeg[mid] <= G) lo = mid;
        else hi = mid - 1;
    }
    g = (G - bw.gbeg[lo]) * bw.stride;
    return bw.items[bw.order[lo]];
}

template <int N>
__global__ void __launch_bounds__(kBlock) k_badj_start(BatchWave bw, AdjState<N> *states, VertexIn<N> *vins, int *qv0,
                                                       unsigned long long *cnt_v0, int *qv1,
                                                       unsigned long long *cnt_v1, int *qs1,
                                                       unsigned long long *cnt_s1, const float3 *totals,
                                                       float3 *evbuf, QueueEnds qx, bool pass_b) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < bw.count;
    long long g = 0;
    const BatchItemDev &it = batch_item(bw, active ? gi : 0, g);
    Ctr c;
    int kind = 0;
    bool next = false, run = false;
    AdjState<N> st;
    const float3 zero = mk(0.f, 0.f, 0.f);
    float3 total = zero, gp = zero;
    AdjCtx adj{it.grad, 0.f};
    if (active) {
        if (pass_b && it.grad) {
            total = totals[gi];
            gp = pixel_dldi(it.rp, it.dimg, g);
        }
        run = !pass_b || (it.grad && !is_zero3(total, 0.f) && !is_zero3(gp, 0.f));
        if (run && replay_start<N>(it.sc, it.rp, stack, g, st, c) && st.mode != 0) {
            VertexIn<N> vin;
            kind = replay_decide<N>(it.sc, it.rp, pass_b, total, gp, adj, c, st, vin);
            if (kind == 1) vins[gi] = vin;
            if (kind == 2) {
                next = replay_surface<N>(it.sc, it.rp, stack, pass_b, gp, adj, c, evbuf + (size_t)gi * kReplayEvents,
                                         st, vin);
                ++st.level;
            }
        }
    }
    push_path(qv0, cnt_v0, (int)gi, kind == 1);
    replay_next<N>(it.sc, it.rp, st, next, pass_b, total, gp, adj, vins, (int)gi, qv1, cnt_v1, qs1, cnt_s1, qx,
                   c);
    if (run) states[gi] = st;
}

template <int N, bool kVolume>
__global__ void __launch_bounds__(kBlock) k_badj_vertex(BatchWave bw, AdjState<N> *states, VertexIn<N> *vins,
                                                        const int *q_in, const unsigned long long *cnt_in,
                                                        int *qv_next, unsigned long long *cnt_v_next, int *qs_next,
                                                        unsigned long long *cnt_s_next, const float3 *totals,
                                                        float3 *evbuf, QueueEnds qx, bool pass_b) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long nf = (long long)*cnt_in, n = nf + (kVolume ? 0 : (long long)cnt_in[qx.back]);
    Ctr c;
    for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < n; i += (long long)gridDim.x * kBlock) {
        const int id = i < nf ? q_in[i] : q_in[qx.cap - 1 - (i - nf)];
        long long g;
        const BatchItemDev &it = batch_item(bw, id, g);
        AdjState<N> st = states[id];
        const VertexIn<N> vin = vins[id];
        const float3 zero = mk(0.f, 0.f, 0.f);
        const float3 total = pass_b ? totals[id] : zero, gp = pass_b ? pixel_dldi(it.rp, it.dimg, g) : zero;
        AdjCtx adj{it.grad, 0.f};
        float3 *ev = evbuf + (size_t)id * kReplayEvents;
        const bool alive = kVolume ? replay_volume<N>(it.sc, it.rp, stack, pass_b, gp, adj, c, ev, st, vin)
                                   : replay_surface<N>(it.sc, it.rp, stack, pass_b, gp, adj, c, ev, st, vin);
        ++st.level;
        replay_next<N>(it.sc, it.rp, st, alive, pass_b, total, gp, adj, vins, id, qv_next, cnt_v_next, qs_next,
                       cnt_s_next, qx, c);
        states[id] = st;
    }
}

// after pass A: each path's value and its item's image sum (a warp whose lanes share one
// item and pixel reduces with shuffles first)
template <int N>
__global__ void __launch_bounds__(kBlock) k_badj_totals(BatchWave bw, const AdjState<N> *states, float3 *totals) {
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < bw.count;
    long long g = 0;
    const BatchItemDev &it = batch_item(bw, active ? gi : 0, g);
    const int pixel = (int)(g / it.rp.spp);
    float3 total = mk(0.f, 0.f, 0.f);
    if (active) {
        total = states[gi].acc;
        totals[gi] = total;
    }
    const unsigned full = 0xffffffffu;
    const unsigned long long key = ((unsigned long long)(&it - bw.items) << 32) | (unsigned)pixel;
    const unsigned long long k0 = __shfl_sync(full, key, 0);
    const bool uniform = __all_sync(full, active && key == k0);
    float v[3] = {total.x * it.rp.inv_spp, total.y * it.rp.inv_spp, total.z * it.rp.inv_spp};
    if (uniform)
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(full, v[k], off);
    if (active && it.img_acc && (!uniform || (threadIdx.x & 31) == 0))
        for (int k = 0; k < 3; ++k)
            if (v[k] != 0.f) atomicAdd(it.img_acc + (size_t)pixel * 3 + k, (double)v[k]);
}

}  // namespace dt
