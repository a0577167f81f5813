// dtrt_gb300 — forward-mode render kernels (templated on the derivative width N).
//
// The reference evaluates VolPathTracerAD::LiAD (volpathAD.cpp:145-620) recursively and
// estimates its boundary terms inline, each edge sample tracing two full Li sub-paths.
// Every contribution is additive into the pixel with a weight known when it is spawned,
// so the recursion flattens into task queues:
//
//   camera     the LiAD chain of a camera path sample as a loop of vertices carrying a
//              dual prefix throughput; emits EdgeRec (surface / volume edge term) and
//              LinsRec (Lins interface term) records instead of recursing. Megakernel
//              k_camera (one thread per path) or wavefront k_cam_start / k_cam_vertex /
//              k_cam_accum (one launch per vertex kind and level over the compacted paths
//              of that kind, each ending with the next level's distance sampling)
//   k_edge     one thread per (edge record, edge sample): FP64 silhouette test and
//              edge-point solve, the visibility gate, then two LiTask sub-paths
//   k_lins     one thread per Lins record: the Lins estimate with its Li sub-paths
//   k_primary  one thread per primary-edge sample (integratorAD.cpp:100-165), samples
//              taken in the order of their edge-selecting random number (k_primary_keys)
//   k_li       one thread per LiTask: the non-AD path Li (volpathAD.cpp:50-142), whose
//              result L adds s_j * w_c * L_c to derivative slot j of its pixel; the two
//              sub-paths of a sample sit in adjacent slots and the pairs are read in the
//              order of their origin / direction cell (k_li_keys + radix sort)
//   k_finalize FP64 accumulators -> float image with the reference's write rules
//
// All pushes are warp-aggregated (ballot + popc, one atomic per warp); a push past a
// queue's capacity sets an error flag and is dropped, never written out of bounds.
#pragma once
#include "dt_device.cuh"

namespace dt {

struct RenderParams {
    uint64_t seed;
    int spp, max_bounces, sppse, mode, jitter;
    float ddist, inv_spp;
    int npix, out_w, out_h, crop_x, crop_y;
    long long path_begin, path_count;
    double prim_weight;  // primary-edge PDF sum / sample count
    double inv_sppse;    // 1 / sppse (0 when sppse is 0)
    long long prim_begin, prim_count;
};

template <int N>
struct EdgeRec {
    float x0[3], x0d[N][3];
    float w[3];      // prefix throughput value / spp
    float wi[3];     // surface: local incident direction; volume: world -ray.dir
    float fs[3], ft[3], fn[3], ng[3];
    int kind, shape, med, phase, depth, pixel;
    uint64_t key;
};

template <int N>
struct LinsRec {
    float p[3], ng[3], n[3], rd[3], fs[3], ft[3], fn[3], wi[3];
    float w[3];      // prefix throughput * sigma_s / (spp * nsamples)
    float s[N];      // hit-distance derivative slots
    int shape, med, phase, depth, pixel, ns;
    uint64_t key;
};

template <int N>
struct LiTask {
    float o[3], d[3], w[3], s[N];
    int med, depth, pixel, flags;  // flags: bit0 include emission, bit1 primary-edge image
    uint64_t key;
};

struct Queue {
    void *data;
    unsigned long long *count;
    unsigned long long cap;
};

// Counter slots: [kernel][rays, nodes, tris, lookups, light samples] then three task counts
enum { K_CAMERA = 0, K_EDGE, K_LI, K_LINS, K_PRIMARY };
constexpr int kCtrPerKernel = 5;
enum { CT_EDGE_SAMPLES = 5 * kCtrPerKernel, CT_LI, CT_PRIMARY, CT_NUM };
// device counter buffer: 8 queue / scratch counts, then the CT_NUM work counters
constexpr int kCountSlots = 64;
static_assert(8 + CT_NUM <= kCountSlots, "counter slots");

DT_D void flush_counters(unsigned long long *ctr, int kernel, const Ctr &c, uint32_t extra_slot = 0xffffffffu,
                         uint32_t extra = 0) {
    if (!ctr) return;
    unsigned long long v[kCtrPerKernel] = {c.rays, c.nodes, c.tris, c.lookups, c.lights};
    const unsigned mask = __activemask();
    bool lead = true;
    if (mask == 0xffffffffu) {  // full warp: reduce with shuffles, one atomic per counter
#pragma unroll
        for (int k = 0; k < kCtrPerKernel; ++k) {
            unsigned long long x = v[k];
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(mask, x, off);
            v[k] = x;
        }
        lead = (threadIdx.x & 31) == 0;
    }
    if (lead)
        for (int k = 0; k < kCtrPerKernel; ++k)
            if (v[k]) atomicAdd(ctr + kCtrPerKernel * kernel + k, v[k]);
    if (extra_slot != 0xffffffffu && extra) atomicAdd(ctr + extra_slot, (unsigned long long)extra);
}

// warp-aggregated slot reservation: returns the slot index or -1 on overflow
DT_D long long queue_reserve(const DevScene &sc, const Queue &q) {
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const unsigned rank = __popc(mask & ((1u << lane) - 1u));
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(q.count, (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    const unsigned long long slot = base + rank;
    if (slot >= q.cap) {
        set_error(sc, ERR_QUEUE);
        return -1;
    }
    return (long long)slot;
}

// warp-aggregated reservation of k consecutive slots per calling lane: returns the first
// slot, or -1 (and the overflow flag) when they do not all fit
DT_D long long queue_reserve_n(const DevScene &sc, const Queue &q, unsigned k) {
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const unsigned rank = __popc(mask & ((1u << lane) - 1u));
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(q.count, (unsigned long long)__popc(mask) * k);
    base = __shfl_sync(mask, base, leader);
    const unsigned long long slot = base + (unsigned long long)rank * k;
    if (slot + k > q.cap) {
        set_error(sc, ERR_QUEUE);
        return -1;
    }
    return (long long)slot;
}

// camera.cpp:52-60 / 75-83 / 40-50
DT_D void camera_ray(const DevCamera &cam, double x, double y, float3 &o, float3 &d) {
    const float3 ndc = mk((float)((x * cam.inv_w - 0.5) * 2.0), (float)((y * cam.inv_h - 0.5) * cam.ndc_ky), 1.f);
    const float *m = cam.ndc2cam;
    float3 dc = normalize(mk(m[0] * ndc.x + m[1] * ndc.y + m[2] * ndc.z, m[3] * ndc.x + m[4] * ndc.y + m[5] * ndc.z,
                             m[6] * ndc.x + m[7] * ndc.y + m[8] * ndc.z));
    const float *c = cam.c2w;
    o = mk(c[3], c[7], c[11]);
    d = mk(c[0] * dc.x + c[1] * dc.y + c[2] * dc.z, c[4] * dc.x + c[5] * dc.y + c[6] * dc.z,
           c[8] * dc.x + c[9] * dc.y + c[10] * dc.z);
}
template <int N>
DT_D RayAD<N> camera_ray_ad(const DevCamera &cam, double x, double y) {
    const float3 ndc = mk((float)((x * cam.inv_w - 0.5) * 2.0), (float)((y * cam.inv_h - 0.5) * cam.ndc_ky), 1.f);
    const float *m = cam.ndc2cam;
    const float3 dc = normalize(mk(m[0] * ndc.x + m[1] * ndc.y + m[2] * ndc.z,
                                   m[3] * ndc.x + m[4] * ndc.y + m[5] * ndc.z,
                                   m[6] * ndc.x + m[7] * ndc.y + m[8] * ndc.z));
    RayAD<N> r;
    r.o = DV<N>(f3(cam.cpos));
    DV<N> s(f3(cam.cframe[0])), t(f3(cam.cframe[1])), n(f3(cam.cframe[2]));
#pragma unroll
    for (int j = 0; j < N; ++j) {
        r.o.set_grad(j, f3(cam.d_cpos[j]));
        s.set_grad(j, f3(cam.d_cframe[j][0]));
        t.set_grad(j, f3(cam.d_cframe[j][1]));
        n.set_grad(j, f3(cam.d_cframe[j][2]));
    }
    r.d = s * dc.x + t * dc.y + n * dc.z;
    return r;
}

// ====================================================================== camera AD paths
// State of one camera path between vertices (volpathAD.cpp:145-620 as a loop): the
// megakernel keeps it in registers, the wavefront schedule in HBM between launches.
template <int N>
struct alignas(16) CamState {  // 16-byte aligned: whole-state copies compile to 128-bit loads and stores
    Rng rng;
    RayAD<N> ray;
    ItsAD<N> its;
    DV<N> P, acc;
    int med, depth, mode, level;
};

// Path start: jittered primary ray and first intersection. False: nothing was hit.
template <int N>
DT_D bool camera_start(const DevScene &sc, const RenderParams &rp, int *stack, long long g, CamState<N> &st, Ctr &c) {
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
    st.P = DV<N>(mk(1.f, 1.f, 1.f));
    st.acc = DV<N>();
    return ray_intersect_ad<N>(sc, stack, st.ray, false, st.its, c);
}

// Random numbers of a vertex drawn before its branch, the distance-sampling throughput and
// the incoming direction: what the volume and interface halves of a vertex share.
template <int N>
struct alignas(16) VertexIn {
    float r2[4], r3a, r3b, r3c;
    DV<N> thr;
    float3 dir_in;
};

// First part of a vertex of camera path g (volpathAD.cpp:160-164, 306-308): the vertex's
// random numbers and distance sampling. 0: the path ends here, 1: volume vertex, 2:
// interface vertex.
template <int N>
DT_D int camera_decide(const DevScene &sc, CamState<N> &st, VertexIn<N> &vin, Ctr &c) {
    Rng &rng = st.rng;
    const float r1a = rng.next1(), r1b = rng.next1();
    vin.r2[0] = rng.next1(); vin.r2[1] = rng.next1(); vin.r2[2] = rng.next1(); vin.r2[3] = rng.next1();
    vin.r3a = rng.next1(); vin.r3b = rng.next1(); vin.r3c = rng.next1();
    vin.thr = DV<N>(mk(1.f, 1.f, 1.f));
    vin.dir_in = st.ray.d.val();
    if (st.med >= 0 && sample_distance_ad<N>(sc, sc.media[st.med], st.ray, st.its.t, r1a, r1b, rng, vin.thr, c))
        return (st.depth == 0 || vin.thr.is_zero()) ? 0 : 1;
    return (!st.its.valid() || vin.thr.is_zero()) ? 0 : 2;
}

// Volume vertex (volpathAD.cpp:164-305): NEE, volume edge record, phase sampling and the
// emitter lookup along the new direction. Returns whether the path continues.
template <int N>
DT_D bool camera_volume(const DevScene &sc, const RenderParams &rp, int *stack, long long g, CamState<N> &st,
                        const VertexIn<N> &vin, const Queue &qe, Ctr &c) {
    Rng &rng = st.rng;
    RayAD<N> &ray = st.ray;
    ItsAD<N> &its = st.its;
    DV<N> &P = st.P, &acc = st.acc;
    int &med = st.med, &depth = st.depth, &mode = st.mode;
    const int level = st.level;
    const int pixel = (int)(g / rp.spp);
    const uint64_t key = (uint64_t)g;
    const float *r2 = vin.r2;
    const float r3a = vin.r3a, r3b = vin.r3b;
    const DV<N> &thr = vin.thr;
    const float3 dir_in = vin.dir_in;
    bool alive = false;
    // ------------------------------------------------ volumetric vertex, volpathAD.cpp:164-305
    const DevPhase &ph = sc.phases[sc.media[med].phase_id];
    const DV<N> Q = cmul(P, thr);
    DV<N> wo;
    float pdf_nee;
    if (mode & MODE_VOLUME_MAIN) {
        DV<N> v = nee_point_ad<N>(sc, stack, ray.o, r2, rng, med, depth - 1, wo, pdf_nee, c);
        if (!v.is_zero()) {
            Df<N> pv = phase_eval_ad<N>(ph, -ray.d, wo);
            if (pv.v > kEps) acc += cmul(Q, v) * (pv * mis_weight(pdf_nee, phase_eval(ph, -dir_in, wo.val())));
        }
    }
    // edge record before the continuation overwrites the vertex state
    if (rp.sppse > 0 && (mode & MODE_VOLUME_BOUNDARY2) && sc.has_edges &&
        (sc.moving_geometry || !ray.o.der_zero(0.f))) {
        const long long slot = queue_reserve(sc, qe);
        if (slot >= 0) {
            EdgeRec<N> &r = reinterpret_cast<EdgeRec<N> *>(qe.data)[slot];
            const float3 x = ray.o.val(), w = cmul(P.val(), thr.val()) * rp.inv_spp, wi = -dir_in;
            r.x0[0] = x.x; r.x0[1] = x.y; r.x0[2] = x.z;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const float3 gj = ray.o.grad(j);
                r.x0d[j][0] = gj.x; r.x0d[j][1] = gj.y; r.x0d[j][2] = gj.z;
            }
            r.w[0] = w.x; r.w[1] = w.y; r.w[2] = w.z;
            r.wi[0] = wi.x; r.wi[1] = wi.y; r.wi[2] = wi.z;
            r.kind = 1; r.shape = -1; r.med = med; r.phase = sc.media[med].phase_id;
            r.depth = depth - 1; r.pixel = pixel; r.key = child_key(key, 1u, (uint32_t)level);
        }
    }
    const Df<N> pvs = phase_sample_ad<N>(ph, -ray.d, r3a, r3b, wo);
    if (pvs.v > kEps) {
        const DV<N> thr1 = thr * pvs;
        ray.d = wo;
        ItsAD<N> its1;
        DV<N> att = look_for_emitter_ad<N>(sc, stack, ray, false, rng, med, depth - 1, its1, pdf_nee, nullptr,
                                           nullptr, c);
        if (!att.is_zero() && (mode & MODE_VOLUME_MAIN))
            acc += cmul(cmul(P, thr1), att) * mis_weight(phase_eval(ph, -wo.val(), wo.val()), pdf_nee);
        its = its1;
        P = cmul(P, thr1);
        depth -= 1;
        mode &= ~MODE_EMISSION;
        alive = true;
    }
    return alive;
}

// Interface vertex (volpathAD.cpp:306-617): emission, Lins and surface edge records, NEE,
// BSDF sampling and the emitter lookup (or null-interface crossing). Returns whether the
// path continues.
template <int N>
DT_D bool camera_surface(const DevScene &sc, const RenderParams &rp, int *stack, long long g, CamState<N> &st,
                         const VertexIn<N> &vin, const Queue &qe, const Queue &ql, Ctr &c) {
    Rng &rng = st.rng;
    RayAD<N> &ray = st.ray;
    ItsAD<N> &its = st.its;
    DV<N> &P = st.P, &acc = st.acc;
    int &med = st.med, &depth = st.depth, &mode = st.mode;
    const int level = st.level;
    const int pixel = (int)(g / rp.spp);
    const uint64_t key = (uint64_t)g;
    const float *r2 = vin.r2;
    const float r3a = vin.r3a, r3b = vin.r3b, r3c = vin.r3c;
    const DV<N> &thr = vin.thr;
    const float3 dir_in = vin.dir_in;
    bool alive = false;
    // ---------------------------------------------------- interface vertex, volpathAD.cpp:306-617
    const DevShape &sh = sc.shapes[its.shape];
    if (is_transition(sh) && target_medium(sc, its.shape, its.ng, -dir_in) != med) return false;
    const DV<N> Q = cmul(P, thr);
    if (sh.light_id >= 0 && (mode & MODE_EMISSION)) acc += cmul(Q, le_ad<N>(sc, its, -ray.d));
    if (depth == 0) return false;
    const DevBsdf &b = sc.bsdfs[sh.bsdf_id];
    const bool is_null = b.type == BSDF_NULL;
    const FrameAD<N> fr = its.frame();
    const Its its0 = its.plain();
    // Lins boundary term, volpathAD.cpp:321-467
    if (med >= 0 && !its.t.der_zero(kDerZeroEps) && (mode & MODE_VOLUME_BOUNDARY1)) {
        const long long slot = queue_reserve(sc, ql);
        if (slot >= 0) {
            LinsRec<N> &r = reinterpret_cast<LinsRec<N> *>(ql.data)[slot];
            float3 n = its0.ng;
            if (dot(n, dir_in) < 0.f) n = -n;
            const int ns = min(max((int)(rp.ddist * its.t.der_max()), 1), 100);
            const float3 sig = sig_s(sc.media[med], its0.p - n * kShadowEps, c);
            const float3 w = cmul(cmul(P.val(), thr.val()), sig) * (rp.inv_spp / (float)ns);
            const float3 *src[8] = {&its0.p, &its0.ng, &n, &dir_in, &its0.fr.s, &its0.fr.t, &its0.fr.n, &its0.wi};
            float *dst[8] = {r.p, r.ng, r.n, r.rd, r.fs, r.ft, r.fn, r.wi};
            for (int k = 0; k < 8; ++k) { dst[k][0] = src[k]->x; dst[k][1] = src[k]->y; dst[k][2] = src[k]->z; }
            r.w[0] = w.x; r.w[1] = w.y; r.w[2] = w.z;
#pragma unroll
            for (int j = 0; j < N; ++j) r.s[j] = its.t.d[j];
            r.shape = its.shape; r.med = med; r.phase = sc.media[med].phase_id; r.depth = depth;
            r.pixel = pixel; r.ns = ns; r.key = child_key(key, 2u, (uint32_t)level);
        }
    }
    // interface edge record, volpathAD.cpp:513-616
    if (!is_null && rp.sppse > 0 && (mode & MODE_SURFACE_BOUNDARY) && sc.has_edges &&
        (sc.moving_geometry || !its.p.der_zero(0.f))) {
        const long long slot = queue_reserve(sc, qe);
        if (slot >= 0) {
            EdgeRec<N> &r = reinterpret_cast<EdgeRec<N> *>(qe.data)[slot];
            const float3 x = its0.p, w = cmul(P.val(), thr.val()) * rp.inv_spp;
            r.x0[0] = x.x; r.x0[1] = x.y; r.x0[2] = x.z;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const float3 gj = its.p.grad(j);
                r.x0d[j][0] = gj.x; r.x0d[j][1] = gj.y; r.x0d[j][2] = gj.z;
            }
            r.w[0] = w.x; r.w[1] = w.y; r.w[2] = w.z;
            r.wi[0] = its0.wi.x; r.wi[1] = its0.wi.y; r.wi[2] = its0.wi.z;
            r.fs[0] = its0.fr.s.x; r.fs[1] = its0.fr.s.y; r.fs[2] = its0.fr.s.z;
            r.ft[0] = its0.fr.t.x; r.ft[1] = its0.fr.t.y; r.ft[2] = its0.fr.t.z;
            r.fn[0] = its0.fr.n.x; r.fn[1] = its0.fr.n.y; r.fn[2] = its0.fr.n.z;
            r.ng[0] = its0.ng.x; r.ng[1] = its0.ng.y; r.ng[2] = its0.ng.z;
            r.kind = 0; r.shape = its.shape; r.med = med; r.phase = -1;
            r.depth = depth - 1; r.pixel = pixel; r.key = child_key(key, 3u, (uint32_t)level);
        }
    }
    // area sampling, volpathAD.cpp:469-511
    DV<N> wo;
    float pdf_nee;
    if (!is_null && (mode & MODE_SURFACE_MAIN)) {
        DV<N> v = nee_surface_ad<N>(sc, stack, its, fr, r2, rng, med, depth - 1, wo, pdf_nee, c, nullptr, &b);
        if (!v.is_zero()) {
            const DV<N> bv = bsdf_eval_ad<N>(b, its.wi, wo);
            const float bp = bsdf_pdf(b, its0.wi, wo.val());
            acc += cmul(cmul(Q, v), bv) * mis_weight(pdf_nee, bp);
        }
    }
    float bpdf, beta;
    const DV<N> bw = bsdf_sample_ad<N>(b, its, fr, its0, r3a, r3b, r3c, wo, bpdf, beta);
    if (!bw.is_zero()) {
        wo = fr.to_world(wo);
        if (!is_null) wo = zero_grad(wo);  // asserted zero in the reference (volpathAD.cpp:489)
        ray.o = its.p;
        ray.d = wo;
        const int med1 = is_transition(sh) ? target_medium(sc, its.shape, its.ng, wo.val()) : med;
        DV<N> thr1 = thr;
        ItsAD<N> its1;
        if (is_null) {
            ray_intersect_ad<N>(sc, stack, ray, true, its1, c);
        } else {
            DV<N> att = look_for_emitter_ad<N>(sc, stack, ray, true, rng, med1, depth - 1, its1, pdf_nee,
                                               nullptr, nullptr, c);
            thr1 = cmul(thr1, bw);
            if (!att.is_zero() && (mode & MODE_SURFACE_MAIN))
                acc += cmul(cmul(P, thr1), att) * mis_weight(bpdf, pdf_nee);
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

// One vertex of camera path g. Returns whether the path continues; st.level is advanced
// by the caller.
template <int N>
DT_D bool camera_step(const DevScene &sc, const RenderParams &rp, int *stack, long long g, CamState<N> &st,
                      const Queue &qe, const Queue &ql, Ctr &c) {
    VertexIn<N> vin;
    const int kind = camera_decide<N>(sc, st, vin, c);
    if (kind == 1) return camera_volume<N>(sc, rp, stack, g, st, vin, qe, c);
    if (kind == 2) return camera_surface<N>(sc, rp, stack, g, st, vin, qe, ql, c);
    return false;
}

// FP64 pixel accumulation of a path's contribution (already divided by spp): a warp
// whose 32 lanes share one pixel reduces with shuffles first. Every lane of the warp calls it.
template <int N>
DT_D void accumulate_path(const RenderParams &rp, bool active, int pixel, const DV<N> &acc, double *acc1) {
    const unsigned full = 0xffffffffu;
    const int p0 = __shfl_sync(full, pixel, 0);
    const bool uniform = __all_sync(full, active && pixel == p0);
    float vals[3 * (N + 1)];
    vals[0] = acc.x.v; vals[1] = acc.y.v; vals[2] = acc.z.v;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        vals[3 * (j + 1)] = acc.x.d[j];
        vals[3 * (j + 1) + 1] = acc.y.d[j];
        vals[3 * (j + 1) + 2] = acc.z.d[j];
    }
    if (uniform) {
#pragma unroll
        for (int k = 0; k < 3 * (N + 1); ++k) {
            float x = vals[k];
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(full, x, off);
            vals[k] = x;
        }
    }
    if (active && (!uniform || (threadIdx.x & 31) == 0)) {
#pragma unroll
        for (int k = 0; k < 3 * (N + 1); ++k) {
            if (vals[k] != 0.f) atomicAdd(acc1 + ((size_t)(k / 3) * rp.npix + pixel) * 3 + (k % 3), (double)vals[k]);
        }
    }
}

// Megakernel schedule: one thread runs its camera path to the end.
template <int N>
__global__ void __launch_bounds__(kBlock) k_camera(DevScene sc, RenderParams rp, Queue qe, Queue ql, double *acc1,
                                                   unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < rp.path_count;
    const long long g = rp.path_begin + (active ? gi : 0);
    Ctr c;
    DV<N> acc;
    if (active) {
        CamState<N> st;
        bool alive = camera_start<N>(sc, rp, stack, g, st, c);
        while (alive && st.mode != 0) {
            alive = camera_step<N>(sc, rp, stack, g, st, qe, ql, c);
            ++st.level;
        }
        acc = st.acc * rp.inv_spp;
    }
    accumulate_path<N>(rp, active, (int)(g / rp.spp), acc, acc1);
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// AUTO schedule: the wavefront from this many camera paths per render batch
constexpr long long kWavefrontMinPaths = 1 << 16;

// Wavefront schedule: paths that continue are compacted into a queue of path indices
// after every vertex, so each launch runs one vertex of live paths only (a warp no longer
// idles on the paths of its lanes that ended early).
DT_D void push_path(int *q, unsigned long long *count, int id, bool pred) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, pred);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(act, base, leader);
    if (pred) q[base + __popc(m & ((1u << lane) - 1u))] = id;  // at most one push per path and level
}

// A level's two-ended interface queue: `cap` slots, and the count of the back end `back`
// entries after the count of the front end
struct QueueEnds {
    long long cap;
    int back;
};

// push from the back of a queue of `cap` slots: entry k at q[cap - 1 - k]
DT_D void push_path_back(int *q, long long cap, unsigned long long *count, int id, bool pred) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, pred);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(act, base, leader);
    if (pred) q[cap - 1 - (long long)(base + __popc(m & ((1u << lane) - 1u)))] = id;
}

// Interface vertices of a level share one queue of `cap` slots: a hit on a diffuse or Phong
// surface is pushed from the front, a hit on a null or rough-dielectric surface from the
// back, so that the warps of the level's launch run one BSDF's branches (at most one warp
// mixes them). Each path is pushed at most once per level: the two ends never meet.
DT_D bool interface_back(const DevScene &sc, int shape) {
    const int t = sc.bsdfs[sc.shapes[shape].bsdf_id].type;
    return t == BSDF_NULL || t == BSDF_ROUGHDIELECTRIC;
}

// After a vertex of level L: a continuing path draws the random numbers and samples the
// distance of level L+1 right away and is queued as a volume or interface vertex of L+1.
template <int N>
DT_D int camera_next(const DevScene &sc, CamState<N> &st, bool alive, VertexIn<N> *vins, int id, int *qv,
                     unsigned long long *cnt_v, int *qs, unsigned long long *cnt_s, unsigned long long *cnt_s_back,
                     long long cap, Ctr &c) {
    int kind = 0;
    if (alive && st.mode != 0) {
        VertexIn<N> vin;
        kind = camera_decide<N>(sc, st, vin, c);
        if (kind) vins[id] = vin;
    }
    const bool back = kind == 2 && interface_back(sc, st.its.shape);
    push_path(qv, cnt_v, id, kind == 1);
    push_path(qs, cnt_s, id, kind == 2 && !back);
    push_path_back(qs, cap, cnt_s_back, id, back);
    return kind;
}

// The path state its next launch reads: all of it before an interface vertex; all but the
// hit record before a volume vertex (which writes the record without reading it); the sums
// alone when the path has ended (k_cam_accum reads nothing else).
template <int N>
DT_D void store_state(CamState<N> *states, int id, const CamState<N> &st, int next_kind) {
    CamState<N> &d = states[id];
    if (next_kind == 2) {
        d = st;
        return;
    }
    d.acc = st.acc;
    if (next_kind == 0) return;
    d.rng = st.rng;
    d.ray = st.ray;
    d.P = st.P;
    d.med = st.med;
    d.depth = st.depth;
    d.mode = st.mode;
    d.level = st.level;
}

// Path start and level 0: primary ray, first hit, the level's random numbers and distance
// sampling. An interface vertex (every path from a camera outside media) runs here too and
// the path goes on to level 1's distance sampling; a volume vertex is queued for level 0.
template <int N>
__global__ void __launch_bounds__(kBlock) k_cam_start(DevScene sc, RenderParams rp, CamState<N> *states,
                                                      VertexIn<N> *vins, int *qv0, unsigned long long *cnt_v0,
                                                      int *qv1, unsigned long long *cnt_v1, int *qs1,
                                                      unsigned long long *cnt_s1, unsigned long long *cnt_s1_back,
                                                      long long cap, Queue qe, Queue ql, unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    int kind = 0;
    CamState<N> st;
    bool next = false;
    if (gi < rp.path_count) {
        const long long g = rp.path_begin + gi;
        if (camera_start<N>(sc, rp, stack, g, st, c) && st.mode != 0) {
            VertexIn<N> vin;
            kind = camera_decide<N>(sc, st, vin, c);
            if (kind == 1) vins[gi] = vin;
            if (kind == 2) {
                next = camera_surface<N>(sc, rp, stack, g, st, vin, qe, ql, c);
                ++st.level;
            }
        }
    }
    push_path(qv0, cnt_v0, (int)gi, kind == 1);
    const int nk = camera_next<N>(sc, st, next, vins, (int)gi, qv1, cnt_v1, qs1, cnt_s1, cnt_s1_back, cap, c);
    if (gi < rp.path_count) store_state<N>(states, (int)gi, st, kind == 1 ? 1 : nk);
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// Vertex level L, one launch per kind: the volume (kVolume) or interface vertices of the
// level; a continuing path then runs level L+1's distance sampling (camera_next).
template <int N, bool kVolume>
__global__ void __launch_bounds__(kBlock) k_cam_vertex(DevScene sc, RenderParams rp, CamState<N> *states,
                                                       VertexIn<N> *vins, const int *q_in,
                                                       const unsigned long long *cnt_in,
                                                       const unsigned long long *cnt_in_back, int *qv_next,
                                                       unsigned long long *cnt_v_next, int *qs_next,
                                                       unsigned long long *cnt_s_next,
                                                       unsigned long long *cnt_s_next_back, long long cap, Queue qe,
                                                       Queue ql, unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long nf = (long long)*cnt_in, n = nf + (cnt_in_back ? (long long)*cnt_in_back : 0);
    Ctr c;
    for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < n; i += (long long)gridDim.x * kBlock) {
        const int id = i < nf ? q_in[i] : q_in[cap - 1 - (i - nf)];
        CamState<N> st;
        if (kVolume) {
            // a volume vertex writes the hit record (of its continuation) without reading it:
            // the record stays in HBM (380 B of 848 at nder 8)
            const CamState<N> &s0 = states[id];
            st.rng = s0.rng;
            st.ray = s0.ray;
            st.P = s0.P;
            st.acc = s0.acc;
            st.med = s0.med;
            st.depth = s0.depth;
            st.mode = s0.mode;
            st.level = s0.level;
        } else {
            st = states[id];
        }
        const VertexIn<N> vin = vins[id];
        const long long g = rp.path_begin + id;
        const bool alive = kVolume ? camera_volume<N>(sc, rp, stack, g, st, vin, qe, c)
                                   : camera_surface<N>(sc, rp, stack, g, st, vin, qe, ql, c);
        ++st.level;
        const int nk = camera_next<N>(sc, st, alive, vins, id, qv_next, cnt_v_next, qs_next, cnt_s_next,
                                      cnt_s_next_back, cap, c);
        store_state<N>(states, id, st, nk);
    }
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

template <int N>
__global__ void __launch_bounds__(kBlock) k_cam_accum(RenderParams rp, const CamState<N> *states, double *acc1) {
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < rp.path_count;
    DV<N> acc;
    if (active) acc = states[gi].acc * rp.inv_spp;
    accumulate_path<N>(rp, active, (int)((rp.path_begin + (active ? gi : 0)) / rp.spp), acc, acc1);
}

// ====================================================================== FP64 edge geometry
// pmf.h:103-167 sampleReuse on a normalised CDF with a leading 0 (n+1 entries). The CDF
// entries and u are non-negative doubles, whose IEEE bit patterns order as 64-bit integers:
// the search compares those on the integer pipe and leaves the FP64 pipe (1/64 of FP32 on
// this GPU) to the reuse of u.
DT_D int sample_reuse(const double *cdf, int n, double &u, double &pdf) {
    const long long ub = __double_as_longlong(u);
    int lo = 0, hi = n + 1;  // lower_bound
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__double_as_longlong(__ldg(cdf + mid)) < ub) lo = mid + 1;
        else hi = mid;
    }
    int idx = min(n - 1, max(0, lo - 1));
    while (idx < n - 1 && __double_as_longlong(__ldg(cdf + idx + 1)) == __double_as_longlong(__ldg(cdf + idx))) ++idx;
    const double c0 = __ldg(cdf + idx);
    pdf = __ldg(cdf + idx + 1) - c0;
    u = (u - c0) / pdf;
    return idx;
}

// shape.cpp:302-335, in FP64. The side of each face plane is the sign of the dot product
// with the face's unnormalised normal (normalising by a positive length keeps the sign).
// Callers test only > 0, which holds for every edge of a mesh without vertex normals (the
// result is then 2 or 1): such meshes skip the face tests.
DT_D int is_silhouette(const DevScene &sc, const DevEdge &e, const double3_ &p) {
    if (e.f0 < 0 || e.f1 < 0) return 2;
    if (!sc.shapes[e.shape].has_normals) return 1;
    const double3_ v0 = tod(f3(__ldg(sc.verts + e.v0))), v1 = tod(f3(__ldg(sc.verts + e.v1)));
    bool ff[2] = {false, false};
    for (int k = 0; k < 2; ++k) {
        const int4 tri = __ldg(sc.tris + (k == 0 ? e.f0 : e.f1));
        const int ids[3] = {tri.x, tri.y, tri.z};
        for (int i = 0; i < 3; ++i) {
            if (ids[i] != e.v0 && ids[i] != e.v1) {
                const double3_ v = tod(f3(__ldg(sc.verts + ids[i])));
                const double3_ n = k == 0 ? crossd(v0 - v, v1 - v) : crossd(v1 - v, v0 - v);
                ff[k] = dotd(n, p - v) > 0.0;
                break;
            }
        }
    }
    if (ff[0] != ff[1]) return 2;
    return sc.shapes[e.shape].has_normals ? 0 : 1;
}

// volpathAD.cpp:231-280 / 540-589 (ALTERNATIVE_EDGE_SAMPLING): the edge point seen from x0
// at parameter t, by angular interpolation between the edge's endpoints, in FP64 (near-
// degenerate triangles cancel). w0 : wb = sin(theta (1 - t)) / l0 : sin(theta t) / l1,
// normalised to a sum of 1; the angular pdf is the edge pdf / theta (theta returned). theta = acos(cos theta) as in the
// reference; sin(theta t) and cos(theta t) come from one sincos and sin(theta (1 - t)) =
// sin(theta) cos(theta t) - cos(theta) sin(theta t), with sin(theta) = |e0 x e1| / (l0 l1).
struct EdgePoint {
    double3_ w1, nrm;   // unit direction to the edge point, unit normal of (x0, v0, v1)
    double dist, inv_dist, w0, wb, theta;
};
DT_D bool edge_point_solve(const DevScene &sc, const DevEdge &e, const double3_ &x0, double t, EdgePoint &ep) {
    const double3_ v0 = tod(f3(__ldg(sc.verts + e.v0))), v1 = tod(f3(__ldg(sc.verts + e.v1)));
    const double3_ e0 = v0 - x0, e1 = v1 - x0;
    const double3_ cr = crossd(e0, e1);
    const double lc = lengthd(cr);
    ep.nrm = cr * (1.0 / lc);
    const double l0 = lengthd(e0), l1 = lengthd(e1), inv_l01 = 1.0 / (l0 * l1);
    const double c = fmin(1.0, fmax(-1.0, dotd(e0, e1) * inv_l01));
    const double theta = acos(c);
    if (theta < kEpsD || theta > kPiD - kEpsD) return false;
    double st, ct;
    sincos(theta * t, &st, &ct);
    // the common factor 1 / sin(theta) of both weights cancels in the normalisation
    double w0 = (lc * inv_l01 * ct - c * st) * l1, wb = st * l0;
    const double inv = 1.0 / (w0 + wb);
    w0 *= inv;
    wb *= inv;
    if (w0 < -kEpsD || wb < -kEpsD || fabs(w0 + wb - 1.0) > kEpsD) return false;
    const double3_ w = e0 * w0 + e1 * wb;
    ep.dist = lengthd(w);
    ep.inv_dist = 1.0 / ep.dist;
    ep.w1 = w * ep.inv_dist;
    ep.w0 = w0;
    ep.wb = wb;
    ep.theta = theta;
    return true;
}

// Derivative slots of the edge-point direction (FP32: they are stored as FP32 weights):
// dw = w0 (dv0 - dx0) + wb (dv1 - dx0), dw1 = (dw - w1 (w1 . dw)) / dist, and the slot
// weight s_j = (n . dw1_j) k2. False where no slot moves the direction (every component at
// most 1e-7) or where dw1 leaves the plane normal to w1 by more than 1e-7: w1 . dw1 =
// (w1 . dw)(1 - |w1|^2) / dist, with |w1|^2 from the FP64 solve.
template <int N>
DT_D bool edge_point_slots(const DevScene &sc, const DevEdge &e, const EdgePoint &ep, const float (*x0d)[3], double k2,
                           float *s) {
    const float3 w1 = tof(ep.w1), nrm = tof(ep.nrm);
    const float w0 = (float)ep.w0, wb = (float)ep.wb, inv_d = (float)ep.inv_dist, k2f = (float)k2;
    const float off_plane = (float)fabs(1.0 - dotd(ep.w1, ep.w1)) * inv_d;
    float mx = 0.f;
    bool moves = false;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        float3 dv0 = mk(0.f, 0.f, 0.f), dv1 = dv0;
        if (sc.vert_der) {
            const float *g0 = sc.vert_der + (size_t)e.v0 * sc.nder * 3 + 3 * j;
            const float *g1 = sc.vert_der + (size_t)e.v1 * sc.nder * 3 + 3 * j;
            dv0 = mk(g0[0], g0[1], g0[2]);
            dv1 = mk(g1[0], g1[1], g1[2]);
        }
        const float3 xd = mk(x0d[j][0], x0d[j][1], x0d[j][2]);
        const float3 dw = (dv0 - xd) * w0 + (dv1 - xd) * wb;
        const float proj = dot(w1, dw);
        const float3 d1 = (dw - w1 * proj) * inv_d;
        mx = fmaxf(mx, fabsf(proj) * off_plane);
        moves = moves || fabsf(d1.x) > (float)kEpsD || fabsf(d1.y) > (float)kEpsD || fabsf(d1.z) > (float)kEpsD;
        s[j] = dot(nrm, d1) * k2f;
    }
    return moves && !(mx > (float)kEpsD);
}

// A reflection-only BSDF at x0 (diffuse.cpp:7-12, phong.cpp:19-53: zero unless wi.z and
// wo.z >= 1e-7) gives an edge sample of a surface record a zero value when the incident
// direction is below the shading plane, or when both edge endpoints lie below it by more
// than 1e-4 of their distance: w1 is a non-negative combination of the directions to the
// endpoints, so its cosine with the normal is then below -1e-4, far beyond FP32 rounding.
// Such samples skip the FP64 silhouette test and edge-point solve; the value test after
// them would reject them all the same (no random numbers are drawn in between).
DT_D bool edge_sample_is_zero(const DevScene &sc, int shape, const float *wi, const float *fn, const float *x0,
                              const DevEdge &e) {
    const int t = sc.bsdfs[sc.shapes[shape].bsdf_id].type;
    if (t != BSDF_DIFFUSE && t != BSDF_PHONG) return false;
    if (wi[2] < kEps) return true;
    const float3 n = mk(fn[0], fn[1], fn[2]), p = mk(x0[0], x0[1], x0[2]);
    const float3 a = f3(__ldg(sc.verts + e.v0)) - p, b = f3(__ldg(sc.verts + e.v1)) - p;
    return dot(a, n) < -1e-4f * length(a) && dot(b, n) < -1e-4f * length(b);
}

// The two sub-path directions of an edge sample, w1 -+ kAngleEps n (volpathAD.cpp:601-605)
DT_D float3 edge_subpath_dir(const EdgePoint &ep, int sgn) {
    const float a = sgn == 0 ? -kAngleEps : kAngleEps;
    return normalize(tof(ep.w1) + tof(ep.nrm) * a);
}

// eight resident blocks per SM: the kernel waits on the FP64 pipe and on traversal latency
template <int N>
__global__ void __launch_bounds__(kBlock, 8) k_edge(DevScene sc, RenderParams rp, Queue qe, long long rec_begin,
                                                 long long rec_count, Queue qli, unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    uint32_t nsamples = 0;
    if (gi < rec_count * rp.sppse) {
        const long long ri = rec_begin + gi / rp.sppse;
        const int i = (int)(gi % rp.sppse);
        const EdgeRec<N> &r = reinterpret_cast<const EdgeRec<N> *>(qe.data)[ri];
        Rng rng;
        rng.init(rp.seed, child_key(r.key, 7u, (uint32_t)i));
        nsamples = 1;
        double u = ((double)i + rng.next1d()) * rp.inv_sppse;
        double pdf_shape, pdf_edge;
        const int sid = sample_reuse(sc.shape_edge_cdf, sc.num_shapes, u, pdf_shape);
        const DevShape &shp = sc.shapes[sid];
        const bool has = shp.num_edges > 0;
        const int k = has ? sample_reuse(sc.edge_cdf + shp.edge_cdf_off, shp.num_edges, u, pdf_edge) : 0;
        double pdf = has ? pdf_shape * pdf_edge : 0.0;
        const DevEdge e = sc.edges[shp.edge_off + (has ? k : 0)];
        const double3_ x0 = mkd(r.x0[0], r.x0[1], r.x0[2]);
        bool ok = has && sc.bsdfs[shp.bsdf_id].type != BSDF_NULL &&
                  !(r.kind == 0 && edge_sample_is_zero(sc, r.shape, r.wi, r.fn, r.x0, e)) &&
                  is_silhouette(sc, e, x0) > 0;
        EdgePoint ep;
        float s[N];
        if (ok) ok = edge_point_solve(sc, e, x0, u, ep);
        // slot weight factor 1 / (angular pdf * sppse), angular pdf = pdf / theta
        if (ok) ok = edge_point_slots<N>(sc, e, ep, r.x0d, ep.theta * rp.inv_sppse / pdf, s);
        float3 val = mk(0.f, 0.f, 0.f);
        int med1 = r.med;
        const float3 w1f = ok ? tof(ep.w1) : mk(0.f, 0.f, 1.f);
        if (ok) {
            if (r.kind == 0) {
                Frame fr;
                fr.s = f3(r.fs); fr.t = f3(r.ft); fr.n = f3(r.fn);
                const DevShape &vs = sc.shapes[r.shape];
                val = cmul(f3(r.w), bsdf_eval(sc.bsdfs[vs.bsdf_id], f3(r.wi), fr.to_local(w1f)));
                if (is_transition(vs)) med1 = dot(w1f, f3(r.ng)) > 0.f ? vs.med_ext : vs.med_int;
            } else {
                val = f3(r.w) * phase_eval(sc.phases[r.phase], f3(r.wi), w1f);
            }
            ok = !is_zero3(val);
        }
        if (ok) {
            const float tr =
                eval_transmittance(sc, stack, tof(x0), w1f, r.kind == 0, med1, (float)ep.dist, rng, r.depth, c);
            ok = tr > kEps;
        }
        if (ok) {
            // the two sub-paths of a sample in adjacent slots: k_li then traces the nearly
            // identical rays (1e-4 rad apart) in neighbouring lanes of one warp
            const long long slot = queue_reserve_n(sc, qli, 2);
            for (int sgn = 0; sgn < 2 && slot >= 0; ++sgn) {
                const float3 w2 = edge_subpath_dir(ep, sgn);
                LiTask<N> &t = reinterpret_cast<LiTask<N> *>(qli.data)[slot + sgn];
                t.o[0] = r.x0[0]; t.o[1] = r.x0[1]; t.o[2] = r.x0[2];
                t.d[0] = w2.x; t.d[1] = w2.y; t.d[2] = w2.z;
                const float sg = sgn == 0 ? 1.f : -1.f;
                t.w[0] = val.x * sg; t.w[1] = val.y * sg; t.w[2] = val.z * sg;
#pragma unroll
                for (int j = 0; j < N; ++j) t.s[j] = s[j];
                t.med = med1; t.depth = r.depth; t.pixel = r.pixel; t.flags = 1;
                t.key = child_key(r.key, 8u + (uint32_t)sgn, (uint32_t)i);
            }
        }
    }
    if (ctr) flush_counters(ctr, K_EDGE, c, CT_EDGE_SAMPLES, nsamples);
}

// ====================================================================== Li sub-paths
// Sort key of the sub-path pair m (slots 2m, 2m + 1, which share origin and, within
// 1e-4 rad, direction): the origin's cell in a 4^3 grid over the scene bounds (high 6 bits)
// and the direction's cell in a 64 x 64 octahedral map (low 12 bits). The Li kernels then
// run pairs of similar rays in the same warps (C2 Li stage 102 -> 78 ms with the sort; a
// 32 x 32 map 81 ms, a 16^3 grid with a 16 x 16 map 85 ms, the direction in the high bits
// the same as in the low).
constexpr int kLiSortOriginBits = 2, kLiSortDirBits = 6;
constexpr int kLiSortKeyBits = (3 * kLiSortOriginBits + 2 * kLiSortDirBits + 3) & ~3;
template <class Task>
__global__ void k_li_keys(DevScene sc, const Task *tasks, long long npairs, unsigned *keys, int *vals) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npairs) return;
    constexpr int ob = kLiSortOriginBits, db = kLiSortDirBits;
    const Task &t = tasks[2 * m];
    const float4 *root = reinterpret_cast<const float4 *>(sc.nodes);
    const float4 bx = __ldg(root), by = __ldg(root + 1), bz = __ldg(root + 2);
    const float lo[3] = {fminf(bx.x, bx.z), fminf(by.x, by.z), fminf(bz.x, bz.z)};
    const float hi[3] = {fmaxf(bx.y, bx.w), fmaxf(by.y, by.w), fmaxf(bz.y, bz.w)};
    unsigned cell = 0;
    const float oc = (float)(1 << ob), dc = (float)(1 << db);
    for (int a = 0; a < 3; ++a) {
        const float ext = hi[a] - lo[a];
        const float u = ext > 0.f ? (t.o[a] - lo[a]) / ext : 0.f;
        cell = (cell << ob) + (unsigned)fminf(fmaxf(u * oc, 0.f), oc - 1.f);
    }
    const float3 d = f3(t.d);
    const float l1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    float u = d.x / l1, v = d.y / l1;
    if (d.z < 0.f) {
        const float uu = (1.f - fabsf(v)) * copysignf(1.f, u), vv = (1.f - fabsf(u)) * copysignf(1.f, v);
        u = uu;
        v = vv;
    }
    const unsigned qu = (unsigned)fminf(fmaxf((u * 0.5f + 0.5f) * dc, 0.f), dc - 1.f);
    const unsigned qv = (unsigned)fminf(fmaxf((v * 0.5f + 0.5f) * dc, 0.f), dc - 1.f);
    keys[m] = (cell << (2 * db)) | (qu << db) | qv;
    vals[m] = (int)m;
}

// Six resident blocks per SM (80 registers, a few spilled): traversal is latency bound and
// the extra warps hide more of it than the spills cost (C2 Li stage 121 -> 102 ms).
template <int N>
__global__ void __launch_bounds__(kBlock, 6) k_li(DevScene sc, RenderParams rp, Queue qli, long long begin, long long count,
                                               double *acc1, double *acc2, const int *perm,
                                               unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    // perm: the pairs in sorted order (a pair's two slots stay in adjacent lanes), or queue order
    const long long slot = perm && gi < count ? 2LL * __ldg(perm + (gi >> 1)) + (gi & 1) : begin + gi;
    Ctr c;
    uint32_t n = 0;
    if (gi < count) {
        const LiTask<N> &t = reinterpret_cast<const LiTask<N> *>(qli.data)[slot];
        Rng rng;
        rng.init(rp.seed, t.key);
        n = 1;
        const float3 L = li_path(sc, stack, rng, f3(t.o), f3(t.d), t.depth, t.med, (t.flags & 1) != 0, c);
        if (!is_zero3(L, 0.f)) {
            const float3 wl = cmul(f3(t.w), L);
            const bool prim = (t.flags & 2) != 0;
            double *acc = prim ? acc2 : acc1 + (size_t)rp.npix * 3;  // slot j of the derivative images
#pragma unroll
            for (int j = 0; j < N; ++j) {
                if (t.s[j] == 0.f) continue;
                double *a = acc + ((size_t)j * rp.npix + t.pixel) * 3;
                atomicAdd(a, (double)(wl.x * t.s[j]));
                atomicAdd(a + 1, (double)(wl.y * t.s[j]));
                atomicAdd(a + 2, (double)(wl.z * t.s[j]));
            }
        }
    }
    if (ctr) flush_counters(ctr, K_LI, c, CT_LI, n);
}

// ====================================================================== Lins records
template <int N>
__global__ void __launch_bounds__(kBlock) k_lins(DevScene sc, RenderParams rp, Queue ql, long long count, double *acc1,
                                                 unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    if (gi < count) {
        const LinsRec<N> &r = reinterpret_cast<const LinsRec<N> *>(ql.data)[gi];
        Rng rng;
        rng.init(rp.seed, r.key);
        Its its0;
        its0.shape = r.shape; its0.p = f3(r.p); its0.ng = f3(r.ng); its0.wi = f3(r.wi);
        its0.fr.s = f3(r.fs); its0.fr.t = f3(r.ft); its0.fr.n = f3(r.fn);
        const float3 n = f3(r.n), rd = f3(r.rd);
        const DevPhase &ph = sc.phases[r.phase];
        const DevShape &sh = sc.shapes[r.shape];
        const DevBsdf &b = sc.bsdfs[sh.bsdf_id];
        const int max_depth = r.depth, med = r.med;
        float3 lins = mk(0.f, 0.f, 0.f);
        for (int smp = 0; smp < r.ns; ++smp) {  // volpathAD.cpp:337-441
            float3 wo, att;
            float pdf_nee, pv;
            Its its1;
            float r4[4];
            r4[0] = rng.next1(); r4[1] = rng.next1(); r4[2] = rng.next1(); r4[3] = rng.next1();
            if (b.type == BSDF_NULL) {
                att = nee_surface(sc, stack, its0, r4, rng, med, max_depth - 1, wo, pdf_nee, true, c);
                if (!is_zero3(att)) {
                    wo = its0.to_world(wo);
                    pv = phase_eval(ph, -rd, wo);
                    if (pv > kEps) lins += att * (pv * mis_weight(pdf_nee, pv));
                }
                const float u = rng.next1(), v = rng.next1();
                if ((pv = phase_sample(ph, -rd, u, v, wo)) > kEps) {
                    int md1 = max_depth - 1;
                    if (dot(wo, n) > kEps) {
                        if (sh.light_id >= 0) lins += le(sc, its0, -wo) * pv;
                        --md1;
                    }
                    if (md1 > 0) {
                        const int med1 = is_transition(sh) ? target_medium(sc, r.shape, its0.ng, wo) : med;
                        att = look_for_emitter(sc, stack, its0.p, wo, true, rng, med1, md1, its1, pdf_nee, c);
                        if (!is_zero3(att)) lins += att * (pv * mis_weight(phase_eval(ph, -rd, wo), pdf_nee));
                        lins += li_path(sc, stack, rng, its0.p, wo, md1, med1, false, c) * pv;
                    }
                }
                continue;
            }
            att = nee_surface(sc, stack, its0, r4, rng, med, max_depth - 1, wo, pdf_nee, false, c);
            if (!is_zero3(att)) {
                wo = its0.to_world(wo);
                if (dot(wo, n) < -kEps) {
                    pv = phase_eval(ph, -rd, wo);
                    if (pv > kEps) lins += att * (pv * mis_weight(pdf_nee, pv));
                }
            }
            const float u = rng.next1(), v = rng.next1();
            if ((pv = phase_sample(ph, -rd, u, v, wo)) > kEps) {
                const float wdn = dot(wo, n);
                if (wdn < -kEps) {
                    att = look_for_emitter(sc, stack, its0.p, wo, true, rng, med, max_depth - 1, its1, pdf_nee, c);
                    if (!is_zero3(att)) lins += att * (pv * mis_weight(phase_eval(ph, -rd, wo), pdf_nee));
                    lins += li_path(sc, stack, rng, its0.p, wo, max_depth - 1, med, false, c) * pv;
                } else if (wdn > kEps) {
                    if (sh.light_id >= 0) lins += le(sc, its0, -wo) * pv;
                    if (max_depth > 1) {
                        Its its2 = its0;
                        its2.wi = its2.to_local(-wo);
                        float r4b[4];
                        r4b[0] = rng.next1(); r4b[1] = rng.next1(); r4b[2] = rng.next1(); r4b[3] = rng.next1();
                        att = nee_surface(sc, stack, its2, r4b, rng, med, max_depth - 2, wo, pdf_nee, false, c);
                        if (!is_zero3(att))
                            lins += cmul(bsdf_eval(b, its2.wi, wo), att) *
                                    (pv * mis_weight(pdf_nee, bsdf_pdf(b, its2.wi, wo)));
                        const float ra = rng.next1(), rb = rng.next1(), rc = rng.next1();
                        float bp, eta;
                        const float3 bv = bsdf_sample(b, its2.wi, ra, rb, rc, wo, bp, eta);
                        if (!is_zero3(bv)) {
                            const float3 t1 = bv * pv;
                            wo = its2.to_world(wo);
                            const int med1 = is_transition(sh) ? target_medium(sc, r.shape, its2.ng, wo) : med;
                            Its its3;
                            att = look_for_emitter(sc, stack, its2.p, wo, true, rng, med1, max_depth - 2, its3, pdf_nee, c);
                            if (!is_zero3(att, 1e-12f)) lins += cmul(t1, att) * mis_weight(bp, pdf_nee);
                            lins += cmul(t1, li_path(sc, stack, rng, its2.p, wo, max_depth - 2, med1, false, c));
                        }
                    }
                }
            }
        }
        const float3 wl = cmul(f3(r.w), lins);
        if (!is_zero3(wl, 0.f)) {
            double *acc = acc1 + (size_t)rp.npix * 3;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                double *a = acc + ((size_t)j * rp.npix + r.pixel) * 3;
                atomicAdd(a, (double)(wl.x * r.s[j]));
                atomicAdd(a + 1, (double)(wl.y * r.s[j]));
                atomicAdd(a + 2, (double)(wl.z * r.s[j]));
            }
        }
    }
    if (ctr) flush_counters(ctr, K_LINS, c);
}

// ====================================================================== primary edges
// A primary-edge sample's point (edge_manager.cpp:112-134, camera.cpp): the screen point at
// parameter u along the edge, its pixel, the edge's unit screen normal, and the distance to
// the edge point in camera space (the edge-point solve of compute_intersection_in_tri,
// utils.cpp:256-266, with the edge's constants precomputed on the host), in FP64.
struct PrimaryPoint {
    double px, py, nx, ny;
    int ipx, ipy;
    float maxd;
};
DT_D void primary_edge_point(const DevCamera &cam, const DevPrimaryEdge &e, double u, PrimaryPoint &pp) {
    pp.px = e.v0s[0] + (e.v1s[0] - e.v0s[0]) * u;
    pp.py = e.v0s[1] + (e.v1s[1] - e.v0s[1]) * u;
    pp.ipx = (int)floor(pp.px);
    pp.ipy = (int)floor(pp.py);
    pp.nx = e.n[0];
    pp.ny = e.n[1];
    const double a0 = (pp.px * cam.inv_w - 0.5) * cam.plane_kx - e.v0p[0];
    const double a1 = (pp.py * cam.inv_h - 0.5) * cam.plane_ky - e.v0p[1];
    const double a2 = 1.0 - e.v0p[2];
    const double t0 = sqrt(a0 * a0 + a1 * a1 + a2 * a2) * e.inv_lenp;
    const double bx = (1.0 - t0) * e.cb, by = t0 * e.cc;
    const double t1 = by / (bx + by);
    double pc[3];
    for (int q = 0; q < 3; ++q) pc[q] = e.v0c[q] + t1 * (e.v1c[q] - e.v0c[q]);
    pp.maxd = (float)sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
}

// Sort key of primary-edge sample k: the top 20 bits of its first random number, which
// picks the edge and the point on it (sample_reuse): samples in key order lie along the
// edge list, so a warp traces neighbouring camera rays (C2 primary-edge stage 26.4 ->
// 16.3 ms with the sort). The sample's random numbers stay keyed by k.
template <int Unused = 0>
__global__ void k_primary_keys(RenderParams rp, unsigned *keys, int *vals) {
    const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= rp.prim_count) return;
    const long long k = rp.prim_begin + gi;
    Rng rng;
    rng.init(rp.seed, child_key(0x5052494DULL, (uint32_t)(k >> 32), (uint32_t)k));
    keys[gi] = rng.next_u32() >> 12;
    vals[gi] = (int)gi;
}

template <int N>
__global__ void __launch_bounds__(kBlock) k_primary(DevScene sc, RenderParams rp, Queue qli, const int *perm,
                                                    unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    uint32_t n = 0;
    if (gi < rp.prim_count) {
        const long long k = rp.prim_begin + (perm ? (long long)__ldg(perm + gi) : gi);
        Rng rng;
        rng.init(rp.seed, child_key(0x5052494DULL, (uint32_t)(k >> 32), (uint32_t)k));
        n = 1;
        double u = rng.next1d(), pdf;
        const int idx = sample_reuse(sc.pedge_cdf, sc.num_pedges, u, pdf);
        const DevPrimaryEdge &e = sc.pedges[idx];
        const DevCamera &cam = sc.cam;
        PrimaryPoint pp;
        primary_edge_point(cam, e, u, pp);
        // screen velocity of the edge point along its normal, per slot (FP32)
        const float uf = (float)u, nxf = (float)pp.nx, nyf = (float)pp.ny;
        float sv[N];
        bool moving = false;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const float pdx = e.d0[j][0] + (e.d1[j][0] - e.d0[j][0]) * uf;
            const float pdy = e.d0[j][1] + (e.d1[j][1] - e.d0[j][1]) * uf;
            moving = moving || fabsf(pdx) > kEps || fabsf(pdy) > kEps;
            sv[j] = nxf * pdx + nyf * pdy;
        }
        const int ipx = pp.ipx, ipy = pp.ipy;
        const double fx = pp.px - ipx, fy = pp.py - ipy, nx = pp.nx, ny = pp.ny;
        const float maxd = pp.maxd;
        const int lx = ipx - rp.crop_x, ly = ipy - rp.crop_y;
        if (moving && lx >= 0 && ly >= 0 && lx < rp.out_w && ly < rp.out_h) {
            float3 o, d;
            camera_ray(cam, ipx + fx, ipy + fy, o, d);
            const float tr = eval_transmittance(sc, stack, o, d, false, cam.med_id, maxd, rng, rp.max_bounces - 1, c);
            if (tr > kEps) {
                const long long slot = queue_reserve_n(sc, qli, 2);  // the pair in adjacent slots
                for (int sgn = 0; sgn < 2 && slot >= 0; ++sgn) {
                    const double delta = sgn == 0 ? -1e-4 : 1e-4;
                    float3 o2, d2;
                    camera_ray(cam, ipx + fx + nx * delta, ipy + fy + ny * delta, o2, d2);
                    LiTask<N> &t = reinterpret_cast<LiTask<N> *>(qli.data)[slot + sgn];
                    t.o[0] = o2.x; t.o[1] = o2.y; t.o[2] = o2.z;
                    t.d[0] = d2.x; t.d[1] = d2.y; t.d[2] = d2.z;
                    const float w = (float)(sgn == 0 ? rp.prim_weight : -rp.prim_weight);
                    t.w[0] = w; t.w[1] = w; t.w[2] = w;
#pragma unroll
                    for (int j = 0; j < N; ++j) t.s[j] = sv[j];
                    t.med = cam.med_id; t.depth = rp.max_bounces; t.pixel = lx + rp.out_w * ly; t.flags = 1 | 2;
                    t.key = child_key(0x50524D31ULL + (uint64_t)k, 9u + (uint32_t)sgn, 0u);
                }
            }
        }
    }
    if (ctr) flush_counters(ctr, K_PRIMARY, c, CT_PRIMARY, n);
}

// ====================================================================== finalize
// integratorAD.cpp:59-87 and 154-162: a pixel is written only if its value is
// non-negative, a derivative only if finite; primary-edge sums are then added.
template <int N>
__global__ void k_finalize(RenderParams rp, const double *acc1, const double *acc2, float *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= rp.npix) return;
    const double *a = acc1 + (size_t)p * 3;
    const bool nonneg = a[0] >= 0.0 && a[1] >= 0.0 && a[2] >= 0.0;
    for (int c = 0; c < 3; ++c) out[(size_t)p * 3 + c] = nonneg ? (float)a[c] : 0.f;
    for (int j = 0; j < N; ++j) {
        const double *d = acc1 + ((size_t)(j + 1) * rp.npix + p) * 3;
        const bool fin = isfinite(d[0]) && isfinite(d[1]) && isfinite(d[2]);
        const double *e = acc2 + ((size_t)j * rp.npix + p) * 3;
        for (int c = 0; c < 3; ++c)
            out[((size_t)(j + 1) * rp.npix + p) * 3 + c] = (fin ? (float)d[c] : 0.f) + (float)e[c];
    }
}

}  // namespace dt
