// dtrt_gb300 — reverse-mode adjoint with respect to vertex positions (surface scenes).
//
// Scope: scenes without participating media, without per-vertex shading normals and with
// AreaLight emitters (the C2 mesh configuration and its kind). The forward-mode estimator
// (volpathAD.cpp:306-617 interface branch, the surface edge term 513-616 and the primary
// edges of integratorAD.cpp:100-165) depends on vertex positions through three routes, and
// each has its transpose here:
//
//   frame factors    at a non-null surface vertex on triangle T, the BSDF value of the NEE
//                    event (a factor of that event) and the BSDF sampling weight (a factor of
//                    every later event) depend on T's unit normal n (the local wi/wo of the
//                    dual shading frame). Their gradient in n comes from a 3-slot local
//                    forward mode (slot k = d/dn_k), is weighted by dot(dL/dI, event or
//                    suffix radiance)/value, and is mapped to T's vertices through
//                    n = normalize((v1-v0) x (v2-v0)).
//   secondary edges  an edge sample's derivative is m . (w0 dv0 + wb dv1 - dx0) with
//                    m = (n_e - (n_e.w1) w1) / (dist pdf sppse) (volpathAD.cpp:545-609); its
//                    Li sub-paths scatter K m w0 and K m wb to the edge vertices and K (-m)
//                    to the gradient slot of the path vertex x0, K = dot(dL/dI, w (x) Li).
//   x0 chain         x0 = o + t d moves with its triangle and with its ray origin (the
//                    previous vertex); a final replay of each camera path walks the slots
//                    back to front, mapping them to triangle vertices (dt/dv) and to the
//                    previous vertex ((I - d n^T/(d.n))^T).
//   primary edges    the screen-space edge point moves with the two edge vertices through
//                    the projection Jacobian built on the host (with near-plane and image
//                    clipping); its two Li sub-paths scatter K n_s.J to both vertices.
//
// Every camera path is replayed from its RNG seed (value pass, scatter pass, chain pass);
// edge records and Li tasks use the same child streams as the forward kernels, so for the
// same seed <grad, V> equals sum(dL/dI * forward derivative image along velocities V).
#pragma once
#include "dt_adjoint.cuh"

namespace dt {

struct VEdgeRec {
    float x0[3], w[3], wi[3], fs[3], ft[3], fn[3], ng[3];
    int shape, depth, pixel, chain;  // chain: gradient slot of x0 (path in batch * levels + level)
    uint64_t key;
};

struct VLiTask {
    float o[3], d[3], w[3];
    float c0[3], c1[3], cx[3];  // gradient coefficients of edge vertex v0, v1 and of x0
    int v0, v1, chain, med, depth, pixel, flags;
    uint64_t key;
};

DT_D void scatter3(float *g, int v, float3 x) {
    if (x.x != 0.f) atomicAdd(g + 3 * (size_t)v, x.x);
    if (x.y != 0.f) atomicAdd(g + 3 * (size_t)v + 1, x.y);
    if (x.z != 0.f) atomicAdd(g + 3 * (size_t)v + 2, x.z);
}

// gradient on the unit face normal of triangle prim -> its three vertices
DT_D void normal_to_vertices(const DevScene &sc, int prim, float3 gn, float *grad) {
    if (!isfinite(gn.x) || !isfinite(gn.y) || !isfinite(gn.z)) return;
    const int4 tri = __ldg(sc.tris + prim);
    const float3 v0 = f3(__ldg(sc.verts + tri.x)), e1 = f3(__ldg(sc.verts + tri.y)) - v0,
                 e2 = f3(__ldg(sc.verts + tri.z)) - v0;
    const float3 c = cross(e1, e2);
    const float len = length(c);
    if (!(len > 1e-12f)) return;
    const float3 n = c / len;
    const float3 graw = (gn - n * dot(n, gn)) / len;  // d normalize(c) = (I - n n^T) dc / |c|
    const float3 g1 = cross(e2, graw), g2 = cross(graw, e1);
    scatter3(grad, tri.x, -(g1 + g2));
    scatter3(grad, tri.y, g1);
    scatter3(grad, tri.z, g2);
}

// gradient gx on the hit point p = o + t d of triangle prim -> its vertices; returns the
// gradient on the ray origin o (t = (v0 - o).n / (d.n), n = (v1-v0) x (v2-v0))
DT_D float3 hit_to_vertices(const DevScene &sc, int prim, float3 d, float3 p, float3 gx, float *grad) {
    const int4 tri = __ldg(sc.tris + prim);
    const float3 v0 = f3(__ldg(sc.verts + tri.x)), e1 = f3(__ldg(sc.verts + tri.y)) - v0,
                 e2 = f3(__ldg(sc.verts + tri.z)) - v0;
    const float3 n = cross(e1, e2);
    const float dn = dot(d, n);
    if (fabsf(dn) < kEps) return mk(0.f, 0.f, 0.f);  // the forward divisor is clamped: no derivative
    const float gt = dot(gx, d);
    const float3 a = (v0 - p) / dn;
    const float3 t1 = cross(e2, a), t2 = cross(a, e1), t0 = n / dn - t1 - t2;
    if (gt != 0.f) {
        scatter3(grad, tri.x, t0 * gt);
        scatter3(grad, tri.y, t1 * gt);
        scatter3(grad, tri.z, t2 * gt);
    }
    return gx - n * (gt / dn);
}

// d(value)/d(unit normal) of the BSDF value of the NEE event and of the BSDF sampling
// weight at a surface vertex, by 3-slot forward mode (slot k = d/dn_k). Channel c of the
// result is the 3-vector (dv_c/dn_x, dv_c/dn_y, dv_c/dn_z).
DT_D DV<3> local_normal_frame(float3 n) {
    DV<3> ns(n);
    ns.set_grad(0, mk(1.f, 0.f, 0.f));
    ns.set_grad(1, mk(0.f, 1.f, 0.f));
    ns.set_grad(2, mk(0.f, 0.f, 1.f));
    return ns;
}

// weighted sum over channels of (w_c / value_c) * d value_c / dn
DT_D float3 channel_grad(const DV<3> &v, float3 w) {
    float3 g = mk(0.f, 0.f, 0.f);
    const Df<3> *ch[3] = {&v.x, &v.y, &v.z};
    const float wc[3] = {w.x, w.y, w.z};
    for (int c = 0; c < 3; ++c) {
        if (wc[c] == 0.f || ch[c]->v == 0.f) continue;
        const float s = wc[c] / ch[c]->v;
        g = g + mk(ch[c]->d[0], ch[c]->d[1], ch[c]->d[2]) * s;
    }
    return g;
}

// Stage of a camera-path replay
enum { VR_VALUE = 0, VR_FRAME = 1, VR_CHAIN = 2 };

// One camera path of k_camera's loop on a surface scene (no media: NEE, emitter lookups
// and edge visibility consume no random numbers beyond the 9 draws per level), value-only.
//   VR_VALUE: returns the sum of event contributions; pushes a VEdgeRec per non-null vertex
//   VR_FRAME: scatters the frame-factor gradients (needs `total`, `gpix`)
//   VR_CHAIN: walks the x0 gradient slots back to front (needs xadj)
constexpr int kVMaxLevels = 32;

DT_D float3 vreplay_path(const DevScene &sc, const RenderParams &rp, int *stack, long long g, int pixel, int stage,
                         float3 total, float3 gpix, float *grad, Queue qe, const float *xadj, long long chain_base,
                         Ctr &c) {
    const float3 zero = mk(0.f, 0.f, 0.f);
    const int ix = rp.crop_x + pixel % rp.out_w, iy = rp.crop_y + pixel / rp.out_w;
    Rng rng;
    rng.init(rp.seed, (uint64_t)g);
    double jx = 0.5, jy = 0.5;
    if (rp.jitter) {
        jx = rng.next1d();
        jy = rng.next1d();
    }
    RayAD<1> ray = camera_ray_ad<1>(sc.cam, ix + jx, iy + jy);
    ItsAD<1> its;
    int depth = rp.max_bounces;
    int mode = rp.mode;
    float3 P = mk(1.f, 1.f, 1.f), acc = zero;
    // chain stage: hit sequence of this path
    int cprim[kVMaxLevels];
    float3 cd[kVMaxLevels], cp[kVMaxLevels];
    int nlev = 0;
    bool alive = ray_intersect_ad<1>(sc, stack, ray, false, its, c);
    for (int level = 0; alive && mode != 0; ++level) {
        alive = false;
        rng.next1(); rng.next1();  // distance-sampling draws (no medium)
        float r2[4];
        r2[0] = rng.next1(); r2[1] = rng.next1(); r2[2] = rng.next1(); r2[3] = rng.next1();
        const float r3a = rng.next1(), r3b = rng.next1(), r3c = rng.next1();
        const float3 dir_in = ray.d.val();
        if (!its.valid()) break;
        if (stage == VR_CHAIN && level < kVMaxLevels) {
            cprim[level] = its.prim;
            cd[level] = dir_in;
            cp[level] = its.p.val();
            nlev = level + 1;
        }
        const DevShape &sh = sc.shapes[its.shape];
        const float3 Q = P;
        if (sh.light_id >= 0 && (mode & MODE_EMISSION)) acc = acc + cmul(Q, le_ad<1>(sc, its, -ray.d).val());
        if (depth == 0) break;
        const DevBsdf &b = sc.bsdfs[sh.bsdf_id];
        const bool is_null = b.type == BSDF_NULL;
        const FrameAD<1> fr = its.frame();
        const Its its0 = its.plain();
        // edge record (interface edge term), volpathAD.cpp:513-616
        if (stage == VR_VALUE && !is_null && rp.sppse > 0 && (mode & MODE_SURFACE_BOUNDARY) && sc.has_edges &&
            level < kVMaxLevels) {
            const long long slot = queue_reserve(sc, qe);
            if (slot >= 0) {
                VEdgeRec &r = reinterpret_cast<VEdgeRec *>(qe.data)[slot];
                const float3 x = its0.p, w = P * rp.inv_spp;
                r.x0[0] = x.x; r.x0[1] = x.y; r.x0[2] = x.z;
                r.w[0] = w.x; r.w[1] = w.y; r.w[2] = w.z;
                r.wi[0] = its0.wi.x; r.wi[1] = its0.wi.y; r.wi[2] = its0.wi.z;
                r.fs[0] = its0.fr.s.x; r.fs[1] = its0.fr.s.y; r.fs[2] = its0.fr.s.z;
                r.ft[0] = its0.fr.t.x; r.ft[1] = its0.fr.t.y; r.ft[2] = its0.fr.t.z;
                r.fn[0] = its0.fr.n.x; r.fn[1] = its0.fr.n.y; r.fn[2] = its0.fr.n.z;
                r.ng[0] = its0.ng.x; r.ng[1] = its0.ng.y; r.ng[2] = its0.ng.z;
                r.shape = its.shape; r.depth = depth - 1; r.pixel = pixel;
                r.chain = (int)(chain_base + level);
                r.key = child_key((uint64_t)g, 3u, (uint32_t)level);
            }
        }
        // local 3-slot frame for the normal gradients of this vertex
        float3 gn = zero;
        DV<3> ns3;
        FrameAD<3> fr3;
        DV<3> wi3;
        if (stage == VR_FRAME && !is_null) {
            ns3 = local_normal_frame(its0.fr.n);
            fr3 = FrameAD<3>(ns3);
            wi3 = fr3.to_local(-dir_in);
        }
        DV<1> wo;
        float pdf_nee;
        if (!is_null && (mode & MODE_SURFACE_MAIN)) {
            DV<1> v = nee_surface_ad<1>(sc, stack, its, fr, r2, rng, -1, depth - 1, wo, pdf_nee, c);
            if (!v.is_zero()) {
                const DV<1> bv = bsdf_eval_ad<1>(b, its.wi, wo);
                const float bp = bsdf_pdf(b, its0.wi, wo.val());
                const float3 e = cmul(cmul(Q, v.val()), bv.val()) * mis_weight(pdf_nee, bp);
                if (stage == VR_FRAME && !is_zero3(e, 0.f)) {
                    const float3 dir = its0.to_world(wo.val());
                    const DV<3> bv3 = bsdf_eval_ad<3>(b, wi3, fr3.to_local(dir));
                    gn = gn + channel_grad(bv3, cmul(gpix, e) * rp.inv_spp);
                }
                acc = acc + e;
            }
        }
        float bpdf, beta;
        const DV<1> bw = bsdf_sample_ad<1>(b, its, fr, its0, r3a, r3b, r3c, wo, bpdf, beta);
        if (!bw.is_zero()) {
            if (stage == VR_FRAME && !is_null) {  // the sampling weight multiplies every later event
                ItsAD<3> its3;
                its3.wi = wi3;
                DV<3> wo3;
                float p3, e3;
                const DV<3> bw3 = bsdf_sample_ad<3>(b, its3, fr3, its0, r3a, r3b, r3c, wo3, p3, e3);
                gn = gn + channel_grad(bw3, cmul(gpix, total - acc) * rp.inv_spp);
            }
            wo = fr.to_world(wo);
            if (!is_null) wo = zero_grad(wo);
            ray.o = its.p;
            ray.d = wo;
            float3 thr1 = mk(1.f, 1.f, 1.f);
            ItsAD<1> its1;
            if (is_null) {
                ray_intersect_ad<1>(sc, stack, ray, true, its1, c);
            } else {
                DV<1> att = look_for_emitter_ad<1>(sc, stack, ray, true, rng, -1, depth - 1, its1, pdf_nee, nullptr,
                                                   nullptr, c);
                thr1 = bw.val();
                if (!att.is_zero() && (mode & MODE_SURFACE_MAIN))
                    acc = acc + cmul(cmul(P, thr1), att.val()) * mis_weight(bpdf, pdf_nee);
                mode &= ~MODE_EMISSION;
            }
            its = its1;
            P = cmul(P, thr1);
            depth -= 1;
            alive = true;
        }
        if (stage == VR_FRAME && !is_null && !is_zero3(gn, 0.f)) normal_to_vertices(sc, its0.prim, gn, grad);
    }
    if (stage == VR_CHAIN) {  // back to front: x_k = o_k + t_k d_k, o_k = x_{k-1}
        float3 gx = zero;
        for (int k = nlev - 1; k >= 0; --k) {
            const float *q = xadj + 3 * (size_t)(chain_base + k);
            gx = gx + mk(q[0], q[1], q[2]);
            if (is_zero3(gx, 0.f)) continue;
            gx = hit_to_vertices(sc, cprim[k], cd[k], cp[k], gx, grad);  // now the gradient on o_k = x_{k-1}
        }
    }
    return acc;
}

// one thread per camera path: value pass (edge records), then the frame-factor pass
__global__ void __launch_bounds__(kBlock) k_vadj_camera(DevScene sc, RenderParams rp, const float *dimg, float *grad,
                                                        Queue qe, double *img_acc, int levels,
                                                        unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    const bool active = gi < rp.path_count;
    const long long g = rp.path_begin + (active ? gi : 0);
    const int pixel = (int)(g / rp.spp);
    Ctr c;
    float3 total = mk(0.f, 0.f, 0.f);
    if (active) {
        total = vreplay_path(sc, rp, stack, g, pixel, VR_VALUE, total, total, grad, qe, nullptr, gi * levels, c);
        const float3 gp = mk(__ldg(dimg + 3 * (size_t)pixel), __ldg(dimg + 3 * (size_t)pixel + 1),
                             __ldg(dimg + 3 * (size_t)pixel + 2));
        if (!is_zero3(total, 0.f) && !is_zero3(gp, 0.f))
            vreplay_path(sc, rp, stack, g, pixel, VR_FRAME, total, gp, grad, qe, nullptr, gi * levels, c);
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
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// one thread per camera path: the x0 gradient slots back to front
__global__ void __launch_bounds__(kBlock) k_vadj_chain(DevScene sc, RenderParams rp, float *grad, const float *xadj,
                                                       int levels, unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (gi >= rp.path_count) return;
    const long long g = rp.path_begin + gi;
    Ctr c;
    Queue none{nullptr, nullptr, 0};
    const float3 z = mk(0.f, 0.f, 0.f);
    vreplay_path(sc, rp, s_stack + threadIdx.x, g, (int)(g / rp.spp), VR_CHAIN, z, z, grad, none, xadj, gi * levels, c);
    if (ctr) flush_counters(ctr, K_CAMERA, c);
}

// one thread per (edge record, edge sample): k_edge's geometry, then two VLiTasks carrying
// the gradient coefficients instead of per-slot scalars
__global__ void __launch_bounds__(kBlock) k_vadj_edge(DevScene sc, RenderParams rp, Queue qe, long long rec_begin,
                                                      long long rec_count, Queue qli, unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    uint32_t nsamples = 0;
    if (gi < rec_count * rp.sppse) {
        const long long ri = rec_begin + gi / rp.sppse;
        const int i = (int)(gi % rp.sppse);
        const VEdgeRec &r = reinterpret_cast<const VEdgeRec *>(qe.data)[ri];
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
                  !edge_sample_is_zero(sc, r.shape, r.wi, r.fn, r.x0, e) && is_silhouette(sc, e, x0) > 0;
        // the edge-point solve of k_edge: direction, pdf and interpolation weights
        EdgePoint ep;
        if (ok) ok = edge_point_solve(sc, e, x0, u, ep);
        const double3_ w1 = ok ? ep.w1 : mkd(0.0, 0.0, 1.0), nrm = ok ? ep.nrm : mkd(0.0, 0.0, 1.0);
        const double dist = ok ? ep.dist : 0.0, w0 = ok ? ep.w0 : 0.0, wb = ok ? ep.wb : 0.0;
        float3 val = mk(0.f, 0.f, 0.f);
        int med1 = -1;
        const float3 w1f = ok ? tof(w1) : mk(0.f, 0.f, 1.f);
        if (ok) {
            Frame fr;
            fr.s = f3(r.fs); fr.t = f3(r.ft); fr.n = f3(r.fn);
            const DevShape &vs = sc.shapes[r.shape];
            val = cmul(f3(r.w), bsdf_eval(sc.bsdfs[vs.bsdf_id], f3(r.wi), fr.to_local(w1f)));
            ok = !is_zero3(val);
        }
        if (ok) {
            const float tr = eval_transmittance(sc, stack, tof(x0), w1f, true, med1, (float)dist, rng, r.depth, c);
            ok = tr > kEps;
        }
        if (ok) {
            // s(V) = m . (w0 dv0 + wb dv1 - dx0), m = (n_e - (n_e.w1) w1) / (dist pdf sppse)
            // 1 / (dist * angular pdf * sppse), angular pdf = pdf / theta
            const double nw = dotd(nrm, w1), k2 = ep.theta * rp.inv_sppse / (dist * pdf);
            const double3_ m = (nrm - w1 * nw) * k2;
            const float3 c0 = tof(m * w0), c1 = tof(m * wb), cx = tof(m * (-(w0 + wb)));
            const long long slot = queue_reserve_n(sc, qli, 2);  // the pair in adjacent slots
            for (int sgn = 0; sgn < 2 && slot >= 0; ++sgn) {
                const float3 w2 = edge_subpath_dir(ep, sgn);
                VLiTask &t = reinterpret_cast<VLiTask *>(qli.data)[slot + sgn];
                t.o[0] = r.x0[0]; t.o[1] = r.x0[1]; t.o[2] = r.x0[2];
                t.d[0] = w2.x; t.d[1] = w2.y; t.d[2] = w2.z;
                const float sg = sgn == 0 ? 1.f : -1.f;
                t.w[0] = val.x * sg; t.w[1] = val.y * sg; t.w[2] = val.z * sg;
                t.c0[0] = c0.x; t.c0[1] = c0.y; t.c0[2] = c0.z;
                t.c1[0] = c1.x; t.c1[1] = c1.y; t.c1[2] = c1.z;
                t.cx[0] = cx.x; t.cx[1] = cx.y; t.cx[2] = cx.z;
                t.v0 = e.v0; t.v1 = e.v1; t.chain = r.chain;
                t.med = med1; t.depth = r.depth; t.pixel = r.pixel; t.flags = 1;
                t.key = child_key(r.key, 8u + (uint32_t)sgn, (uint32_t)i);
            }
        }
    }
    if (ctr) flush_counters(ctr, K_EDGE, c, CT_EDGE_SAMPLES, nsamples);
}

// one thread per primary-edge sample: k_primary's geometry with the projection Jacobian
__global__ void __launch_bounds__(kBlock) k_vadj_primary(DevScene sc, RenderParams rp, Queue qli, const int *perm,
                                                         unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    uint32_t n = 0;
    if (gi < rp.prim_count) {
        const long long k = rp.prim_begin + (perm ? (long long)__ldg(perm + gi) : gi);  // sorted order, as k_primary
        Rng rng;
        rng.init(rp.seed, child_key(0x5052494DULL, (uint32_t)(k >> 32), (uint32_t)k));
        n = 1;
        double u = rng.next1d(), pdf;
        const int idx = sample_reuse(sc.pedge_cdf, sc.num_pedges, u, pdf);
        const DevPrimaryEdge &e = sc.pedges[idx];
        const DevCamera &cam = sc.cam;
        PrimaryPoint pp;
        primary_edge_point(cam, e, u, pp);
        const int ipx = pp.ipx, ipy = pp.ipy;
        const double fx = pp.px - ipx, fy = pp.py - ipy, nx = pp.nx, ny = pp.ny;
        const float maxd = pp.maxd;
        const int lx = ipx - rp.crop_x, ly = ipy - rp.crop_y;
        if (lx >= 0 && ly >= 0 && lx < rp.out_w && ly < rp.out_h) {
            // screen velocity of the edge point: ((1-u) J0 + u J1) [dv0; dv1], J in pixels
            const float *J = sc.pedge_jac + (size_t)idx * 24;  // [end][coord][6]
            float cv[6];
            for (int q = 0; q < 6; ++q) {
                const double jx = J[q] * (1.0 - u) + J[12 + q] * u, jy = J[6 + q] * (1.0 - u) + J[18 + q] * u;
                cv[q] = (float)(nx * jx + ny * jy);
            }
            float3 o, d;
            camera_ray(cam, ipx + fx, ipy + fy, o, d);
            const float tr = eval_transmittance(sc, stack, o, d, false, cam.med_id, maxd, rng, rp.max_bounces - 1, c);
            if (tr > kEps) {
                const long long slot = queue_reserve_n(sc, qli, 2);  // the pair in adjacent slots
                for (int sgn = 0; sgn < 2 && slot >= 0; ++sgn) {
                    const double delta = sgn == 0 ? -1e-4 : 1e-4;
                    float3 o2, d2;
                    camera_ray(cam, ipx + fx + nx * delta, ipy + fy + ny * delta, o2, d2);
                    VLiTask &t = reinterpret_cast<VLiTask *>(qli.data)[slot + sgn];
                    t.o[0] = o2.x; t.o[1] = o2.y; t.o[2] = o2.z;
                    t.d[0] = d2.x; t.d[1] = d2.y; t.d[2] = d2.z;
                    const float w = (float)(sgn == 0 ? rp.prim_weight : -rp.prim_weight);
                    t.w[0] = w; t.w[1] = w; t.w[2] = w;
                    t.c0[0] = cv[0]; t.c0[1] = cv[1]; t.c0[2] = cv[2];
                    t.c1[0] = cv[3]; t.c1[1] = cv[4]; t.c1[2] = cv[5];
                    t.cx[0] = t.cx[1] = t.cx[2] = 0.f;
                    t.v0 = sc.pedge_verts[2 * idx]; t.v1 = sc.pedge_verts[2 * idx + 1]; t.chain = -1;
                    t.med = cam.med_id; t.depth = rp.max_bounces; t.pixel = lx + rp.out_w * ly; t.flags = 1 | 2;
                    t.key = child_key(0x50524D31ULL + (uint64_t)k, 9u + (uint32_t)sgn, 0u);
                }
            }
        }
    }
    if (ctr) flush_counters(ctr, K_PRIMARY, c, CT_PRIMARY, n);
}

// one thread per VLiTask: Li, then K = dot(dL/dI, w (x) Li) times the coefficients; six
// resident blocks per SM and the pairs in sorted order (perm, or queue order), as k_li
__global__ void __launch_bounds__(kBlock, 6) k_vadj_li(DevScene sc, RenderParams rp, Queue qli, long long count,
                                                    const float *dimg, float *grad, float *xadj, const int *perm,
                                                    unsigned long long *ctr) {
    __shared__ int s_stack[kStackDepth * kBlock];
    int *stack = s_stack + threadIdx.x;
    const long long gi = (long long)blockIdx.x * kBlock + threadIdx.x;
    Ctr c;
    uint32_t n = 0;
    if (gi < count) {
        const long long slot = perm ? 2LL * __ldg(perm + (gi >> 1)) + (gi & 1) : gi;
        const VLiTask &t = reinterpret_cast<const VLiTask *>(qli.data)[slot];
        Rng rng;
        rng.init(rp.seed, t.key);
        n = 1;
        const float3 L = li_path(sc, stack, rng, f3(t.o), f3(t.d), t.depth, t.med, (t.flags & 1) != 0, c);
        const float3 gp = mk(__ldg(dimg + 3 * (size_t)t.pixel), __ldg(dimg + 3 * (size_t)t.pixel + 1),
                             __ldg(dimg + 3 * (size_t)t.pixel + 2));
        const float K = dot(gp, cmul(f3(t.w), L));
        if (K != 0.f && isfinite(K)) {
            scatter3(grad, t.v0, f3(t.c0) * K);
            scatter3(grad, t.v1, f3(t.c1) * K);
            if (t.chain >= 0) scatter3(xadj, t.chain, f3(t.cx) * K);
        }
    }
    if (ctr) flush_counters(ctr, K_LI, c, CT_LI, n);
}

}  // namespace dt
