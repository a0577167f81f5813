// dtrt_gb300 — device scene queries: BVH traversal, hit records, BSDFs, phase
// functions, emitters, media and the transmittance / NEE / emitter-lookup chains.
//
// Each function states the reference function it restates (uci-rendering/dtrt paths).
// Plain versions carry FP32 values; *_ad versions carry FP32 duals (Df<N>, DV<N>).
#pragma once
#include "dt_common.cuh"
#include "dt_scene.h"

namespace dt {

// Per-thread work counters, flushed once per thread when counters are enabled.
struct Ctr {
    uint32_t rays = 0, nodes = 0, tris = 0, lookups = 0, lights = 0;  // lights: emitter samples (CDF searches)
};

DT_D void set_error(const DevScene &sc, unsigned int bit) {
    if (sc.error_flags) atomicOr(sc.error_flags, bit);
}

// ------------------------------------------------------------------ generic scalar helpers
DT_HD float val(float x) { return x; }
template <int N> DT_HD float val(const Df<N> &x) { return x.v; }
DT_HD float dsqrt(float x) { return sqrtf(x); }
DT_HD float dexp(float x) { return expf(x); }
DT_HD float dabs(float x) { return fabsf(x); }
DT_HD float dpow(float a, float e) { return powf(a, e); }
template <class S> struct VecOf;
template <> struct VecOf<float> { typedef float3 T; };
template <int N> struct VecOf<Df<N>> { typedef DV<N> T; };
DT_HD float3 make_vec(float a, float b, float c) { return mk(a, b, c); }
template <int N> DT_HD DV<N> make_vec(const Df<N> &a, const Df<N> &b, const Df<N> &c) { return DV<N>(a, b, c); }
DT_HD float3 vval(float3 a) { return a; }
template <int N> DT_HD float3 vval(const DV<N> &a) { return a.val(); }

template <int N> DT_D Df<N> load_dual(float v, const float *d) {
    Df<N> r(v);
#pragma unroll
    for (int j = 0; j < N; ++j) r.d[j] = d[j];
    return r;
}
template <int N> DT_D DV<N> load_dual3(const float *v, const float (*d)[3]) {
    DV<N> r(mk(v[0], v[1], v[2]));
#pragma unroll
    for (int j = 0; j < N; ++j) r.set_grad(j, mk(d[j][0], d[j][1], d[j][2]));
    return r;
}
DT_D float3 f3(const float *p) { return mk(p[0], p[1], p[2]); }
DT_D float3 f3(float4 a) { return mk(a.x, a.y, a.z); }

// ------------------------------------------------------------------ BVH closest hit
// Replaces rtcIntersect1 (src/scene.cpp:172 and its other call sites): closest
// triangle with t in [tmin, tmax]. Two-child node tests against the current best
// distance; the per-thread stack lives in shared memory (stride kBlock).
constexpr int kStackExit = (int)0x80000000;
// Hard bound on null-interface crossings of one transmittance / emitter-lookup chain
// (the reference bounds them by max_interactions, which can be -1 = unbounded).
constexpr int kMaxInteractions = 4096;

DT_HEAVY int closest_hit(const DevScene &sc, int *stack, float3 o, float3 d, float tmin, float tmax, float &t_hit,
                     Ctr &c) {
    c.rays++;
    const float3 inv = mk(1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x)),
                          1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y)),
                          1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z)));
    const float3 oi = cmul(o, inv);
    int best = -1;
    float best_t = tmax;
    int sp = 0;
    int code = sc.num_nodes > 0 ? 0 : kStackExit;
    while (code != kStackExit) {
        while (code >= 0) {
            const float4 *np = reinterpret_cast<const float4 *>(sc.nodes + code);
            const float4 nx = __ldg(np), ny = __ldg(np + 1), nz = __ldg(np + 2);
            const int4 ch = __ldg(reinterpret_cast<const int4 *>(np + 3));
            c.nodes++;
            // left child slabs
            float a0 = nx.x * inv.x - oi.x, a1 = nx.y * inv.x - oi.x;
            float b0 = ny.x * inv.y - oi.y, b1 = ny.y * inv.y - oi.y;
            float c0 = nz.x * inv.z - oi.z, c1 = nz.y * inv.z - oi.z;
            float ln = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), tmin));
            float lf = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(c0, c1), best_t));
            // right child slabs
            a0 = nx.z * inv.x - oi.x; a1 = nx.w * inv.x - oi.x;
            b0 = ny.z * inv.y - oi.y; b1 = ny.w * inv.y - oi.y;
            c0 = nz.z * inv.z - oi.z; c1 = nz.w * inv.z - oi.z;
            float rn = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), tmin));
            float rf = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(c0, c1), best_t));
            bool hl = ln <= lf, hr = rn <= rf;
            if (hl && hr) {
                int nearc = ln <= rn ? ch.x : ch.y, farc = ln <= rn ? ch.y : ch.x;
                if (sp >= kStackDepth) {
                    set_error(sc, ERR_STACK);
                    code = kStackExit;
                    break;
                }
                stack[sp * kBlock] = farc;
                ++sp;
                code = nearc;
            } else if (hl) {
                code = ch.x;
            } else if (hr) {
                code = ch.y;
            } else {
                code = sp > 0 ? stack[(--sp) * kBlock] : kStackExit;
            }
        }
        if (code == kStackExit) break;
        // leaf: ~(first << 3 | (count - 1))
        const int enc = ~code;
        const int first = enc >> 3, count = (enc & 7) + 1;
        for (int k = 0; k < count; ++k) {
            const float4 *tp = sc.leaf_tris + 3 * (first + k);
            const float4 A = __ldg(tp), E1 = __ldg(tp + 1), E2 = __ldg(tp + 2);
            c.tris++;
            const float3 e1 = f3(E1), e2 = f3(E2);
            const float3 pv = cross(d, e2);
            const float det = dot(e1, pv);
            if (det == 0.f) continue;
            const float idet = 1.0f / det;
            const float3 s = o - f3(A);
            const float u = dot(s, pv) * idet;
            if (u < 0.f || u > 1.f) continue;
            const float3 q = cross(s, e1);
            const float v = dot(d, q) * idet;
            if (v < 0.f || u + v > 1.f) continue;
            const float t = dot(e2, q) * idet;
            if (t >= tmin && t <= best_t) {
                best_t = t;
                best = __float_as_int(A.w);
            }
        }
        code = sp > 0 ? stack[(--sp) * kBlock] : kStackExit;
    }
    t_hit = best_t;
    return best;
}

// ------------------------------------------------------------------ hit records
struct Its {  // include/intersection.h:15-58 (value part)
    int shape = -1, prim = -1;
    float t = INFINITY;
    float3 p, ng, wi;
    Frame fr;  // shading frame
    DT_D bool valid() const { return shape >= 0; }
    DT_D float3 to_local(float3 v) const { return fr.to_local(v); }
    DT_D float3 to_world(float3 v) const { return fr.to_world(v); }
};

template <int N>
struct ItsAD {  // include/intersectionAD.h:8-56; the shading frame is rebuilt from ns on demand
    int shape = -1, prim = -1;
    Df<N> t = Df<N>(INFINITY);
    DV<N> p, ns, wi;
    float3 ng;  // geometric normal value (only its value is used downstream)
    DT_D bool valid() const { return shape >= 0; }
    DT_D FrameAD<N> frame() const { return FrameAD<N>(ns); }
    DT_D Its plain() const {
        Its r;
        r.shape = shape; r.prim = prim; r.t = t.v; r.p = p.val(); r.ng = ng; r.wi = wi.val();
        r.fr = Frame(ns.val());
        return r;
    }
};

DT_D int target_medium(const DevScene &sc, int shape, float3 ng, float3 d) {
    const DevShape &s = sc.shapes[shape];
    return dot(d, ng) > 0.f ? s.med_ext : s.med_int;
}
DT_D bool is_transition(const DevShape &s) { return s.med_ext >= 0 || s.med_int >= 0; }
DT_D bool bsdf_is_null(const DevScene &sc, int shape) { return sc.bsdfs[sc.shapes[shape].bsdf_id].type == BSDF_NULL; }

template <int N>
DT_D DV<N> vertex_ad(const DevScene &sc, int v) {
    DV<N> r(f3(__ldg(sc.verts + v)));
    if (sc.vert_der) {
        const float *g = sc.vert_der + (size_t)v * sc.nder * 3;
#pragma unroll
        for (int j = 0; j < N; ++j) r.set_grad(j, mk(g[3 * j], g[3 * j + 1], g[3 * j + 2]));
    }
    return r;
}

// utils.cpp:218-235 Moller-Trumbore with the divisor clamp; shape.cpp:166-208
DT_D void shape_intersect(const DevScene &sc, int prim, float3 o, float3 d, Its &its) {
    const int4 tri = __ldg(sc.tris + prim);
    const float3 v0 = f3(__ldg(sc.verts + tri.x)), v1 = f3(__ldg(sc.verts + tri.y)), v2 = f3(__ldg(sc.verts + tri.z));
    const float3 e1 = v1 - v0, e2 = v2 - v0, pv = cross(d, e2);
    float div = dot(pv, e1);
    if (fabsf(div) < kEps) div = div > 0.f ? kEps : -kEps;
    const float3 s = o - v0, q = cross(s, e1);
    const float u = dot(s, pv) / div, v = dot(d, q) / div, t = dot(e2, q) / div, w = 1.f - (u + v);
    float3 gn = f3(__ldg(sc.face_n + prim)), sn = gn;
    const DevShape &sh = sc.shapes[tri.w];
    if (sh.has_normals) {
        sn = normalize(f3(__ldg(sc.normals + tri.x)) * w + f3(__ldg(sc.normals + tri.y)) * u +
                       f3(__ldg(sc.normals + tri.z)) * v);
        if (dot(gn, sn) < 0.f) gn = -gn;
    }
    its.shape = tri.w;
    its.prim = prim;
    its.t = t;
    its.p = o + d * t;
    its.ng = gn;
    its.fr = Frame(sn);
    its.wi = its.fr.to_local(-d);
}

template <int N>
struct RayAD {
    DV<N> o, d;
};

// utils.cpp:237-254 and shape.cpp:210-252
template <int N>
DT_HEAVY void shape_intersect_ad(const DevScene &sc, int prim, const RayAD<N> &ray, ItsAD<N> &its) {
    if (!sc.vert_der && !sc.face_n_der && !sc.normal_der && ray.o.der_zero(0.f) && ray.d.der_zero(0.f)) {
        // static geometry hit by a ray without derivatives: every slot is zero; the values
        // below follow the dual expressions operation for operation
        const int4 tri = __ldg(sc.tris + prim);
        const float3 o = ray.o.val(), d = ray.d.val();
        const float3 v0 = f3(__ldg(sc.verts + tri.x)), e1 = f3(__ldg(sc.verts + tri.y)) - v0,
                     e2 = f3(__ldg(sc.verts + tri.z)) - v0, pv = cross(d, e2);
        float div = dot(pv, e1);
        if (fabsf(div) < kEps) div = div > 0.f ? kEps : -kEps;
        const float3 s = o - v0, q = cross(s, e1);
        const float idiv = 1.0f / div;
        const float u = dot(s, pv) * idiv, v = dot(d, q) * idiv, t = dot(e2, q) * idiv, w = 1.f - (u + v);
        float3 gn = f3(__ldg(sc.face_n + prim)), sn = gn;
        const DevShape &sh = sc.shapes[tri.w];
        if (sh.has_normals) {
            sn = normalize(f3(__ldg(sc.normals + tri.x)) * w + f3(__ldg(sc.normals + tri.y)) * u +
                           f3(__ldg(sc.normals + tri.z)) * v);
            if (dot(gn, sn) < 0.f) gn = -gn;
        }
        its.shape = tri.w;
        its.prim = prim;
        its.t = Df<N>(t);
        its.p = DV<N>(o + d * t);
        its.ng = gn;
        its.ns = DV<N>(sn);
        its.wi = DV<N>(Frame(sn).to_local(-d));
        return;
    }
    const int4 tri = __ldg(sc.tris + prim);
    const DV<N> v0 = vertex_ad<N>(sc, tri.x), v1 = vertex_ad<N>(sc, tri.y), v2 = vertex_ad<N>(sc, tri.z);
    const DV<N> e1 = v1 - v0, e2 = v2 - v0, pv = cross(ray.d, e2);
    Df<N> div = dot(pv, e1);
    if (fabsf(div.v) < kEps) div = Df<N>(div.v > 0.f ? kEps : -kEps);
    const DV<N> s = ray.o - v0, q = cross(s, e1);
    const Df<N> idiv = 1.0f / div;
    const Df<N> u = dot(s, pv) * idiv, v = dot(ray.d, q) * idiv, t = dot(e2, q) * idiv;
    const Df<N> w = 1.f - (u + v);
    DV<N> gn(f3(__ldg(sc.face_n + prim)));
    if (sc.face_n_der) {
        const float *g = sc.face_n_der + (size_t)prim * sc.nder * 3;
#pragma unroll
        for (int j = 0; j < N; ++j) gn.set_grad(j, mk(g[3 * j], g[3 * j + 1], g[3 * j + 2]));
    }
    DV<N> sn = gn;
    const DevShape &sh = sc.shapes[tri.w];
    if (sh.has_normals) {
        auto nrm = [&](int vi) {
            DV<N> r(f3(__ldg(sc.normals + vi)));
            if (sc.normal_der) {
                const float *g = sc.normal_der + (size_t)vi * sc.nder * 3;
#pragma unroll
                for (int j = 0; j < N; ++j) r.set_grad(j, mk(g[3 * j], g[3 * j + 1], g[3 * j + 2]));
            }
            return r;
        };
        sn = normalize(nrm(tri.x) * w + nrm(tri.y) * u + nrm(tri.z) * v);
        if (dot(gn.val(), sn.val()) < 0.f) gn = -gn;
    }
    its.shape = tri.w;
    its.prim = prim;
    its.t = t;
    its.p = ray.o + ray.d * t;
    its.ng = gn.val();
    its.ns = sn;
    its.wi = FrameAD<N>(sn).to_local(-ray.d);
}

// ------------------------------------------------------------------ microfacet.h
template <class S>
DT_D S beckmann_d(const S &alpha, const typename VecOf<S>::T &m) {  // microfacet.h:24-51
    if (val(m.z) < kEps) return S(0.f);
    S cos2 = m.z * m.z;
    S expo = (m.x * m.x + m.y * m.y) / (alpha * alpha * cos2);
    S r = dexp(-expo) / (kPi * alpha * alpha * cos2 * cos2);
    if (val(r) * val(m.z) < 1e-20f) r = S(0.f);
    return r;
}
template <class S>
DT_D S tan_theta(const typename VecOf<S>::T &v) {  // frame.h:64-67
    S tmp = 1.f - v.z * v.z;
    return val(tmp) < kEps ? S(0.f) : dsqrt(tmp) / v.z;
}
template <class S>
DT_D S smith_g1(const S &alpha, const typename VecOf<S>::T &v, const typename VecOf<S>::T &m) {  // microfacet.h:118-155
    if (val(dot(v, m)) * val(v.z) < kEps) return S(1.f) * 0.f;
    S tt = dabs(tan_theta<S>(v));
    if (val(tt) == 0.f) return S(1.f);
    S a = 1.f / (alpha * tt);
    if (val(a) >= 1.6f) return S(1.f);
    S a2 = a * a;
    return (3.535f * a + 2.181f * a2) / (1.f + 2.276f * a + 2.577f * a2);
}

// math_func.cpp:6-54 of the reference: A&S 7.1.26 erf and Giles' erfinv approximations
DT_D float approx_erf(float x) {
    const float a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f, a4 = -1.453152027f,
                a5 = 1.061405429f, p = 0.3275911f;
    float sign = signum(x);
    x = fabsf(x);
    float t = 1.f / (1.f + p * x);
    float y = 1.f - (((((a5 * t + a4) * t) + a3) * t + a2) * t + a1) * t * expf(-x * x);
    return sign * y;
}
DT_D float approx_erfinv(float x) {
    float w = -logf((1.f - x) * (1.f + x)), p;
    if (w < 5.f) {
        w = w - 2.5f;
        p = 2.81022636e-08f;
        p = 3.43273939e-07f + p * w;
        p = -3.5233877e-06f + p * w;
        p = -4.39150654e-06f + p * w;
        p = 0.00021858087f + p * w;
        p = -0.00125372503f + p * w;
        p = -0.00417768164f + p * w;
        p = 0.246640727f + p * w;
        p = 1.50140941f + p * w;
    } else {
        w = sqrtf(w) - 3.f;
        p = -0.000200214257f;
        p = 0.000100950558f + p * w;
        p = 0.00134934322f + p * w;
        p = -0.00367342844f + p * w;
        p = 0.00573950773f + p * w;
        p = -0.0076224613f + p * w;
        p = 0.00943887047f + p * w;
        p = 1.00167406f + p * w;
        p = 2.83297682f + p * w;
    }
    return p * x;
}
DT_HEAVY void sample_visible11(float theta_i, float u, float v, float &sx, float &sy) {  // microfacet.h:178-244
    const float SQRT_PI_INV = 0.56418958354775628f;
    if (theta_i < 1e-4f) {
        float r = sqrtf(-logf(1.f - u));
        float sp, cp;
        sincosf(2.f * kPi * v, &sp, &cp);
        sx = r * cp;
        sy = r * sp;
        return;
    }
    float tan_i = tanf(theta_i), cot_i = 1.f / tan_i;
    float a = -1.f, c = approx_erf(cot_i);
    float ux = fmaxf(u, 1e-6f);
    float fit = 1.f + theta_i * (-0.876f + theta_i * (0.4265f - 0.0594f * theta_i));
    float b = c - (1.f + c) * powf(1.f - ux, fit);
    float normalization = 1.f / (1.f + c + SQRT_PI_INV * tan_i * expf(-cot_i * cot_i));
    for (int it = 1; it < 10; ++it) {
        if (!(b >= a && b <= c)) b = 0.5f * (a + c);
        float ie = approx_erfinv(b);
        float value = normalization * (1.f + b + SQRT_PI_INV * tan_i * expf(-ie * ie)) - ux;
        float deriv = normalization * (1.f - ie * tan_i);
        if (fabsf(value) < 1e-5f) break;
        if (value > 0.f) c = b;
        else a = b;
        b -= value / deriv;
    }
    sx = approx_erfinv(b);
    sy = approx_erfinv(2.f * fmaxf(v, 1e-6f) - 1.f);
}
DT_D float3 microfacet_sample(float alpha, float3 wi_in, float u, float v) {  // microfacet.h:65-92
    float3 wi = normalize(mk(alpha * wi_in.x, alpha * wi_in.y, wi_in.z));
    float theta = 0.f, phi = 0.f;
    if (wi.z < 0.99999f) {
        theta = acosf(wi.z);
        phi = atan2f(wi.y, wi.x);
    }
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float sx, sy;
    sample_visible11(theta, u, v, sx, sy);
    float tx = (cp * sx - sp * sy) * alpha, ty = (sp * sx + cp * sy) * alpha;
    float nrm = 1.f / sqrtf(tx * tx + ty * ty + 1.f);
    return mk(-tx * nrm, -ty * nrm, nrm);
}
DT_D float microfacet_pdf(float alpha, float3 wi, float3 m) {  // microfacet.h:96-99
    if (fabsf(wi.z) < kEps) return 0.f;
    return smith_g1<float>(alpha, wi, m) * fabsf(dot(wi, m)) * beckmann_d<float>(alpha, m) / fabsf(wi.z);
}

// utils.cpp:119-184 (plain and dual)
template <class S>
DT_D S fresnel_dielectric(const S &cos_i_in, S &cos_t_out, const S &eta) {
    if (fabsf(val(eta) - 1.f) < kEps) {
        cos_t_out = -cos_i_in;
        return S(0.f);
    }
    S scale = val(cos_i_in) > 0.f ? 1.f / eta : eta;
    S cos_t_sqr = 1.f - (1.f - cos_i_in * cos_i_in) * (scale * scale);
    if (val(cos_t_sqr) < kEps) {
        cos_t_out = S(0.f);
        return S(1.f);
    }
    S ci = dabs(cos_i_in), ct = dsqrt(cos_t_sqr);
    S rs = (ci - eta * ct) / (ci + eta * ct);
    S rp = (eta * ci - ct) / (eta * ci + ct);
    cos_t_out = val(cos_i_in) > 0.f ? -ct : ct;
    return 0.5f * (rs * rs + rp * rp);
}

// ------------------------------------------------------------------ BSDFs
template <class S>
DT_D typename VecOf<S>::T rough_dielectric_eval(const S &alpha, const S &eta, const S &inv_eta,
                                                const typename VecOf<S>::T &wi, const typename VecOf<S>::T &wo) {
    typedef typename VecOf<S>::T V;  // roughdielectric.cpp:9-118 / 121-170
    if (fabsf(val(wi.z)) < kEps || fabsf(val(wo.z)) < kEps) return V();
    const bool refl = val(wi.z) * val(wo.z) > 0.f;
    V H = refl ? normalize(wo + wi) : normalize(wi + wo * (val(wi.z) > 0.f ? eta : inv_eta));
    H = H * signum(val(H.z));
    S D = beckmann_d<S>(alpha, H);
    if (fabsf(val(D)) < kEps) return V();
    S ct;
    S F = fresnel_dielectric<S>(dot(wi, H), ct, eta);
    S G = smith_g1<S>(alpha, wi, H) * smith_g1<S>(alpha, wo, H);
    S r;
    if (refl) {
        r = F * D * G / (4.f * dabs(wi.z));
    } else {
        const S e = val(wi.z) > 0.f ? eta : inv_eta;
        S sd = dot(wi, H) + e * dot(wo, H);
        S value = ((1.f - F) * D * G * e * e * dot(wi, H) * dot(wo, H)) / (wi.z * sd * sd);
        const S factor = val(wi.z) > 0.f ? inv_eta : eta;
        r = dabs(value * factor * factor);
    }
    return make_vec(r, r, r);
}

template <class S>
DT_D typename VecOf<S>::T phong_eval(const typename VecOf<S>::T &kd, const typename VecOf<S>::T &ks, const S &e,
                                     const typename VecOf<S>::T &wi, const typename VecOf<S>::T &wo) {
    typedef typename VecOf<S>::T V;  // phong.cpp:19-53
    if (val(wi.z) < kEps || val(wo.z) < kEps) return V();
    S a = dot(wo, make_vec(-wi.x, -wi.y, wi.z));
    V r = kd * kInvPi;
    if (val(a) > 0.f) r = r + ks * ((e + 2.f) * dpow(a, e) * kInvTwoPi);
    return r * wo.z;
}

DT_D float3 bsdf_eval(const DevBsdf &b, float3 wi, float3 wo) {
    switch (b.type) {
        case BSDF_NULL: return mk(1.f, 1.f, 1.f);
        case BSDF_DIFFUSE:  // diffuse.cpp:7-12
            if (wi.z < kEps || wo.z < kEps) return mk(0.f, 0.f, 0.f);
            return f3(b.diffuse) * (kInvPi * wo.z);
        case BSDF_PHONG: return phong_eval<float>(f3(b.diffuse), f3(b.specular), b.exponent, wi, wo);
        default: return rough_dielectric_eval<float>(b.alpha, b.eta, b.inv_eta, wi, wo);
    }
}

template <int N>
DT_D DV<N> bsdf_eval_ad(const DevBsdf &b, const DV<N> &wi, const DV<N> &wo) {
    // no parameter slots and fixed directions: the plain evaluation, lifted (all slots zero)
    if (!b.has_der && wi.der_zero(0.f) && wo.der_zero(0.f)) return DV<N>(bsdf_eval(b, wi.val(), wo.val()));
    switch (b.type) {
        case BSDF_NULL: return DV<N>(mk(1.f, 1.f, 1.f));
        case BSDF_DIFFUSE:  // diffuse.cpp:15-20
            if (wi.z.v < kEps || wo.z.v < kEps) return DV<N>();
            return load_dual3<N>(b.diffuse, b.d_diffuse) * (wo.z * kInvPi);
        case BSDF_PHONG:
            return phong_eval<Df<N>>(load_dual3<N>(b.diffuse, b.d_diffuse), load_dual3<N>(b.specular, b.d_specular),
                                     load_dual<N>(b.exponent, b.d_exponent), wi, wo);
        default:
            return rough_dielectric_eval<Df<N>>(load_dual<N>(b.alpha, b.d_alpha), load_dual<N>(b.eta, b.d_eta),
                                                load_dual<N>(b.inv_eta, b.d_inv_eta), wi, wo);
    }
}

DT_D float bsdf_pdf(const DevBsdf &b, float3 wi, float3 wo) {
    switch (b.type) {
        case BSDF_NULL: return 1.f;
        case BSDF_DIFFUSE:  // diffuse.cpp:33-38
            if (wi.z < kEps || wo.z < kEps) return 0.f;
            return cosine_hemisphere_pdf(wo);
        case BSDF_PHONG: {  // phong.cpp:82-95
            if (wi.z < kEps || wo.z < kEps) return 0.f;
            float dp = cosine_hemisphere_pdf(wo), sp = 0.f;
            float a = dot(wo, mk(-wi.x, -wi.y, wi.z));
            if (a > 0.f) sp = powf(a, b.exponent) * (b.exponent + 1.f) / (2.f * kPi);
            return b.spec_weight * sp + (1.f - b.spec_weight) * dp;
        }
        default: {  // roughdielectric.cpp:172-206
            const bool refl = wi.z * wo.z > 0.f;
            float3 H;
            float dwh;
            if (refl) {
                H = normalize(wi + wo);
                dwh = 1.f / (4.f * dot(wo, H));
            } else {
                float e = wi.z > 0.f ? b.eta : b.inv_eta;
                H = normalize(wi + wo * e);
                float sd = dot(wi, H) + e * dot(wo, H);
                dwh = (e * e * dot(wo, H)) / (sd * sd);
            }
            H = H * signum(H.z);
            float prob = microfacet_pdf(b.alpha, wi * signum(wi.z), H);
            float ct;
            float F = fresnel_dielectric<float>(dot(wi, H), ct, b.eta);
            prob *= refl ? F : (1.f - F);
            return fabsf(prob * dwh);
        }
    }
}

DT_HEAVY float3 bsdf_sample(const DevBsdf &b, float3 wi, float r0, float r1, float r2, float3 &wo, float &pdf,
                        float &eta) {
    const float3 zero = mk(0.f, 0.f, 0.f);
    switch (b.type) {
        case BSDF_NULL:  // null.cpp:13-18
            wo = -wi;
            pdf = 1.f;
            eta = 1.f;
            return mk(1.f, 1.f, 1.f);
        case BSDF_DIFFUSE:  // diffuse.cpp:23-30
            if (wi.z < kEps) return zero;
            wo = square_to_cosine_hemisphere(r0, r1);
            eta = 1.f;
            pdf = cosine_hemisphere_pdf(wo);
            return f3(b.diffuse);
        case BSDF_PHONG: {  // phong.cpp:56-80
            if (r2 < b.spec_weight) {
                float3 R = mk(-wi.x, -wi.y, wi.z);
                float sa = sqrtf(fmaxf(0.f, 1.f - powf(r1, 2.f / (b.exponent + 1.f))));
                float ca = powf(r1, 1.f / (b.exponent + 1.f));
                float sp, cp;
                sincosf(2.f * kPi * r0, &sp, &cp);
                wo = Frame(R).to_world(mk(sa * cp, sa * sp, ca));
                if (wo.z < kEps) return zero;
            } else {
                wo = square_to_cosine_hemisphere(r0, r1);
            }
            eta = 1.f;
            pdf = bsdf_pdf(b, wi, wo);
            if (pdf < kEps) return zero;
            return bsdf_eval(b, wi, wo) / pdf;
        }
        default: {  // roughdielectric.cpp:120-170
            const float3 wis = wi * signum(wi.z);
            const float3 m = microfacet_sample(b.alpha, wis, r0, r1);
            const float mpdf = microfacet_pdf(b.alpha, wis, m);
            if (mpdf < kEps) return zero;
            pdf = mpdf;
            float ct;
            const float F = fresnel_dielectric<float>(dot(wi, m), ct, b.eta);
            float weight = 1.f, dwh;
            const bool sref = !(r2 > F);
            pdf *= sref ? F : (1.f - F);
            if (sref) {
                wo = m * (2.f * dot(wi, m)) - wi;
                eta = 1.f;
                if (wi.z * wo.z < kEps) return zero;
                dwh = 1.f / (4.f * dot(wo, m));
            } else {
                if (fabsf(ct) < kEps) return zero;
                const float e = ct < 0.f ? b.eta : b.inv_eta;  // refract() inverts eta when cos_t < 0
                const float er = ct < 0.f ? 1.f / b.eta : b.eta;
                wo = m * (dot(wi, m) * er + ct) - wi * er;
                eta = e;
                if (wi.z * wo.z >= 0.f) return zero;
                const float factor = ct < 0.f ? b.inv_eta : b.eta;
                weight *= factor * factor;
                const float sd = dot(wi, m) + eta * dot(wo, m);
                dwh = (eta * eta * dot(wo, m)) / (sd * sd);
            }
            weight *= smith_g1<float>(b.alpha, wo, m);
            pdf *= fabsf(dwh);
            return mk(weight, weight, weight);
        }
    }
}

// bsdf.cpp:11-21 (null.cpp:20-25 for the null BSDF)
template <int N>
DT_D DV<N> bsdf_sample_ad(const DevBsdf &b, const ItsAD<N> &its, const FrameAD<N> &fr, const Its &its0, float r0,
                          float r1, float r2, DV<N> &wo, float &pdf, float &eta) {
    if (b.type == BSDF_NULL) {
        wo = -its.wi;
        pdf = 1.f;
        eta = 1.f;
        return DV<N>(mk(1.f, 1.f, 1.f));
    }
    float3 wo0;
    DV<N> ret;
    const bool fixed = !b.has_der && its.wi.der_zero(0.f) && fr.n.der_zero(0.f);
    if (!is_zero3(bsdf_sample(b, its0.wi, r0, r1, r2, wo0, pdf, eta)))
        if (pdf > kEps) {
            if (fixed) {  // no slot can become non-zero: plain evaluation, lifted
                const float3 w = fr.plain().to_local(its0.to_world(wo0));
                wo = DV<N>(w);
                ret = DV<N>(bsdf_eval(b, its.wi.val(), w) / pdf);
            } else {
                wo = fr.to_local(its0.to_world(wo0));
                ret = bsdf_eval_ad<N>(b, its.wi, wo) / pdf;
            }
        }
    return ret;
}

// ------------------------------------------------------------------ phase functions, phase.h
DT_D float phase_eval(const DevPhase &p, float3 wi, float3 wo) {
    if (p.type == PHASE_ISOTROPIC) return kInvFourPi;
    float g = p.g, tmp = 1.f + g * g + 2.f * g * dot(wi, wo);
    return kInvFourPi * (1.f - g * g) / (tmp * sqrtf(tmp));
}
template <int N>
DT_D Df<N> phase_eval_ad(const DevPhase &p, const DV<N> &wi, const DV<N> &wo) {
    if (p.type == PHASE_ISOTROPIC) return Df<N>(kInvFourPi);
    if (!p.has_der && wi.der_zero(0.f) && wo.der_zero(0.f)) return Df<N>(phase_eval(p, wi.val(), wo.val()));
    Df<N> g = load_dual<N>(p.g, p.d_g);
    Df<N> tmp = 1.f + g * g + 2.f * g * dot(wi, wo);
    return kInvFourPi * (1.f - g * g) / dpow(tmp, 1.5f);
}
// phase.h:40-51: the HG local frame is built around wi (the reference's convention, kept)
DT_D float phase_sample(const DevPhase &p, float3 wi, float u, float v, float3 &wo) {
    if (p.type == PHASE_ISOTROPIC) {
        wo = square_to_uniform_sphere(u, v);
        return 1.f;
    }
    float g = p.g, ct;
    if (fabsf(g) < kEps) {
        ct = 1.f - 2.f * u;
    } else {
        float sq = (1.f - g * g) / (1.f - g + 2.f * g * u);
        ct = (1.f + g * g - sq * sq) / (2.f * g);
    }
    float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
    float sp, cp;
    sincosf(2.f * kPi * v, &sp, &cp);
    wo = Frame(wi).to_world(mk(st * cp, st * sp, ct));
    return 1.f;
}
template <int N>
DT_D Df<N> phase_sample_ad(const DevPhase &p, const DV<N> &wi, float u, float v, DV<N> &wo) {
    float3 w;
    phase_sample(p, wi.val(), u, v, w);
    wo = DV<N>(w);
    if (p.type == PHASE_ISOTROPIC) return Df<N>(1.f);  // phase.h:14-19 with evalAD == pdf
    Df<N> tmp = phase_eval_ad<N>(p, wi, wo);           // phase.h:53-58
    return tmp.v > kEps ? tmp / tmp.v : Df<N>(0.f);
}

// ------------------------------------------------------------------ emitters, area*.cpp
DT_D float3 le_normal(const DevEmitter &e, float3 n, float3 w) {
    if (e.type == EMITTER_AREA) return (e.two_sided || dot(n, w) > 0.f) ? f3(e.intensity) : mk(0.f, 0.f, 0.f);
    float t = dot(n, w);
    if (t > kEps) return f3(e.intensity) * (e.kappa * kInvTwoPi * expf(e.kappa * (t - 1.f)));
    return mk(0.f, 0.f, 0.f);
}
DT_D float3 le(const DevScene &sc, const Its &its, float3 w) {
    const DevEmitter &e = sc.emitters[sc.shapes[its.shape].light_id];
    return le_normal(e, e.type == EMITTER_AREA ? its.ng : its.fr.n, w);
}
template <int N>
DT_D DV<N> le_ad(const DevScene &sc, const ItsAD<N> &its, const DV<N> &w) {
    const DevEmitter &e = sc.emitters[sc.shapes[its.shape].light_id];
    if (e.type == EMITTER_AREA)
        return (e.two_sided || dot(its.ng, w.val()) > 0.f) ? DV<N>(f3(e.intensity)) : DV<N>();
    Df<N> t = dot(its.ns, w);
    if (t.v > kEps) {
        Df<N> k = load_dual<N>(e.kappa, e.d_kappa);
        return load_dual3<N>(e.intensity, e.d_intensity) * (dexp(k * (t - 1.f)) * k * kInvTwoPi);
    }
    return DV<N>();
}

// scene.cpp:302-313 light selection + shape.cpp:151-164 position sampling
DT_D int sample_light(const DevScene &sc, const float rnd[4], float3 &pos, float3 &n, float &pdf) {
    const int nl = sc.num_emitters;
    if (nl <= 0) {  // no emitter: every NEE estimate is zero
        pdf = 0.f;
        return -1;
    }
    int l = 0;
    while (l < nl && !(rnd[0] < sc.light_cdf[l])) ++l;  // upper_bound
    l = min(max(l, 0), nl - 1);
    const DevShape &s = sc.shapes[sc.emitters[l].shape_id];
    const float *cdf = sc.area_cdf + sc.area_cdf_begin[l];
    int lo = 0, hi = s.nt;
    while (lo < hi) {  // upper_bound
        int mid = (lo + hi) >> 1;
        if (rnd[1] < cdf[mid]) hi = mid;
        else lo = mid + 1;
    }
    const int t = min(max(lo, 0), s.nt - 1);
    const int4 tri = __ldg(sc.tris + s.tri_off + t);
    const float3 v0 = f3(__ldg(sc.verts + tri.x)), e1 = f3(__ldg(sc.verts + tri.y)) - v0,
                 e2 = f3(__ldg(sc.verts + tri.z)) - v0;
    const float a = sqrtf(rnd[2]), b1 = 1.f - a, b2 = a * rnd[3];
    n = normalize(cross(e1, e2));
    pos = v0 + e1 * b1 + e2 * b2;
    pdf = sc.light_pmf[l] / sc.light_area[l];
    return l;
}

// ------------------------------------------------------------------ grids, gridvolume.h
DT_D float3 grid_point(const DevGrid &g, float3 pw) {  // worldToVolume + volumeToGrid
    const float *m = g.w2v;
    float3 p = mk(m[0] * pw.x + m[1] * pw.y + m[2] * pw.z + m[3], m[4] * pw.x + m[5] * pw.y + m[6] * pw.z + m[7],
                  m[8] * pw.x + m[9] * pw.y + m[10] * pw.z + m[11]);
    return mk((p.x - g.mn[0]) * g.to_grid[0], (p.y - g.mn[1]) * g.to_grid[1], (p.z - g.mn[2]) * g.to_grid[2]);
}
template <int N>
DT_D DV<N> grid_point_ad(const DevGrid &g, const DV<N> &pw) {  // gridvolume.h:301-326
    const float *m = g.w2v;
    const float3 pv = pw.val();
    DV<N> p(grid_point(g, pv));
    const float3 q = pv - f3(g.center);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        float3 gg = pw.grad(j) - cross(f3(g.rot_vel[j]), q) - f3(g.trans_vel[j]);
        float3 gv = mk(m[0] * gg.x + m[1] * gg.y + m[2] * gg.z, m[4] * gg.x + m[5] * gg.y + m[6] * gg.z,
                       m[8] * gg.x + m[9] * gg.y + m[10] * gg.z);
        p.set_grad(j, mk(gv.x * g.to_grid[0], gv.y * g.to_grid[1], gv.z * g.to_grid[2]));
    }
    return p;
}
// Cell of the lower trilinear corner, or false when the 2x2x2 stencil leaves the grid
// (gridvolume.h:152-153: out of range reads as 0). The test runs on the float coordinate,
// where it is exact for finite values (0 <= floor(x) <= res-2 <=> 0 <= x < res-1) and
// also rejects NaN and +-inf, which an int conversion would map into range or saturate.
DT_D bool grid_cell(const DevGrid &g, float3 p, int &x1, int &y1, int &z1) {
    if (!(p.x >= 0.f && p.x < (float)(g.res[0] - 1) && p.y >= 0.f && p.y < (float)(g.res[1] - 1) && p.z >= 0.f &&
          p.z < (float)(g.res[2] - 1)))
        return false;
    x1 = (int)floorf(p.x);
    y1 = (int)floorf(p.y);
    z1 = (int)floorf(p.z);
    return true;
}
DT_D float grid_lookup(const DevGrid &g, float3 pw, Ctr &c) {  // gridvolume.h:144-171
    c.lookups++;
    const float3 p = grid_point(g, pw);
    int x1, y1, z1;
    if (!grid_cell(g, p, x1, y1, z1)) return 0.f;
    const float fx = p.x - x1, fy = p.y - y1, fz = p.z - z1, gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    const int sx = 1, sy = g.res[0], sz = g.res[0] * g.res[1];
    const float *d = g.data + (size_t)z1 * sz + (size_t)y1 * sy + x1;
    const float d000 = __ldg(d), d001 = __ldg(d + sx), d010 = __ldg(d + sy), d011 = __ldg(d + sy + sx);
    const float d100 = __ldg(d + sz), d101 = __ldg(d + sz + sx), d110 = __ldg(d + sz + sy), d111 = __ldg(d + sz + sy + sx);
    return ((d000 * gx + d001 * fx) * gy + (d010 * gx + d011 * fx) * fy) * gz +
           ((d100 * gx + d101 * fx) * gy + (d110 * gx + d111 * fx) * fy) * fz;
}
template <int N>
DT_D Df<N> grid_lookup_ad(const DevGrid &g, const DV<N> &pw, Ctr &c) {  // gridvolume.h:174-201
    const bool voxel_dirs = g.dgrid != nullptr && g.dgrid_n == N;
    // A static grid sampled at a point without derivatives has none either: the plain
    // lookup gives the same dual exactly (all slots zero) at a fraction of the cost.
    if (!g.moving && !voxel_dirs && pw.der_zero(0.f)) return Df<N>(grid_lookup(g, pw.val(), c));
    c.lookups++;
    const DV<N> p = grid_point_ad<N>(g, pw);
    int x1, y1, z1;
    if (!grid_cell(g, p.val(), x1, y1, z1)) return Df<N>(0.f);
    const Df<N> fx = p.x - (float)x1, fy = p.y - (float)y1, fz = p.z - (float)z1;
    const Df<N> gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    const int sx = 1, sy = g.res[0], sz = g.res[0] * g.res[1];
    const size_t base = (size_t)z1 * sz + (size_t)y1 * sy + x1;
    const float *d = g.data + base;
    const float d000 = __ldg(d), d001 = __ldg(d + sx), d010 = __ldg(d + sy), d011 = __ldg(d + sy + sx);
    const float d100 = __ldg(d + sz), d101 = __ldg(d + sz + sx), d110 = __ldg(d + sz + sy), d111 = __ldg(d + sz + sy + sx);
    Df<N> r = ((gx * d000 + fx * d001) * gy + (gx * d010 + fx * d011) * fy) * gz +
              ((gx * d100 + fx * d101) * gy + (gx * d110 + fx * d111) * fy) * fz;
    if (voxel_dirs) {
        // per-voxel directions: the value derivative d(density)/d(theta_j) at the point
        const float w[8] = {gx.v * gy.v * gz.v, fx.v * gy.v * gz.v, gx.v * fy.v * gz.v, fx.v * fy.v * gz.v,
                            gx.v * gy.v * fz.v, fx.v * gy.v * fz.v, gx.v * fy.v * fz.v, fx.v * fy.v * fz.v};
        const size_t off[8] = {0, (size_t)sx, (size_t)sy, (size_t)(sy + sx), (size_t)sz, (size_t)(sz + sx),
                               (size_t)(sz + sy), (size_t)(sz + sy + sx)};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float *q = g.dgrid + (base + off[k]) * N;
#pragma unroll
            for (int j = 0; j < N; ++j) r.d[j] += w[k] * __ldg(q + j);
        }
    }
    return r;
}

// ------------------------------------------------------------------ adjoint scatter
// Reverse-mode hook of the density lookups: the replay kernel sets `w` to the adjoint
// weight of the log-derivative factor being evaluated; every lookup that feeds that
// factor adds w * (its coefficient) * (trilinear weight) to the 8 voxels it read.
struct AdjCtx {
    float *grad;  // density gradient of all heterogeneous media (DevMedium::grad_off)
    float w;
};
DT_D void grid_scatter(const DevGrid &g, float *grad, float3 pw, float w) {
    // a zero weight adds nothing; a non-finite one (a factor whose suffix is zero times an
    // unbounded segment) would poison the gradient, as a non-finite pixel derivative is
    // dropped by the forward write rule
    if (w == 0.f || !isfinite(w)) return;
    const float3 p = grid_point(g, pw);
    int x1, y1, z1;
    if (!grid_cell(g, p, x1, y1, z1)) return;
    const float fx = p.x - x1, fy = p.y - y1, fz = p.z - z1, gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    const int sy = g.res[0], sz = g.res[0] * g.res[1];
    float *q = grad + (size_t)z1 * sz + (size_t)y1 * sy + x1;
    atomicAdd(q, w * gx * gy * gz);
    atomicAdd(q + 1, w * fx * gy * gz);
    atomicAdd(q + sy, w * gx * fy * gz);
    atomicAdd(q + sy + 1, w * fx * fy * gz);
    atomicAdd(q + sz, w * gx * gy * fz);
    atomicAdd(q + sz + 1, w * fx * gy * fz);
    atomicAdd(q + sz + sy, w * gx * fy * fz);
    atomicAdd(q + sz + sy + 1, w * fx * fy * fz);
}
DT_D float3 grid_lookup3(const DevGrid &g, float3 pw) {  // gridvolume.h:204-232
    const float3 p = grid_point(g, pw);
    int x1, y1, z1;
    if (!grid_cell(g, p, x1, y1, z1)) return mk(0.f, 0.f, 0.f);
    const float fx = p.x - x1, fy = p.y - y1, fz = p.z - z1, gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    float r[3];
    for (int ch = 0; ch < 3; ++ch) {
        auto D = [&](int z, int y, int x) { return __ldg(g.data + (((size_t)z * g.res[1] + y) * g.res[0] + x) * 3 + ch); };
        r[ch] = ((D(z1, y1, x1) * gx + D(z1, y1, x1 + 1) * fx) * gy + (D(z1, y1 + 1, x1) * gx + D(z1, y1 + 1, x1 + 1) * fx) * fy) * gz +
                ((D(z1 + 1, y1, x1) * gx + D(z1 + 1, y1, x1 + 1) * fx) * gy + (D(z1 + 1, y1 + 1, x1) * gx + D(z1 + 1, y1 + 1, x1 + 1) * fx) * fy) * fz;
    }
    return mk(r[0], r[1], r[2]);
}
template <int N>
DT_D DV<N> grid_lookup3_ad(const DevGrid &g, const DV<N> &pw) {  // gridvolume.h:235-263
    const DV<N> p = grid_point_ad<N>(g, pw);
    int x1, y1, z1;
    if (!grid_cell(g, p.val(), x1, y1, z1)) return DV<N>();
    const Df<N> fx = p.x - (float)x1, fy = p.y - (float)y1, fz = p.z - (float)z1;
    const Df<N> gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    Df<N> r[3];
    for (int ch = 0; ch < 3; ++ch) {
        auto D = [&](int z, int y, int x) { return __ldg(g.data + (((size_t)z * g.res[1] + y) * g.res[0] + x) * 3 + ch); };
        r[ch] = ((gx * D(z1, y1, x1) + fx * D(z1, y1, x1 + 1)) * gy + (gx * D(z1, y1 + 1, x1) + fx * D(z1, y1 + 1, x1 + 1)) * fy) * gz +
                ((gx * D(z1 + 1, y1, x1) + fx * D(z1 + 1, y1, x1 + 1)) * gy + (gx * D(z1 + 1, y1 + 1, x1) + fx * D(z1 + 1, y1 + 1, x1 + 1)) * fy) * fz;
    }
    return DV<N>(r[0], r[1], r[2]);
}
// aabb.h:185-215 slab test
DT_D bool aabb_hit(const DevGrid &g, float3 o, float3 d, float &tn, float &tf) {
    tn = -INFINITY;
    tf = INFINITY;
    for (int i = 0; i < 3; ++i) {
        const float oo = comp(o, i), dd = comp(d, i);
        if (dd == 0.f) {
            if (oo < g.lo[i] || oo > g.hi[i]) return false;
        } else {
            float t1 = (g.lo[i] - oo) / dd, t2 = (g.hi[i] - oo) / dd;
            if (t1 > t2) { float tmp = t1; t1 = t2; t2 = tmp; }
            tn = fmaxf(t1, tn);
            tf = fminf(t2, tf);
            if (!(tn <= tf)) return false;
        }
    }
    return true;
}

// ------------------------------------------------------------------ media
DT_D float3 sig_s(const DevMedium &m, float3 x, Ctr &c) {  // homogeneous.h:57, heterogeneous.h:88-90
    if (m.type == MEDIUM_HOMOGENEOUS) return f3(m.sigma_s);
    return f3(m.albedo) * (m.scale * grid_lookup(m.density, x, c));
}

// homogeneous.cpp:6-24 / heterogeneous.cpp:9-37; moves `o` to the scatter point
DT_HEAVY bool sample_distance(const DevScene &sc, const DevMedium &m, float3 &o, float3 d, float tmax, float r0, float r1,
                          Rng &rng, float3 &thr, Ctr &c) {
    if (m.type == MEDIUM_HOMOGENEOUS) {
        if (m.sampling_weight > kEps) {
            const float t = -logf(r0) / m.sigma_t;
            if (t < tmax) {
                o = o + d * t;
                if (r1 < m.sampling_weight) thr = cmul(thr, f3(m.albedo) / m.sampling_weight);
                else thr = mk(0.f, 0.f, 0.f);
                return true;
            }
            return false;
        }
        thr = thr * expf(-tmax * m.sigma_t);
        return false;
    }
    float tn, tf;
    if (!aabb_hit(m.density, o, d, tn, tf)) return false;
    tn = fmaxf(tn, 0.f);
    tf = fminf(tf, tmax);
    float t = tn;
    for (int dep = 0;; ++dep) {
        t -= logf(rng.next1()) * m.max_inv_density;
        if (t > tf) break;
        if (dep > sc.tracking_cap) {
            set_error(sc, ERR_TRACK_CAP);
            break;
        }
        const float3 p = o + d * t;
        const float dens = grid_lookup(m.density, p, c);
        if (rng.next1() * m.density.max_value < dens) {
            o = p;
            thr = cmul(thr, m.albedo_vol.valid ? grid_lookup3(m.albedo_vol, p) : f3(m.albedo));
            return true;
        }
    }
    return false;
}

// heterogeneous.cpp:121-141: -d/dtheta of the optical depth over [tmin, tmax]
// With `adj`, each sample also scatters adj->w * (-scale * len / 10) into the gradient:
// the factor exp(-optical depth) has log-derivative -(this integral).
template <int N>
DT_HEAVY void int_sig_t(const DevScene &sc, const DevMedium &m, const RayAD<N> &ray, const Df<N> &tmin, const Df<N> &tmax,
                    Rng &rng, float out[N], Ctr &c, const AdjCtx *adj = nullptr) {
    const Df<N> scale = load_dual<N>(m.scale, m.d_scale);
#pragma unroll
    for (int j = 0; j < N; ++j) out[j] = 0.f;
    const float len = tmax.v - tmin.v;
    const bool scatter = adj != nullptr && m.grad_off >= 0 && adj->w != 0.f;
    if (scale.der_zero(0.f) && !m.density.moving && !(m.density.dgrid && m.density.dgrid_n == N) &&
        ray.o.der_zero(0.f) && ray.d.der_zero(0.f) && tmin.der_zero(1e-6f) && tmax.der_zero(1e-6f)) {
        // nothing in the integral carries a derivative: every slot is zero. Draw the same
        // random numbers; the scatter pass only needs the sample positions.
        const float3 o = ray.o.val(), d = ray.d.val();
        for (int i = 0; i < 10; ++i) {
            const float r = ((float)i + rng.next1()) * 0.1f;
            if (scatter) {
                const float tt = tmin.v + len * r;
                grid_scatter(m.density, adj->grad + m.grad_off, o + d * tt, -adj->w * m.scale * len * 0.1f);
            }
        }
        return;
    }
    if (!m.density.moving && !(m.density.dgrid && m.density.dgrid_n == N) && ray.o.der_zero(0.f) &&
        ray.d.der_zero(0.f) && tmin.der_zero(0.f) && !scatter) {
        // sample positions without derivatives on a static grid: each sample's derivative is
        // d_scale[j] * density(p), so the integral needs only the sum of ten plain lookups
        const float3 o = ray.o.val(), d = ray.d.val();
        float sum = 0.f;
#pragma unroll
        for (int i = 0; i < 10; ++i) {
            const float r = ((float)i + rng.next1()) * 0.1f;
            sum += grid_lookup(m.density, o + d * (tmin.v + len * r), c);
        }
#pragma unroll
        for (int j = 0; j < N; ++j) out[j] = scale.d[j] * sum * (len * 0.1f);
    } else {
        for (int i = 0; i < 10; ++i) {
            const float r = ((float)i + rng.next1()) * 0.1f;
            const Df<N> tt = tmin + len * r;
            const DV<N> pt = ray.o + ray.d * tt;
            const Df<N> s = scale * grid_lookup_ad<N>(m.density, pt, c);
#pragma unroll
            for (int j = 0; j < N; ++j) out[j] += s.d[j];
            if (scatter) grid_scatter(m.density, adj->grad + m.grad_off, pt.val(), -adj->w * m.scale * len * 0.1f);
        }
#pragma unroll
        for (int j = 0; j < N; ++j) out[j] *= len * 0.1f;
    }
    const float3 o = ray.o.val(), d = ray.d.val();
    if (!tmax.der_zero(1e-6f)) {
        const float dv = m.scale * grid_lookup(m.density, o + d * (tmax.v - kEps), c);
#pragma unroll
        for (int j = 0; j < N; ++j) out[j] += tmax.d[j] * dv;
    }
    if (!tmin.der_zero(1e-6f)) {
        const float dv = m.scale * grid_lookup(m.density, o + d * (tmin.v + kEps), c);
#pragma unroll
        for (int j = 0; j < N; ++j) out[j] -= tmin.d[j] * dv;
    }
}

// homogeneous.cpp:27-49 / heterogeneous.cpp:40-75; moves ray.o to the scatter point
// With `adj`, the factor applied to `thr` scatters adj->w times its log-derivative.
template <int N>
DT_HEAVY bool sample_distance_ad(const DevScene &sc, const DevMedium &m, RayAD<N> &ray, const Df<N> &tmax, float r0,
                             float r1, Rng &rng, DV<N> &thr, Ctr &c, const AdjCtx *adj = nullptr) {
    if (m.type == MEDIUM_HOMOGENEOUS) {
        const Df<N> sig = load_dual<N>(m.sigma_t, m.d_sigma_t);
        if (m.sampling_weight > kEps) {
            const float t = -logf(r0) / m.sigma_t;
            if (t < tmax.v) {
                ray.o = ray.o + ray.d * t;
                if (r1 < m.sampling_weight) {
                    Df<N> tmp = sig * dexp(-t * sig);
                    Df<N> k = tmp / (tmp.v * m.sampling_weight);
                    thr = cmul(thr, load_dual3<N>(m.albedo, m.d_albedo) * k);
                } else {
                    thr = DV<N>();
                }
                return true;
            }
            Df<N> tmp = dexp(-(tmax * sig));
            thr = thr * (tmp / tmp.v);
            return false;
        }
        thr = thr * dexp(-(tmax * sig));
        return false;
    }
    float tn, tf;
    const float3 o = ray.o.val(), d = ray.d.val();
    if (!aabb_hit(m.density, o, d, tn, tf)) return false;
    tn = fmaxf(tn, 0.f);
    tf = fminf(tf, tmax.v);
    float t = tn;
    for (int dep = 0;; ++dep) {
        t -= logf(rng.next1()) * m.max_inv_density;
        if (t > tf) break;
        if (dep > sc.tracking_cap) {
            set_error(sc, ERR_TRACK_CAP);
            break;
        }
        // the acceptance test needs the density value only; a null collision discards the
        // derivative slots, so the dual lookup runs at an accepted collision (same point)
        const DV<N> p = ray.o + ray.d * t;
        const float dv = grid_lookup(m.density, p.val(), c);
        if (rng.next1() * m.density.max_value < dv) {
            Ctr again;  // the lookup just counted, repeated with its derivative slots
            const Df<N> dens = grid_lookup_ad<N>(m.density, p, again);
            // The reference aliases p_scatter with ray.org (volpathAD.cpp:164), so the
            // line integral below runs from the scatter point forward over [0, t].
            // EST_SCATTER_FROM_ORIGIN integrates the segment actually travelled instead.
            const RayAD<N> ray0 = ray;
            ray.o = p;
            const DV<N> alb = m.albedo_vol.valid ? grid_lookup3_ad<N>(m.albedo_vol, p) : load_dual3<N>(m.albedo, m.d_albedo);
            const Df<N> sig = load_dual<N>(m.scale, m.d_scale) * dens;
            if (adj != nullptr && m.grad_off >= 0)  // d log(sigma_t(p)) = d density / density
                grid_scatter(m.density, adj->grad + m.grad_off, p.val(), adj->w / dens.v);
            float ist[N];
            int_sig_t<N>(sc, m, (sc.est_flags & EST_SCATTER_FROM_ORIGIN) ? ray0 : ray, Df<N>(0.f), Df<N>(t), rng, ist,
                         c, adj);
            Df<N> tmp(1.f);
#pragma unroll
            for (int j = 0; j < N; ++j) tmp.d[j] = -ist[j];
            thr = cmul(thr, alb * (sig * tmp / sig.v));
            return true;
        }
    }
    float ist[N];
    int_sig_t<N>(sc, m, ray, Df<N>(0.f), tmax, rng, ist, c, adj);
    Df<N> tmp(1.f);
#pragma unroll
    for (int j = 0; j < N; ++j) tmp.d[j] = -ist[j];
    thr = thr * tmp;
    return false;
}

// homogeneous.cpp:52-55 / heterogeneous.cpp:78-91 (residual ratio tracking)
DT_HEAVY float medium_transmittance(const DevScene &sc, const DevMedium &m, float3 o, float3 d, float tmin, float tmax,
                                Rng &rng, Ctr &c) {
    if (m.type == MEDIUM_HOMOGENEOUS) return expf((tmin - tmax) * m.sigma_t);
    float ret = 1.f, t = tmin;
    int steps = 0;
    while (ret > kEps) {
        t -= logf(rng.next1()) * m.max_inv_density;
        if (t > tmax) break;
        if (++steps > sc.tracking_cap) {
            set_error(sc, ERR_TRACK_CAP);
            break;
        }
        ret *= 1.f - grid_lookup(m.density, o + d * t, c) / m.density.max_value;
    }
    return ret;
}
template <int N>
DT_HEAVY Df<N> medium_transmittance_ad(const DevScene &sc, const DevMedium &m, const RayAD<N> &ray, float tmin,
                                   const Df<N> &tmax, Rng &rng, Ctr &c, const AdjCtx *adj = nullptr) {
    if (m.type == MEDIUM_HOMOGENEOUS) return dexp((tmin - tmax) * load_dual<N>(m.sigma_t, m.d_sigma_t));
    Df<N> ret(medium_transmittance(sc, m, ray.o.val(), ray.d.val(), tmin, tmax.v, rng, c));  // heterogeneous.cpp:113-118
    float ist[N];
    int_sig_t<N>(sc, m, ray, Df<N>(tmin), tmax, rng, ist, c, adj);
#pragma unroll
    for (int j = 0; j < N; ++j) ret.d[j] = -ret.v * ist[j];
    return ret;
}

// ------------------------------------------------------------------ scene queries, scene.cpp
DT_D bool ray_intersect(const DevScene &sc, int *stack, float3 o, float3 d, bool on_surface, Its &its, Ctr &c) {
    float th;
    const int prim = closest_hit(sc, stack, o, d, on_surface ? kShadowEps : 0.f, INFINITY, th, c);
    if (prim < 0) {
        its.shape = -1;
        its.t = INFINITY;
        return false;
    }
    shape_intersect(sc, prim, o, d, its);
    return true;
}

template <int N>
DT_D bool ray_intersect_ad(const DevScene &sc, int *stack, const RayAD<N> &ray, bool on_surface, ItsAD<N> &its,
                           Ctr &c) {
    float th;
    const int prim = closest_hit(sc, stack, ray.o.val(), ray.d.val(), on_surface ? kShadowEps : 0.f, INFINITY, th, c);
    if (prim < 0) {
        its.shape = -1;
        its.t = Df<N>(INFINITY);
        return false;
    }
    shape_intersect_ad<N>(sc, prim, ray, its);
    return true;
}

// scene.cpp:177-237
DT_HEAVY float eval_transmittance(const DevScene &sc, int *stack, float3 o, float3 d, bool on_surface, int med,
                              float remaining, Rng &rng, int max_inter, Ctr &c) {
    float tmin = on_surface ? kShadowEps : 0.f;
    float tfar = (1.f - kShadowEps) * remaining;
    float tr = 1.f;
    int inter = 0;
    while (remaining > 0.f) {
        if (inter >= kMaxInteractions) return 0.f;  // also bounds max_inter == -1
        float tmax = remaining, th;
        const int prim = closest_hit(sc, stack, o, d, tmin, tfar, th, c);
        Its its;
        if (prim >= 0) {
            const int shape = __ldg(sc.tris + prim).w;
            if (inter == max_inter || !bsdf_is_null(sc, shape)) return 0.f;
            shape_intersect(sc, prim, o, d, its);
            if (its.t < tmax) tmax = its.t;
        }
        if (med >= 0) tr *= medium_transmittance(sc, sc.media[med], o, d, tmin, tmax, rng, c);
        if (prim < 0) break;
        const DevShape &s = sc.shapes[its.shape];
        if (is_transition(s)) med = dot(its.ng, d) > 0.f ? s.med_ext : s.med_int;
        o = o + d * tmax;
        tmin = kShadowEps;
        remaining -= tmax;
        tfar = (1.f - kShadowEps) * remaining;
        ++inter;
    }
    return tr;
}

// scene.cpp:617-701
DT_HEAVY float3 look_for_emitter(const DevScene &sc, int *stack, float3 o, float3 d, bool on_surface, Rng &rng, int med,
                             int max_inter, Its &its, float &pdf_nee, Ctr &c) {
    float tmin = on_surface ? kShadowEps : 0.f, th;
    const float3 scatter = o;
    int prim = closest_hit(sc, stack, o, d, tmin, INFINITY, th, c);
    const float3 zero = mk(0.f, 0.f, 0.f);
    if (prim < 0) {
        its.shape = -1;
        its.t = INFINITY;
        return zero;
    }
    shape_intersect(sc, prim, o, d, its);
    if (sc.has_grid_media) {  // geometry first: chains that miss every emitter skip transmittance
        float3 o1 = o;
        Its n1 = its;
        int p1 = prim;
        bool emitter = false;
        for (int inter = 0; inter < kMaxInteractions; ++inter) {
            if (inter > 0) shape_intersect(sc, p1, o1, d, n1);
            const DevShape &s = sc.shapes[n1.shape];
            if (s.light_id >= 0) {
                emitter = true;
                break;
            }
            if (inter == max_inter || sc.bsdfs[s.bsdf_id].type != BSDF_NULL) break;
            o1 = o1 + d * n1.t;
            p1 = closest_hit(sc, stack, o1, d, kShadowEps, INFINITY, th, c);
            if (p1 < 0) break;
        }
        if (!emitter) return zero;
    }
    float tr = 1.f;
    Its ni = its;
    for (int inter = 0; inter < kMaxInteractions; ++inter) {
        if (inter > 0) shape_intersect(sc, prim, o, d, ni);
        const float tmax = ni.t;
        if (med >= 0) tr *= medium_transmittance(sc, sc.media[med], o, d, tmin, tmax, rng, c);
        const DevShape &s = sc.shapes[ni.shape];
        if (s.light_id >= 0) {
            const float3 dp = ni.p - scatter;
            const float G = ni.wi.z / dot(dp, dp);
            pdf_nee = sc.light_pmf[s.light_id] / (sc.light_area[s.light_id] * G);
            return le(sc, ni, -d) * tr;
        }
        if (inter == max_inter || sc.bsdfs[s.bsdf_id].type != BSDF_NULL) return zero;
        if (is_transition(s)) med = dot(ni.ng, d) > 0.f ? s.med_ext : s.med_int;
        o = o + d * tmax;
        tmin = kShadowEps;
        prim = closest_hit(sc, stack, o, d, tmin, INFINITY, th, c);
        if (prim < 0) return zero;
    }
    return zero;
}

// scene.cpp:703-793
template <int N>
DT_HEAVY DV<N> look_for_emitter_ad(const DevScene &sc, int *stack, RayAD<N> ray, bool on_surface, Rng &rng, int med,
                               int max_inter, ItsAD<N> &its, float &pdf_nee, int *far_shape, float *far_t, Ctr &c,
                               const AdjCtx *adj = nullptr) {
    float tmin = on_surface ? kShadowEps : 0.f, th;
    const float3 scatter = ray.o.val();
    int prim = closest_hit(sc, stack, ray.o.val(), ray.d.val(), tmin, INFINITY, th, c);
    if (prim < 0) {
        its.shape = -1;
        its.t = Df<N>(INFINITY);
        return DV<N>();
    }
    shape_intersect_ad<N>(sc, prim, ray, its);
    if (sc.has_grid_media) {
        // Geometry first: follow null interfaces to the surface that ends the chain. A chain
        // that does not end at an emitter contributes nothing, so its transmittance (a
        // tracking estimate through the grid, with random numbers) is never evaluated. The
        // reference evaluates it segment by segment before the emitter test
        // (scene.cpp:660-690); the contribution is the same, its random numbers are not drawn.
        RayAD<N> r1 = ray;
        ItsAD<N> n1 = its;
        int p1 = prim;
        bool emitter = false;
        for (int inter = 0; inter < kMaxInteractions; ++inter) {
            if (inter > 0) shape_intersect_ad<N>(sc, p1, r1, n1);
            const DevShape &s = sc.shapes[n1.shape];
            if (s.light_id >= 0) {
                emitter = true;
                break;
            }
            if (inter == max_inter || sc.bsdfs[s.bsdf_id].type != BSDF_NULL) break;
            r1.o = r1.o + r1.d * n1.t;
            p1 = closest_hit(sc, stack, r1.o.val(), r1.d.val(), kShadowEps, INFINITY, th, c);
            if (p1 < 0) break;
        }
        if (!emitter) return DV<N>();
    }
    Df<N> tr(1.f), dist(0.f);
    ItsAD<N> ni = its;
    for (int inter = 0; inter < kMaxInteractions; ++inter) {
        if (inter > 0) shape_intersect_ad<N>(sc, prim, ray, ni);
        const Df<N> tmax = ni.t;
        dist += ni.t;
        if (med >= 0) tr *= medium_transmittance_ad<N>(sc, sc.media[med], ray, tmin, tmax, rng, c, adj);
        const DevShape &s = sc.shapes[ni.shape];
        if (s.light_id >= 0) {
            const float3 dp = ni.p.val() - scatter;
            const float G = ni.wi.z.v / dot(dp, dp);
            pdf_nee = sc.light_pmf[s.light_id] / (sc.light_area[s.light_id] * G);
            if (far_shape) {
                *far_shape = ni.shape;
                *far_t = dist.v;
            }
            return le_ad<N>(sc, ni, -ray.d) * tr;
        }
        if (inter == max_inter || sc.bsdfs[s.bsdf_id].type != BSDF_NULL) return DV<N>();
        if (is_transition(s)) med = dot(ni.ng, ray.d.val()) > 0.f ? s.med_ext : s.med_int;
        ray.o = ray.o + ray.d * tmax;
        tmin = kShadowEps;
        prim = closest_hit(sc, stack, ray.o.val(), ray.d.val(), tmin, INFINITY, th, c);
        if (prim < 0) return DV<N>();
    }
    return DV<N>();
}

// scene.cpp:399-426 (from a point in a medium; wo in world space)
DT_HEAVY float3 nee_point(const DevScene &sc, int *stack, float3 p, const float rnd[4], Rng &rng, int med, int max_inter,
                      float3 &wo, float &pdf, Ctr &c) {
    float3 lp, ln;
    const int l = sample_light(sc, rnd, lp, ln, pdf);
    ++c.lights;
    if (l < 0) return mk(0.f, 0.f, 0.f);
    float3 dir = lp - p;
    if (dot(dir, ln) < 0.f && pdf != 0.f) {
        const float dist = length(dir);
        dir = dir / dist;
        const float tr = eval_transmittance(sc, stack, p, dir, false, med, dist, rng, max_inter, c);
        if (tr != 0.f) {
            pdf *= dist * dist / dot(ln, -dir);
            wo = dir;
            return le_normal(sc.emitters[l], ln, -dir) * (tr / pdf);
        }
    }
    return mk(0.f, 0.f, 0.f);
}

// scene.cpp:456-491 (from a surface; wo in the local shading frame)
DT_HEAVY float3 nee_surface(const DevScene &sc, int *stack, const Its &its, const float rnd[4], Rng &rng, int med,
                        int max_inter, float3 &wo, float &pdf, bool flag, Ctr &c) {
    float3 lp, ln;
    const int l = sample_light(sc, rnd, lp, ln, pdf);
    ++c.lights;
    if (l < 0) return mk(0.f, 0.f, 0.f);
    float3 dir = lp - its.p;
    const bool transmissive = sc.bsdfs[sc.shapes[sc.emitters[l].shape_id].bsdf_id].type == BSDF_NULL ||
                              sc.bsdfs[sc.shapes[sc.emitters[l].shape_id].bsdf_id].type == BSDF_ROUGHDIELECTRIC;
    if ((transmissive || dot(dir, its.fr.n) > 0.f) && dot(dir, ln) < 0.f && pdf != 0.f) {
        const DevShape &s = sc.shapes[its.shape];
        if (is_transition(s)) med = dot(dir, its.ng) > 0.f ? s.med_ext : s.med_int;
        const float dist = length(dir);
        dir = dir / dist;
        wo = its.to_local(dir);
        if (flag && signum(its.wi.z) != signum(wo.z)) --max_inter;
        if (max_inter >= 0) {
            const float tr = eval_transmittance(sc, stack, its.p, dir, true, med, dist, rng, max_inter, c);
            if (tr != 0.f) {
                pdf *= dist * dist / dot(ln, -dir);
                return le_normal(sc.emitters[l], ln, -dir) * (tr / pdf);
            }
        }
    }
    return mk(0.f, 0.f, 0.f);
}

// scene.cpp:428-454 (AD, from a point; the light sample carries no derivative)
template <int N>
DT_HEAVY DV<N> nee_point_ad(const DevScene &sc, int *stack, const DV<N> &p, const float rnd[4], Rng &rng, int med,
                        int max_inter, DV<N> &wo, float &pdf, Ctr &c, const AdjCtx *adj = nullptr) {
    float3 lp, ln;
    float pdf0;
    const int l = sample_light(sc, rnd, lp, ln, pdf0);
    ++c.lights;
    if (l < 0) return DV<N>();
    float3 dir = lp - p.val();
    if (dot(dir, ln) < 0.f) {
        const float dist = length(dir);
        dir = dir / dist;
        ItsAD<N> near_its;
        int far_shape = -1;
        float far_t = 0.f;
        RayAD<N> r{p, DV<N>(dir)};
        DV<N> v = look_for_emitter_ad<N>(sc, stack, r, false, rng, med, max_inter, near_its, pdf, &far_shape, &far_t, c,
                                         adj);
        if (!v.is_zero() && pdf > kEps && far_shape == sc.emitters[l].shape_id && fabsf(far_t - dist) < kShadowEps) {
            wo = DV<N>(dir);
            return v / pdf;
        }
    }
    return DV<N>();
}

// scene.cpp:493-524 (AD, from a surface; wo in the dual shading frame)
template <int N>
// With `bsdf` (a BSDF without derivative slots, whose value the caller multiplies in), a
// light sample where that value is exactly zero returns zero before its visibility chain is
// traced: the contribution is zero either way (a near-specular dielectric is zero for almost
// every light sample). Random numbers such a chain would have drawn are not drawn.
DT_HEAVY DV<N> nee_surface_ad(const DevScene &sc, int *stack, const ItsAD<N> &its, const FrameAD<N> &fr, const float rnd[4],
                          Rng &rng, int med, int max_inter, DV<N> &wo, float &pdf, Ctr &c, const AdjCtx *adj = nullptr,
                          const DevBsdf *bsdf = nullptr) {
    float3 lp, ln;
    float pdf0;
    const int l = sample_light(sc, rnd, lp, ln, pdf0);
    ++c.lights;
    if (l < 0) return DV<N>();
    float3 dir = lp - its.p.val();
    const int lb = sc.bsdfs[sc.shapes[sc.emitters[l].shape_id].bsdf_id].type;
    const bool transmissive = lb == BSDF_NULL || lb == BSDF_ROUGHDIELECTRIC;
    if ((transmissive || dot(dir, its.ns.val()) > 0.f) && dot(dir, ln) < 0.f) {
        const DevShape &s = sc.shapes[its.shape];
        if (is_transition(s)) med = dot(dir, its.ng) > 0.f ? s.med_ext : s.med_int;
        const float dist = length(dir);
        dir = dir / dist;
        if (bsdf && !bsdf->has_der && is_zero3(bsdf_eval(*bsdf, its.wi.val(), fr.plain().to_local(dir)), 0.f))
            return DV<N>();
        ItsAD<N> near_its;
        int far_shape = -1;
        float far_t = 0.f;
        RayAD<N> r{its.p, DV<N>(dir)};
        DV<N> v = look_for_emitter_ad<N>(sc, stack, r, true, rng, med, max_inter, near_its, pdf, &far_shape, &far_t, c,
                                         adj);
        if (!v.is_zero() && pdf > kEps && far_shape == sc.emitters[l].shape_id && fabsf(far_t - dist) < kShadowEps) {
            wo = fr.to_local(dir);
            return v / pdf;
        }
    }
    return DV<N>();
}

// ------------------------------------------------------------------ non-AD path, volpathAD.cpp:50-142
// (the same loop is VolPathTracer::radiance, volpath.cpp:10-103, whose first hit is traced
// from the camera: on_surface = false). State between vertices: li_path keeps it in
// registers, the wavefront Li schedule in HBM.
struct alignas(16) LiState {
    Rng rng;
    Its its;
    float3 o, d, ret, thr;
    int med, depth, max_depth, inc_emission;
};

// First hit of the path; false when the loop would not run at all.
DT_D bool li_start(const DevScene &sc, int *stack, LiState &s, float3 o, float3 d, int max_depth, int med,
                   bool inc_emission, Ctr &c, bool on_surface = true) {
    s.its = Its();
    s.o = o;
    s.d = d;
    s.ret = mk(0.f, 0.f, 0.f);
    s.thr = mk(1.f, 1.f, 1.f);
    s.med = med;
    s.depth = 0;
    s.max_depth = max_depth;
    s.inc_emission = inc_emission ? 1 : 0;
    ray_intersect(sc, stack, o, d, on_surface, s.its, c);
    return s.depth <= s.max_depth;
}

// One vertex (one iteration of the loop at s.depth): false when the path ends.
DT_D bool li_step(const DevScene &sc, int *stack, LiState &s, Ctr &c) {
    Rng &rng = s.rng;
    Its &its = s.its;
    float3 &o = s.o, &d = s.d, &ret = s.ret, &thr = s.thr;
    int &med = s.med;
    const int depth = s.depth, max_depth = s.max_depth;
    const int max_inter = max_depth - depth - 1;
    const float r1a = rng.next1(), r1b = rng.next1();
    float r2[4];
    r2[0] = rng.next1(); r2[1] = rng.next1(); r2[2] = rng.next1(); r2[3] = rng.next1();
    const float r3a = rng.next1(), r3b = rng.next1(), r3c = rng.next1();
    const bool inside = med >= 0 && sample_distance(sc, sc.media[med], o, d, its.t, r1a, r1b, rng, thr, c);
    if (inside) {
        if (depth >= max_depth) return false;
        if (is_zero3(thr)) return false;
        const DevPhase &ph = sc.phases[sc.media[med].phase_id];
        float3 wo;
        float pdf_nee;
        const float3 v = nee_point(sc, stack, o, r2, rng, med, max_inter, wo, pdf_nee, c);
        if (!is_zero3(v)) {
            const float pv = phase_eval(ph, -d, wo);
            if (pv > kEps) ret += cmul(thr, v) * (mis_weight(pdf_nee, pv) * pv);
        }
        const float pv = phase_sample(ph, -d, r3a, r3b, wo);
        if (pv < kEps) return false;
        thr = thr * pv;
        d = wo;
        const float3 att = look_for_emitter(sc, stack, o, d, false, rng, med, max_inter, its, pdf_nee, c);
        if (!is_zero3(att)) ret += cmul(thr, att) * mis_weight(phase_eval(ph, -d, wo), pdf_nee);
        s.inc_emission = 0;
    } else {
        if (!its.valid()) return false;
        const DevShape &sh = sc.shapes[its.shape];
        if (sh.light_id >= 0 && s.inc_emission) ret += cmul(thr, le(sc, its, -d));
        if (depth >= max_depth) return false;
        const DevBsdf &b = sc.bsdfs[sh.bsdf_id];
        float3 wo;
        float pdf_nee;
        if (b.type != BSDF_NULL) {
            const float3 v = nee_surface(sc, stack, its, r2, rng, med, max_inter, wo, pdf_nee, false, c);
            if (!is_zero3(v))
                ret += cmul(cmul(thr, v), bsdf_eval(b, its.wi, wo)) * mis_weight(pdf_nee, bsdf_pdf(b, its.wi, wo));
        }
        float bpdf, beta;
        const float3 bw = bsdf_sample(b, its.wi, r3a, r3b, r3c, wo, bpdf, beta);
        if (is_zero3(bw)) return false;
        wo = its.to_world(wo);
        o = its.p;
        d = wo;
        if (is_transition(sh)) med = dot(wo, its.ng) > 0.f ? sh.med_ext : sh.med_int;
        if (b.type == BSDF_NULL) {
            ray_intersect(sc, stack, o, d, true, its, c);
        } else {
            const float3 att = look_for_emitter(sc, stack, o, d, true, rng, med, max_inter, its, pdf_nee, c);
            thr = cmul(thr, bw);
            if (!is_zero3(att, 1e-12f)) ret += cmul(thr, att) * mis_weight(bpdf, pdf_nee);
            s.inc_emission = 0;
        }
    }
    ++s.depth;
    return s.depth <= max_depth;
}

DT_D float3 li_path(const DevScene &sc, int *stack, Rng &rng, float3 o, float3 d, int max_depth, int med,
                    bool inc_emission, Ctr &c, bool on_surface = true) {
    LiState s;
    s.rng = rng;
    bool alive = li_start(sc, stack, s, o, d, max_depth, med, inc_emission, c, on_surface);
    while (alive) alive = li_step(sc, stack, s, c);
    rng = s.rng;
    return s.ret;
}

}  // namespace dt
