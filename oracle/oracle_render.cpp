// TEST INFRASTRUCTURE — CPU oracle materials, scene queries, integrator and C API.
// FP64 restatement of (uci-rendering/dtrt): src/bsdf.cpp, src/bsdf/{null,diffuse,phong,
// roughdielectric}.cpp, src/bsdf/microfacet.h, include/phase.h, src/emitter/area*.cpp,
// src/scene.cpp:150-793, src/integrator/differential/volpathAD.cpp and integratorAD.cpp.
#include <omp.h>

#include <cstdio>
#include <memory>

#include "dtrt_oracle.h"
#include "oracle_scene.h"

namespace orc {

#define FL(x) ((double)(x##f))  // a float literal of the reference widened to double

// ------------------------------------------------------------------ microfacet.h
template <class S>
static S beckmann_d(const S &alpha, const Vec3<S> &m) {  // microfacet.h:24-51
    if (val(m.z) < kEps) return S(0.0);
    S cos2 = m.z * m.z;
    S expo = (m.x * m.x + m.y * m.y) / (alpha * alpha * cos2);
    S r = d_exp(-expo) / (kPi * alpha * alpha * cos2 * cos2);
    if (val(r) * val(m.z) < 1e-20) r = S(0.0);
    return r;
}
template <class S>
static S smith_g1(const S &alpha, const Vec3<S> &v, const Vec3<S> &m) {  // microfacet.h:118-155
    if (val(dot(v, m)) * val(v.z) < kEps) return S(0.0);
    S tt = d_abs(tan_theta(v));
    if (val(tt) == 0.0) return S(1.0);
    S a = 1.0 / (alpha * tt);
    if (val(a) >= FL(1.6)) return S(1.0);
    S a2 = a * a;
    return (FL(3.535) * a + FL(2.181) * a2) / (1.0 + FL(2.276) * a + FL(2.577) * a2);
}
static void sample_visible11(double theta_i, double u, double v, double &sx, double &sy) {  // microfacet.h:178-244
    const double SQRT_PI_INV = 1.0 / std::sqrt(kPi);
    if (theta_i < FL(1e-4)) {
        double r = std::sqrt(-std::log(1.0 - u));
        double ph = 2.0 * kPi * v;
        sx = r * std::cos(ph);
        sy = r * std::sin(ph);
        return;
    }
    double tan_i = std::tan(theta_i), cot_i = 1.0 / tan_i;
    double a = -1.0, c = approx_erf(cot_i);
    double ux = std::max(u, 1e-6);
    double fit = 1.0 + theta_i * (FL(-0.876) + theta_i * (FL(0.4265) - FL(0.0594) * theta_i));
    double b = c - (1.0 + c) * std::pow(1.0 - ux, fit);
    double normalization = 1.0 / (1.0 + c + SQRT_PI_INV * tan_i * std::exp(-cot_i * cot_i));
    int it = 0;
    while (++it < 10) {
        if (!(b >= a && b <= c)) b = 0.5 * (a + c);
        double ie = approx_erfinv(b);
        double value = normalization * (1.0 + b + SQRT_PI_INV * tan_i * std::exp(-ie * ie)) - ux;
        double deriv = normalization * (1.0 - ie * tan_i);
        if (std::abs(value) < FL(1e-5)) break;
        if (value > 0) c = b;
        else a = b;
        b -= value / deriv;
    }
    sx = approx_erfinv(b);
    sy = approx_erfinv(2.0 * std::max(v, (double)1e-6f) - 1.0);
}
static V3 microfacet_sample(double alpha, const V3 &wi_in, double u, double v) {  // microfacet.h:65-92
    V3 wi = normalized(V3(alpha * wi_in.x, alpha * wi_in.y, wi_in.z));
    double theta = 0, phi = 0;
    if (wi.z < 0.99999) {
        theta = std::acos(wi.z);
        phi = std::atan2(wi.y, wi.x);
    }
    double sp = std::sin(phi), cp = std::cos(phi);
    double sx, sy;
    sample_visible11(theta, u, v, sx, sy);
    double tx = cp * sx - sp * sy, ty = sp * sx + cp * sy;
    tx *= alpha;
    ty *= alpha;
    double nrm = 1.0 / std::sqrt(tx * tx + ty * ty + 1.0);
    return V3(-tx * nrm, -ty * nrm, nrm);
}
static double microfacet_pdf(double alpha, const V3 &wi, const V3 &m) {  // microfacet.h:96-99
    if (std::abs(wi.z) < kEps) return 0.0;
    return smith_g1(alpha, wi, m) * std::abs(dot(wi, m)) * beckmann_d(alpha, m) / std::abs(wi.z);
}

// ------------------------------------------------------------------ BSDF eval (plain and dual)
template <class S>
static Vec3<S> rough_dielectric_eval(const S &alpha, const S &eta_in, const S &inv_eta, const Vec3<S> &wi,
                                     const Vec3<S> &wo) {  // roughdielectric.cpp:9-118 / 121-170
    if (std::abs(val(wi.z)) < kEps || std::abs(val(wo.z)) < kEps) return Vec3<S>();
    bool refl = val(wi.z) * val(wo.z) > 0;
    Vec3<S> H;
    if (refl) {
        H = normalized(wo + wi);
    } else {
        const S &e = val(wi.z) > 0 ? eta_in : inv_eta;
        H = normalized(wi + wo * e);
    }
    H = H * signum(val(H.z));
    S D = beckmann_d(alpha, H);
    if (std::abs(val(D)) < kEps) return Vec3<S>();
    S F = fresnel_dielectric_ext(dot(wi, H), eta_in);
    S G = smith_g1(alpha, wi, H) * smith_g1(alpha, wo, H);
    S r;
    if (refl) {
        r = F * D * G / (4.0 * d_abs(wi.z));
    } else {
        const S &e = val(wi.z) > 0.0 ? eta_in : inv_eta;
        S sd = dot(wi, H) + e * dot(wo, H);
        S value = ((1.0 - F) * D * G * e * e * dot(wi, H) * dot(wo, H)) / (wi.z * sd * sd);
        const S &factor = val(wi.z) > 0 ? inv_eta : eta_in;
        r = d_abs(value * factor * factor);
    }
    return Vec3<S>(r, r, r);
}
template <class S>
static Vec3<S> phong_eval(const Vec3<S> &kd, const Vec3<S> &ks, const S &e, const Vec3<S> &wi,
                          const Vec3<S> &wo) {  // phong.cpp:19-53
    if (val(wi.z) < kEps || val(wo.z) < kEps) return Vec3<S>();
    Vec3<S> result;
    S a = dot(wo, Vec3<S>(-wi.x, -wi.y, wi.z));
    if (val(a) > 0.0) result += ks * ((e + 2.0) * d_pow(a, e) * kInvTwoPi);
    result += kd * kInvPi;
    return result * wo.z;
}

template <int N>
V3 Scene<N>::bsdf_eval(const Its &its, const V3 &wo) const {
    const Bsdf<N> &b = bsdfs[shapes[its.shape].bsdf_id];
    switch (b.type) {
        case DTRT_BSDF_NULL: return V3(1, 1, 1);  // null.cpp:5-7
        case DTRT_BSDF_DIFFUSE:  // diffuse.cpp:7-12
            if (its.wi.z < kEps || wo.z < kEps) return V3();
            return val(b.diffuse) * (kInvPi * wo.z);
        case DTRT_BSDF_PHONG: return phong_eval<double>(val(b.diffuse), val(b.specular), b.exponent.v, its.wi, wo);
        default: return rough_dielectric_eval<double>(b.alpha.v, b.eta.v, b.inv_eta.v, its.wi, wo);
    }
}

template <int N>
DV3<N> Scene<N>::bsdf_eval_ad(const ItsAD<N> &its, const DV3<N> &wo) const {
    const Bsdf<N> &b = bsdfs[shapes[its.shape].bsdf_id];
    switch (b.type) {
        case DTRT_BSDF_NULL: return lift<N>(V3(1, 1, 1));
        case DTRT_BSDF_DIFFUSE:  // diffuse.cpp:15-20
            if (its.wi.z.v < kEps || wo.z.v < kEps) return DV3<N>();
            return b.diffuse * (kInvPi * wo.z);
        case DTRT_BSDF_PHONG: return phong_eval<Dual<N>>(b.diffuse, b.specular, b.exponent, its.wi, wo);
        default: return rough_dielectric_eval<Dual<N>>(b.alpha, b.eta, b.inv_eta, its.wi, wo);
    }
}

template <int N>
double Scene<N>::bsdf_pdf(const Its &its, const V3 &wo) const {
    const Bsdf<N> &b = bsdfs[shapes[its.shape].bsdf_id];
    const V3 &wi = its.wi;
    switch (b.type) {
        case DTRT_BSDF_NULL: return 1.0;
        case DTRT_BSDF_DIFFUSE:  // diffuse.cpp:33-38
            if (wi.z < kEps || wo.z < kEps) return 0.0;
            return cosine_hemisphere_pdf(wo);
        case DTRT_BSDF_PHONG: {  // phong.cpp:82-95
            if (wi.z < kEps || wo.z < kEps) return 0.0;
            double dp = cosine_hemisphere_pdf(wo), sp = 0.0;
            double a = dot(wo, V3(-wi.x, -wi.y, wi.z));
            if (a > 0) sp = std::pow(a, b.exponent.v) * (b.exponent.v + 1.0) / (2.0 * kPi);
            return b.spec_weight * sp + (1.0 - b.spec_weight) * dp;
        }
        default: {  // roughdielectric.cpp:172-206
            bool refl = wi.z * wo.z > 0;
            V3 H;
            double dwh;
            if (refl) {
                H = normalized(wi + wo);
                dwh = 1.0 / (4.0 * dot(wo, H));
            } else {
                double e = wi.z > 0 ? b.eta.v : b.inv_eta.v;
                H = normalized(wi + wo * e);
                double sd = dot(wi, H) + e * dot(wo, H);
                dwh = (e * e * dot(wo, H)) / (sd * sd);
            }
            H = H * signum(H.z);
            double prob = microfacet_pdf(b.alpha.v, wi * signum(wi.z), H);
            double F = fresnel_dielectric_ext(dot(wi, H), b.eta.v);
            prob *= refl ? F : (1.0 - F);
            return std::abs(prob * dwh);
        }
    }
}

template <int N>
V3 Scene<N>::bsdf_sample(const Its &its, const double rnd[3], V3 &wo, double &pdf, double &eta) const {
    const Bsdf<N> &b = bsdfs[shapes[its.shape].bsdf_id];
    const V3 &wi = its.wi;
    switch (b.type) {
        case DTRT_BSDF_NULL:  // null.cpp:13-18
            wo = -wi;
            pdf = 1.0;
            eta = 1.0;
            return V3(1, 1, 1);
        case DTRT_BSDF_DIFFUSE:  // diffuse.cpp:23-30
            if (wi.z < kEps) return V3();
            wo = square_to_cosine_hemisphere(rnd[0], rnd[1]);
            eta = 1.0;
            pdf = cosine_hemisphere_pdf(wo);
            return val(b.diffuse);
        case DTRT_BSDF_PHONG: {  // phong.cpp:56-80
            if (rnd[2] < b.spec_weight) {
                V3 R(-wi.x, -wi.y, wi.z);
                double e = b.exponent.v;
                double sa = std::sqrt(1.0 - std::pow(rnd[1], 2.0 / (e + 1.0)));
                double ca = std::pow(rnd[1], 1.0 / (e + 1.0));
                double ph = 2.0 * kPi * rnd[0];
                wo = Frame(R).to_world(V3(sa * std::cos(ph), sa * std::sin(ph), ca));
                if (wo.z < kEps) return V3();
            } else {
                wo = square_to_cosine_hemisphere(rnd[0], rnd[1]);
            }
            eta = 1.0;
            pdf = bsdf_pdf(its, wo);
            if (pdf < kEps) return V3();
            return bsdf_eval(its, wo) / pdf;
        }
        default: {  // roughdielectric.cpp:120-170
            double mpdf;
            V3 wis = wi * signum(wi.z);
            V3 m = microfacet_sample(b.alpha.v, wis, rnd[0], rnd[1]);
            mpdf = microfacet_pdf(b.alpha.v, wis, m);
            if (mpdf < kEps) return V3();
            pdf = mpdf;
            double cos_t;
            double F = fresnel_dielectric_ext(dot(wi, m), cos_t, b.eta.v);
            double weight = 1.0;
            bool sref = !(rnd[2] > F);
            pdf *= sref ? F : (1.0 - F);
            double dwh;
            if (sref) {
                wo = reflect(wi, m);
                eta = 1.0;
                if (wi.z * wo.z < kEps) return V3();
                dwh = 1.0 / (4.0 * dot(wo, m));
            } else {
                if (std::abs(cos_t) < kEps) return V3();
                wo = refract(wi, m, b.eta.v, cos_t);
                eta = cos_t < 0 ? b.eta.v : b.inv_eta.v;
                if (wi.z * wo.z >= 0) return V3();
                double factor = cos_t < 0 ? b.inv_eta.v : b.eta.v;
                weight *= factor * factor;
                double sd = dot(wi, m) + eta * dot(wo, m);
                dwh = (eta * eta * dot(wo, m)) / (sd * sd);
            }
            weight *= smith_g1(b.alpha.v, wo, m);
            pdf *= std::abs(dwh);
            return V3(weight, weight, weight);
        }
    }
}

template <int N>
DV3<N> Scene<N>::bsdf_sample_ad(const ItsAD<N> &its, const double rnd[3], DV3<N> &wo, double &pdf,
                                double &eta) const {
    const Bsdf<N> &b = bsdfs[shapes[its.shape].bsdf_id];
    if (b.type == DTRT_BSDF_NULL) {  // null.cpp:20-25
        wo = -its.wi;
        pdf = 1.0;
        eta = 1.0;
        return lift<N>(V3(1, 1, 1));
    }
    // bsdf.cpp:11-21: sample in the plain frame, re-evaluate with duals
    Its its0 = its.plain();
    V3 wo0;
    DV3<N> ret;
    if (!is_zero(bsdf_sample(its0, rnd, wo0, pdf, eta), kEps))
        if (pdf > kEps) {
            wo = its.to_local(lift<N>(its0.to_world(wo0)));
            ret = bsdf_eval_ad(its, wo) / pdf;
        }
    return ret;
}

// ------------------------------------------------------------------ phase.h
template <int N>
double Scene<N>::phase_eval(int ph, const V3 &wi, const V3 &wo) const {
    const Phase<N> &p = phases[ph];
    if (p.type == DTRT_PHASE_ISOTROPIC) return kInvFourPi;
    double g = p.g.v, tmp = 1.0 + g * g + 2.0 * g * dot(wi, wo);
    return kInvFourPi * (1.0 - g * g) / (tmp * std::sqrt(tmp));
}
template <int N>
Dual<N> Scene<N>::phase_eval_ad(int ph, const DV3<N> &wi, const DV3<N> &wo) const {
    const Phase<N> &p = phases[ph];
    if (p.type == DTRT_PHASE_ISOTROPIC) return Dual<N>(kInvFourPi);
    Dual<N> tmp = 1.0 + p.g * p.g + 2.0 * p.g * dot(wi, wo);
    return kInvFourPi * (1.0 - p.g * p.g) / d_pow(tmp, 1.5);
}
template <int N>
double Scene<N>::phase_sample(int ph, const V3 &wi, double u, double v, V3 &wo) const {
    const Phase<N> &p = phases[ph];
    if (p.type == DTRT_PHASE_ISOTROPIC) {  // phase.h:72-75
        wo = square_to_uniform_sphere(u, v);
        return 1.0;
    }
    // phase.h:40-51: the local frame is built around wi itself (not -wi), as in the reference
    double g = p.g.v, ct;
    if (std::abs(g) < kEps) {
        ct = 1.0 - 2.0 * u;
    } else {
        double sq = (1.0 - g * g) / (1.0 - g + 2.0 * g * u);
        ct = (1.0 + g * g - sq * sq) / (2.0 * g);
    }
    double st = std::sqrt(1.0 - ct * ct);
    double sp = std::sin(2.0 * kPi * v), cp = std::cos(2.0 * kPi * v);
    wo = Frame(wi).to_world(V3(st * cp, st * sp, ct));
    return 1.0;
}
template <int N>
Dual<N> Scene<N>::phase_sample_ad(int ph, const DV3<N> &wi, double u, double v, DV3<N> &wo) const {
    V3 w;
    phase_sample(ph, val(wi), u, v, w);
    wo = lift<N>(w);
    const Phase<N> &p = phases[ph];
    if (p.type == DTRT_PHASE_ISOTROPIC) return Dual<N>(1.0);  // phase.h:14-19 with evalAD = pdf = 1/4pi
    Dual<N> tmp = phase_eval_ad(ph, wi, wo);                   // phase.h:53-58
    return tmp.v > kEps ? tmp / tmp.v : Dual<N>(0.0);
}

// ------------------------------------------------------------------ emitters
template <int N>
V3 Scene<N>::le(const Its &its, const V3 &w) const {
    const Emitter<N> &e = emitters[shapes[its.shape].light_id];
    if (e.type == DTRT_EMITTER_AREA) return (e.two_sided || dot(its.geo.n, w) > 0) ? e.intensity_val() : V3();
    double t = dot(its.sh.n, w);  // area2.cpp:5-11
    if (t > kEps) return e.intensity_val() * (e.kappa.v * kInvTwoPi * std::exp(e.kappa.v * (t - 1.0)));
    return V3();
}
template <int N>
DV3<N> Scene<N>::le_ad(const ItsAD<N> &its, const DV3<N> &w) const {
    const Emitter<N> &e = emitters[shapes[its.shape].light_id];
    if (e.type == DTRT_EMITTER_AREA)
        return (e.two_sided || dot(val(its.geo.n), val(w)) > 0) ? lift<N>(e.intensity_val()) : DV3<N>();
    Dual<N> t = dot(its.sh.n, w);  // area2.cpp:13-18
    if (t.v > kEps) return e.intensity * (d_exp(e.kappa * (t - 1.0)) * e.kappa * kInvTwoPi);
    return DV3<N>();
}
// emitter eval with an explicit normal (NEE), area.cpp:13-15, area2.cpp:21-27
template <int N>
static V3 le_normal(const Emitter<N> &e, const V3 &n, const V3 &w) {
    if (e.type == DTRT_EMITTER_AREA) return (e.two_sided || dot(n, w) > 0) ? e.intensity_val() : V3();
    double t = dot(n, w);
    if (t > kEps) return e.intensity_val() * (e.kappa.v * kInvTwoPi * std::exp(e.kappa.v * (t - 1.0)));
    return V3();
}

// ------------------------------------------------------------------ scene queries
template <int N>
int Scene<N>::sample_light(const double rnd[4], V3 &pos, V3 &n, double &pdf) const {
    int nl = (int)emitters.size();
    int l = (int)(std::upper_bound(light_cdf.begin(), light_cdf.end(), rnd[0]) - light_cdf.begin());
    l = std::min(std::max(l, 0), nl - 1);
    const Shape<N> &s = shapes[emitters[l].shape_id];
    auto b = area_cdf_pool.begin() + area_cdf_begin[l];
    int t = (int)(std::upper_bound(b, b + s.nt, rnd[1]) - b);
    t = std::min(std::max(t, 0), s.nt - 1);
    s.sample_position(t, rnd[2], rnd[3], pos, n);
    pdf = light_pmf[l] / light_areas[l];
    return l;
}

template <int N>
double Scene<N>::eval_transmittance(const Ray &ray_in, bool on_surface, int med, double remaining, Rng &rng,
                                    int max_interactions) const {  // scene.cpp:177-237
    Ray ray = ray_in;
    double tmin = on_surface ? kShadowEps : 0.0;
    double tfar = (1.0 - kShadowEps) * remaining;
    double tr = 1.0;
    int inter = 0;
    while (remaining > 0) {
        double tmax = remaining;
        int s = -1, p = -1;
        double th;
        bool hit = trace(ray.o, ray.d, tmin, tfar, s, p, th);
        Its its;
        if (hit) {
            if (inter == max_interactions || !bsdfs[shapes[s].bsdf_id].is_null()) return 0.0;
            shape_intersect(s, p, ray, its);
            if (its.t < tmax) tmax = its.t;
        }
        if (med >= 0) tr *= medium_transmittance(med, ray, tmin, tmax, rng);
        if (!hit) break;
        if (shapes[s].is_medium_transition()) med = dot(its.geo.n, ray.d) > 0.0 ? shapes[s].med_ext : shapes[s].med_int;
        ray.o = ray.at(tmax);
        tmin = kShadowEps;
        remaining -= tmax;
        tfar = (1.0 - kShadowEps) * remaining;
        inter++;
    }
    return tr;
}

template <int N>
V3 Scene<N>::sample_attenuated_emitter_direct(const V3 &ps, const double rnd[4], Rng &rng, int med,
                                              int max_interactions, V3 &wo, double &pdf) const {  // scene.cpp:399-426
    V3 lp, ln;
    int l = sample_light(rnd, lp, ln, pdf);
    V3 dir = lp - ps;
    if (dot(dir, ln) < 0 && pdf != 0) {
        double dist = norm(dir);
        dir = dir / dist;
        double tr = eval_transmittance(Ray{ps, dir}, false, med, dist, rng, max_interactions);
        if (tr != 0) {
            pdf *= dist * dist / dot(ln, -dir);
            wo = dir;
            return le_normal(emitters[l], ln, -dir) * (tr / pdf);
        }
    }
    return V3();
}

template <int N>
V3 Scene<N>::sample_attenuated_emitter_direct(const Its &its, const double rnd[4], Rng &rng, int med,
                                              int max_interactions, V3 &wo, double &pdf,
                                              bool flag) const {  // scene.cpp:456-491
    V3 lp, ln;
    int l = sample_light(rnd, lp, ln, pdf);
    V3 dir = lp - its.p;
    bool transmissive = bsdfs[shapes[emitters[l].shape_id].bsdf_id].is_transmissive();
    if ((transmissive || dot(dir, its.sh.n) > 0) && dot(dir, ln) < 0 && pdf != 0) {
        if (shapes[its.shape].is_medium_transition()) med = target_medium(its, dir);
        double dist = norm(dir);
        dir = dir / dist;
        wo = its.to_local(dir);
        if (flag && signum(its.wi.z) != signum(wo.z)) --max_interactions;
        if (max_interactions >= 0) {
            double tr = eval_transmittance(Ray{its.p, dir}, true, med, dist, rng, max_interactions);
            if (tr != 0) {
                pdf *= dist * dist / dot(ln, -dir);
                return le_normal(emitters[l], ln, -dir) * (tr / pdf);
            }
        }
    }
    return V3();
}

template <int N>
DV3<N> Scene<N>::sample_attenuated_emitter_direct_ad(const DV3<N> &ps, const double rnd[4], Rng &rng, int med,
                                                     int max_interactions, DV3<N> &wo,
                                                     double &pdf) const {  // scene.cpp:428-454
    V3 lp, ln;
    double pdf0;
    int l = sample_light(rnd, lp, ln, pdf0);
    V3 dir = lp - val(ps);
    if (dot(dir, ln) < 0) {
        double dist = norm(dir);
        dir = dir / dist;
        ItsAD<N> near_its, far_its;
        DV3<N> r = ray_intersect_and_look_for_emitter_ad(RayAD<N>{ps, lift<N>(dir)}, false, rng, med, max_interactions,
                                                         near_its, pdf, &far_its);
        if (!is_zero(r, kEps) && pdf > kEps && far_its.shape == emitters[l].shape_id &&
            std::abs(far_its.t.v - dist) < kShadowEps) {
            wo = lift<N>(dir);
            return r / pdf;
        }
    }
    return DV3<N>();
}

template <int N>
DV3<N> Scene<N>::sample_attenuated_emitter_direct_ad(const ItsAD<N> &its, const double rnd[4], Rng &rng, int med,
                                                     int max_interactions, DV3<N> &wo,
                                                     double &pdf) const {  // scene.cpp:493-524
    V3 lp, ln;
    double pdf0;
    int l = sample_light(rnd, lp, ln, pdf0);
    V3 dir = lp - val(its.p);
    bool transmissive = bsdfs[shapes[emitters[l].shape_id].bsdf_id].is_transmissive();
    if ((transmissive || dot(dir, val(its.sh.n)) > 0) && dot(dir, ln) < 0) {
        if (shapes[its.shape].is_medium_transition())
            med = dot(dir, val(its.geo.n)) > 0 ? shapes[its.shape].med_ext : shapes[its.shape].med_int;
        double dist = norm(dir);
        dir = dir / dist;
        ItsAD<N> near_its, far_its;
        DV3<N> r = ray_intersect_and_look_for_emitter_ad(RayAD<N>{its.p, lift<N>(dir)}, true, rng, med,
                                                         max_interactions, near_its, pdf, &far_its);
        if (!is_zero(r, kEps) && pdf > kEps && far_its.shape == emitters[l].shape_id &&
            std::abs(far_its.t.v - dist) < kShadowEps) {
            wo = its.to_local(lift<N>(dir));
            return r / pdf;
        }
    }
    return DV3<N>();
}

template <int N>
V3 Scene<N>::ray_intersect_and_look_for_emitter(const Ray &ray_in, bool on_surface, Rng &rng, int med,
                                                int max_interactions, Its &its,
                                                double &pdf_nee) const {  // scene.cpp:617-701
    Ray ray = ray_in;
    double tmin = on_surface ? kShadowEps : 0.0;
    int inter = 0;
    V3 scatter_pos = ray.o;
    int s, p;
    double th;
    if (!trace(ray.o, ray.d, tmin, INFINITY, s, p, th)) {
        its.shape = -1;
        its.t = INFINITY;
        return V3();
    }
    shape_intersect(s, p, ray, its);
    double tr = 1.0;
    while (true) {
        Its ni;
        shape_intersect(s, p, ray, ni);
        double tmax = ni.t;
        if (med >= 0) tr *= medium_transmittance(med, ray, tmin, tmax, rng);
        const Shape<N> &sh = shapes[s];
        if (sh.is_emitter()) {
            double d2 = sq_norm(ni.p - scatter_pos);
            double G = ni.wi.z / d2;
            pdf_nee = light_pmf[sh.light_id] / (light_areas[sh.light_id] * G);
            return le(ni, -ray.d) * tr;
        }
        if (inter == max_interactions || !bsdfs[sh.bsdf_id].is_null()) return V3();
        if (sh.is_medium_transition()) med = dot(ni.geo.n, ray.d) > 0.0 ? sh.med_ext : sh.med_int;
        ray.o = ray.o + ray.d * tmax;
        tmin = kShadowEps;
        inter++;
        if (!trace(ray.o, ray.d, tmin, INFINITY, s, p, th)) return V3();
    }
}

template <int N>
DV3<N> Scene<N>::ray_intersect_and_look_for_emitter_ad(const RayAD<N> &ray_in, bool on_surface, Rng &rng, int med,
                                                       int max_interactions, ItsAD<N> &its, double &pdf_nee,
                                                       ItsAD<N> *its_far) const {  // scene.cpp:703-793
    RayAD<N> ray = ray_in;
    double tmin = on_surface ? kShadowEps : 0.0;
    int inter = 0;
    V3 scatter_pos = val(ray.o);
    int s, p;
    double th;
    if (!trace(val(ray.o), val(ray.d), tmin, INFINITY, s, p, th)) {
        its.shape = -1;
        its.t = Dual<N>(INFINITY);
        return DV3<N>();
    }
    shape_intersect_ad(s, p, ray, its);
    Dual<N> tr(1.0), dist(0.0);
    while (true) {
        ItsAD<N> ni;
        shape_intersect_ad(s, p, ray, ni);
        Dual<N> tmax = ni.t;
        dist += ni.t;
        if (med >= 0) tr *= medium_transmittance_ad(med, ray, Dual<N>(tmin), tmax, rng);
        const Shape<N> &sh = shapes[s];
        if (sh.is_emitter()) {
            double d2 = sq_norm(val(ni.p) - scatter_pos);
            double G = ni.wi.z.v / d2;
            pdf_nee = light_pmf[sh.light_id] / (light_areas[sh.light_id] * G);
            if (its_far) {
                *its_far = ni;
                its_far->t = dist;
            }
            return le_ad(ni, -ray.d) * tr;
        }
        if (inter == max_interactions || !bsdfs[sh.bsdf_id].is_null()) return DV3<N>();
        if (sh.is_medium_transition()) med = dot(val(ni.geo.n), val(ray.d)) > 0.0 ? sh.med_ext : sh.med_int;
        ray.o = ray.o + ray.d * tmax;
        tmin = kShadowEps;
        inter++;
        if (!trace(val(ray.o), val(ray.d), tmin, INFINITY, s, p, th)) return DV3<N>();
    }
}

// ------------------------------------------------------------------ integrator
static inline double mis(double a, double b) {  // volpathAD.cpp:43-47 power heuristic
    a *= a;
    b *= b;
    return a / (a + b);
}

template <int N>
struct Integrator {
    const Scene<N> &sc;
    int sppse;
    double ddist;
    explicit Integrator(const Scene<N> &s, int se, double dd) : sc(s), sppse(se), ddist(dd) {}

    // volpathAD.cpp:50-142
    // (also VolPathTracer::radiance, volpath.cpp:10-103, with on_surface = false)
    V3 li(Rng &rng, const Ray &ray_in, int max_depth, int init_med, bool inc_emission = true,
          bool on_surface = true) const {
        Ray ray = ray_in;
        int med = init_med;
        Its its;
        V3 ret, thr(1, 1, 1);
        sc.ray_intersect(ray, on_surface, its);
        for (int depth = 0; depth <= max_depth; ++depth) {
            int max_inter = max_depth - depth - 1;
            double r1[2] = {rng.next1(), rng.next1()};
            double r2[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
            double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
            bool inside = med >= 0 && sc.sample_distance(med, ray, its.t, r1, rng, thr);
            if (inside) {
                if (depth >= max_depth) break;
                if (is_zero(thr, kEps)) break;
                int ph = sc.media[med].phase_id;
                V3 wo;
                double pdf_nee;
                V3 v = sc.sample_attenuated_emitter_direct(ray.o, r2, rng, med, max_inter, wo, pdf_nee);
                if (!is_zero(v, kEps)) {
                    double pv = sc.phase_eval(ph, -ray.d, wo);
                    if (pv > kEps) ret += cmul(thr, v) * (mis(pdf_nee, sc.phase_eval(ph, -ray.d, wo)) * pv);
                }
                double pv = sc.phase_sample(ph, -ray.d, r3[0], r3[1], wo);
                if (pv < kEps) break;
                thr = thr * pv;
                ray.d = wo;
                V3 att = sc.ray_intersect_and_look_for_emitter(ray, false, rng, med, max_inter, its, pdf_nee);
                if (!is_zero(att, kEps)) {
                    double pp = sc.phase_eval(ph, -ray.d, wo);
                    ret += cmul(thr, att) * mis(pp, pdf_nee);
                }
                inc_emission = false;
            } else {
                if (!its.valid()) break;
                const Shape<N> &sh = sc.shapes[its.shape];
                if (sh.is_emitter() && inc_emission) ret += cmul(thr, sc.le(its, -ray.d));
                if (depth >= max_depth) break;
                V3 wo;
                double pdf_nee;
                bool is_null = sc.bsdfs[sh.bsdf_id].is_null();
                if (!is_null) {
                    V3 v = sc.sample_attenuated_emitter_direct(its, r2, rng, med, max_inter, wo, pdf_nee);
                    if (!is_zero(v, kEps)) {
                        V3 bv = sc.bsdf_eval(its, wo);
                        double bp = sc.bsdf_pdf(its, wo);
                        ret += cmul(cmul(thr, v), bv) * mis(pdf_nee, bp);
                    }
                }
                double bpdf, beta;
                V3 bw = sc.bsdf_sample(its, r3, wo, bpdf, beta);
                if (is_zero(bw, kEps)) break;
                wo = its.to_world(wo);
                ray = Ray{its.p, wo};
                if (sh.is_medium_transition()) med = sc.target_medium(its, wo);
                if (is_null) {
                    sc.ray_intersect(ray, true, its);
                    continue;
                }
                V3 att = sc.ray_intersect_and_look_for_emitter(ray, true, rng, med, max_inter, its, pdf_nee);
                thr = cmul(thr, bw);
                if (!is_zero(att, 1e-12)) ret += cmul(thr, att) * mis(bpdf, pdf_nee);
                inc_emission = false;
            }
        }
        return ret;
    }

    // edge-point construction shared by the volume and interface edge terms,
    // volpathAD.cpp:231-280 and 540-589 (ALTERNATIVE_EDGE_SAMPLING branch)
    bool edge_direction(const Shape<N> &shape, const Edge &e, const DV3<N> &x0, double t, double &edge_pdf,
                        DV3<N> &w1, double &dist, V3 &nrm) const {
        DV3<N> e0 = shape.verts[e.v0] - x0, e1 = shape.verts[e.v1] - x0;
        nrm = normalized(cross(val(e0), val(e1)));
        V3 ne0 = normalized(val(e0)), ne1 = normalized(val(e1));
        double theta = std::acos(dot(ne0, ne1)), st = std::sin(theta);
        if (theta < kEps || theta > kPi - kEps) return false;
        double w0 = std::sin(theta * (1.0 - t)) / st, wb = std::sin(theta * t) / st;
        w0 /= norm(val(e0));
        wb /= norm(val(e1));
        double tmp = w0 + wb;
        w0 /= tmp;
        wb /= tmp;
        if (w0 < -kEps || wb < -kEps || std::abs(w0 + wb - 1.0) > kEps) return false;
        w1 = e0 * w0 + e1 * wb;
        Dual<N> dad = norm(w1);
        w1 = w1 / dad;
        dist = dad.v;
        edge_pdf /= theta;
        V3 wv = val(w1);
        double mx = 0;
        for (int j = 0; j < N; ++j) mx = std::max(mx, std::abs(dot(grad(w1, j), wv)));
        if (mx > kEps) return false;
        return true;
    }

    // volpathAD.cpp:145-620
    DV3<N> li_ad(const ItsAD<N> &its, Rng &rng, const RayAD<N> &ray_in, int med, int max_depth, int mode) const {
        if (mode == 0) return DV3<N>();
        RayAD<N> ray = ray_in;
        double r1[2] = {rng.next1(), rng.next1()};
        double r2[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
        double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
        DV3<N> ret, thr = lift<N>(V3(1, 1, 1));
        ItsAD<N> its1;
        if (med >= 0 && sc.sample_distance_ad(med, ray, its.t, r1, rng, thr)) {
            // ---- volumetric
            if (max_depth == 0 || is_zero(thr, kEps)) return ret;
            int ph = sc.media[med].phase_id;
            double pdf_nee;
            DV3<N> wo;
            if (mode & DTRT_MODE_VOLUME_MAIN) {
                DV3<N> v = sc.sample_attenuated_emitter_direct_ad(ray.o, r2, rng, med, max_depth - 1, wo, pdf_nee);
                if (!is_zero(v, kEps)) {
                    Dual<N> pv = sc.phase_eval_ad(ph, -ray.d, wo);
                    if (pv.v > kEps) {
                        double pp = sc.phase_eval(ph, -val(ray.d), val(wo));
                        ret += cmul(thr, v) * (pv * mis(pdf_nee, pp));
                    }
                }
            }
            Dual<N> pv = sc.phase_sample_ad(ph, -ray.d, r3[0], r3[1], wo);
            if (pv.v > kEps) {
                DV3<N> thr1 = thr * pv;
                ray.d = wo;
                DV3<N> att = sc.ray_intersect_and_look_for_emitter_ad(ray, false, rng, med, max_depth - 1, its1, pdf_nee);
                if (!is_zero(att, kEps) && (mode & DTRT_MODE_VOLUME_MAIN)) {
                    double pp = sc.phase_eval(ph, -val(ray.d), val(wo));
                    ret += cmul(thr1, att) * mis(pp, pdf_nee);
                }
                ret += cmul(thr1, li_ad(its1, rng, ray, med, max_depth - 1, mode & ~DTRT_MODE_EMISSION));
            }
            if (sppse > 0 && (mode & DTRT_MODE_VOLUME_BOUNDARY2) && sc.edges_distrb.size() > 0) {
                std::vector<V3> der(N);
                const DV3<N> &x1 = ray.o;
                V3 x1v = val(x1);
                for (int i = 0; i < sppse; ++i) {
                    double rnd = (i + rng.next1()) / sppse;
                    int sid;
                    double epdf;
                    const Edge *e = sc.sample_edge(x1v, rnd, sid, epdf);
                    double t = rnd;
                    const Shape<N> &shape = sc.shapes[sid];
                    int sil = shape.is_silhouette(*e, x1v);
                    if (!(sil > 0 && !sc.bsdfs[shape.bsdf_id].is_null())) continue;
                    DV3<N> w1;
                    double dist;
                    V3 nrm;
                    if (!edge_direction(shape, *e, x1, t, epdf, w1, dist, nrm)) continue;
                    if (der_is_zero(w1, kEps)) continue;
                    V3 pval = val(thr) * sc.phase_eval(ph, -val(ray_in.d), val(w1));
                    if (is_zero(pval, kEps)) continue;
                    double tr = sc.eval_transmittance(Ray{x1v, val(w1)}, false, med, dist, rng, max_depth - 1);
                    if (!(tr > kEps)) continue;
                    V3 w2 = normalized(val(w1) - nrm * kAngleEps);
                    V3 delta = li(rng, Ray{x1v, w2}, max_depth - 1, med);
                    w2 = normalized(val(w1) + nrm * kAngleEps);
                    delta -= li(rng, Ray{x1v, w2}, max_depth - 1, med);
                    if (is_zero(delta, kEps)) continue;
                    for (int j = 0; j < N; ++j) der[j] += cmul(pval, delta) * (dot(nrm, grad(w1, j)) / epdf);
                }
                for (int j = 0; j < N; ++j) {
                    ret.x.d[j] += der[j].x / sppse;
                    ret.y.d[j] += der[j].y / sppse;
                    ret.z.d[j] += der[j].z / sppse;
                }
            }
            return ret;
        }
        // ---- interfacial
        if (!its.valid() || is_zero(thr, kEps)) return ret;
        const Shape<N> &sh = sc.shapes[its.shape];
        Its its0 = its.plain();
        if (sh.is_medium_transition() && sc.target_medium(its0, -val(ray.d)) != med) return ret;
        if (sh.is_emitter() && (mode & DTRT_MODE_EMISSION)) ret += cmul(thr, sc.le_ad(its, -ray.d));
        if (max_depth == 0) return ret;
        bool is_null = sc.bsdfs[sh.bsdf_id].is_null();
        // Lins boundary term, volpathAD.cpp:321-467 (ALTERNATIVE_LINS_BOUNDARY_SAMPLING)
        if (med >= 0 && !its.t.der_is_zero(kEps) && (mode & DTRT_MODE_VOLUME_BOUNDARY1)) {
            double dmax = its.t.der_max_abs();
            V3 n = its0.geo.n;
            if (dot(n, val(ray.d)) < 0.0) n = -n;
            V3 sig = sc.sig_s(med, its0.p - n * kShadowEps);
            int ph = sc.media[med].phase_id;
            int ns = std::min(std::max((int)(ddist * dmax), 1), 100);
            V3 lins;
            V3 rd = val(ray.d);
            for (int i = 0; i < ns; ++i) lins += lins_sample(its0, n, rd, ph, med, max_depth, rng);
            lins = lins / (double)ns;
            V3 w = cmul(cmul(sig, lins), val(thr));
            for (int j = 0; j < N; ++j) {
                ret.x.d[j] += its.t.d[j] * w.x;
                ret.y.d[j] += its.t.d[j] * w.y;
                ret.z.d[j] += its.t.d[j] * w.z;
            }
        }
        // area sampling, volpathAD.cpp:469-511
        {
            DV3<N> wo;
            double pdf_nee;
            if (!is_null && (mode & DTRT_MODE_SURFACE_MAIN)) {
                DV3<N> v = sc.sample_attenuated_emitter_direct_ad(its, r2, rng, med, max_depth - 1, wo, pdf_nee);
                if (!is_zero(v, kEps)) {
                    DV3<N> bv = sc.bsdf_eval_ad(its, wo);
                    double bp = sc.bsdf_pdf(its0, val(wo));
                    ret += cmul(cmul(thr, v), bv) * mis(pdf_nee, bp);
                }
            }
            double bpdf, beta;
            DV3<N> bw = sc.bsdf_sample_ad(its, r3, wo, bpdf, beta);
            if (!is_zero(bw, kEps)) {
                wo = its.to_world(wo);
                if (!is_null) wo = zero_grad(wo);  // asserted zero at volpathAD.cpp:489
                ray = RayAD<N>{its.p, wo};
                int med1 = sh.is_medium_transition() ? sc.target_medium(its0, val(wo)) : med;
                DV3<N> thr1 = thr;
                int mode1;
                if (is_null) {
                    sc.ray_intersect_ad(ray, true, its1);
                    mode1 = mode;
                } else {
                    DV3<N> att = sc.ray_intersect_and_look_for_emitter_ad(ray, true, rng, med1, max_depth - 1, its1, pdf_nee);
                    thr1 = cmul(thr1, bw);
                    if (!is_zero(att, kEps) && (mode & DTRT_MODE_SURFACE_MAIN)) ret += cmul(thr1, att) * mis(bpdf, pdf_nee);
                    mode1 = mode & ~DTRT_MODE_EMISSION;
                }
                ret += cmul(thr1, li_ad(its1, rng, ray, med1, max_depth - 1, mode1));
            }
        }
        // interface edge term, volpathAD.cpp:513-616
        if (!is_null && sppse > 0 && (mode & DTRT_MODE_SURFACE_BOUNDARY) && sc.edges_distrb.size() > 0) {
            std::vector<V3> der(N);
            const DV3<N> &x0 = its.p;
            V3 x0v = val(x0);
            for (int i = 0; i < sppse; ++i) {
                double rnd = (i + rng.next1()) / sppse;
                int sid;
                double epdf;
                const Edge *e = sc.sample_edge(x0v, rnd, sid, epdf);
                double t = rnd;
                const Shape<N> &shape = sc.shapes[sid];
                int sil = shape.is_silhouette(*e, x0v);
                if (!(sil > 0 && !sc.bsdfs[shape.bsdf_id].is_null())) continue;
                DV3<N> w1;
                double dist;
                V3 nrm;
                if (!edge_direction(shape, *e, x0, t, epdf, w1, dist, nrm)) continue;
                if (der_is_zero(w1, kEps)) continue;
                V3 bval = cmul(val(thr), sc.bsdf_eval(its0, its0.to_local(val(w1))));
                if (is_zero(bval, kEps)) continue;
                int med1 = sh.is_medium_transition() ? sc.target_medium(its0, val(w1)) : med;
                double tr = sc.eval_transmittance(Ray{x0v, val(w1)}, true, med1, dist, rng, max_depth - 1);
                if (!(tr > kEps)) continue;
                V3 w2 = normalized(val(w1) - nrm * kAngleEps);
                V3 delta = li(rng, Ray{x0v, w2}, max_depth - 1, med1);
                w2 = normalized(val(w1) + nrm * kAngleEps);
                delta -= li(rng, Ray{x0v, w2}, max_depth - 1, med1);
                if (is_zero(delta, kEps)) continue;
                for (int j = 0; j < N; ++j) der[j] += cmul(bval, delta) * (dot(nrm, grad(w1, j)) / epdf);
            }
            for (int j = 0; j < N; ++j) {
                ret.x.d[j] += der[j].x / sppse;
                ret.y.d[j] += der[j].y / sppse;
                ret.z.d[j] += der[j].z / sppse;
            }
        }
        return ret;
    }

    // ================================================================ surface integrators
    // PathTracerAD (pathAD.cpp:10-213) and DirectIntegratorAD (directAD.cpp:7-150): surface
    // scenes only. Their own random-number order, MIS heuristics, occlusion test and edge
    // parametrisations are restated; media are not traced (the reference ignores them).

    // Scene::isVisible, scene.cpp:150-175
    bool is_visible(const V3 &p, bool p_on_surface, const V3 &q, bool q_on_surface) const {
        V3 dir = q - p;
        double dist = norm(dir);
        dir = dir / dist;
        int s, pr;
        double th;
        return !sc.trace(p, dir, p_on_surface ? kShadowEps : 0.0, q_on_surface ? (1.0 - kShadowEps) * dist : dist, s,
                         pr, th);
    }

    // Scene::pdfEmitterSample, scene.cpp:526-536, divided by the geometry term at the hit
    double emitter_hit_pdf(int shape, double dist_sq, double cos_wi) const {
        int l = sc.shapes[shape].light_id;
        return sc.light_pmf[l] / sc.light_areas[l] / (cos_wi / dist_sq);
    }

    // AreaLight::eval / AreaLightEx::evalAD with an explicit normal (area.cpp:13-15, area2.cpp:13-27)
    DV3<N> emitter_eval_ad(const Emitter<N> &e, const DV3<N> &n, const DV3<N> &w) const {
        if (e.type == DTRT_EMITTER_AREA)
            return (e.two_sided || dot(val(n), val(w)) > 0) ? lift<N>(e.intensity_val()) : DV3<N>();
        Dual<N> t = dot(n, w);
        if (t.v > kEps) return e.intensity * (d_exp(e.kappa * (t - 1.0)) * e.kappa * kInvTwoPi);
        return DV3<N>();
    }

    // Scene::sampleEmitterDirect, scene.cpp:302-345: one occlusion test from the shading
    // point (no null-interface pass-through); the segment counts only when the sampled
    // light's own triangle closes it within ShadowEpsilon.
    V3 sample_emitter_direct(const Its &its, const double rnd[4], V3 &wo, double &pdf) const {
        V3 lp, ln;
        int l = sc.sample_light(rnd, lp, ln, pdf);
        V3 dir = lp - its.p;
        if (dot(dir, its.sh.n) > 0 && dot(dir, ln) < 0 && pdf != 0) {
            double dist = norm(dir);
            dir = dir / dist;
            int s, pr;
            double th;
            if (sc.trace(its.p, dir, kShadowEps, INFINITY, s, pr, th) && s == sc.emitters[l].shape_id) {
                Its ni;
                sc.shape_intersect(s, pr, Ray{its.p, dir}, ni);
                if (std::abs(ni.t - dist) < kShadowEps) {
                    pdf *= dist * dist / dot(ln, -dir);
                    wo = its.to_local(dir);
                    return le_normal(sc.emitters[l], ni.sh.n, -dir) / pdf;
                }
            }
        }
        return V3();
    }

    // Scene::sampleEmitterDirectAD, scene.cpp:347-392
    DV3<N> sample_emitter_direct_ad(const ItsAD<N> &its, const double rnd[4], DV3<N> &wo, double &pdf) const {
        V3 lp, ln;
        int l = sc.sample_light(rnd, lp, ln, pdf);
        V3 dir = lp - val(its.p);
        if (dot(dir, val(its.sh.n)) > 0 && dot(dir, ln) < 0 && pdf != 0) {
            double dist = norm(dir);
            dir = dir / dist;
            int s, pr;
            double th;
            if (sc.trace(val(its.p), dir, kShadowEps, INFINITY, s, pr, th) && s == sc.emitters[l].shape_id) {
                ItsAD<N> ni;
                sc.shape_intersect_ad(s, pr, RayAD<N>{its.p, lift<N>(dir)}, ni);
                if (std::abs(ni.t.v - dist) < kShadowEps) {
                    pdf *= dist * dist / dot(ln, -dir);
                    wo = its.to_local(lift<N>(dir));
                    return emitter_eval_ad(sc.emitters[l], ni.sh.n, lift<N>(-dir)) / pdf;
                }
            }
        }
        return DV3<N>();
    }

    // PathTracerAD::Li, pathAD.cpp:10-58 (the non-AD sub-path of its edge term and of the
    // primary edges)
    V3 path_li(Rng &rng, const Ray &ray_in, int max_depth) const {
        Ray ray = ray_in;
        Its its;
        V3 ret;
        sc.ray_intersect(ray, true, its);
        if (!its.valid()) return ret;
        V3 thr(1, 1, 1);
        int depth = 0;
        while (depth <= max_depth && its.valid()) {
            const Shape<N> &sh = sc.shapes[its.shape];
            if (sh.is_emitter() && depth == 0) ret += cmul(thr, sc.le(its, -ray.d));
            if (depth >= max_depth) break;
            double r4[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
            double pdf_nee;
            V3 wo;
            V3 value = sample_emitter_direct(its, r4, wo, pdf_nee);
            if (!is_zero(value, 1e-12)) {
                V3 bv = sc.bsdf_eval(its, wo);
                double bp = sc.bsdf_pdf(its, wo);
                ret += cmul(cmul(thr, value), bv) * mis(pdf_nee, bp);
            }
            double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
            double bpdf, beta;
            V3 bw = sc.bsdf_sample(its, r3, wo, bpdf, beta);
            if (is_zero(bw, 1e-12)) break;
            wo = its.to_world(wo);
            ray = Ray{its.p, wo};
            if (!sc.ray_intersect(ray, true, its)) break;
            thr = cmul(thr, bw);
            if (sc.shapes[its.shape].is_emitter()) {
                V3 lc = sc.le(its, -ray.d);
                if (!is_zero(lc, 1e-12)) {
                    double pn = emitter_hit_pdf(its.shape, sq_norm(its.p - ray.o), its.wi.z);
                    ret += cmul(thr, lc) * mis(bpdf, pn);
                }
            }
            depth++;
        }
        return ret;
    }

    // PathTracerAD::LiAD, pathAD.cpp:61-213 (ALTERNATIVE_EDGE_SAMPLING)
    DV3<N> path_li_ad(const ItsAD<N> &its, Rng &rng, const RayAD<N> &ray_in, int max_depth, int mode,
                      bool inc_emission) const {
        if (mode == 0) return DV3<N>();
        DV3<N> ret;
        if (!its.valid()) return ret;
        const Shape<N> &sh = sc.shapes[its.shape];
        if (sh.is_emitter() && (mode & DTRT_MODE_EMISSION) && inc_emission) ret += sc.le_ad(its, -ray_in.d);
        if (max_depth == 0) return ret;
        Its its0 = its.plain();
        DV3<N> wo;
        double pdf_nee;
        if (mode & DTRT_MODE_SURFACE_MAIN) {
            double r4[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
            DV3<N> value = sample_emitter_direct_ad(its, r4, wo, pdf_nee);
            if (!is_zero(value, kEps)) {
                DV3<N> bv = sc.bsdf_eval_ad(its, wo);
                double bp = sc.bsdf_pdf(its0, val(wo));
                ret += cmul(value, bv) * mis(pdf_nee, bp);
            }
        }
        double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
        double bpdf, beta;
        DV3<N> value = sc.bsdf_sample_ad(its, r3, wo, bpdf, beta);
        if (!is_zero(value, kEps)) {
            wo = zero_grad(its.to_world(wo));  // asserted derivative-free at pathAD.cpp:97
            RayAD<N> ray{its.p, wo};
            ItsAD<N> its1;
            if (sc.ray_intersect_ad(ray, true, its1)) {
                if (sc.shapes[its1.shape].is_emitter() && (mode & DTRT_MODE_SURFACE_MAIN)) {
                    DV3<N> lc = sc.le_ad(its1, -ray.d);
                    if (!is_zero(val(lc), 1e-12)) {
                        double pn = emitter_hit_pdf(its1.shape, sq_norm(val(its1.p) - val(ray.o)), its1.wi.z.v);
                        ret += cmul(value, lc) * mis(bpdf, pn);
                    }
                }
                ret += cmul(value, path_li_ad(its1, rng, ray, max_depth - 1, mode, false));
            }
        }
        if (sppse > 0 && (mode & DTRT_MODE_SURFACE_BOUNDARY) && sc.edges_distrb.size() > 0) {
            std::vector<V3> der(N);
            V3 x1v = val(its.p);
            for (int i = 0; i < sppse; ++i) {
                double rnd = rng.next1();
                int sid;
                double epdf;
                const Edge *e = sc.sample_edge(x1v, rnd, sid, epdf);
                if (!e) continue;
                double t = rnd;
                const Shape<N> &shape = sc.shapes[sid];
                if (!shape.is_silhouette(*e, x1v)) continue;
                DV3<N> w1;
                double dist;
                V3 nrm;
                if (!edge_direction(shape, *e, its.p, t, epdf, w1, dist, nrm)) continue;
                if (der_is_zero(w1, kEps)) continue;
                V3 bval = sc.bsdf_eval(its0, its0.to_local(val(w1)));
                if (is_zero(bval, kEps)) continue;
                if (!is_visible(x1v, true, x1v + val(w1) * dist, true)) continue;
                V3 w2 = normalized(val(w1) - nrm * kAngleEps);
                V3 delta = path_li(rng, Ray{x1v, w2}, max_depth - 1);
                w2 = normalized(val(w1) + nrm * kAngleEps);
                delta -= path_li(rng, Ray{x1v, w2}, max_depth - 1);
                if (is_zero(delta, kEps)) continue;
                for (int j = 0; j < N; ++j) der[j] += cmul(bval, delta) * (dot(nrm, grad(w1, j)) / epdf);
            }
            for (int j = 0; j < N; ++j) {
                ret.x.d[j] += der[j].x / sppse;
                ret.y.d[j] += der[j].y / sppse;
                ret.z.d[j] += der[j].z / sppse;
            }
        }
        return ret;
    }

    // DirectIntegratorAD::radiance, directAD.cpp:110-140 (power heuristic)
    V3 direct(Rng &rng, const Ray &ray_in) const {
        Ray ray = ray_in;
        Its its;
        V3 ret;
        sc.ray_intersect(ray, true, its);
        if (!its.valid()) return ret;
        if (sc.shapes[its.shape].is_emitter()) ret += sc.le(its, -ray.d);
        double r4[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
        double pdf_nee;
        V3 wo;
        V3 value = sample_emitter_direct(its, r4, wo, pdf_nee);
        if (!is_zero(value, 1e-12)) {
            V3 bv = sc.bsdf_eval(its, wo);
            double bp = sc.bsdf_pdf(its, wo);
            ret += cmul(value, bv) * mis(pdf_nee, bp);
        }
        double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
        double bpdf, beta;
        V3 bw = sc.bsdf_sample(its, r3, wo, bpdf, beta);
        if (!is_zero(bw, 1e-12)) {
            wo = its.to_world(wo);
            ray = Ray{its.p, wo};
            if (sc.ray_intersect(ray, true, its) && sc.shapes[its.shape].is_emitter()) {
                V3 lc = sc.le(its, -ray.d);
                if (!is_zero(lc, 1e-12)) {
                    double pn = emitter_hit_pdf(its.shape, sq_norm(its.p - ray.o), its.wi.z);
                    ret += cmul(bw, lc) * mis(bpdf, pn);
                }
            }
        }
        return ret;
    }

    // DirectIntegratorAD::radianceAD, directAD.cpp:7-107: balance-heuristic MIS, and the
    // edge term of the first hit with the linear edge parametrisation (sinTheta / dist
    // Jacobian) and emitter-only delta functions
    DV3<N> direct_ad(Rng &rng, const RayAD<N> &ray_in) const {
        RayAD<N> ray = ray_in;
        ItsAD<N> its;
        DV3<N> ret;
        sc.ray_intersect_ad(ray, true, its);
        if (!its.valid()) return ret;
        if (sc.shapes[its.shape].is_emitter()) ret += sc.le_ad(its, -ray.d);
        Its its0 = its.plain();
        {
            double r4[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
            double pdf_nee;
            DV3<N> wo;
            DV3<N> value = sample_emitter_direct_ad(its, r4, wo, pdf_nee);
            if (!is_zero(value, kEps)) {
                DV3<N> bv = sc.bsdf_eval_ad(its, wo);
                double bp = sc.bsdf_pdf(its0, val(wo));
                ret += cmul(value, bv) * (pdf_nee / (pdf_nee + bp));
            }
            double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
            double bpdf, beta;
            value = sc.bsdf_sample_ad(its, r3, wo, bpdf, beta);
            if (!is_zero(value, kEps)) {
                wo = zero_grad(its.to_world(wo));  // asserted derivative-free at directAD.cpp:38
                RayAD<N> r1{its.p, wo};
                ItsAD<N> its1;
                if (sc.ray_intersect_ad(r1, true, its1) && sc.shapes[its1.shape].is_emitter()) {
                    DV3<N> lc = sc.le_ad(its1, -r1.d);
                    if (!is_zero(val(lc), 1e-12)) {
                        double pn = emitter_hit_pdf(its1.shape, sq_norm(val(its1.p) - val(r1.o)), its1.wi.z.v);
                        ret += cmul(value, lc) * (bpdf / (pn + bpdf));
                    }
                }
            }
        }
        if (sppse > 0 && sc.edges_distrb.size() > 0) {
            std::vector<V3> der(N);
            const DV3<N> &x1 = its.p;
            V3 x1v = val(x1);
            for (int i = 0; i < sppse; ++i) {
                // Scene::sampleEdge(p, frame, rnd, shape_id, t, pdf), scene.h:103-108
                double t = rng.next1();
                int sid;
                double epdf;
                const Edge *e = sc.sample_edge(x1v, t, sid, epdf);
                if (!e) continue;
                epdf /= e->length;
                const Shape<N> &shape = sc.shapes[sid];
                if (!shape.is_silhouette(*e, x1v)) continue;
                const DV3<N> &v0 = shape.verts[e->v0], &v1 = shape.verts[e->v1];
                DV3<N> y1 = v0 * (1.0 - t) + v1 * t, w1 = y1 - x1;
                V3 tang = normalized(val(v1) - val(v0));
                V3 nrm = normalized(cross(val(v0) - x1v, val(v1) - x1v));
                Dual<N> dist = norm(w1);
                w1 = w1 / dist;
                double mx = 0;
                for (int j = 0; j < N; ++j) mx = std::max(mx, std::abs(dot(grad(w1, j), val(w1))));
                if (mx >= kEps) continue;  // asserted below Epsilon at directAD.cpp:75
                V3 bval = sc.bsdf_eval(its0, its0.to_local(val(w1)));
                if (is_zero(bval, kEps) || !is_visible(x1v, true, val(y1), true)) continue;
                V3 delta;
                Its its1;
                V3 w2 = normalized(val(w1) - nrm * kAngleEps);
                if (sc.ray_intersect(Ray{x1v, w2}, true, its1) && sc.shapes[its1.shape].is_emitter())
                    delta += sc.le(its1, -val(w1));
                w2 = normalized(val(w1) + nrm * kAngleEps);
                if (sc.ray_intersect(Ray{x1v, w2}, true, its1) && sc.shapes[its1.shape].is_emitter())
                    delta -= sc.le(its1, -val(w1));
                if (is_zero(delta, kEps)) continue;
                double cos_t = -dot(val(w1), tang), sin_t = std::sqrt(1.0 - cos_t * cos_t);
                for (int j = 0; j < N; ++j)
                    der[j] += cmul(bval, delta) * (dot(nrm, grad(w1, j)) * sin_t / (epdf * dist.v));
            }
            for (int j = 0; j < N; ++j) {
                ret.x.d[j] += der[j].x / sppse;
                ret.y.d[j] += der[j].y / sppse;
                ret.z.d[j] += der[j].z / sppse;
            }
        }
        return ret;
    }

    // one Lins sample, volpathAD.cpp:337-441
    V3 lins_sample(const Its &its0, const V3 &n, const V3 &rd, int ph, int med, int max_depth, Rng &rng) const {
        V3 lins, wo, att;
        double pdf_nee, pp, pv;
        Its its1;
        const Shape<N> &sh = sc.shapes[its0.shape];
        if (sc.bsdfs[sh.bsdf_id].is_null()) {
            double r4[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
            att = sc.sample_attenuated_emitter_direct(its0, r4, rng, med, max_depth - 1, wo, pdf_nee, true);
            if (!is_zero(att, kEps)) {
                wo = its0.to_world(wo);
                pv = sc.phase_eval(ph, -rd, wo);
                if (pv > kEps) {
                    pp = sc.phase_eval(ph, -rd, wo);
                    lins += att * (pv * mis(pdf_nee, pp));
                }
            }
            double u = rng.next1(), v = rng.next1();
            if ((pv = sc.phase_sample(ph, -rd, u, v, wo)) > kEps) {
                int md1 = max_depth - 1;
                if (dot(wo, n) > kEps) {
                    if (sh.is_emitter()) lins += sc.le(its0, -wo) * pv;
                    --md1;
                }
                if (md1 > 0) {
                    int med1 = sh.is_medium_transition() ? sc.target_medium(its0, wo) : med;
                    Ray r1{its0.p, wo};
                    att = sc.ray_intersect_and_look_for_emitter(r1, true, rng, med1, md1, its1, pdf_nee);
                    if (!is_zero(att, kEps)) {
                        pp = sc.phase_eval(ph, -rd, wo);
                        lins += att * (pv * mis(pp, pdf_nee));
                    }
                    lins += li(rng, r1, md1, med1, false) * pv;
                }
            }
            return lins;
        }
        double r4[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
        att = sc.sample_attenuated_emitter_direct(its0, r4, rng, med, max_depth - 1, wo, pdf_nee);
        if (!is_zero(att, kEps)) {
            wo = its0.to_world(wo);
            if (dot(wo, n) < -kEps) {
                pv = sc.phase_eval(ph, -rd, wo);
                if (pv > kEps) {
                    pp = sc.phase_eval(ph, -rd, wo);
                    lins += att * (pv * mis(pdf_nee, pp));
                }
            }
        }
        double u = rng.next1(), v = rng.next1();
        if ((pv = sc.phase_sample(ph, -rd, u, v, wo)) > kEps) {
            double wdn = dot(wo, n);
            if (wdn < -kEps) {
                Ray r1{its0.p, wo};
                att = sc.ray_intersect_and_look_for_emitter(r1, true, rng, med, max_depth - 1, its1, pdf_nee);
                if (!is_zero(att, kEps)) {
                    pp = sc.phase_eval(ph, -rd, wo);
                    lins += att * (pv * mis(pp, pdf_nee));
                }
                lins += li(rng, r1, max_depth - 1, med, false) * pv;
            } else if (wdn > kEps) {
                if (sh.is_emitter()) lins += sc.le(its0, -wo) * pv;
                if (max_depth > 1) {
                    its1 = its0;
                    its1.wi = its1.to_local(-wo);
                    double r4b[4] = {rng.next1(), rng.next1(), rng.next1(), rng.next1()};
                    att = sc.sample_attenuated_emitter_direct(its1, r4b, rng, med, max_depth - 2, wo, pdf_nee);
                    if (!is_zero(att, kEps)) {
                        V3 bv = sc.bsdf_eval(its1, wo);
                        double bp = sc.bsdf_pdf(its1, wo);
                        lins += cmul(bv, att) * (pv * mis(pdf_nee, bp));
                    }
                    double r3[3] = {rng.next1(), rng.next1(), rng.next1()};
                    double bp, eta;
                    V3 bv = sc.bsdf_sample(its1, r3, wo, bp, eta);
                    if (!is_zero(bv, kEps)) {
                        V3 t1 = bv * pv;
                        wo = its1.to_world(wo);
                        int med1 = sh.is_medium_transition() ? sc.target_medium(its1, wo) : med;
                        Ray r1{its1.p, wo};
                        Its its2;
                        att = sc.ray_intersect_and_look_for_emitter(r1, true, rng, med1, max_depth - 2, its2, pdf_nee);
                        if (!is_zero(att, 1e-12)) lins += cmul(t1, att) * mis(bp, pdf_nee);
                        lins += cmul(t1, li(rng, r1, max_depth - 2, med1, false));
                    }
                }
            }
        }
        return lins;
    }

};

}  // namespace orc

// ====================================================================== render + C API
namespace {

thread_local std::string g_err;

template <int N>
int render_impl(const dtrt_scene_desc &d, const dtrt_render_options &o, float *out, int nthreads, bool pass1,
                bool pass2, unsigned est_flags = 0, const float *const *density_dirs = nullptr,
                int integrator = ORACLE_VOLPATH_AD) {
    using namespace orc;
    auto sc = std::make_unique<Scene<N>>();
    std::string err = sc->build(d);
    if (!err.empty()) {
        g_err = err;
        return 1;
    }
    if (integrator != ORACLE_VOLPATH_AD) {  // the surface integrators trace no media
        if (!sc->media.empty() || sc->cam.med_id >= 0) {
            g_err = "PathTracerAD / DirectAD oracle: surface scenes only (no media)";
            return 1;
        }
        for (const auto &b : sc->bsdfs)
            if (b.is_null()) {
                g_err = "PathTracerAD / DirectAD oracle: null BSDFs block light in the reference's occlusion test";
                return 1;
            }
    }
    sc->est_flags = est_flags;
    for (int mi = 0; density_dirs && mi < d.num_media; ++mi) {
        Grid<N> &g = sc->media[mi].density;
        if (!density_dirs[mi]) continue;
        if (sc->media[mi].type != DTRT_MEDIUM_HETEROGENEOUS) {
            g_err = "density directions given for a homogeneous medium";
            return 1;
        }
        const size_t n = (size_t)g.res[0] * g.res[1] * g.res[2];
        g.dgrid.assign(n * N, 0.f);  // [nder][voxel] -> [voxel][nder]
        for (int j = 0; j < N; ++j)
            for (size_t v = 0; v < n; ++v) g.dgrid[v * N + j] = density_dirs[mi][(size_t)j * n + v];
    }
    Integrator<N> in(*sc, o.sppse, o.ddist_coeff);
    const Camera<N> &cam = sc->cam;
    const bool cropped = cam.cropped();
    const int npix = cropped ? cam.crop_w * cam.crop_h : cam.width * cam.height;
    const int width = cropped ? cam.crop_w : cam.width;
    if (nthreads <= 0) nthreads = omp_get_num_procs();
    const int mode = o.mode >= 0 ? o.mode : DTRT_MODE_ALL;
    // pass 1, integratorAD.cpp:31-98
    if (pass1 && o.spp > 0) {
        const int nblock = (npix + 3) / 4;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
        for (int b = 0; b < nblock; ++b) {
            for (int pix = b * 4; pix < std::min((b + 1) * 4, npix); ++pix) {
                int ix = cropped ? cam.crop_x + pix % width : pix % width;
                int iy = cropped ? cam.crop_y + pix / width : pix / width;
                Rng rng(o.seed, (uint64_t)pix);
                DV3<N> acc;
                for (int s = 0; s < o.spp; ++s) {
                    double jx = 0.5, jy = 0.5;
                    if (o.sppe >= 0) {
                        jx = rng.next1();
                        jy = rng.next1();
                    }
                    // pixelColorAD, volpathAD.cpp:632-642 / pathAD.cpp:222-228 / directAD.cpp:153-156
                    RayAD<N> ray = cam.sample_primary_ray_ad(ix + jx, iy + jy);
                    ItsAD<N> its;
                    if (integrator == ORACLE_DIRECT_AD) {
                        acc += in.direct_ad(rng, ray);
                    } else if (sc->ray_intersect_ad(ray, false, its)) {
                        acc += integrator == ORACLE_PATH_AD ? in.path_li_ad(its, rng, ray, o.max_bounces, mode, true)
                                                            : in.li_ad(its, rng, ray, cam.med_id, o.max_bounces, mode);
                    }
                }
                acc = acc / (double)o.spp;
                V3 v = val(acc);
                if (min_coeff(v) >= 0.0) {
                    out[pix * 3 + 0] = (float)v.x;
                    out[pix * 3 + 1] = (float)v.y;
                    out[pix * 3 + 2] = (float)v.z;
                }
                for (int j = 0; j < N; ++j) {
                    V3 g = grad(acc, j);
                    if (std::isfinite(g.x) && std::isfinite(g.y) && std::isfinite(g.z)) {
                        size_t off = ((size_t)(j + 1) * npix + pix) * 3;
                        out[off] = (float)g.x;
                        out[off + 1] = (float)g.y;
                        out[off + 2] = (float)g.z;
                    }
                }
            }
        }
    }
    // pass 2, integratorAD.cpp:100-165. The reference keeps one sampler per OpenMP
    // worker under dynamic scheduling (not reproducible); here each 128-sample block
    // owns RndSampler(seed, npix + block) so the oracle is deterministic.
    if (pass2 && o.sppe > 0 && sc->primary_edges.size() > 0) {
        const double pdfsum = sc->primary_distrb.sum;
        const int nblock = (int)std::ceil(pdfsum * o.sppe / 128.0);
        const long nsamp = (long)nblock * 128;
        std::vector<std::vector<double>> contrib(nthreads, std::vector<double>((size_t)npix * N * 3, 0.0));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
        for (int b = 0; b < nblock; ++b) {
            std::vector<double> &ec = contrib[omp_get_thread_num()];
            Rng rng(o.seed, (uint64_t)npix + (uint64_t)b);
            for (int k = 0; k < 128; ++k) {
                int px, py;
                Dual<N> p[2];
                double nrm[2];
                double maxd = sc->sample_primary_edge(rng.next1(), px, py, p, nrm);
                bool moving = !(p[0].der_is_zero(kEps) && p[1].der_is_zero(kEps));
                if (!moving) continue;
                Ray ray = cam.sample_primary_ray(px, py, p[0].v, p[1].v);
                double tr = sc->eval_transmittance(ray, false, cam.med_id, maxd, rng, o.max_bounces - 1);
                if (!(tr > kEps)) continue;
                const double delta = (double)1e-4f;
                double x1 = px + p[0].v - nrm[0] * delta, y1 = py + p[1].v - nrm[1] * delta;
                // pixelColor of the integrator (volpathAD.cpp:622-629, pathAD.cpp:216-219, directAD.cpp:147-150)
                auto pixel_color = [&](const Ray &r) {
                    if (integrator == ORACLE_PATH_AD) return in.path_li(rng, r, o.max_bounces);
                    if (integrator == ORACLE_DIRECT_AD) return in.direct(rng, r);
                    return in.li(rng, r, o.max_bounces, cam.med_id);
                };
                V3 dv = pixel_color(cam.sample_primary_ray(x1, y1));
                x1 = px + p[0].v + nrm[0] * delta;
                y1 = py + p[1].v + nrm[1] * delta;
                dv -= pixel_color(cam.sample_primary_ray(x1, y1));
                int lx = cropped ? px - cam.crop_x : px, ly = cropped ? py - cam.crop_y : py;
                int lw = cropped ? cam.crop_w : cam.width, lh = cropped ? cam.crop_h : cam.height;
                if (lx < 0 || ly < 0 || lx >= lw || ly >= lh) continue;  // edge point on the far image border
                int pix = lx + lw * ly;
                for (int j = 0; j < N; ++j) {
                    double s = (nrm[0] * p[0].d[j] + nrm[1] * p[1].d[j]) * pdfsum;
                    size_t off = ((size_t)j * npix + pix) * 3;
                    ec[off] += dv.x * s;
                    ec[off + 1] += dv.y * s;
                    ec[off + 2] += dv.z * s;
                }
            }
        }
        for (size_t i = 0; i < (size_t)npix * N * 3; ++i) {
            double s = 0;
            for (int t = 0; t < nthreads; ++t) s += contrib[t][i];
            out[(size_t)npix * 3 + i] += (float)(s / (double)nsamp);
        }
    }
    return 0;
}

// VolPathTracer::render (volpath.cpp:105-140): per pixel RndSampler(seed, pixel), spp
// jittered primary rays, radiance() averaged and written unconditionally
template <int N>
int render_primal_impl(const dtrt_scene_desc &d, const dtrt_render_options &o, float *out, int nthreads) {
    using namespace orc;
    auto sc = std::make_unique<Scene<N>>();
    std::string err = sc->build(d);
    if (!err.empty()) {
        g_err = err;
        return 1;
    }
    Integrator<N> in(*sc, 0, 0.0);
    const Camera<N> &cam = sc->cam;
    const bool cropped = cam.cropped();
    const int npix = cropped ? cam.crop_w * cam.crop_h : cam.width * cam.height;
    const int width = cropped ? cam.crop_w : cam.width;
    if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
    for (int pix = 0; pix < npix; ++pix) {
        int ix = cropped ? cam.crop_x + pix % width : pix % width;
        int iy = cropped ? cam.crop_y + pix / width : pix / width;
        Rng rng(o.seed, (uint64_t)pix);
        V3 acc;
        for (int s = 0; s < o.spp; ++s) {
            double jx = rng.next1(), jy = rng.next1();
            acc += in.li(rng, cam.sample_primary_ray(ix + jx, iy + jy), o.max_bounces, cam.med_id, true, false);
        }
        if (o.spp > 0) acc = acc / (double)o.spp;
        out[pix * 3 + 0] = (float)acc.x;
        out[pix * 3 + 1] = (float)acc.y;
        out[pix * 3 + 2] = (float)acc.z;
    }
    return 0;
}

template <class F>
int dispatch(int nder, F &&f) {
    switch (nder) {
        case 1: return f(std::integral_constant<int, 1>());
        case 3: return f(std::integral_constant<int, 3>());
        case 4: return f(std::integral_constant<int, 4>());
        case 8: return f(std::integral_constant<int, 8>());
        default: g_err = "unsupported nder (1, 3, 4 or 8)"; return 4;
    }
}

}  // namespace

extern "C" {

int oracle_render(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads) {
    if (!desc || !opts || !out) { g_err = "null argument"; return 1; }
    return dispatch(desc->nder, [&](auto n) { return render_impl<decltype(n)::value>(*desc, *opts, out, nthreads, true, true); });
}

int oracle_render_ext(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads,
                      unsigned est_flags, const float *const *density_dirs) {
    if (!desc || !opts || !out) { g_err = "null argument"; return 1; }
    return dispatch(desc->nder, [&](auto n) {
        return render_impl<decltype(n)::value>(*desc, *opts, out, nthreads, true, true, est_flags, density_dirs);
    });
}

int oracle_render_integrator(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads,
                             int integrator) {
    if (!desc || !opts || !out) { g_err = "null argument"; return 1; }
    if (integrator < ORACLE_VOLPATH_AD || integrator > ORACLE_DIRECT_AD) { g_err = "unknown integrator"; return 1; }
    return dispatch(desc->nder, [&](auto n) {
        return render_impl<decltype(n)::value>(*desc, *opts, out, nthreads, true, true, 0, nullptr, integrator);
    });
}

int oracle_render_primal(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads) {
    if (!desc || !opts || !out) { g_err = "null argument"; return 1; }
    return dispatch(desc->nder, [&](auto n) { return render_primal_impl<decltype(n)::value>(*desc, *opts, out, nthreads); });
}

int oracle_render_primary_edges(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads) {
    if (!desc || !opts || !out) { g_err = "null argument"; return 1; }
    // out is [nder][H][W][3]; render_impl writes slots 1..nder of a (nder+1)-slot image
    int npix = desc->camera.crop_width > 0 ? desc->camera.crop_width * desc->camera.crop_height
                                          : desc->camera.width * desc->camera.height;
    std::vector<float> tmp((size_t)(desc->nder + 1) * npix * 3, 0.0f);
    int r = dispatch(desc->nder, [&](auto n) { return render_impl<decltype(n)::value>(*desc, *opts, tmp.data(), nthreads, false, true); });
    if (r) return r;
    for (size_t i = 0; i < (size_t)desc->nder * npix * 3; ++i) out[i] += tmp[(size_t)npix * 3 + i];
    return 0;
}

void oracle_pcg32(uint64_t seed, uint64_t idx, int n, uint32_t *out) {
    orc::Rng r(seed, idx);
    for (int i = 0; i < n; ++i) out[i] = r.next_u32();
}

void oracle_next1d(uint64_t seed, uint64_t idx, int n, double *out) {
    orc::Rng r(seed, idx);
    for (int i = 0; i < n; ++i) out[i] = r.next1();
}

int oracle_trace_closest(const dtrt_scene_desc *desc, const double *rays, int n, int *hits, double *t) {
    return dispatch(desc->nder, [&](auto nn) {
        constexpr int N = decltype(nn)::value;
        auto sc = std::make_unique<orc::Scene<N>>();
        std::string err = sc->build(*desc);
        if (!err.empty()) { g_err = err; return 1; }
        int tri_base = 0;
        std::vector<int> base(sc->shapes.size());
        for (size_t s = 0; s < sc->shapes.size(); ++s) { base[s] = tri_base; tri_base += sc->shapes[s].nt; }
        for (int i = 0; i < n; ++i) {
            const double *r = rays + 8 * i;
            int s, p;
            double th;
            if (sc->trace(orc::V3(r[0], r[1], r[2]), orc::V3(r[4], r[5], r[6]), r[3], r[7], s, p, th)) {
                hits[2 * i] = base[s] + p;
                hits[2 * i + 1] = s;
                t[i] = th;
            } else {
                hits[2 * i] = -1;
                hits[2 * i + 1] = -1;
                t[i] = INFINITY;
            }
        }
        return 0;
    });
}

int oracle_edge_summary(const dtrt_scene_desc *desc, int *num_edges, double *total_length, int *num_primary,
                        double *primary_pdf_sum) {
    return dispatch(desc->nder, [&](auto nn) {
        constexpr int N = decltype(nn)::value;
        auto sc = std::make_unique<orc::Scene<N>>();
        std::string err = sc->build(*desc);
        if (!err.empty()) { g_err = err; return 1; }
        int ne = 0;
        double tl = 0;
        for (auto &s : sc->shapes) { ne += (int)s.edges.size(); tl += s.edge_distrb.sum; }
        *num_edges = ne;
        *total_length = tl;
        *num_primary = (int)sc->primary_edges.size();
        *primary_pdf_sum = sc->primary_distrb.sum;
        return 0;
    });
}

double oracle_closed_form(int which, double a, double b) {
    using namespace orc;
    switch (which) {
        case 0: return fresnel_dielectric_ext<double>(a, b);
        case 1: {
            double g = a, tmp = 1.0 + g * g + 2.0 * g * b;
            return kInvFourPi * (1.0 - g * g) / (tmp * std::sqrt(tmp));
        }
        case 2: {
            double st = std::sqrt(std::max(0.0, 1 - b * b));
            return beckmann_d<double>(a, V3(st, 0, b));
        }
        case 3: {
            double st = std::sqrt(std::max(0.0, 1 - b * b));
            return smith_g1<double>(a, V3(st, 0, b), V3(0, 0, 1));
        }
        case 4: return approx_erf(a);
        case 5: return approx_erfinv(a);
    }
    return NAN;
}

int oracle_bsdf_albedo(const dtrt_bsdf_desc *bsdf, double cos_i, int nsamples, uint64_t seed, double *out3) {
    using namespace orc;
    // one-triangle scene carrying the BSDF; the sampling weight averages to the albedo
    Scene<1> sc;
    sc.bsdfs.resize(1);
    Bsdf<1> &o = sc.bsdfs[0];
    o.type = bsdf->type;
    o.diffuse = lift<1>(V3(bsdf->diffuse[0], bsdf->diffuse[1], bsdf->diffuse[2]));
    o.specular = lift<1>(V3(bsdf->specular[0], bsdf->specular[1], bsdf->specular[2]));
    o.exponent = Dual<1>(bsdf->exponent);
    if (o.type == DTRT_BSDF_PHONG) {
        double v0 = (bsdf->diffuse[0] + bsdf->diffuse[1] + bsdf->diffuse[2]) / 3.0;
        double v1 = (bsdf->specular[0] + bsdf->specular[1] + bsdf->specular[2]) / 3.0;
        o.spec_weight = v1 / (v0 + v1);
    }
    o.alpha = Dual<1>(std::max((double)bsdf->alpha, (double)1e-4f));
    o.eta = Dual<1>((double)(bsdf->int_ior / bsdf->ext_ior));
    o.inv_eta = 1.0 / o.eta;
    sc.shapes.resize(1);
    sc.shapes[0].bsdf_id = 0;
    Its its;
    its.shape = 0;
    its.wi = V3(std::sqrt(std::max(0.0, 1 - cos_i * cos_i)), 0, cos_i);
    Rng rng(seed, 0);
    V3 acc;
    for (int i = 0; i < nsamples; ++i) {
        double r[3] = {rng.next1(), rng.next1(), rng.next1()};
        V3 wo;
        double pdf, eta;
        acc += sc.bsdf_sample(its, r, wo, pdf, eta);
    }
    for (int c = 0; c < 3; ++c) out3[c] = acc[c] / nsamples;
    return 0;
}

const char *oracle_last_error(void) { return g_err.c_str(); }

}  // extern "C"
