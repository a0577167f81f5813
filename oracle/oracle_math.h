// TEST INFRASTRUCTURE — the CPU oracle of dtrt_gb300. Only tests/, the smoke check
// and bench.py's CPU-baseline leg may build, load or run anything under oracle/.
//
// FP64 restatement of the reference's math layer (uci-rendering/dtrt):
//   include/fwd.h (Float = double, Epsilon = 1e-7), include/config.h (ShadowEpsilon,
//   AngleEpsilon), include/simpleAD.h (forward-mode dual numbers), include/frame.h,
//   include/frameAD.h, src/utils.cpp, src/sampler.cpp, include/pmf.h, include/aabb.h.
// Eigen and the reference's headers are not used; every type here is written anew.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

// include/fwd.h:10-18 (DOUBLE_PRECISION branch), include/config.h:5-7
constexpr double kEps = 1e-7;
constexpr double kPi = 3.14159265358979323846;
constexpr double kInvPi = 0.31830988618379067154;
constexpr double kInvTwoPi = 0.15915494309189534561;
constexpr double kInvFourPi = 0.07957747154594766788;
constexpr double kShadowEps = (double)1e-3f;  // config.h:6 (float literal widened)
constexpr double kAngleEps = (double)1e-4f;   // config.h:7

// ---------------------------------------------------------------- scalar dual
// include/simpleAD.h:20-245: value + nder-wide derivative, the usual chain rules.
template <int N>
struct Dual {
    double v;
    double d[N];
    Dual() : v(0) { for (int i = 0; i < N; ++i) d[i] = 0; }
    Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0; }
    static Dual make(double x, const double *der) {
        Dual r(x);
        for (int i = 0; i < N; ++i) r.d[i] = der[i];
        return r;
    }
    bool der_is_zero(double eps) const {
        for (int i = 0; i < N; ++i) if (std::abs(d[i]) > eps) return false;
        return true;
    }
    double der_max_abs() const {
        double m = 0;
        for (int i = 0; i < N; ++i) m = std::max(m, std::abs(d[i]));
        return m;
    }
};

template <int N> inline double val(const Dual<N> &a) { return a.v; }
inline double val(double a) { return a; }

template <int N> inline Dual<N> operator-(const Dual<N> &a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator+(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator/(const Dual<N> &a, const Dual<N> &b) { Dual<N> r; r.v = a.v / b.v; double b2 = b.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / b2; return r; }
template <int N> inline Dual<N> operator+(const Dual<N> &a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> inline Dual<N> operator+(double b, const Dual<N> &a) { return a + b; }
template <int N> inline Dual<N> operator-(const Dual<N> &a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> inline Dual<N> operator-(double b, const Dual<N> &a) { return (-a) + b; }
template <int N> inline Dual<N> operator*(const Dual<N> &a, double b) { Dual<N> r; r.v = a.v * b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b; return r; }
template <int N> inline Dual<N> operator*(double b, const Dual<N> &a) { return a * b; }
template <int N> inline Dual<N> operator/(const Dual<N> &a, double b) { Dual<N> r; r.v = a.v / b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b; return r; }
template <int N> inline Dual<N> operator/(double a, const Dual<N> &b) { Dual<N> r; r.v = a / b.v; for (int i = 0; i < N; ++i) r.d[i] = -a * b.d[i] / (b.v * b.v); return r; }
template <int N> inline Dual<N> &operator+=(Dual<N> &a, const Dual<N> &b) { a = a + b; return a; }
template <int N> inline Dual<N> &operator-=(Dual<N> &a, const Dual<N> &b) { a = a - b; return a; }
template <int N> inline Dual<N> &operator*=(Dual<N> &a, const Dual<N> &b) { a = a * b; return a; }
template <int N> inline Dual<N> &operator/=(Dual<N> &a, const Dual<N> &b) { a = a / b; return a; }

template <int N> inline Dual<N> d_sqrt(const Dual<N> &a) { Dual<N> r; r.v = std::sqrt(a.v); for (int i = 0; i < N; ++i) r.d[i] = 0.5 * a.d[i] / r.v; return r; }
template <int N> inline Dual<N> d_exp(const Dual<N> &a) { Dual<N> r; r.v = std::exp(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * r.v; return r; }
template <int N> inline Dual<N> d_log(const Dual<N> &a) { Dual<N> r; r.v = std::log(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v; return r; }
template <int N> inline Dual<N> d_abs(const Dual<N> &a) { Dual<N> r; r.v = std::abs(a.v); double s = a.v > 0.0 ? 1.0 : -1.0; for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i]; return r; }
template <int N> inline Dual<N> d_asin(const Dual<N> &a) { Dual<N> r; r.v = std::asin(a.v); double k = 1.0 / std::sqrt(1.0 - a.v * a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * k; return r; }
// simpleAD.h:215-218: x^a with a constant
template <int N> inline Dual<N> d_pow(const Dual<N> &a, double e) { Dual<N> r; double t = std::pow(a.v, e - 1.0); r.v = a.v * t; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * e * t; return r; }
// simpleAD.h:211-213: x^y = exp(y log x)
template <int N> inline Dual<N> d_pow(const Dual<N> &a, const Dual<N> &e) { return d_exp(e * d_log(a)); }

inline double d_sqrt(double a) { return std::sqrt(a); }
inline double d_exp(double a) { return std::exp(a); }
inline double d_abs(double a) { return std::abs(a); }
inline double d_pow(double a, double e) { return std::pow(a, e); }

// ---------------------------------------------------------------- 3-vectors
template <class S>
struct Vec3 {
    S x, y, z;
    Vec3() : x(0.0), y(0.0), z(0.0) {}
    Vec3(S a, S b, S c) : x(a), y(b), z(c) {}
    S &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const S &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
typedef Vec3<double> V3;

template <class S> inline Vec3<S> operator+(const Vec3<S> &a, const Vec3<S> &b) { return Vec3<S>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class S> inline Vec3<S> operator-(const Vec3<S> &a, const Vec3<S> &b) { return Vec3<S>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class S> inline Vec3<S> operator-(const Vec3<S> &a) { return Vec3<S>(-a.x, -a.y, -a.z); }
template <class S, class T> inline Vec3<S> operator*(const Vec3<S> &a, const T &s) { return Vec3<S>(a.x * s, a.y * s, a.z * s); }
template <class S, class T> inline Vec3<S> operator*(const T &s, const Vec3<S> &a) { return Vec3<S>(a.x * s, a.y * s, a.z * s); }
template <class S, class T> inline Vec3<S> operator/(const Vec3<S> &a, const T &s) { return Vec3<S>(a.x / s, a.y / s, a.z / s); }
template <class S> inline Vec3<S> cmul(const Vec3<S> &a, const Vec3<S> &b) { return Vec3<S>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class S> inline Vec3<S> &operator+=(Vec3<S> &a, const Vec3<S> &b) { a = a + b; return a; }
template <class S> inline Vec3<S> &operator-=(Vec3<S> &a, const Vec3<S> &b) { a = a - b; return a; }
template <class S> inline S dot(const Vec3<S> &a, const Vec3<S> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S> inline Vec3<S> cross(const Vec3<S> &a, const Vec3<S> &b) {
    return Vec3<S>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class S> inline S sq_norm(const Vec3<S> &a) { return dot(a, a); }
template <class S> inline S norm(const Vec3<S> &a) { return d_sqrt(sq_norm(a)); }
template <class S> inline Vec3<S> normalized(const Vec3<S> &a) { S n = norm(a); return a / n; }

// Dual-valued vector helpers (VectorAD, simpleAD.h:681-1000)
template <int N> using DV3 = Vec3<Dual<N>>;
template <int N> inline V3 val(const DV3<N> &a) { return V3(a.x.v, a.y.v, a.z.v); }
inline V3 val(const V3 &a) { return a; }
template <int N> inline DV3<N> lift(const V3 &a) { return DV3<N>(Dual<N>(a.x), Dual<N>(a.y), Dual<N>(a.z)); }
template <int N> inline V3 grad(const DV3<N> &a, int j) { return V3(a.x.d[j], a.y.d[j], a.z.d[j]); }
template <int N> inline void set_grad(DV3<N> &a, int j, const V3 &g) { a.x.d[j] = g.x; a.y.d[j] = g.y; a.z.d[j] = g.z; }
template <int N> inline bool der_is_zero(const DV3<N> &a, double eps) {
    return a.x.der_is_zero(eps) && a.y.der_is_zero(eps) && a.z.der_is_zero(eps);
}
template <int N> inline DV3<N> zero_grad(const DV3<N> &a) { return lift<N>(val(a)); }
// Array1D::isZero checks the value part only (simpleAD.h:386)
template <class S> inline bool is_zero(const Vec3<S> &a, double eps) {
    return std::abs(val(a.x)) <= eps && std::abs(val(a.y)) <= eps && std::abs(val(a.z)) <= eps;
}
inline double max_coeff(const V3 &a) { return std::max(a.x, std::max(a.y, a.z)); }
inline double min_coeff(const V3 &a) { return std::min(a.x, std::min(a.y, a.z)); }

// ---------------------------------------------------------------- matrices
struct M3 {
    double m[9];  // row-major
    V3 operator*(const V3 &v) const {
        return V3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
                  m[6] * v.x + m[7] * v.y + m[8] * v.z);
    }
    template <int N> DV3<N> mul(const DV3<N> &v) const {
        return DV3<N>(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
                      m[6] * v.x + m[7] * v.y + m[8] * v.z);
    }
    M3 transpose() const {
        M3 r;
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i * 3 + j] = m[j * 3 + i];
        return r;
    }
};
struct M4 {
    double m[16];  // row-major
    static M4 identity() { M4 r; for (int i = 0; i < 16; ++i) r.m[i] = (i % 5 == 0) ? 1.0 : 0.0; return r; }
};
bool invert4(const M4 &a, M4 &out);
bool invert3(const M3 &a, M3 &out);
// utils.cpp:7-15
inline V3 xfm_point(const M4 &T, const V3 &p) {
    double x = T.m[0] * p.x + T.m[1] * p.y + T.m[2] * p.z + T.m[3];
    double y = T.m[4] * p.x + T.m[5] * p.y + T.m[6] * p.z + T.m[7];
    double z = T.m[8] * p.x + T.m[9] * p.y + T.m[10] * p.z + T.m[11];
    double w = T.m[12] * p.x + T.m[13] * p.y + T.m[14] * p.z + T.m[15];
    return V3(x / w, y / w, z / w);
}
inline V3 xfm_vector(const M4 &T, const V3 &v) {
    return V3(T.m[0] * v.x + T.m[1] * v.y + T.m[2] * v.z, T.m[4] * v.x + T.m[5] * v.y + T.m[6] * v.z,
              T.m[8] * v.x + T.m[9] * v.y + T.m[10] * v.z);
}

// ---------------------------------------------------------------- RNG
// src/sampler.cpp:3-37: PCG32 XSH-RR, stream (idx+1)<<1|1, seed added to the state,
// FP64 uniforms built from 32 random bits.
struct Rng {
    uint64_t state, inc;
    Rng(uint64_t seed, uint64_t idx) {
        state = 0u;
        inc = ((idx + 1) << 1u) | 1u;
        next_u32();
        state += (0x853c49e6748fea9bULL + seed);
        next_u32();
    }
    uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + (inc | 1);
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((-rot) & 31));
    }
    double next1() {
        uint64_t u = ((uint64_t)next_u32() << 20) | 0x3ff0000000000000ULL;
        double d;
        std::memcpy(&d, &u, 8);
        return d - 1.0;
    }
};

// ---------------------------------------------------------------- frames
// utils.cpp:54-82: orthonormal basis with a fixed pre-rotation (angle 0.1 about
// normalize(0.1,0.2,0.3), float literals widened to double as in the reference).
const M3 &frame_prerotation();
template <class S>
inline void coordinate_system(const Vec3<S> &n_in, Vec3<S> &s, Vec3<S> &t) {
    const M3 &R = frame_prerotation();
    M3 Rt = R.transpose();
    Vec3<S> n(R.m[0] * n_in.x + R.m[1] * n_in.y + R.m[2] * n_in.z, R.m[3] * n_in.x + R.m[4] * n_in.y + R.m[5] * n_in.z,
              R.m[6] * n_in.x + R.m[7] * n_in.y + R.m[8] * n_in.z);
    if (std::abs(val(n.x)) > std::abs(val(n.y))) {
        S inv_len = 1.0 / d_sqrt(n.x * n.x + n.z * n.z);
        t = Vec3<S>(n.z * inv_len, S(0.0), -n.x * inv_len);
    } else {
        S inv_len = 1.0 / d_sqrt(n.y * n.y + n.z * n.z);
        t = Vec3<S>(S(0.0), n.z * inv_len, -n.y * inv_len);
    }
    s = cross(t, n);
    auto rot = [&](const Vec3<S> &v) {
        return Vec3<S>(Rt.m[0] * v.x + Rt.m[1] * v.y + Rt.m[2] * v.z, Rt.m[3] * v.x + Rt.m[4] * v.y + Rt.m[5] * v.z,
                       Rt.m[6] * v.x + Rt.m[7] * v.y + Rt.m[8] * v.z);
    };
    s = rot(s);
    t = rot(t);
}

// include/frame.h / include/frameAD.h
template <class S>
struct FrameT {
    Vec3<S> s, t, n;
    FrameT() {}
    explicit FrameT(const Vec3<S> &nn) : n(nn) { coordinate_system(nn, s, t); }
    Vec3<S> to_local(const Vec3<S> &v) const { return Vec3<S>(dot(v, s), dot(v, t), dot(v, n)); }
    Vec3<S> to_world(const Vec3<S> &v) const { return s * v.x + t * v.y + n * v.z; }
};
typedef FrameT<double> Frame;
template <int N> inline Frame val(const FrameT<Dual<N>> &f) {
    Frame r;
    r.s = val(f.s); r.t = val(f.t); r.n = val(f.n);
    return r;
}
inline Frame val(const Frame &f) { return f; }
// frame.h:57-67 / frameAD.h:136-146
template <class S> inline S sin_theta(const Vec3<S> &v) {
    S tmp = 1.0 - v.z * v.z;
    return val(tmp) < kEps ? S(0.0) : d_sqrt(tmp);
}
template <class S> inline S tan_theta(const Vec3<S> &v) {
    S tmp = 1.0 - v.z * v.z;
    return val(tmp) < kEps ? S(0.0) : d_sqrt(tmp) / v.z;
}

// ---------------------------------------------------------------- warps
// utils.cpp:18-52
inline void square_to_disk_concentric(double sx, double sy, double &ox, double &oy) {
    double r1 = 2.0 * sx - 1.0, r2 = 2.0 * sy - 1.0, phi, r;
    if (r1 == 0 && r2 == 0) {
        r = phi = 0;
    } else if (r1 * r1 > r2 * r2) {
        r = r1;
        phi = (kPi / 4.0) * (r2 / r1);
    } else {
        r = r2;
        phi = (kPi / 2.0) - (r1 / r2) * (kPi / 4.0);
    }
    // the reference names sin(phi) "cosPhi" and returns (r sin phi, r cos phi)
    ox = r * std::sin(phi);
    oy = r * std::cos(phi);
}
inline V3 square_to_cosine_hemisphere(double sx, double sy) {
    double px, py;
    square_to_disk_concentric(sx, sy, px, py);
    double z = std::sqrt(std::max(0.0, 1.0 - px * px - py * py));
    return V3(px, py, z);
}
inline double cosine_hemisphere_pdf(const V3 &d) { return kInvPi * d.z; }
inline V3 square_to_uniform_sphere(double sx, double sy) {
    double z = 1.0 - 2.0 * sy;
    double r = std::sqrt(1.0 - z * z);
    return V3(r * std::cos(2.0 * kPi * sx), r * std::sin(2.0 * kPi * sx), z);
}
inline double luminance(const V3 &v) {  // utils.cpp:84-88
    return (double)0.212671f * v.x + (double)0.715160f * v.y + (double)0.072169f * v.z;
}
inline double signum(double v) { return std::copysign(1.0, v); }

// utils.cpp:119-184 (shared by the plain and dual versions)
template <class S>
inline S fresnel_dielectric_ext(const S &cos_i_in, S &cos_t_out, const S &eta) {
    if (std::abs(val(eta) - 1.0) < kEps) {
        cos_t_out = -cos_i_in;
        return S(0.0);
    }
    S scale = val(cos_i_in) > 0.0 ? 1.0 / eta : eta;
    S cos_t_sqr = 1.0 - (1.0 - cos_i_in * cos_i_in) * (scale * scale);
    if (val(cos_t_sqr) < kEps) {
        cos_t_out = S(0.0);
        return S(1.0);
    }
    S cos_i = d_abs(cos_i_in);
    S cos_t = d_sqrt(cos_t_sqr);
    S Rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    S Rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    cos_t_out = val(cos_i_in) > 0.0 ? -cos_t : cos_t;
    return 0.5 * (Rs * Rs + Rp * Rp);
}
template <class S> inline S fresnel_dielectric_ext(const S &cos_i, const S &eta) {
    S c;
    return fresnel_dielectric_ext(cos_i, c, eta);
}
inline V3 reflect(const V3 &wi, const V3 &n) { return n * (2.0 * dot(wi, n)) - wi; }
// utils.cpp:186-189
inline V3 refract(const V3 &wi, const V3 &n, double eta, double cos_t) {
    if (cos_t < 0) eta = 1.0 / eta;
    return n * (dot(wi, n) * eta + cos_t) - wi * eta;
}

// utils.cpp:218-254: Moller-Trumbore with the divisor clamp ("hack"), returning (u, v, t)
template <class S>
inline Vec3<S> ray_intersect_triangle(const Vec3<S> &v0, const Vec3<S> &v1, const Vec3<S> &v2,
                                      const Vec3<S> &org, const Vec3<S> &dir) {
    Vec3<S> e1 = v1 - v0, e2 = v2 - v0;
    Vec3<S> pvec = cross(dir, e2);
    S divisor = dot(pvec, e1);
    if (std::abs(val(divisor)) < kEps) divisor = S(val(divisor) > 0 ? kEps : -kEps);
    Vec3<S> s = org - v0;
    S u = dot(s, pvec) / divisor;
    Vec3<S> qvec = cross(s, e1);
    S v = dot(dir, qvec) / divisor;
    S t = dot(e2, qvec) / divisor;
    return Vec3<S>(u, v, t);
}

// utils.cpp:256-266
inline double compute_intersection_in_tri(const V3 &a, const V3 &b0, const V3 &c0, const V3 &b1, const V3 &c1,
                                          double t0) {
    double cb = norm(b0 - a) / norm(b1 - a);
    double cc = norm(c0 - a) / norm(c1 - a);
    double bx = (1 - t0) * cb, by = t0 * cc;
    double s = bx + by;
    return by / s;
}

// ---------------------------------------------------------------- discrete distribution
// include/pmf.h:8-190
struct Distrib {
    std::vector<double> cdf{0.0};
    double sum = 0, normalization = 0;
    void clear() { cdf.assign(1, 0.0); sum = normalization = 0; }
    void append(double p) { cdf.push_back(cdf.back() + p); }
    size_t size() const { return cdf.size() - 1; }
    double operator[](size_t i) const { return cdf[i + 1] - cdf[i]; }
    double normalize() {
        sum = cdf.back();
        if (sum > 0) {
            normalization = 1.0 / sum;
            for (size_t i = 1; i < cdf.size(); ++i) cdf[i] *= normalization;
            cdf.back() = 1.0;
        } else {
            normalization = 0.0;
        }
        return sum;
    }
    size_t sample(double u) const {
        auto it = std::lower_bound(cdf.begin(), cdf.end(), u);
        ptrdiff_t k = (it - cdf.begin()) - 1;
        size_t index = std::min(cdf.size() - 2, (size_t)std::max((ptrdiff_t)0, k));
        while ((*this)[index] == 0 && index < cdf.size() - 1) ++index;
        return index;
    }
    size_t sample_reuse(double &u) const {
        size_t i = sample(u);
        u = (u - cdf[i]) / (cdf[i + 1] - cdf[i]);
        return i;
    }
    size_t sample_reuse(double &u, double &pdf) const {
        size_t i = sample(u);
        pdf = (*this)[i];
        u = (u - cdf[i]) / (cdf[i + 1] - cdf[i]);
        return i;
    }
};

// include/aabb.h:185-215 slab test
struct AABB {
    V3 mn{1e300, 1e300, 1e300}, mx{-1e300, -1e300, -1e300};
    void expand(const V3 &p) {
        mn = V3(std::min(mn.x, p.x), std::min(mn.y, p.y), std::min(mn.z, p.z));
        mx = V3(std::max(mx.x, p.x), std::max(mx.y, p.y), std::max(mx.z, p.z));
    }
    bool ray_intersect(const V3 &o, const V3 &d, double &near_t, double &far_t) const {
        near_t = -INFINITY;
        far_t = INFINITY;
        for (int i = 0; i < 3; ++i) {
            double origin = o[i], lo = mn[i], hi = mx[i];
            if (d[i] == 0) {
                if (origin < lo || origin > hi) return false;
            } else {
                double t1 = (lo - origin) / d[i], t2 = (hi - origin) / d[i];
                if (t1 > t2) std::swap(t1, t2);
                near_t = std::max(t1, near_t);
                far_t = std::min(t2, far_t);
                if (!(near_t <= far_t)) return false;
            }
        }
        return true;
    }
};

}  // namespace orc
