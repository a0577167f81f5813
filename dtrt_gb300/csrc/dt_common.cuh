// dtrt_gb300 — device math: FP32 forward-mode duals, vectors, frames, PCG32, warps.
//
// The path state is FP32; the dual type carries the value plus N derivative slots,
// following the chain rules of the reference's include/simpleAD.h. FP64 is used only
// by the edge-sampling geometry and the pixel accumulators (see dt_edge.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define DT_HD __host__ __device__ __forceinline__
#define DT_D __device__ __forceinline__
// Large scene queries (BVH traversal, transmittance chains, NEE, BSDF sampling) are called
// from many places of the path kernels; keeping them out of line keeps each kernel's code
// inside the instruction cache. DT_INLINE_HEAVY inlines them instead.
#ifdef DT_INLINE_HEAVY
#define DT_HEAVY static __device__ __forceinline__
#else
#define DT_HEAVY static __device__ __noinline__
#endif

namespace dt {

// include/fwd.h:10-18 and include/config.h:5-7 of the reference
constexpr float kEps = 1e-7f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInvTwoPi = 0.15915494309189534561f;
constexpr float kInvFourPi = 0.07957747154594766788f;
constexpr float kShadowEps = 1e-3f;
constexpr float kAngleEps = 1e-4f;
constexpr double kEpsD = 1e-7;
constexpr double kPiD = 3.14159265358979323846;
// A derivative slot smaller than this is treated as exactly zero where the reference
// tests `der.isZero(1e-7)` on quantities that are analytically zero but carry FP32
// rounding here (e.g. the hit distance of a ray that moves with the surface it hits).
constexpr float kDerZeroEps = 1e-5f;

// ------------------------------------------------------------------ float3 helpers
DT_HD float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
DT_HD float3 operator+(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
DT_HD float3 operator-(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
DT_HD float3 operator-(float3 a) { return mk(-a.x, -a.y, -a.z); }
DT_HD float3 operator*(float3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
DT_HD float3 operator*(float s, float3 a) { return mk(a.x * s, a.y * s, a.z * s); }
DT_HD float3 operator/(float3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
DT_HD float3 cmul(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
DT_HD float3 &operator+=(float3 &a, float3 b) { a = a + b; return a; }
DT_HD float3 &operator-=(float3 &a, float3 b) { a = a - b; return a; }
DT_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DT_HD float3 cross(float3 a, float3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
DT_HD float length(float3 a) { return sqrtf(dot(a, a)); }
DT_HD float3 normalize(float3 a) { return a / sqrtf(dot(a, a)); }
DT_HD bool is_zero3(float3 a, float eps = kEps) { return fabsf(a.x) <= eps && fabsf(a.y) <= eps && fabsf(a.z) <= eps; }
DT_HD float max3(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
DT_HD float min3(float3 a) { return fminf(a.x, fminf(a.y, a.z)); }
DT_HD float comp(float3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
DT_HD float signum(float v) { return copysignf(1.0f, v); }

struct double3_ { double x, y, z; };
DT_HD double3_ mkd(double x, double y, double z) { double3_ r; r.x = x; r.y = y; r.z = z; return r; }
DT_HD double3_ tod(float3 a) { return mkd(a.x, a.y, a.z); }
DT_HD float3 tof(double3_ a) { return mk((float)a.x, (float)a.y, (float)a.z); }
DT_HD double3_ operator+(double3_ a, double3_ b) { return mkd(a.x + b.x, a.y + b.y, a.z + b.z); }
DT_HD double3_ operator-(double3_ a, double3_ b) { return mkd(a.x - b.x, a.y - b.y, a.z - b.z); }
DT_HD double3_ operator*(double3_ a, double s) { return mkd(a.x * s, a.y * s, a.z * s); }
DT_HD double dotd(double3_ a, double3_ b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DT_HD double3_ crossd(double3_ a, double3_ b) { return mkd(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
DT_HD double lengthd(double3_ a) { return sqrt(dotd(a, a)); }
DT_HD double3_ normalized(double3_ a) { return a * (1.0 / lengthd(a)); }

// ------------------------------------------------------------------ FP32 dual number
// value + N derivative slots; simpleAD.h:20-245 chain rules
template <int N>
struct Df {
    float v;
    float d[N];
    DT_HD Df() : v(0.f) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = 0.f;
    }
    DT_HD Df(float x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = 0.f;
    }
    DT_HD bool der_zero(float eps) const {
        bool z = true;
#pragma unroll
        for (int i = 0; i < N; ++i) z = z && fabsf(d[i]) <= eps;
        return z;
    }
    DT_HD float der_max() const {
        float m = 0.f;
#pragma unroll
        for (int i = 0; i < N; ++i) m = fmaxf(m, fabsf(d[i]));
        return m;
    }
};

#define DF_LOOP _Pragma("unroll") for (int i = 0; i < N; ++i)
template <int N> DT_HD Df<N> operator-(const Df<N> &a) { Df<N> r; r.v = -a.v; DF_LOOP r.d[i] = -a.d[i]; return r; }
template <int N> DT_HD Df<N> operator+(const Df<N> &a, const Df<N> &b) { Df<N> r; r.v = a.v + b.v; DF_LOOP r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> DT_HD Df<N> operator-(const Df<N> &a, const Df<N> &b) { Df<N> r; r.v = a.v - b.v; DF_LOOP r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> DT_HD Df<N> operator*(const Df<N> &a, const Df<N> &b) { Df<N> r; r.v = a.v * b.v; DF_LOOP r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> DT_HD Df<N> operator/(const Df<N> &a, const Df<N> &b) {
    Df<N> r; float ib = 1.0f / b.v; r.v = a.v * ib; DF_LOOP r.d[i] = (a.d[i] - r.v * b.d[i]) * ib; return r;
}
template <int N> DT_HD Df<N> operator+(const Df<N> &a, float b) { Df<N> r = a; r.v += b; return r; }
template <int N> DT_HD Df<N> operator+(float b, const Df<N> &a) { Df<N> r = a; r.v += b; return r; }
template <int N> DT_HD Df<N> operator-(const Df<N> &a, float b) { Df<N> r = a; r.v -= b; return r; }
template <int N> DT_HD Df<N> operator-(float b, const Df<N> &a) { Df<N> r = -a; r.v += b; return r; }
template <int N> DT_HD Df<N> operator*(const Df<N> &a, float b) { Df<N> r; r.v = a.v * b; DF_LOOP r.d[i] = a.d[i] * b; return r; }
template <int N> DT_HD Df<N> operator*(float b, const Df<N> &a) { return a * b; }
template <int N> DT_HD Df<N> operator/(const Df<N> &a, float b) { return a * (1.0f / b); }
template <int N> DT_HD Df<N> operator/(float a, const Df<N> &b) {
    Df<N> r; r.v = a / b.v; float k = -r.v / b.v; DF_LOOP r.d[i] = k * b.d[i]; return r;
}
template <int N> DT_HD Df<N> &operator+=(Df<N> &a, const Df<N> &b) { a.v += b.v; DF_LOOP a.d[i] += b.d[i]; return a; }
template <int N> DT_HD Df<N> &operator*=(Df<N> &a, const Df<N> &b) { a = a * b; return a; }
template <int N> DT_HD Df<N> dsqrt(const Df<N> &a) { Df<N> r; r.v = sqrtf(a.v); float k = 0.5f / r.v; DF_LOOP r.d[i] = a.d[i] * k; return r; }
template <int N> DT_HD Df<N> dexp(const Df<N> &a) { Df<N> r; r.v = expf(a.v); DF_LOOP r.d[i] = a.d[i] * r.v; return r; }
template <int N> DT_HD Df<N> dlog(const Df<N> &a) { Df<N> r; r.v = logf(a.v); float k = 1.0f / a.v; DF_LOOP r.d[i] = a.d[i] * k; return r; }
template <int N> DT_HD Df<N> dabs(const Df<N> &a) { Df<N> r; r.v = fabsf(a.v); float s = a.v > 0.f ? 1.f : -1.f; DF_LOOP r.d[i] = a.d[i] * s; return r; }
template <int N> DT_HD Df<N> dpow(const Df<N> &a, float e) { Df<N> r; float t = powf(a.v, e - 1.0f); r.v = a.v * t; float k = e * t; DF_LOOP r.d[i] = a.d[i] * k; return r; }
template <int N> DT_HD Df<N> dpow(const Df<N> &a, const Df<N> &e) { return dexp(e * dlog(a)); }

// ------------------------------------------------------------------ dual 3-vectors
template <int N>
struct DV {
    Df<N> x, y, z;
    DT_HD DV() {}
    DT_HD DV(const Df<N> &a, const Df<N> &b, const Df<N> &c) : x(a), y(b), z(c) {}
    DT_HD explicit DV(float3 a) : x(a.x), y(a.y), z(a.z) {}
    DT_HD float3 val() const { return mk(x.v, y.v, z.v); }
    DT_HD float3 grad(int j) const { return mk(x.d[j], y.d[j], z.d[j]); }
    DT_HD void set_grad(int j, float3 g) { x.d[j] = g.x; y.d[j] = g.y; z.d[j] = g.z; }
    DT_HD bool der_zero(float eps) const { return x.der_zero(eps) && y.der_zero(eps) && z.der_zero(eps); }
    DT_HD bool is_zero(float eps = kEps) const { return fabsf(x.v) <= eps && fabsf(y.v) <= eps && fabsf(z.v) <= eps; }
};
template <int N> DT_HD DV<N> operator+(const DV<N> &a, const DV<N> &b) { return DV<N>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <int N> DT_HD DV<N> operator-(const DV<N> &a, const DV<N> &b) { return DV<N>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <int N> DT_HD DV<N> operator-(const DV<N> &a) { return DV<N>(-a.x, -a.y, -a.z); }
template <int N> DT_HD DV<N> operator*(const DV<N> &a, const Df<N> &s) { return DV<N>(a.x * s, a.y * s, a.z * s); }
template <int N> DT_HD DV<N> operator*(const DV<N> &a, float s) { return DV<N>(a.x * s, a.y * s, a.z * s); }
template <int N> DT_HD DV<N> operator/(const DV<N> &a, const Df<N> &s) { Df<N> k = 1.0f / s; return a * k; }
template <int N> DT_HD DV<N> operator/(const DV<N> &a, float s) { return a * (1.0f / s); }
template <int N> DT_HD DV<N> operator+(const DV<N> &a, float3 b) { return DV<N>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <int N> DT_HD DV<N> operator-(const DV<N> &a, float3 b) { return DV<N>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <int N> DT_HD DV<N> &operator+=(DV<N> &a, const DV<N> &b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
template <int N> DT_HD DV<N> cmul(const DV<N> &a, const DV<N> &b) { return DV<N>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <int N> DT_HD DV<N> cmul(const DV<N> &a, float3 b) { return DV<N>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <int N> DT_HD Df<N> dot(const DV<N> &a, const DV<N> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <int N> DT_HD Df<N> dot(const DV<N> &a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <int N> DT_HD DV<N> cross(const DV<N> &a, const DV<N> &b) {
    return DV<N>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <int N> DT_HD Df<N> length(const DV<N> &a) { return dsqrt(dot(a, a)); }
template <int N> DT_HD DV<N> normalize(const DV<N> &a) { return a / length(a); }
template <int N> DT_HD DV<N> zero_grad(const DV<N> &a) { return DV<N>(a.val()); }

// ------------------------------------------------------------------ frames
// utils.cpp:54-82 of the reference: a fixed pre-rotation (angle 0.1 about
// normalize(0.1,0.2,0.3)) before the usual branchy orthonormal-basis construction.
// Row-major R = Rodrigues(angle 0.1, axis normalize(0.1, 0.2, 0.3)), rounded to FP32.
#define DT_PREROT_INIT                                                                                  \
    {9.953610105e-01f, -7.933111998e-02f, 5.443374181e-02f, 8.075850132e-02f, 9.964315465e-01f,      \
     -2.454053082e-02f, -5.229266974e-02f, 2.882267496e-02f, 9.982157733e-01f}

DT_D float3 rot_apply(const float *m, float3 v) {
    return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}
DT_D float3 rot_apply_t(const float *m, float3 v) {
    return mk(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
              m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

struct Frame {
    float3 s, t, n;
    DT_D Frame() {}
    DT_D explicit Frame(float3 nn) : n(nn) {
        const float R[9] = DT_PREROT_INIT;
        float3 q = rot_apply(R, nn);
        float3 tt;
        if (fabsf(q.x) > fabsf(q.y)) {
            float il = 1.0f / sqrtf(q.x * q.x + q.z * q.z);
            tt = mk(q.z * il, 0.f, -q.x * il);
        } else {
            float il = 1.0f / sqrtf(q.y * q.y + q.z * q.z);
            tt = mk(0.f, q.z * il, -q.y * il);
        }
        float3 ss = cross(tt, q);
        s = rot_apply_t(R, ss);
        t = rot_apply_t(R, tt);
    }
    DT_D float3 to_local(float3 v) const { return mk(dot(v, s), dot(v, t), dot(v, n)); }
    DT_D float3 to_world(float3 v) const { return s * v.x + t * v.y + n * v.z; }
};

template <int N>
struct FrameAD {
    DV<N> s, t, n;
    DT_D FrameAD() {}
    DT_D explicit FrameAD(const DV<N> &nn) : n(nn) {
        if (nn.der_zero(0.f)) {  // a fixed normal: the plain frame, lifted
            const Frame f(nn.val());
            s = DV<N>(f.s);
            t = DV<N>(f.t);
            return;
        }
        const float R[9] = DT_PREROT_INIT;
        DV<N> q(R[0] * nn.x + R[1] * nn.y + R[2] * nn.z, R[3] * nn.x + R[4] * nn.y + R[5] * nn.z,
                R[6] * nn.x + R[7] * nn.y + R[8] * nn.z);
        DV<N> tt;
        if (fabsf(q.x.v) > fabsf(q.y.v)) {
            Df<N> il = 1.0f / dsqrt(q.x * q.x + q.z * q.z);
            tt = DV<N>(q.z * il, Df<N>(0.f), -q.x * il);
        } else {
            Df<N> il = 1.0f / dsqrt(q.y * q.y + q.z * q.z);
            tt = DV<N>(Df<N>(0.f), q.z * il, -q.y * il);
        }
        DV<N> ss = cross(tt, q);
        s = DV<N>(R[0] * ss.x + R[3] * ss.y + R[6] * ss.z, R[1] * ss.x + R[4] * ss.y + R[7] * ss.z,
                  R[2] * ss.x + R[5] * ss.y + R[8] * ss.z);
        t = DV<N>(R[0] * tt.x + R[3] * tt.y + R[6] * tt.z, R[1] * tt.x + R[4] * tt.y + R[7] * tt.z,
                  R[2] * tt.x + R[5] * tt.y + R[8] * tt.z);
    }
    DT_D DV<N> to_local(const DV<N> &v) const { return DV<N>(dot(v, s), dot(v, t), dot(v, n)); }
    DT_D DV<N> to_local(float3 v) const { return DV<N>(dot(s, v), dot(t, v), dot(n, v)); }
    DT_D DV<N> to_world(const DV<N> &v) const { return s * v.x + t * v.y + n * v.z; }
    DT_D Frame plain() const {
        Frame f;
        f.s = s.val(); f.t = t.val(); f.n = n.val();
        return f;
    }
};

// ------------------------------------------------------------------ RNG
// PCG32 XSH-RR seeded like the reference's RndSampler(seed, idx) (src/sampler.cpp:3-9).
struct Rng {
    uint64_t state, inc;
    DT_HD uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    DT_HD void init(uint64_t seed, uint64_t idx) {
        state = 0u;
        inc = ((idx + 1) << 1u) | 1u;
        next_u32();
        state += (0x853c49e6748fea9bULL + seed);
        next_u32();
    }
    // FP32 uniform in [0,1) from the top 24 bits
    DT_HD float next1() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
    // FP64 uniform in [0,1) from 32 bits (as the reference, sampler.cpp:21-27)
    DT_HD double next1d() { return (double)next_u32() * (1.0 / 4294967296.0); }
};

// 64-bit mixer for sub-task stream ids (splitmix64 finaliser)
DT_HD uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}
DT_HD uint64_t child_key(uint64_t parent, uint32_t a, uint32_t b) {
    return mix64(parent * 0x9E3779B97F4A7C15ULL + ((uint64_t)a << 32 | b) + 0x632BE59BD9B4E019ULL);
}

// ------------------------------------------------------------------ warps and helpers
// utils.cpp:18-52 of the reference (concentric disk with sin/cos swapped, cosine hemisphere,
// uniform sphere)
DT_D float3 square_to_cosine_hemisphere(float sx, float sy) {
    float r1 = 2.f * sx - 1.f, r2 = 2.f * sy - 1.f, phi, r;
    if (r1 == 0.f && r2 == 0.f) {
        r = phi = 0.f;
    } else if (r1 * r1 > r2 * r2) {
        r = r1;
        phi = (kPi / 4.f) * (r2 / r1);
    } else {
        r = r2;
        phi = (kPi / 2.f) - (r1 / r2) * (kPi / 4.f);
    }
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float px = r * sp, py = r * cp;
    float z = sqrtf(fmaxf(0.f, 1.f - px * px - py * py));
    return mk(px, py, z);
}
DT_D float cosine_hemisphere_pdf(float3 d) { return kInvPi * d.z; }
DT_D float3 square_to_uniform_sphere(float sx, float sy) {
    float z = 1.f - 2.f * sy;
    float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp, cp;
    sincosf(2.f * kPi * sx, &sp, &cp);
    return mk(r * cp, r * sp, z);
}
DT_D float mis_weight(float a, float b) {  // volpathAD.cpp:43-47
    a *= a;
    b *= b;
    return a / (a + b);
}
DT_D float luminance(float3 v) { return 0.212671f * v.x + 0.715160f * v.y + 0.072169f * v.z; }

}  // namespace dt
