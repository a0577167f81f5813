// dtrt_gb300 — C ABI (include/dtrt_gb300.h): scene construction on the host, device
// upload, and dispatch of the render entry points by derivative width.
//
// Scene construction restates the reference's constructors (uci-rendering/dtrt):
// Camera (src/camera.cpp:8-38, 103-111), Shape (src/shape.cpp:10-52, 109-126, 254-300),
// the BSDF / phase / emitter / medium constructors (src/dtrt.cpp:55-93 and their
// headers), Scene light tables (src/scene.cpp:45-98), the secondary-edge manager
// (src/edge_manager/bruteforce.cpp:4-20) and primary-edge projection
// (src/edge_manager/edge_manager.cpp:6-110, include/line_clip.h:37-95).
#include <atomic>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dt_bvh.h"
#include "dt_host.h"

namespace dt {

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }

bool ensure_buffer(void **ptr, size_t *have, size_t need) {
    if (*have >= need && *ptr) return true;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(ptr, std::max<size_t>(need, 256));
    if (e != cudaSuccess) {
        set_last_error(std::string("cudaMalloc(") + std::to_string(need) + "): " + cudaGetErrorString(e));
        *ptr = nullptr;
        return false;
    }
    *have = std::max<size_t>(need, 256);
    return true;
}

namespace {

// ------------------------------------------------------------------ host FP64 duals (8 slots)
struct HD {
    double v = 0, d[kMaxNder] = {0, 0, 0, 0, 0, 0, 0, 0};
    HD() {}
    HD(double x) : v(x) {}
};
HD operator+(const HD &a, const HD &b) { HD r(a.v + b.v); for (int i = 0; i < kMaxNder; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
HD operator-(const HD &a, const HD &b) { HD r(a.v - b.v); for (int i = 0; i < kMaxNder; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
HD operator*(const HD &a, const HD &b) { HD r(a.v * b.v); for (int i = 0; i < kMaxNder; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
HD operator/(const HD &a, const HD &b) { HD r(a.v / b.v); for (int i = 0; i < kMaxNder; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v); return r; }
HD operator*(const HD &a, double s) { HD r(a.v * s); for (int i = 0; i < kMaxNder; ++i) r.d[i] = a.d[i] * s; return r; }
HD hsqrt(const HD &a) { HD r(std::sqrt(a.v)); for (int i = 0; i < kMaxNder; ++i) r.d[i] = 0.5 * a.d[i] / r.v; return r; }
struct HV {
    HD x, y, z;
    HD &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const HD &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
HV operator+(const HV &a, const HV &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
HV operator-(const HV &a, const HV &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
HV operator*(const HV &a, const HD &s) { return {a.x * s, a.y * s, a.z * s}; }
HV operator*(const HV &a, double s) { return {a.x * s, a.y * s, a.z * s}; }
HV operator/(const HV &a, const HD &s) { return {a.x / s, a.y / s, a.z / s}; }
HD hdot(const HV &a, const HV &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HV hcross(const HV &a, const HV &b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
struct D3 {
    double x, y, z;
};
D3 val(const HV &a) { return {a.x.v, a.y.v, a.z.v}; }
D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dnorm(D3 a) { return std::sqrt(ddot(a, a)); }
D3 dnormalize(D3 a) { double l = dnorm(a); return {a.x / l, a.y / l, a.z / l}; }

bool invert4(const double *m, double *out) {
    double inv[16];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0 || !std::isfinite(det)) return false;
    for (int i = 0; i < 16; ++i) out[i] = inv[i] / det;
    return true;
}
bool invert3(const double *m, double *out) {
    double c0 = m[4] * m[8] - m[5] * m[7], c1 = m[5] * m[6] - m[3] * m[8], c2 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c0 + m[1] * c1 + m[2] * c2;
    if (det == 0 || !std::isfinite(det)) return false;
    double id = 1.0 / det;
    out[0] = c0 * id; out[1] = (m[2] * m[7] - m[1] * m[8]) * id; out[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    out[3] = c1 * id; out[4] = (m[0] * m[8] - m[2] * m[6]) * id; out[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    out[6] = c2 * id; out[7] = (m[1] * m[6] - m[0] * m[7]) * id; out[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return true;
}
D3 xfm_point(const double *T, D3 p) {
    double x = T[0] * p.x + T[1] * p.y + T[2] * p.z + T[3], y = T[4] * p.x + T[5] * p.y + T[6] * p.z + T[7];
    double z = T[8] * p.x + T[9] * p.y + T[10] * p.z + T[11], w = T[12] * p.x + T[13] * p.y + T[14] * p.z + T[15];
    return {x / w, y / w, z / w};
}

int read_vol(const char *path, int res[3], int &ch, float vmin[3], float vmax[3], std::vector<float> *data) {
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_last_error(std::string("cannot open volume file ") + path);
        return DTRT_ERR_IO;
    }
    char hdr[3];
    unsigned char ver = 0;
    int type = 0;
    bool ok = std::fread(hdr, 1, 3, f) == 3 && std::strncmp(hdr, "VOL", 3) == 0 && std::fread(&ver, 1, 1, f) == 1 &&
              ver == 3 && std::fread(&type, 4, 1, f) == 1 && std::fread(res, 4, 3, f) == 3 &&
              std::fread(&ch, 4, 1, f) == 1 && type == 1 && (ch == 1 || ch == 3) && std::fread(vmin, 4, 3, f) == 3 &&
              std::fread(vmax, 4, 3, f) == 3 && res[0] > 0 && res[1] > 0 && res[2] > 0;
    if (ok && data) {
        size_t n = (size_t)res[0] * res[1] * res[2] * ch;
        data->resize(n);
        ok = std::fread(data->data(), 4, n, f) == n;
    }
    std::fclose(f);
    if (!ok) {
        set_last_error(std::string("invalid VOL v3 file ") + path);
        return DTRT_ERR_IO;
    }
    return DTRT_OK;
}

// Device uploads of one scene build. Every upload call takes the next slot of
// s->allocs (an empty array takes a null slot), so two builds of scenes with the same
// structure issue their arrays in the same slot order. Given the allocations of the scene
// being replaced (`reuse`, in that slot order), an upload of the same byte size takes the
// old buffer, and the copy is deferred to commit(): nothing on the device changes until
// the whole host build has succeeded.
struct Builder {
    struct Slot {
        void *p;
        size_t bytes;
    };
    dtrt_scene *s;
    std::vector<Slot> *reuse = nullptr;
    std::vector<std::pair<void *, std::vector<char>>> pending;
    std::vector<char> taken;  // per slot of s->allocs: the buffer came from `reuse`
    int reused = 0, allocated = 0;
    double ms_alloc = 0.0;
    explicit Builder(dtrt_scene *sc, std::vector<Slot> *old = nullptr) : s(sc), reuse(old) {}
    template <class T>
    bool upload(const std::vector<T> &v, const T **dst) {
        const size_t k = s->allocs.size(), bytes = v.size() * sizeof(T);
        void *p = nullptr;
        bool from_old = false;
        if (bytes) {
            if (reuse && k < reuse->size() && (*reuse)[k].p && (*reuse)[k].bytes == bytes) {
                p = (*reuse)[k].p;
                (*reuse)[k].p = nullptr;
                from_old = true;
                ++reused;
            } else {
                const auto ta = std::chrono::steady_clock::now();
                cudaError_t e = cudaMalloc(&p, bytes);
                ms_alloc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - ta).count();
                if (e != cudaSuccess) {
                    set_last_error(std::string("scene upload: ") + cudaGetErrorString(e));
                    return false;
                }
                ++allocated;
            }
        }
        s->allocs.push_back(p);
        s->alloc_bytes.push_back(bytes);
        taken.push_back(from_old ? 1 : 0);
        *dst = (const T *)p;
        if (!bytes) return true;
        if (reuse) {
            const char *b = reinterpret_cast<const char *>(v.data());
            pending.emplace_back(p, std::vector<char>(b, b + bytes));
            return true;
        }
        cudaError_t e = cudaMemcpy(p, v.data(), bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_last_error(std::string("scene upload: ") + cudaGetErrorString(e));
            return false;
        }
        return true;
    }
    // take over a device allocation written elsewhere (never reused from the old scene, so
    // a failed update leaves the old scene's arrays untouched)
    template <class T>
    void adopt(T *p, size_t bytes, const T **dst) {
        s->allocs.push_back(p);
        s->alloc_bytes.push_back(bytes);
        taken.push_back(0);
        *dst = p;
        ++allocated;
    }
    // deferred copies (reuse mode)
    int commit() {
        for (auto &pc : pending) {
            cudaError_t e = cudaMemcpy(pc.first, pc.second.data(), pc.second.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                set_last_error(std::string("scene upload: ") + cudaGetErrorString(e));
                return DTRT_ERR_CUDA;
            }
        }
        pending.clear();
        return DTRT_OK;
    }
    // a failed reuse-mode build: free what it allocated, hand the taken buffers back
    void discard() {
        for (size_t k = 0; k < s->allocs.size(); ++k) {
            if (taken[k]) (*reuse)[k].p = s->allocs[k];
            else if (s->allocs[k]) cudaFree(s->allocs[k]);
        }
        s->allocs.clear();
        s->alloc_bytes.clear();
        taken.clear();
        pending.clear();
    }
};

// Cohen-Sutherland on screen coordinates carrying duals (line_clip.h:37-95)
int out_code(double x, double y, double xmin, double xmax, double ymin, double ymax) {
    int c = 0;
    if (x < xmin - 1e-7) c |= 1;
    else if (x > xmax + 1e-7) c |= 2;
    if (y < ymin - 1e-7) c |= 4;
    else if (y > ymax + 1e-7) c |= 8;
    return c;
}
bool clip_line(const HD v0[2], const HD v1[2], HD c0[2], HD c1[2], double xmin, double xmax, double ymin, double ymax) {
    c0[0] = v0[0]; c0[1] = v0[1]; c1[0] = v1[0]; c1[1] = v1[1];
    int o0 = out_code(c0[0].v, c0[1].v, xmin, xmax, ymin, ymax), o1 = out_code(c1[0].v, c1[1].v, xmin, xmax, ymin, ymax);
    for (int guard = 0; guard < 64; ++guard) {
        if (!(o0 | o1)) return true;
        if (o0 & o1) return false;
        const int oo = o0 ? o0 : o1;
        double k;
        if (oo & 8) k = (ymax - c0[1].v) / (c1[1].v - c0[1].v);
        else if (oo & 4) k = (ymin - c0[1].v) / (c1[1].v - c0[1].v);
        else if (oo & 2) k = (xmax - c0[0].v) / (c1[0].v - c0[0].v);
        else k = (xmin - c0[0].v) / (c1[0].v - c0[0].v);
        HD p[2] = {c0[0] + (c1[0] - c0[0]) * k, c0[1] + (c1[1] - c0[1]) * k};
        if (oo == o0) {
            c0[0] = p[0]; c0[1] = p[1];
            o0 = out_code(c0[0].v, c0[1].v, xmin, xmax, ymin, ymax);
        } else {
            c1[0] = p[0]; c1[1] = p[1];
            o1 = out_code(c1[0].v, c1[1].v, xmin, xmax, ymin, ymax);
        }
    }
    return false;
}
double intersection_in_tri(D3 b0, D3 c0, D3 b1, D3 c1, double t0) {  // utils.cpp:256-266
    double cb = dnorm(b0) / dnorm(b1), cc = dnorm(c0) / dnorm(c1);
    double bx = (1 - t0) * cb, by = t0 * cc;
    return by / (bx + by);
}

bool load_grid(DevGrid &g, Builder &bld, const char *file, const float *arr, const int *res, int ch, const float *vmin,
               const float *vmax, const float *to_world, int &status) {
    std::vector<float> data;
    int r[3] = {0, 0, 0}, c = ch;
    float mn[3], mx[3];
    if (file) {
        if ((status = read_vol(file, r, c, mn, mx, &data))) return false;
        if (c != ch) {
            set_last_error("volume channel count mismatch");
            status = DTRT_ERR_INVALID;
            return false;
        }
    } else {
        if (!arr || res[0] < 2 || res[1] < 2 || res[2] < 2) {
            set_last_error("heterogeneous medium without a density grid (>= 2 voxels per axis)");
            status = DTRT_ERR_INVALID;
            return false;
        }
        for (int i = 0; i < 3; ++i) { r[i] = res[i]; mn[i] = vmin[i]; mx[i] = vmax[i]; }
        data.assign(arr, arr + (size_t)r[0] * r[1] * r[2] * ch);
    }
    float maxv = 0.f;
    for (float &v : data) {  // gridvolume.h:128-131
        v = std::max(v, 0.0f);
        maxv = std::max(maxv, v);
    }
    double v2w[16], w2v[16];
    for (int i = 0; i < 16; ++i) v2w[i] = to_world[i];
    if (!invert4(v2w, w2v)) {
        set_last_error("singular medium to_world matrix");
        status = DTRT_ERR_INVALID;
        return false;
    }
    std::memset(&g, 0, sizeof(g));
    const float *dptr = nullptr;
    if (!bld.upload(data, &dptr)) {
        status = DTRT_ERR_CUDA;
        return false;
    }
    g.data = dptr;
    g.channels = ch;
    g.valid = 1;
    g.max_value = maxv;
    for (int i = 0; i < 3; ++i) {
        g.res[i] = r[i];
        g.mn[i] = mn[i];
        g.to_grid[i] = (float)((double)(r[i] - 1) / ((double)mx[i] - mn[i]));
    }
    for (int i = 0; i < 12; ++i) {
        g.w2v[i] = (float)w2v[i];
        g.v2w[i] = (float)v2w[i];
    }
    D3 c0 = xfm_point(v2w, {0.5 * (mn[0] + mx[0]), 0.5 * (mn[1] + mx[1]), 0.5 * (mn[2] + mx[2])});
    g.center[0] = (float)c0.x; g.center[1] = (float)c0.y; g.center[2] = (float)c0.z;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < 8; ++k) {  // gridvolume.h:135-141
        D3 p = xfm_point(v2w, {(k & 1) ? mx[0] : mn[0], (k & 2) ? mx[1] : mn[1], (k & 4) ? mx[2] : mn[2]});
        const double pv[3] = {p.x, p.y, p.z};
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], pv[a]); hi[a] = std::max(hi[a], pv[a]); }
    }
    for (int a = 0; a < 3; ++a) { g.lo[a] = (float)lo[a]; g.hi[a] = (float)hi[a]; }
    return true;
}

// fn(i) for i in [0, n) on up to 16 host threads in contiguous chunks of at least `grain`;
// fn writes only to slot i of preallocated outputs, so results do not depend on the threads.
template <class F>
void parallel_for(int n, int grain, F &&fn) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int nt = std::min(std::min((int)(hw ? hw : 1), 16), (n + grain - 1) / std::max(grain, 1));
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) fn(i);
        return;
    }
    const int chunk = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) {
        const int lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        try {
            th.emplace_back([&fn, lo, hi] {
                for (int i = lo; i < hi; ++i) fn(i);
            });
        } catch (...) {  // no thread to be had: run that chunk here
            for (int i = lo; i < hi; ++i) fn(i);
        }
    }
    for (int i = 0; i < std::min(n, chunk); ++i) fn(i);
    for (auto &x : th) x.join();
}

// Build the device scene from a description. With s->topo valid (a rebuild of a scene
// with the same triangles) the edge adjacency is taken from it and the BVH is refit unless
// `rebuild_bvh`; `info` (optional) reports which.
int build_scene(dtrt_scene *s, const dtrt_scene_desc *d, Builder &bld, bool rebuild_bvh, dtrt_update_stats *info) {
    const int N = d->nder;
    DevScene &ds = s->dev;
    std::memset(&ds, 0, sizeof(ds));
    ds.nder = N;
    ds.tracking_cap = 10000;
    SceneTopology &tp = s->topo;
    const bool cached = tp.valid;
    auto fail = [](const std::string &m) {
        set_last_error(m);
        return DTRT_ERR_INVALID;
    };
    if (d->num_shapes < 0 || d->num_bsdfs < 0 || d->num_emitters < 0 || d->num_phases < 0 || d->num_media < 0)
        return fail("negative element count");
    // ------------------------------------------------------------ camera, camera.cpp:8-38
    const dtrt_camera_desc &c = d->camera;
    if (c.width <= 0 || c.height <= 0 || !c.cam_to_world || !c.cam_to_ndc) return fail("invalid camera");
    double c2w[16], w2c[16], c2ndc[9], ndc2cam[9];
    for (int i = 0; i < 16; ++i) c2w[i] = c.cam_to_world[i];
    for (int i = 0; i < 9; ++i) c2ndc[i] = c.cam_to_ndc[i];
    if (!invert4(c2w, w2c) || !invert3(c2ndc, ndc2cam)) return fail("singular camera matrix");
    DevCamera &cam = ds.cam;
    cam.width = c.width;
    cam.height = c.height;
    cam.med_id = c.med_id;
    cam.clip_near = c.clip_near;
    cam.fov = (float)c2ndc[0];
    {
        const double aspect = (double)c.width / c.height, fov = (double)cam.fov;
        cam.inv_w = 1.0 / c.width;
        cam.inv_h = 1.0 / c.height;
        cam.ndc_ky = -2.0 / aspect;
        cam.plane_kx = 2.0 / fov;
        cam.plane_ky = -2.0 / (aspect * fov);
    }
    const bool cropped = c.crop_width > 0 && c.crop_height > 0;
    cam.crop_x = cropped ? c.crop_offset_x : 0;
    cam.crop_y = cropped ? c.crop_offset_y : 0;
    cam.crop_w = cropped ? c.crop_width : 0;
    cam.crop_h = cropped ? c.crop_height : 0;
    if (cropped && (cam.crop_x < 0 || cam.crop_y < 0 || cam.crop_x + cam.crop_w > c.width || cam.crop_y + cam.crop_h > c.height))
        return fail("crop rectangle outside the image");
    for (int i = 0; i < 12; ++i) cam.c2w[i] = (float)c2w[i];
    for (int i = 0; i < 9; ++i) cam.ndc2cam[i] = (float)ndc2cam[i];
    D3 fr[3] = {{c2w[0], c2w[4], c2w[8]}, {c2w[1], c2w[5], c2w[9]}, {c2w[2], c2w[6], c2w[10]}};
    const D3 cpos = {c2w[3], c2w[7], c2w[11]};
    cam.cpos[0] = (float)cpos.x; cam.cpos[1] = (float)cpos.y; cam.cpos[2] = (float)cpos.z;
    for (int k = 0; k < 3; ++k) { cam.cframe[k][0] = (float)fr[k].x; cam.cframe[k][1] = (float)fr[k].y; cam.cframe[k][2] = (float)fr[k].z; }
    HV cposd, cfd[3];  // dual camera position and frame for the primary-edge projection
    cposd = {HD(cpos.x), HD(cpos.y), HD(cpos.z)};
    for (int k = 0; k < 3; ++k) cfd[k] = {HD(fr[k].x), HD(fr[k].y), HD(fr[k].z)};
    if (c.med_id >= d->num_media) return fail("camera medium id out of range");
    if (c.velocities) {  // camera.cpp:103-111: translations then rotation axes
        for (int j = 0; j < N; ++j) {
            const float *dx = c.velocities + 3 * j, *dw = c.velocities + 3 * (N + j);
            const D3 w = {dw[0], dw[1], dw[2]};
            for (int a = 0; a < 3; ++a) { cam.d_cpos[j][a] = dx[a]; cposd[a].d[j] = dx[a]; }
            for (int k = 0; k < 3; ++k) {
                const D3 g = dcross(w, fr[k]);
                cam.d_cframe[j][k][0] = (float)g.x; cam.d_cframe[j][k][1] = (float)g.y; cam.d_cframe[j][k][2] = (float)g.z;
                cfd[k].x.d[j] = g.x; cfd[k].y.d[j] = g.y; cfd[k].z.d[j] = g.z;
            }
        }
    }
    // ------------------------------------------------------------ shapes, shape.cpp:10-52
    std::vector<DevShape> shapes(d->num_shapes);
    std::vector<float4> verts, normals, facen;
    std::vector<float> vder, nder_, fder;
    std::vector<int4> tris;
    std::vector<std::vector<HV>> vad(d->num_shapes);  // dual vertices per shape
    bool any_vel = false, any_normals = false;
    for (int i = 0; i < d->num_shapes; ++i) {
        any_vel = any_vel || d->shapes[i].velocities;
        any_normals = any_normals || d->shapes[i].normals;
    }
    int vtot = 0, ttot = 0;
    for (int si = 0; si < d->num_shapes; ++si) {
        const dtrt_shape_desc &sd = d->shapes[si];
        if (!sd.vertices || !sd.indices || sd.num_vertices <= 0 || sd.num_triangles <= 0) return fail("shape without geometry");
        if (sd.bsdf_id < 0 || sd.bsdf_id >= d->num_bsdfs) return fail("shape bsdf_id out of range");
        if (sd.light_id >= d->num_emitters || sd.med_int_id >= d->num_media || sd.med_ext_id >= d->num_media)
            return fail("shape light/medium id out of range");
        DevShape &sh = shapes[si];
        sh.vert_off = vtot;
        sh.tri_off = ttot;
        sh.nv = sd.num_vertices;
        sh.nt = sd.num_triangles;
        sh.light_id = sd.light_id;
        sh.bsdf_id = sd.bsdf_id;
        sh.med_int = sd.med_int_id;
        sh.med_ext = sd.med_ext_id;
        sh.has_normals = sd.normals != nullptr;
        vad[si].resize(sh.nv);
        for (int v = 0; v < sh.nv; ++v) {
            const float *p = sd.vertices + 3 * v;
            if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2])) return fail("non-finite vertex");
            verts.push_back(make_float4(p[0], p[1], p[2], 0.f));
            vad[si][v] = {HD(p[0]), HD(p[1]), HD(p[2])};
            if (sd.normals) {
                D3 n = dnormalize({sd.normals[3 * v], sd.normals[3 * v + 1], sd.normals[3 * v + 2]});
                normals.push_back(make_float4((float)n.x, (float)n.y, (float)n.z, 0.f));
            } else if (any_normals) {
                normals.push_back(make_float4(0.f, 0.f, 1.f, 0.f));
            }
            for (int j = 0; j < N && any_vel; ++j) {
                float g[3] = {0, 0, 0};
                if (sd.velocities) {
                    const float *q = sd.velocities + 3 * ((size_t)j * sh.nv + v);
                    g[0] = q[0]; g[1] = q[1]; g[2] = q[2];
                }
                for (int a = 0; a < 3; ++a) { vder.push_back(g[a]); vad[si][v][a].d[j] = g[a]; }
            }
            for (int j = 0; j < N && any_normals; ++j) {
                float g[3] = {0, 0, 0};
                if (sd.velocities && sd.normals) {  // shape.cpp:45: one fixed offset for every slot
                    const float *q = sd.velocities + (size_t)sh.nv * 3 * N + 3 * v;
                    g[0] = q[0]; g[1] = q[1]; g[2] = q[2];
                }
                for (int a = 0; a < 3; ++a) nder_.push_back(g[a]);
            }
        }
        for (int t = 0; t < sh.nt; ++t) {
            const int *f = sd.indices + 3 * t;
            for (int k = 0; k < 3; ++k)
                if (f[k] < 0 || f[k] >= sh.nv) return fail("triangle index out of range");
            tris.push_back(make_int4(vtot + f[0], vtot + f[1], vtot + f[2], si));
        }
        // face normals with derivatives, shape.cpp:109-126 (one slot per triangle, host threads)
        facen.resize((size_t)ttot + sh.nt);
        if (any_vel) fder.resize(((size_t)ttot + sh.nt) * N * 3);
        const std::vector<HV> &vs = vad[si];
        parallel_for(sh.nt, 2048, [&](int t) {
            const int *f = sd.indices + 3 * t;
            HV n = hcross(vs[f[1]] - vs[f[0]], vs[f[2]] - vs[f[0]]);
            HD len = hsqrt(hdot(n, n));
            if (len.v >= 1e-7) n = n / len;
            const size_t ft = (size_t)ttot + t;
            facen[ft] = make_float4((float)n.x.v, (float)n.y.v, (float)n.z.v, 0.f);
            for (int j = 0; j < N && any_vel; ++j) {
                fder[(ft * N + j) * 3 + 0] = (float)n.x.d[j];
                fder[(ft * N + j) * 3 + 1] = (float)n.y.d[j];
                fder[(ft * N + j) * 3 + 2] = (float)n.z.d[j];
            }
        });
        vtot += sh.nv;
        ttot += sh.nt;
    }
    ds.num_shapes = d->num_shapes;
    ds.num_verts = vtot;
    ds.num_tris = ttot;
    ds.moving_geometry = any_vel ? 1 : 0;
    // ------------------------------------------------------------ edges, shape.cpp:254-300
    std::vector<DevEdge> edges;
    std::vector<double> edge_cdf;
    s->shape_edge_len.assign(d->num_shapes, 0.f);
    s->shape_skip.assign(d->num_shapes, 0);
    if (!cached) {  // edge adjacency from the triangle lists: sorted unique vertex pairs and their faces
        tp.adj.clear();
        tp.adj_off.assign(1, 0);
        // each triangle side as (sorted vertex pair, face), stably sorted by the pair: the runs
        // are the edges in increasing (a, b) order, their faces in triangle order
        std::vector<std::pair<uint64_t, int>> he;
        for (int si = 0; si < d->num_shapes; ++si) {
            const DevShape &sh = shapes[si];
            he.resize(3 * (size_t)sh.nt);
            for (int t = 0; t < sh.nt; ++t) {
                const int4 tr = tris[sh.tri_off + t];
                const int ids[3] = {tr.x - sh.vert_off, tr.y - sh.vert_off, tr.z - sh.vert_off};
                for (int e = 0; e < 3; ++e) {
                    const int a = std::min(ids[e], ids[(e + 1) % 3]), b = std::max(ids[e], ids[(e + 1) % 3]);
                    he[3 * (size_t)t + e] = {((uint64_t)(uint32_t)a << 32) | (uint32_t)b, t};
                }
            }
            std::stable_sort(he.begin(), he.end(), [](const std::pair<uint64_t, int> &x, const std::pair<uint64_t, int> &y) {
                return x.first < y.first;
            });
            for (size_t i = 0; i < he.size();) {
                size_t j = i + 1;
                while (j < he.size() && he[j].first == he[i].first) ++j;
                if (j - i > 2) return fail("non-manifold mesh: an edge is shared by more than 2 faces");
                if (j - i == 2 && he[i].second == he[i + 1].second) return fail("duplicated faces");
                tp.adj.push_back(make_int4((int)(he[i].first >> 32), (int)(he[i].first & 0xffffffffu), he[i].second,
                                           j - i == 2 ? he[i + 1].second : -1));
                i = j;
            }
            tp.adj_off.push_back((int)tp.adj.size());
        }
    }
    for (int si = 0; si < d->num_shapes; ++si) {
        DevShape &sh = shapes[si];
        sh.edge_off = (int)edges.size();
        sh.edge_cdf_off = (int)edge_cdf.size();
        double sum = 0;
        std::vector<double> lens;
        for (int k = tp.adj_off[si]; k < tp.adj_off[si + 1]; ++k) {
            const int4 ad = tp.adj[k];
            const float4 va = verts[sh.vert_off + ad.x], vb = verts[sh.vert_off + ad.y];
            const double len = dnorm({(double)va.x - vb.x, (double)va.y - vb.y, (double)va.z - vb.z});
            DevEdge e{sh.vert_off + ad.x, sh.vert_off + ad.y, sh.tri_off + ad.z, -1, si, (float)len};
            if (ad.w >= 0) {
                const float4 n0 = facen[sh.tri_off + ad.z], n1 = facen[sh.tri_off + ad.w];
                const double cc = (double)n0.x * n1.x + (double)n0.y * n1.y + (double)n0.z * n1.z;
                if (cc < -1.0 + 1e-7) return fail("inconsistent normal orientation");
                if (!(cc < 1.0 - 1e-7)) continue;  // flat edge
                e.f1 = sh.tri_off + ad.w;
            }
            edges.push_back(e);
            lens.push_back(len);
            sum += len;
        }
        sh.num_edges = (int)lens.size();
        edge_cdf.push_back(0.0);
        double acc = 0;
        for (size_t k = 0; k < lens.size(); ++k) {
            acc += lens[k];
            // non-negative entries (no NaN): the device search compares their bit patterns
            edge_cdf.push_back(k + 1 == lens.size() ? 1.0 : (sum > 0 ? acc / sum : 0.0));
        }
        s->shape_edge_len[si] = (float)sum;
        s->shape_skip[si] = 0;
    }
    // ------------------------------------------------------------ BVH
    {
        std::vector<float> tv((size_t)ttot * 9);
        for (int t = 0; t < ttot; ++t) {
            const int4 tr = tris[t];
            const float4 a = verts[tr.x], b = verts[tr.y], cc = verts[tr.z];
            const float vv[9] = {a.x, a.y, a.z, b.x, b.y, b.z, cc.x, cc.y, cc.z};
            std::memcpy(&tv[9 * (size_t)t], vv, sizeof(vv));
        }
        // refit while the surface-area cost stays within kRefitCostLimit of the cost at the
        // last full build; past it (or when asked) build the tree again. The cost is relative
        // to the root box, so shape changes that a new tree cannot undo (a stretch) raise it
        // too: on a 5,120-triangle sphere a 3x stretch gave 1.9x for the refit tree and the
        // same cost for a new one, while folds that interleave distant parts gave 3-6x, where
        // a new tree halves the cost.
        constexpr double kRefitCostLimit = 2.0;
        const auto tb = std::chrono::steady_clock::now();
        const int choice = bvh_builder_setting();
        bool on_device = choice == DTRT_BVH_DEVICE || (choice == DTRT_BVH_AUTO && ttot >= DTRT_BVH_DEVICE_MIN_TRIS);
        if (on_device && ttot >= 2) {
            DeviceBvh db;
            std::string err;
            const int r = build_bvh_device(tv, ttot, db, err);
            if (r == 2) {
                set_last_error(err);
                return DTRT_ERR_CUDA;
            }
            on_device = r == 0;
            if (on_device) {
                tp.bvh = BvhBuildOut();  // updates build this tree again instead of refitting a host copy
                tp.sah_build = 0.0;
                ds.num_nodes = db.num_nodes;
                bld.adopt(db.nodes, (size_t)db.num_nodes * sizeof(BvhNode), &ds.nodes);
                bld.adopt(db.leaf_tris, db.leaf_tris_bytes, &ds.leaf_tris);
                const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
                s->bvh_info = dtrt_bvh_info{DTRT_BVH_DEVICE, 0, db.num_nodes, db.max_depth, ms};
                if (info) {
                    info->bvh_refit = 0;
                    info->sah_ratio = 1.f;
                    info->ms_bvh = ms;
                }
            }
        } else {
            on_device = false;
        }
        bool refit = !on_device && cached && !rebuild_bvh && !tp.bvh.nodes.empty();
        double ratio = 1.0;
        if (!on_device) {
        if (refit) {
            refit_bvh(tv, tp.bvh);
            ratio = tp.sah_build > 0.0 ? bvh_sah_cost(tp.bvh) / tp.sah_build : 1.0;
            if (!(ratio <= kRefitCostLimit)) refit = false;
        }
        if (!refit) {
            build_bvh(tv, ttot, tp.bvh);
            tp.sah_build = bvh_sah_cost(tp.bvh);
        }
        if (info) {
            info->bvh_refit = refit ? 1 : 0;
            info->sah_ratio = (float)ratio;
            info->ms_bvh = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
        }
        ds.num_nodes = (int)tp.bvh.nodes.size();
        if (!bld.upload(tp.bvh.nodes, &ds.nodes) || !bld.upload(tp.bvh.leaf_tris, &ds.leaf_tris)) return DTRT_ERR_CUDA;
        s->bvh_info = dtrt_bvh_info{DTRT_BVH_HOST, refit ? 1 : 0, ds.num_nodes, tp.bvh.max_depth,
                                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count()};
        }
    }
    // ------------------------------------------------------------ materials
    std::vector<DevBsdf> bsdfs(d->num_bsdfs);
    for (int b = 0; b < d->num_bsdfs; ++b) {
        const dtrt_bsdf_desc &bd = d->bsdfs[b];
        DevBsdf &o = bsdfs[b];
        std::memset(&o, 0, sizeof(o));
        if (bd.type < 0 || bd.type > 3) return fail("unknown BSDF type");
        o.type = bd.type;
        for (int a = 0; a < 3; ++a) { o.diffuse[a] = bd.diffuse[a]; o.specular[a] = bd.specular[a]; }
        o.exponent = bd.exponent;
        o.alpha = std::max(bd.alpha, 1e-4f);  // microfacet.h:11-14 clamps the value only
        o.eta = bd.int_ior / bd.ext_ior;
        o.inv_eta = 1.0f / o.eta;
        if (bd.type == BSDF_PHONG) {  // phong.h:9-15
            double v0 = ((double)bd.diffuse[0] + bd.diffuse[1] + bd.diffuse[2]) / 3.0;
            double v1 = ((double)bd.specular[0] + bd.specular[1] + bd.specular[2]) / 3.0;
            o.spec_weight = (float)(v1 / (v0 + v1));
        }
        for (int j = 0; j < N; ++j) {
            for (int a = 0; a < 3; ++a) {
                if (bd.d_diffuse) o.d_diffuse[j][a] = bd.d_diffuse[3 * j + a];
                if (bd.d_specular) o.d_specular[j][a] = bd.d_specular[3 * j + a];
            }
            if (bd.d_exponent) o.d_exponent[j] = bd.d_exponent[j];
            if (bd.d_alpha) o.d_alpha[j] = bd.d_alpha[j];
            if (bd.d_eta) o.d_eta[j] = bd.d_eta[j];
            o.d_inv_eta[j] = -o.d_eta[j] / (o.eta * o.eta);
            for (int a = 0; a < 3; ++a) o.has_der |= (o.d_diffuse[j][a] != 0.f) | (o.d_specular[j][a] != 0.f);
            o.has_der |= (o.d_exponent[j] != 0.f) | (o.d_alpha[j] != 0.f) | (o.d_eta[j] != 0.f);
        }
    }
    std::vector<DevPhase> phases(d->num_phases);
    for (int p = 0; p < d->num_phases; ++p) {
        std::memset(&phases[p], 0, sizeof(DevPhase));
        phases[p].type = d->phases[p].type;
        phases[p].g = d->phases[p].g;
        if (d->phases[p].d_g)
            for (int j = 0; j < N; ++j) {
                phases[p].d_g[j] = d->phases[p].d_g[j];
                phases[p].has_der |= phases[p].d_g[j] != 0.f;
            }
    }
    std::vector<DevEmitter> ems(d->num_emitters);
    for (int e = 0; e < d->num_emitters; ++e) {
        const dtrt_emitter_desc &ed = d->emitters[e];
        DevEmitter &o = ems[e];
        std::memset(&o, 0, sizeof(o));
        if (ed.shape_id < 0 || ed.shape_id >= d->num_shapes) return fail("emitter shape_id out of range");
        o.type = ed.type;
        o.shape_id = ed.shape_id;
        o.two_sided = ed.two_sided;
        o.kappa = ed.kappa;
        for (int a = 0; a < 3; ++a) o.intensity[a] = ed.intensity[a];
        for (int j = 0; j < N; ++j) {
            for (int a = 0; a < 3; ++a)
                if (ed.d_intensity) o.d_intensity[j][a] = ed.d_intensity[3 * j + a];
            if (ed.d_kappa) o.d_kappa[j] = ed.d_kappa[j];
        }
    }
    std::vector<DevMedium> media(d->num_media);
    for (int mi = 0; mi < d->num_media; ++mi) {
        const dtrt_medium_desc &md = d->media[mi];
        DevMedium &o = media[mi];
        std::memset(&o, 0, sizeof(o));
        o.grad_off = -1;
        if (md.phase_id < 0 || md.phase_id >= d->num_phases) return fail("medium phase_id out of range");
        o.type = md.type;
        o.phase_id = md.phase_id;
        for (int a = 0; a < 3; ++a) o.albedo[a] = md.albedo[a];
        for (int j = 0; j < N; ++j)
            for (int a = 0; a < 3; ++a)
                if (md.d_albedo) o.d_albedo[j][a] = md.d_albedo[3 * j + a];
        if (md.type == MEDIUM_HOMOGENEOUS) {  // homogeneous.h:13-27
            o.sigma_t = md.sigma_t;
            for (int j = 0; j < N; ++j)
                if (md.d_sigma_t) o.d_sigma_t[j] = md.d_sigma_t[j];
            for (int a = 0; a < 3; ++a) o.sigma_s[a] = md.sigma_t * md.albedo[a];
            o.sampling_weight = std::max(md.albedo[0], std::max(md.albedo[1], md.albedo[2]));
        } else if (md.type == MEDIUM_HETEROGENEOUS) {  // heterogeneous.h:13-75
            int st = DTRT_OK;
            if (!load_grid(o.density, bld, md.density_file, md.density, md.res, 1, md.vol_min, md.vol_max, md.to_world, st))
                return st;
            if (md.albedo_file || md.albedo_grid) {
                if (!load_grid(o.albedo_vol, bld, md.albedo_file, md.albedo_grid, md.albedo_res, 3, md.albedo_min,
                               md.albedo_max, md.to_world, st))
                    return st;
                for (int a = 0; a < 3; ++a) o.albedo[a] = 0.f;  // m_albedo stays zero with an albedo grid
                std::memset(o.d_albedo, 0, sizeof(o.d_albedo));
            }
            o.scale = md.density_scale;
            for (int j = 0; j < N; ++j) {
                if (md.d_density_scale) o.d_scale[j] = md.d_density_scale[j];
                for (int a = 0; a < 3; ++a) {
                    if (md.trans_velocities) o.density.trans_vel[j][a] = md.trans_velocities[3 * j + a];
                    if (md.rot_velocities) o.density.rot_vel[j][a] = md.rot_velocities[3 * j + a];
                    if (o.density.trans_vel[j][a] != 0.f || o.density.rot_vel[j][a] != 0.f) o.density.moving = 1;
                }
            }
            if (!(o.scale > 0.f) || !(o.density.max_value > 0.f)) return fail("heterogeneous medium with zero majorant");
            o.max_inv_density = (float)(1.0 / ((double)o.scale * o.density.max_value));
            o.grad_off = s->density_voxels;
            s->density_voxels += (long long)o.density.res[0] * o.density.res[1] * o.density.res[2];
        } else {
            return fail("unknown medium type");
        }
        if (cached && (tp.media_type[mi] != o.type ||
                       (o.type == MEDIUM_HETEROGENEOUS && (tp.media_res[3 * mi] != o.density.res[0] ||
                                                           tp.media_res[3 * mi + 1] != o.density.res[1] ||
                                                           tp.media_res[3 * mi + 2] != o.density.res[2]))))
            return fail("scene update: a medium changed its type or grid resolution");
    }
    for (const DevMedium &m : media) ds.has_grid_media |= m.type == MEDIUM_HETEROGENEOUS ? 1 : 0;
    // ------------------------------------------------------------ light tables, scene.cpp:45-98
    std::vector<float> light_pmf(d->num_emitters), light_cdf(d->num_emitters), light_area(d->num_emitters), area_cdf;
    std::vector<int> area_begin(d->num_emitters);
    double total = 0;
    std::vector<double> pmf(d->num_emitters);
    for (int l = 0; l < d->num_emitters; ++l) {
        const DevShape &sh = shapes[ems[l].shape_id];
        area_begin[l] = (int)area_cdf.size();
        std::vector<double> cum;
        double sum = 0;
        for (int t = 0; t < sh.nt; ++t) {
            const int4 tr = tris[sh.tri_off + t];
            const float4 a = verts[tr.x], b = verts[tr.y], cc = verts[tr.z];
            const D3 e1 = {(double)b.x - a.x, (double)b.y - a.y, (double)b.z - a.z};
            const D3 e2 = {(double)cc.x - a.x, (double)cc.y - a.y, (double)cc.z - a.z};
            sum += 0.5 * dnorm(dcross(e1, e2));
            cum.push_back(sum);
        }
        for (double v : cum) area_cdf.push_back((float)(v / sum));
        light_area[l] = (float)sum;
        const double lum = 0.212671 * ems[l].intensity[0] + 0.715160 * ems[l].intensity[1] + 0.072169 * ems[l].intensity[2];
        pmf[l] = sum * lum * 3.14159265358979323846;
        total += pmf[l];
    }
    if (d->num_emitters > 0) {
        if (!(total > 0)) return fail("emitters carry no power");
        double acc = 0;
        for (int l = 0; l < d->num_emitters; ++l) {
            light_pmf[l] = (float)(pmf[l] / total);
            acc += pmf[l] / total;
            light_cdf[l] = (float)acc;
        }
    }
    // ------------------------------------------------------------ primary edges, edge_manager.cpp:6-110
    std::vector<DevPrimaryEdge> pedges;
    std::vector<double> plen;
    std::vector<float> pjac;
    std::vector<int> pverts;
    const double aspect = (double)c.width / c.height, fov = c2ndc[0];
    // every edge is projected on its own (host threads, one output slot per candidate
    // edge), then the kept ones are gathered in edge order: the same arrays as a serial loop
    struct PEdgeOut {
        DevPrimaryEdge pe;
        float jac[24];
        bool ok;
    };
    std::vector<int2> cand;  // (shape, edge of the shape)
    for (int si = 0; si < d->num_shapes; ++si) {
        const DevShape &sh = shapes[si];
        if (bsdfs[sh.bsdf_id].type == BSDF_NULL && sh.light_id < 0) continue;
        for (int k = 0; k < sh.num_edges; ++k) cand.push_back(make_int2(si, k));
    }
    std::vector<PEdgeOut> pout(cand.size());
    parallel_for((int)cand.size(), 1024, [&](int ci) {
        PEdgeOut &po = pout[ci];
        po.ok = false;
        const int si = cand[ci].x;
        const DevShape &sh = shapes[si];
        {
            const DevEdge &e = edges[sh.edge_off + cand[ci].y];
            // silhouette test against the camera position (shape.cpp:302-335)
            if (e.f1 >= 0) {
                const float4 a = verts[e.v0], b = verts[e.v1];
                const D3 v0 = {a.x, a.y, a.z}, v1 = {b.x, b.y, b.z};
                bool ff[2];
                for (int q = 0; q < 2; ++q) {
                    const int4 tr = tris[q == 0 ? e.f0 : e.f1];
                    const int ids[3] = {tr.x, tr.y, tr.z};
                    ff[q] = false;
                    for (int i = 0; i < 3; ++i)
                        if (ids[i] != e.v0 && ids[i] != e.v1) {
                            const float4 vv = verts[ids[i]];
                            const D3 v = {vv.x, vv.y, vv.z};
                            const D3 n = q == 0 ? dnormalize(dcross(sub(v0, v), sub(v1, v))) : dnormalize(dcross(sub(v1, v), sub(v0, v)));
                            ff[q] = ddot(n, sub(cpos, v)) > 0.0;
                            break;
                        }
                }
                const int sil = ff[0] != ff[1] ? 2 : (sh.has_normals ? 0 : 1);
                if (sil <= 0) return;
            }
            HV v0 = vad[si][e.v0 - sh.vert_off], v1 = vad[si][e.v1 - sh.vert_off];
            const double cn[3] = {fr[2].x, fr[2].y, fr[2].z};
            const double z0 = (v0.x.v - cpos.x) * cn[0] + (v0.y.v - cpos.y) * cn[1] + (v0.z.v - cpos.z) * cn[2];
            const double z1 = (v1.x.v - cpos.x) * cn[0] + (v1.y.v - cpos.y) * cn[1] + (v1.z.v - cpos.z) * cn[2];
            const double near = c.clip_near;
            if (z0 < near && z1 < near) return;
            if (z0 < near) v0 = v0 + (v1 - v0) * ((near - z0) / (z1 - z0));
            else if (z1 < near) v1 = v1 + (v0 - v1) * ((near - z1) / (z0 - z1));
            D3 v0l = xfm_point(w2c, val(v0)), v1l = xfm_point(w2c, val(v1));
            v0 = (v0 - cposd) / hdot(v0 - cposd, cfd[2]);
            v1 = (v1 - cposd) / hdot(v1 - cposd, cfd[2]);
            v0 = {hdot(v0, cfd[0]), hdot(v0, cfd[1]), hdot(v0, cfd[2])};
            v1 = {hdot(v1, cfd[0]), hdot(v1, cfd[1]), hdot(v1, cfd[2])};
            HD r0[2] = {v0.x * (fov * 0.5) + HD(0.5), v0.y * (fov * -0.5 * aspect) + HD(0.5)};
            HD r1[2] = {v1.x * (fov * 0.5) + HD(0.5), v1.y * (fov * -0.5 * aspect) + HD(0.5)};
            double xmin = 0, xmax = 1, ymin = 0, ymax = 1;
            if (cropped) {
                xmin = (double)((float)c.crop_offset_x / c.width);
                xmax = (double)((float)(c.crop_offset_x + c.crop_width) / c.width);
                ymin = (double)((float)c.crop_offset_y / c.height);
                ymax = (double)((float)(c.crop_offset_y + c.crop_height) / c.height);
            }
            HD c0[2], c1[2];
            if (!clip_line(r0, r1, c0, c1, xmin, xmax, ymin, ymax)) return;
            D3 v0p = val(v0), v1p = val(v1);
            const D3 t0v = v0l, t1v = v1l;
            const D3 dv = sub(val(v1), val(v0));
            if (std::hypot(r0[0].v - c0[0].v, r0[1].v - c0[1].v) > 1e-7) {
                const D3 pc = {(c0[0].v - 0.5) * 2.0 / fov, (c0[1].v - 0.5) * (-2.0) / (aspect * fov), 1.0};
                const double t0 = dnorm(sub(pc, val(v0))) / dnorm(dv);
                v0p = {val(v0).x + t0 * dv.x, val(v0).y + t0 * dv.y, val(v0).z + t0 * dv.z};
                const double t1 = intersection_in_tri(val(v0), val(v1), t0v, t1v, t0);
                v0l = {t0v.x + t1 * (t1v.x - t0v.x), t0v.y + t1 * (t1v.y - t0v.y), t0v.z + t1 * (t1v.z - t0v.z)};
            }
            if (std::hypot(r1[0].v - c1[0].v, r1[1].v - c1[1].v) > 1e-7) {
                const D3 pc = {(c1[0].v - 0.5) * 2.0 / fov, (c1[1].v - 0.5) * (-2.0) / (aspect * fov), 1.0};
                const double t0 = dnorm(sub(pc, val(v0))) / dnorm(dv);
                v1p = {val(v0).x + t0 * dv.x, val(v0).y + t0 * dv.y, val(v0).z + t0 * dv.z};
                const double t1 = intersection_in_tri(val(v0), val(v1), t0v, t1v, t0);
                v1l = {t0v.x + t1 * (t1v.x - t0v.x), t0v.y + t1 * (t1v.y - t0v.y), t0v.z + t1 * (t1v.z - t0v.z)};
            }
            DevPrimaryEdge pe;
            std::memset(&pe, 0, sizeof(pe));
            pe.v0s[0] = c0[0].v * c.width; pe.v0s[1] = c0[1].v * c.height;
            pe.v1s[0] = c1[0].v * c.width; pe.v1s[1] = c1[1].v * c.height;
            for (int j = 0; j < N; ++j) {
                pe.d0[j][0] = (float)(c0[0].d[j] * c.width); pe.d0[j][1] = (float)(c0[1].d[j] * c.height);
                pe.d1[j][0] = (float)(c1[0].d[j] * c.width); pe.d1[j][1] = (float)(c1[1].d[j] * c.height);
            }
            const double *srcs[4] = {&v0p.x, &v1p.x, &v0l.x, &v1l.x};
            double *dsts[4] = {pe.v0p, pe.v1p, pe.v0c, pe.v1c};
            for (int q = 0; q < 4; ++q)
                for (int a = 0; a < 3; ++a) dsts[q][a] = srcs[q][a];
            {
                const double nx = pe.v1s[1] - pe.v0s[1], ny = pe.v0s[0] - pe.v1s[0], nl = std::sqrt(nx * nx + ny * ny);
                pe.n[0] = nx / nl;
                pe.n[1] = ny / nl;
                pe.inv_lenp = 1.0 / dnorm(sub(v1p, v0p));
                pe.cb = dnorm(v0p) / dnorm(v0l);
                pe.cc = dnorm(v1p) / dnorm(v1l);
            }
            po.pe = pe;
            // Jacobian of the two clipped screen endpoints (pixels) w.r.t. the edge's vertex
            // positions (dual slots 0-2: v0, 3-5: v1) for a static camera: the same near-plane
            // clip, projection and image clip as above, for the vertex-position adjoint
            {
                const HV o0 = vad[si][e.v0 - sh.vert_off], o1 = vad[si][e.v1 - sh.vert_off];
                HV a = {HD(o0.x.v), HD(o0.y.v), HD(o0.z.v)}, b = {HD(o1.x.v), HD(o1.y.v), HD(o1.z.v)};
                for (int q = 0; q < 3; ++q) { a[q].d[q] = 1.0; b[q].d[3 + q] = 1.0; }
                if (z0 < near) a = a + (b - a) * ((near - z0) / (z1 - z0));
                else if (z1 < near) b = b + (a - b) * ((near - z1) / (z0 - z1));
                const HV cp0 = {HD(cpos.x), HD(cpos.y), HD(cpos.z)};
                const HV cf0[3] = {{HD(fr[0].x), HD(fr[0].y), HD(fr[0].z)}, {HD(fr[1].x), HD(fr[1].y), HD(fr[1].z)},
                                   {HD(fr[2].x), HD(fr[2].y), HD(fr[2].z)}};
                a = (a - cp0) / hdot(a - cp0, cf0[2]);
                b = (b - cp0) / hdot(b - cp0, cf0[2]);
                a = {hdot(a, cf0[0]), hdot(a, cf0[1]), hdot(a, cf0[2])};
                b = {hdot(b, cf0[0]), hdot(b, cf0[1]), hdot(b, cf0[2])};
                HD q0[2] = {a.x * (fov * 0.5) + HD(0.5), a.y * (fov * -0.5 * aspect) + HD(0.5)};
                HD q1[2] = {b.x * (fov * 0.5) + HD(0.5), b.y * (fov * -0.5 * aspect) + HD(0.5)};
                HD k0[2], k1[2];
                const bool vis = clip_line(q0, q1, k0, k1, xmin, xmax, ymin, ymax);
                for (int q = 0; q < 6; ++q) {
                    po.jac[q] = vis ? (float)(k0[0].d[q] * c.width) : 0.f;
                    po.jac[6 + q] = vis ? (float)(k0[1].d[q] * c.height) : 0.f;
                    po.jac[12 + q] = vis ? (float)(k1[0].d[q] * c.width) : 0.f;
                    po.jac[18 + q] = vis ? (float)(k1[1].d[q] * c.height) : 0.f;
                }
                po.ok = true;
            }
        }
    });
    for (size_t ci = 0; ci < cand.size(); ++ci) {
        const PEdgeOut &po = pout[ci];
        if (!po.ok) continue;
        const DevEdge &e = edges[shapes[cand[ci].x].edge_off + cand[ci].y];
        pedges.push_back(po.pe);
        plen.push_back(std::hypot(po.pe.v0s[0] - po.pe.v1s[0], po.pe.v0s[1] - po.pe.v1s[1]));
        pjac.insert(pjac.end(), po.jac, po.jac + 24);
        pverts.push_back(e.v0);
        pverts.push_back(e.v1);
    }
    std::vector<double> pcdf;
    double psum = 0;
    for (double v : plen) psum += v;
    if (!pedges.empty()) {
        pcdf.push_back(0.0);
        double acc = 0;
        for (size_t k = 0; k < plen.size(); ++k) {
            acc += plen[k];
            pcdf.push_back(k + 1 == plen.size() ? 1.0 : (psum > 0 ? acc / psum : 0.0));
        }
    }
    ds.num_pedges = psum > 0 ? (int)pedges.size() : 0;
    ds.pedge_sum = psum;
    // ------------------------------------------------------------ upload
    if (!bld.upload(shapes, &ds.shapes) || !bld.upload(verts, &ds.verts) || !bld.upload(vder, &ds.vert_der) ||
        !bld.upload(normals, &ds.normals) || !bld.upload(nder_, &ds.normal_der) || !bld.upload(tris, &ds.tris) ||
        !bld.upload(facen, &ds.face_n) || !bld.upload(fder, &ds.face_n_der) || !bld.upload(bsdfs, &ds.bsdfs) ||
        !bld.upload(phases, &ds.phases) || !bld.upload(ems, &ds.emitters) || !bld.upload(media, &ds.media) ||
        !bld.upload(light_cdf, &ds.light_cdf) || !bld.upload(light_pmf, &ds.light_pmf) ||
        !bld.upload(light_area, &ds.light_area) || !bld.upload(area_cdf, &ds.area_cdf) ||
        !bld.upload(area_begin, &ds.area_cdf_begin) || !bld.upload(edges, &ds.edges) ||
        !bld.upload(edge_cdf, &ds.edge_cdf) || !bld.upload(pedges, &ds.pedges) || !bld.upload(pcdf, &ds.pedge_cdf) ||
        !bld.upload(pjac, &ds.pedge_jac) || !bld.upload(pverts, &ds.pedge_verts) ||
        !bld.upload(std::vector<double>(d->num_shapes + 1, 0.0), &ds.shape_edge_cdf))  // filled by set_edge_weights
        return DTRT_ERR_CUDA;
    if (!any_normals) ds.normal_der = nullptr;
    ds.num_bsdfs = d->num_bsdfs;
    ds.num_phases = d->num_phases;
    ds.num_emitters = d->num_emitters;
    ds.num_media = d->num_media;
    s->media_host = media;
    s->dgrid_bufs.assign(d->num_media, nullptr);
    s->num_shapes = d->num_shapes;
    for (int si = 0; si < d->num_shapes; ++si)
        s->shape_skip[si] = (bsdfs[shapes[si].bsdf_id].type == BSDF_NULL && shapes[si].light_id < 0) ? 1 : 0;
    if (!cached) {
        tp.shape_nv.resize(d->num_shapes);
        tp.shape_nt.resize(d->num_shapes);
        tp.indices.clear();
        for (int si = 0; si < d->num_shapes; ++si) {
            tp.shape_nv[si] = shapes[si].nv;
            tp.shape_nt[si] = shapes[si].nt;
            tp.indices.insert(tp.indices.end(), d->shapes[si].indices, d->shapes[si].indices + 3 * (size_t)shapes[si].nt);
        }
        tp.media_type.resize(d->num_media);
        tp.media_res.assign(3 * (size_t)d->num_media, 0);
        for (int mi = 0; mi < d->num_media; ++mi) {
            tp.media_type[mi] = media[mi].type;
            for (int a = 0; a < 3 && media[mi].type == MEDIUM_HETEROGENEOUS; ++a) tp.media_res[3 * mi + a] = media[mi].density.res[a];
        }
        tp.valid = true;
    }
    return DTRT_OK;
}

// Same triangles as the scene was built with: derivative width, shape count, per shape
// vertex and triangle counts and the index lists; the same number of media.
int check_same_topology(const dtrt_scene *s, const dtrt_scene_desc *d) {
    const SceneTopology &tp = s->topo;
    auto fail = [](const std::string &m) {
        set_last_error("scene update: " + m);
        return DTRT_ERR_INVALID;
    };
    if (!tp.valid) return fail("the scene holds no topology");
    if (d->nder != s->nder) return fail("nder differs from the scene's");
    if (d->num_shapes != s->num_shapes || (d->num_shapes > 0 && !d->shapes)) return fail("the number of shapes changed");
    if (d->num_media != (int)tp.media_type.size()) return fail("the number of media changed");
    size_t off = 0;
    for (int si = 0; si < d->num_shapes; ++si) {
        const dtrt_shape_desc &sd = d->shapes[si];
        if (sd.num_vertices != tp.shape_nv[si] || sd.num_triangles != tp.shape_nt[si] || !sd.indices)
            return fail("shape " + std::to_string(si) + " changed its vertex or triangle count");
        const size_t n = 3 * (size_t)sd.num_triangles;
        if (std::memcmp(sd.indices, tp.indices.data() + off, n * sizeof(int)) != 0)
            return fail("shape " + std::to_string(si) + " changed its triangle indices");
        off += n;
    }
    return DTRT_OK;
}

// bruteforce.cpp:4-20: shape selection proportional to total edge length x weight
int set_edge_weights(dtrt_scene *s, const float *w) {
    std::vector<double> sw(s->num_shapes);
    double sum = 0;
    for (int i = 0; i < s->num_shapes; ++i) {
        const double wi = w ? (double)w[i] : 1.0;
        if (!(wi >= 0.0)) {
            set_last_error("edge sampling weights must be >= 0");
            return DTRT_ERR_INVALID;
        }
        sw[i] = (s->shape_skip[i] ? 0.0 : s->shape_edge_len[i]) * wi;
        sum += sw[i];
    }
    std::vector<double> cdf(s->num_shapes + 1, 0.0);
    double acc = 0;
    for (int i = 0; i < s->num_shapes; ++i) {
        acc += sw[i];
        cdf[i + 1] = sum > 0 ? acc / sum : 0.0;
    }
    if (sum > 0) cdf[s->num_shapes] = 1.0;
    s->dev.has_edges = sum > 1e-7 ? 1 : 0;
    cudaError_t e = cudaMemcpy((void *)s->dev.shape_edge_cdf, cdf.data(), cdf.size() * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    return DTRT_OK;
}

void free_scratch(Scratch &b) {
    void *ptrs[] = {b.acc1,     b.acc2,     b.out,     b.qe,     b.ql,      b.qli,       b.counts,   b.err,
                    b.adj_dimg, b.adj_grad, b.adj_out, b.adj_img, b.cam_state, b.cam_q, b.cam_cnt, b.li_sort};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    b = Scratch();
}

size_t scratch_bytes(const Scratch &b) {
    return b.acc1_n + b.acc2_n + b.out_n + b.qe_bytes + b.ql_bytes + b.qli_bytes + b.adj_dimg_n + b.adj_grad_n +
           b.adj_out_n + b.adj_img_n + b.cam_state_bytes + b.cam_q_bytes + b.cam_cnt_bytes + b.li_sort_bytes;
}

// Render work buffers (queues of 16-24 Mi records, path states, accumulators: GBs) of the
// last destroyed scene, kept for the next scene created on the same device: a loop that
// builds a scene per iteration (the reference's render_scene) allocates them once.
struct ScratchCache {
    std::mutex mu;
    Scratch buf;
    int device = -1;
    bool held = false;
};
ScratchCache &scratch_cache() {
    static ScratchCache c;
    return c;
}

void adopt_cached_scratch(dtrt_scene *s) {
    ScratchCache &c = scratch_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    if (c.held && c.device == s->device) {
        s->scratch = c.buf;
        c.buf = Scratch();
        c.held = false;
    }
}

void free_scene(dtrt_scene *s) {
    for (void *p : s->allocs)
        if (p) cudaFree(p);
    s->allocs.clear();
    s->alloc_bytes.clear();
    for (void *p : s->dgrid_bufs)
        if (p) cudaFree(p);
    s->dgrid_bufs.clear();
    // keep the larger of the cached and the destroyed scene's buffers (a scene that never
    // rendered has none)
    ScratchCache &c = scratch_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    Scratch &b = s->scratch;
    if (!c.held || scratch_bytes(b) > scratch_bytes(c.buf) || c.device != s->device) {
        if (c.held) free_scratch(c.buf);
        c.buf = b;
        c.device = s->device;
        c.held = true;
    } else {
        free_scratch(b);
    }
    b = Scratch();
}

// re-upload the host copy of the media array after a parameter change
int upload_media(dtrt_scene *s) {
    if (s->media_host.empty()) return DTRT_OK;
    cudaError_t e = cudaMemcpy((void *)s->dev.media, s->media_host.data(), s->media_host.size() * sizeof(DevMedium),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_last_error(std::string("media upload: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    return DTRT_OK;
}

int check_grid_medium(const dtrt_scene *s, int medium_id) {
    if (!s || medium_id < 0 || medium_id >= (int)s->media_host.size() ||
        s->media_host[medium_id].type != MEDIUM_HETEROGENEOUS) {
        set_last_error("medium_id does not name a heterogeneous medium");
        return DTRT_ERR_INVALID;
    }
    return DTRT_OK;
}

}  // namespace
std::atomic<int> g_bvh_builder{DTRT_BVH_AUTO};
int bvh_builder_setting() { return g_bvh_builder.load(); }

}  // namespace dt

// ====================================================================== C ABI
extern "C" {

int dtrt_set_bvh_builder(int builder) {
    if (builder != DTRT_BVH_AUTO && builder != DTRT_BVH_HOST && builder != DTRT_BVH_DEVICE) {
        dt::set_last_error("unknown BVH builder");
        return DTRT_ERR_INVALID;
    }
    dt::g_bvh_builder.store(builder);
    return DTRT_OK;
}

int dtrt_scene_bvh_info(const dtrt_scene *scene, dtrt_bvh_info *out) {
    if (!scene || !out) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    *out = scene->bvh_info;
    return DTRT_OK;
}

int dtrt_abi_version(void) { return DTRT_ABI_VERSION; }

int dtrt_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int dtrt_nder_supported(int nder) { return nder == 1 || nder == 3 || nder == 4 || nder == 8; }

const char *dtrt_last_error(void) { return dt::g_last_error.c_str(); }

int dtrt_scene_create(const dtrt_scene_desc *desc, dtrt_scene **out) {
    if (!desc || !out) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    *out = nullptr;
    if (!dtrt_nder_supported(desc->nder)) {
        dt::set_last_error("nder must be 1, 3, 4 or 8");
        return DTRT_ERR_UNSUPPORTED;
    }
    if (dtrt_device_count() <= 0) {
        dt::set_last_error("no CUDA device visible");
        return DTRT_ERR_NO_DEVICE;
    }
    std::unique_ptr<dtrt_scene> s(new dtrt_scene());
    s->nder = desc->nder;
    cudaGetDevice(&s->device);
    dt::adopt_cached_scratch(s.get());
    dt::Builder bld(s.get());
    int st = dt::build_scene(s.get(), desc, bld, true, nullptr);
    if (st == DTRT_OK) st = dt::set_edge_weights(s.get(), desc->edge_weights);
    if (st != DTRT_OK) {
        dt::free_scene(s.get());
        return st;
    }
    *out = s.release();
    return DTRT_OK;
}

int dtrt_scene_set_edge_weights(dtrt_scene *scene, const float *weights, int num_shapes) {
    if (!scene || !weights || num_shapes != scene->num_shapes) {
        dt::set_last_error("edge weights need one entry per shape");
        return DTRT_ERR_INVALID;
    }
    return dt::set_edge_weights(scene, weights);
}

int dtrt_scene_destroy(dtrt_scene *scene) {
    if (!scene) return DTRT_OK;
    dt::free_scene(scene);
    delete scene;
    return DTRT_OK;
}

int dtrt_release_cached_memory(void) {
    dt::ScratchCache &c = dt::scratch_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    if (c.held) dt::free_scratch(c.buf);
    c.held = false;
    return DTRT_OK;
}

int dtrt_scene_update(dtrt_scene *scene, const dtrt_scene_desc *desc, unsigned flags, dtrt_update_stats *stats) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!scene || !desc) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    if (flags & ~(unsigned)DTRT_UPDATE_REBUILD_BVH) {
        dt::set_last_error("unknown scene update flag");
        return DTRT_ERR_INVALID;
    }
    int st = dt::check_same_topology(scene, desc);
    if (st) return st;
    if (desc->edge_weights)  // validated up front: set_edge_weights runs after the device copies
        for (int i = 0; i < desc->num_shapes; ++i)
            if (!(desc->edge_weights[i] >= 0.f)) {
                dt::set_last_error("edge sampling weights must be >= 0");
                return DTRT_ERR_INVALID;
            }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        dt::set_last_error(std::string("scene update: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    // build into a fresh scene object that takes over the old arrays of unchanged size
    std::unique_ptr<dtrt_scene> t(new dtrt_scene());
    t->nder = scene->nder;
    t->device = scene->device;
    t->topo = scene->topo;
    std::vector<dt::Builder::Slot> pool(scene->allocs.size());
    for (size_t k = 0; k < pool.size(); ++k) pool[k] = {scene->allocs[k], scene->alloc_bytes[k]};
    dt::Builder bld(t.get(), &pool);
    dtrt_update_stats info{};
    const auto t1 = std::chrono::steady_clock::now();
    st = dt::build_scene(t.get(), desc, bld, (flags & DTRT_UPDATE_REBUILD_BVH) != 0, &info);
    const auto t2 = std::chrono::steady_clock::now();
    if (st == DTRT_OK) st = bld.commit();
    if (st != DTRT_OK) {
        bld.discard();
        return st;
    }
    // state set on the scene after creation
    t->dev.est_flags = scene->dev.est_flags;
    t->dev.tracking_cap = scene->dev.tracking_cap;
    bool dgrid = false;
    for (size_t mi = 0; mi < scene->dgrid_bufs.size(); ++mi) {
        if (!scene->dgrid_bufs[mi]) continue;  // media types and resolutions are unchanged
        t->dgrid_bufs[mi] = scene->dgrid_bufs[mi];
        scene->dgrid_bufs[mi] = nullptr;
        t->media_host[mi].density.dgrid = (const float *)t->dgrid_bufs[mi];
        t->media_host[mi].density.dgrid_n = scene->media_host[mi].density.dgrid_n;
        dgrid = true;
    }
    for (auto &sl : pool)  // old arrays whose size changed
        if (sl.p) cudaFree(sl.p);
    for (void *p : scene->dgrid_bufs)
        if (p) cudaFree(p);
    scene->dev = t->dev;
    scene->allocs.swap(t->allocs);
    scene->alloc_bytes.swap(t->alloc_bytes);
    scene->media_host.swap(t->media_host);
    scene->dgrid_bufs.swap(t->dgrid_bufs);
    scene->shape_edge_len.swap(t->shape_edge_len);
    scene->shape_skip.swap(t->shape_skip);
    scene->density_voxels = t->density_voxels;
    scene->num_shapes = t->num_shapes;
    scene->topo = std::move(t->topo);
    scene->bvh_info = t->bvh_info;
    st = dt::set_edge_weights(scene, desc->edge_weights);
    if (st == DTRT_OK && dgrid) st = dt::upload_media(scene);
    info.buffers_reused = bld.reused;
    info.buffers_allocated = bld.allocated;
    const auto t3 = std::chrono::steady_clock::now();
    info.host_ms = std::chrono::duration<double, std::milli>(t3 - t0).count();
    // allocations happen inside the build; everything after it is device work
    info.ms_arrays = std::chrono::duration<double, std::milli>(t2 - t1).count() - info.ms_bvh - bld.ms_alloc;
    info.ms_device = bld.ms_alloc + std::chrono::duration<double, std::milli>(t3 - t2).count();
    if (stats) *stats = info;
    return st;
}

int dtrt_render_fwd(dtrt_scene *scene, const dtrt_render_options *opts, float *out, int out_on_device, void *stream) {
    if (!scene || !opts || !out) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    if (opts->spp < 0 || opts->sppse < 0) {
        dt::set_last_error("spp and sppse must be >= 0");
        return DTRT_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    switch (scene->nder) {
        case 1: return dt::render_n<1>(scene, opts, out, out_on_device, st);
        case 3: return dt::render_n<3>(scene, opts, out, out_on_device, st);
        case 4: return dt::render_n<4>(scene, opts, out, out_on_device, st);
        case 8: return dt::render_n<8>(scene, opts, out, out_on_device, st);
    }
    dt::set_last_error("unsupported nder");
    return DTRT_ERR_UNSUPPORTED;
}

int dtrt_scene_enable_counters(dtrt_scene *scene, int enable) {
    if (!scene) return DTRT_ERR_INVALID;
    scene->counters = enable != 0;
    return DTRT_OK;
}

int dtrt_scene_last_stats(const dtrt_scene *scene, dtrt_render_stats *out) {
    if (!scene || !out) return DTRT_ERR_INVALID;
    *out = scene->last;
    return DTRT_OK;
}

int dtrt_scene_set_queue_capacity(dtrt_scene *scene, uint64_t max_tasks) {
    if (!scene) return DTRT_ERR_INVALID;
    scene->queue_cap = max_tasks;
    return DTRT_OK;
}

int dtrt_scene_set_camera_schedule(dtrt_scene *scene, int schedule) {
    if (!scene || schedule < DTRT_CAMERA_AUTO || schedule > DTRT_CAMERA_WAVEFRONT) {
        dt::set_last_error("unknown camera schedule");
        return DTRT_ERR_INVALID;
    }
    scene->camera_schedule = schedule;
    return DTRT_OK;
}

int dtrt_scene_set_tracking_cap(dtrt_scene *scene, int max_steps) {
    if (!scene || max_steps < 0) return DTRT_ERR_INVALID;
    scene->dev.tracking_cap = max_steps;
    return DTRT_OK;
}

int dtrt_scene_set_estimator_flags(dtrt_scene *scene, unsigned flags) {
    if (!scene || (flags & ~(unsigned)DTRT_EST_SCATTER_SEGMENT_FROM_ORIGIN)) {
        dt::set_last_error("unknown estimator flag");
        return DTRT_ERR_INVALID;
    }
    scene->dev.est_flags = flags;
    return DTRT_OK;
}

int dtrt_scene_gradient_sizes(const dtrt_scene *scene, int64_t *density_voxels, int64_t *vertices) {
    if (!scene) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    if (density_voxels) *density_voxels = scene->density_voxels;
    if (vertices) *vertices = scene->dev.num_verts;
    return DTRT_OK;
}

int dtrt_scene_set_density(dtrt_scene *scene, int medium_id, const float *density) {
    int st = dt::check_grid_medium(scene, medium_id);
    if (st) return st;
    if (!density) {
        dt::set_last_error("null density");
        return DTRT_ERR_INVALID;
    }
    dt::DevMedium &m = scene->media_host[medium_id];
    const size_t n = (size_t)m.density.res[0] * m.density.res[1] * m.density.res[2];
    std::vector<float> v(density, density + n);
    float maxv = 0.f;
    for (float &x : v) {  // gridvolume.h:128-131
        x = std::max(x, 0.0f);
        maxv = std::max(maxv, x);
    }
    if (!(maxv > 0.f)) {
        dt::set_last_error("heterogeneous medium with zero majorant");
        return DTRT_ERR_INVALID;
    }
    cudaError_t e = cudaMemcpy((void *)m.density.data, v.data(), n * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        dt::set_last_error(std::string("density upload: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    m.density.max_value = maxv;
    m.max_inv_density = (float)(1.0 / ((double)m.scale * maxv));
    return dt::upload_media(scene);
}

int dtrt_scene_set_density_derivatives(dtrt_scene *scene, int medium_id, const float *grids) {
    int st = dt::check_grid_medium(scene, medium_id);
    if (st) return st;
    dt::DevMedium &m = scene->media_host[medium_id];
    void *&buf = scene->dgrid_bufs[medium_id];
    if (buf) cudaFree(buf);
    buf = nullptr;
    m.density.dgrid = nullptr;
    m.density.dgrid_n = 0;
    if (grids) {
        const int N = scene->nder;
        const size_t n = (size_t)m.density.res[0] * m.density.res[1] * m.density.res[2];
        std::vector<float> il(n * N);  // [nder][voxel] -> [voxel][nder]
        for (int j = 0; j < N; ++j)
            for (size_t v = 0; v < n; ++v) il[v * N + j] = grids[(size_t)j * n + v];
        cudaError_t e = cudaMalloc(&buf, il.size() * 4);
        if (e == cudaSuccess) e = cudaMemcpy(buf, il.data(), il.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (buf) cudaFree(buf);
            buf = nullptr;
            dt::set_last_error(std::string("density derivative upload: ") + cudaGetErrorString(e));
            dt::upload_media(scene);
            return DTRT_ERR_CUDA;
        }
        m.density.dgrid = (const float *)buf;
        m.density.dgrid_n = N;
    }
    return dt::upload_media(scene);
}

int dtrt_render_adjoint(dtrt_scene *scene, const dtrt_render_options *opts, const float *d_image, float *image,
                        float *d_density, float *d_vertices, int on_device, void *stream) {
    if (!scene || !opts || (!image && !d_density && !d_vertices)) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    if ((d_density || d_vertices) && !d_image) {
        dt::set_last_error("d_density and d_vertices need d_image");
        return DTRT_ERR_INVALID;
    }
    if (opts->spp < 0 || opts->sppse < 0) {
        dt::set_last_error("spp and sppse must be >= 0");
        return DTRT_ERR_INVALID;
    }
    if (d_vertices) {
        if (d_density && scene->density_voxels > 0) {
            dt::set_last_error("the vertex-position adjoint needs a scene without participating media");
            return DTRT_ERR_UNSUPPORTED;
        }
        return dt::render_vertex_adjoint(scene, opts, d_image, image, d_vertices, on_device, (cudaStream_t)stream);
    }
    return dt::render_adjoint(scene, opts, d_image, image, d_density, on_device, (cudaStream_t)stream);
}

}  // extern "C"

namespace dt {
__global__ void __launch_bounds__(kBlock) k_trace(DevScene sc, const float *rays, int n, int *hits, float *t) {
    __shared__ int s_stack[kStackDepth * kBlock];
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    const float *r = rays + 8 * (size_t)i;
    Ctr c;
    float th;
    const int prim = closest_hit(sc, s_stack + threadIdx.x, mk(r[0], r[1], r[2]), mk(r[4], r[5], r[6]), r[3], r[7], th, c);
    hits[2 * i] = prim;
    hits[2 * i + 1] = prim >= 0 ? sc.tris[prim].w : -1;
    t[i] = prim >= 0 ? th : INFINITY;
}

// Three fresh streams of RndSampler(seed, idx): raw outputs, FP32 and FP64 uniforms.
__global__ void k_rng_sequence(uint64_t seed, uint64_t idx, int n, uint32_t *u32, float *f32, double *f64) {
    const int which = threadIdx.x;  // one thread per stream: the draws are sequential
    Rng r;
    r.init(seed, idx);
    for (int i = 0; i < n; ++i) {
        if (which == 0) u32[i] = r.next_u32();
        else if (which == 1) f32[i] = r.next1();
        else f64[i] = r.next1d();
    }
}
}  // namespace dt

extern "C" {

int dtrt_trace_closest(dtrt_scene *scene, const float *rays, int n, int *hits, float *t) {
    if (!scene || !rays || !hits || !t || n < 0) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    if (n == 0) return DTRT_OK;
    float *dr = nullptr, *dt_ = nullptr;
    int *dh = nullptr;
    cudaError_t e = cudaMalloc(&dr, (size_t)n * 8 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dh, (size_t)n * 2 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dt_, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMemcpy(dr, rays, (size_t)n * 8 * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        dt::DevScene sc = scene->dev;
        sc.error_flags = nullptr;
        dt::k_trace<<<(n + dt::kBlock - 1) / dt::kBlock, dt::kBlock>>>(sc, dr, n, dh, dt_);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(hits, dh, (size_t)n * 2 * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(t, dt_, (size_t)n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dr);
    cudaFree(dh);
    cudaFree(dt_);
    if (e != cudaSuccess) {
        dt::set_last_error(std::string("dtrt_trace_closest: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    return DTRT_OK;
}

int dtrt_rng_sequence(uint64_t seed, uint64_t idx, int n, uint32_t *u32, float *f32, double *f64) {
    if (n < 0 || n > (1 << 20)) {
        dt::set_last_error("dtrt_rng_sequence: n must be in [0, 1<<20]");
        return DTRT_ERR_INVALID;
    }
    if (n == 0) return DTRT_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        dt::set_last_error("no CUDA device");
        return DTRT_ERR_NO_DEVICE;
    }
    void *buf = nullptr;
    const size_t nb = (size_t)n * (4 + 4 + 8);
    cudaError_t e = cudaMalloc(&buf, nb);
    uint32_t *du = (uint32_t *)buf;
    float *df = (float *)(du + n);
    double *dd = (double *)((char *)buf + (size_t)n * 8);
    if (e == cudaSuccess) {
        dt::k_rng_sequence<<<1, 3>>>(seed, idx, n, du, df, dd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && u32) e = cudaMemcpy(u32, du, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && f32) e = cudaMemcpy(f32, df, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && f64) e = cudaMemcpy(f64, dd, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(buf);
    if (e != cudaSuccess) {
        dt::set_last_error(std::string("dtrt_rng_sequence: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    return DTRT_OK;
}

int dtrt_vol_read(const char *path, int *res, int *channels, float *vmin, float *vmax, float *data) {
    if (!path || !res || !channels || !vmin || !vmax) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    std::vector<float> buf;
    int st = dt::read_vol(path, res, *channels, vmin, vmax, data ? &buf : nullptr);
    if (st == DTRT_OK && data) std::memcpy(data, buf.data(), buf.size() * 4);
    return st;
}

}  // extern "C"
