// TEST INFRASTRUCTURE — CPU oracle scene model implementation (see oracle_scene.h).
#include "oracle_scene.h"

#include <cstdio>
#include <numeric>

namespace orc {

// ------------------------------------------------------------------ small linear algebra
bool invert4(const M4 &a, M4 &out) {
    double inv[16], det;
    const double *m = a.m;
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
    det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0) return false;
    for (int i = 0; i < 16; ++i) out.m[i] = inv[i] / det;
    return true;
}

bool invert3(const M3 &a, M3 &out) {
    const double *m = a.m;
    double c0 = m[4] * m[8] - m[5] * m[7], c1 = m[5] * m[6] - m[3] * m[8], c2 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c0 + m[1] * c1 + m[2] * c2;
    if (det == 0) return false;
    double id = 1.0 / det;
    out.m[0] = c0 * id; out.m[1] = (m[2] * m[7] - m[1] * m[8]) * id; out.m[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    out.m[3] = c1 * id; out.m[4] = (m[0] * m[8] - m[2] * m[6]) * id; out.m[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    out.m[6] = c2 * id; out.m[7] = (m[1] * m[6] - m[0] * m[7]) * id; out.m[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return true;
}

const M3 &frame_prerotation() {
    // Rodrigues rotation of angle 0.1f about normalize(0.1f, 0.2f, 0.3f), utils.cpp:55
    static const M3 R = [] {
        double ax = (double)0.1f, ay = (double)0.2f, az = (double)0.3f;
        double l = std::sqrt(ax * ax + ay * ay + az * az);
        ax /= l; ay /= l; az /= l;
        double th = (double)0.1f, c = std::cos(th), s = std::sin(th), C = 1 - c;
        M3 r;
        r.m[0] = c + ax * ax * C;      r.m[1] = ax * ay * C - az * s; r.m[2] = ax * az * C + ay * s;
        r.m[3] = ay * ax * C + az * s; r.m[4] = c + ay * ay * C;      r.m[5] = ay * az * C - ax * s;
        r.m[6] = az * ax * C - ay * s; r.m[7] = az * ay * C + ax * s; r.m[8] = c + az * az * C;
        return r;
    }();
    return R;
}

// math_func.cpp:6-23 (A&S 7.1.26)
double approx_erf(double x) {
    const double a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741, a4 = -1.453152027, a5 = 1.061405429,
                 p = 0.3275911;
    double sign = signum(x);
    x = std::abs(x);
    double t = 1.0 / (1.0 + p * x);
    double y = 1.0 - (((((a5 * t + a4) * t) + a3) * t + a2) * t + a1) * t * std::exp(-x * x);
    return sign * y;
}

// math_func.cpp:26-54 (Giles, "Approximating the erfinv function")
double approx_erfinv(double x) {
    double w = -std::log((1.0 - x) * (1.0 + x)), p;
    if (w < 5.0) {
        w = w - 2.5;
        p = 2.81022636e-08;
        p = 3.43273939e-07 + p * w;
        p = -3.5233877e-06 + p * w;
        p = -4.39150654e-06 + p * w;
        p = 0.00021858087 + p * w;
        p = -0.00125372503 + p * w;
        p = -0.00417768164 + p * w;
        p = 0.246640727 + p * w;
        p = 1.50140941 + p * w;
    } else {
        w = std::sqrt(w) - 3.0;
        p = -0.000200214257;
        p = 0.000100950558 + p * w;
        p = 0.00134934322 + p * w;
        p = -0.00367342844 + p * w;
        p = 0.00573950773 + p * w;
        p = -0.0076224613 + p * w;
        p = 0.00943887047 + p * w;
        p = 1.00167406 + p * w;
        p = 2.83297682 + p * w;
    }
    return p * x;
}

// ------------------------------------------------------------------ shape
template <int N>
void Shape<N>::compute_face_normals() {
    face_normals.resize(nt);
    for (int i = 0; i < nt; ++i) {
        const auto &f = idx[i];
        DV3<N> n = cross(verts[f[1]] - verts[f[0]], verts[f[2]] - verts[f[0]]);
        double l = norm(val(n));
        face_normals[i] = (l < kEps) ? n : normalized(n);  // shape.cpp:117-124 (vanishing normal kept)
    }
}

template <int N>
void Shape<N>::construct_edges() {
    std::map<std::pair<int, int>, std::vector<int>> m;
    for (int t = 0; t < nt; ++t)
        for (int e = 0; e < 3; ++e) {
            int a = idx[t][e], b = idx[t][(e + 1) % 3];
            m[a < b ? std::make_pair(a, b) : std::make_pair(b, a)].push_back(t);
        }
    edges.clear();
    for (auto const &kv : m) {
        double len = norm(vert(kv.first.first) - vert(kv.first.second));
        if (kv.second.size() > 2) continue;  // non-manifold: the reference asserts (shape.cpp:272-275)
        if (kv.second.size() == 2) {
            if (kv.second[0] == kv.second[1]) continue;
            double c = dot(val(face_normals[kv.second[0]]), val(face_normals[kv.second[1]]));
            if (c < -1.0 + kEps) continue;  // inconsistent orientation: asserted in the reference
            if (c < 1.0 - kEps) edges.push_back(Edge{kv.first.first, kv.first.second, kv.second[0], kv.second[1], len});
        } else {
            edges.push_back(Edge{kv.first.first, kv.first.second, kv.second[0], -1, len});
        }
    }
    edge_distrb.clear();
    for (const Edge &e : edges) edge_distrb.append(e.length);
    if (!edges.empty()) edge_distrb.normalize();
}

template <int N>
double Shape<N>::area(int t) const {
    const auto &f = idx[t];
    return 0.5 * norm(cross(vert(f[1]) - vert(f[0]), vert(f[2]) - vert(f[0])));
}

template <int N>
void Shape<N>::sample_position(int t, double u, double v, V3 &pos, V3 &n) const {
    const auto &f = idx[t];
    V3 v0 = vert(f[0]), e1 = vert(f[1]) - v0, e2 = vert(f[2]) - v0;
    double a = std::sqrt(u), b1 = 1.0 - a, b2 = a * v;
    n = normalized(cross(e1, e2));
    pos = v0 + e1 * b1 + e2 * b2;
}

template <int N>
int Shape<N>::is_silhouette(const Edge &e, const V3 &p) const {
    if (e.f0 == -1 || e.f1 == -1) return 2;
    V3 v0 = vert(e.v0), v1 = vert(e.v1);
    bool ff0 = false, ff1 = false;
    for (int i = 0; i < 3; ++i) {
        int k = idx[e.f0][i];
        if (k != e.v0 && k != e.v1) {
            V3 v = vert(k);
            ff0 = dot(normalized(cross(v0 - v, v1 - v)), p - v) > 0.0;
            break;
        }
    }
    for (int i = 0; i < 3; ++i) {
        int k = idx[e.f1][i];
        if (k != e.v0 && k != e.v1) {
            V3 v = vert(k);
            ff1 = dot(normalized(cross(v1 - v, v0 - v)), p - v) > 0.0;
            break;
        }
    }
    if (ff0 != ff1) return 2;
    return has_normals() ? 0 : 1;
}

// ------------------------------------------------------------------ grid
template <int N>
void Grid<N>::configure() {  // gridvolume.h:135-141
    V3 c = (mn + mx) * 0.5;
    center = xfm_point(v2w, c);
    aabb = AABB();
    for (int i = 0; i < 8; ++i) {
        V3 corner((i & 1) ? mx.x : mn.x, (i & 2) ? mx.y : mn.y, (i & 4) ? mx.z : mn.z);
        aabb.expand(xfm_point(v2w, corner));
    }
}

template <int N>
V3 Grid<N>::to_grid(const V3 &pw) const {  // gridvolume.h:296-317
    V3 p = xfm_point(w2v, pw);
    return V3((p.x - mn.x) * (res[0] - 1) / extent.x, (p.y - mn.y) * (res[1] - 1) / extent.y,
              (p.z - mn.z) * (res[2] - 1) / extent.z);
}

template <int N>
DV3<N> Grid<N>::to_grid_ad(const DV3<N> &pw) const {  // gridvolume.h:301-326 (rotation about the centre)
    V3 pv = val(pw);
    DV3<N> p = lift<N>(xfm_point(w2v, pv));
    V3 q = pv - center;
    for (int j = 0; j < N; ++j) {
        V3 g = grad(pw, j) - cross(rot_vel[j], q) - trans_vel[j];
        V3 gv(w2v.m[0] * g.x + w2v.m[1] * g.y + w2v.m[2] * g.z, w2v.m[4] * g.x + w2v.m[5] * g.y + w2v.m[6] * g.z,
              w2v.m[8] * g.x + w2v.m[9] * g.y + w2v.m[10] * g.z);
        set_grad(p, j, gv);
    }
    DV3<N> r;
    r.x = (p.x - mn.x) * ((double)(res[0] - 1) / extent.x);
    r.y = (p.y - mn.y) * ((double)(res[1] - 1) / extent.y);
    r.z = (p.z - mn.z) * ((double)(res[2] - 1) / extent.z);
    return r;
}

template <int N>
double Grid<N>::lookup(const V3 &pw) const {  // gridvolume.h:144-171
    V3 p = to_grid(pw);
    if (!in_cell_range(p.x, p.y, p.z)) return {};
    int x1 = (int)std::floor(p.x), y1 = (int)std::floor(p.y), z1 = (int)std::floor(p.z);
    int x2 = x1 + 1, y2 = y1 + 1, z2 = z1 + 1;
    if (x1 < 0 || x2 >= res[0] || y1 < 0 || y2 >= res[1] || z1 < 0 || z2 >= res[2]) return 0.0;
    double fx = p.x - x1, fy = p.y - y1, fz = p.z - z1, gx = 1 - fx, gy = 1 - fy, gz = 1 - fz;
    auto D = [&](int z, int y, int x) { return (double)data[((size_t)z * res[1] + y) * res[0] + x]; };
    return ((D(z1, y1, x1) * gx + D(z1, y1, x2) * fx) * gy + (D(z1, y2, x1) * gx + D(z1, y2, x2) * fx) * fy) * gz +
           ((D(z2, y1, x1) * gx + D(z2, y1, x2) * fx) * gy + (D(z2, y2, x1) * gx + D(z2, y2, x2) * fx) * fy) * fz;
}

template <int N>
Dual<N> Grid<N>::lookup_ad(const DV3<N> &pw) const {  // gridvolume.h:174-201
    DV3<N> p = to_grid_ad(pw);
    if (!in_cell_range(p.x.v, p.y.v, p.z.v)) return {};
    int x1 = (int)std::floor(p.x.v), y1 = (int)std::floor(p.y.v), z1 = (int)std::floor(p.z.v);
    int x2 = x1 + 1, y2 = y1 + 1, z2 = z1 + 1;
    if (x1 < 0 || x2 >= res[0] || y1 < 0 || y2 >= res[1] || z1 < 0 || z2 >= res[2]) return Dual<N>(0.0);
    Dual<N> fx = p.x - (double)x1, fy = p.y - (double)y1, fz = p.z - (double)z1;
    Dual<N> gx = 1.0 - fx, gy = 1.0 - fy, gz = 1.0 - fz;
    auto D = [&](int z, int y, int x) { return (double)data[((size_t)z * res[1] + y) * res[0] + x]; };
    Dual<N> r = ((D(z1, y1, x1) * gx + D(z1, y1, x2) * fx) * gy + (D(z1, y2, x1) * gx + D(z1, y2, x2) * fx) * fy) * gz +
                ((D(z2, y1, x1) * gx + D(z2, y1, x2) * fx) * gy + (D(z2, y2, x1) * gx + D(z2, y2, x2) * fx) * fy) * fz;
    if (!dgrid.empty()) {  // per-voxel directions: value derivative at the point
        for (int k = 0; k < 8; ++k) {
            const int dx = k & 1, dy = (k >> 1) & 1, dz = (k >> 2) & 1;
            const double w = (dx ? fx.v : gx.v) * (dy ? fy.v : gy.v) * (dz ? fz.v : gz.v);
            const float *q = &dgrid[(((size_t)(z1 + dz) * res[1] + (y1 + dy)) * res[0] + (x1 + dx)) * N];
            for (int j = 0; j < N; ++j) r.d[j] += w * (double)q[j];
        }
    }
    return r;
}

template <int N>
V3 Grid<N>::lookup3(const V3 &pw) const {  // gridvolume.h:204-232
    V3 p = to_grid(pw);
    if (!in_cell_range(p.x, p.y, p.z)) return {};
    int x1 = (int)std::floor(p.x), y1 = (int)std::floor(p.y), z1 = (int)std::floor(p.z);
    int x2 = x1 + 1, y2 = y1 + 1, z2 = z1 + 1;
    if (x1 < 0 || x2 >= res[0] || y1 < 0 || y2 >= res[1] || z1 < 0 || z2 >= res[2]) return V3();
    double fx = p.x - x1, fy = p.y - y1, fz = p.z - z1, gx = 1 - fx, gy = 1 - fy, gz = 1 - fz;
    V3 r;
    for (int c = 0; c < 3; ++c) {
        auto D = [&](int z, int y, int x) { return (double)data[(((size_t)z * res[1] + y) * res[0] + x) * 3 + c]; };
        r[c] = ((D(z1, y1, x1) * gx + D(z1, y1, x2) * fx) * gy + (D(z1, y2, x1) * gx + D(z1, y2, x2) * fx) * fy) * gz +
               ((D(z2, y1, x1) * gx + D(z2, y1, x2) * fx) * gy + (D(z2, y2, x1) * gx + D(z2, y2, x2) * fx) * fy) * fz;
    }
    return r;
}

template <int N>
DV3<N> Grid<N>::lookup3_ad(const DV3<N> &pw) const {  // gridvolume.h:235-263
    DV3<N> p = to_grid_ad(pw);
    if (!in_cell_range(p.x.v, p.y.v, p.z.v)) return {};
    int x1 = (int)std::floor(p.x.v), y1 = (int)std::floor(p.y.v), z1 = (int)std::floor(p.z.v);
    int x2 = x1 + 1, y2 = y1 + 1, z2 = z1 + 1;
    if (x1 < 0 || x2 >= res[0] || y1 < 0 || y2 >= res[1] || z1 < 0 || z2 >= res[2]) return DV3<N>();
    Dual<N> fx = p.x - (double)x1, fy = p.y - (double)y1, fz = p.z - (double)z1;
    Dual<N> gx = 1.0 - fx, gy = 1.0 - fy, gz = 1.0 - fz;
    DV3<N> r;
    for (int c = 0; c < 3; ++c) {
        auto D = [&](int z, int y, int x) { return (double)data[(((size_t)z * res[1] + y) * res[0] + x) * 3 + c]; };
        r[c] = ((D(z1, y1, x1) * gx + D(z1, y1, x2) * fx) * gy + (D(z1, y2, x1) * gx + D(z1, y2, x2) * fx) * fy) * gz +
               ((D(z2, y1, x1) * gx + D(z2, y1, x2) * fx) * gy + (D(z2, y2, x1) * gx + D(z2, y2, x2) * fx) * fy) * fz;
    }
    return r;
}

// ------------------------------------------------------------------ BVH
void Bvh::build(const std::vector<std::array<V3, 3>> &tris) {
    tri_verts = tris;
    int n = (int)tris.size();
    tri_order.resize(n);
    std::iota(tri_order.begin(), tri_order.end(), 0);
    std::vector<V3> cen(n);
    for (int i = 0; i < n; ++i) cen[i] = (tris[i][0] + tris[i][1] + tris[i][2]) * (1.0 / 3.0);
    nodes.clear();
    nodes.reserve(2 * n + 1);
    struct Item { int node, first, count; };
    nodes.push_back(Node());
    std::vector<Item> stack{{0, 0, n}};
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        Node &nd = nodes[it.node];
        nd.box = AABB();
        AABB cb;
        for (int i = it.first; i < it.first + it.count; ++i) {
            int t = tri_order[i];
            for (int k = 0; k < 3; ++k) nd.box.expand(tris[t][k]);
            cb.expand(cen[t]);
        }
        if (it.count <= 4) {
            nd.first = it.first;
            nd.count = it.count;
            continue;
        }
        V3 ext = cb.mx - cb.mn;
        int axis = (ext.x > ext.y && ext.x > ext.z) ? 0 : (ext.y > ext.z ? 1 : 2);
        int mid = it.first + it.count / 2;
        std::nth_element(tri_order.begin() + it.first, tri_order.begin() + mid, tri_order.begin() + it.first + it.count,
                         [&](int a, int b) { return cen[a][axis] < cen[b][axis]; });
        int l = (int)nodes.size();
        nodes.push_back(Node());
        nodes.push_back(Node());
        nodes[it.node].left = l;
        nodes[it.node].right = l + 1;
        nodes[it.node].count = 0;
        stack.push_back({l, it.first, mid - it.first});
        stack.push_back({l + 1, mid, it.first + it.count - mid});
    }
}

int Bvh::closest(const V3 &o, const V3 &d, double tmin, double tmax, double &t_hit) const {
    if (nodes.empty()) return -1;
    int best = -1;
    double best_t = tmax;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    V3 inv(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
    while (sp) {
        const Node &nd = nodes[stack[--sp]];
        double t0 = tmin, t1 = best_t;
        bool hit = true;
        for (int a = 0; a < 3 && hit; ++a) {
            double ta = (nd.box.mn[a] - o[a]) * inv[a], tb = (nd.box.mx[a] - o[a]) * inv[a];
            if (ta > tb) std::swap(ta, tb);
            if (std::isnan(ta) || std::isnan(tb)) { ta = -INFINITY; tb = INFINITY; }  // 0 * inf on a slab plane
            t0 = std::max(t0, ta);
            t1 = std::min(t1, tb * (1 + 1e-12) + 1e-12);
            hit = t0 <= t1;
        }
        if (!hit) continue;
        if (nd.left < 0) {
            for (int i = nd.first; i < nd.first + nd.count; ++i) {
                int t = tri_order[i];
                const V3 &a = tri_verts[t][0];
                V3 e1 = tri_verts[t][1] - a, e2 = tri_verts[t][2] - a;
                V3 pv = cross(d, e2);
                double det = dot(e1, pv);
                if (det == 0) continue;
                double inv_det = 1.0 / det;
                V3 s = o - a;
                double u = dot(s, pv) * inv_det;
                if (u < 0 || u > 1) continue;
                V3 q = cross(s, e1);
                double v = dot(d, q) * inv_det;
                if (v < 0 || u + v > 1) continue;
                double tt = dot(e2, q) * inv_det;
                if (tt >= tmin && tt <= best_t) {
                    best_t = tt;
                    best = t;
                }
            }
        } else {
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
    }
    t_hit = best_t;
    return best;
}

// ------------------------------------------------------------------ camera
template <int N>
Ray Camera<N>::sample_primary_ray(double x, double y) const {
    x /= width;
    y /= height;
    double aspect = (double)width / (double)height;
    V3 ndc((x - 0.5) * 2.0, (y - 0.5) * (-2.0) / aspect, 1.0);
    V3 dir = normalized(ndc2cam * ndc);
    return Ray{xfm_point(c2w, V3()), xfm_vector(c2w, dir)};
}
template <int N>
Ray Camera<N>::sample_primary_ray(int px, int py, double fx, double fy) const {
    double sx = (px + fx) / (double)width, sy = (py + fy) / (double)height;
    double aspect = (double)width / (double)height;
    V3 ndc((sx - 0.5) * 2.0, (sy - 0.5) * (-2.0) / aspect, 1.0);
    V3 dir = normalized(ndc2cam * ndc);
    return Ray{xfm_point(c2w, V3()), xfm_vector(c2w, dir)};
}
template <int N>
RayAD<N> Camera<N>::sample_primary_ray_ad(double x, double y) const {
    x /= width;
    y /= height;
    double aspect = (double)width / (double)height;
    V3 ndc((x - 0.5) * 2.0, (y - 0.5) * (-2.0) / aspect, 1.0);
    V3 dir = normalized(ndc2cam * ndc);
    return RayAD<N>{cpos, cframe.to_world(lift<N>(dir))};
}

// ------------------------------------------------------------------ scene build
static bool read_vol(const char *path, int res[3], int &ch, V3 &mn, V3 &mx, std::vector<float> &data,
                     std::string &err) {  // gridvolume.h:88-132
    FILE *f = std::fopen(path, "rb");
    if (!f) { err = std::string("cannot open volume file ") + path; return false; }
    char hdr[3];
    unsigned char ver;
    int type;
    float pmin[3], pmax[3];
    bool ok = std::fread(hdr, 1, 3, f) == 3 && std::strncmp(hdr, "VOL", 3) == 0 && std::fread(&ver, 1, 1, f) == 1 &&
              ver == 3 && std::fread(&type, 4, 1, f) == 1 && std::fread(res, 4, 3, f) == 3 &&
              std::fread(&ch, 4, 1, f) == 1 && type == 1 && (ch == 1 || ch == 3) && std::fread(pmin, 4, 3, f) == 3 &&
              std::fread(pmax, 4, 3, f) == 3;
    if (ok) {
        size_t n = (size_t)res[0] * res[1] * res[2] * ch;
        data.resize(n);
        ok = std::fread(data.data(), 4, n, f) == n;
    }
    std::fclose(f);
    if (!ok) { err = std::string("invalid VOL v3 file ") + path; return false; }
    mn = V3(pmin[0], pmin[1], pmin[2]);
    mx = V3(pmax[0], pmax[1], pmax[2]);
    return true;
}

template <int N>
static bool load_grid(Grid<N> &g, const char *file, const float *arr, const int *res, int ch, const float *vmin,
                      const float *vmax, const float *to_world, std::string &err) {
    if (file) {
        int r[3];
        int c;
        if (!read_vol(file, r, c, g.mn, g.mx, g.data, err)) return false;
        if (c != ch) { err = "volume channel count mismatch"; return false; }
        for (int i = 0; i < 3; ++i) g.res[i] = r[i];
    } else {
        if (!arr) { err = "heterogeneous medium without density data"; return false; }
        for (int i = 0; i < 3; ++i) g.res[i] = res[i];
        size_t n = (size_t)res[0] * res[1] * res[2] * ch;
        g.data.assign(arr, arr + n);
        g.mn = V3(vmin[0], vmin[1], vmin[2]);
        g.mx = V3(vmax[0], vmax[1], vmax[2]);
    }
    g.channels = ch;
    g.extent = g.mx - g.mn;
    g.max_value = 0;
    for (float &v : g.data) {
        v = std::max(v, 0.0f);
        if (v > g.max_value) g.max_value = v;
    }
    for (int i = 0; i < 16; ++i) g.v2w.m[i] = to_world[i];
    if (!invert4(g.v2w, g.w2v)) { err = "singular volume to_world"; return false; }
    for (int j = 0; j < N; ++j) g.trans_vel[j] = g.rot_vel[j] = V3();
    g.configure();
    g.valid = true;
    return true;
}

template <int N>
std::string Scene<N>::build(const dtrt_scene_desc &d) {
    if (d.nder != N) return "nder mismatch";
    // camera.cpp:8-38
    const dtrt_camera_desc &c = d.camera;
    cam.width = c.width;
    cam.height = c.height;
    cam.clip_near = c.clip_near;
    cam.med_id = c.med_id;
    cam.crop_x = c.crop_offset_x; cam.crop_y = c.crop_offset_y;
    cam.crop_w = c.crop_width > 0 ? c.crop_width : -1;
    cam.crop_h = c.crop_height > 0 ? c.crop_height : -1;
    for (int i = 0; i < 16; ++i) cam.c2w.m[i] = c.cam_to_world[i];
    for (int i = 0; i < 9; ++i) cam.c2ndc.m[i] = c.cam_to_ndc[i];
    if (!invert4(cam.c2w, cam.w2c) || !invert3(cam.c2ndc, cam.ndc2cam)) return "singular camera matrix";
    cam.cpos = lift<N>(V3(cam.c2w.m[3], cam.c2w.m[7], cam.c2w.m[11]));
    cam.cframe.s = lift<N>(V3(cam.c2w.m[0], cam.c2w.m[4], cam.c2w.m[8]));
    cam.cframe.t = lift<N>(V3(cam.c2w.m[1], cam.c2w.m[5], cam.c2w.m[9]));
    cam.cframe.n = lift<N>(V3(cam.c2w.m[2], cam.c2w.m[6], cam.c2w.m[10]));
    if (c.velocities) {  // camera.cpp:103-111
        for (int j = 0; j < N; ++j) {
            V3 dx(c.velocities[3 * j], c.velocities[3 * j + 1], c.velocities[3 * j + 2]);
            V3 dw(c.velocities[3 * (N + j)], c.velocities[3 * (N + j) + 1], c.velocities[3 * (N + j) + 2]);
            set_grad(cam.cpos, j, dx);
            set_grad(cam.cframe.s, j, cross(dw, val(cam.cframe.s)));
            set_grad(cam.cframe.t, j, cross(dw, val(cam.cframe.t)));
            set_grad(cam.cframe.n, j, cross(dw, val(cam.cframe.n)));
        }
    }
    // shapes, shape.cpp:10-52
    shapes.resize(d.num_shapes);
    std::vector<std::array<V3, 3>> tris;
    tri_shape.clear();
    tri_prim.clear();
    for (int s = 0; s < d.num_shapes; ++s) {
        const dtrt_shape_desc &sd = d.shapes[s];
        Shape<N> &sh = shapes[s];
        sh.nv = sd.num_vertices;
        sh.nt = sd.num_triangles;
        sh.light_id = sd.light_id;
        sh.bsdf_id = sd.bsdf_id;
        sh.med_int = sd.med_int_id;
        sh.med_ext = sd.med_ext_id;
        if (sh.bsdf_id < 0 || sh.bsdf_id >= d.num_bsdfs) return "shape without a valid bsdf_id";
        sh.verts.resize(sh.nv);
        for (int i = 0; i < sh.nv; ++i) sh.verts[i] = lift<N>(V3(sd.vertices[3 * i], sd.vertices[3 * i + 1], sd.vertices[3 * i + 2]));
        if (sd.normals) {
            sh.normals.resize(sh.nv);
            for (int i = 0; i < sh.nv; ++i)
                sh.normals[i] = lift<N>(normalized(V3(sd.normals[3 * i], sd.normals[3 * i + 1], sd.normals[3 * i + 2])));
        }
        sh.idx.resize(sh.nt);
        for (int i = 0; i < sh.nt; ++i) {
            for (int k = 0; k < 3; ++k) {
                int v = sd.indices[3 * i + k];
                if (v < 0 || v >= sh.nv) return "triangle index out of range";
                sh.idx[i][k] = v;
            }
        }
        if (sd.velocities) {
            for (int j = 0; j < N; ++j)
                for (int i = 0; i < sh.nv; ++i) {
                    const float *p = sd.velocities + 3 * ((size_t)j * sh.nv + i);
                    set_grad(sh.verts[i], j, V3(p[0], p[1], p[2]));
                    if (sd.normals) {
                        // shape.cpp:45: the normal velocities are read at one fixed offset for every derivative
                        const float *q = sd.velocities + (size_t)sh.nv * 3 * N + 3 * i;
                        set_grad(sh.normals[i], j, V3(q[0], q[1], q[2]));
                    }
                }
        }
        sh.compute_face_normals();
        sh.construct_edges();
        for (int t = 0; t < sh.nt; ++t) {
            tris.push_back({sh.vert(sh.idx[t][0]), sh.vert(sh.idx[t][1]), sh.vert(sh.idx[t][2])});
            tri_shape.push_back(s);
            tri_prim.push_back(t);
        }
    }
    bvh.build(tris);
    // BSDFs
    bsdfs.resize(d.num_bsdfs);
    for (int b = 0; b < d.num_bsdfs; ++b) {
        const dtrt_bsdf_desc &bd = d.bsdfs[b];
        Bsdf<N> &o = bsdfs[b];
        o.type = bd.type;
        o.diffuse = lift<N>(V3(bd.diffuse[0], bd.diffuse[1], bd.diffuse[2]));
        o.specular = lift<N>(V3(bd.specular[0], bd.specular[1], bd.specular[2]));
        o.exponent = Dual<N>(bd.exponent);
        if (bd.type == DTRT_BSDF_PHONG) {  // phong.h:9-15
            double v0 = (val(o.diffuse).x + val(o.diffuse).y + val(o.diffuse).z) / 3.0;
            double v1 = (val(o.specular).x + val(o.specular).y + val(o.specular).z) / 3.0;
            o.spec_weight = v1 / (v0 + v1);
        }
        // microfacet.h:11-14: alpha clamped (value only) to >= 1e-4
        o.alpha = Dual<N>(bd.alpha);
        if (o.alpha.v < (double)1e-4f) o.alpha.v = (double)1e-4f;
        o.eta = Dual<N>((double)(bd.int_ior / bd.ext_ior));
        for (int j = 0; j < N; ++j) {
            if (bd.d_diffuse) { o.diffuse.x.d[j] = bd.d_diffuse[3 * j]; o.diffuse.y.d[j] = bd.d_diffuse[3 * j + 1]; o.diffuse.z.d[j] = bd.d_diffuse[3 * j + 2]; }
            if (bd.d_specular) { o.specular.x.d[j] = bd.d_specular[3 * j]; o.specular.y.d[j] = bd.d_specular[3 * j + 1]; o.specular.z.d[j] = bd.d_specular[3 * j + 2]; }
            if (bd.d_exponent) o.exponent.d[j] = bd.d_exponent[j];
            if (bd.d_alpha) o.alpha.d[j] = bd.d_alpha[j];
            if (bd.d_eta) o.eta.d[j] = bd.d_eta[j];
        }
        o.inv_eta = 1.0 / o.eta;
    }
    // phases, phase.h
    phases.resize(d.num_phases);
    for (int p = 0; p < d.num_phases; ++p) {
        phases[p].type = d.phases[p].type;
        phases[p].g = Dual<N>(d.phases[p].g);
        if (d.phases[p].d_g) for (int j = 0; j < N; ++j) phases[p].g.d[j] = d.phases[p].d_g[j];
    }
    // emitters
    emitters.resize(d.num_emitters);
    for (int e = 0; e < d.num_emitters; ++e) {
        const dtrt_emitter_desc &ed = d.emitters[e];
        Emitter<N> &o = emitters[e];
        o.type = ed.type;
        o.shape_id = ed.shape_id;
        if (o.shape_id < 0 || o.shape_id >= d.num_shapes) return "emitter with invalid shape_id";
        o.intensity = lift<N>(V3(ed.intensity[0], ed.intensity[1], ed.intensity[2]));
        o.kappa = Dual<N>(ed.kappa);
        o.two_sided = ed.two_sided != 0;
        for (int j = 0; j < N; ++j) {
            if (ed.d_intensity) { o.intensity.x.d[j] = ed.d_intensity[3 * j]; o.intensity.y.d[j] = ed.d_intensity[3 * j + 1]; o.intensity.z.d[j] = ed.d_intensity[3 * j + 2]; }
            if (ed.d_kappa) o.kappa.d[j] = ed.d_kappa[j];
        }
    }
    // media
    media.resize(d.num_media);
    std::string err;
    for (int m = 0; m < d.num_media; ++m) {
        const dtrt_medium_desc &md = d.media[m];
        Medium<N> &o = media[m];
        o.type = md.type;
        o.phase_id = md.phase_id;
        if (o.phase_id < 0 || o.phase_id >= d.num_phases) return "medium with invalid phase_id";
        o.albedo = lift<N>(V3(md.albedo[0], md.albedo[1], md.albedo[2]));
        if (md.d_albedo) for (int j = 0; j < N; ++j) { o.albedo.x.d[j] = md.d_albedo[3 * j]; o.albedo.y.d[j] = md.d_albedo[3 * j + 1]; o.albedo.z.d[j] = md.d_albedo[3 * j + 2]; }
        if (md.type == DTRT_MEDIUM_HOMOGENEOUS) {  // homogeneous.h:13-27
            o.sigma_t = Dual<N>(md.sigma_t);
            if (md.d_sigma_t) for (int j = 0; j < N; ++j) o.sigma_t.d[j] = md.d_sigma_t[j];
            o.sigma_s = val(o.albedo) * o.sigma_t.v;
            o.sampling_weight = std::max((double)md.albedo[0], std::max((double)md.albedo[1], (double)md.albedo[2]));
        } else {  // heterogeneous.h:13-75
            o.scale = Dual<N>(md.density_scale);
            if (md.d_density_scale) for (int j = 0; j < N; ++j) o.scale.d[j] = md.d_density_scale[j];
            if (!load_grid(o.density, md.density_file, md.density, md.res, 1, md.vol_min, md.vol_max, md.to_world, err))
                return err;
            if (md.albedo_file || md.albedo_grid) {
                if (!load_grid(o.albedo_vol, md.albedo_file, md.albedo_grid, md.albedo_res, 3, md.albedo_min,
                               md.albedo_max, md.to_world, err))
                    return err;
                o.albedo = DV3<N>();  // m_albedo stays default-constructed with an albedo grid
            }
            for (int j = 0; j < N; ++j) {
                if (md.trans_velocities) o.density.trans_vel[j] = V3(md.trans_velocities[3 * j], md.trans_velocities[3 * j + 1], md.trans_velocities[3 * j + 2]);
                if (md.rot_velocities) o.density.rot_vel[j] = V3(md.rot_velocities[3 * j], md.rot_velocities[3 * j + 1], md.rot_velocities[3 * j + 2]);
            }
            o.max_inv_density = 1.0 / (o.scale.v * o.density.max_value);
        }
    }
    for (const Shape<N> &s : shapes) {
        if (s.med_int >= d.num_media || s.med_ext >= d.num_media) return "shape medium id out of range";
        if (s.light_id >= d.num_emitters) return "shape light id out of range";
    }
    // scene.cpp:45-98 light tables
    int nl = d.num_emitters;
    light_pmf.assign(nl, 0);
    light_cdf.assign(nl, 0);
    light_areas.assign(nl, 0);
    area_cdf_begin.assign(nl, 0);
    area_cdf_pool.clear();
    double total = 0;
    for (int l = 0; l < nl; ++l) {
        const Shape<N> &s = shapes[emitters[l].shape_id];
        area_cdf_begin[l] = (int)area_cdf_pool.size();
        double sum = 0;
        for (int t = 0; t < s.nt; ++t) {
            sum += s.area(t);
            area_cdf_pool.push_back(sum);
        }
        for (int t = 0; t < s.nt; ++t) area_cdf_pool[area_cdf_begin[l] + t] /= sum;
        light_areas[l] = sum;
        light_pmf[l] = sum * luminance(emitters[l].intensity_val()) * kPi;
        total += light_pmf[l];
    }
    if (nl > 0) {
        if (!(total > 0)) return "emitters carry no power";
        for (int l = 0; l < nl; ++l) light_pmf[l] /= total;
        light_cdf[0] = light_pmf[0];
        for (int l = 1; l < nl; ++l) light_cdf[l] = light_cdf[l - 1] + light_pmf[l];
    }
    std::vector<double> w(shapes.size(), 1.0);
    if (d.edge_weights) for (size_t i = 0; i < shapes.size(); ++i) w[i] = d.edge_weights[i];
    init_edges(w);
    init_primary_edges();
    return "";
}

template <int N>
void Scene<N>::init_edges(const std::vector<double> &weights) {  // bruteforce.cpp:4-20
    edges_distrb.clear();
    std::vector<double> sw(shapes.size());
    double sum = 0;
    for (size_t i = 0; i < shapes.size(); ++i) {
        bool ignore = bsdfs[shapes[i].bsdf_id].is_null() && shapes[i].light_id < 0;
        sw[i] = (ignore ? 0.0 : shapes[i].edge_distrb.sum) * weights[i];
        sum += sw[i];
    }
    if (sum > kEps) {
        for (double v : sw) edges_distrb.append(v);
        edges_distrb.normalize();
    }
}

// line_clip.h:37-95 (Cohen-Sutherland on a dual 2-vector; the clip parameter is a plain value)
static int out_code(double x, double y, double xmin, double xmax, double ymin, double ymax) {
    int code = 0;
    if (x < xmin - kEps) code |= 1;
    else if (x > xmax + kEps) code |= 2;
    if (y < ymin - kEps) code |= 4;
    else if (y > ymax + kEps) code |= 8;
    return code;
}
template <int N>
static bool clip_line(const Dual<N> v0[2], const Dual<N> v1[2], Dual<N> c0[2], Dual<N> c1[2], double xmin,
                      double xmax, double ymin, double ymax) {
    c0[0] = v0[0]; c0[1] = v0[1]; c1[0] = v1[0]; c1[1] = v1[1];
    int o0 = out_code(c0[0].v, c0[1].v, xmin, xmax, ymin, ymax), o1 = out_code(c1[0].v, c1[1].v, xmin, xmax, ymin, ymax);
    for (int guard = 0; guard < 64; ++guard) {
        if (!(o0 | o1)) return true;
        if (o0 & o1) return false;
        int oo = o0 ? o0 : o1;
        double k;
        if (oo & 8) k = (ymax - c0[1].v) / (c1[1].v - c0[1].v);
        else if (oo & 4) k = (ymin - c0[1].v) / (c1[1].v - c0[1].v);
        else if (oo & 2) k = (xmax - c0[0].v) / (c1[0].v - c0[0].v);
        else k = (xmin - c0[0].v) / (c1[0].v - c0[0].v);
        Dual<N> p[2] = {c0[0] + (c1[0] - c0[0]) * k, c0[1] + (c1[1] - c0[1]) * k};
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

template <int N>
void Scene<N>::init_primary_edges() {  // edge_manager.cpp:6-110
    primary_edges.clear();
    primary_distrb.clear();
    const V3 cp = val(cam.cpos);
    const V3 cn = val(cam.cframe.n);
    double fov = cam.c2ndc.m[0];
    double aspect = (double)cam.width / (double)cam.height;
    for (const Shape<N> &s : shapes) {
        if (bsdfs[s.bsdf_id].is_null() && s.light_id < 0) continue;
        for (const Edge &e : s.edges) {
            if (s.is_silhouette(e, cp) <= 0) continue;
            DV3<N> v0 = s.verts[e.v0], v1 = s.verts[e.v1];
            double clip_near = (double)cam.clip_near;
            double z0 = dot(val(v0) - cp, cn), z1 = dot(val(v1) - cp, cn);
            if (z0 < clip_near && z1 < clip_near) continue;
            if (z0 < clip_near) v0 = v0 + (v1 - v0) * ((clip_near - z0) / (z1 - z0));
            else if (z1 < clip_near) v1 = v1 + (v0 - v1) * ((clip_near - z1) / (z0 - z1));
            V3 v0_local = xfm_point(cam.w2c, val(v0)), v1_local = xfm_point(cam.w2c, val(v1));
            v0 = (v0 - cam.cpos) / dot(v0 - cam.cpos, cam.cframe.n);
            v1 = (v1 - cam.cpos) / dot(v1 - cam.cpos, cam.cframe.n);
            v0 = cam.cframe.to_local(v0);
            v1 = cam.cframe.to_local(v1);
            Dual<N> r0[2] = {v0.x * fov * 0.5 + 0.5, v0.y * fov * (-0.5) * aspect + 0.5};
            Dual<N> r1[2] = {v1.x * fov * 0.5 + 0.5, v1.y * fov * (-0.5) * aspect + 0.5};
            double xmin = 0, xmax = 1, ymin = 0, ymax = 1;
            if (cam.cropped()) {
                xmin = (double)(float)((float)cam.crop_x / cam.width);
                xmax = (double)(float)((float)(cam.crop_x + cam.crop_w) / cam.width);
                ymin = (double)(float)((float)cam.crop_y / cam.height);
                ymax = (double)(float)((float)(cam.crop_y + cam.crop_h) / cam.height);
            }
            Dual<N> c0[2], c1[2];
            if (!clip_line<N>(r0, r1, c0, c1, xmin, xmax, ymin, ymax)) continue;
            V3 v0_plane = val(v0), v1_plane = val(v1);
            V3 t0v = v0_local, t1v = v1_local;
            if (std::hypot(r0[0].v - c0[0].v, r0[1].v - c0[1].v) > kEps) {
                V3 pc((c0[0].v - 0.5) * 2.0 / fov, (c0[1].v - 0.5) * (-2.0) / (aspect * fov), 1.0);
                double t0 = norm(pc - val(v0)) / norm(val(v1) - val(v0));
                v0_plane = val(v0) + (val(v1) - val(v0)) * t0;
                double t1 = compute_intersection_in_tri(V3(), val(v0), val(v1), t0v, t1v, t0);
                v0_local = t0v + (t1v - t0v) * t1;
            }
            if (std::hypot(r1[0].v - c1[0].v, r1[1].v - c1[1].v) > kEps) {
                V3 pc((c1[0].v - 0.5) * 2.0 / fov, (c1[1].v - 0.5) * (-2.0) / (aspect * fov), 1.0);
                double t0 = norm(pc - val(v0)) / norm(val(v1) - val(v0));
                v1_plane = val(v0) + (val(v1) - val(v0)) * t0;
                double t1 = compute_intersection_in_tri(V3(), val(v0), val(v1), t0v, t1v, t0);
                v1_local = t0v + (t1v - t0v) * t1;
            }
            PrimaryEdge<N> pe;
            pe.v0s[0] = c0[0] * (double)cam.width; pe.v0s[1] = c0[1] * (double)cam.height;
            pe.v1s[0] = c1[0] * (double)cam.width; pe.v1s[1] = c1[1] * (double)cam.height;
            pe.v0p = v0_plane; pe.v1p = v1_plane; pe.v0c = v0_local; pe.v1c = v1_local;
            primary_edges.push_back(pe);
            primary_distrb.append(std::hypot(pe.v0s[0].v - pe.v1s[0].v, pe.v0s[1].v - pe.v1s[1].v));
        }
    }
    if (primary_distrb.size() > 0) primary_distrb.normalize();
}

template <int N>
double Scene<N>::sample_primary_edge(double rnd, int &px, int &py, Dual<N> p[2], double nrm[2]) const {
    // edge_manager.cpp:112-134
    int idx = (int)primary_distrb.sample_reuse(rnd);
    const PrimaryEdge<N> &e = primary_edges[idx];
    p[0] = e.v0s[0] + (e.v1s[0] - e.v0s[0]) * rnd;
    p[1] = e.v0s[1] + (e.v1s[1] - e.v0s[1]) * rnd;
    double fov = cam.c2ndc.m[0], aspect = (double)cam.width / (double)cam.height;
    V3 tmp((p[0].v / cam.width - 0.5) * 2.0 / fov, (p[1].v / cam.height - 0.5) * (-2.0) / (aspect * fov), 1.0);
    px = (int)std::floor(p[0].v);
    py = (int)std::floor(p[1].v);
    double nx = e.v1s[1].v - e.v0s[1].v, ny = e.v0s[0].v - e.v1s[0].v, nl = std::hypot(nx, ny);
    nrm[0] = nx / nl;
    nrm[1] = ny / nl;
    p[0].v -= px;
    p[1].v -= py;
    double t0 = norm(tmp - e.v0p) / norm(e.v1p - e.v0p);
    double t1 = compute_intersection_in_tri(V3(), e.v0p, e.v1p, e.v0c, e.v1c, t0);
    return norm(e.v0c + (e.v1c - e.v0c) * t1);
}

template <int N>
const Edge *Scene<N>::sample_edge(const V3 &, double &rnd, int &shape_id, double &pdf) const {
    // bruteforce.cpp:22-26 + shape.cpp:337-342
    shape_id = (int)edges_distrb.sample_reuse(rnd, pdf);
    double pdf1;
    const Shape<N> &s = shapes[shape_id];
    int k = (int)s.edge_distrb.sample_reuse(rnd, pdf1);
    pdf *= pdf1;
    return &s.edges[k];
}

// ------------------------------------------------------------------ intersection
template <int N>
bool Scene<N>::trace(const V3 &o, const V3 &d, double tmin, double tmax, int &shape, int &prim, double &t) const {
    int g = bvh.closest(o, d, tmin, tmax, t);
    if (g < 0) return false;
    shape = tri_shape[g];
    prim = tri_prim[g];
    return true;
}

template <int N>
void Scene<N>::shape_intersect(int shape, int prim, const Ray &ray, Its &its) const {
    const Shape<N> &s = shapes[shape];
    const auto &f = s.idx[prim];
    V3 uvt = ray_intersect_triangle(s.vert(f[0]), s.vert(f[1]), s.vert(f[2]), ray.o, ray.d);
    double u = uvt.x, v = uvt.y, w = 1.0 - (u + v), t = uvt.z;
    V3 gn = val(s.face_normals[prim]), shn = gn;
    if (s.has_normals()) {
        V3 nn = val(s.normals[f[0]]) * w + val(s.normals[f[1]]) * u + val(s.normals[f[2]]) * v;
        shn = normalized(nn);
        if (dot(gn, shn) < 0.0) gn = -gn;
    }
    its.shape = shape;
    its.geo = Frame(gn);
    its.sh = Frame(shn);
    its.p = ray.o + ray.d * t;
    its.t = t;
    its.wi = its.sh.to_local(-ray.d);
}

template <int N>
void Scene<N>::shape_intersect_ad(int shape, int prim, const RayAD<N> &ray, ItsAD<N> &its) const {
    const Shape<N> &s = shapes[shape];
    const auto &f = s.idx[prim];
    DV3<N> uvt = ray_intersect_triangle(s.verts[f[0]], s.verts[f[1]], s.verts[f[2]], ray.o, ray.d);
    Dual<N> u = uvt.x, v = uvt.y, w = 1.0 - (u + v), t = uvt.z;
    DV3<N> gn = s.face_normals[prim], shn = gn;
    if (s.has_normals()) {
        DV3<N> nn = s.normals[f[0]] * w + s.normals[f[1]] * u + s.normals[f[2]] * v;
        shn = normalized(nn);
        if (dot(gn, shn).v < 0.0) gn = -gn;
    }
    its.shape = shape;
    its.geo = FrameT<Dual<N>>(gn);
    its.sh = FrameT<Dual<N>>(shn);
    its.p = ray.o + ray.d * t;
    its.t = t;
    its.wi = its.sh.to_local(-ray.d);
}

template <int N>
bool Scene<N>::ray_intersect(const Ray &ray, bool on_surface, Its &its) const {
    int s, p;
    double t;
    if (!trace(ray.o, ray.d, on_surface ? kShadowEps : 0.0, INFINITY, s, p, t)) {
        its.shape = -1;
        its.t = INFINITY;
        return false;
    }
    shape_intersect(s, p, ray, its);
    return true;
}

template <int N>
bool Scene<N>::ray_intersect_ad(const RayAD<N> &ray, bool on_surface, ItsAD<N> &its) const {
    int s, p;
    double t;
    V3 o = val(ray.o), d = val(ray.d);
    if (!trace(o, d, on_surface ? kShadowEps : 0.0, INFINITY, s, p, t)) {
        its.shape = -1;
        its.t = Dual<N>(INFINITY);
        return false;
    }
    shape_intersect_ad(s, p, ray, its);
    return true;
}

// ------------------------------------------------------------------ media
template <int N>
V3 Scene<N>::sig_s(int med, const V3 &x) const {
    const Medium<N> &m = media[med];
    if (m.type == DTRT_MEDIUM_HOMOGENEOUS) return m.sigma_s;
    return val(m.albedo) * (m.scale.v * m.density.lookup(x));  // heterogeneous.h:88-90
}

template <int N>
bool Scene<N>::sample_distance(int med, Ray &ray, double tmax, const double rnd2[2], Rng &rng, V3 &thr) const {
    const Medium<N> &m = media[med];
    if (m.type == DTRT_MEDIUM_HOMOGENEOUS) {  // homogeneous.cpp:6-24
        if (m.sampling_weight > kEps) {
            double t = -std::log(rnd2[0]) / m.sigma_t.v;
            if (t < tmax) {
                ray.o = ray.at(t);
                if (rnd2[1] < m.sampling_weight) thr = cmul(thr, val(m.albedo) / m.sampling_weight);
                else thr = V3();
                return true;
            }
            return false;
        }
        thr = thr * std::exp(-tmax * m.sigma_t.v);
        return false;
    }
    // heterogeneous.cpp:9-37 delta tracking against the global majorant
    double tn, tf;
    if (!m.density.aabb.ray_intersect(ray.o, ray.d, tn, tf)) return false;
    tn = std::max(tn, 0.0);
    tf = std::min(tf, tmax);
    double t = tn;
    for (long dep = 0;; ++dep) {
        t -= std::log(rng.next1()) * m.max_inv_density;
        if (t > tf) break;
        if (dep > tracking_cap) break;
        V3 p = ray.at(t);
        double dens = m.density.lookup(p);
        if (rng.next1() * m.density.max_value < dens) {
            ray.o = p;
            thr = cmul(thr, m.albedo_vol.valid ? m.albedo_vol.lookup3(p) : val(m.albedo));
            return true;
        }
    }
    return false;
}

template <int N>
void Scene<N>::int_sig_t(const Medium<N> &m, const RayAD<N> &ray, const Dual<N> &tmin, const Dual<N> &tmax, Rng &rng,
                         double out[N]) const {  // heterogeneous.cpp:121-141
    for (int j = 0; j < N; ++j) out[j] = 0;
    double len = tmax.v - tmin.v;
    for (int i = 0; i < 10; ++i) {
        double r = (i + rng.next1()) / 10.0;
        Dual<N> s = m.scale * m.density.lookup_ad(ray.at(tmin + len * r));
        for (int j = 0; j < N; ++j) out[j] += s.d[j];
    }
    for (int j = 0; j < N; ++j) out[j] *= len / 10.0;
    Ray r0 = ray.plain();
    if (!tmax.der_is_zero(kEps)) {
        double dv = m.scale.v * m.density.lookup(r0.at(tmax.v - kEps));
        for (int j = 0; j < N; ++j) out[j] += tmax.d[j] * dv;
    }
    if (!tmin.der_is_zero(kEps)) {
        double dv = m.scale.v * m.density.lookup(r0.at(tmin.v + kEps));
        for (int j = 0; j < N; ++j) out[j] -= tmin.d[j] * dv;
    }
}

template <int N>
bool Scene<N>::sample_distance_ad(int med, RayAD<N> &ray, const Dual<N> &tmax, const double rnd2[2], Rng &rng,
                                  DV3<N> &thr) const {
    const Medium<N> &m = media[med];
    if (m.type == DTRT_MEDIUM_HOMOGENEOUS) {  // homogeneous.cpp:27-49
        if (m.sampling_weight > kEps) {
            double t = -std::log(rnd2[0]) / m.sigma_t.v;
            if (t < tmax.v) {
                ray.o = ray.at(t);
                if (rnd2[1] < m.sampling_weight) {
                    Dual<N> tmp = m.sigma_t * d_exp(-t * m.sigma_t);
                    Dual<N> k = tmp / (tmp.v * m.sampling_weight);
                    thr = cmul(thr, m.albedo * k);
                } else {
                    thr = DV3<N>();
                }
                return true;
            }
            Dual<N> tmp = d_exp(-tmax * m.sigma_t);
            thr = thr * (tmp / tmp.v);
            return false;
        }
        thr = thr * d_exp(-tmax * m.sigma_t);
        return false;
    }
    // heterogeneous.cpp:40-75
    double tn, tf;
    Ray r0 = ray.plain();
    if (!m.density.aabb.ray_intersect(r0.o, r0.d, tn, tf)) return false;
    tn = std::max(tn, 0.0);
    tf = std::min(tf, tmax.v);
    double t = tn;
    for (long dep = 0;; ++dep) {
        t -= std::log(rng.next1()) * m.max_inv_density;
        if (t > tf) break;
        if (dep > tracking_cap) break;
        DV3<N> p = ray.at(t);
        Dual<N> dens = m.density.lookup_ad(p);
        if (rng.next1() * m.density.max_value < dens.v) {
            // The reference passes ray.org as p_scatter while `ray` is the same object
            // (volpathAD.cpp:164), so intSigT below integrates from the scatter point
            // forward over [0, t]. That aliasing is part of the estimator and is kept.
            const RayAD<N> ray0 = ray;
            ray.o = p;
            DV3<N> alb = m.albedo_vol.valid ? m.albedo_vol.lookup3_ad(p) : m.albedo;
            Dual<N> sig = m.scale * dens;
            double ist[N];
            int_sig_t(m, (est_flags & DTRT_EST_SCATTER_SEGMENT_FROM_ORIGIN) ? ray0 : ray, Dual<N>(0.0), Dual<N>(t), rng,
                      ist);
            Dual<N> tmp(1.0);
            for (int j = 0; j < N; ++j) tmp.d[j] = -ist[j];
            thr = cmul(thr, alb * (sig * tmp / sig.v));
            return true;
        }
    }
    double ist[N];
    int_sig_t(m, ray, Dual<N>(0.0), tmax, rng, ist);
    Dual<N> tmp(1.0);
    for (int j = 0; j < N; ++j) tmp.d[j] = -ist[j];
    thr = thr * tmp;
    return false;
}

template <int N>
double Scene<N>::medium_transmittance(int med, const Ray &ray, double tmin, double tmax, Rng &rng) const {
    const Medium<N> &m = media[med];
    if (m.type == DTRT_MEDIUM_HOMOGENEOUS) return std::exp((tmin - tmax) * m.sigma_t.v);  // homogeneous.cpp:52-55
    // heterogeneous.cpp:78-91 residual ratio tracking
    double ret = 1.0, t = tmin;
    long steps = 0;
    while (ret > kEps) {
        t -= std::log(rng.next1()) * m.max_inv_density;
        if (t > tmax) break;
        if (++steps > tracking_cap) break;
        ret *= 1.0 - m.density.lookup(ray.at(t)) / m.density.max_value;
    }
    return ret;
}

template <int N>
Dual<N> Scene<N>::medium_transmittance_ad(int med, const RayAD<N> &ray, const Dual<N> &tmin, const Dual<N> &tmax,
                                          Rng &rng) const {
    const Medium<N> &m = media[med];
    if (m.type == DTRT_MEDIUM_HOMOGENEOUS) return d_exp((tmin - tmax) * m.sigma_t);  // homogeneous.cpp:57-59
    Dual<N> ret(medium_transmittance(med, ray.plain(), tmin.v, tmax.v, rng));  // heterogeneous.cpp:113-118
    double ist[N];
    int_sig_t(m, ray, tmin, tmax, rng, ist);
    for (int j = 0; j < N; ++j) ret.d[j] = -ret.v * ist[j];
    return ret;
}

#define ORC_INSTANTIATE(N) \
    template struct Shape<N>;  \
    template struct Grid<N>;   \
    template struct Camera<N>; \
    template struct Scene<N>;
ORC_INSTANTIATE(1)
ORC_INSTANTIATE(3)
ORC_INSTANTIATE(4)
ORC_INSTANTIATE(8)

}  // namespace orc
