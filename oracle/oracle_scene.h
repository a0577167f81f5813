// TEST INFRASTRUCTURE — CPU oracle scene model (see oracle_math.h header note).
//
// FP64 restatement of the reference's scene layer (uci-rendering/dtrt):
//   src/shape.cpp, src/camera.cpp, src/bsdf*.cpp, src/bsdf/microfacet.h,
//   src/emitter/area*.cpp, include/phase.h, src/medium/*.cpp, src/medium/gridvolume.h,
//   src/edge_manager/*.cpp, include/line_clip.h, src/scene.cpp (minus Embree, which is
//   replaced by the FP64 BVH below returning the same (shape, primitive) identity).
#pragma once
#include <map>
#include <string>

#include "../include/dtrt_gb300.h"
#include "oracle_math.h"

namespace orc {

// src/math_func.cpp:6-54 — erf (Abramowitz & Stegun 7.1.26) and erfinv (Giles)
double approx_erf(double x);
double approx_erfinv(double x);

// ------------------------------------------------------------------ edges
// include/edge_manager.h:14-26
struct Edge {
    int v0, v1, f0, f1;
    double length;
};

// ------------------------------------------------------------------ shapes
template <int N>
struct Shape {
    std::vector<DV3<N>> verts, normals, face_normals;
    std::vector<std::array<int, 3>> idx;
    int nv = 0, nt = 0, light_id = -1, bsdf_id = -1, med_int = -1, med_ext = -1;
    std::vector<Edge> edges;
    Distrib edge_distrb;
    bool has_normals() const { return !normals.empty(); }
    bool is_emitter() const { return light_id >= 0; }
    bool is_medium_transition() const { return med_ext >= 0 || med_int >= 0; }
    const V3 vert(int i) const { return val(verts[i]); }
    void compute_face_normals();   // shape.cpp:109-126
    void construct_edges();        // shape.cpp:254-300
    double area(int t) const;      // shape.cpp:135-141
    void sample_position(int t, double u, double v, V3 &pos, V3 &n) const;  // shape.cpp:151-164
    int is_silhouette(const Edge &e, const V3 &p) const;                  // shape.cpp:302-335
};

// ------------------------------------------------------------------ BSDF
template <int N>
struct Bsdf {
    int type = DTRT_BSDF_NULL;
    DV3<N> diffuse, specular;
    Dual<N> exponent;
    double spec_weight = 0;
    Dual<N> alpha, eta, inv_eta;
    bool is_null() const { return type == DTRT_BSDF_NULL; }
    bool is_transmissive() const { return type == DTRT_BSDF_NULL || type == DTRT_BSDF_ROUGHDIELECTRIC; }
};

template <int N>
struct Phase {
    int type = DTRT_PHASE_ISOTROPIC;
    Dual<N> g;
};

template <int N>
struct Emitter {
    int type = DTRT_EMITTER_AREA;
    int shape_id = -1;
    DV3<N> intensity;
    Dual<N> kappa;
    bool two_sided = false;
    V3 intensity_val() const { return val(intensity); }
};

// src/medium/gridvolume.h:15-351 (single- or three-channel grid with rigid motion)
template <int N>
struct Grid {
    bool valid = false;
    int res[3] = {0, 0, 0};
    int channels = 0;
    V3 mn, mx, extent, center;
    AABB aabb;
    std::vector<float> data;
    double max_value = 0;
    M4 v2w, w2v;
    V3 trans_vel[N], rot_vel[N];
    // per-voxel derivative directions [voxel][N] (extension, no reference counterpart):
    // derivative slot j of lookup_ad gains the trilinear interpolation of direction j
    std::vector<float> dgrid;
    // the 2x2x2 stencil at grid coordinate (x, y, z) lies inside the grid; false for
    // NaN / inf as well (gridvolume.h:152-153 reads out of range as 0)
    bool in_cell_range(double x, double y, double z) const {
        return x >= 0.0 && x < res[0] - 1 && y >= 0.0 && y < res[1] - 1 && z >= 0.0 && z < res[2] - 1;
    }
    void configure();
    V3 to_grid(const V3 &pw) const;
    DV3<N> to_grid_ad(const DV3<N> &pw) const;
    double lookup(const V3 &p) const;
    Dual<N> lookup_ad(const DV3<N> &p) const;
    V3 lookup3(const V3 &p) const;
    DV3<N> lookup3_ad(const DV3<N> &p) const;
};

template <int N>
struct Medium {
    int type = DTRT_MEDIUM_HOMOGENEOUS;
    int phase_id = 0;
    // homogeneous.h:11-58
    Dual<N> sigma_t;
    DV3<N> albedo;
    V3 sigma_s;
    double sampling_weight = 0;
    // heterogeneous.h:12-107
    Dual<N> scale;
    Grid<N> density, albedo_vol;
    double max_inv_density = 0;
};

// ------------------------------------------------------------------ rays / hits
struct Ray {
    V3 o, d;
    V3 at(double t) const { return o + d * t; }
};
template <int N>
struct RayAD {
    DV3<N> o, d;
    DV3<N> at(const Dual<N> &t) const { return o + d * t; }
    DV3<N> at(double t) const { return o + d * t; }
    Ray plain() const { return Ray{val(o), val(d)}; }
};

struct Its {  // include/intersection.h:15-58
    int shape = -1;
    double t = INFINITY;
    V3 p, wi;
    Frame geo, sh;
    bool valid() const { return shape >= 0; }
    V3 to_world(const V3 &v) const { return sh.to_world(v); }
    V3 to_local(const V3 &v) const { return sh.to_local(v); }
};
template <int N>
struct ItsAD {  // include/intersectionAD.h:8-56
    int shape = -1;
    Dual<N> t = Dual<N>(INFINITY);
    DV3<N> p, wi;
    FrameT<Dual<N>> geo, sh;
    bool valid() const { return shape >= 0; }
    Its plain() const {
        Its r;
        r.shape = shape; r.t = t.v; r.p = val(p); r.wi = val(wi); r.geo = val(geo); r.sh = val(sh);
        return r;
    }
    DV3<N> to_world(const DV3<N> &v) const { return sh.to_world(v); }
    DV3<N> to_local(const DV3<N> &v) const { return sh.to_local(v); }
};

// ------------------------------------------------------------------ BVH (Embree substitute)
struct Bvh {
    struct Node {
        AABB box;
        int left = -1, right = -1, first = 0, count = 0;
    };
    std::vector<Node> nodes;
    std::vector<int> tri_order;                 // leaf order -> global triangle
    std::vector<std::array<V3, 3>> tri_verts;   // per global triangle (FP64)
    void build(const std::vector<std::array<V3, 3>> &tris);
    // closest hit with t in [tmin, tmax]; returns global triangle or -1
    int closest(const V3 &o, const V3 &d, double tmin, double tmax, double &t_hit) const;
};

// ------------------------------------------------------------------ primary edges
template <int N>
struct PrimaryEdge {  // include/edge_manager.h:28-33
    Dual<N> v0s[2], v1s[2];
    V3 v0p, v1p, v0c, v1c;
};

template <int N>
struct Camera {  // include/camera.h:29-55
    int width = 0, height = 0;
    int crop_x = 0, crop_y = 0, crop_w = -1, crop_h = -1;
    M4 c2w, w2c;
    M3 c2ndc, ndc2cam;
    DV3<N> cpos;
    FrameT<Dual<N>> cframe;
    float clip_near = 1e-2f;
    int med_id = -1;
    bool cropped() const { return crop_w > 0 && crop_h > 0; }
    Ray sample_primary_ray(double x, double y) const;             // camera.cpp:52-60
    Ray sample_primary_ray(int px, int py, double fx, double fy) const;  // camera.cpp:40-50
    RayAD<N> sample_primary_ray_ad(double x, double y) const;    // camera.cpp:75-83
};

template <int N>
struct Scene {
    Camera<N> cam;
    std::vector<Shape<N>> shapes;
    std::vector<Bsdf<N>> bsdfs;
    std::vector<Emitter<N>> emitters;
    std::vector<Phase<N>> phases;
    std::vector<Medium<N>> media;
    // scene.cpp:45-98 light sampling tables
    std::vector<double> light_pmf, light_cdf, light_areas, area_cdf_pool;
    std::vector<int> area_cdf_begin;
    // BVH over all triangles; global triangle id -> (shape, prim)
    Bvh bvh;
    std::vector<int> tri_shape, tri_prim;
    // edge managers
    Distrib edges_distrb;  // bruteforce.cpp:4-20
    std::vector<PrimaryEdge<N>> primary_edges;
    Distrib primary_distrb;
    long tracking_cap = 10000;  // heterogeneous.cpp:6
    // DTRT_EST_SCATTER_SEGMENT_FROM_ORIGIN: integrate the scatter-event derivative over the
    // segment travelled instead of the reference's aliased one (extension, default off)
    unsigned est_flags = 0;

    std::string build(const dtrt_scene_desc &desc);
    void init_edges(const std::vector<double> &weights);
    void init_primary_edges();

    // geometry queries, scene.cpp
    bool trace(const V3 &o, const V3 &d, double tmin, double tmax, int &shape, int &prim, double &t) const;
    void shape_intersect(int shape, int prim, const Ray &ray, Its &its) const;          // shape.cpp:166-208
    void shape_intersect_ad(int shape, int prim, const RayAD<N> &ray, ItsAD<N> &its) const;  // 210-252
    bool ray_intersect(const Ray &ray, bool on_surface, Its &its) const;               // 538-575
    bool ray_intersect_ad(const RayAD<N> &ray, bool on_surface, ItsAD<N> &its) const;  // 577-615
    double eval_transmittance(const Ray &ray, bool on_surface, int med, double remaining, Rng &rng,
                              int max_interactions) const;  // 177-237
    V3 sample_attenuated_emitter_direct(const V3 &p, const double rnd[4], Rng &rng, int med, int max_interactions,
                                        V3 &wo, double &pdf) const;  // 399-426
    V3 sample_attenuated_emitter_direct(const Its &its, const double rnd[4], Rng &rng, int med, int max_interactions,
                                        V3 &wo, double &pdf, bool flag = false) const;  // 456-491
    DV3<N> sample_attenuated_emitter_direct_ad(const DV3<N> &p, const double rnd[4], Rng &rng, int med,
                                               int max_interactions, DV3<N> &wo, double &pdf) const;  // 428-454
    DV3<N> sample_attenuated_emitter_direct_ad(const ItsAD<N> &its, const double rnd[4], Rng &rng, int med,
                                               int max_interactions, DV3<N> &wo, double &pdf) const;  // 493-524
    V3 ray_intersect_and_look_for_emitter(const Ray &ray, bool on_surface, Rng &rng, int med, int max_interactions,
                                          Its &its, double &pdf_nee) const;  // 617-701
    DV3<N> ray_intersect_and_look_for_emitter_ad(const RayAD<N> &ray, bool on_surface, Rng &rng, int med,
                                                 int max_interactions, ItsAD<N> &its, double &pdf_nee,
                                                 ItsAD<N> *its_far = nullptr) const;  // 703-793
    int sample_light(const double rnd[4], V3 &pos, V3 &n, double &pdf) const;

    // materials
    int target_medium(const Its &its, const V3 &d) const {
        const Shape<N> &s = shapes[its.shape];
        return dot(d, its.geo.n) > 0 ? s.med_ext : s.med_int;
    }
    V3 le(const Its &its, const V3 &w) const;               // area.cpp:5-7, area2.cpp:5-11
    DV3<N> le_ad(const ItsAD<N> &its, const DV3<N> &w) const;
    V3 bsdf_eval(const Its &its, const V3 &wo) const;       // per-BSDF eval
    DV3<N> bsdf_eval_ad(const ItsAD<N> &its, const DV3<N> &wo) const;
    double bsdf_pdf(const Its &its, const V3 &wo) const;
    V3 bsdf_sample(const Its &its, const double rnd[3], V3 &wo, double &pdf, double &eta) const;
    DV3<N> bsdf_sample_ad(const ItsAD<N> &its, const double rnd[3], DV3<N> &wo, double &pdf, double &eta) const;
    double phase_eval(int ph, const V3 &wi, const V3 &wo) const;
    Dual<N> phase_eval_ad(int ph, const DV3<N> &wi, const DV3<N> &wo) const;
    double phase_sample(int ph, const V3 &wi, double u, double v, V3 &wo) const;
    Dual<N> phase_sample_ad(int ph, const DV3<N> &wi, double u, double v, DV3<N> &wo) const;

    // media
    bool sample_distance(int med, Ray &ray, double tmax, const double rnd2[2], Rng &rng, V3 &thr) const;
    bool sample_distance_ad(int med, RayAD<N> &ray, const Dual<N> &tmax, const double rnd2[2], Rng &rng,
                            DV3<N> &thr) const;
    double medium_transmittance(int med, const Ray &ray, double tmin, double tmax, Rng &rng) const;
    Dual<N> medium_transmittance_ad(int med, const RayAD<N> &ray, const Dual<N> &tmin, const Dual<N> &tmax,
                                    Rng &rng) const;
    void int_sig_t(const Medium<N> &m, const RayAD<N> &ray, const Dual<N> &tmin, const Dual<N> &tmax, Rng &rng,
                   double out[N]) const;
    V3 sig_s(int med, const V3 &x) const;

    // edges
    const Edge *sample_edge(const V3 &p, double &rnd, int &shape_id, double &pdf) const;
    double sample_primary_edge(double rnd, int &px, int &py, Dual<N> p[2], double nrm[2]) const;
};

}  // namespace orc
