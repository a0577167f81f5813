// dtrt_gb300 — device-resident scene layout (plain structs shared by host and device).
//
// Layout in HBM (all arrays are struct-of-arrays over a global vertex / triangle
// numbering; shape s owns vertices [vert_off, vert_off+nv) and triangles
// [tri_off, tri_off+nt)):
//   verts      float4[num_verts]            xyz value
//   vert_der   float[num_verts][nder][3]    vertex velocities (NULL: static geometry)
//   normals    float4[num_verts]            shading normals (shapes with normals only)
//   tris       int4[num_tris]               global vertex ids + shape id
//   face_n     float4[num_tris]             normalised geometric normal value
//   face_n_der float[num_tris][nder][3]     its derivative (NULL: static geometry)
//   nodes      BvhNode[num_nodes]           2-wide BVH, 64 B per node
//   leaf_tris  float4[3*num_tris]           (v0, tri id) (e1, 0) (e2, 0) in leaf order
// Materials, media and emitters are small arrays of the structs below with their
// derivative slots inline (kMaxNder).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dt {

constexpr int kMaxNder = 8;
constexpr int kStackDepth = 48;   // BVH traversal stack entries per thread
constexpr int kBlock = 128;       // threads per block of every path kernel

enum { BSDF_NULL = 0, BSDF_DIFFUSE = 1, BSDF_PHONG = 2, BSDF_ROUGHDIELECTRIC = 3 };
enum { PHASE_ISOTROPIC = 0, PHASE_HG = 1 };
enum { EMITTER_AREA = 0, EMITTER_AREA_EX = 1 };
enum { MEDIUM_HOMOGENEOUS = 0, MEDIUM_HETEROGENEOUS = 1 };
enum {
    MODE_EMISSION = 0x01, MODE_SURFACE_MAIN = 0x02, MODE_SURFACE_BOUNDARY = 0x04,
    MODE_VOLUME_MAIN = 0x08, MODE_VOLUME_BOUNDARY1 = 0x10, MODE_VOLUME_BOUNDARY2 = 0x20, MODE_ALL = 0x3f
};

struct DevBsdf {
    int type;
    float diffuse[3], specular[3], exponent, alpha, eta, inv_eta, spec_weight;
    float d_diffuse[kMaxNder][3], d_specular[kMaxNder][3], d_exponent[kMaxNder];
    float d_alpha[kMaxNder], d_eta[kMaxNder], d_inv_eta[kMaxNder];
    int has_der;  // any non-zero derivative slot (else the plain evaluation is exact)
};

struct DevPhase {
    int type;
    float g;
    float d_g[kMaxNder];
    int has_der;  // any non-zero derivative slot
};

struct DevEmitter {
    int type, shape_id, two_sided;
    float intensity[3], kappa;
    float d_intensity[kMaxNder][3], d_kappa[kMaxNder];
};

struct DevGrid {
    const float *data;   // [rz][ry][rx][channels]
    int res[3], channels, valid;
    float mn[3], to_grid[3];       // grid coordinate = (p_volume - mn) * to_grid
    float w2v[12], v2w[12];        // row-major 3x4
    float center[3], lo[3], hi[3]; // rotation centre and world AABB
    float max_value;
    float trans_vel[kMaxNder][3], rot_vel[kMaxNder][3];
    int moving;  // any non-zero velocity slot
    // per-voxel derivative directions (density grids only): [voxel][dgrid_n]; slot j of a
    // lookup's derivative gains the trilinear interpolation of direction j. NULL: none.
    const float *dgrid;
    int dgrid_n;
};

struct DevMedium {
    int type, phase_id;
    float sigma_t, d_sigma_t[kMaxNder];
    float albedo[3], d_albedo[kMaxNder][3];
    float sigma_s[3], sampling_weight;
    float scale, d_scale[kMaxNder], max_inv_density;
    DevGrid density, albedo_vol;
    long long grad_off;  // offset of this medium's voxels in the adjoint density gradient (-1: none)
};

struct DevShape {
    int vert_off, tri_off, nv, nt;
    int light_id, bsdf_id, med_int, med_ext;
    int has_normals;
    int edge_off, num_edges, edge_cdf_off;
};

struct DevCamera {
    int width, height, crop_x, crop_y, crop_w, crop_h, med_id;
    float clip_near, fov;  // fov = cam_to_ndc(0,0)
    float c2w[12];       // row-major 3x4
    float ndc2cam[9];
    float cpos[3], cframe[3][3];              // frame rows: s, t, n
    float d_cpos[kMaxNder][3], d_cframe[kMaxNder][3][3];
    // reciprocals of the divisions on every camera ray and primary-edge sample (the FP64
    // pipe runs at 1/64 of FP32: one division is about ten of its instructions)
    double inv_w, inv_h;     // 1 / width, 1 / height
    double ndc_ky;           // -2 / aspect
    double plane_kx, plane_ky;  // 2 / fov, -2 / (aspect fov): pixel to image plane
};

struct DevEdge {
    int v0, v1, f0, f1;  // global vertex / triangle ids (f1 = -1 for a boundary edge)
    int shape;
    float length;
};

struct DevPrimaryEdge {
    double v0s[2], v1s[2];               // screen position in pixels
    float d0[kMaxNder][2], d1[kMaxNder][2];
    double v0p[3], v1p[3], v0c[3], v1c[3]; // image plane and camera-space endpoints
    // per-edge constants of the edge-point solve (utils.cpp:256-266): unit screen-space
    // normal, 1 / |v1p - v0p|, |v0p| / |v0c| and |v1p| / |v1c|
    double n[2], inv_lenp, cb, cc;
};

struct __align__(16) BvhNode {
    float4 x, y, z;  // (left.lo, left.hi, right.lo, right.hi) per axis
    int4 child;      // child[0..1]: >= 0 inner node, < 0 leaf = ~(first << 3 | (count-1))
};

struct DevScene {
    int nder;
    int num_shapes, num_tris, num_verts, num_nodes;
    const DevShape *shapes;
    const float4 *verts;
    const float *vert_der;
    const float4 *normals;
    const float *normal_der;
    const int4 *tris;
    const float4 *face_n;
    const float *face_n_der;
    const BvhNode *nodes;
    const float4 *leaf_tris;
    const DevBsdf *bsdfs;
    const DevPhase *phases;
    const DevEmitter *emitters;
    const DevMedium *media;
    int num_bsdfs, num_phases, num_emitters, num_media;
    // light sampling, scene.cpp:45-98
    const float *light_cdf, *light_pmf, *light_area, *area_cdf;
    const int *area_cdf_begin;
    // secondary edges, bruteforce.cpp + shape.cpp:254-300
    const DevEdge *edges;
    const double *edge_cdf;        // per shape: num_edges+1 entries at edge_cdf_off
    const double *shape_edge_cdf;  // num_shapes+1 entries
    int has_edges;
    // primary edges, edge_manager.cpp
    const DevPrimaryEdge *pedges;
    const float *pedge_jac;        // [num_pedges][end][x,y][6]: screen-point Jacobian (pixels) w.r.t. (v0, v1)
    const int *pedge_verts;        // [num_pedges][2] global vertex ids of the edge
    const double *pedge_cdf;       // num_pedges+1 entries
    int num_pedges;
    double pedge_sum;
    DevCamera cam;
    int tracking_cap;
    int moving_geometry;           // any vertex velocity present
    int has_grid_media;            // a heterogeneous medium exists (transmittance is a random estimate)
    unsigned est_flags;            // estimator variants, EST_* (0: the reference's estimator)
    unsigned int *error_flags;     // device flags: bit0 stack overflow, bit1 tracking cap, bit2 queue overflow
};

enum { ERR_STACK = 1u, ERR_TRACK_CAP = 2u, ERR_QUEUE = 4u };
// EST_SCATTER_FROM_ORIGIN: the free-flight derivative integral of a scatter event runs over
// [ray origin, scatter point] instead of the reference's [scatter point, scatter point + t*d]
enum { EST_SCATTER_FROM_ORIGIN = 1u };

}  // namespace dt
