/*
 * dtrt_gb300 — C ABI of the GB300 differentiable volumetric path tracer.
 *
 * This is the boundary a host binding (ctypes, pybind11, cgo, JNI …) calls.
 * Signatures carry plain pointers and sizes only; no C++ or torch types.
 *
 * The entry points replace, in the reference (uci-rendering/dtrt):
 *   - the scene object graph built by the pybind constructors
 *       src/dtrt.cpp:35-102 (Camera, Shape, BSDF_*, HG/Isotropic, AreaLight[Ex],
 *       Homogeneous/Heterogeneous, Scene + initEdges) and Scene::Scene
 *       src/scene.cpp:9-136;
 *   - VolPathTracerAD::render, i.e. IntegratorAD::render
 *       src/integrator/differential/integratorAD.cpp:19-166, bound at
 *       src/dtrt.cpp:148-150;
 *   - RenderOptions, include/integrator.h:10-25 and src/dtrt.cpp:104-115.
 *
 * Error convention: every entry point returns an int status (DTRT_OK == 0).
 * On failure dtrt_last_error() returns a thread-local message. Nothing aborts
 * the caller's process (the reference asserts, src/scene.cpp:568 et al.).
 *
 * Ownership: every pointer in a description is borrowed for the duration of
 * the call only; dtrt_scene_create copies what it needs to the device
 * (the reference copies at construction: src/shape.cpp:14-31,
 * src/camera.cpp:13-27).
 */
#ifndef DTRT_GB300_H
#define DTRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DTRT_ABI_VERSION 1
#define DTRT_MAX_NDER 8

enum dtrt_status {
    DTRT_OK = 0,
    DTRT_ERR_INVALID = 1,     /* bad argument or scene description            */
    DTRT_ERR_CUDA = 2,        /* a CUDA runtime call failed                    */
    DTRT_ERR_OVERFLOW = 3,    /* a device work queue ran out of capacity       */
    DTRT_ERR_UNSUPPORTED = 4, /* nder or feature not built                     */
    DTRT_ERR_IO = 5,          /* volume file could not be read                 */
    DTRT_ERR_STEP_CAP = 6,    /* a bounded device loop hit its iteration cap   */
    DTRT_ERR_NO_DEVICE = 7    /* no CUDA device visible                        */
};

enum dtrt_bsdf_type { DTRT_BSDF_NULL = 0, DTRT_BSDF_DIFFUSE = 1, DTRT_BSDF_PHONG = 2, DTRT_BSDF_ROUGHDIELECTRIC = 3 };
enum dtrt_phase_type { DTRT_PHASE_ISOTROPIC = 0, DTRT_PHASE_HG = 1 };
enum dtrt_emitter_type { DTRT_EMITTER_AREA = 0, DTRT_EMITTER_AREA_EX = 1 };
enum dtrt_medium_type { DTRT_MEDIUM_HOMOGENEOUS = 0, DTRT_MEDIUM_HETEROGENEOUS = 1 };

/* EMode bitmask, include/integratorAD.h:12-24 */
enum dtrt_mode {
    DTRT_MODE_EMISSION = 0x01,
    DTRT_MODE_SURFACE_MAIN = 0x02,
    DTRT_MODE_SURFACE_BOUNDARY = 0x04,
    DTRT_MODE_VOLUME_MAIN = 0x08,
    DTRT_MODE_VOLUME_BOUNDARY1 = 0x10,
    DTRT_MODE_VOLUME_BOUNDARY2 = 0x20,
    DTRT_MODE_ALL = 0x3f
};

/* dtrt.Camera(w, h, c2w, c2ndc, clip_near, med_id, vel) + set_rect, src/camera.cpp:8-38 */
typedef struct {
    int width, height;
    const float *cam_to_world; /* [16] row-major 4x4 */
    const float *cam_to_ndc;   /* [9]  row-major 3x3 */
    float clip_near;
    int med_id;                /* -1: camera in vacuum */
    const float *velocities;   /* NULL or [2*nder][3]: nder translations, then nder rotation axes */
    int crop_offset_x, crop_offset_y, crop_width, crop_height; /* crop_width <= 0: full frame */
} dtrt_camera_desc;

/* dtrt.Shape(V, F, UV, N, nV, nT, light_id, bsdf_id, med_int, med_ext, vel), src/shape.cpp:10-52 */
typedef struct {
    const float *vertices;   /* [nv][3] */
    const int *indices;      /* [nt][3] */
    const float *uvs;        /* NULL or [nv][2] (accepted, unused by the shading model) */
    const float *normals;    /* NULL or [nv][3] */
    int num_vertices, num_triangles;
    int light_id, bsdf_id, med_int_id, med_ext_id;
    const float *velocities; /* NULL or [nder*nv][3]; with normals, followed by [nv][3] normal velocities */
} dtrt_shape_desc;

/* BSDF_null / BSDF_diffuse / BSDF_Phong / BSDF_roughdielectric, src/dtrt.cpp:55-67 */
typedef struct {
    int type;
    float diffuse[3];        /* diffuse: reflectance; phong: diffuse reflectance */
    float specular[3];       /* phong */
    float exponent;          /* phong */
    float alpha, int_ior, ext_ior; /* roughdielectric */
    const float *d_diffuse;  /* NULL or [nder][3] */
    const float *d_specular; /* NULL or [nder][3] */
    const float *d_exponent; /* NULL or [nder] */
    const float *d_alpha;    /* NULL or [nder] */
    const float *d_eta;      /* NULL or [nder] */
} dtrt_bsdf_desc;

/* AreaLight(shape_id, I, two_sided) / AreaLightEx(shape_id, I, kappa[, dI, dK]), src/dtrt.cpp:76-81 */
typedef struct {
    int type;
    int shape_id;
    float intensity[3];
    int two_sided;
    float kappa;
    const float *d_intensity; /* NULL or [nder][3] (AreaLightEx) */
    const float *d_kappa;     /* NULL or [nder]    (AreaLightEx) */
} dtrt_emitter_desc;

/* HG(g[, dG]) / Isotropic(), src/dtrt.cpp:69-74 */
typedef struct {
    int type;
    float g;
    const float *d_g; /* NULL or [nder] */
} dtrt_phase_desc;

/* Homogeneous(...) / Heterogeneous(...), src/dtrt.cpp:83-93 */
typedef struct {
    int type;
    int phase_id;
    /* homogeneous */
    float sigma_t;
    float albedo[3];          /* also the constant albedo of a heterogeneous medium */
    const float *d_sigma_t;   /* NULL or [nder] */
    const float *d_albedo;    /* NULL or [nder][3] (both medium types) */
    /* heterogeneous density grid: a Mitsuba VOL v3 file, or arrays when the file is NULL */
    const char *density_file;
    const float *density;     /* [res_z][res_y][res_x] */
    int res[3];
    float vol_min[3], vol_max[3];
    /* optional 3-channel albedo grid (gridvolume albedo), same conventions */
    const char *albedo_file;
    const float *albedo_grid; /* [res_z][res_y][res_x][3] */
    int albedo_res[3];
    float albedo_min[3], albedo_max[3];
    float to_world[16];       /* row-major 4x4 volume-to-world */
    float density_scale;
    const float *d_density_scale;  /* NULL or [nder] */
    const float *trans_velocities; /* NULL or [nder][3] */
    const float *rot_velocities;   /* NULL or [nder][3] */
} dtrt_medium_desc;

/* Scene(camera, shapes, bsdfs, emitters, phases, media) + initEdges(w), src/scene.cpp:9-142 */
typedef struct {
    int nder;                 /* derivative slots carried per path: 1, 3, 4 or 8 */
    dtrt_camera_desc camera;
    int num_shapes;   const dtrt_shape_desc *shapes;
    int num_bsdfs;    const dtrt_bsdf_desc *bsdfs;
    int num_emitters; const dtrt_emitter_desc *emitters;
    int num_phases;   const dtrt_phase_desc *phases;
    int num_media;    const dtrt_medium_desc *media;
    const float *edge_weights; /* NULL or [num_shapes] secondary-edge sampling weights */
} dtrt_scene_desc;

/* RenderOptions(seed, spp, max_bounces, sppe, sppse, quiet[, mode[, ddistCoeff]]), include/integrator.h:10-25 */
typedef struct {
    uint64_t seed;
    int spp;          /* num_samples */
    int max_bounces;
    int sppe;         /* num_samples_primary_edge */
    int sppse;        /* num_samples_secondary_edge */
    int quiet;
    int mode;         /* < 0: all terms */
    float ddist_coeff;
} dtrt_render_options;

/* Work counters and stage timings of the last render on a scene (device counters). */
typedef struct {
    uint64_t camera_paths;
    uint64_t edge_records;    /* secondary-edge vertex records                      */
    uint64_t edge_samples;    /* secondary-edge samples evaluated                   */
    uint64_t lins_records;    /* Lins boundary records                              */
    uint64_t primary_edge_samples;
    uint64_t li_tasks;        /* non-AD sub-paths traced (edge, Lins, primary edge) */
    uint64_t rays;            /* closest-hit queries                                */
    uint64_t node_visits;     /* BVH nodes fetched                                  */
    uint64_t tri_tests;       /* triangles fetched and tested                       */
    uint64_t grid_lookups;    /* trilinear density lookups (8 voxels each)          */
    uint64_t batches;         /* camera-path chunks the render was split into       */
    uint64_t kernel_launches; /* device kernels launched by the render              */
    /* per-kernel counters, index: 0 camera, 1 edge, 2 Li, 3 Lins, 4 primary edge */
    uint64_t k_rays[5], k_node_visits[5], k_tri_tests[5], k_grid_lookups[5];
    double ms_total;
    double ms_camera;         /* camera AD path kernel(s)                           */
    double ms_edge;           /* secondary-edge kernel(s)                           */
    double ms_li;             /* Li sub-path kernel(s)                              */
    double ms_primary;        /* primary-edge kernel(s)                             */
    double ms_setup;          /* scene upload / derived data for this render        */
    int counters_enabled;
    int camera_schedule;      /* DTRT_CAMERA_MEGAKERNEL or DTRT_CAMERA_WAVEFRONT (forward renders) */
    uint64_t light_samples;   /* emitter samples (light and area CDF searches)        */
    uint64_t k_light_samples[5];
    uint64_t camera_state_bytes; /* wavefront camera stage: path-state bytes read + written */
} dtrt_render_stats;

/* Opaque scene handle (device-resident geometry, BVH, media, edge tables). */
typedef struct dtrt_scene dtrt_scene;

/* ABI version of the loaded library (DTRT_ABI_VERSION). */
int dtrt_abi_version(void);

/* Number of visible CUDA devices (0 on a machine without a GPU). */
int dtrt_device_count(void);

/* Whether nder is one of the compiled derivative widths. Replaces the compile-time
 * constant `nder` of include/config.h:5 (exported as dtrt.nder, src/dtrt.cpp:152). */
int dtrt_nder_supported(int nder);

/* Thread-local message for the last non-zero status. */
const char *dtrt_last_error(void);

/* Build a device scene: copies geometry and parameters, builds the BVH, light and
 * edge distributions. Replaces Scene::Scene (src/scene.cpp:9-136) and the
 * constructors it consumes. */
int dtrt_scene_create(const dtrt_scene_desc *desc, dtrt_scene **out);

/* Secondary-edge sampling weights per shape. Replaces Scene::initEdgesPy,
 * include/scene.h:37-39 / src/scene.cpp:138-142. */
int dtrt_scene_set_edge_weights(dtrt_scene *scene, const float *weights, int num_shapes);

/* Release the scene's own device allocations. Its render work buffers (record queues,
 * path states, accumulators; several GB at full size) are kept for the next scene created
 * on the same device, so that a loop building one scene per iteration allocates them once;
 * dtrt_release_cached_memory frees them. */
int dtrt_scene_destroy(dtrt_scene *scene);
int dtrt_release_cached_memory(void);

/* In-place rebuild of a scene from a description with the same triangles: the same nder,
 * number of shapes, per-shape vertex and triangle counts and index lists, the same number
 * of media with unchanged types and grid resolutions. Everything else (vertex positions,
 * normals, velocities, camera, materials, emitters, media values, edge weights) is taken
 * from `desc` as dtrt_scene_create would. What the rebuild reuses instead of recomputing:
 * the edge adjacency of every mesh, the BVH topology (refit bottom-up to the new positions
 * while its surface-area cost stays within 2x of its cost when last built, else built
 * again), and every device array whose size did not change (rewritten in place, so device
 * pointers stay valid). Kept from the scene: estimator flags, tracking cap, queue capacity,
 * counters and per-voxel density derivative directions. The reference builds a new scene
 * for every render (pydtrt/scene_renderer.py:110-316 -> src/scene.cpp:17-43 Embree build,
 * src/shape.cpp:254-300 edge lists); this replaces that rebuild inside an optimisation loop.
 * Waits for the device to be idle first (renders in flight may read the arrays). On any
 * error the scene is unchanged (except a DTRT_ERR_CUDA from the final device copies).
 * A batch holds a snapshot of its scenes: create it again after an update. */
#define DTRT_UPDATE_REBUILD_BVH 1u /* build the BVH again instead of refitting it */
typedef struct dtrt_update_stats {
    int bvh_refit;         /* 1: refit; 0: built again (flag or surface-area cost past the limit) */
    int buffers_reused;    /* device arrays rewritten in place */
    int buffers_allocated; /* device arrays allocated anew (their size changed) */
    float sah_ratio;       /* surface-area cost of the refit tree / cost at its last full build */
    double host_ms;        /* wall time of the update, device copies included */
    double ms_bvh;         /* of which: BVH refit or build */
    double ms_arrays;      /* of which: every other host array (geometry, edges, tables) */
    double ms_device;      /* of which: device allocations and copies */
} dtrt_update_stats;
int dtrt_scene_update(dtrt_scene *scene, const dtrt_scene_desc *desc, unsigned flags, dtrt_update_stats *stats);

/* Forward-mode render: image plus nder derivative images, float[(nder+1)][H][W][3]
 * row-major (crop size when a crop rectangle is set). `out` is a host pointer when
 * out_on_device == 0, else a device pointer. `stream` is a cudaStream_t or NULL.
 * Primary-edge contributions are added to the derivative slots, matching
 * IntegratorAD::render (integratorAD.cpp:19-166) as bound at src/dtrt.cpp:148-150.
 * The call blocks until the result is written. */
int dtrt_render_fwd(dtrt_scene *scene, const dtrt_render_options *opts, float *out,
                    int out_on_device, void *stream);

/* Forward-mode render that allocates no device memory. No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc during a render: code running under a memory
 * budget fixed at start-up, an embedding runtime that owns all device allocations, or a
 * host thread that must not take the allocator's locks. Every work buffer this render
 * needs (FP64 accumulators, task queues, counters, the staging copy of a host `out`)
 * lives in one file-scope device array of DTRT_NOALLOC_SCRATCH_BYTES (6 MiB), which every
 * GPU that loads the library keeps until the process exits.
 *
 * Limits, rejected with DTRT_ERR_INVALID and a message: at most DTRT_NOALLOC_MAX_PIXELS
 * output pixels (e.g. 64x64), max_bounces <= 31, sppse <= 8192. Results equal
 * dtrt_render_fwd's for the same seed up to the order of floating-point atomic adds.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress),
 * so make that first call before any stream capture. All calls share the one array:
 * calls whose work overlaps on the GPU (other streams, other host threads) race and
 * must be serialised by the caller. The call blocks until `out` is written. The scene's
 * device must be the current device (else DTRT_ERR_INVALID); the cached array address
 * belongs to that device's primary context and is not looked up again after a device
 * reset. The scene settings dtrt_scene_enable_counters, dtrt_scene_set_camera_schedule
 * and dtrt_scene_set_queue_capacity do not apply here: this render always runs the
 * megakernel schedule with fixed queue capacities and no work counters. */
#define DTRT_NOALLOC_MAX_PIXELS 4096
#define DTRT_NOALLOC_SCRATCH_BYTES (6u << 20)
int dtrt_render_fwd_noalloc(dtrt_scene *scene, const dtrt_render_options *opts, float *out,
                            int out_on_device, void *stream);

/* Primal render without derivatives: float[H][W][3] (crop size when cropped). Replaces
 * VolPathTracer::render (src/integrator/volpath.cpp:105-140, bound at src/dtrt.cpp:132-134):
 * `spp` jittered primary rays per pixel through VolPathTracer::radiance
 * (volpath.cpp:10-103); the pixel is written unconditionally (volpath.cpp:134-136). One
 * thread per camera path, no dual numbers; sppe, sppse, mode and ddist_coeff are ignored
 * as in the reference. `out` is host or device memory as in dtrt_render_fwd. */
int dtrt_render_primal(dtrt_scene *scene, const dtrt_render_options *opts, float *out, int out_on_device,
                       void *stream);

/* Enable (1) or disable (0) device work counters for later renders of a scene. */
int dtrt_scene_enable_counters(dtrt_scene *scene, int enable);

/* Counters and timings of the last render on the scene. */
int dtrt_scene_last_stats(const dtrt_scene *scene, dtrt_render_stats *out);

/* Maximum work-queue capacity in sub-path tasks (0 = automatic). Lets tests force
 * a small queue; an overflow is reported as DTRT_ERR_OVERFLOW, never a hang. */
int dtrt_scene_set_queue_capacity(dtrt_scene *scene, uint64_t max_tasks);

/* Iteration cap of delta / ratio tracking loops (reference: 10000,
 * src/medium/heterogeneous.cpp:6). A path that hits it is dropped and the render
 * returns DTRT_ERR_STEP_CAP. */
int dtrt_scene_set_tracking_cap(dtrt_scene *scene, int max_steps);

/* How renders run their camera paths: the forward-mode pass 1 (integratorAD.cpp:19-98),
 * the density adjoint's replay and the primal render. MEGAKERNEL: one thread carries its
 * path to the end in one launch; WAVEFRONT: launches per path vertex over the paths still
 * alive, compacted into queues after every vertex (path state in device memory between
 * launches); AUTO picks per render (wavefront from 65,536 paths; for the primal render only
 * in scenes with grid media). Same code and random numbers per path and pixel sums in path
 * order: forward and primal images are identical under both, the density gradient equal up
 * to the order of its FP32 atomic sums. dtrt_render_fwd_noalloc, the vertex adjoint and the
 * batch's persistent schedule always use the megakernel. */
#define DTRT_CAMERA_AUTO 0
#define DTRT_CAMERA_MEGAKERNEL 1
#define DTRT_CAMERA_WAVEFRONT 2
int dtrt_scene_set_camera_schedule(dtrt_scene *scene, int schedule);

/* ---------------------------------------------------------------- reverse mode and density
 * parameters. None of these has a counterpart in the reference: its heterogeneous medium
 * differentiates the lookup position, the density scale and the albedo only
 * (src/medium/heterogeneous.h:46-75, include/gridvolume.h:174-201), and it has no reverse
 * mode; pydtrt re-reads the VOL file to change a grid (pydtrt/scene_manager.py:286-297). */

/* Estimator variants (bit mask, 0 = the reference's estimator).
 * DTRT_EST_SCATTER_SEGMENT_FROM_ORIGIN: at a delta-tracking scatter event the derivative of
 * the free-flight optical depth is integrated over the segment travelled, [ray origin,
 * scatter point]. The reference passes ray.org as the scatter-point output of
 * sampleDistanceAD (volpathAD.cpp:164), so its intSigT(ray, 0, t) runs over
 * [scatter point, scatter point + t*d] (heterogeneous.cpp:65); that is the default here too. */
#define DTRT_EST_SCATTER_SEGMENT_FROM_ORIGIN 1u
int dtrt_scene_set_estimator_flags(dtrt_scene *scene, unsigned flags);

/* Sizes of the adjoint outputs: voxels of all heterogeneous media (concatenated in medium
 * order, each [res_z][res_y][res_x]) and scene vertices (shape order). Either may be NULL. */
int dtrt_scene_gradient_sizes(const dtrt_scene *scene, int64_t *density_voxels, int64_t *vertices);

/* Replace the density grid of heterogeneous medium `medium_id` (same resolution, values
 * clamped at 0 as on load); the majorant is recomputed. */
int dtrt_scene_set_density(dtrt_scene *scene, int medium_id, const float *density);

/* Per-voxel directional derivatives of a heterogeneous medium's density for forward mode:
 * grids is [nder][res_z][res_y][res_x]; derivative slot j of every density lookup in the
 * medium gains the trilinear interpolation of grids[j] (its directional derivative along
 * grid j). NULL removes them. */
int dtrt_scene_set_density_derivatives(dtrt_scene *scene, int medium_id, const float *grids);

/* Reverse-mode adjoint by path replay: the gradient of sum(d_image * I) with respect to
 * every density voxel (d_density) or every vertex position (d_vertices), where I is the
 * expected image of dtrt_render_fwd slot 0 for these options. Camera paths are replayed
 * from their RNG seeds; nothing is stored per path. The estimate is the exact transpose of
 * the forward-mode derivative of the same paths: projecting the gradient on a direction
 * equals sum(d_image * derivative image) of dtrt_render_fwd with that direction set as a
 * derivative slot (dtrt_scene_set_density_derivatives, or shape vertex velocities), for the
 * same seed, up to rounding.
 *   d_image    [H][W][3] dL/dI (crop size when cropped); required with a gradient output
 *   image      NULL or out [H][W][3]: the image of the same paths
 *   d_density  NULL or out [density_voxels] (dtrt_scene_gradient_sizes), overwritten
 *   d_vertices NULL or out [vertices][3] (global vertex order: shapes in order), overwritten.
 *              Covers the interior term (BSDF frames), secondary edges (sppse) and primary
 *              edges (sppe) of scenes without media, vertex normals or AreaLightEx emitters
 *              (else DTRT_ERR_UNSUPPORTED); max_bounces < 32.
 * Pointers are host memory when on_device == 0, else device memory on `stream`. */
int dtrt_render_adjoint(dtrt_scene *scene, const dtrt_render_options *opts, const float *d_image, float *image,
                        float *d_density, float *d_vertices, int on_device, void *stream);

/* ---------------------------------------------------------------- batches of scenes
 * No counterpart in the reference, which renders one scene per blocking call
 * (integratorAD.cpp:19-166). A batch is a fixed list of scenes with their own options and
 * device buffers, rendered together as one persistent launch: the image and, where a
 * scene has density grids and d_image is given, the density adjoint of each item (the
 * work of dtrt_render_adjoint). Paths of all items are cut into chunks that warps take
 * from one counter; the item order and chunk size are autotuned; the launch is captured
 * in a CUDA graph that dtrt_batch_launch replays. The items' buffers are borrowed for the
 * batch's lifetime and are rewritten by every launch. */
typedef struct {
    dtrt_scene *scene;
    dtrt_render_options opts;  /* seed, spp, max_bounces, sppe (< 0: no pixel jitter), mode */
    const float *d_image;      /* NULL or device [H][W][3] dL/dI (needed with d_density / d_vertices) */
    float *image;              /* NULL or device [H][W][3] */
    float *d_density;          /* NULL or device [density_voxels] */
    float *d_vertices;         /* NULL or device [vertices][3]: the vertex-position adjoint of a
                                  surface scene (dtrt_render_adjoint's contract). Such an item
                                  (with its image) is rendered after the batch's captured launch
                                  by the vertex replay, whose chunking waits on the host, and it
                                  takes no other output (d_density must be NULL). */
} dtrt_batch_item;

#define DTRT_BATCH_AUTOTUNE 1u /* measure item costs and pick item order and chunk size */
#define DTRT_BATCH_GRAPH 2u    /* capture the launch in a CUDA graph */
#define DTRT_BATCH_TUNE_FULL 4u /* also time the two best sampled schedules on whole items (every fourth by cost) */
#define DTRT_BATCH_WAVEFRONT 8u /* one replay wavefront over the paths of all items, without tuning */
#define DTRT_BATCH_MAX_ITEMS 256
#define DTRT_BATCH_MAX_TRIALS 16

typedef struct {
    int num_items;
    uint64_t total_paths;
    int grid_blocks, blocks_per_sm; /* persistent grid: resident blocks only */
    int schedule;                   /* 0: persistent launch, 1: one launch per item, 2: one wavefront over all items */
    int streams;                    /* streams of the per-item schedule */
    int chunk_paths;                /* paths a warp takes per counter increment (schedule 0) */
    int order_longest_first;        /* 1: items ordered by measured cost, longest first */
    int graph;                      /* 1: launches replay a CUDA graph */
    int num_trials;
    int trial_chunk[DTRT_BATCH_MAX_TRIALS], trial_order[DTRT_BATCH_MAX_TRIALS];
    float trial_ms[DTRT_BATCH_MAX_TRIALS]; /* tuning launches on a strided path sample;
                                              trial_chunk < 0: per-item schedule on -chunk streams,
                                              trial_chunk == 0: the batch wavefront */
    int64_t tune_sample_stride;
    float full_ms[4];               /* DTRT_BATCH_TUNE_FULL: persistent, per-item on 1, 2, 4 streams, on
                                       every fourth item by cost (-1: not confirmed; the two best on
                                       the strided sample are) */
    double item_ms_estimate[DTRT_BATCH_MAX_ITEMS]; /* measured cost of each item (probe) */
    int order[DTRT_BATCH_MAX_ITEMS];
    float full_ms_wavefront;        /* DTRT_BATCH_TUNE_FULL: the batch wavefront (-1: not confirmed) */
    int64_t wave_capacity;          /* paths per workspace of the batch wavefront (0: not available) */
    int vertex_items;               /* items with d_vertices (rendered after the captured launch) */
} dtrt_batch_stats;

typedef struct dtrt_batch dtrt_batch;

/* Build (and, with the flags, tune and capture) a batch on the current device. Tuning
 * launches run on `stream`, which must not be capturing. */
int dtrt_batch_create(const dtrt_batch_item *items, int n, unsigned flags, void *stream, dtrt_batch **out);
/* Render every item; blocks until done. */
int dtrt_batch_launch(dtrt_batch *batch, void *stream);
int dtrt_batch_stats_get(const dtrt_batch *batch, dtrt_batch_stats *out);
int dtrt_batch_destroy(dtrt_batch *batch);

/* ---------------------------------------------------------------- BVH builder
 * Replaces the Embree scene build of the reference (src/scene.cpp:17-43), which runs on
 * the host for every Scene. DTRT_BVH_HOST: binned-SAH build on the host (leaves of <= 8
 * triangles; updates refit it). DTRT_BVH_DEVICE: linear BVH built on the GPU (Morton
 * codes, radix sort, radix tree, bottom-up boxes; leaves of <= 4 triangles; updates build
 * it again), falling back to the host build when the tree would be deeper than the
 * traversal stack. DTRT_BVH_AUTO (default): the device build from
 * DTRT_BVH_DEVICE_MIN_TRIS triangles, where the host build time outweighs the device
 * tree's slower traversal (its spatial-median splits visit more nodes per ray than the
 * host's SAH splits). The setting is process-wide and applies to scenes
 * created or updated afterwards. Closest hits do not depend on the tree except at exact
 * ties. */
#define DTRT_BVH_AUTO 0
#define DTRT_BVH_HOST 1
#define DTRT_BVH_DEVICE 2
#define DTRT_BVH_DEVICE_MIN_TRIS 65536
int dtrt_set_bvh_builder(int builder);

typedef struct {
    int builder;        /* DTRT_BVH_HOST or DTRT_BVH_DEVICE: the builder that made the tree */
    int refit;          /* 1: the last update refit the host tree instead of building it */
    int num_nodes;
    int max_depth;      /* host: tree depth; device: depth of the binary tree before leaf collapse */
    double ms_build;    /* wall time of the build or refit (device: kernels and copies included) */
} dtrt_bvh_info;
int dtrt_scene_bvh_info(const dtrt_scene *scene, dtrt_bvh_info *out);

/* Closest-hit queries against the scene BVH (device kernel), for tests of the
 * traversal. rays: [n][8] = org.xyz, tmin, dir.xyz, tmax (host arrays).
 * hits: [n][2] int = (global triangle id or -1, shape id); t: [n] float. */
int dtrt_trace_closest(dtrt_scene *scene, const float *rays, int n, int *hits, float *t);

/* Draws of the device PCG32 stream RndSampler(seed, idx) (src/sampler.cpp:3-41), for
 * bit-exact tests of the generator every device kernel uses: u32[n] raw outputs,
 * f32[n] the FP32 uniforms and f64[n] the FP64 uniforms, each from a fresh stream of
 * the same (seed, idx). Any output pointer may be NULL. Host arrays; n <= 1<<20. */
int dtrt_rng_sequence(uint64_t seed, uint64_t idx, int n, uint32_t *u32, float *f32, double *f64);

/* Mitsuba VOL v3 grid reader (gridvolume.h:88-132). Pass data == NULL to query
 * res/channels/bounds; then call again with data of res_x*res_y*res_z*channels floats. */
int dtrt_vol_read(const char *path, int *res, int *channels, float *vmin, float *vmax, float *data);

#ifdef __cplusplus
}
#endif

#endif /* DTRT_GB300_H */
