/*
 * TEST INFRASTRUCTURE — C API of the dtrt_gb300 CPU oracle.
 *
 * The oracle is an FP64 C++17 + OpenMP restatement of the reference's CPU
 * renderer (uci-rendering/dtrt: IntegratorAD::render + VolPathTracerAD and
 * everything beneath it). It consumes the same dtrt_scene_desc as the CUDA
 * library (include/dtrt_gb300.h) so both sides see identical inputs.
 *
 * Parity status: the reference itself cannot be built here (it needs Eigen 3
 * and Embree 3, neither present) and ships no golden vectors or tests, so the
 * oracle is pinned only by its own known-answer tests (PCG32 published
 * outputs, closed-form BSDF/phase/Fresnel identities, furnace and analytic
 * transmittance cases). Parity against the reference's own outputs is
 * therefore unpinned.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library.
 */
#ifndef DTRT_ORACLE_H
#define DTRT_ORACLE_H

#include "../include/dtrt_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Render like IntegratorAD::render (integratorAD.cpp:19-166) into
 * out[(nder+1)][H][W][3] (zero-initialised by the caller). nthreads <= 0: all cores.
 * Returns 0 on success; non-zero with oracle_last_error() otherwise. */
int oracle_render(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads);

/* oracle_render with the extensions of the CUDA library that have no reference
 * counterpart: estimator flags (dtrt_scene_set_estimator_flags) and per-voxel density
 * directions per medium (dtrt_scene_set_density_derivatives; density_dirs[m] NULL or
 * [nder][res_z][res_y][res_x]; density_dirs itself may be NULL). */
int oracle_render_ext(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads,
                      unsigned est_flags, const float *const *density_dirs);

/* oracle_render with another AD integrator behind IntegratorAD::render:
 * ORACLE_VOLPATH_AD (VolPathTracerAD, volpathAD.cpp), ORACLE_PATH_AD (PathTracerAD,
 * pathAD.cpp:10-228) or ORACLE_DIRECT_AD (DirectIntegratorAD, directAD.cpp:1-163).
 * The last two accept surface scenes only (no media, no null BSDFs). */
#define ORACLE_VOLPATH_AD 0
#define ORACLE_PATH_AD 1
#define ORACLE_DIRECT_AD 2
int oracle_render_integrator(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads,
                             int integrator);

/* VolPathTracer::render (src/integrator/volpath.cpp:105-140): the primal image
 * out[H][W][3] (no derivatives), written unconditionally. */
int oracle_render_primal(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out, int nthreads);

/* Render only the primary-edge pass (integratorAD.cpp:100-165) with a caller-chosen
 * sample count, into out[nder][H][W][3] (added to). */
int oracle_render_primary_edges(const dtrt_scene_desc *desc, const dtrt_render_options *opts, float *out,
                                int nthreads);

/* First n raw PCG32 outputs / FP64 uniforms of RndSampler(seed, idx), src/sampler.cpp. */
void oracle_pcg32(uint64_t seed, uint64_t idx, int n, uint32_t *out);
void oracle_next1d(uint64_t seed, uint64_t idx, int n, double *out);

/* Closest hit (shape-global triangle id, shape id, t) against the oracle BVH.
 * rays: [n][8] = org.xyz, tmin, dir.xyz, tmax. */
int oracle_trace_closest(const dtrt_scene_desc *desc, const double *rays, int n, int *hits, double *t);

/* Sum over the scene's secondary edges (length-weighted) and primary-edge PDF sum
 * (projected length in pixels), for edge-table tests. */
int oracle_edge_summary(const dtrt_scene_desc *desc, int *num_edges, double *total_length, int *num_primary,
                        double *primary_pdf_sum);

/* Closed-form pieces for known-answer tests.
 * which: 0 = fresnel(cos_i, eta) ; 1 = HG eval(g, cos) ; 2 = Beckmann D(alpha, cos_theta_m)
 *        3 = smithG1(alpha, cos_theta_v) with m = normal ; 4 = erf(x) ; 5 = erfinv(x) */
double oracle_closed_form(int which, double a, double b);

/* Monte Carlo integral of a BSDF's sampling weight over its sampling density,
 * E[weight] = albedo, for diffuse / phong / roughdielectric at a given incident
 * cosine. desc_bsdf is one dtrt_bsdf_desc (nder ignored). */
int oracle_bsdf_albedo(const dtrt_bsdf_desc *bsdf, double cos_i, int nsamples, uint64_t seed, double *out3);

const char *oracle_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
