/*
 * oracle.h — CPU restatement of the WavefrontPathTracer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * in kiraray_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs may load it.  The product never links or calls it.
 *
 * Parity status: the reference cannot be built here (OptiX, Eigen, NanoVDB
 * and the Vulkan stack are absent and the build is Windows-only), and it has
 * no tests or golden vectors.  Shading, sampling, light and medium code follow
 * the cited reference files line by line; ray/triangle intersection restates
 * the published watertight test of Woop, Benthin and Wald (JCGT 2013) because
 * the reference delegates it to OptiX (closed).  Parity is therefore
 * UNPINNED against reference outputs; it is pinned against known answers
 * (PCG32 published sequence, analytic furnace / Fresnel / transmittance
 * values) in tests/.
 *
 * Built with -ffp-contract=off so that every float operation rounds exactly
 * as written.
 */
#ifndef KRR_ORACLE_H
#define KRR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_bvh oracle_bvh;

/* Binned-SAH binary BVH over world-space triangles (float3 x 3 per triangle). */
int oracle_bvh_build(const float *vertices, int64_t n_tris, int threads, oracle_bvh **out);
void oracle_bvh_free(oracle_bvh *bvh);
/* Triangles whose mask byte is 0 are ignored by any-hit queries. */
void oracle_bvh_set_mask(oracle_bvh *bvh, const uint8_t *mask);

/* rays: 8 floats each (o.xyz, tmin, d.xyz, tmax); hits: (t, b1, b2, prim bits). */
int oracle_trace_closest(const oracle_bvh *bvh, const float *rays, int64_t n, float *hits,
                         int threads);
int oracle_trace_any(const oracle_bvh *bvh, const float *rays, int64_t n, uint8_t *occluded,
                     int threads);
/* Brute force over all triangles (small scenes). */
int oracle_trace_closest_brute(const float *vertices, int64_t n_tris, const float *rays,
                               int64_t n, float *hits);

/* PCG sampler (src/core/sampler.h:13-91): `count` floats drawn after
 * setPixelSample(pixel, sample_index) and advance(advance_by). */
void oracle_pcg_floats(uint32_t px, uint32_t py, uint32_t sample_index, int64_t advance_by,
                       int count, float *out);
/* Raw PCG32 outputs after setSeed(initstate, initseq). */
void oracle_pcg_u32(uint64_t initstate, uint64_t initseq, int count, uint32_t *out);
uint32_t oracle_interleave_32bit(uint32_t x, uint32_t y);

/* Path tracer restatement: scene in the C-ABI description (include/krr_gb300.h). */
struct krr_scene_desc;
struct krr_wf_params;
struct krr_camera_desc;
typedef struct oracle_pt oracle_pt;
int oracle_pt_create(const struct krr_scene_desc *scene, int threads, oracle_pt **out);
void oracle_pt_free(oracle_pt *pt);
/* Renders pixels [px_begin, px_end) of one frame; out_L / out_pixel get 3
 * floats per pixel (L after the frame, and the accumulated pixel). */
int oracle_pt_render(const oracle_pt *pt, const struct krr_wf_params *params,
                     const struct krr_camera_desc *camera, int32_t width, int32_t height,
                     int64_t frame_index, int64_t px_begin, int64_t px_end, float *out_L,
                     float *out_pixel, int threads);

double oracle_medium_transmittance(const oracle_pt *pt, const float *o, const float *d, float tmax,
                                   int n, uint32_t seed);

/* Shading known answers (the material headers of src/render/materials/ and
 * media.cpp:83-111), in the local shading frame.  mat: type (1 diffuse,
 * 2 dielectric, 3 conductor), diffuse rgb, roughness, specular transmission,
 * ior, anisotropic. */
float oracle_fr_dielectric(float cos_i, float eta);
/* f rgb and pdf of n (wo, wi) pairs -> out[4 n] */
void oracle_bsdf_eval(const float *mat, const float *wo, const float *wi, int64_t n, float *out);
/* n samples around one wo from u[n][3] -> out[8 n]: f rgb, wi xyz, pdf, flags */
void oracle_bsdf_sample(const float *mat, const float *wo, const float *u, int64_t n, float *out);
float oracle_hg_p(float g, const float *wo, const float *wi);
/* n samples from u[n][2] -> out[4 n]: wi xyz, pdf */
void oracle_hg_sample(float g, const float *wo, const float *u, int64_t n, float *out);
/* Light sampling (light.h:167-180, shape.h:54-123): n samples of light
 * `light` seen from cp -> out[8 n]: p xyz, L rgb, solid-angle pdf, and the
 * pdf the hit-side MIS weight uses for the same point. */
int oracle_light_sample(const oracle_pt *pt, int32_t light, const float *cp, const float *u, int64_t n,
                        float *out);
int32_t oracle_light_count(const oracle_pt *pt);

#ifdef __cplusplus
}
#endif
#endif
