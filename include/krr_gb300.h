/*
 * krr_gb300.h — C ABI of the GB300 wavefront path tracer.
 *
 * This is the drop-in boundary for KiRaRay's WavefrontPathTracer render pass
 * (src/render/wavefront/integrator.h:24-104).  Every entry point returns an
 * int status (KRR_OK on success); the reference terminates on error instead
 * (src/util/check.h:8-51).  All work is asynchronous on the CUDA stream that
 * is passed in (the reference uses one stream, src/core/device/context.h:45).
 * Pointers named d_* are device pointers, h_* are host pointers.  No torch or
 * other C++ types cross this boundary.
 */
#ifndef KRR_GB300_H
#define KRR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum {
    KRR_OK = 0,
    KRR_ERR_INVALID_ARGUMENT = 1,
    KRR_ERR_CUDA = 2,
    KRR_ERR_OVERFLOW = 3,      /* a device queue or stack ran out of room   */
    KRR_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up         */
    KRR_ERR_NOT_READY = 5,     /* called before set_scene / resize           */
    KRR_ERR_OUT_OF_MEMORY = 6
};

/* Human-readable text of the last error raised on this host thread. */
const char *krr_last_error(void);
const char *krr_status_string(int status);
/* Library version, for the integration check. */
int krr_version(void);

/* ------------------------------------------------------------ ray records */
/* One ray, 32 bytes: origin.xyz + tmin, direction.xyz + tmax.  The
 * direction need not be normalised (the reference's shadow rays are not:
 * src/core/raytracing.h:151-160).  tmin below zero acts as zero (OptiX also
 * requires tmin >= 0). */
typedef struct krr_ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} krr_ray;

/* One closest hit, 16 bytes: t, barycentrics (b1, b2) with the reference's
 * convention b = (1-b1-b2, b1, b2) (src/render/shading.h:78-87) and the
 * global triangle id (instance-major order of the scene's triangles), or
 * KRR_MISS. */
typedef struct krr_hit {
    float t, b1, b2;
    uint32_t prim;
} krr_hit;

#define KRR_MISS 0xFFFFFFFFu

/* ----------------------------------------------------- scene description */
/* Mirrors the reference's material schema (src/scene/krrscene.cpp:195-227)
 * and MaterialType enum order (src/core/raytracing.h:24-31). */
enum {
    KRR_MATERIAL_NULL = 0,
    KRR_MATERIAL_DIFFUSE = 1,
    KRR_MATERIAL_DIELECTRIC = 2,
    KRR_MATERIAL_CONDUCTOR = 3
};

typedef struct krr_material_desc {
    int32_t type;                 /* KRR_MATERIAL_*                          */
    float diffuse[3];             /* "diffuse"                               */
    float specular[3];            /* "specular"                              */
    float roughness;              /* "roughness" (stored as 1-roughness in the
                                     specular alpha, as the reference does)  */
    float specular_transmission;  /* "specular_transmission"                 */
    float eta;                    /* "eta"                                   */
    float anisotropic;            /* "anisotropic"                           */
} krr_material_desc;

/* One triangle mesh (src/core/mesh.h:25-56).  Vertex normals are required:
 * the reference's Triangle::sample reads them unconditionally
 * (src/core/shape.h:61-62). */
typedef struct krr_mesh_desc {
    const float *h_positions;     /* float3 [n_vertices]                     */
    const float *h_normals;       /* float3 [n_vertices]                     */
    const float *h_texcoords;     /* float2 [n_vertices] or NULL             */
    const uint32_t *h_indices;    /* uint3  [n_triangles]                    */
    int64_t n_vertices;
    int64_t n_triangles;
    int32_t material;             /* index into materials, -1 = null material */
    float emission[3];            /* mesh radiance Le; all zero = not a light */
    int32_t medium_inside;        /* index into media or -1                  */
    int32_t medium_outside;       /* index into media or -1                  */
} krr_mesh_desc;

typedef struct krr_instance_desc {
    int32_t mesh;
    float transform[12];          /* row-major 3x4 object-to-world           */
} krr_instance_desc;

/* Infinite (environment) light, src/core/light.h:208-259. */
typedef struct krr_infinite_light_desc {
    float tint[3];
    float scale;
    float rotation[9];            /* row-major 3x3 light-to-world            */
    const float *h_image;         /* float4 [height][width] or NULL          */
    int32_t width, height;
} krr_infinite_light_desc;

/* Heterogeneous medium over a dense FP16 density grid (the reference's
 * NanoVDBMedium<float>, src/render/media.h:144-227). */
typedef struct krr_medium_desc {
    const uint16_t *h_density;    /* IEEE half [nz][ny][nx], or NULL = homogeneous */
    int32_t nx, ny, nz;
    float bounds_min[3], bounds_max[3];
    float sigma_t[3];
    float albedo[3];
    float g;                      /* Henyey-Greenstein asymmetry             */
    float scale;                  /* density scale                           */
    int32_t majorant_res[3];      /* majorant grid resolution                */
} krr_medium_desc;

typedef struct krr_camera_desc {
    float position[3];
    float rotation[9];            /* row-major 3x3 camera-to-world; the camera
                                     looks down its local -Z (src/core/camera.h:45-57) */
    float film_size[2];           /* mm */
    float focal_length;           /* mm */
    float focal_distance;
    float lens_radius;
    float aspect_ratio;
    float shutter_open, shutter_time;
    int32_t medium;               /* medium the camera sits in, or -1        */
} krr_camera_desc;

typedef struct krr_scene_desc {
    const krr_mesh_desc *meshes;        int32_t n_meshes;
    const krr_instance_desc *instances; int32_t n_instances;
    const krr_material_desc *materials; int32_t n_materials;
    const krr_infinite_light_desc *infinite_lights; int32_t n_infinite_lights;
    const krr_medium_desc *media;       int32_t n_media;
} krr_scene_desc;

/* ------------------------------------------------ acceleration structure */
/* Replaces OptixScene::buildTriangleMeshGAS / OptixSceneSingleLevel::
 * buildAccelStructure (src/core/device/optix.cpp:143-250,357-398): builds a
 * Morton-code LBVH on the GPU and collapses it into a compressed 8-wide BVH
 * over the world-space triangles of all instances. */
typedef struct krr_accel krr_accel;

typedef struct krr_accel_stats {
    int64_t n_triangles;
    int64_t n_nodes;          /* 8-wide nodes                               */
    int32_t max_depth;        /* 8-wide levels                              */
    int32_t reserved;
    double build_ms;          /* device time of the last build              */
    double node_bytes;        /* bytes of the node array                    */
    double triangle_bytes;    /* bytes of the leaf-ordered triangle array   */
} krr_accel_stats;

/* Node format of the BVHs built from now on, process-wide: 0 = compressed
 * 8-wide nodes (80 B, 8-bit quantised child boxes; default), 1 = float
 * 8-wide nodes (224 B, fewer instructions per box test).  Hits are the
 * same with either.  krr_accel_stats.reserved reports a build's format. */
int krr_set_bvh_node_format(int32_t format);
/* Largest leaf child of the BVHs built from now on, in triangles (1..3,
 * default 1): smaller leaves test fewer triangles per ray for a few more
 * node visits (a triangle test costs several node-child tests).  Hits are
 * the same with any setting. */
int krr_set_bvh_max_leaf(int32_t triangles);
/* Largest leaf child of a full node (eight children) of the BVHs built from
 * now on, in triangles (max leaf..3, default 1): a child of a full node that
 * covers at most this many triangles becomes a leaf instead of a node of
 * its own with two or three children.  Hits are the same with any setting. */
int krr_set_bvh_full_node_leaf(int32_t triangles);

/* Binary tree behind the BVHs built from now on, process-wide: 0 = Karras
 * radix tree over 63-bit Morton codes of the centroids, each axis scaled to
 * its own extent; 1 = PLOC, parallel locally-ordered clustering (Meister and
 * Bittner 2018) over Morton codes on cubic cells; 2 = the radix tree on
 * cubic cells (default: the fewest node visits on the bench scene).  Either
 * is collapsed into the same 8-wide nodes; hits are the same with any
 * builder. */
int krr_set_bvh_builder(int32_t builder);
/* How the binary tree becomes 8-wide nodes in the BVHs built from now on,
 * process-wide: 0 = greedy (a node opens its largest child until it has
 * eight; default), 1 = cost-optimal (the cut of the binary tree into wide
 * nodes of least surface-area cost, Ylitie, Karras and Laine 2017; with
 * one-triangle leaves every triangle's test costs the same in any cut, so
 * the cut of least total wide-node area; other leaf settings use the
 * greedy collapse).  Replaces nothing in the reference (OptiX builds its
 * own tree); hits are the same with either. */
int krr_set_bvh_collapse(int32_t mode);
/* Treelet restructuring passes (0..3, default 0) over the binary tree of
 * the BVHs built from now on, process-wide, before the collapse: each pass
 * visits the tree bottom-up and rebuilds, at every node over at least eight
 * triangles, the treelet of its seven largest descendants as the binary
 * topology of least total surface area (Karras and Aila, HPG 2013).  A
 * restructured tree deeper than the traversal stack is built again without.
 * Replaces nothing in the reference (OptiX builds its own tree); hits are
 * the same with any setting. */
int krr_set_bvh_treelets(int32_t passes);

/* Build from host arrays of world-space triangles: h_vertices float3[3*n]. */
int krr_accel_create_from_triangles(const float *h_vertices, int64_t n_triangles,
                                    krr_accel **out, void *stream);
int krr_accel_stats_get(const krr_accel *accel, krr_accel_stats *out);
int krr_accel_destroy(krr_accel *accel);
/* New positions for the triangles of a built structure (same count and order,
 * h_vertices float3[3*n]): the boxes are refitted bottom-up over the existing
 * tree (a quarter of a rebuild's time at 10.9M triangles), the device buffers
 * keep their addresses and hits stay exact; the tree's quality follows the
 * motion, so a caller rebuilds after large changes.  The update path of an
 * OptiX AS (used by OptixSceneSingleLevel::updateAccelStructure,
 * optix.cpp:618-642). */
int krr_accel_refit_triangles(krr_accel *accel, const float *h_vertices, int64_t n_triangles,
                              void *stream);

/* Two-level structure, the OptiX GAS-per-mesh + IAS layout of the
 * reference (OptixSceneSingleLevel::buildAccelStructure, src/core/device/
 * optix.cpp:357-398): one BVH per geometry over its object-space triangles
 * (h_geom_vertices float3[3 * total], geometry g holding triangles
 * [h_geom_tri_begin[g], h_geom_tri_begin[g + 1]), n_geoms + 1 entries
 * starting at 0) and one BVH over the instances (instance i draws geometry
 * h_instances[i].mesh with its row-major 3x4 object-to-world transform;
 * h_instance_mask[i] == 0 lets any-hit rays through, NULL = all opaque).
 * Hit ids are global as in the flattened structure: instance-major, the
 * instance's first triangle id plus the triangle's index in its geometry.
 * t is the parameter of the ray carried into the instance's object space
 * (the world ray's t up to rounding); traced with the same entry points as
 * the flattened structure (no counter replay, refit or tuning).  Instances
 * share their geometry's tree, so the structure holds each geometry once. */
int krr_accel_create_instanced(const float *h_geom_vertices, const int64_t *h_geom_tri_begin,
                               int32_t n_geoms, const krr_instance_desc *h_instances,
                               int32_t n_instances, const uint8_t *h_instance_mask,
                               krr_accel **out, void *stream);
/* New object-to-world transforms for every instance (12 floats each): the
 * instance level is rebuilt, the geometry trees are kept (the OptiX IAS
 * update, optix.cpp:618-669). */
int krr_accel_update_instances(krr_accel *accel, const float *h_transforms, void *stream);
/* The world-to-object 3x4 matrices the traversal uses (12 floats per
 * instance), for checking hits against an independent implementation. */
int krr_accel_instance_inverse(const krr_accel *accel, float *h_out, int32_t n_instances);

/* Closest hit for n rays (the reference's __raygen__Closest +
 * __closesthit__Closest, src/render/wavefront/device.cu:43-81, without the
 * shading setup).  Ties in t go to the smaller triangle id. */
int krr_accel_trace_closest(const krr_accel *accel, const krr_ray *d_rays, int64_t n,
                            krr_hit *d_hits, void *stream);
/* Any hit in (tmin, tmax] (the reference's __raygen__Shadow,
 * src/render/wavefront/device.cu:83-100).  d_occluded[i] = 1 if blocked.
 * Triangles whose mask byte is zero are ignored (null-material surfaces). */
int krr_accel_trace_any(const krr_accel *accel, const krr_ray *d_rays, int64_t n,
                        uint8_t *d_occluded, void *stream);
/* Per-triangle any-hit mask (global triangle order); NULL = all opaque. */
int krr_accel_set_mask(krr_accel *accel, const uint8_t *h_mask);

/* Device-side error flags of the traces on this structure since the last
 * call (cleared on read; synchronises the stream): bit 0 = a ray needed more
 * traversal stack than the limit allows and was cut off.  A cut-off
 * closest-hit ray reports t = NaN with prim = KRR_MISS; a cut-off any-hit ray
 * reports occluded = 0xFF (counted as blocked).  The entry points that wait
 * for their results (krr_accel_trace_stats, _noalloc, _closest_host) return
 * KRR_ERR_OVERFLOW instead.  The reference stops on errors
 * (src/util/check.h:8-51). */
int krr_accel_device_errors(const krr_accel *accel, uint32_t *out_flags, void *stream);
/* Traversal stack entries a ray may use, 1..48 (default 48).  The build
 * rejects trees deeper than 48 levels, so with the default no ray is cut off;
 * a smaller limit exercises the overflow path above. */
int krr_accel_set_stack_limit(krr_accel *accel, int32_t entries);

/* Counter-instrumented replay of a trace: h_counts[0] = 8-wide nodes visited,
 * h_counts[1] = triangles tested, summed over the n rays.  Used to compute
 * the algorithmic bytes per ray of the roofline.  Synchronous. */
int krr_accel_trace_stats(const krr_accel *accel, const krr_ray *d_rays, int64_t n,
                          int32_t any_hit, unsigned long long *h_counts, void *stream);

/* No-allocation variant of krr_accel_trace_stats (this entry point has no
 * counterpart in the reference).  For callers that must not allocate device
 * memory during their work, such as render loops with a fixed per-frame
 * memory budget (cudaMalloc/cudaFree can synchronise the device and stall the
 * frame) or hosts whose pool allocator owns all device memory.  Its scratch
 * (per-ray hit records and counters) lives in one static device array of
 * KRR_NOALLOC_MAX_RAYS rays (about 1 MiB), resident on every GPU that loads
 * the library until exit; n must be 1..KRR_NOALLOC_MAX_RAYS or the call
 * returns KRR_ERR_INVALID_ARGUMENT.  The first call on each device looks up
 * the array's device address and keeps it for the life of the process:
 * make that first call before any stream capture begins on the device, and
 * do not reset the device after it.  The call is synchronous (it waits for
 * the stream and writes h_counts).  All calls share the array, so calls that
 * overlap on the GPU race; counters are cleared at the start of each call.
 * Calls no cudaMalloc, cudaFree or other allocating routine.  Returns
 * KRR_ERR_OVERFLOW when the stack limit cut a ray off. */
#define KRR_NOALLOC_MAX_RAYS 65536
int krr_accel_trace_stats_noalloc(const krr_accel *accel, const krr_ray *d_rays, int64_t n,
                                  int32_t any_hit, unsigned long long *h_counts, void *stream);

/* Traversal tuning: refill a warp's idle lanes from the ray counter when
 * fewer than refill_below (1..32) lanes are busy; postpone a node's
 * triangles while fewer than postpone_pct % of the busy lanes have
 * triangles (0 = never).  Defaults 20 and 0.  Results do not depend on it. */
int krr_accel_set_tuning(krr_accel *accel, int32_t refill_below, int32_t postpone_pct);
/* Autotuner: times closest-hit traversal of the given rays for a grid of
 * tuning settings (repeats launches each) and keeps the fastest. */
int krr_accel_autotune(krr_accel *accel, const krr_ray *d_rays, int64_t n, int32_t repeats,
                       int32_t *out_refill, int32_t *out_postpone, float *out_ms, void *stream);

/* Same as krr_accel_trace_closest, with host buffers; returns when the hits
 * are in h_hits.  Page-locked buffers on a coherently linked host (Grace
 * NVLink-C2C) are read and written in place by the traversal kernel;
 * otherwise the rays are copied in and the hits out in chunks over two
 * streams.  Not reentrant per handle (staging and counters are shared). */
int krr_accel_trace_closest_host(const krr_accel *accel, const krr_ray *h_rays, int64_t n,
                                 krr_hit *h_hits, void *stream);

/* -------------------------------------------- wavefront path tracer pass */
typedef struct krr_wf krr_wf;

/* Pass parameters (WavefrontPathTracer::from_json,
 * src/render/wavefront/integrator.h:96-103). */
typedef struct krr_wf_params {
    int32_t nee;              /* "nee", default 1            */
    int32_t enable_medium;    /* "enable_medium", default 1  */
    int32_t max_depth;        /* "max_depth", default 10     */
    float rr;                 /* "rr", default 0.8           */
    int32_t enable_clamp;     /* "enable_clamp", default 0   */
    float clamp_max;          /* "clamp_max", default 1e3    */
    int32_t spp;              /* samples per pixel per frame */
    uint32_t seed;            /* added to the per-pixel sample index */
    /* 0 (default): as the reference, the path radiance L is not cleared
     * between the samples of one frame, so with spp > 1 the pixel sums
     * running totals (integrator.cpp:205-221 clears L once per frame,
     * :255-258 adds L after every sample).  1: L is cleared before every
     * sample, so the frame is the plain mean of spp independent samples. */
    int32_t independent_samples;
} krr_wf_params;

void krr_wf_params_default(krr_wf_params *p);
/* The pass's JSON parameters, as WavefrontPathTracer::from_json reads them
 * (src/render/wavefront/integrator.h:85-103): "nee", "enable_medium",
 * "max_depth", "rr", "enable_clamp", "clamp_max" (plus "spp", "seed",
 * "independent_samples"); absent keys keep the defaults, other keys are
 * ignored; malformed JSON or a key of the wrong type returns
 * KRR_ERR_INVALID_ARGUMENT. */
int krr_wf_params_from_json(const char *params_json, krr_wf_params *out);

int krr_wf_create(const krr_wf_params *params, krr_wf **out);
/* krr_wf_create from the pass's JSON parameters (the `params` object of a
 * passes[] entry, RenderPassFactory::deserizeInstance, src/main/renderer.cpp:
 * 274-286); NULL = all defaults. */
int krr_wf_create_json(const char *params_json, krr_wf **out);
int krr_wf_destroy(krr_wf *wf);
int krr_wf_set_params(krr_wf *wf, const krr_wf_params *params);
int krr_wf_get_params(const krr_wf *wf, krr_wf_params *out);
/* Changes the keys present in params_json, keeping the others. */
int krr_wf_set_params_json(krr_wf *wf, const char *params_json);
/* RenderPass::setScene (integrator.cpp:186-203): uploads the scene and
 * builds the BVH. */
int krr_wf_set_scene(krr_wf *wf, const krr_scene_desc *scene, void *stream);
/* Several scenes (1..255) in one pass, so that views of different scenes
 * share one wavefront: every stage of a bounce is one launch over the items
 * of all views.  Each view names its scene (krr_view.scene); each scene keeps
 * its own lights, environment, media and BVH (one tree per scene in one node
 * array, each ray starting at its scene's root), and a view's frame equals
 * the same view of a pass holding its scene alone, bit for bit.  With a
 * radiance cache attached, each scene's positions are offset so that the
 * scenes occupy disjoint regions of the cache's box (krr_wf_cache_box).
 * Instance updates (krr_wf_update_instances) and the megakernel variant
 * take one scene only; krr_wf_rebuild_bvh rebuilds every scene's tree. */
int krr_wf_set_scenes(krr_wf *wf, const krr_scene_desc *scenes, int32_t n_scenes, void *stream);
/* Path depth of one scene of the pass (max_depth >= 0), or -1 for the
 * pass's max_depth (the default): a view of that scene then equals its
 * scene's pass with that max_depth. */
int krr_wf_set_scene_max_depth(krr_wf *wf, int32_t scene, int32_t max_depth);
/* Acceleration structure of the pass's scene from the next set_scene on (or
 * rebuilt now): 1 = the instances flattened into one world-space BVH
 * (default; the fastest traversal), 2 = the two-level structure of
 * krr_accel_create_instanced (each mesh geometry once, so less memory, and
 * krr_wf_update_instances rebuilds only the instance level).  Two levels
 * take a pass with one scene; the megakernel variant traces one level. */
int krr_wf_set_accel_levels(krr_wf *wf, int32_t levels);
/* Box the radiance cache should cover for this pass (scene_lo/hi of its
 * krr_nrc_config): the union of the scenes' boxes after their offsets. */
int krr_wf_cache_box(krr_wf *wf, float *out_lo3, float *out_hi3);
/* Scene::update for animated instances (src/core/scene.cpp:17-31,
 * src/core/device/optix.cpp:618-642): instance h_indices[k] gets the
 * row-major 3x4 transform h_transforms[12k..12k+11]; the world-space
 * triangles are re-flattened and the BVH's boxes refitted over its tree
 * (krr_accel_refit_triangles).  Device buffers stay in place: a captured
 * frame graph stays valid.  Frames equal those of a fresh scene. */
int krr_wf_update_instances(krr_wf *wf, int32_t n, const int32_t *h_indices,
                            const float *h_transforms, void *stream);
/* Full BVH build over the current instance transforms (restores the tree's
 * quality after large motion; about 13 ms for 10.9M triangles).  Drops a
 * captured frame graph (capture again). */
int krr_wf_rebuild_bvh(krr_wf *wf, void *stream);
/* RenderPass::resize (integrator.cpp:181-184): reallocates queues. */
int krr_wf_resize(krr_wf *wf, int32_t width, int32_t height);
/* RenderPass::beginFrame (integrator.cpp:205-221). frame_index is 1-based. */
int krr_wf_begin_frame(krr_wf *wf, int64_t frame_index, const krr_camera_desc *camera,
                       void *stream);
/* RenderPass::render (integrator.cpp:223-267): writes float4 RGBA per pixel,
 * row-major, row 0 at the top (the reference's y-flipped surface write). */
int krr_wf_render(krr_wf *wf, float *d_out_rgba, void *stream);

/* The same frame as krr_wf_render computed by one persistent kernel, one
 * thread per pixel path (no queues): equal to krr_wf_render bit for bit, for
 * an A/B of queue traffic against register pressure.  Counterpart of the
 * reference's MegakernelPathTracer pass (src/render/megakernel/device.cu:
 * 148-195) in structure, with the wavefront pass's sampling.  Surfaces only:
 * returns KRR_ERR_INVALID_ARGUMENT for scenes with media or with a cache
 * attached. */
int krr_wf_render_megakernel(krr_wf *wf, float *d_out_rgba, void *stream);
/* Coherence step of the megakernel variant (default 1): the 128 paths of a
 * block advance one bounce at a time and, after each closest hit, are
 * regrouped through shared memory by hit class (miss / null, diffuse,
 * dielectric, conductor, finished), as the reference's megakernel calls
 * optixReorder(hit, 1) (src/render/megakernel/device.cu:173-176).  0: one
 * path per thread from start to end.  Frames are the same either way. */
int krr_wf_set_megakernel_reorder(krr_wf *wf, int32_t reorder);
/* Order of the medium tracking launches (default 0, queue order): with 1
 * their items are taken class by class of estimated optical depth (the
 * ray's length inside the media's boxes times the largest sigma_t), so that
 * a warp's rays take similar numbers of null collisions.  The ordering costs
 * more than it saves on the 1024x1024 volume frame (11.1 against 10.1 ms),
 * hence off by default.  Frames are the same either way. */
int krr_wf_set_media_order(krr_wf *wf, int32_t order);
/* Order in which the camera stage queues each view's pixels (default 1):
 * 1 = 8x8 pixel tiles (bands of eight rows, eight columns at a time, the
 * last tile of a band and the last band narrower), 0 = row-major, the order
 * in which the reference's generateCameraRays pushes them
 * (src/render/wavefront/integrator.cpp:166-179).  Frames are the same
 * either way; the tiles keep the rays a warp traces close together. */
int krr_wf_set_camera_order(krr_wf *wf, int32_t order);

/* Stage timers, the counterpart of the reference's PROFILE("...") events
 * (src/util/profiler.h:212-235; stage names from integrator.cpp and
 * medium.cpp): with profiling on (default off), every stage's launches are
 * bracketed by two CUDA events on the stage's stream (not while the stream
 * is being captured into a graph).  krr_wf_profile_read waits for the
 * recorded events, writes up to `cap` stages with their call counts and
 * summed device milliseconds since the last read, sets *n_out to the number
 * of stages that ran, and starts a new interval. */
typedef struct krr_stage_time {
    char name[40];
    int64_t calls;
    double ms;
} krr_stage_time;
int krr_wf_set_profiling(krr_wf *wf, int32_t on);
int krr_wf_profile_read(krr_wf *wf, krr_stage_time *out, int32_t cap, int32_t *n_out);

/* Batched views: many cameras of different sizes in one wavefront (one
 * launch per stage per bounce).  krr_wf_resize_views replaces resize; each
 * frame krr_wf_begin_frame_views gives the cameras (sizes must match) and
 * per-view seeds (sample index = frame_index * spp + seed); render writes
 * the views one after another, each row-major with row 0 at the top. */
typedef struct krr_view {
    krr_camera_desc camera;
    int32_t width, height;
    uint32_t seed;
    int32_t scene;    /* scene of the view (krr_wf_set_scenes), 0 with one scene;
                         camera.medium indexes that scene's media */
} krr_view;
int krr_wf_resize_views(krr_wf *wf, const krr_view *views, int32_t n_views);
int krr_wf_begin_frame_views(krr_wf *wf, int64_t frame_index, const krr_view *views,
                             int32_t n_views, void *stream);
/* Captures one whole frame (constants upload, beginFrame, render into
 * d_out) into a CUDA graph on a non-default stream; krr_wf_launch_frame
 * replays it for a new frame index (views NULL keeps the cameras).  Run one
 * ordinary frame first so that every lazily sized buffer exists. */
int krr_wf_capture_frame(krr_wf *wf, float *d_out, void *stream);
int krr_wf_launch_frame(krr_wf *wf, int64_t frame_index, const krr_view *views, int32_t n_views,
                        void *stream);

/* Launch shapes of the stage kernels and the queue capacity: threads per
 * block (64, 128 or 256; default 256), resident blocks per SM of the
 * grid-stride stage kernels (1..32; default 8), and `wave`, the pixels that
 * go through the bounces together in render() (0 = all of them, the
 * reference's W*H queues, integrator.cpp:25; default).  Queues hold
 * min(wave, pixels) items, so a smaller wave needs less memory; frames are
 * the same with any setting.  The stage entry points need wave 0.
 * Reallocates the queues when the wave changes (drops a captured frame). */
int krr_wf_set_launch(krr_wf *wf, int32_t block, int32_t blocks_per_sm, int64_t wave);
int krr_wf_get_launch(const krr_wf *wf, int32_t *block, int32_t *blocks_per_sm, int64_t *wave,
                      int64_t *queue_capacity);
typedef struct krr_wf_tuning {
    int32_t block, blocks_per_sm;
    int64_t wave, queue_capacity;
    float frame_ms;             /* median frame time with the chosen settings */
    float default_frame_ms;     /* with the defaults (256 threads, 8 per SM, all pixels) */
    int32_t candidates;
    int32_t reserved;
} krr_wf_tuning;
/* Autotuner: renders `frames` frames per candidate setting of
 * krr_wf_set_launch (128/256 threads x 4/8/16 blocks per SM x waves of all,
 * half or a quarter of the pixels) with the current cameras into d_out,
 * keeps the fastest and reports it.  An attached cache does not train
 * during the trials.  Synchronises the stream. */
int krr_wf_autotune(krr_wf *wf, float *d_out_rgba, int32_t frames, krr_wf_tuning *out, void *stream);

/* Frame groups: several passes (for instance two scenes, each with its own
 * batched views) captured as one CUDA graph whose branches run the passes'
 * frames concurrently.  Each pass must have rendered one ordinary frame
 * before krr_wf_group_capture; krr_wf_group_launch renders frame
 * `frame_index` of every pass with its current cameras into its d_outs[i].
 * A pass's results equal the pass rendered alone. */
typedef struct krr_wf_group krr_wf_group;
int krr_wf_group_create(krr_wf *const *passes, float *const *d_outs, int32_t n, krr_wf_group **out);
int krr_wf_group_capture(krr_wf_group *group, void *stream);
int krr_wf_group_launch(krr_wf_group *group, int64_t frame_index, void *stream);
int krr_wf_group_destroy(krr_wf_group *group);

/* Stage entry points, for stage-level tests and for subclasses in the manner
 * of PPGPathTracer (src/misc/render/ppg/integrator.h:13). */
int krr_wf_generate_camera_rays(krr_wf *wf, void *stream);
int krr_wf_trace_closest(krr_wf *wf, int32_t depth, void *stream);
int krr_wf_handle_hit(krr_wf *wf, void *stream);
int krr_wf_handle_miss(krr_wf *wf, void *stream);
int krr_wf_generate_scatter_rays(krr_wf *wf, int32_t depth, void *stream);
int krr_wf_trace_shadow(krr_wf *wf, void *stream);
int krr_wf_sample_medium_interaction(krr_wf *wf, int32_t depth, void *stream);
int krr_wf_sample_medium_scattering(krr_wf *wf, int32_t depth, void *stream);
int krr_wf_reset_queues(krr_wf *wf, int32_t depth, void *stream);

enum {
    KRR_QUEUE_RAY0 = 0, KRR_QUEUE_RAY1 = 1, KRR_QUEUE_MISS = 2, KRR_QUEUE_HIT_LIGHT = 3,
    KRR_QUEUE_SHADOW = 4, KRR_QUEUE_SCATTER = 5, KRR_QUEUE_MEDIUM_SAMPLE = 6,
    KRR_QUEUE_MEDIUM_SCATTER = 7, KRR_QUEUE_COUNT = 8
};
/* Current item count of a queue (synchronises the stream). */
int krr_wf_queue_size(krr_wf *wf, int32_t queue, int32_t *out_size, void *stream);
/* Device pointer to the per-pixel radiance: float4 per pixel (L.xyz,
 * lambda[0]), the reference's PixelState::L (workqueue.h:15-26). */
int krr_wf_pixel_radiance(krr_wf *wf, const float **d_L);
/* Copies the per-pixel radiance (float4 per pixel) into d_dst on the stream. */
int krr_wf_read_radiance(krr_wf *wf, float *d_dst, void *stream);
/* Device pointers to planes of the ray queue used at `depth`: float4 per item
 * (origin.xyz | tmin), (direction.xyz | tmax) and (pu.xyz | pixel id bits);
 * the item count is krr_wf_queue_size(depth & 1). */
int krr_wf_ray_queue(krr_wf *wf, int32_t depth, const float **d_origin_tmin,
                     const float **d_dir_tmax, const float **d_pu_pixel, int32_t *capacity);
/* SoA view of any queue (the reference's queue pointers that stage-level
 * subclasses read, workqueue.h:159-359): `channels` planes of float4, plane
 * c of item i at d_base + 4 * (c * capacity + i) floats; the layouts per
 * queue are those of the pass (Ray/Miss: o|tmin, d|tmax, ctx.p|medium,
 * ctx.n|bsdfType, thp|depth, pu|pixel, pl|time; Shadow: o|tmin, d|tmax,
 * Ld|pixel, pu|medium, pl|time; ...).  Valid until the next resize. */
int krr_wf_queue_view(krr_wf *wf, int32_t queue, const float **d_base, int32_t *channels,
                      int32_t *capacity);
/* Error flags raised by device code since the last call (cleared on read):
 * bit 0 traversal stack limit, bit 1 queue overflow (consumers then read
 * only the queue's capacity), bit 2 loop limit (medium tracking, interface
 * crossings, tensor-core waits). */
int krr_wf_device_errors(krr_wf *wf, uint32_t *out_flags, void *stream);
/* Bounds of the medium tracking loops of the launches after this call:
 * null collisions per majorant walk (default 2^20) and null-interface
 * crossings per shadow ray (default 64).  A walk that runs out ends (the
 * path or shadow ray carries no further radiance) and raises bit 2 of
 * krr_wf_device_errors; the reference loops without bound
 * (src/render/wavefront/wavefront.h:34-139).  A captured frame keeps the
 * limits it was captured with. */
int krr_wf_set_loop_limits(krr_wf *wf, int32_t max_null_collisions,
                           int32_t max_interface_crossings);
/* The BVH of the current scene (owned by the pass). */
int krr_wf_accel(krr_wf *wf, const krr_accel **out);

/* ------------------------------------------------- neural radiance cache */
/* Online-trained radiance cache (no counterpart in the reference; it plugs
 * into the pass the way PPGPathTracer records per-vertex radiance,
 * src/misc/render/ppg/guideditem.h:119-166).  Query/training records are
 * float[13]: position (world), shading normal, roughness, albedo, outgoing
 * direction wo (unit, towards the previous path vertex). */
typedef struct krr_nrc krr_nrc;

typedef struct krr_nrc_config {
    int32_t n_levels;            /* hash-grid levels (16)                    */
    int32_t features_per_level;  /* 2                                        */
    int32_t log2_table_size;     /* entries per hashed level, log2 (19)      */
    int32_t base_resolution;     /* 16                                       */
    int32_t max_resolution;      /* 2048                                     */
    int32_t hidden_layers;       /* width-64 ReLU layers (5)                 */
    float learning_rate;         /* Adam (1e-2)                              */
    float beta1, beta2, epsilon; /* 0.9, 0.99, 1e-15                         */
    float loss_scale;            /* backward-pass loss scale (128)           */
    int32_t batch_size;          /* training records per frame (65536)       */
    int32_t train_pixel_stride;  /* 1 of this many pixels trains (16)        */
    uint32_t seed;
    float scene_lo[3], scene_hi[3];   /* box mapped to the unit cube         */
    int32_t tensor_cores;        /* 1: forward passes on tcgen05 (default);
                                    0: CUDA-core kernels (reference path) */
    float termination_spread;    /* in a pass: a path stops at a vertex
                                    and takes the cache's answer once its
                                    spread a(x1..xn) exceeds this fraction
                                    of a0 (0.01; 0 = at the first bounce) */
    float ema_decay;             /* 0 (default): queries read the trained
                                    parameters; d in (0, 1): queries read an
                                    exponential moving average of them,
                                    e <- d e + (1 - d) w after each Adam
                                    step (not in the reference, which has no
                                    cache)                                  */
} krr_nrc_config;

typedef struct krr_nrc_info_t {
    int64_t n_params_mlp;
    int64_t n_table_entries;
    int32_t n_levels;
    int32_t resolution[16];
    uint32_t level_offset[16];
    uint32_t level_size[16];
    int64_t step;
} krr_nrc_info_t;

void krr_nrc_config_default(krr_nrc_config *config);
int krr_nrc_create(const krr_nrc_config *config, krr_nrc **out);
int krr_nrc_destroy(krr_nrc *nrc);
int krr_nrc_info(const krr_nrc *nrc, krr_nrc_info_t *info);
/* d_out[3*i..] = predicted RGB radiance of record i. */
int krr_nrc_query(krr_nrc *nrc, const float *d_inputs, int64_t count, float *d_out, void *stream);
/* One Adam step on (inputs, RGB targets); h_loss (optional) gets the loss. */
int krr_nrc_train_step(krr_nrc *nrc, const float *d_inputs, const float *d_targets, int64_t count,
                       float *h_loss, void *stream);
/* Gradients of the loss for one batch without updating (host arrays sized
 * as krr_nrc_get_params); synchronises the device. */
int krr_nrc_gradients(krr_nrc *nrc, const float *d_inputs, const float *d_targets, int64_t count,
                      float *h_grad_mlp, float *h_grad_table, float *h_loss);
/* which: 0 = MLP weights [layer][out rows][64], 1 = hash table [entry][2];
 * get_params also 2, 3 = the same arrays of the queries' moving average
 * (ema_decay > 0).  set_params restarts that average from the new values. */
int krr_nrc_get_params(const krr_nrc *nrc, int32_t which, float *h_dst, int64_t count);
int krr_nrc_set_params(krr_nrc *nrc, int32_t which, const float *h_src, int64_t count);
/* Device-side status of the cache (synchronises the stream): out_flags =
 * error flags of its kernels since the last call (bit 2: a bounded
 * tensor-core wait gave up; cleared on read); out_diverged = 1 once a
 * training step's loss was not finite.  A diverged cache takes no more
 * training steps and a pass with it attached renders as the plain tracer
 * (no path stops at the cache) until krr_nrc_set_params or krr_nrc_load
 * gives it new parameters. */
int krr_nrc_status(krr_nrc *nrc, uint32_t *out_flags, int32_t *out_diverged, void *stream);
/* Checkpoint of the cache's training state to a file: FP32 weights and hash
 * table with their Adam moments, the step counter and bias corrections, the
 * configuration (training settings and scene box) and the divergence flag
 * (a flat binary file with a header).  krr_nrc_load restores it into a cache
 * with the same encoding and network shape (else KRR_ERR_INVALID_ARGUMENT);
 * training then continues from the saved step.  Both synchronise the
 * device.  The reference has no checkpoints. */
int krr_nrc_save(const krr_nrc *nrc, const char *path);
int krr_nrc_load(krr_nrc *nrc, const char *path);
/* Attaches a cache to the pass (NULL detaches: the plain tracer).  With a
 * cache, paths of 1 in train_pixel_stride pixels run unbiased and record
 * training targets; the others stop at the vertex after their first
 * non-specular bounce and add throughput x cache(vertex). */
int krr_wf_set_nrc(krr_wf *wf, krr_nrc *nrc, int32_t train);

/* ------------------------------------------------ accumulation and error */
/* d_accum (double RGB per pixel) += d_rgba.rgb (float4 per pixel): the
 * reference's AccumulatePass in "double" precision
 * (src/render/passes/accumulate/accumulate.cu:30-79). */
int krr_accumulate_f64(const float *d_rgba, double *d_accum, int64_t n_pixels, void *stream);
/* Error of the image scale * d_accum against d_ref_rgba (float4 per pixel):
 * metric 0 = relMSE, 1 = MSE, per pixel clamped at 100 and averaged, as the
 * reference's ErrorMeasurePass (src/render/passes/errormeasure/metrics.cu:
 * 64-128), reduced in FP64.  Synchronises the stream. */
int krr_image_error(const double *d_accum, double scale, const float *d_ref_rgba,
                    int64_t n_pixels, int32_t metric, double *h_out, void *stream);
/* ToneMappingPass (src/render/passes/tonemapping/tonemapping.cu:60-88): per
 * pixel color * exposure, then operator op (0 linear, 1 reinhard, 2 aces,
 * 3 uncharted2, 4 hejihable; the pass's JSON "operator"), then pow(1/2.2)
 * when gamma is set; alpha 1.  In place when d_out == d_in. */
int krr_tonemap(const float *d_in_rgba, float *d_out_rgba, int64_t n_pixels, int32_t op,
                float exposure, int32_t gamma, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* KRR_GB300_H */
