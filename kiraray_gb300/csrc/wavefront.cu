// Wavefront path tracer: the WavefrontPathTracer render pass of the reference
// (src/render/wavefront/integrator.{h,cpp}) re-designed for one GB300.
//
// Stages per bounce (integrator.cpp:223-267), each one kernel on the caller's
// stream with queue sizes kept on the device (no host synchronisation inside
// render):
//   reset queues -> trace closest (BVH traversal + hit processing, the
//   reference's __raygen__/__closesthit__/__miss__Closest) -> [medium sample]
//   -> handle hit -> handle miss -> [medium scatter] -> generate scatter rays
//   (RR, NEE, BSDF sampling) -> trace shadow rays (any hit + radiance).
// Queues are SoA planes of float4 (16-byte vector loads and stores); pushes
// use one atomic per warp.  Consumers run persistent grid-stride loops over
// the live queue size read from device memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "accel.h"
#include "internal.h"
#include "nrc.h"
#include "shading.cuh"
#include "wavefront.h"
#include "accel_device.cuh"
#include <cuda_fp16.h>

using namespace krr;

namespace krr {
int accel_set_mask(krr_accel *a, const uint8_t *d_mask, cudaStream_t s);
int launch_medium_sample(krr_wf *wf, int depth, cudaStream_t s);
int launch_medium_scatter(krr_wf *wf, int depth, cudaStream_t s, bool to_tracker = false);
int launch_trace_shadow_tr(krr_wf *wf, cudaStream_t s);
int launch_shadow_tracker(krr_wf *wf, cudaStream_t s);
int launch_shadow_split(krr_wf *wf, cudaStream_t s, bool media_candidates);
bool split_shadows(const krr_wf *wf);
int ensure_split_buffers(krr_wf *wf);
}

struct DevCamera {
    float pos[3];
    float rot[9];
    float tan_fov;         // tan(atan2(filmSize.y / 2, focalLength)), per frame
    float aspect;
    float lens_radius, focal_distance;
    float shutter_open, shutter_time;
    int32_t medium;
};

// One camera view of a batch: its pixels occupy [offset, offset + w*h) of
// the pass's pixel state (row-major per view).
struct DevView {
    DevCamera cam;
    int32_t w, h;
    int64_t offset;
    uint32_t sample_index;   // frame_index * spp + seed of the view
    uint32_t seed;           // seed of the view (kept for replays without new views)
    int32_t part;            // scene of the view (krr_wf_set_scenes)
    int32_t pad;
};

// Per-frame constants read by kernels from device memory (so that a frame
// captured in a CUDA graph can be replayed with new values).
struct FrameConst {
    int32_t n_views;
    int32_t nrc_offset;      // training pixels: (pixel + offset) % stride == 0
    int64_t frame_index;
};

constexpr int kMaxViews = 256;

enum { Q_RAY0 = 0, Q_RAY1 = 1, Q_MISS = 2, Q_HIT_LIGHT = 3, Q_SHADOW = 4, Q_SCATTER = 5,
       Q_MEDIUM_SAMPLE = 6, Q_MEDIUM_SCATTER = 7, Q_COUNT = 8 };
static const int kChannels[Q_COUNT] = {kRayCh, kRayCh, kMissCh, kHitLightCh, kShadowCh,
                                       kScatterCh, kMediumSampleCh, kMediumScatterCh};

struct krr_wf {
    krr_wf_params params{};
    int32_t width = 0, height = 0;
    int64_t n = 0;
    int64_t frame_index = 0;
    DevCamera cam{};
    bool has_scene = false;
    bool medium = false;        // enable_medium && scene has media
    DevScene scene{};
    krr_accel accel{};
    // scenes of the pass (krr_wf_set_scenes): first global triangle id of each
    // (and the total at the end), light ranges, first medium, bounding-sphere
    // radius, the scene of each infinite light, the cache's box
    std::vector<int64_t> part_tri_begin{0, 0};
    std::vector<DevScenePart> parts{DevScenePart{}};
    std::vector<int32_t> part_media_begin{0};
    std::vector<float> part_radius{1.f};
    std::vector<int32_t> inf_part;
    std::vector<int32_t> part_own_depth;   // -1: the pass's max_depth
    int32_t levels = 1;                    // 1: flattened instances, 2: two-level structure
    int32_t mk_reorder = 1;                // megakernel: reorder paths by hit class per bounce
    int32_t media_order = 0;               // 1: tracking kernels take their items by work class
    int32_t camera_order = 1;              // 1: camera rays in 8x8 pixel tiles, 0: row-major
    // stage timers (krr_wf_set_profiling): event pairs recorded since the
    // last krr_wf_profile_read, and a pool of spare events
    int32_t profiling = 0;
    struct ProfRecord { int32_t stage; cudaEvent_t e0, e1; };
    std::vector<ProfRecord> prof;
    std::vector<cudaEvent_t> prof_pool;
    int32_t *work_counts = nullptr;        // [32] work-class counts and cursors
    std::vector<DevMesh> h_mesh;           // host copies of the device meshes
    std::vector<int64_t> h_mesh_tris;      // triangles per mesh
    int32_t n_parts = 1;
    uint8_t *d_pixel_part = nullptr;   // [n] scene of each pixel's view
    // launch shapes and queue capacity (krr_wf_set_launch, krr_wf_autotune):
    // threads per block and resident blocks per SM of the stage kernels, and
    // the pixels traced together in render() (queue capacity; 0 = all)
    int32_t block = 256;
    int32_t blocks_per_sm = 8;
    int64_t wave = 0;
    int64_t qcap = 0;                  // allocated queue capacity
    float cache_lo[3] = {0, 0, 0}, cache_hi[3] = {1, 1, 1};
    std::vector<void *> scene_allocs;
    std::vector<DevInstance> h_instances;     // host copies for instance updates
    float *d_world = nullptr;                 // flattened triangles, kept for refits
    std::vector<DevInfinite> h_infinite;
    int32_t n_instances = 0;
    uint64_t n_tris = 0;
    // queues and pixel state
    float4 *qbuf[Q_COUNT] = {};
    int32_t *d_counts = nullptr;   // [0..7] queue sizes, [8] error flags, [9-10] cache
                                   // batches, [11] ratio-tracked shadow rays, [12-15]
                                   // scatter items per material class, [16] shadow
                                   // rays of scenes with media (split routing)
    float4 *media_shadow = nullptr;   // [kShadowCh][qcap], split routing only
    float4 *hits = nullptr;
    uint8_t *occluded = nullptr;
    int32_t *scatter_lists = nullptr;   // [2][n] scatter items by material class
    PixelState ps{};
    int grid = 0;
    // view table (pinned host copy, device copy) and per-frame constants
    DevView *h_views = nullptr, *d_views = nullptr;
    FrameConst *h_frame = nullptr, *d_frame = nullptr;
    int32_t n_views = 1;
    std::vector<DevView> layout;           // views of the current layout (w, h, offset)
    cudaGraphExec_t graph = nullptr;       // captured frame (krr_wf_capture_frame)
    // neural radiance cache hooks
    krr_nrc *nrc = nullptr;
    bool nrc_train = false;
    float *nrc_q_in = nullptr;       // [n][10] query records
    float4 *nrc_q_meta = nullptr;    // [n] throughput | pixel
    float *nrc_q_out = nullptr;      // [n][3]
    float *nrc_rec = nullptr;        // [slots][max_rec][16] training vertices
    int32_t *nrc_rec_count = nullptr;
    int32_t nrc_rec_max = 0;
    int64_t nrc_slots = 0;
    float *nrc_b_in = nullptr, *nrc_b_t = nullptr;   // training batch
    float2 *nrc_spread = nullptr;    // [n] path spread (a0, sum of sqrt spreads)
    int32_t max_null_collisions = kMaxNullCollisions;       // krr_wf_set_loop_limits
    int32_t max_interface_crossings = kMaxInterfaceCrossings;

    Queue q(int k) const { return Queue{qbuf[k], (int32_t)qcap, d_counts + k}; }
    int32_t *nrc_q_count() const { return d_counts + 9; }
    int32_t *nrc_b_count() const { return d_counts + 10; }
    int32_t *shadow_tracked_count() const { return d_counts + 11; }
    int32_t *scatter_class_counts() const { return d_counts + 12; }
    int32_t *media_shadow_count() const { return d_counts + 16; }
    uint32_t *err() const { return reinterpret_cast<uint32_t *>(d_counts + 8); }
    WfConst consts() const {
        WfConst c;
        c.width = width; c.height = height;
        c.nee = params.nee; c.max_depth = params.max_depth;
        c.enable_medium = medium ? 1 : 0; c.enable_clamp = params.enable_clamp;
        c.spp = params.spp; c.rr = params.rr; c.clamp_max = params.clamp_max;
        return c;
    }
};

static int sync_part_depths(krr_wf *wf);

// Stage timers, the pass's counterpart of the reference's PROFILE("...")
// events (src/util/profiler.h:212-235, names from integrator.cpp and
// medium.cpp): with profiling on, each stage's launches are bracketed by two
// CUDA events on the stage's stream; krr_wf_profile_read waits for them and
// sums the device time per stage.  Off by default; nothing is recorded while
// the stream is being captured into a graph, and at most kProfMaxRecords
// pairs are kept between reads.
enum ProfStage : int {
    PS_BEGIN_FRAME, PS_CAMERA, PS_TRACE_CLOSEST, PS_ROUTE, PS_HIT, PS_MISS, PS_SCATTER, PS_SHADOW,
    PS_SHADOW_NEXT, PS_MEDIUM_SAMPLE, PS_MEDIUM_SCATTER, PS_CACHE_QUERY, PS_CACHE_TRAIN, PS_RESOLVE,
    PS_COUNT
};
static const char *const kProfNames[PS_COUNT] = {
    "Begin frame", "Generate camera rays", "Trace intersect rays", "Route closest hits",
    "Process intersected rays", "Process escaped rays", "Generate scatter rays", "Trace shadow rays",
    "Trace shadow and next rays", "Sample medium interaction", "Sample medium scattering",
    "Cache queries", "Cache training", "Accumulate and resolve"};
constexpr size_t kProfMaxRecords = 1 << 16;

static cudaEvent_t prof_event(krr_wf *wf) {
    if (!wf->prof_pool.empty()) {
        cudaEvent_t e = wf->prof_pool.back();
        wf->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

struct ProfScope {
    krr_wf *wf;
    int stage;
    cudaStream_t st;
    cudaEvent_t e0 = nullptr;
    ProfScope(krr_wf *w, int s, cudaStream_t t) : wf(w), stage(s), st(t) {
        if (!wf->profiling || wf->prof.size() >= kProfMaxRecords) return;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            return;
        }
        e0 = prof_event(wf);
        if (e0 && cudaEventRecord(e0, st) != cudaSuccess) {
            cudaGetLastError();
            wf->prof_pool.push_back(e0);
            e0 = nullptr;
        }
    }
    ~ProfScope() {
        if (!e0) return;
        cudaEvent_t e1 = prof_event(wf);
        if (!e1 || cudaEventRecord(e1, st) != cudaSuccess) {
            cudaGetLastError();
            wf->prof_pool.push_back(e0);
            if (e1) wf->prof_pool.push_back(e1);
            return;
        }
        wf->prof.push_back(krr_wf::ProfRecord{stage, e0, e1});
    }
    ProfScope(const ProfScope &) = delete;
    ProfScope &operator=(const ProfScope &) = delete;
};

// Bounces of the render loop: the largest path depth of the pass's scenes.
static int loop_depth(const krr_wf *wf) {
    int d = wf->params.max_depth;
    for (const DevScenePart &p : wf->parts) d = std::max(d, p.max_depth);
    return d;
}

namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------- pushes
// Warp-aggregated push: every active lane of the warp must push to the same
// queue (one atomic per warp).
__device__ __forceinline__ int push_slot(int32_t *count, int cap, uint32_t *err) {
    unsigned m = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(m, base, leader);
    int slot = base + __popc(m & ((1u << lane) - 1u));
    if (slot >= cap) {
        atomicOr(err, (uint32_t)kErrQueueOverflow);
        return -1;
    }
    return slot;
}

// push_slot for a push whose queue differs between the lanes of a warp: the
// lanes are grouped by counter and each group takes its slots together.
__device__ __forceinline__ int push_slot_grouped(int32_t *count, int cap, uint32_t *err) {
    const unsigned m = __activemask();
    const unsigned peers = __match_any_sync(m, (unsigned long long)(uintptr_t)count);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    const int slot = base + __popc(peers & ((1u << lane) - 1u));
    if (slot >= cap) {
        atomicOr(err, (uint32_t)kErrQueueOverflow);
        return -1;
    }
    return slot;
}

__device__ __forceinline__ float fbits(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ uint32_t ubits(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float ibits(int32_t i) { return __int_as_float(i); }
__device__ __forceinline__ int32_t sbits(float f) { return __float_as_int(f); }

__device__ __forceinline__ Pcg load_rng(const PixelState &ps, uint32_t pixel) {
    ulonglong2 s = ps.rng[pixel];
    return Pcg{s.x, s.y};
}
__device__ __forceinline__ void store_rng(const PixelState &ps, uint32_t pixel, const Pcg &p) {
    ps.rng[pixel] = make_ulonglong2(p.state, p.inc);
}

// PixelStateBuffer::addRadiance, workqueue.h:24-26
__device__ __forceinline__ void add_radiance(const PixelState &ps, uint32_t pixel, V3 v) {
    float4 l = ps.L[pixel];
    ps.L[pixel] = make_float4(v.x + l.x, v.y + l.y, v.z + l.z, l.w);
}

// ----------------------------------------------------------- interaction
struct Surf {
    V3 p, wo, n, t, b;
    float u, v;
    int32_t material;
    int32_t mesh;
    int32_t light;          // light-list index or -1
    int32_t interface_in, interface_out;   // medium interface (-2 = none)
};

// prepareSurfaceInteraction, src/render/shading.h:115-226 (no textures).
__device__ Surf prepare_surface(const DevScene &s, float b1, float b2, uint32_t gid, V3 ray_dir) {
    Surf o;
    uint32_t inst = s.tri_instance[gid];
    const DevInstance &I = s.instances[inst];
    const DevMesh &M = s.meshes[I.mesh];
    uint32_t prim = gid - I.prim_offset;
    float b0 = 1 - b1 - b2;
    uint32_t i0 = M.idx[3 * prim], i1 = M.idx[3 * prim + 1], i2 = M.idx[3 * prim + 2];
    V3 wo = -normalize(ray_dir);
    o.wo = normalize(wo);
    V3 p0{M.pos[3 * i0], M.pos[3 * i0 + 1], M.pos[3 * i0 + 2]};
    V3 p1{M.pos[3 * i1], M.pos[3 * i1 + 1], M.pos[3 * i1 + 2]};
    V3 p2{M.pos[3 * i2], M.pos[3 * i2 + 1], M.pos[3 * i2 + 2]};
    V3 p = p0 * b0 + p1 * b1 + p2 * b2;
    V3 n0{M.nrm[3 * i0], M.nrm[3 * i0 + 1], M.nrm[3 * i0 + 2]};
    V3 n1{M.nrm[3 * i1], M.nrm[3 * i1 + 1], M.nrm[3 * i1 + 2]};
    V3 n2{M.nrm[3 * i2], M.nrm[3 * i2 + 1], M.nrm[3 * i2 + 2]};
    V3 n = normalize(n0 * b0 + n1 * b1 + n2 * b2);
    V3 t = get_perpendicular(n);
    V3 b = normalize(cross(n, t));
    o.u = 0.f;
    o.v = 0.f;
    if (M.uv) {
        o.u = M.uv[2 * i0] * b0 + M.uv[2 * i1] * b1 + M.uv[2 * i2] * b2;
        o.v = M.uv[2 * i0 + 1] * b0 + M.uv[2 * i1 + 1] * b1 + M.uv[2 * i2 + 1] * b2;
    }
    o.light = I.light_offset >= 0 ? I.light_offset + (int32_t)prim : -1;
    o.material = M.material;
    o.mesh = I.mesh;
    bool transition = M.medium_inside != M.medium_outside;
    o.interface_in = transition ? M.medium_inside : -2;
    o.interface_out = transition ? M.medium_outside : -2;
    o.p = xform_point(I.xf, p);
    o.n = normalize(mat3_mul(I.nxf, n));
    o.t = normalize(mat3_mul(I.nxf, t));
    o.b = normalize(mat3_mul(I.nxf, b));
    return o;
}

// offsetRayOrigin, src/core/raytracing.h:106-111
__device__ __forceinline__ V3 offset_ray_origin(V3 p, V3 n, V3 w) {
    V3 off = n * kRayEps;
    if (dot(n, w) < 0.f) off = -off;
    return p + off;
}

// Interaction::getMedium(w), raytracing.h:162-166
__device__ __forceinline__ int32_t medium_towards(int32_t in, int32_t out, int32_t medium, V3 n,
                                                  V3 w) {
    if (in != -2) return dot(w, n) > 0 ? out : in;
    return medium;
}

__device__ __forceinline__ ShadingData shading_data(const DevScene &s, int32_t material) {
    const DevMaterial &m = s.materials[material];
    ShadingData sd;
    sd.type = m.type;
    sd.diffuse = V3{m.diffuse[0], m.diffuse[1], m.diffuse[2]};
    sd.roughness = 1.f - m.spec_alpha;   // SpecularGlossiness, shading.h:215-220
    sd.spec_trans = m.spec_trans;
    sd.ior = m.eta;
    sd.anisotropic = m.anisotropic;
    return sd;
}

// ----------------------------------------------------------------- lights
__device__ __forceinline__ void light_triangle(const DevScene &s, const DevLight &l, V3 &p0, V3 &p1,
                                               V3 &p2, uint32_t &i0, uint32_t &i1, uint32_t &i2,
                                               const DevInstance *&I, const DevMesh *&M) {
    I = &s.instances[l.index];
    M = &s.meshes[I->mesh];
    i0 = M->idx[3 * l.prim];
    i1 = M->idx[3 * l.prim + 1];
    i2 = M->idx[3 * l.prim + 2];
    p0 = V3{M->pos[3 * i0], M->pos[3 * i0 + 1], M->pos[3 * i0 + 2]};
    p1 = V3{M->pos[3 * i1], M->pos[3 * i1 + 1], M->pos[3 * i1 + 2]};
    p2 = V3{M->pos[3 * i2], M->pos[3 * i2 + 1], M->pos[3 * i2 + 2]};
}

// Triangle::area, src/core/shape.h:29-38 (world-space vertices)
__device__ __forceinline__ float tri_area(const DevInstance &I, V3 p0, V3 p1, V3 p2) {
    V3 w0 = xform_point(I.xf, p0), w1 = xform_point(I.xf, p1), w2 = xform_point(I.xf, p2);
    return 0.5f * length(cross(w1 - w0, w2 - w0));
}

// DiffuseAreaLight::L, src/core/light.h:182-188 (one-sided)
__device__ __forceinline__ V3 area_L(const DevInstance &I, V3 n, V3 w) {
    if (dot(n, w) < 0.f) return v3(0.f);
    return I.le_scale * V3{I.le[0], I.le[1], I.le[2]};
}

// Triangle::pdf(sample, ctx), src/core/shape.h:114-123
__device__ __forceinline__ float area_pdf(const DevScene &s, const DevLight &l, V3 sp, V3 sn, V3 cp) {
    V3 p0, p1, p2;
    uint32_t i0, i1, i2;
    const DevInstance *I;
    const DevMesh *M;
    light_triangle(s, l, p0, p1, p2, i0, i1, i2, I, M);
    V3 wi = normalize(sp - cp);
    float pdf = (1 / tri_area(*I, p0, p1, p2)) / (fabsf(dot(sn, -wi)) / length_sq(cp - sp));
    if (length(wi) == 0 || isinf(pdf)) pdf = 0;
    return pdf;
}

// Bilinear lookup with wrap addressing and normalised coordinates (the
// reference samples a cudaFilterModeLinear texture, texture.cpp:237-243).
__device__ __forceinline__ V3 env_lookup(const DevInfinite &e, float u, float v) {
    float x = u * (float)e.w - 0.5f, y = v * (float)e.h - 0.5f;
    float fx0 = floorf(x), fy0 = floorf(y);
    float fx = x - fx0, fy = y - fy0;
    int x0 = (int)fx0, y0 = (int)fy0;
    int xa = ((x0 % e.w) + e.w) % e.w, xb = (((x0 + 1) % e.w) + e.w) % e.w;
    int ya = ((y0 % e.h) + e.h) % e.h, yb = (((y0 + 1) % e.h) + e.h) % e.h;
    float4 c00 = e.image[(size_t)ya * e.w + xa], c10 = e.image[(size_t)ya * e.w + xb];
    float4 c01 = e.image[(size_t)yb * e.w + xa], c11 = e.image[(size_t)yb * e.w + xb];
    V3 top = f3(c00) * (1.f - fx) + f3(c10) * fx;
    V3 bot = f3(c01) * (1.f - fx) + f3(c11) * fx;
    return top * (1.f - fy) + bot * fy;
}

// InfiniteLight::Li, src/core/light.h:242-247
__device__ __forceinline__ V3 env_Li(const DevInfinite &e, V3 wi) {
    float u, v;
    world_to_latlong(mat3_mul_transposed(e.rot, wi), u, v);
    V3 tint{e.tint[0], e.tint[1], e.tint[2]};
    V3 L = e.image ? tint * env_lookup(e, u, v) : tint;
    return e.scale * L;
}

struct LightSample {
    V3 p, n;      // n = 0 for the infinite light
    V3 L;
    float pdf;
};

// Light::sampleLi for triangle area lights (light.h:167-180, shape.h:54-108)
// and the infinite light (light.h:222-231).
__device__ LightSample sample_li(const DevScene &s, const DevLight &l, float u0, float u1, V3 cp) {
    LightSample ls;
    if (l.kind == 1) {
        const DevInfinite &e = s.infinite[l.index];
        V3 wi = uniform_sample_sphere(u0, u1);
        ls.p = cp + wi * 2 * e.scene_radius;
        ls.n = v3(0.f);
        ls.L = env_Li(e, wi);
        ls.pdf = kInv4Pi;
        return ls;
    }
    V3 p0, p1, p2;
    uint32_t i0, i1, i2;
    const DevInstance *I;
    const DevMesh *M;
    light_triangle(s, l, p0, p1, p2, i0, i1, i2, I, M);
    V3 n0{M->nrm[3 * i0], M->nrm[3 * i0 + 1], M->nrm[3 * i0 + 2]};
    V3 n1{M->nrm[3 * i1], M->nrm[3 * i1 + 1], M->nrm[3 * i1 + 2]};
    V3 n2{M->nrm[3 * i2], M->nrm[3 * i2 + 1], M->nrm[3 * i2 + 2]};
    V3 b = uniform_sample_triangle(u0, u1);
    V3 p = p0 * b.x + p1 * b.y + p2 * b.z;
    V3 n = normalize(cross(p1 - p0, p2 - p0));
    V3 ns = normalize(n0 * b.x + n1 * b.y + n2 * b.z);
    if (dot(n, ns) < 0) n = n * -1.f;
    p = xform_point(I->xf, p);
    n = normalize(mat3_mul(I->nxf, n));
    float pdf = 1 / tri_area(*I, p0, p1, p2);
    V3 wi = normalize(p - cp);
    pdf = pdf / (fabsf(dot(n, wi)) / length_sq(cp - p));
    if (length(wi) == 0 || isinf(pdf)) pdf = 0;
    ls.p = p;
    ls.n = n;
    V3 wo = normalize(cp - p);
    ls.L = area_L(*I, n, wo);
    ls.pdf = pdf;
    return ls;
}

}  // namespace
#include "media.cuh"
namespace {

// ---------------------------------------------------------------- kernels
// View owning global pixel g (binary search over view offsets).
__device__ __forceinline__ int view_of(const DevView *__restrict__ v, int n_views, int64_t g) {
    int lo = 0, hi = n_views - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (v[mid].offset <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// beginFrame, integrator.cpp:205-221 (per view: pixel coordinates and the
// advance(256 * pixelId) are view-local)
__global__ void k_begin_frame(PixelState ps, const DevView *__restrict__ views,
                              const FrameConst *__restrict__ fc, int64_t n) {
    const int nv = fc->n_views;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
         g += (int64_t)gridDim.x * blockDim.x) {
        const DevView &v = views[view_of(views, nv, g)];
        int64_t i = g - v.offset;
        uint32_t x = (uint32_t)(i % v.w), y = (uint32_t)(i / v.w);
        Pcg p;
        p.set_seed(interleave_32bit(x, y), v.sample_index);
        p.advance(256 * i);
        float u = p.get1d();
        float lambda0 = (1.f - u) * 360.f + u * 830.f;   // sampleUniform, spectrum.h:47-58
        ps.L[g] = make_float4(0.f, 0.f, 0.f, lambda0);
        ps.pixel[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        store_rng(ps, (uint32_t)g, p);
    }
}

// generateCameraRays + CameraData::getRay, integrator.cpp:166-179, camera.h:32-58
// Camera order: a view's pixels in bands of kCamTile rows, each band in
// chunks of kCamTile columns (8x8 tiles, row-major inside a tile; the last
// chunk of a band and the last band may be narrower).  Position i of the
// order -> row-major pixel index; a bijection on the view's w x h pixels.
constexpr int kCamTile = 8;
__device__ __forceinline__ int64_t tile_pixel(int64_t i, int w, int h) {
    const int64_t band_px = (int64_t)w * kCamTile;
    const int64_t band = i / band_px;
    const int bh = min(kCamTile, h - (int)band * kCamTile);
    const int64_t r = i - band * band_px;
    const int c = (int)(r / (kCamTile * bh));
    const int o = (int)(r - (int64_t)c * kCamTile * bh);
    const int cw = min(kCamTile, w - c * kCamTile);
    return (int64_t)((int)band * kCamTile + o / cw) * w + c * kCamTile + o % cw;
}

// Positions [p0, p0 + n) of the frame's camera order into ray queue items
// 0..n-1.  tiled = 0: position = pixel (row-major); tiled = 1: each view's
// pixels in 8x8 tiles (tile_pixel), so that the rays a warp takes up
// together cover a compact patch of the image (a few per cent fewer node
// visits' worth of time in the traversal on the 1920x1080 camera rays).
// Each view's positions map onto its own pixels, so waves (ranges of
// positions) still cover every pixel once; a path depends only on its
// pixel, so frames are the same in either order.
__global__ void k_camera_rays(PixelState ps, Queue rq, const DevView *__restrict__ views,
                              const FrameConst *__restrict__ fc, int64_t p0, int64_t n, int tiled) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *rq.count = (int32_t)n;
    const int nv = fc->n_views;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = p0 + q;
        const DevView &v = views[view_of(views, nv, pos)];
        const DevCamera &cam = v.cam;
        const int64_t i = tiled ? tile_pixel(pos - v.offset, v.w, v.h) : pos - v.offset;
        const int64_t g = v.offset + i;
        Pcg p = load_rng(ps, (uint32_t)g);
        float fx = p.get1d(), fy = p.get1d();
        float lx = p.get1d(), ly = p.get1d();
        float tm = p.get1d();
        store_rng(ps, (uint32_t)g, p);
        (void)lx; (void)ly;
        float px = (float)(i % v.w) + 0.5f + fx;
        float py = (float)(i / v.w) + 0.5f + fy;
        float ndcx = (2 * px) / (float)v.w + (-1.f);
        float ndcy = (2 * py) / (float)v.h + (-1.f);
        V3 fd = normalize(V3{cam.tan_fov * cam.aspect * ndcx, cam.tan_fov * ndcy, -1.f});
        V3 o = V3{cam.pos[0], cam.pos[1], cam.pos[2]};
        V3 d = mat3_mul(cam.rot, fd);
        float time = cam.shutter_open + cam.shutter_time * tm;
        rq.at(0, q) = f4(o, 0.f);
        rq.at(1, q) = f4(d, INFINITY);
        rq.at(2, q) = make_float4(0.f, 0.f, 0.f, ibits(cam.medium));
        rq.at(3, q) = make_float4(0.f, 0.f, 0.f, fbits(0u));
        rq.at(4, q) = make_float4(1.f, 1.f, 1.f, fbits(0u));
        rq.at(5, q) = make_float4(1.f, 1.f, 1.f, fbits((uint32_t)g));
        rq.at(6, q) = make_float4(1.f, 1.f, 1.f, time);
    }
}

__global__ void k_reset_queues(int32_t *counts, int cur, int all) {
    if (threadIdx.x == 0) {
        for (int k = 0; k < Q_COUNT; ++k)
            if (all || k != cur) counts[k] = 0;
    }
}

__device__ __forceinline__ void copy_ray_item(const Queue &src, int i, const Queue &dst, int j) {
    for (int c = 0; c < kRayCh; ++c) dst.at(c, j) = src.at(c, i);
}


// Cache hooks of the closest-hit stage.  mode 0: off; 1: on.  A pixel is a
// training pixel when (pixel + offset) % stride == 0; its slot is
// pixel / stride.
struct NrcHook {
    int32_t mode;
    const uint32_t *diverged;  // non-zero: the cache diverged, trace as without it
    int32_t stride;
    const FrameConst *frame;   // offset = frame->nrc_offset
    float *q_in;
    float4 *q_meta;
    int32_t *q_count;
    int32_t q_cap;
    float *rec;
    int32_t *rec_count;
    int32_t rec_max;
    float2 *spread;            // per pixel: a0, running sum of sqrt spreads
    float spread_c;            // termination threshold c of a(x1..xn) > c a0
};

// Cache record of a surface vertex; in a pass of several scenes the position
// is offset so that each scene has its own region of the cache's box.
__device__ __forceinline__ void nrc_features(const DevScene &s, const Surf &sf, uint32_t pixel,
                                             float *dst) {
    const DevMaterial &m = s.materials[sf.material];
    dst[0] = sf.p.x; dst[1] = sf.p.y; dst[2] = sf.p.z;
    if (s.pixel_part) {
        const DevScenePart &P = part_of(s, pixel);
        dst[0] += P.cache_offset[0]; dst[1] += P.cache_offset[1]; dst[2] += P.cache_offset[2];
    }
    dst[3] = sf.n.x; dst[4] = sf.n.y; dst[5] = sf.n.z;
    dst[6] = 1.f - m.spec_alpha;
    dst[7] = m.diffuse[0]; dst[8] = m.diffuse[1]; dst[9] = m.diffuse[2];
    dst[10] = sf.wo.x; dst[11] = sf.wo.y; dst[12] = sf.wo.z;
}

// Returns true when the path stops here and the cache answers for it.
// Termination follows the path-spread rule of neural radiance caching
// (Mueller et al. 2021): with a0 = t0^2 / (4 pi |cos theta1|) at the primary
// vertex and a(x1..xn) = (sum_i sqrt(t_{i-1}^2 / (p_i |cos theta_i|)))^2,
// the path stops at the first non-delta vertex where a > c a0.  Specular
// samples add no spread.  Training pixels record instead of stopping.
__device__ __forceinline__ bool nrc_vertex(const NrcHook &h, const DevScene &s, const Surf &sf,
                                           const PixelState &ps, uint32_t pixel, uint32_t depth,
                                           uint32_t prev_flags, V3 thp, float t, V3 dir, V3 pu,
                                           V3 pl, uint32_t *err) {
    if (!h.mode || *h.diverged) return false;
    const float cosv = fmaxf(fabsf(dot(sf.n, dir)), 1e-4f);
    if (depth == 0) {
        h.spread[pixel] = make_float2(t * t / (4.f * kPi * cosv), 0.f);
        return false;
    }
    float2 sp = h.spread[pixel];
    if (!(prev_flags & BSDF_SPECULAR) && pl.x > 0.f) {
        const float pdf = pu.x / pl.x;   // pl = pu / pdf (generateScatterRays)
        if (pdf > 0.f) sp.y += sqrtf(t * t / (pdf * cosv));
    }
    h.spread[pixel] = sp;
    const DevMaterial &m = s.materials[sf.material];
    if (m.type != MAT_DIFFUSE && 1.f - m.spec_alpha <= 1e-3f) return false;   // delta BSDF
    if (sp.y * sp.y <= h.spread_c * sp.x) return false;
    if ((pixel + (uint32_t)h.frame->nrc_offset) % (uint32_t)h.stride == 0u) {
        if (!h.rec) return false;
        uint32_t slot = pixel / (uint32_t)h.stride;
        int k = h.rec_count[slot];
        if (k < h.rec_max) {
            float *r = h.rec + ((size_t)slot * h.rec_max + k) * kNrcRecFloats;
            nrc_features(s, sf, pixel, r);
            float4 l = ps.L[pixel];
            r[kNrcInputs + 0] = thp.x; r[kNrcInputs + 1] = thp.y; r[kNrcInputs + 2] = thp.z;
            r[kNrcInputs + 3] = l.x; r[kNrcInputs + 4] = l.y; r[kNrcInputs + 5] = l.z;
            h.rec_count[slot] = k + 1;
        }
        return false;
    }
    int j = push_slot(h.q_count, h.q_cap, err);
    if (j >= 0) {
        nrc_features(s, sf, pixel, h.q_in + (size_t)kNrcInputs * j);
        h.q_meta[j] = make_float4(thp.x, thp.y, thp.z, __uint_as_float(pixel));
    }
    return true;
}

// L[pixel] += throughput x max(cache, 0)
__global__ void k_nrc_apply(const float *__restrict__ out, const float4 *__restrict__ meta,
                            const int32_t *count, int cap, PixelState ps) {
    int n = min(*count, cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 m = meta[i];
        V3 c{fmaxf(out[3 * i], 0.f), fmaxf(out[3 * i + 1], 0.f), fmaxf(out[3 * i + 2], 0.f)};
        add_radiance(ps, __float_as_uint(m.w), V3{m.x, m.y, m.z} * c);
    }
}

// Training targets (L_final - L_at_vertex) / throughput of every recorded
// vertex, appended to the batch up to its capacity.
__global__ void k_nrc_targets(const float *__restrict__ rec, const int32_t *__restrict__ rec_count,
                              int64_t slots, int rec_max, int stride, const FrameConst *fc,
                              int64_t n_pixels, PixelState ps, float *b_in, float *b_t,
                              int32_t *b_count, int b_cap) {
    const int offset = fc->nrc_offset;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < slots;
         s += (int64_t)gridDim.x * blockDim.x) {
        int k_n = rec_count[s];
        if (k_n == 0) continue;
        int64_t pixel = s * stride + ((stride - offset % stride) % stride);
        if (pixel >= n_pixels) continue;
        float4 lf = ps.L[pixel];
        for (int k = 0; k < k_n; ++k) {
            const float *r = rec + ((size_t)s * rec_max + k) * kNrcRecFloats;
            float t[3];
            float lfin[3] = {lf.x, lf.y, lf.z};
            bool ok = true;
            for (int c = 0; c < 3; ++c) {
                float thp = r[kNrcInputs + c];
                t[c] = thp > 0.f ? (lfin[c] - r[kNrcInputs + 3 + c]) / thp : 0.f;
                ok = ok && isfinite(t[c]);
            }
            if (!ok) continue;
            int j = atomicAdd(b_count, 1);
            if (j >= b_cap) return;
            for (int q = 0; q < kNrcInputs; ++q) b_in[(size_t)kNrcInputs * j + q] = r[q];
            for (int c = 0; c < 3; ++c) b_t[3 * (size_t)j + c] = fmaxf(t[c], 0.f);
        }
    }
}

__global__ void k_clamp_count(int32_t *count, int cap) {
    if (threadIdx.x == 0 && *count > cap) *count = cap;
}

// Radiance of an emissive hit (handleHit, integrator.cpp:78-90): emitted
// radiance times throughput, MIS-weighted against light sampling.
__device__ __forceinline__ V3 hit_light_radiance(const DevScene &s, const DevScenePart &P,
                                                  int32_t light, V3 p, V3 nrm, V3 wo, V3 ctx_p,
                                                  uint32_t bsdf_type, uint32_t depth, V3 thp, V3 pu,
                                                  V3 pl, int nee) {
    const float lsel_pdf = 1.f / (float)P.n_lights;
    const DevLight &l = s.lights[light];
    const DevInstance &I = s.instances[l.index];
    V3 Le = area_L(I, nrm, wo) * thp;
    if (nee && depth && !(bsdf_type & BSDF_DELTA)) {
        float light_pdf = area_pdf(s, l, p, nrm, ctx_p) * lsel_pdf;
        Le = Le / mean(pl * light_pdf + pu);
    } else {
        Le = Le / mean(pu);
    }
    return Le;
}

// Radiance of a miss (handleMiss, integrator.cpp:92-108): every infinite
// light, MIS-weighted against light sampling, times throughput.
__device__ __forceinline__ V3 miss_radiance(const DevScene &s, const DevScenePart &P, V3 dir,
                                             uint32_t bsdf_type, uint32_t depth, V3 thp, V3 pu, V3 pl,
                                             int nee) {
    const float lsel_pdf = 1.f / (float)P.n_lights;
    V3 L = v3(0.f);
    for (int k = 0; k < P.n_infinite; ++k) {
        const DevInfinite &e = s.infinite[P.inf_begin + k];
        if (nee && depth && !(bsdf_type & BSDF_DELTA)) {
            float light_pdf = kInv4Pi * lsel_pdf;
            L += env_Li(e, dir) / mean(pu + pl * light_pdf);
        } else {
            L += env_Li(e, dir) / mean(pu);
        }
    }
    return thp * L;
}

// Routing of a closest hit (__closesthit__/__miss__Closest, device.cu:43-74).
// Four blocks per SM (64 registers): the mesh gathers are latency-bound.
// With `inline_lights` (render()) the radiance of a miss and of an emissive
// hit of a ray outside every medium is added here instead of through the
// miss and hit-light queues: a path has one item per bounce, so each pixel's
// sum gets the same terms in the same order as handleHit/handleMiss after
// this stage.
__global__ void __launch_bounds__(kThreads, 4)
k_hit_process(DevScene s, Queue rq, const float4 *__restrict__ hits, Queue next, Queue miss,
              Queue hitl, Queue scat, Queue msq, int enable_medium, uint32_t *err, NrcHook hook,
              PixelState ps, int inline_lights, int nee) {
    int n = min(*rq.count, rq.cap);   // an overflowed queue holds cap items
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 h = hits[i];
        uint32_t gid = ubits(h.w);
        float4 c2 = rq.at(2, i);
        int32_t ray_medium = sbits(c2.w);
        bool in_medium = enable_medium && ray_medium >= 0;
        if (gid == KRR_MISS) {
            if (in_medium) {
                int j = push_slot(msq.count, msq.cap, err);
                if (j >= 0) {
                    copy_ray_item(rq, i, msq, j);
                    msq.at(7, j) = make_float4(INFINITY, 0.f, 0.f, fbits(KRR_MISS));
                }
            } else if (inline_lights) {
                if (s.n_infinite > 0) {
                    float4 c1 = rq.at(1, i), c3 = rq.at(3, i), c4 = rq.at(4, i), c5 = rq.at(5, i),
                           c6 = rq.at(6, i);
                    const DevScenePart &P = part_of(s, ubits(c5.w));
                    if (P.n_infinite > 0)
                        add_radiance(ps, ubits(c5.w),
                                     miss_radiance(s, P, f3(c1), ubits(c3.w), ubits(c4.w), f3(c4),
                                                   f3(c5), f3(c6), nee));
                }
            } else {
                int j = push_slot(miss.count, miss.cap, err);
                if (j >= 0) copy_ray_item(rq, i, miss, j);
            }
            continue;
        }
        if (in_medium) {
            int j = push_slot(msq.count, msq.cap, err);
            if (j >= 0) {
                copy_ray_item(rq, i, msq, j);
                msq.at(7, j) = h;
            }
            continue;
        }
        float4 c0 = rq.at(0, i), c1 = rq.at(1, i);
        V3 dir = f3(c1);
        Surf sf = prepare_surface(s, h.y, h.z, gid, dir);
        float4 c3 = rq.at(3, i), c4 = rq.at(4, i), c5 = rq.at(5, i), c6 = rq.at(6, i);
        if (sf.material < 0) {
            // null material: continue through the interface (device.cu:54-58)
            int j = push_slot(next.count, next.cap, err);
            if (j >= 0) {
                V3 o = offset_ray_origin(sf.p, sf.n, dir);
                int32_t med = medium_towards(sf.interface_in, sf.interface_out, ray_medium, sf.n, dir);
                next.at(0, j) = f4(o, 0.f);
                next.at(1, j) = f4(dir, INFINITY);
                next.at(2, j) = make_float4(c2.x, c2.y, c2.z, ibits(med));
                next.at(3, j) = c3;
                next.at(4, j) = c4;
                next.at(5, j) = c5;
                next.at(6, j) = c6;
            }
            continue;
        }
        (void)c0;
        V3 thp = f3(c4);
        if (hook.mode && nrc_vertex(hook, s, sf, ps, ubits(c5.w), ubits(c4.w), ubits(c3.w), thp, h.x,
                                    dir, f3(c5), f3(c6), err))
            continue;
        if (sf.light >= 0 && inline_lights) {
            add_radiance(ps, ubits(c5.w),
                         hit_light_radiance(s, part_of(s, ubits(c5.w)), sf.light, sf.p, sf.n, sf.wo,
                                            f3(c2), ubits(c3.w), ubits(c4.w), thp, f3(c5), f3(c6), nee));
        } else if (sf.light >= 0) {
            int j = push_slot(hitl.count, hitl.cap, err);
            if (j >= 0) {
                hitl.at(0, j) = f4(sf.p, ibits(sf.light));
                hitl.at(1, j) = f4(sf.n, sf.u);
                hitl.at(2, j) = f4(sf.wo, sf.v);
                hitl.at(3, j) = make_float4(c2.x, c2.y, c2.z, c3.w);
                hitl.at(4, j) = make_float4(c3.x, c3.y, c3.z, c4.w);
                hitl.at(5, j) = make_float4(c4.x, c4.y, c4.z, c5.w);
                hitl.at(6, j) = c5;
                hitl.at(7, j) = c6;
            }
        }
        if (any(thp)) {
            int j = push_slot(scat.count, scat.cap, err);
            if (j >= 0) {
                scat.at(0, j) = f4(sf.p, ibits(sf.material));
                scat.at(1, j) = f4(sf.wo, c4.w);
                scat.at(2, j) = f4(sf.n, c5.w);
                scat.at(3, j) = f4(sf.t, ibits(sf.mesh));
                scat.at(4, j) = f4(sf.b, sf.u);
                scat.at(5, j) = f4(thp, sf.v);
                scat.at(6, j) = make_float4(c5.x, c5.y, c5.z, c6.w);
                scat.at(7, j) = make_float4(ibits(ray_medium), 0.f, 0.f, 0.f);
            }
        }
    }
}

// handleHit, integrator.cpp:78-90
__global__ void k_handle_hit(DevScene s, Queue hitl, PixelState ps, int nee) {
    int n = min(*hitl.count, hitl.cap);   // an overflowed queue holds cap items
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 c0 = hitl.at(0, i), c1 = hitl.at(1, i), c2 = hitl.at(2, i), c3 = hitl.at(3, i);
        float4 c4 = hitl.at(4, i), c5 = hitl.at(5, i), c6 = hitl.at(6, i), c7 = hitl.at(7, i);
        add_radiance(ps, ubits(c5.w),
                     hit_light_radiance(s, part_of(s, ubits(c5.w)), sbits(c0.w), f3(c0), f3(c1), f3(c2),
                                        f3(c3), ubits(c3.w), ubits(c4.w), f3(c5), f3(c6), f3(c7), nee));
    }
}

// handleMiss, integrator.cpp:92-108
__global__ void k_handle_miss(DevScene s, Queue miss, PixelState ps, int nee) {
    int n = min(*miss.count, miss.cap);   // an overflowed queue holds cap items
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 c1 = miss.at(1, i), c3 = miss.at(3, i), c4 = miss.at(4, i), c5 = miss.at(5, i),
               c6 = miss.at(6, i);
        add_radiance(ps, ubits(c5.w),
                     miss_radiance(s, part_of(s, ubits(c5.w)), f3(c1), ubits(c3.w), ubits(c4.w), f3(c4),
                                   f3(c5), f3(c6), nee));
    }
}

// generateScatterRays (integrator.cpp:110-164) for one item whose Russian
// roulette draw has survived; `rng` is the pixel's sampler after that draw.
// When `tracked` has a counter (a pass of several scenes, some with media),
// the shadow ray of a scene with media goes straight to the transmittance
// tracker's queue and `shadow` keeps only the rays that an any-hit test
// decides.
__device__ __forceinline__ void scatter_item(const DevScene &s, const Queue &scat, int i, Pcg rng,
                                             const Queue &next, const Queue &shadow_q,
                                             const Queue &tracked, const PixelState &ps, int nee,
                                             float rr, uint32_t *err) {
    float4 c0 = scat.at(0, i), c1 = scat.at(1, i), c2 = scat.at(2, i), c3 = scat.at(3, i);
    float4 c4 = scat.at(4, i), c5 = scat.at(5, i), c6 = scat.at(6, i), c7 = scat.at(7, i);
    uint32_t pixel = ubits(c2.w), depth = ubits(c1.w);
    V3 thp = f3(c5) / rr;
    V3 p = f3(c0), wo = f3(c1), nrm = f3(c2), tg = f3(c3), bt = f3(c4), pu = f3(c6);
    float time = c6.w;
    int32_t material = sbits(c0.w), mesh = sbits(c3.w), ray_medium = sbits(c7.x);
    const DevMesh &M = s.meshes[mesh];
    bool transition = M.medium_inside != M.medium_outside;
    int32_t mi = transition ? M.medium_inside : -2, mo = transition ? M.medium_outside : -2;
    auto to_local = [&](V3 v) { return V3{dot(tg, v), dot(bt, v), dot(nrm, v)}; };
    V3 wo_local = to_local(wo);
    ShadingData sd = shading_data(s, material);
    uint32_t bsdf_type = bsdf_type_of(sd);
    Bsdf bsdf = Bsdf::setup(sd);
    // a scene without emitters has nothing to sample (the reference indexes an
    // empty light list there); NEE and its draws are skipped
    const DevScenePart &P = part_of(s, pixel);
    const Queue &shadow = (tracked.count && P.has_media) ? tracked : shadow_q;
    if (nee && (bsdf_type & BSDF_SMOOTH) && P.n_lights > 0) {
        float ul = rng.get1d();
        uint32_t lid = (uint32_t)(ul * (float)P.n_lights);
        float sel_pdf = 1.f / (float)P.n_lights;
        float u0 = rng.get1d(), u1 = rng.get1d();
        LightSample ls = sample_li(s, s.lights[P.light_begin + lid], u0, u1, p);
        // spawnRayTo(Interaction), raytracing.h:151-160
        V3 to = offset_ray_origin(ls.p, ls.n, p - ls.p);
        V3 po = offset_ray_origin(p, nrm, to - p);
        V3 d = to - po;
        V3 wi_world = normalize(d);
        V3 wi_local = to_local(wi_world);
        float light_pdf = sel_pdf * ls.pdf;
        V3 fv = bsdf.f(wo_local, wi_local);
        float bsdf_pdf = bsdf.pdf(wo_local, wi_local);
        if (light_pdf > 0 && any(fv)) {
            V3 Ld = ls.L * thp * fv * fabsf(wi_local.z);
            if (any(Ld)) {
                // with a tracker queue the lanes of a warp may push to two queues
                int j = tracked.count ? push_slot_grouped(shadow.count, shadow.cap, err)
                                      : push_slot(shadow.count, shadow.cap, err);
                if (j >= 0) {
                    int32_t med = medium_towards(mi, mo, ray_medium, nrm, d);
                    shadow.at(0, j) = f4(po, 0.f);
                    shadow.at(1, j) = f4(d, 1.f);
                    shadow.at(2, j) = f4(Ld, fbits(pixel));
                    shadow.at(3, j) = f4(pu * bsdf_pdf, ibits(med));
                    shadow.at(4, j) = f4(pu * light_pdf, time);
                }
            }
        }
    }
    BsdfSample bs = bsdf.sample(wo_local, [&]() { return rng.get1d(); });
    store_rng(ps, pixel, rng);
    if (bs.pdf != 0 && any(bs.f)) {
        V3 wi_world = tg * bs.wi.x + bt * bs.wi.y + nrm * bs.wi.z;
        V3 nthp = thp * bs.f * fabsf(bs.wi.z) / bs.pdf;
        if (any(nthp)) {
            int j = push_slot(next.count, next.cap, err);
            if (j >= 0) {
                V3 o = offset_ray_origin(p, nrm, wi_world);
                int32_t med = medium_towards(mi, mo, ray_medium, nrm, wi_world);
                next.at(0, j) = f4(o, 0.f);
                next.at(1, j) = f4(wi_world, INFINITY);
                next.at(2, j) = f4(p, ibits(med));
                next.at(3, j) = f4(nrm, fbits(bs.flags));
                next.at(4, j) = f4(nthp, fbits(depth + 1));
                next.at(5, j) = f4(pu, fbits(pixel));
                next.at(6, j) = f4(pu / bs.pdf, time);
            }
        }
    }
}

// generateScatterRays (integrator.cpp:110-164) as two launches over the whole
// queue.  The first draws every item's Russian roulette (integrator.cpp:
// 116-118; an ended path stores its sampler and stops) and appends each
// survivor to the index list of its material class, warp-aggregated: classes
// 0 and 1 fill `lists[0..n)` from the front and from the back, classes 2 and
// 3 fill `lists[n..2n)` likewise.  The second walks the four lists in class
// order with no block barrier, so that a warp runs one BSDF except at the
// three class boundaries.  Every item is computed exactly as alone (its
// sampler stream is its pixel's); only the order of the queue pushes changes.
__global__ void k_scatter_classify(DevScene s, Queue scat, PixelState ps, float rr,
                                   int32_t *__restrict__ lists, int32_t *__restrict__ counts) {
    const int cap = scat.cap, n = min(*scat.count, cap);
    const int lane = threadIdx.x & 31;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t pixel = ubits(scat.at(2, i).w);
        // a path of a scene with a smaller depth than the pass's ends here,
        // as its scene's pass ends the bounce loop (no draws)
        if (s.pixel_part && (int)ubits(scat.at(1, i).w) >= part_of(s, pixel).max_depth) continue;
        Pcg rng = load_rng(ps, pixel);
        if (rng.get1d() >= rr) {
            store_rng(ps, pixel, rng);   // the path ends here
            continue;
        }
        const int cls = min(max(s.materials[sbits(scat.at(0, i).w)].type, 0), 3);
        const unsigned peers = __match_any_sync(__activemask(), cls);
        const int leader = __ffs(peers) - 1;
        int slot = 0;
        if (lane == leader) slot = atomicAdd(&counts[cls], __popc(peers));
        slot = __shfl_sync(peers, slot, leader) + __popc(peers & ((1u << lane) - 1u));
        int32_t *list = lists + (cls >> 1) * (size_t)cap;
        list[(cls & 1) ? cap - 1 - slot : slot] = i;
    }
}

// Three blocks per SM (80 registers, 104 bytes spilled): 0.8 % faster per
// 1080p frame than four blocks at 64 registers (236 bytes spilled).
__global__ void __launch_bounds__(kThreads, 3)
k_scatter_process(DevScene s, Queue scat, const int32_t *__restrict__ lists,
                  const int32_t *__restrict__ counts, Queue next, Queue shadow, Queue tracked,
                  PixelState ps, int nee, float rr, uint32_t *err) {
    const int cap = scat.cap;
    const int c0 = counts[0], c01 = c0 + counts[1], c012 = c01 + counts[2], total = c012 + counts[3];
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = g < c0 ? lists[g]
                    : g < c01 ? lists[cap - 1 - (g - c0)]
                    : g < c012 ? lists[cap + (g - c01)]
                    : lists[2 * (size_t)cap - 1 - (g - c012)];
        Pcg rng = load_rng(ps, ubits(scat.at(2, i).w));
        rng.get1d();   // the roulette draw taken by k_scatter_classify
        scatter_item(s, scat, i, rng, next, shadow, tracked, ps, nee, rr, err);
    }
}

// Radiance of unoccluded shadow rays (__raygen__Shadow, device.cu:92-100).
__global__ void k_shadow_resolve(Queue shadow, const uint8_t *__restrict__ occluded, PixelState ps) {
    int n = min(*shadow.count, shadow.cap);   // an overflowed queue holds cap items
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (occluded[i]) continue;
        float4 c2 = shadow.at(2, i), c3 = shadow.at(3, i), c4 = shadow.at(4, i);
        add_radiance(ps, ubits(c2.w), f3(c2) / mean(f3(c4) + f3(c3)));
    }
}

// ------------------------------------------------------ media work order
// The tracking kernels loop over null collisions, whose number grows with
// the optical depth a ray crosses; in queue order the lanes of a warp hold
// rays of very different depths and wait for the longest.  Before each
// tracking launch the items are counted into kWorkClasses classes of
// estimated optical depth (log2 of 1 + the length of the ray inside the
// media's boxes times the largest density-scaled sigma_t) and an index
// permutation lists them class by class, so that warps hold rays of similar
// work.  Each item is computed as before; only the order changes.
constexpr int kWorkClasses = 16;

__device__ __forceinline__ float box_overlap(const DevMedium &m, V3 o, V3 d, float tmax) {
    float t0 = 0.f, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        const float oa = get(o, a), da = get(d, a);
        if (fabsf(da) < 1e-20f) {
            if (oa < m.lo[a] || oa > m.hi[a]) return 0.f;
            continue;
        }
        float ta = (m.lo[a] - oa) / da, tb = (m.hi[a] - oa) / da;
        if (ta > tb) { float q = ta; ta = tb; tb = q; }
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
    }
    return t1 > t0 ? (t1 - t0) * length(d) : 0.f;
}

__device__ __forceinline__ int work_class(const DevScene &s, V3 o, V3 d, float tmax) {
    float tau = 0.f;
    for (int k = 0; k < s.n_media; ++k) {
        const DevMedium &m = s.media[k];
        const float sig = fmaxf(m.sigma_t[0], fmaxf(m.sigma_t[1], m.sigma_t[2])) * (m.density ? m.scale : 1.f);
        tau += box_overlap(m, o, d, isinf(tmax) ? 3.402823466e38f : tmax) * sig;
    }
    return min(kWorkClasses - 1, (int)log2f(1.f + fminf(tau, 1e30f)));
}

// counts[0..16): items per class; classes[i]: item i's class.  ITEMS 0: a
// medium-sample queue (plane 0 origin, 1 direction, 7 hit with t), 1: a
// tracked shadow queue (plane 0 origin, 1 direction | tmax).
template <int ITEMS>
__global__ void k_work_classes(DevScene s, Queue q, uint8_t *__restrict__ classes, int32_t *counts) {
    const int n = min(*q.count, q.cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 c0 = q.at(0, i), c1 = q.at(1, i);
        const float tmax = ITEMS == 0 ? q.at(7, i).x : c1.w;
        const int k = work_class(s, f3(c0), f3(c1), tmax);
        classes[i] = (uint8_t)k;
        const unsigned peers = __match_any_sync(__activemask(), k);
        if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(counts + k, __popc(peers));
    }
}

// order: the item indices class by class (counts[16..32) are the cursors).
__global__ void k_work_order(Queue q, const uint8_t *__restrict__ classes, int32_t *counts,
                             int32_t *__restrict__ order) {
    __shared__ int32_t start[kWorkClasses];
    if (threadIdx.x == 0) {
        int32_t acc = 0;
        for (int k = 0; k < kWorkClasses; ++k) { start[k] = acc; acc += counts[k]; }
    }
    __syncthreads();
    const int n = min(*q.count, q.cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = classes[i];
        const unsigned peers = __match_any_sync(__activemask(), k);
        const int leader = __ffs(peers) - 1;
        int base = 0;
        if ((threadIdx.x & 31) == leader) base = atomicAdd(counts + kWorkClasses + k, __popc(peers));
        base = __shfl_sync(peers, base, leader);
        order[start[k] + base + __popc(peers & ((1u << (threadIdx.x & 31)) - 1u))] = i;
    }
}

// sampleMediumInteraction, medium.cpp:13-103 (the medium has no emission).
// Three blocks of 256 per SM (at most 80 registers): the tracking loops are
// latency-bound, and the extra warps outweigh a few spilled registers.
__global__ void __launch_bounds__(kThreads, 3)
k_medium_sample(DevScene s, Queue msq, Queue next, Queue miss, Queue hitl, Queue scat,
                Queue mscat, PixelState ps, const int32_t *__restrict__ order, uint32_t *err) {
    int n = min(*msq.count, msq.cap);   // an overflowed queue holds cap items
    for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < n; ii += gridDim.x * blockDim.x) {
        const int i = order ? order[ii] : ii;
        float4 c0 = msq.at(0, i), c1 = msq.at(1, i), c2 = msq.at(2, i), c3 = msq.at(3, i);
        float4 c4 = msq.at(4, i), c5 = msq.at(5, i), c6 = msq.at(6, i), h = msq.at(7, i);
        V3 o = f3(c0), dir = f3(c1);
        V3 thp = f3(c4), pu = f3(c5), pl = f3(c6);
        uint32_t depth = ubits(c4.w), pixel = ubits(c5.w);
        int32_t medium = sbits(c2.w);
        float time = c6.w;
        float tmax_hit = h.x;
        Pcg rng = load_rng(ps, pixel);
        int ch = main_index(ps.L[pixel].w);
        const DevMedium &m = s.media[medium];
        bool scattered = false;
        bool aborted;
        V3 T_maj = sample_t_maj(m, o, dir, tmax_hit, rng, ch, s.max_null_collisions, err, aborted,
            [&](V3 p, const MediumProps &mp, V3 sigma_maj, V3 Tm) -> bool {
                float p_absorb = get(mp.sigma_a, ch) / get(sigma_maj, ch);
                float p_scatter = get(mp.sigma_s, ch) / get(sigma_maj, ch);
                float p_null = fmaxf(0.f, 1.f - p_absorb - p_scatter);
                int mode = sample_discrete3(p_absorb, p_scatter, p_null, rng.get1d());
                if (mode == 0) {
                    thp = v3(0.f);
                    return false;
                }
                if (mode == 1) {
                    float pr = get(Tm, ch) * get(mp.sigma_s, ch);
                    V3 q = div_g(Tm * mp.sigma_s, pr);
                    thp *= q;
                    pu *= q;
                    if (any(thp) && any(pu)) {
                        int j = push_slot(mscat.count, mscat.cap, err);
                        if (j >= 0) {
                            mscat.at(0, j) = f4(p, ibits(medium));
                            mscat.at(1, j) = f4(-dir, fbits(depth));
                            mscat.at(2, j) = f4(thp, fbits(pixel));
                            mscat.at(3, j) = f4(pu, time);
                        }
                    }
                    scattered = true;
                    return false;
                }
                V3 sigma_n = vmax(sigma_maj - mp.sigma_a - mp.sigma_s, v3(0.f));
                float pr = get(Tm, ch) * get(sigma_n, ch);
                V3 qn = div_g(Tm * sigma_n, pr);
                thp *= qn;
                if (pr == 0) thp = v3(0.f);
                pu *= qn;
                pl *= div_g(Tm * sigma_maj, pr);
                return any(thp) && any(pu);
            });
        if (aborted) thp = v3(0.f);
        store_rng(ps, pixel, rng);
        if (!scattered && any(thp)) {
            V3 r = div_g(T_maj, get(T_maj, ch));
            thp *= r;
            pu *= r;
            pl *= r;
        }
        if (scattered || !any(thp) || !any(pu) || (int)depth == part_of(s, pixel).max_depth) continue;
        if (isinf(tmax_hit)) {
            int j = push_slot(miss.count, miss.cap, err);
            if (j >= 0) {
                miss.at(0, j) = c0; miss.at(1, j) = c1; miss.at(2, j) = c2; miss.at(3, j) = c3;
                miss.at(4, j) = f4(thp, c4.w); miss.at(5, j) = f4(pu, c5.w); miss.at(6, j) = f4(pl, c6.w);
            }
            continue;
        }
        uint32_t gid = ubits(h.w);
        Surf sf = prepare_surface(s, h.y, h.z, gid, dir);
        if (sf.material < 0) {
            int j = push_slot(next.count, next.cap, err);
            if (j >= 0) {
                V3 no = offset_ray_origin(sf.p, sf.n, dir);
                int32_t med = medium_towards(sf.interface_in, sf.interface_out, medium, sf.n, dir);
                next.at(0, j) = f4(no, 0.f);
                next.at(1, j) = f4(dir, INFINITY);
                next.at(2, j) = make_float4(c2.x, c2.y, c2.z, ibits(med));
                next.at(3, j) = c3;
                next.at(4, j) = f4(thp, c4.w);
                next.at(5, j) = f4(pu, c5.w);
                next.at(6, j) = f4(pl, c6.w);
            }
            continue;
        }
        if (sf.light >= 0) {
            int j = push_slot(hitl.count, hitl.cap, err);
            if (j >= 0) {
                hitl.at(0, j) = f4(sf.p, ibits(sf.light));
                hitl.at(1, j) = f4(sf.n, sf.u);
                hitl.at(2, j) = f4(sf.wo, sf.v);
                hitl.at(3, j) = make_float4(c2.x, c2.y, c2.z, c3.w);
                hitl.at(4, j) = make_float4(c3.x, c3.y, c3.z, c4.w);
                hitl.at(5, j) = f4(thp, c5.w);
                hitl.at(6, j) = f4(pu, c5.w);
                hitl.at(7, j) = f4(pl, c6.w);
            }
        }
        int j = push_slot(scat.count, scat.cap, err);
        if (j >= 0) {
            scat.at(0, j) = f4(sf.p, ibits(sf.material));
            scat.at(1, j) = f4(sf.wo, c4.w);
            scat.at(2, j) = f4(sf.n, c5.w);
            scat.at(3, j) = f4(sf.t, ibits(sf.mesh));
            scat.at(4, j) = f4(sf.b, sf.u);
            scat.at(5, j) = f4(thp, sf.v);
            scat.at(6, j) = f4(pu, time);
            scat.at(7, j) = make_float4(ibits(medium), 0.f, 0.f, 0.f);
        }
    }
}

// sampleMediumScattering, medium.cpp:105-153.  Every item is in a scene
// with media: with `tracked` given (a counter set), its shadow ray goes
// straight to the transmittance tracker's queue, as in scatter_item.
__global__ void k_medium_scatter(DevScene s, Queue mscat, Queue next, Queue shadow_q, Queue tracked,
                                 PixelState ps, int nee, uint32_t *err) {
    const Queue &shadow = tracked.count ? tracked : shadow_q;
    int n = min(*mscat.count, mscat.cap);   // an overflowed queue holds cap items
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 c0 = mscat.at(0, i), c1 = mscat.at(1, i), c2 = mscat.at(2, i), c3 = mscat.at(3, i);
        V3 p = f3(c0), wo = f3(c1), wthp = f3(c2), wpu = f3(c3);
        int32_t medium = sbits(c0.w);
        uint32_t depth = ubits(c1.w), pixel = ubits(c2.w);
        if (s.pixel_part && (int)depth >= part_of(s, pixel).max_depth) continue;   // as k_scatter_classify
        float time = c3.w;
        float g = s.media[medium].g;
        Pcg rng = load_rng(ps, pixel);
        const DevScenePart &P = part_of(s, pixel);
        const float sel_pdf = 1.f / (float)P.n_lights;
        if (nee && P.n_lights > 0) {
            float ul = rng.get1d();
            uint32_t lid = (uint32_t)(ul * (float)P.n_lights);
            float u0 = rng.get1d(), u1 = rng.get1d();
            LightSample ls = sample_li(s, s.lights[P.light_begin + lid], u0, u1, p);
            V3 to = offset_ray_origin(ls.p, ls.n, p - ls.p);
            V3 d = to - p;
            V3 wi = normalize(d);
            V3 thp = wthp * hg_p(g, wo, wi);
            float light_pdf = sel_pdf * ls.pdf;
            float phase_pdf = hg_p(g, wo, wi);
            V3 Ld = thp * ls.L;
            if (any(Ld) && light_pdf > 0) {
                int j = push_slot(shadow.count, shadow.cap, err);
                if (j >= 0) {
                    shadow.at(0, j) = f4(p, 0.f);
                    shadow.at(1, j) = f4(d, 1.f);
                    shadow.at(2, j) = f4(Ld, fbits(pixel));
                    shadow.at(3, j) = f4(wpu * phase_pdf, ibits(medium));
                    shadow.at(4, j) = f4(wpu * light_pdf, time);
                }
            }
        }
        float u0 = rng.get1d(), u1 = rng.get1d();
        float pdf;
        V3 wi = hg_sample(g, wo, u0, u1, pdf);
        float pp = pdf;   // PhaseFunctionSample{wi, p, pdf} with p == pdf
        V3 thp = wthp * pp / pdf;
        float rr = max_coeff(thp / mean(wpu));
        bool killed = false;
        if (depth >= 1 && rr < 1) {
            if (rng.get1d() >= rr) killed = true;
            else thp /= rr;
        }
        store_rng(ps, pixel, rng);
        if (killed) continue;
        bool has_nan = isnan(thp.x) || isnan(thp.y) || isnan(thp.z);
        if (!is_zero(thp) && !has_nan) {
            int j = push_slot(next.count, next.cap, err);
            if (j >= 0) {
                next.at(0, j) = f4(p, 0.f);
                next.at(1, j) = f4(wi, INFINITY);
                next.at(2, j) = f4(p, ibits(medium));
                next.at(3, j) = make_float4(0.f, 0.f, 0.f, fbits(BSDF_SMOOTH));
                next.at(4, j) = f4(thp, fbits(depth + 1));
                next.at(5, j) = f4(wpu, fbits(pixel));
                next.at(6, j) = f4(wpu / pdf, time);
            }
        }
    }
}

// traceTransmittance (wavefront.h:80-139) for every shadow ray when media
// are enabled: closest hits through null-material interfaces with ratio
// tracking inside media.
// Three blocks per SM, as k_medium_sample.
// With a two-level structure (iv.inst != nullptr) every traversal goes
// through the instance level.
// LEVELS 2: the two-level structure (a compile-time choice, so that a
// kernel holds one traversal stack, not one per structure).
template <bool ANY, int FMT, bool MASKED, int LEVELS>
__device__ __forceinline__ float4 shadow_trace(const InstancedView &iv, const float4 *__restrict__ nodes,
                                               const float4 *__restrict__ tris, V3 o, V3 d, float tmax,
                                               int *trace_err, uint32_t root) {
    if constexpr (LEVELS == 2) return trace_two_level<ANY, FMT, MASKED>(iv, o, d, 0.f, tmax, trace_err);
    else return traverse_ray<ANY, FMT, MASKED>(nodes, tris, o, d, 0.f, tmax, trace_err, root);
}

template <int FMT, int LEVELS>
__global__ void __launch_bounds__(kThreads, 3)
k_shadow_tr(DevScene s, const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
            InstancedView iv, Queue shadow, PixelState ps, const int32_t *__restrict__ order,
            uint32_t *err, int *trace_err) {
    int n = min(*shadow.count, shadow.cap);   // an overflowed queue holds cap items
    for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < n; ii += gridDim.x * blockDim.x) {
        const int i = order ? order[ii] : ii;
        float4 c0 = shadow.at(0, i), c1 = shadow.at(1, i), c2 = shadow.at(2, i), c3 = shadow.at(3, i),
               c4 = shadow.at(4, i);
        V3 o = f3(c0), d = f3(c1);
        float tmax = c1.w;
        uint32_t pixel = ubits(c2.w);
        int32_t medium = sbits(c3.w);
        V3 p_light = o + d * tmax;
        Pcg rng = load_rng(ps, pixel);
        int ch = main_index(ps.L[pixel].w);
        V3 T_ray = v3(1.f), pu = v3(1.f), pl = v3(1.f);
        int crossings = 0;
        const uint32_t root = root_of(s, pixel);
        while (fabsf(d.x) > kRayEps * 2 || fabsf(d.y) > kRayEps * 2 || fabsf(d.z) > kRayEps * 2) {
            float4 h = shadow_trace<false, FMT, true, LEVELS>(iv, nodes, tris, o, d, tmax, trace_err, root);
            bool visible = ubits(h.w) == KRR_MISS;
            Surf sf;
            if (!visible) {
                sf = prepare_surface(s, h.y, h.z, ubits(h.w), d);
                if (sf.material >= 0) {
                    T_ray = v3(0.f);
                    break;
                }
            }
            if (medium >= 0) {
                float t_end = visible ? tmax : length(sf.p - o) / length(d);
                bool aborted;
                V3 T_maj = sample_t_maj(s.media[medium], o, d, t_end, rng, ch, s.max_null_collisions,
                                        err, aborted,
                    [&](V3, const MediumProps &mp, V3 sigma_maj, V3 Tm) -> bool {
                        V3 sigma_n = vmax(sigma_maj - mp.sigma_a - mp.sigma_s, v3(0.f));
                        float pr = get(Tm, ch) * get(sigma_maj, ch);
                        V3 qn = div_g(Tm * sigma_n, pr);
                        T_ray *= qn;
                        pl *= div_g(Tm * sigma_maj, pr);
                        pu *= qn;
                        V3 Tr = div_g(T_ray, mean(pu + pl));
                        if (max_coeff(Tr) < 0.05f) {
                            if (rng.get1d() < 0.75f) T_ray = v3(0.f);
                            else T_ray /= 0.25f;
                        }
                        return any(T_ray);
                    });
                if (aborted) T_ray = v3(0.f);
                V3 r = div_g(T_maj, get(T_maj, ch));
                T_ray *= r;
                pu *= r;
                pl *= r;
            }
            if (visible || is_zero(T_ray)) break;
            // Interaction::spawnRayTo(pLight) from the null surface
            V3 po = offset_ray_origin(sf.p, sf.n, p_light - sf.p);
            V3 nd = p_light - po;
            medium = medium_towards(sf.interface_in, sf.interface_out, medium, sf.n, nd);
            o = po;
            d = nd;
            if (++crossings > s.max_interface_crossings) {
                atomicOr(err, (uint32_t)kErrLoopLimit);
                T_ray = v3(0.f);
                break;
            }
        }
        store_rng(ps, pixel, rng);
        if (any(T_ray))
            add_radiance(ps, pixel, f3(c2) * T_ray / mean(f3(c3) * pu + f3(c4) * pl));
    }
}

// First pass of the transmittance shadow stage.  A shadow ray that starts
// outside every medium and crosses no triangle at all (null-material
// interfaces included) is the reference loop's first iteration ending with
// `visible` and T_ray = pu = pl = 1, no sampler draw: its radiance is added
// here with the same expression.  Every other ray (one that starts in a
// medium, meets a surface or has a zero-length direction) is copied to
// `tracked` for k_shadow_tr, so that the tracker's warps hold only the long
// ratio-tracking loops.  In a pass of several scenes, the shadow rays of a
// scene without media need no tracking at all: the transmittance loop there
// draws no samples and ends at the first opaque surface, so an any-hit test
// that ignores null-material surfaces decides them, as traceShadow does
// without media.
template <int FMT, int LEVELS>
__global__ void k_shadow_split(DevScene s, const float4 *__restrict__ nodes,
                               const float4 *__restrict__ tris, InstancedView iv, Queue shadow,
                               Queue tracked, PixelState ps, uint32_t *err, int *trace_err) {
    int n = min(*shadow.count, shadow.cap);   // an overflowed queue holds cap items
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 c0 = shadow.at(0, i), c1 = shadow.at(1, i), c2 = shadow.at(2, i), c3 = shadow.at(3, i);
        V3 d = f3(c1);
        const uint32_t pixel = ubits(c2.w);
        const uint32_t root = root_of(s, pixel);
        bool moving = fabsf(d.x) > kRayEps * 2 || fabsf(d.y) > kRayEps * 2 || fabsf(d.z) > kRayEps * 2;
        if (s.pixel_part && !part_of(s, pixel).has_media) {
            float4 h = shadow_trace<true, FMT, true, LEVELS>(iv, nodes, tris, f3(c0), d, c1.w, trace_err, root);
            if (ubits(h.w) == KRR_MISS) {
                float4 c4 = shadow.at(4, i);
                add_radiance(ps, pixel, f3(c2) * v3(1.f) / mean(f3(c3) * v3(1.f) + f3(c4) * v3(1.f)));
            }
            continue;
        }
        if (sbits(c3.w) < 0 && moving) {
            float4 h = shadow_trace<true, FMT, false, LEVELS>(iv, nodes, tris, f3(c0), d, c1.w, trace_err, root);
            if (ubits(h.w) == KRR_MISS) {
                float4 c4 = shadow.at(4, i);
                add_radiance(ps, pixel, f3(c2) * v3(1.f) / mean(f3(c3) * v3(1.f) + f3(c4) * v3(1.f)));
                continue;
            }
        }
        int j = push_slot(tracked.count, tracked.cap, err);
        if (j < 0) continue;
        for (int c = 0; c < kShadowCh; ++c) tracked.at(c, j) = shadow.at(c, i);
    }
}

// pixel += L after each sample (integrator.cpp:255-258); with `clear` the
// next sample starts from L = 0 (the reference keeps L for the whole frame).
__global__ void k_accumulate(PixelState ps, int64_t n, int clear) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 l = ps.L[i], p = ps.pixel[i];
        ps.pixel[i] = make_float4(p.x + l.x, p.y + l.y, p.z + l.z, 0.f);
        if (clear) ps.L[i] = make_float4(0.f, 0.f, 0.f, l.w);
    }
}

// Final write (integrator.cpp:262-266); rows flipped as the reference's
// surface write does (src/core/device/cuda.h:33-37), per view.
__global__ void k_resolve(PixelState ps, float4 *out, const DevView *__restrict__ views,
                          const FrameConst *__restrict__ fc, int64_t n, float spp, int clamp,
                          float clamp_max) {
    const int nv = fc->n_views;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
         g += (int64_t)gridDim.x * blockDim.x) {
        const DevView &v = views[view_of(views, nv, g)];
        int64_t i = g - v.offset;
        float4 p = ps.pixel[g];
        V3 c = V3{p.x, p.y, p.z} / spp;
        if (clamp) c = vmin(vmax(c, v3(0.f)), v3(clamp_max));
        int64_t x = i % v.w, y = i / v.w;
        out[v.offset + (v.h - 1 - y) * (int64_t)v.w + x] = f4(c, 1.f);
    }
}

// ---------------------------------------------------------------- megakernel
// The stage loop of integrator.cpp:223-266 run as one kernel, one thread per
// pixel path: each bounce's closest hit, emission or environment, NEE shadow
// ray and BSDF sample are taken in registers in the stages' order, with the
// same device functions, so a pixel's radiance equals the wavefront pass's
// bit for bit.  It is the queue-free side of an A/B against the wavefront
// (the reference's MegakernelPathTracer, src/render/megakernel/device.cu:
// 148-195, has the same structure but its own sampling and MIS).  Surfaces
// only: no media and no cache hooks.

// One path of the megakernel between bounces.
struct MkPath {
    V3 ro, rd, thp, pu, pl, ctx_p, L, acc;
    ulonglong2 rng;        // Pcg state, inc
    float4 hit;            // closest hit of ro, rd: t, b1, b2, id
    uint32_t pixel, flags, depth;
    int32_t medium;
    uint32_t alive;
};

// generateCameraRays for the path's pixel (integrator.cpp:166-179).
__device__ __forceinline__ void mk_camera(MkPath &p, Pcg &rng, const DevView &v, int64_t i) {
    const DevCamera &cam = v.cam;
    float fx = rng.get1d(), fy = rng.get1d();
    float lx = rng.get1d(), ly = rng.get1d();
    float tm = rng.get1d();
    (void)lx; (void)ly; (void)tm;
    float px = (float)(i % v.w) + 0.5f + fx;
    float py = (float)(i / v.w) + 0.5f + fy;
    float ndcx = (2 * px) / (float)v.w + (-1.f);
    float ndcy = (2 * py) / (float)v.h + (-1.f);
    V3 fd = normalize(V3{cam.tan_fov * cam.aspect * ndcx, cam.tan_fov * ndcy, -1.f});
    p.ro = V3{cam.pos[0], cam.pos[1], cam.pos[2]};
    p.rd = mat3_mul(cam.rot, fd);
    p.ctx_p = v3(0.f);
    p.thp = p.pu = p.pl = v3(1.f);
    p.flags = 0u;
    p.depth = 0u;
    p.medium = cam.medium;
    p.alive = 1u;
}

// One bounce after the closest hit p.hit: handleMiss / handleHit, then
// generateScatterRays with its NEE shadow ray traced in place; returns
// whether the path continues (its next ray in p.ro, p.rd).
template <int FMT>
__device__ __forceinline__ bool mk_bounce(const DevScene &s, const WfConst &c, const float4 *__restrict__ nodes,
                                          const float4 *__restrict__ tris, MkPath &p, Pcg &rng, int iter,
                                          float lsel_pdf, int *trace_err) {
    const float4 h = p.hit;
    const uint32_t gid = ubits(h.w);
    bool next = false, scatter = false;
    Surf sf;
    if (gid == KRR_MISS) {
        if (s.n_infinite > 0) {
            V3 Lm = v3(0.f);
            for (int k = 0; k < s.n_infinite; ++k) {
                const DevInfinite &e = s.infinite[k];
                if (c.nee && p.depth && !(p.flags & BSDF_DELTA)) {
                    float light_pdf = kInv4Pi * lsel_pdf;
                    Lm += env_Li(e, p.rd) / mean(p.pu + p.pl * light_pdf);
                } else {
                    Lm += env_Li(e, p.rd) / mean(p.pu);
                }
            }
            V3 add = p.thp * Lm;
            p.L = add + p.L;
        }
    } else {
        sf = prepare_surface(s, h.y, h.z, gid, p.rd);
        if (sf.material < 0) {
            // null material: the same ray continues from the interface
            p.ro = offset_ray_origin(sf.p, sf.n, p.rd);
            p.medium = medium_towards(sf.interface_in, sf.interface_out, p.medium, sf.n, p.rd);
            next = true;
        } else {
            if (sf.light >= 0) {
                const DevLight &l = s.lights[sf.light];
                const DevInstance &I = s.instances[l.index];
                V3 Le = area_L(I, sf.n, sf.wo) * p.thp;
                if (c.nee && p.depth && !(p.flags & BSDF_DELTA)) {
                    float light_pdf = area_pdf(s, l, sf.p, sf.n, p.ctx_p) * lsel_pdf;
                    Le = Le / mean(p.pl * light_pdf + p.pu);
                } else {
                    Le = Le / mean(p.pu);
                }
                p.L = Le + p.L;
            }
            scatter = any(p.thp);
        }
    }
    if (iter == c.max_depth) return false;
    if (scatter) {
        if (rng.get1d() >= c.rr) return false;
        V3 sthp = p.thp / c.rr;
        const DevMesh &M = s.meshes[sf.mesh];
        bool transition = M.medium_inside != M.medium_outside;
        int32_t mi = transition ? M.medium_inside : -2, mo = transition ? M.medium_outside : -2;
        const V3 tg = sf.t, bt = sf.b, nrm = sf.n, pp = sf.p;
        auto to_local = [&](V3 w) { return V3{dot(tg, w), dot(bt, w), dot(nrm, w)}; };
        V3 wo_local = to_local(sf.wo);
        ShadingData sd = shading_data(s, sf.material);
        uint32_t bsdf_type = bsdf_type_of(sd);
        Bsdf bsdf = Bsdf::setup(sd);
        if (c.nee && (bsdf_type & BSDF_SMOOTH) && s.n_lights > 0) {
            float ul = rng.get1d();
            uint32_t lid = (uint32_t)(ul * (float)s.n_lights);
            float sel_pdf = 1.f / (float)s.n_lights;
            float u0 = rng.get1d(), u1 = rng.get1d();
            LightSample ls = sample_li(s, s.lights[lid], u0, u1, pp);
            V3 to = offset_ray_origin(ls.p, ls.n, pp - ls.p);
            V3 po = offset_ray_origin(pp, nrm, to - pp);
            V3 d = to - po;
            V3 wi_world = normalize(d);
            V3 wi_local = to_local(wi_world);
            float light_pdf = sel_pdf * ls.pdf;
            V3 fv = bsdf.f(wo_local, wi_local);
            float bsdf_pdf = bsdf.pdf(wo_local, wi_local);
            if (light_pdf > 0 && any(fv)) {
                V3 Ld = ls.L * sthp * fv * fabsf(wi_local.z);
                if (any(Ld)) {
                    // traceShadow + resolve
                    float4 sh = traverse_ray<true, FMT>(nodes, tris, po, d, 0.f, 1.f, trace_err);
                    if (ubits(sh.w) == KRR_MISS) {
                        V3 add = Ld / mean(p.pu * light_pdf + p.pu * bsdf_pdf);
                        p.L = add + p.L;
                    }
                }
            }
        }
        BsdfSample bs = bsdf.sample(wo_local, [&]() { return rng.get1d(); });
        if (bs.pdf != 0 && any(bs.f)) {
            V3 wi_world = tg * bs.wi.x + bt * bs.wi.y + nrm * bs.wi.z;
            V3 nthp = sthp * bs.f * fabsf(bs.wi.z) / bs.pdf;
            if (any(nthp)) {
                p.ro = offset_ray_origin(pp, nrm, wi_world);
                p.medium = medium_towards(mi, mo, p.medium, nrm, wi_world);
                p.rd = wi_world;
                p.ctx_p = pp;
                p.flags = bs.flags;
                p.thp = nthp;
                p.depth = p.depth + 1;
                p.pl = p.pu / bs.pdf;
                next = true;
            }
        }
    }
    return next;
}

__device__ __forceinline__ void mk_finish_pixel(const MkPath &p, const DevView &v, int64_t i, const WfConst &c,
                                                float4 *__restrict__ out) {
    V3 col = p.acc / (float)c.spp;
    if (c.enable_clamp) col = vmin(vmax(col, v3(0.f)), v3(c.clamp_max));
    const int64_t x = i % v.w, y = i / v.w;
    out[v.offset + (v.h - 1 - y) * (int64_t)v.w + x] = f4(col, 1.f);
}

template <int FMT>
__global__ void __launch_bounds__(128)
k_megakernel(DevScene s, const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
             const DevView *__restrict__ views, const FrameConst *__restrict__ fc, PixelState ps,
             WfConst c, int independent, int64_t n, float4 *__restrict__ out, uint32_t *err,
             int *trace_err) {
    const int nv = fc->n_views;
    const float lsel_pdf = 1.f / (float)s.n_lights;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
         g += (int64_t)gridDim.x * blockDim.x) {
        const DevView &v = views[view_of(views, nv, g)];
        const int64_t i = g - v.offset;
        Pcg rng = load_rng(ps, (uint32_t)g);
        const float4 l0 = ps.L[g], p0 = ps.pixel[g];
        MkPath p;
        p.L = f3(l0);
        p.acc = f3(p0);
        for (int sample = 0; sample < c.spp; ++sample) {
            mk_camera(p, rng, v, i);
            for (int iter = 0;; ++iter) {
                p.hit = traverse_ray<false, FMT>(nodes, tris, p.ro, p.rd, 0.f, INFINITY, trace_err);
                if (!mk_bounce<FMT>(s, c, nodes, tris, p, rng, iter, lsel_pdf, trace_err)) break;
            }
            p.acc = V3{p.acc.x + p.L.x, p.acc.y + p.L.y, p.acc.z + p.L.z};
            if (independent && sample + 1 < c.spp) p.L = v3(0.f);
        }
        store_rng(ps, (uint32_t)g, rng);
        ps.L[g] = make_float4(p.L.x, p.L.y, p.L.z, l0.w);
        ps.pixel[g] = make_float4(p.acc.x, p.acc.y, p.acc.z, 0.f);
        mk_finish_pixel(p, v, i, c, out);
    }
}

// The megakernel with a coherence step in the manner of the reference's
// optixReorder(hit, 1) (src/render/megakernel/device.cu:173-176): the 128
// paths of a block advance one bounce at a time; after each closest hit the
// paths move between the block's threads (through shared memory) so that
// paths that missed, paths on each material class and finished paths are
// contiguous, and each warp shades paths of one class.  A path's arithmetic
// is unchanged, so the frame equals the unsorted megakernel's and the
// wavefront's bit for bit.
constexpr int kMkThreads = 128;

__device__ __forceinline__ int mk_class(const DevScene &s, const MkPath &p) {
    if (!p.alive) return 4;
    const uint32_t gid = ubits(p.hit.w);
    if (gid == KRR_MISS) return 0;
    const DevInstance &I = s.instances[s.tri_instance[gid]];
    const int32_t m = s.meshes[I.mesh].material;
    return m < 0 ? 0 : min(max(s.materials[m].type, 0), 3);
}

template <int FMT>
__global__ void __launch_bounds__(kMkThreads)
k_megakernel_sorted(DevScene s, const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
                    const DevView *__restrict__ views, const FrameConst *__restrict__ fc, PixelState ps,
                    WfConst c, int independent, int64_t n, float4 *__restrict__ out, uint32_t *err,
                    int *trace_err) {
    __shared__ MkPath sh[kMkThreads];
    __shared__ int counts[5];
    const int nv = fc->n_views;
    const float lsel_pdf = 1.f / (float)s.n_lights;
    const int tid = threadIdx.x;
    for (int64_t base = blockIdx.x * (int64_t)kMkThreads; base < n; base += (int64_t)gridDim.x * kMkThreads) {
        const int64_t g0 = base + tid;
        for (int sample = 0; sample < c.spp; ++sample) {
            MkPath p;
            if (g0 < n) {
                const DevView &v = views[view_of(views, nv, g0)];
                Pcg rng = load_rng(ps, (uint32_t)g0);
                const float4 l0 = ps.L[g0], p0 = ps.pixel[g0];
                p.L = f3(l0);
                p.acc = f3(p0);
                p.pixel = (uint32_t)g0;
                mk_camera(p, rng, v, g0 - v.offset);
                p.rng = make_ulonglong2(rng.state, rng.inc);
            } else {
                p.alive = 0u;
                p.pixel = 0xFFFFFFFFu;
            }
            for (int iter = 0;; ++iter) {
                if (!__syncthreads_or(p.alive)) break;
                if (p.alive) p.hit = traverse_ray<false, FMT>(nodes, tris, p.ro, p.rd, 0.f, INFINITY, trace_err);
                // reorder: counting sort of the block's paths by class
                const int cls = mk_class(s, p);
                if (tid < 5) counts[tid] = 0;
                __syncthreads();
                const int rank = atomicAdd(&counts[cls], 1);
                __syncthreads();
                int off = 0;
                for (int k = 0; k < cls; ++k) off += counts[k];
                sh[off + rank] = p;
                __syncthreads();
                p = sh[tid];
                __syncthreads();
                if (p.alive) {
                    Pcg rng{p.rng.x, p.rng.y};
                    const bool next = mk_bounce<FMT>(s, c, nodes, tris, p, rng, iter, lsel_pdf, trace_err);
                    p.rng = make_ulonglong2(rng.state, rng.inc);
                    if (!next) {
                        // the path's sample ends: its pixel's sums and sampler
                        p.acc = V3{p.acc.x + p.L.x, p.acc.y + p.L.y, p.acc.z + p.L.z};
                        if (independent && sample + 1 < c.spp) p.L = v3(0.f);
                        ps.rng[p.pixel] = p.rng;
                        ps.L[p.pixel] = make_float4(p.L.x, p.L.y, p.L.z, ps.L[p.pixel].w);
                        ps.pixel[p.pixel] = make_float4(p.acc.x, p.acc.y, p.acc.z, 0.f);
                        p.alive = 0u;
                    }
                }
            }
            __syncthreads();   // every path of the block has stored its pixel
        }
        if (g0 < n) {
            const DevView &v = views[view_of(views, nv, g0)];
            const float4 a = ps.pixel[g0];
            MkPath q;
            q.acc = f3(a);
            mk_finish_pixel(q, v, g0 - v.offset, c, out);
        }
        __syncthreads();
    }
}

// Instance flattening: world-space vertices in instance-major triangle order,
// each row m0*x + m1*y + m2*z + m3 rounded operation by operation.
__global__ void k_flatten(const DevScene s, int n_inst, float *out, int64_t n_tris) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n_tris;
         g += (int64_t)gridDim.x * blockDim.x) {
        uint32_t inst = s.tri_instance[g];
        const DevInstance &I = s.instances[inst];
        const DevMesh &M = s.meshes[I.mesh];
        uint32_t prim = (uint32_t)g - I.prim_offset;
        for (int k = 0; k < 3; ++k) {
            uint32_t vi = M.idx[3 * prim + k];
            float x = M.pos[3 * vi], y = M.pos[3 * vi + 1], z = M.pos[3 * vi + 2];
            for (int r = 0; r < 3; ++r) {
                const float *m = I.xf + 4 * r;
                float acc = __fmul_rn(m[0], x);
                acc = __fadd_rn(acc, __fmul_rn(m[1], y));
                acc = __fadd_rn(acc, __fmul_rn(m[2], z));
                out[9 * g + 3 * k + r] = __fadd_rn(acc, m[3]);
            }
        }
    }
}

__global__ void k_fill_instance_ids(uint32_t *tri_instance, const uint32_t *offsets, int n_inst,
                                    int64_t n_tris) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n_tris;
         g += (int64_t)gridDim.x * blockDim.x) {
        // binary search over instance offsets
        int lo = 0, hi = n_inst - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (offsets[mid] <= (uint32_t)g) lo = mid;
            else hi = mid - 1;
        }
        tri_instance[g] = (uint32_t)lo;
    }
}

__global__ void k_null_mask(const DevScene s, int64_t n_tris, uint8_t *mask) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n_tris;
         g += (int64_t)gridDim.x * blockDim.x) {
        const DevInstance &I = s.instances[s.tri_instance[g]];
        mask[g] = s.meshes[I.mesh].material >= 0 ? 1 : 0;
    }
}

}  // namespace

// --------------------------------------------------------------- host side
namespace {

int grid_for(int64_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int64_t g = (n + kThreads - 1) / kThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)sms * 8));
}

// Blocks of the grid-stride stage kernels: enough for n items, at most the
// pass's blocks per SM on every SM.
int stage_grid(const krr_wf *wf, int64_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int64_t g = (n + wf->block - 1) / wf->block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)sms * wf->blocks_per_sm));
}

template <typename T>
int dev_upload(krr_wf *wf, T **dst, const T *src, size_t count) {
    *dst = nullptr;
    if (count == 0) return KRR_OK;
    KRR_CUDA(cudaMalloc(dst, count * sizeof(T)));
    wf->scene_allocs.push_back(*dst);
    KRR_CUDA(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return KRR_OK;
}

void free_scene(krr_wf *wf) {
    cudaFree(wf->d_world);
    wf->d_world = nullptr;
    for (void *p : wf->scene_allocs) cudaFree(p);
    wf->scene_allocs.clear();
    accel_free(&wf->accel);
    wf->scene = DevScene{};
    wf->has_scene = false;
}

void free_queues(krr_wf *wf) {
    for (auto &q : wf->qbuf) { cudaFree(q); q = nullptr; }
    cudaFree(wf->d_counts); wf->d_counts = nullptr;
    cudaFree(wf->hits); wf->hits = nullptr;
    cudaFree(wf->occluded); wf->occluded = nullptr;
    cudaFree(wf->media_shadow); wf->media_shadow = nullptr;
    cudaFree(wf->scatter_lists); wf->scatter_lists = nullptr;
    cudaFree(wf->work_counts); wf->work_counts = nullptr;
    cudaFree(wf->ps.L); cudaFree(wf->ps.pixel); cudaFree(wf->ps.rng);
    wf->ps = PixelState{};
    cudaFree(wf->d_pixel_part); wf->d_pixel_part = nullptr;
    wf->scene.pixel_part = nullptr;
}

// 3x3 inverse-transpose of a row-major 3x4 transform's linear part, in double.
void inverse_transpose(const float *m, float *out) {
    double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    double D = -(b * i - c * h), E = a * i - c * g, F = -(a * h - b * g);
    double G = b * f - c * e, H = -(a * f - c * d), I = a * e - b * d;
    double det = a * A + b * B + c * C;
    // inverse = adj^T / det; its transpose = cofactor matrix / det
    double cof[9] = {A, B, C, D, E, F, G, H, I};
    for (int k = 0; k < 9; ++k) out[k] = (float)(cof[k] / det);
}

}  // namespace


static void free_nrc_buffers(krr_wf *wf) {
    for (void *p : {(void *)wf->nrc_q_in, (void *)wf->nrc_q_meta, (void *)wf->nrc_q_out,
                    (void *)wf->nrc_rec, (void *)wf->nrc_rec_count, (void *)wf->nrc_b_in,
                    (void *)wf->nrc_b_t, (void *)wf->nrc_spread})
        cudaFree(p);
    wf->nrc_q_in = nullptr; wf->nrc_q_meta = nullptr; wf->nrc_q_out = nullptr;
    wf->nrc_rec = nullptr; wf->nrc_rec_count = nullptr; wf->nrc_b_in = nullptr; wf->nrc_b_t = nullptr;
    wf->nrc_spread = nullptr;
    wf->nrc_slots = 0;
}

static int alloc_nrc_buffers(krr_wf *wf) {
    free_nrc_buffers(wf);
    if (!wf->nrc || !wf->n) return KRR_OK;
    int stride = nrc_train_stride(wf->nrc);
    wf->nrc_slots = (wf->n + stride - 1) / stride;
    wf->nrc_rec_max = std::min(16, std::max(1, loop_depth(wf) + 1));
    int64_t batch = nrc_batch_size(wf->nrc);
    KRR_CUDA(cudaMalloc(&wf->nrc_q_in, (size_t)wf->n * kNrcInputs * sizeof(float)));
    KRR_CUDA(cudaMalloc(&wf->nrc_q_meta, (size_t)wf->n * sizeof(float4)));
    KRR_CUDA(cudaMalloc(&wf->nrc_q_out, (size_t)wf->n * 3 * sizeof(float)));
    KRR_CUDA(cudaMalloc(&wf->nrc_rec, (size_t)wf->nrc_slots * wf->nrc_rec_max * kNrcRecFloats * sizeof(float)));
    KRR_CUDA(cudaMalloc(&wf->nrc_spread, (size_t)wf->n * sizeof(float2)));
    KRR_CUDA(cudaMalloc(&wf->nrc_rec_count, (size_t)wf->nrc_slots * sizeof(int32_t)));
    KRR_CUDA(cudaMemset(wf->nrc_rec_count, 0, (size_t)wf->nrc_slots * sizeof(int32_t)));
    KRR_CUDA(cudaMalloc(&wf->nrc_b_in, (size_t)batch * kNrcInputs * sizeof(float)));
    KRR_CUDA(cudaMalloc(&wf->nrc_b_t, (size_t)batch * 3 * sizeof(float)));
    return KRR_OK;
}

// End of a frame with training: build the batch from the recorded vertices
// and take one optimiser step.
static int nrc_train_frame(krr_wf *wf, cudaStream_t st) {
    ProfScope prof(wf, PS_CACHE_TRAIN, st);
    int stride = nrc_train_stride(wf->nrc);
    int64_t batch = nrc_batch_size(wf->nrc);
    KRR_CUDA(cudaMemsetAsync(wf->nrc_b_count(), 0, sizeof(int32_t), st));
    k_nrc_targets<<<grid_for(wf->nrc_slots), kThreads, 0, st>>>(
        wf->nrc_rec, wf->nrc_rec_count, wf->nrc_slots, wf->nrc_rec_max, stride, wf->d_frame, wf->n, wf->ps,
        wf->nrc_b_in, wf->nrc_b_t, wf->nrc_b_count(), (int)batch);
    k_clamp_count<<<1, 32, 0, st>>>(wf->nrc_b_count(), (int)batch);
    KRR_CUDA(cudaGetLastError());
    return nrc_train_device(wf->nrc, wf->nrc_b_in, wf->nrc_b_t, wf->nrc_b_count(), batch, st);
}

extern "C" int krr_wf_set_nrc(krr_wf *wf, krr_nrc *nrc, int32_t train) {
    KRR_CHECK_ARG(wf != nullptr, "pass is NULL");
    cudaDeviceSynchronize();
    wf->nrc = nrc;
    wf->nrc_train = nrc && train;
    return alloc_nrc_buffers(wf);
}

extern "C" void krr_wf_params_default(krr_wf_params *p) {
    if (!p) return;
    p->nee = 1;
    p->enable_medium = 1;
    p->max_depth = 10;
    p->rr = 0.8f;
    p->enable_clamp = 0;
    p->clamp_max = 1e3f;
    p->spp = 1;
    p->seed = 0;
    p->independent_samples = 0;
}

extern "C" int krr_wf_create(const krr_wf_params *params, krr_wf **out) {
    KRR_CHECK_ARG(out != nullptr, "out is NULL");
    krr_wf *wf = new krr_wf();
    if (params) wf->params = *params;
    else krr_wf_params_default(&wf->params);
    if (wf->params.spp < 1) wf->params.spp = 1;
    *out = wf;
    return KRR_OK;
}

extern "C" int krr_wf_destroy(krr_wf *wf) {
    if (!wf) return KRR_OK;
    cudaDeviceSynchronize();
    free_queues(wf);
    free_scene(wf);
    free_nrc_buffers(wf);
    if (wf->graph) cudaGraphExecDestroy(wf->graph);
    for (auto &r : wf->prof) { cudaEventDestroy(r.e0); cudaEventDestroy(r.e1); }
    for (cudaEvent_t e : wf->prof_pool) cudaEventDestroy(e);
    cudaFreeHost(wf->h_views);
    cudaFreeHost(wf->h_frame);
    cudaFree(wf->d_views);
    cudaFree(wf->d_frame);
    delete wf;
    return KRR_OK;
}

extern "C" int krr_wf_get_params(const krr_wf *wf, krr_wf_params *out) {
    KRR_CHECK_ARG(wf && out, "NULL argument");
    *out = wf->params;
    return KRR_OK;
}

extern "C" int krr_wf_set_params(krr_wf *wf, const krr_wf_params *params) {
    KRR_CHECK_ARG(wf && params, "NULL argument");
    KRR_CHECK_ARG(params->max_depth >= 0 && params->spp >= 1, "bad parameters");
    wf->params = *params;
    wf->medium = wf->params.enable_medium && wf->scene.n_media > 0;
    KRR_TRY(ensure_split_buffers(wf));
    return sync_part_depths(wf);
}

extern "C" int krr_wf_set_scene_max_depth(krr_wf *wf, int32_t scene, int32_t max_depth) {
    KRR_CHECK_ARG(wf && wf->has_scene, "no scene");
    KRR_CHECK_ARG(scene >= 0 && scene < wf->n_parts, "scene index out of range");
    KRR_CHECK_ARG(max_depth >= -1, "max_depth >= 0, or -1 for the pass's");
    wf->part_own_depth.resize(wf->parts.size(), -1);
    wf->part_own_depth[scene] = max_depth;
    KRR_TRY(sync_part_depths(wf));
    if (wf->n) KRR_TRY(alloc_nrc_buffers(wf));   // training records per path vertex
    return KRR_OK;
}

// Flattens the instances to world space and builds the BVH over them, with
// the null-material any-hit mask; sets the scene radius (the length of the
// bounding-box diagonal, src/core/device/scene.cpp:108).
// World-space triangles of the instances into the BVH: a full build, or with
// `refit` new boxes over the existing tree (same triangles, moved).
// The scene of each pixel (its view's) for a pass with several scenes; the
// views must name scenes the pass holds.
static int fill_pixel_parts(krr_wf *wf, cudaStream_t st) {
    for (const DevView &v : wf->layout)
        KRR_CHECK_ARG(v.part >= 0 && (!wf->has_scene || v.part < wf->n_parts),
                      "a view names a scene the pass does not hold");
    if (wf->n_parts <= 1 || !wf->n) {
        wf->scene.pixel_part = nullptr;
        return KRR_OK;
    }
    if (!wf->d_pixel_part) KRR_CUDA(cudaMalloc(&wf->d_pixel_part, (size_t)wf->n));
    for (const DevView &v : wf->layout)
        KRR_CUDA(cudaMemsetAsync(wf->d_pixel_part + v.offset, v.part, (size_t)v.w * v.h, st));
    wf->scene.pixel_part = wf->d_pixel_part;
    return KRR_OK;
}

// Each scene's path depth: its own (krr_wf_set_scene_max_depth) or the
// pass's; uploaded with the scene parts.
static int sync_part_depths(krr_wf *wf) {
    wf->part_own_depth.resize(wf->parts.size(), -1);
    for (size_t p = 0; p < wf->parts.size(); ++p)
        wf->parts[p].max_depth = wf->part_own_depth[p] >= 0 ? wf->part_own_depth[p] : wf->params.max_depth;
    if (wf->scene.parts)
        KRR_CUDA(cudaMemcpy(const_cast<DevScenePart *>(wf->scene.parts), wf->parts.data(),
                            wf->parts.size() * sizeof(DevScenePart), cudaMemcpyHostToDevice));
    return KRR_OK;
}

// After a build or update: per scene the bounding-box diagonal (scene
// radius of the infinite lights, src/core/device/scene.cpp:108) and the
// cache offset that puts the scenes side by side along x.
static int finish_bvh(krr_wf *wf, cudaStream_t st) {
    DevScene &s = wf->scene;
    (void)st;
    // the scenes side by side along x, one scene width apart
    const krr_accel &a = wf->accel;
    const int np = wf->n_parts;
    std::vector<float> b(6 * (size_t)np);
    for (int p = 0; p < np; ++p)
        for (int k = 0; k < 6; ++k)
            b[6 * p + k] = np == 1 ? (k < 3 ? a.scene_lo[k] : a.scene_hi[k - 3])
                                   : a.part_bounds[6 * (size_t)p + k];
    wf->part_radius.assign(np, 0.f);
    float x_end = 0.f;
    for (int k = 0; k < 3; ++k) { wf->cache_lo[k] = INFINITY; wf->cache_hi[k] = -INFINITY; }
    for (int p = 0; p < np; ++p) {
        const float dx = b[6 * p + 3] - b[6 * p], dy = b[6 * p + 4] - b[6 * p + 1], dz = b[6 * p + 5] - b[6 * p + 2];
        wf->part_radius[p] = std::sqrt(dx * dx + dy * dy + dz * dz);
        DevScenePart &P = wf->parts[p];
        P.cache_offset[0] = p == 0 ? 0.f : x_end + std::max(dx, 1e-3f) - b[6 * p];
        P.cache_offset[1] = P.cache_offset[2] = 0.f;
        x_end = b[6 * p + 3] + P.cache_offset[0];
        for (int k = 0; k < 3; ++k) {
            wf->cache_lo[k] = std::min(wf->cache_lo[k], b[6 * p + k] + P.cache_offset[k]);
            wf->cache_hi[k] = std::max(wf->cache_hi[k], b[6 * p + 3 + k] + P.cache_offset[k]);
        }
    }
    if (s.parts)
        KRR_CUDA(cudaMemcpy(const_cast<DevScenePart *>(s.parts), wf->parts.data(),
                            wf->parts.size() * sizeof(DevScenePart), cudaMemcpyHostToDevice));
    s.part_roots = np > 1 ? wf->accel.d_roots : nullptr;
    if (!wf->h_infinite.empty() && s.infinite) {
        for (size_t i = 0; i < wf->h_infinite.size(); ++i)
            wf->h_infinite[i].scene_radius = wf->part_radius[wf->inf_part[i]];
        KRR_CUDA(cudaMemcpy(const_cast<DevInfinite *>(s.infinite), wf->h_infinite.data(),
                            wf->h_infinite.size() * sizeof(DevInfinite), cudaMemcpyHostToDevice));
    }
    return KRR_OK;
}


// The two-level structure of the pass's instances: one tree per distinct
// mesh geometry (meshes that share arrays share one), an instance tree over
// them; an update rebuilds only the instance tree.  Null-material meshes
// let any-hit rays through by their instance's mask.
static int build_two_level(krr_wf *wf, cudaStream_t st, bool update) {
    const int n = wf->n_instances;
    std::vector<float> xf(12 * (size_t)std::max(n, 1));
    for (int i = 0; i < n; ++i) std::memcpy(&xf[12 * (size_t)i], wf->h_instances[i].xf, 12 * sizeof(float));
    if (update) return accel_update_instances(&wf->accel, xf.data(), st);
    std::vector<DevMesh> meshes(wf->h_mesh);
    std::vector<int32_t> geom_of_mesh(meshes.size(), -1), inst_geom(n);
    std::vector<int64_t> geom_begin{0};
    std::vector<int32_t> geom_mesh;
    std::vector<uint8_t> mask(n);
    for (int i = 0; i < n; ++i) {
        const int m = wf->h_instances[i].mesh;
        if (geom_of_mesh[m] < 0) {
            for (size_t g = 0; g < geom_mesh.size(); ++g) {
                const DevMesh &o = meshes[geom_mesh[g]];
                if (o.pos == meshes[m].pos && o.idx == meshes[m].idx &&
                    wf->h_mesh_tris[geom_mesh[g]] == wf->h_mesh_tris[m]) {
                    geom_of_mesh[m] = (int32_t)g;
                    break;
                }
            }
            if (geom_of_mesh[m] < 0) {
                geom_of_mesh[m] = (int32_t)geom_mesh.size();
                geom_mesh.push_back(m);
                geom_begin.push_back(geom_begin.back() + wf->h_mesh_tris[m]);
            }
        }
        inst_geom[i] = geom_of_mesh[m];
        mask[i] = meshes[m].material >= 0 ? 1 : 0;
    }
    if (geom_mesh.empty()) {   // no instances: one empty geometry
        geom_mesh.push_back(-1);
        geom_begin.push_back(0);
    }
    float *d_obj = nullptr;
    KRR_CUDA(cudaMalloc(&d_obj, std::max<int64_t>(geom_begin.back(), 1) * 9 * sizeof(float)));
    int stat = KRR_OK;
    for (size_t g = 0; g < geom_mesh.size() && stat == KRR_OK; ++g)
        if (geom_mesh[g] >= 0)
            stat = geometry_triangles(meshes[geom_mesh[g]].pos, meshes[geom_mesh[g]].idx,
                                      geom_begin[g + 1] - geom_begin[g], d_obj + 9 * geom_begin[g], st);
    InstancedInput in{d_obj, geom_begin.data(), (int)geom_mesh.size(), inst_geom.data(), xf.data(),
                      mask.data(), n};
    if (stat == KRR_OK) stat = accel_build_instanced(&wf->accel, in, st);
    cudaStreamSynchronize(st);
    cudaFree(d_obj);
    return stat;
}

static int rebuild_bvh(krr_wf *wf, cudaStream_t st, bool refit = false) {
    const uint64_t n_tris = wf->n_tris;
    DevScene &s = wf->scene;
    if (wf->levels == 2) {
        KRR_TRY(build_two_level(wf, st, refit));
        return finish_bvh(wf, st);
    }
    // the flattened triangles: kept after a refit (the next update refits
    // again), freed after a build (a scene that never moves does not hold them)
    if (!wf->d_world)
        KRR_CUDA(cudaMalloc(&wf->d_world, std::max<uint64_t>(n_tris, 1) * 9 * sizeof(float)));
    float *d_world = wf->d_world;
    if (n_tris) k_flatten<<<grid_for(n_tris), kThreads, 0, st>>>(s, wf->n_instances, d_world, n_tris);
    KRR_CUDA(cudaGetLastError());
    int stat = refit ? accel_refit(&wf->accel, d_world, (int64_t)n_tris, st)
                     : accel_build_parts(&wf->accel, d_world, wf->part_tri_begin.data(), wf->n_parts, st);
    if (stat == KRR_OK) stat = cuda_status(cudaStreamSynchronize(st), "BVH", __FILE__, __LINE__);
    if (!refit || stat != KRR_OK) {
        cudaFree(wf->d_world);
        wf->d_world = nullptr;
    }
    if (stat != KRR_OK) return stat;
    // null-material triangles never block shadow rays (device.cu:83-88); a
    // refit keeps the mask words of the triangle records
    if (n_tris && !refit) {
        uint8_t *mask = nullptr;
        KRR_CUDA(cudaMalloc(&mask, n_tris));
        k_null_mask<<<grid_for(n_tris), kThreads, 0, st>>>(s, (int64_t)n_tris, mask);
        stat = cuda_status(cudaGetLastError(), "k_null_mask", __FILE__, __LINE__);
        if (stat == KRR_OK) stat = accel_set_mask(&wf->accel, mask, st);
        if (stat == KRR_OK) stat = cuda_status(cudaStreamSynchronize(st), "mask", __FILE__, __LINE__);
        cudaFree(mask);
        if (stat != KRR_OK) return stat;
    }
    return finish_bvh(wf, st);
}

extern "C" int krr_wf_set_scene(krr_wf *wf, const krr_scene_desc *sd, void *stream) {
    KRR_CHECK_ARG(wf && sd, "NULL argument");
    return krr_wf_set_scenes(wf, sd, 1, stream);
}

extern "C" int krr_wf_set_scenes(krr_wf *wf, const krr_scene_desc *scenes, int32_t n_scenes,
                                 void *stream) {
    KRR_CHECK_ARG(wf && scenes, "NULL argument");
    KRR_CHECK_ARG(n_scenes >= 1 && n_scenes <= 255, "1..255 scenes");
    for (int p = 0; p < n_scenes; ++p)
        KRR_CHECK_ARG(scenes[p].n_meshes >= 0 && scenes[p].n_instances >= 0 &&
                          scenes[p].n_materials >= 0 && scenes[p].n_infinite_lights >= 0 &&
                          scenes[p].n_media >= 0,
                      "negative counts");
    cudaStream_t st = as_stream(stream);
    cudaDeviceSynchronize();
    free_scene(wf);

    // where each scene's meshes, materials, instances, infinite lights and
    // media start in the pass's arrays
    std::vector<int32_t> mesh0(n_scenes + 1, 0), mat0(n_scenes + 1, 0), inst0(n_scenes + 1, 0),
        inf0(n_scenes + 1, 0), med0(n_scenes + 1, 0);
    for (int p = 0; p < n_scenes; ++p) {
        mesh0[p + 1] = mesh0[p] + scenes[p].n_meshes;
        mat0[p + 1] = mat0[p] + scenes[p].n_materials;
        inst0[p + 1] = inst0[p] + scenes[p].n_instances;
        inf0[p + 1] = inf0[p] + scenes[p].n_infinite_lights;
        med0[p + 1] = med0[p] + scenes[p].n_media;
    }

    // meshes
    std::vector<DevMesh> meshes(mesh0[n_scenes]);
    for (int p = 0; p < n_scenes; ++p) {
        const krr_scene_desc *sd = scenes + p;
        for (int i = 0; i < sd->n_meshes; ++i) {
            const krr_mesh_desc &m = sd->meshes[i];
            KRR_CHECK_ARG(m.h_positions && m.h_normals && m.h_indices, "mesh arrays missing (normals are required)");
            KRR_CHECK_ARG(m.material < sd->n_materials, "mesh material out of range");
            KRR_CHECK_ARG(m.medium_inside < sd->n_media && m.medium_outside < sd->n_media,
                          "mesh medium out of range");
            // meshes that share arrays (same host pointers) share device copies
            int shared = -1;
            for (int j = 0; j < i; ++j)
                if (sd->meshes[j].h_positions == m.h_positions && sd->meshes[j].h_indices == m.h_indices &&
                    sd->meshes[j].n_vertices == m.n_vertices && sd->meshes[j].n_triangles == m.n_triangles &&
                    sd->meshes[j].h_normals == m.h_normals && sd->meshes[j].h_texcoords == m.h_texcoords) {
                    shared = mesh0[p] + j;
                    break;
                }
            DevMesh d{};
            if (shared >= 0) {
                d = meshes[shared];
            } else {
                for (int64_t k = 0; k < 3 * m.n_triangles; ++k)
                    KRR_CHECK_ARG(m.h_indices[k] < (uint64_t)m.n_vertices, "mesh index out of range");
                KRR_TRY(dev_upload(wf, const_cast<float **>(&d.pos), m.h_positions, 3 * m.n_vertices));
                KRR_TRY(dev_upload(wf, const_cast<float **>(&d.nrm), m.h_normals, 3 * m.n_vertices));
                if (m.h_texcoords) KRR_TRY(dev_upload(wf, const_cast<float **>(&d.uv), m.h_texcoords, 2 * m.n_vertices));
                KRR_TRY(dev_upload(wf, const_cast<uint32_t **>(&d.idx), m.h_indices, 3 * m.n_triangles));
            }
            d.material = m.material >= 0 ? m.material + mat0[p] : m.material;
            d.medium_inside = m.medium_inside >= 0 ? m.medium_inside + med0[p] : m.medium_inside;
            d.medium_outside = m.medium_outside >= 0 ? m.medium_outside + med0[p] : m.medium_outside;
            meshes[mesh0[p] + i] = d;
        }
    }
    // materials (src/scene/krrscene.cpp:208-227: specular alpha = 1 - roughness)
    std::vector<DevMaterial> mats(std::max(1, mat0[n_scenes]));
    for (int p = 0; p < n_scenes; ++p)
        for (int i = 0; i < scenes[p].n_materials; ++i) {
            const krr_material_desc &m = scenes[p].materials[i];
            KRR_CHECK_ARG(m.type >= 0 && m.type <= 3, "unknown material type");
            DevMaterial d{};
            d.type = m.type;
            for (int k = 0; k < 3; ++k) d.diffuse[k] = m.diffuse[k];
            d.spec_alpha = 1.f - m.roughness;
            d.spec_trans = m.specular_transmission;
            d.eta = m.eta;
            d.anisotropic = m.anisotropic;
            mats[mat0[p] + i] = d;
        }
    // instances, triangle offsets and each scene's light list
    // (src/core/device/scene.cpp:93-132): its mesh lights, then its infinite
    // lights
    std::vector<DevInstance> insts(inst0[n_scenes]);
    std::vector<DevLight> lights;
    std::vector<uint32_t> offsets(std::max(1, inst0[n_scenes]));
    std::vector<DevScenePart> parts(n_scenes);
    std::vector<int64_t> tri_begin(n_scenes + 1, 0);
    uint64_t n_tris = 0;
    for (int p = 0; p < n_scenes; ++p) {
        const krr_scene_desc *sd = scenes + p;
        DevScenePart &P = parts[p];
        P.light_begin = (int32_t)lights.size();
        tri_begin[p] = (int64_t)n_tris;
        for (int i = 0; i < sd->n_instances; ++i) {
            const krr_instance_desc &in = sd->instances[i];
            KRR_CHECK_ARG(in.mesh >= 0 && in.mesh < sd->n_meshes, "instance mesh out of range");
            const krr_mesh_desc &m = sd->meshes[in.mesh];
            const int gi = inst0[p] + i;
            DevInstance d{};
            std::memcpy(d.xf, in.transform, sizeof(d.xf));
            inverse_transpose(in.transform, d.nxf);
            d.mesh = in.mesh + mesh0[p];
            d.prim_offset = (uint32_t)n_tris;
            offsets[gi] = (uint32_t)n_tris;
            d.light_offset = -1;
            float le[3] = {m.emission[0], m.emission[1], m.emission[2]};
            if (le[0] > 0.f || le[1] > 0.f || le[2] > 0.f) {
                float scale = std::max(le[0], std::max(le[1], le[2]));   // mesh.cpp:47-48
                for (int k = 0; k < 3; ++k) d.le[k] = le[k] / scale;
                d.le_scale = scale;
                d.light_offset = (int32_t)lights.size();
                for (int64_t t = 0; t < m.n_triangles; ++t) lights.push_back(DevLight{0, gi, (uint32_t)t, 0});
            }
            insts[gi] = d;
            n_tris += (uint64_t)m.n_triangles;
            KRR_CHECK_ARG(n_tris < 0x7fffffffull, "too many triangles");
        }
        // infinite lights follow the scene's mesh lights
        P.inf_begin = inf0[p];
        P.n_infinite = sd->n_infinite_lights;
        for (int i = 0; i < sd->n_infinite_lights; ++i) lights.push_back(DevLight{1, inf0[p] + i, 0, 0});
        P.n_lights = (int32_t)lights.size() - P.light_begin;
        P.has_media = sd->n_media > 0 ? 1 : 0;
    }
    tri_begin[n_scenes] = (int64_t)n_tris;
    std::vector<DevInfinite> infs(std::max(0, inf0[n_scenes]));
    std::vector<int32_t> inf_part(inf0[n_scenes]);
    for (int p = 0; p < n_scenes; ++p)
        for (int i = 0; i < scenes[p].n_infinite_lights; ++i) {
            const krr_infinite_light_desc &l = scenes[p].infinite_lights[i];
            DevInfinite d{};
            for (int k = 0; k < 3; ++k) d.tint[k] = l.tint[k];
            d.scale = l.scale;
            std::memcpy(d.rot, l.rotation, sizeof(d.rot));
            if (l.h_image) {
                KRR_CHECK_ARG(l.width > 0 && l.height > 0, "environment image size");
                float4 *img = nullptr;
                KRR_TRY(dev_upload(wf, &img, reinterpret_cast<const float4 *>(l.h_image),
                                   (size_t)l.width * l.height));
                d.image = img;
                d.w = l.width;
                d.h = l.height;
            }
            infs[inf0[p] + i] = d;
            inf_part[inf0[p] + i] = p;
        }
    // A scene without lights is accepted: light sampling is skipped (every
    // NEE site tests the scene's light count) and its frames are black.

    DevScene s{};
    KRR_TRY(dev_upload(wf, const_cast<DevMesh **>(&s.meshes), meshes.data(), meshes.size()));
    KRR_TRY(dev_upload(wf, const_cast<DevMaterial **>(&s.materials), mats.data(), mats.size()));
    KRR_TRY(dev_upload(wf, const_cast<DevInstance **>(&s.instances), insts.data(), insts.size()));
    KRR_TRY(dev_upload(wf, const_cast<DevLight **>(&s.lights), lights.data(), lights.size()));
    s.n_lights = (int32_t)lights.size();
    KRR_TRY(dev_upload(wf, const_cast<DevScenePart **>(&s.parts), parts.data(), parts.size()));
    s.n_parts = n_scenes;
    uint32_t *d_offsets = nullptr;
    KRR_TRY(dev_upload(wf, &d_offsets, offsets.data(), offsets.size()));
    uint32_t *tri_inst = nullptr;
    KRR_CUDA(cudaMalloc(&tri_inst, std::max<uint64_t>(n_tris, 1) * sizeof(uint32_t)));
    wf->scene_allocs.push_back(tri_inst);
    if (n_tris)
        k_fill_instance_ids<<<grid_for(n_tris), kThreads, 0, st>>>(tri_inst, d_offsets,
                                                                   inst0[n_scenes], n_tris);
    KRR_CUDA(cudaGetLastError());
    s.tri_instance = tri_inst;
    KRR_TRY(dev_upload(wf, const_cast<DevInfinite **>(&s.infinite), infs.data(), infs.size()));
    s.n_infinite = (int32_t)infs.size();

    // media
    std::vector<DevMedium> media(med0[n_scenes]);
    for (int p = 0; p < n_scenes; ++p)
        for (int i = 0; i < scenes[p].n_media; ++i) {
            const krr_medium_desc &m = scenes[p].media[i];
            DevMedium d{};
            d.nx = m.nx; d.ny = m.ny; d.nz = m.nz;
            for (int k = 0; k < 3; ++k) {
                d.lo[k] = m.bounds_min[k]; d.hi[k] = m.bounds_max[k];
                d.sigma_t[k] = m.sigma_t[k]; d.albedo[k] = m.albedo[k];
                d.mres[k] = std::max(1, m.majorant_res[k]);
                d.idx_scale[k] = (float)(k == 0 ? m.nx : k == 1 ? m.ny : m.nz) / (d.hi[k] - d.lo[k]);
            }
            d.g = m.g;
            d.scale = m.scale;
            if (m.h_density) {
                KRR_CHECK_ARG(m.nx > 0 && m.ny > 0 && m.nz > 0, "density grid size");
                const size_t nv = (size_t)m.nx * m.ny * m.nz;
                uint16_t *lin = nullptr;
                uint4 *octets = nullptr;
                KRR_CUDA(cudaMalloc(&octets, nv * sizeof(uint4)));
                wf->scene_allocs.push_back(octets);
                KRR_CUDA(cudaMalloc(&lin, nv * sizeof(uint16_t)));
                cudaError_t ce = cudaMemcpyAsync(lin, m.h_density, nv * sizeof(uint16_t), cudaMemcpyHostToDevice, st);
                if (ce == cudaSuccess) {
                    k_octet_density<<<grid_for((int64_t)nv), kThreads, 0, st>>>(lin, m.nx, m.ny, m.nz,
                                                                                (int64_t)nv, octets);
                    ce = cudaGetLastError();
                }
                if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
                cudaFree(lin);
                if (ce != cudaSuccess) return cuda_status(ce, "density upload", __FILE__, __LINE__);
                d.density = reinterpret_cast<const uint16_t *>(octets);
                float *maj = nullptr;
                size_t nm = (size_t)d.mres[0] * d.mres[1] * d.mres[2];
                KRR_CUDA(cudaMalloc(&maj, nm * sizeof(float)));
                wf->scene_allocs.push_back(maj);
                k_build_majorant<<<grid_for((int64_t)nm), kThreads, 0, st>>>(d, maj);
                KRR_CUDA(cudaGetLastError());
                d.majorant = maj;
            }
            media[med0[p] + i] = d;
        }
    KRR_TRY(dev_upload(wf, const_cast<DevMedium **>(&s.media), media.data(), media.size()));
    s.n_media = med0[n_scenes];
    s.max_null_collisions = wf->max_null_collisions;
    s.max_interface_crossings = wf->max_interface_crossings;
    s.pixel_part = n_scenes > 1 ? wf->d_pixel_part : nullptr;

    // world-space triangles and the BVHs (one tree per scene)
    KRR_CHECK_ARG(wf->levels == 1 || n_scenes == 1, "a two-level structure takes a pass with one scene");
    wf->n_instances = inst0[n_scenes];
    wf->n_tris = n_tris;
    wf->h_mesh = meshes;
    wf->h_mesh_tris.assign(meshes.size(), 0);
    for (int p = 0; p < n_scenes; ++p)
        for (int i = 0; i < scenes[p].n_meshes; ++i) wf->h_mesh_tris[mesh0[p] + i] = scenes[p].meshes[i].n_triangles;
    wf->h_instances = insts;
    wf->h_infinite = infs;
    wf->inf_part = inf_part;
    wf->parts = parts;
    wf->n_parts = n_scenes;
    wf->part_own_depth.assign(n_scenes, -1);
    for (auto &P : wf->parts) P.max_depth = wf->params.max_depth;
    wf->part_tri_begin = tri_begin;
    wf->part_media_begin.assign(med0.begin(), med0.end() - 1);
    wf->scene = s;   // rebuild_bvh reads the uploaded instances and updates parts and radii
    KRR_TRY(rebuild_bvh(wf, st));
    wf->has_scene = true;
    KRR_TRY(ensure_split_buffers(wf));
    wf->medium = wf->params.enable_medium && wf->scene.n_media > 0;
    KRR_TRY(fill_pixel_parts(wf, st));
    KRR_CUDA(cudaStreamSynchronize(st));
    return KRR_OK;
}

extern "C" int krr_wf_set_accel_levels(krr_wf *wf, int32_t levels) {
    KRR_CHECK_ARG(wf != nullptr, "NULL argument");
    KRR_CHECK_ARG(levels == 1 || levels == 2, "levels must be 1 (flattened) or 2 (two-level)");
    KRR_CHECK_ARG(levels == 1 || wf->n_parts == 1, "a two-level structure takes a pass with one scene");
    wf->levels = levels;
    if (!wf->has_scene) return KRR_OK;
    cudaDeviceSynchronize();
    if (wf->graph) { cudaGraphExecDestroy(wf->graph); wf->graph = nullptr; }
    return rebuild_bvh(wf, 0);
}

extern "C" int krr_wf_cache_box(krr_wf *wf, float *lo, float *hi) {
    KRR_CHECK_ARG(wf && lo && hi, "NULL argument");
    KRR_CHECK_ARG(wf->has_scene, "no scene");
    for (int k = 0; k < 3; ++k) { lo[k] = wf->cache_lo[k]; hi[k] = wf->cache_hi[k]; }
    return KRR_OK;
}

// Allocates queues and pixel state for the views of `layout` (offsets set).
static int set_layout(krr_wf *wf, std::vector<DevView> layout) {
    int64_t n = 0;
    for (auto &v : layout) {
        KRR_CHECK_ARG(v.w > 0 && v.h > 0, "bad view size");
        v.offset = n;
        n += (int64_t)v.w * v.h;
    }
    KRR_CHECK_ARG(n > 0 && n < (1ll << 30), "frame too large");
    KRR_CHECK_ARG(layout.size() <= (size_t)kMaxViews, "too many views");
    cudaDeviceSynchronize();
    if (wf->graph) { cudaGraphExecDestroy(wf->graph); wf->graph = nullptr; }
    free_queues(wf);
    if (!wf->h_views) {
        KRR_CUDA(cudaMallocHost(&wf->h_views, kMaxViews * sizeof(DevView)));
        KRR_CUDA(cudaMalloc(&wf->d_views, kMaxViews * sizeof(DevView)));
        KRR_CUDA(cudaMallocHost(&wf->h_frame, sizeof(FrameConst)));
        KRR_CUDA(cudaMalloc(&wf->d_frame, sizeof(FrameConst)));
    }
    wf->layout = layout;
    wf->n_views = (int32_t)layout.size();
    wf->width = layout.size() == 1 ? layout[0].w : 0;
    wf->height = layout.size() == 1 ? layout[0].h : 0;
    wf->n = n;
    wf->qcap = wf->wave > 0 ? std::min(wf->wave, n) : n;
    for (int k = 0; k < Q_COUNT; ++k)
        KRR_CUDA(cudaMalloc(&wf->qbuf[k], (size_t)kChannels[k] * wf->qcap * sizeof(float4)));
    KRR_CUDA(cudaMalloc(&wf->d_counts, 32 * sizeof(int32_t)));
    KRR_CUDA(cudaMemset(wf->d_counts, 0, 32 * sizeof(int32_t)));
    KRR_CUDA(cudaMalloc(&wf->hits, wf->qcap * sizeof(float4)));
    KRR_CUDA(cudaMalloc(&wf->occluded, wf->qcap));
    KRR_CUDA(cudaMalloc(&wf->scatter_lists, 2 * wf->qcap * sizeof(int32_t)));
    KRR_CUDA(cudaMalloc(&wf->work_counts, 2 * kWorkClasses * sizeof(int32_t)));
    KRR_CUDA(cudaMalloc(&wf->ps.L, wf->n * sizeof(float4)));
    KRR_CUDA(cudaMalloc(&wf->ps.pixel, wf->n * sizeof(float4)));
    KRR_CUDA(cudaMalloc(&wf->ps.rng, wf->n * sizeof(ulonglong2)));
    wf->grid = stage_grid(wf, wf->n);
    KRR_TRY(fill_pixel_parts(wf, 0));
    KRR_CUDA(cudaDeviceSynchronize());
    KRR_TRY(ensure_split_buffers(wf));
    return alloc_nrc_buffers(wf);
}

// Scene::update for animated instances (src/core/scene.cpp:17-31,
// OptixSceneSingleLevel::updateAccelStructure, src/core/device/optix.cpp:
// 618-642): new 3x4 transforms for some instances, then the world-space
// triangles are re-flattened and the BVH's boxes refitted over its existing
// tree (the reference rebuilds its instance level over static mesh
// structures; here instances are flattened into one BVH).  Every device
// buffer stays in place, so a captured frame graph stays valid.
// krr_wf_rebuild_bvh restores the tree's quality after large motion.
extern "C" int krr_wf_rebuild_bvh(krr_wf *wf, void *stream) {
    KRR_CHECK_ARG(wf && wf->has_scene, "no scene");
    cudaStream_t st = as_stream(stream);
    KRR_CUDA(cudaStreamSynchronize(st));
    if (wf->graph) {   // the rebuilt BVH lives in new buffers
        cudaGraphExecDestroy(wf->graph);
        wf->graph = nullptr;
    }
    return rebuild_bvh(wf, st);
}

extern "C" int krr_wf_update_instances(krr_wf *wf, int32_t n, const int32_t *h_indices,
                                       const float *h_transforms, void *stream) {
    KRR_CHECK_ARG(wf && wf->has_scene, "no scene");
    KRR_CHECK_ARG(wf->n_parts == 1, "instance updates take a pass with one scene");
    KRR_CHECK_ARG(n >= 0 && (n == 0 || (h_indices && h_transforms)), "bad argument");
    for (int k = 0; k < n; ++k)
        KRR_CHECK_ARG(h_indices[k] >= 0 && h_indices[k] < wf->n_instances, "instance index out of range");
    if (n == 0) return KRR_OK;
    cudaStream_t st = as_stream(stream);
    for (int k = 0; k < n; ++k) {
        DevInstance &d = wf->h_instances[h_indices[k]];
        std::memcpy(d.xf, h_transforms + 12 * k, sizeof(d.xf));
        inverse_transpose(h_transforms + 12 * k, d.nxf);
    }
    KRR_CUDA(cudaStreamSynchronize(st));
    KRR_CUDA(cudaMemcpy(const_cast<DevInstance *>(wf->scene.instances), wf->h_instances.data(),
                        wf->h_instances.size() * sizeof(DevInstance), cudaMemcpyHostToDevice));
    // a refit keeps every device buffer in place, so a captured frame stays valid
    return rebuild_bvh(wf, st, true);
}

extern "C" int krr_wf_resize(krr_wf *wf, int32_t width, int32_t height) {
    KRR_CHECK_ARG(wf && width > 0 && height > 0, "bad frame size");
    DevView v{};
    v.w = width;
    v.h = height;
    return set_layout(wf, {v});
}

extern "C" int krr_wf_resize_views(krr_wf *wf, const krr_view *views, int32_t n_views) {
    KRR_CHECK_ARG(wf && views && n_views >= 1, "bad views");
    std::vector<DevView> layout(n_views);
    for (int i = 0; i < n_views; ++i) {
        layout[i] = DevView{};
        layout[i].w = views[i].width;
        layout[i].h = views[i].height;
        layout[i].seed = (uint32_t)views[i].seed;
        layout[i].part = views[i].scene;
    }
    return set_layout(wf, layout);
}

static int ready(krr_wf *wf) {
    if (!wf) return fail(KRR_ERR_INVALID_ARGUMENT, "pass is NULL");
    if (!wf->has_scene) return fail(KRR_ERR_NOT_READY, "set_scene has not been called");
    if (!wf->n) return fail(KRR_ERR_NOT_READY, "resize has not been called");
    return KRR_OK;
}

static int make_camera(const krr_camera_desc *c, DevCamera &d) {
    KRR_CHECK_ARG(c != nullptr, "camera is NULL");
    KRR_CHECK_ARG(c->lens_radius <= 1e-5f, "thin-lens cameras are not supported");
    d = DevCamera{};
    for (int k = 0; k < 3; ++k) d.pos[k] = c->position[k];
    for (int k = 0; k < 9; ++k) d.rot[k] = c->rotation[k];
    float fov = std::atan2(c->film_size[1] * 0.5f, c->focal_length);
    d.tan_fov = std::tan(fov);
    d.aspect = c->aspect_ratio;
    d.lens_radius = c->lens_radius;
    d.focal_distance = c->focal_distance;
    d.shutter_open = c->shutter_open;
    d.shutter_time = c->shutter_time;
    d.medium = c->medium;
    return KRR_OK;
}

// Fills the view table and frame constants of frame `frame_index` into the
// given host arrays (cameras == nullptr keeps the current cameras).
static int fill_frame(krr_wf *wf, int64_t frame_index, const krr_camera_desc *single,
                      const krr_view *views, int32_t n_views, DevView *dv, FrameConst *fc) {
    // a camera's medium indexes its scene's media
    auto camera_medium = [&](DevView &v) {
        if (v.cam.medium >= 0 && v.part < (int)wf->part_media_begin.size())
            v.cam.medium += wf->part_media_begin[v.part];
    };
    if (single) {
        KRR_CHECK_ARG(wf->n_views == 1, "the pass has a multi-view layout: use begin_frame_views");
        DevView v = wf->layout[0];
        KRR_TRY(make_camera(single, v.cam));
        camera_medium(v);
        v.seed = (uint32_t)wf->params.seed;
        v.sample_index = (uint32_t)(frame_index * wf->params.spp + v.seed);
        wf->layout[0] = v;
    } else if (views) {
        KRR_CHECK_ARG(n_views == wf->n_views, "view count differs from the layout");
        for (int i = 0; i < n_views; ++i) {
            KRR_CHECK_ARG(views[i].width == wf->layout[i].w && views[i].height == wf->layout[i].h,
                          "view size differs from the layout");
            KRR_CHECK_ARG(views[i].scene == wf->layout[i].part, "view scene differs from the layout");
            KRR_TRY(make_camera(&views[i].camera, wf->layout[i].cam));
            camera_medium(wf->layout[i]);
            wf->layout[i].seed = (uint32_t)views[i].seed;
            wf->layout[i].sample_index = (uint32_t)(frame_index * wf->params.spp + views[i].seed);
        }
    } else {
        // same cameras, next frame
        for (int i = 0; i < wf->n_views; ++i)
            wf->layout[i].sample_index = (uint32_t)(frame_index * wf->params.spp + wf->layout[i].seed);
    }
    for (int i = 0; i < wf->n_views; ++i) dv[i] = wf->layout[i];
    fc->n_views = wf->n_views;
    fc->frame_index = frame_index;
    fc->nrc_offset = wf->nrc ? (int32_t)(frame_index % nrc_train_stride(wf->nrc)) : 0;
    wf->cam = wf->layout[0].cam;
    wf->frame_index = frame_index;
    return KRR_OK;
}

static int launch_begin_frame(krr_wf *wf, cudaStream_t st) {
    ProfScope prof(wf, PS_BEGIN_FRAME, st);
    k_begin_frame<<<wf->grid, wf->block, 0, st>>>(wf->ps, wf->d_views, wf->d_frame, wf->n);
    KRR_CUDA(cudaGetLastError());
    if (wf->nrc && wf->nrc_rec_count)
        KRR_CUDA(cudaMemsetAsync(wf->nrc_rec_count, 0, wf->nrc_slots * sizeof(int32_t), st));
    return KRR_OK;
}

static int begin_frame_common(krr_wf *wf, int64_t frame_index, const krr_camera_desc *single,
                              const krr_view *views, int32_t n_views, cudaStream_t st) {
    // pageable staging: the copies below take the values before returning
    std::vector<DevView> dv(wf->n_views);
    FrameConst fc{};
    KRR_TRY(fill_frame(wf, frame_index, single, views, n_views, dv.data(), &fc));
    KRR_CUDA(cudaMemcpyAsync(wf->d_views, dv.data(), dv.size() * sizeof(DevView),
                             cudaMemcpyHostToDevice, st));
    KRR_CUDA(cudaMemcpyAsync(wf->d_frame, &fc, sizeof(FrameConst), cudaMemcpyHostToDevice, st));
    KRR_CUDA(cudaStreamSynchronize(st));
    return launch_begin_frame(wf, st);
}

extern "C" int krr_wf_begin_frame(krr_wf *wf, int64_t frame_index, const krr_camera_desc *c,
                                  void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(c != nullptr, "camera is NULL");
    return begin_frame_common(wf, frame_index, c, nullptr, 0, as_stream(stream));
}

extern "C" int krr_wf_begin_frame_views(krr_wf *wf, int64_t frame_index, const krr_view *views,
                                        int32_t n_views, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(views != nullptr, "views are NULL");
    return begin_frame_common(wf, frame_index, nullptr, views, n_views, as_stream(stream));
}

static int camera_rays(krr_wf *wf, int64_t p0, int64_t count, cudaStream_t st) {
    ProfScope prof(wf, PS_CAMERA, st);
    k_camera_rays<<<stage_grid(wf, count), wf->block, 0, st>>>(wf->ps, wf->q(Q_RAY0), wf->d_views,
                                                               wf->d_frame, p0, count, wf->camera_order);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_generate_camera_rays(krr_wf *wf, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(wf->qcap == wf->n,
                  "the stage entry points trace every pixel at once: the queue capacity must be the "
                  "pixel count (krr_wf_set_launch with wave 0)");
    return camera_rays(wf, 0, wf->n, as_stream(stream));
}

extern "C" int krr_wf_reset_queues(krr_wf *wf, int32_t depth, void *stream) {
    KRR_TRY(ready(wf));
    k_reset_queues<<<1, 32, 0, as_stream(stream)>>>(wf->d_counts, depth & 1, depth < 0 ? 1 : 0);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

// Several scenes: each ray starts at its pixel's scene's root; the pixel id
// is in plane `pix_plane` of the queue.
static void set_roots(const krr_wf *wf, TraceLaunch &l, const Queue &q, int pix_plane, bool any_set) {
    if (wf->n_parts <= 1) return;
    l.roots = wf->accel.d_roots;
    l.pixel_part = wf->d_pixel_part;
    (any_set ? l.any_pix : l.ray_pix) = q.base + (size_t)pix_plane * q.cap;
}

static TraceLaunch closest_launch(krr_wf *wf, int depth) {
    Queue rq = wf->q(depth & 1);
    TraceLaunch l{};
    l.ray_o = rq.base;
    l.ray_d = rq.base + rq.cap;
    l.ray_stride = 1;
    l.n = rq.cap;
    l.d_count = rq.count;
    l.hits = wf->hits;
    l.counter = wf->accel.d_scratch;
    l.err = wf->accel.d_scratch + 4;
    set_roots(wf, l, rq, 5, false);   // Ray: plane 5 = pu | pixel
    return l;
}

// L[pixel] += throughput x cache(query) for the queued cache queries.
static int nrc_evaluate_queries(krr_wf *wf, cudaStream_t st) {
    ProfScope prof(wf, PS_CACHE_QUERY, st);
    KRR_TRY(nrc_query_device(wf->nrc, wf->nrc_q_in, wf->nrc_q_count(), wf->n, wf->nrc_q_out, st));
    k_nrc_apply<<<wf->grid, wf->block, 0, st>>>(wf->nrc_q_out, wf->nrc_q_meta, wf->nrc_q_count(),
                                                (int)wf->n, wf->ps);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

// Routing of the closest hits of ray queue `depth` (already traced into
// wf->hits when `traced`).  With a cache attached, the paths that stop at it
// are evaluated and their radiance added here, or, with `in_render`, left in
// the query buffer for one evaluation at the end of the sample; `in_render`
// without media also adds miss and emission radiance in the routing kernel
// (render() then skips handleHit/handleMiss).
static int closest_stage(krr_wf *wf, int depth, cudaStream_t st, bool traced,
                         bool in_render = false) {
    // In render() the radiance of misses and emissive hits of rays outside
    // every medium is added here; rays inside a medium go to the medium
    // stage, which queues theirs for handleHit/handleMiss.  A path has one
    // item per bounce, so each pixel's sum gets the same terms in the same
    // order either way.
    const bool defer_cache = in_render;
    const int inline_lights = in_render ? 1 : 0;
    int cur = depth & 1;
    Queue rq = wf->q(cur);
    if (!traced) {
        ProfScope prof(wf, PS_TRACE_CLOSEST, st);
        KRR_TRY(launch_trace_closest(&wf->accel, closest_launch(wf, depth), st));
    }
    NrcHook hook{};
    if (wf->nrc) {
        hook.mode = 1;
        hook.diverged = nrc_diverged_flag(wf->nrc);
        hook.stride = nrc_train_stride(wf->nrc);
        hook.frame = wf->d_frame;
        hook.q_in = wf->nrc_q_in;
        hook.q_meta = wf->nrc_q_meta;
        hook.q_count = wf->nrc_q_count();
        hook.q_cap = (int32_t)wf->n;
        hook.rec = wf->nrc_train ? wf->nrc_rec : nullptr;
        hook.rec_count = wf->nrc_rec_count;
        hook.rec_max = wf->nrc_rec_max;
        hook.spread = wf->nrc_spread;
        hook.spread_c = nrc_termination_spread(wf->nrc);
        if (!defer_cache) KRR_CUDA(cudaMemsetAsync(wf->nrc_q_count(), 0, sizeof(int32_t), st));
    }
    {
        ProfScope prof(wf, PS_ROUTE, st);
        k_hit_process<<<wf->grid, wf->block, 0, st>>>(wf->scene, rq, wf->hits, wf->q(cur ^ 1),
                                                      wf->q(Q_MISS), wf->q(Q_HIT_LIGHT), wf->q(Q_SCATTER),
                                                      wf->q(Q_MEDIUM_SAMPLE), wf->medium ? 1 : 0, wf->err(),
                                                      hook, wf->ps, inline_lights, wf->params.nee);
        KRR_CUDA(cudaGetLastError());
    }
    if (wf->nrc && !defer_cache) KRR_TRY(nrc_evaluate_queries(wf, st));
    return KRR_OK;
}

extern "C" int krr_wf_trace_closest(krr_wf *wf, int32_t depth, void *stream) {
    KRR_TRY(ready(wf));
    return closest_stage(wf, depth, as_stream(stream), false);
}

// Shadow rays of bounce `depth` and the closest-hit rays of bounce depth+1
// in one traversal launch (surfaces only: with media the shadow rays need
// transmittance tracking).  The shadow results are resolved right away, as
// traceShadow does; the hits wait in wf->hits for closest_stage(depth + 1).
static int trace_shadow_and_next(krr_wf *wf, int depth, cudaStream_t st) {
    ProfScope prof(wf, PS_SHADOW_NEXT, st);
    Queue sq = wf->q(Q_SHADOW);
    TraceLaunch l = closest_launch(wf, depth + 1);
    l.any_o = sq.base;
    l.any_d = sq.base + sq.cap;
    l.d_any_count = sq.count;
    l.occluded = wf->occluded;
    set_roots(wf, l, sq, 2, true);   // Shadow: plane 2 = Ld | pixel
    KRR_TRY(launch_trace_mixed(&wf->accel, l, st));
    k_shadow_resolve<<<wf->grid, wf->block, 0, st>>>(sq, wf->occluded, wf->ps);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_handle_hit(krr_wf *wf, void *stream) {
    KRR_TRY(ready(wf));
    ProfScope prof(wf, PS_HIT, as_stream(stream));
    k_handle_hit<<<wf->grid, wf->block, 0, as_stream(stream)>>>(wf->scene, wf->q(Q_HIT_LIGHT), wf->ps,
                                                               wf->params.nee);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_handle_miss(krr_wf *wf, void *stream) {
    KRR_TRY(ready(wf));
    if (wf->scene.n_infinite == 0) return KRR_OK;
    ProfScope prof(wf, PS_MISS, as_stream(stream));
    k_handle_miss<<<wf->grid, wf->block, 0, as_stream(stream)>>>(wf->scene, wf->q(Q_MISS), wf->ps,
                                                                wf->params.nee);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

// generateScatterRays; with `to_tracker` the shadow rays of scenes with
// media go to their own queue for k_shadow_split (split_shadows()).
static int scatter_stage(krr_wf *wf, int depth, cudaStream_t st, bool to_tracker) {
    ProfScope prof(wf, PS_SCATTER, st);
    int cur = depth & 1;
    const Queue tracked = to_tracker ? Queue{wf->media_shadow, (int32_t)wf->qcap, wf->media_shadow_count()}
                                     : Queue{};
    KRR_CUDA(cudaMemsetAsync(wf->scatter_class_counts(), 0, 4 * sizeof(int32_t), st));
    k_scatter_classify<<<wf->grid, wf->block, 0, st>>>(wf->scene, wf->q(Q_SCATTER), wf->ps,
                                                      wf->params.rr, wf->scatter_lists,
                                                      wf->scatter_class_counts());
    k_scatter_process<<<wf->grid, wf->block, 0, st>>>(wf->scene, wf->q(Q_SCATTER), wf->scatter_lists,
                                                     wf->scatter_class_counts(), wf->q(cur ^ 1),
                                                     wf->q(Q_SHADOW), tracked, wf->ps, wf->params.nee,
                                                     wf->params.rr, wf->err());
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_generate_scatter_rays(krr_wf *wf, int32_t depth, void *stream) {
    KRR_TRY(ready(wf));
    return scatter_stage(wf, depth, as_stream(stream), false);
}

extern "C" int krr_wf_trace_shadow(krr_wf *wf, void *stream) {
    KRR_TRY(ready(wf));
    cudaStream_t st = as_stream(stream);
    ProfScope prof(wf, PS_SHADOW, st);
    if (wf->medium) return launch_trace_shadow_tr(wf, st);
    Queue sq = wf->q(Q_SHADOW);
    TraceLaunch l{};
    l.ray_o = sq.base;
    l.ray_d = sq.base + sq.cap;
    l.ray_stride = 1;
    l.n = sq.cap;
    l.d_count = sq.count;
    l.occluded = wf->occluded;
    l.counter = wf->accel.d_scratch;
    l.err = wf->accel.d_scratch + 4;
    set_roots(wf, l, sq, 2, false);
    KRR_TRY(launch_trace_any(&wf->accel, l, st));
    k_shadow_resolve<<<wf->grid, wf->block, 0, st>>>(sq, wf->occluded, wf->ps);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_sample_medium_interaction(krr_wf *wf, int32_t depth, void *stream) {
    KRR_TRY(ready(wf));
    if (!wf->medium) return KRR_OK;
    ProfScope prof(wf, PS_MEDIUM_SAMPLE, as_stream(stream));
    return launch_medium_sample(wf, depth, as_stream(stream));
}

extern "C" int krr_wf_sample_medium_scattering(krr_wf *wf, int32_t depth, void *stream) {
    KRR_TRY(ready(wf));
    if (!wf->medium) return KRR_OK;
    return launch_medium_scatter(wf, depth, as_stream(stream));
}

extern "C" int krr_wf_set_launch(krr_wf *wf, int32_t block, int32_t blocks_per_sm, int64_t wave) {
    KRR_CHECK_ARG(wf != nullptr, "NULL argument");
    KRR_CHECK_ARG(block == 64 || block == 128 || block == 256, "block must be 64, 128 or 256 threads");
    KRR_CHECK_ARG(blocks_per_sm >= 1 && blocks_per_sm <= 32, "blocks per SM must be 1..32");
    KRR_CHECK_ARG(wave >= 0, "wave must be >= 0 (0 = every pixel at once)");
    const bool realloc = wave != wf->wave;
    wf->block = block;
    wf->blocks_per_sm = blocks_per_sm;
    wf->wave = wave;
    if (realloc && wf->n) return set_layout(wf, wf->layout);   // queues of the new capacity
    if (wf->n) wf->grid = stage_grid(wf, wf->n);
    return KRR_OK;
}

extern "C" int krr_wf_get_launch(const krr_wf *wf, int32_t *block, int32_t *blocks_per_sm,
                                 int64_t *wave, int64_t *queue_capacity) {
    KRR_CHECK_ARG(wf != nullptr, "NULL argument");
    if (block) *block = wf->block;
    if (blocks_per_sm) *blocks_per_sm = wf->blocks_per_sm;
    if (wave) *wave = wf->wave;
    if (queue_capacity) *queue_capacity = wf->qcap;
    return KRR_OK;
}

// Autotuner of the pass's launch shapes and queue capacity: renders
// `frames` frames (the current cameras, frame indices from 1) with each
// candidate (threads per block 128 / 256 x blocks per SM 4 / 8 / 16 x waves
// of all, half or a quarter of the pixels, the last two only from 2^20
// pixels up), times them with CUDA events on the stream, keeps the fastest
// by median frame time and applies it.  An attached cache does not train
// during the trials.  The frames are the same with every candidate.
extern "C" int krr_wf_autotune(krr_wf *wf, float *d_out, int32_t frames, krr_wf_tuning *out,
                               void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_out && out && frames >= 1, "bad argument");
    cudaStream_t st = as_stream(stream);
    const bool train = wf->nrc_train;
    wf->nrc_train = false;
    const int32_t block0 = wf->block, bps0 = wf->blocks_per_sm;
    const int64_t wave0 = wf->wave;
    std::vector<int64_t> waves{0};
    if (wf->n >= (1 << 20))
        for (int d : {2, 4}) waves.push_back(((wf->n + d - 1) / d + 4095) / 4096 * 4096);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = INFINITY, first = INFINITY;
    int32_t bb = block0, bbps = bps0;
    int64_t bw = wave0;
    int st_code = KRR_OK, n_cand = 0;
    for (int64_t w : waves) {
        for (int32_t b : {256, 128}) {
            for (int32_t bps : {8, 4, 16}) {
                st_code = krr_wf_set_launch(wf, b, bps, w);
                if (st_code != KRR_OK) break;
                std::vector<float> ms;
                for (int f = 0; f <= frames && st_code == KRR_OK; ++f) {   // frame 0 warms up
                    st_code = begin_frame_common(wf, 1 + f, nullptr, nullptr, 0, st);
                    if (st_code != KRR_OK) break;
                    cudaEventRecord(e0, st);
                    st_code = krr_wf_render(wf, d_out, stream);
                    cudaEventRecord(e1, st);
                    cudaEventSynchronize(e1);
                    float t = 0.f;
                    cudaEventElapsedTime(&t, e0, e1);
                    if (f > 0) ms.push_back(t);
                }
                if (st_code != KRR_OK) break;
                std::sort(ms.begin(), ms.end());
                const float med = ms[ms.size() / 2];
                if (n_cand++ == 0) first = med;
                if (med < best) { best = med; bb = b; bbps = bps; bw = w; }
            }
            if (st_code != KRR_OK) break;
        }
        if (st_code != KRR_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    wf->nrc_train = train;
    if (st_code != KRR_OK) {
        krr_wf_set_launch(wf, block0, bps0, wave0);
        return st_code;
    }
    KRR_TRY(krr_wf_set_launch(wf, bb, bbps, bw));
    out->block = bb;
    out->blocks_per_sm = bbps;
    out->wave = bw;
    out->queue_capacity = wf->qcap;
    out->frame_ms = best;
    out->default_frame_ms = first;
    out->candidates = n_cand;
    return KRR_OK;
}

extern "C" int krr_wf_render(krr_wf *wf, float *d_out, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_out != nullptr, "output is NULL");
    cudaStream_t st = as_stream(stream);
    // Without media, the shadow rays of a bounce and the next bounce's rays
    // are traced in one launch; results and their order of use are those of
    // the stage-by-stage loop (integrator.cpp:223-254).
    // With a cache attached, the paths that stop at it (at any depth) are
    // evaluated in one launch at the end of the sample: a stopped path gets no
    // other radiance afterwards, so each pixel's sum is the same, in the same
    // order, as with one evaluation per depth.
    // The pixels go through the bounces in waves of the queue capacity (all
    // at once by default); a pixel's path touches only its own state, so the
    // waves give the same frame as one pass over all pixels.
    // In a pass of several scenes where only some have media, the shadow
    // rays of the scenes without media are traced with the next bounce's
    // rays too; those of the scenes with media go to the tracker
    // (split_shadows()).
    const bool split = split_shadows(wf) && wf->media_shadow;
    const bool fuse = (wf->params.nee && !wf->medium) || split;
    for (int s = 0; s < wf->params.spp; ++s) {
        for (int64_t p0 = 0; p0 < wf->n; p0 += wf->qcap) {
            KRR_TRY(krr_wf_reset_queues(wf, -1, stream));
            KRR_TRY(camera_rays(wf, p0, std::min(wf->qcap, wf->n - p0), st));
            if (wf->nrc) KRR_CUDA(cudaMemsetAsync(wf->nrc_q_count(), 0, sizeof(int32_t), st));
            bool traced = false;
            for (int depth = 0;; ++depth) {
                KRR_TRY(krr_wf_reset_queues(wf, depth, stream));
                KRR_TRY(closest_stage(wf, depth, st, traced, true));
                if (wf->medium) {
                    KRR_TRY(krr_wf_sample_medium_interaction(wf, depth, stream));
                    KRR_TRY(krr_wf_handle_hit(wf, stream));
                    KRR_TRY(krr_wf_handle_miss(wf, stream));
                }
                if (depth == loop_depth(wf)) break;
                if (split) {
                    KRR_CUDA(cudaMemsetAsync(wf->shadow_tracked_count(), 0, sizeof(int32_t), st));
                    KRR_CUDA(cudaMemsetAsync(wf->media_shadow_count(), 0, sizeof(int32_t), st));
                }
                if (wf->medium) KRR_TRY(launch_medium_scatter(wf, depth, st, split));
                KRR_TRY(scatter_stage(wf, depth, st, split));
                if (split) {
                    ProfScope prof(wf, PS_SHADOW, st);
                    KRR_TRY(launch_shadow_split(wf, st, true));
                    KRR_TRY(launch_shadow_tracker(wf, st));
                }
                traced = fuse;
                if (fuse) KRR_TRY(trace_shadow_and_next(wf, depth, st));
                else if (wf->params.nee) KRR_TRY(krr_wf_trace_shadow(wf, stream));
            }
            if (wf->nrc) KRR_TRY(nrc_evaluate_queries(wf, st));
        }
        if (wf->nrc && wf->nrc_train) KRR_TRY(nrc_train_frame(wf, st));
        ProfScope prof(wf, PS_RESOLVE, st);
        k_accumulate<<<wf->grid, wf->block, 0, st>>>(wf->ps, wf->n,
                                                     wf->params.independent_samples && s + 1 < wf->params.spp);
        KRR_CUDA(cudaGetLastError());
    }
    ProfScope prof(wf, PS_RESOLVE, st);
    k_resolve<<<wf->grid, wf->block, 0, st>>>(wf->ps, reinterpret_cast<float4 *>(d_out), wf->d_views,
                                              wf->d_frame, wf->n, (float)wf->params.spp,
                                              wf->params.enable_clamp, wf->params.clamp_max);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_set_media_order(krr_wf *wf, int32_t order) {
    KRR_CHECK_ARG(wf && (order == 0 || order == 1), "order must be 0 or 1");
    wf->media_order = order;
    return KRR_OK;
}

extern "C" int krr_wf_set_camera_order(krr_wf *wf, int32_t order) {
    KRR_CHECK_ARG(wf && (order == 0 || order == 1), "order must be 0 or 1");
    wf->camera_order = order;
    return KRR_OK;
}

extern "C" int krr_wf_set_profiling(krr_wf *wf, int32_t on) {
    KRR_CHECK_ARG(wf && (on == 0 || on == 1), "profiling must be 0 or 1");
    wf->profiling = on;
    return KRR_OK;
}

extern "C" int krr_wf_profile_read(krr_wf *wf, krr_stage_time *out, int32_t cap, int32_t *n_out) {
    KRR_CHECK_ARG(wf && n_out && cap >= 0 && (cap == 0 || out), "NULL argument");
    double ms[PS_COUNT] = {};
    int64_t calls[PS_COUNT] = {};
    int status = KRR_OK;
    for (const auto &r : wf->prof) {
        float t = 0.f;
        cudaError_t e = cudaEventSynchronize(r.e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.e0, r.e1);
        if (e != cudaSuccess && status == KRR_OK)
            status = cuda_status(e, "cudaEventElapsedTime", __FILE__, __LINE__);
        ms[r.stage] += t;
        ++calls[r.stage];
        wf->prof_pool.push_back(r.e0);
        wf->prof_pool.push_back(r.e1);
    }
    wf->prof.clear();
    int32_t n = 0;
    for (int k = 0; k < PS_COUNT; ++k) {
        if (!calls[k]) continue;
        if (n < cap) {
            krr_stage_time &o = out[n];
            std::memset(o.name, 0, sizeof(o.name));
            std::strncpy(o.name, kProfNames[k], sizeof(o.name) - 1);
            o.calls = calls[k];
            o.ms = ms[k];
        }
        ++n;
    }
    *n_out = n;
    return status;
}

extern "C" int krr_wf_set_megakernel_reorder(krr_wf *wf, int32_t reorder) {
    KRR_CHECK_ARG(wf && (reorder == 0 || reorder == 1), "reorder must be 0 or 1");
    wf->mk_reorder = reorder;
    return KRR_OK;
}

extern "C" int krr_wf_render_megakernel(krr_wf *wf, float *d_out, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_out != nullptr, "output is NULL");
    KRR_CHECK_ARG(!wf->medium, "the megakernel pass traces surfaces only; the scene has media");
    KRR_CHECK_ARG(wf->n_parts == 1, "the megakernel pass takes one scene");
    KRR_CHECK_ARG(wf->levels == 1, "the megakernel pass traces the flattened structure");
    KRR_CHECK_ARG(!wf->nrc, "the megakernel pass has no cache hooks; detach the cache first");
    cudaStream_t st = as_stream(stream);
    static int grid[2][2] = {{0, 0}, {0, 0}};
    const int fmt = wf->accel.node_format, sorted = wf->mk_reorder;
    if (!grid[sorted][fmt]) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const void *fn = sorted ? (fmt == 1 ? (const void *)k_megakernel_sorted<1> : (const void *)k_megakernel_sorted<0>)
                                : (fmt == 1 ? (const void *)k_megakernel<1> : (const void *)k_megakernel<0>);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 128, 0);
        grid[sorted][fmt] = std::max(1, sms) * std::max(1, per_sm);
    }
    const int blocks = (int)std::min<int64_t>(grid[sorted][fmt], (wf->n + 127) / 128);
    WfConst c = wf->consts();
    float4 *out = reinterpret_cast<float4 *>(d_out);
    int *terr = wf->accel.d_scratch + 4;
    const int ind = wf->params.independent_samples;
#define KRR_MK_LAUNCH(K) K<<<blocks, 128, 0, st>>>(wf->scene, wf->accel.d_nodes, wf->accel.d_tris, wf->d_views, \
                                                   wf->d_frame, wf->ps, c, ind, wf->n, out, wf->err(), terr)
    if (sorted) {
        if (fmt == 1) KRR_MK_LAUNCH(k_megakernel_sorted<1>);
        else KRR_MK_LAUNCH(k_megakernel_sorted<0>);
    } else {
        if (fmt == 1) KRR_MK_LAUNCH(k_megakernel<1>);
        else KRR_MK_LAUNCH(k_megakernel<0>);
    }
#undef KRR_MK_LAUNCH
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_wf_queue_size(krr_wf *wf, int32_t queue, int32_t *out, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(queue >= 0 && queue < Q_COUNT && out, "bad queue");
    KRR_CUDA(cudaMemcpyAsync(out, wf->d_counts + queue, sizeof(int32_t), cudaMemcpyDeviceToHost,
                             as_stream(stream)));
    KRR_CUDA(cudaStreamSynchronize(as_stream(stream)));
    return KRR_OK;
}

extern "C" int krr_wf_pixel_radiance(krr_wf *wf, const float **d_L) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_L != nullptr, "NULL argument");
    *d_L = reinterpret_cast<const float *>(wf->ps.L);
    return KRR_OK;
}

extern "C" int krr_wf_read_radiance(krr_wf *wf, float *d_dst, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_dst != nullptr, "NULL argument");
    KRR_CUDA(cudaMemcpyAsync(d_dst, wf->ps.L, wf->n * sizeof(float4), cudaMemcpyDeviceToDevice,
                             as_stream(stream)));
    return KRR_OK;
}

extern "C" int krr_wf_ray_queue(krr_wf *wf, int32_t depth, const float **d_origin_tmin,
                                const float **d_dir_tmax, const float **d_pu_pixel,
                                int32_t *capacity) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_origin_tmin && d_dir_tmax, "NULL argument");
    const float4 *b = wf->qbuf[depth & 1];
    *d_origin_tmin = reinterpret_cast<const float *>(b);
    *d_dir_tmax = reinterpret_cast<const float *>(b + wf->qcap);
    if (d_pu_pixel) *d_pu_pixel = reinterpret_cast<const float *>(b + 5 * wf->qcap);
    if (capacity) *capacity = (int32_t)wf->qcap;
    return KRR_OK;
}

extern "C" int krr_wf_queue_view(krr_wf *wf, int32_t queue, const float **d_base, int32_t *channels,
                                 int32_t *capacity) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(queue >= 0 && queue < Q_COUNT && d_base, "bad queue");
    *d_base = reinterpret_cast<const float *>(wf->qbuf[queue]);
    if (channels) *channels = kChannels[queue];
    if (capacity) *capacity = (int32_t)wf->qcap;
    return KRR_OK;
}

extern "C" int krr_wf_device_errors(krr_wf *wf, uint32_t *out, void *stream) {
    KRR_CHECK_ARG(wf && out, "NULL argument");
    uint32_t flags[2] = {0, 0};
    cudaStream_t st = as_stream(stream);
    if (wf->d_counts) {
        KRR_CUDA(cudaMemcpyAsync(&flags[0], wf->d_counts + 8, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        KRR_CUDA(cudaMemsetAsync(wf->d_counts + 8, 0, sizeof(uint32_t), st));
    }
    if (wf->accel.d_scratch) {
        KRR_CUDA(cudaMemcpyAsync(&flags[1], wf->accel.d_scratch + 4, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        KRR_CUDA(cudaMemsetAsync(wf->accel.d_scratch + 4, 0, sizeof(uint32_t), st));
    }
    uint32_t cache_flags = 0;
    if (wf->nrc) {   // the attached cache's bounded tensor-core waits
        KRR_CUDA(cudaMemcpyAsync(&cache_flags, nrc_error_flags(wf->nrc), sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, st));
        KRR_CUDA(cudaMemsetAsync(nrc_error_flags(wf->nrc), 0, sizeof(uint32_t), st));
    }
    KRR_CUDA(cudaStreamSynchronize(st));
    *out = flags[0] | flags[1] | cache_flags;
    return KRR_OK;
}

extern "C" int krr_wf_set_loop_limits(krr_wf *wf, int32_t max_null_collisions,
                                      int32_t max_interface_crossings) {
    KRR_CHECK_ARG(wf != nullptr, "NULL argument");
    KRR_CHECK_ARG(max_null_collisions >= 1 && max_interface_crossings >= 1,
                  "loop limits must be at least 1");
    wf->max_null_collisions = max_null_collisions;
    wf->max_interface_crossings = max_interface_crossings;
    wf->scene.max_null_collisions = max_null_collisions;
    wf->scene.max_interface_crossings = max_interface_crossings;
    return KRR_OK;
}

extern "C" int krr_wf_accel(krr_wf *wf, const krr_accel **out) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(out != nullptr, "NULL argument");
    *out = &wf->accel;
    return KRR_OK;
}

// A whole frame (view table upload, beginFrame, render) captured into a CUDA
// graph; replays read the per-frame constants from pinned host memory.
extern "C" int krr_wf_capture_frame(krr_wf *wf, float *d_out, void *stream) {
    KRR_TRY(ready(wf));
    KRR_CHECK_ARG(d_out != nullptr, "output is NULL");
    cudaStream_t st = as_stream(stream);
    KRR_CHECK_ARG(st != nullptr, "capture needs a non-default stream");
    if (wf->graph) { cudaGraphExecDestroy(wf->graph); wf->graph = nullptr; }
    for (int i = 0; i < wf->n_views; ++i) wf->h_views[i] = wf->layout[i];
    KRR_CUDA(cudaStreamSynchronize(st));
    KRR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int status = KRR_OK;
    cudaError_t e = cudaMemcpyAsync(wf->d_views, wf->h_views, wf->n_views * sizeof(DevView),
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(wf->d_frame, wf->h_frame, sizeof(FrameConst), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) status = cuda_status(e, "capture copies", __FILE__, __LINE__);
    if (status == KRR_OK) status = launch_begin_frame(wf, st);
    if (status == KRR_OK) status = krr_wf_render(wf, d_out, stream);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st, &g);
    if (status != KRR_OK) { if (g) cudaGraphDestroy(g); return status; }
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(&wf->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    return KRR_OK;
}

extern "C" int krr_wf_launch_frame(krr_wf *wf, int64_t frame_index, const krr_view *views,
                                   int32_t n_views, void *stream) {
    KRR_TRY(ready(wf));
    if (!wf->graph) return fail(KRR_ERR_NOT_READY, "no captured frame: call krr_wf_capture_frame");
    cudaStream_t st = as_stream(stream);
    // the previous replay must have read the pinned constants before they change
    KRR_CUDA(cudaStreamSynchronize(st));
    KRR_TRY(fill_frame(wf, frame_index, nullptr, views, n_views, wf->h_views, wf->h_frame));
    KRR_CUDA(cudaGraphLaunch(wf->graph, st));
    return KRR_OK;
}

// Several passes (different scenes, each with its batched views) rendered
// as one CUDA graph: the graph forks one branch per pass, each branch runs
// that pass's whole frame, and the branches join, so the passes' launches
// overlap on the GPU and the tail of one pass's bounces is filled by the
// others.
struct krr_wf_group {
    std::vector<krr_wf *> passes;
    std::vector<float *> outs;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;    // fork + one join per pass
    cudaGraphExec_t exec = nullptr;
};

extern "C" int krr_wf_group_create(krr_wf *const *passes, float *const *d_outs, int32_t n,
                                   krr_wf_group **out) {
    KRR_CHECK_ARG(passes && d_outs && out && n >= 1 && n <= 64, "bad group");
    for (int i = 0; i < n; ++i) {
        KRR_CHECK_ARG(passes[i] && d_outs[i], "NULL pass or output");
        KRR_TRY(ready(passes[i]));
        for (int j = 0; j < i; ++j) KRR_CHECK_ARG(passes[j] != passes[i], "a pass appears twice");
    }
    krr_wf_group *g = new krr_wf_group();
    g->passes.assign(passes, passes + n);
    g->outs.assign(d_outs, d_outs + n);
    int status = KRR_OK;
    for (int i = 0; i < n && status == KRR_OK; ++i) {
        cudaStream_t s = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) status = cuda_status(e, "cudaStreamCreate", __FILE__, __LINE__);
        else g->streams.push_back(s);
    }
    for (int i = 0; i <= n && status == KRR_OK; ++i) {
        cudaEvent_t ev = nullptr;
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) status = cuda_status(e, "cudaEventCreate", __FILE__, __LINE__);
        else g->events.push_back(ev);
    }
    if (status != KRR_OK) {
        krr_wf_group_destroy(g);
        return status;
    }
    *out = g;
    return KRR_OK;
}

extern "C" int krr_wf_group_destroy(krr_wf_group *g) {
    if (!g) return KRR_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    for (cudaStream_t s : g->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    for (cudaEvent_t e : g->events) cudaEventDestroy(e);
    delete g;
    return KRR_OK;
}

// Captures the group's frame on `stream` (non-default).  Each pass must have
// rendered one ordinary frame first (lazily sized buffers exist).
extern "C" int krr_wf_group_capture(krr_wf_group *g, void *stream) {
    KRR_CHECK_ARG(g != nullptr, "NULL group");
    cudaStream_t st = as_stream(stream);
    KRR_CHECK_ARG(st != nullptr, "capture needs a non-default stream");
    if (g->exec) { cudaGraphExecDestroy(g->exec); g->exec = nullptr; }
    for (krr_wf *wf : g->passes)
        for (int i = 0; i < wf->n_views; ++i) wf->h_views[i] = wf->layout[i];
    KRR_CUDA(cudaStreamSynchronize(st));
    KRR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int status = KRR_OK;
    cudaError_t e = cudaEventRecord(g->events[0], st);
    const int n = (int)g->passes.size();
    for (int i = 0; i < n && e == cudaSuccess && status == KRR_OK; ++i) {
        krr_wf *wf = g->passes[i];
        cudaStream_t si = g->streams[i];
        e = cudaStreamWaitEvent(si, g->events[0], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(wf->d_views, wf->h_views, wf->n_views * sizeof(DevView),
                                cudaMemcpyHostToDevice, si);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(wf->d_frame, wf->h_frame, sizeof(FrameConst), cudaMemcpyHostToDevice, si);
        if (e != cudaSuccess) break;
        status = launch_begin_frame(wf, si);
        if (status == KRR_OK) status = krr_wf_render(wf, g->outs[i], si);
        if (status == KRR_OK) e = cudaEventRecord(g->events[1 + i], si);
        if (status == KRR_OK && e == cudaSuccess) e = cudaStreamWaitEvent(st, g->events[1 + i], 0);
    }
    if (e != cudaSuccess && status == KRR_OK) status = cuda_status(e, "group capture", __FILE__, __LINE__);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(st, &graph);
    if (status != KRR_OK) { if (graph) cudaGraphDestroy(graph); return status; }
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    return KRR_OK;
}

// One frame of every pass of the group: same cameras, frame `frame_index`.
extern "C" int krr_wf_group_launch(krr_wf_group *g, int64_t frame_index, void *stream) {
    KRR_CHECK_ARG(g != nullptr, "NULL group");
    if (!g->exec) return fail(KRR_ERR_NOT_READY, "no captured group frame: call krr_wf_group_capture");
    cudaStream_t st = as_stream(stream);
    KRR_CUDA(cudaStreamSynchronize(st));
    for (krr_wf *wf : g->passes)
        KRR_TRY(fill_frame(wf, frame_index, nullptr, nullptr, 0, wf->h_views, wf->h_frame));
    KRR_CUDA(cudaGraphLaunch(g->exec, st));
    return KRR_OK;
}

namespace krr {
// The permutation of a tracking queue's items by work class (media work
// order, above), in the scatter-list buffer (free during the media stages).
static int work_order(krr_wf *wf, const Queue &q, int items, cudaStream_t st, const int32_t **order) {
    *order = nullptr;
    if (!wf->media_order) return KRR_OK;
    uint8_t *classes = reinterpret_cast<uint8_t *>(wf->scatter_lists + wf->qcap);
    int32_t *counts = wf->work_counts;
    KRR_CUDA(cudaMemsetAsync(counts, 0, 2 * kWorkClasses * sizeof(int32_t), st));
    if (items == 0) k_work_classes<0><<<wf->grid, wf->block, 0, st>>>(wf->scene, q, classes, counts);
    else k_work_classes<1><<<wf->grid, wf->block, 0, st>>>(wf->scene, q, classes, counts);
    k_work_order<<<wf->grid, wf->block, 0, st>>>(q, classes, counts, wf->scatter_lists);
    KRR_CUDA(cudaGetLastError());
    *order = wf->scatter_lists;
    return KRR_OK;
}

int launch_medium_sample(krr_wf *wf, int depth, cudaStream_t st) {
    const int32_t *order = nullptr;
    KRR_TRY(work_order(wf, wf->q(Q_MEDIUM_SAMPLE), 0, st, &order));
    k_medium_sample<<<wf->grid, wf->block, 0, st>>>(wf->scene, wf->q(Q_MEDIUM_SAMPLE),
                                                    wf->q((depth & 1) ^ 1), wf->q(Q_MISS),
                                                    wf->q(Q_HIT_LIGHT), wf->q(Q_SCATTER),
                                                    wf->q(Q_MEDIUM_SCATTER), wf->ps, order, wf->err());
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}
// The tracked shadow rays are staged in the medium-sample queue's storage
// (consumed earlier in the bounce) with their own counter.
static Queue tracked_queue(krr_wf *wf) {
    return Queue{wf->qbuf[Q_MEDIUM_SAMPLE], (int32_t)wf->qcap, wf->shadow_tracked_count()};
}

// A pass of several scenes of which some have media and some do not: the
// shadow rays of the scenes without media are traced with the next bounce's
// rays in one launch (as in a pass without media); those of the scenes with
// media go through k_shadow_split from a queue of their own (surface
// vertices) or straight to the tracker (medium vertices, which start inside
// a medium).  A pixel's shadow rays all go one way, so each pixel gets the
// same terms in the same order.
bool split_shadows(const krr_wf *wf) {
    if (!wf->medium || !wf->params.nee || wf->n_parts <= 1) return false;
    bool with = false, without = false;
    for (const DevScenePart &P : wf->parts) (P.has_media ? with : without) = true;
    return with && without;
}

// The queue of media-scene shadow rays for split routing, allocated with the
// queues once the scenes and the parameters call for it (never inside a
// frame, so that frames can be captured).
int ensure_split_buffers(krr_wf *wf) {
    if (wf->media_shadow || wf->qcap <= 0 || !split_shadows(wf)) return KRR_OK;
    KRR_CUDA(cudaMalloc(&wf->media_shadow, (size_t)kShadowCh * wf->qcap * sizeof(float4)));
    return KRR_OK;
}

int launch_medium_scatter(krr_wf *wf, int depth, cudaStream_t st, bool to_tracker) {
    ProfScope prof(wf, PS_MEDIUM_SCATTER, st);
    k_medium_scatter<<<wf->grid, wf->block, 0, st>>>(wf->scene, wf->q(Q_MEDIUM_SCATTER),
                                                     wf->q((depth & 1) ^ 1), wf->q(Q_SHADOW),
                                                     to_tracker ? tracked_queue(wf) : Queue{}, wf->ps,
                                                     wf->params.nee, wf->err());
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}
// traceShadow with media (device.cu:102-128): unoccluded rays outside the
// media are finished by k_shadow_split; the rest are staged in the
// medium-sample queue's storage (consumed earlier in the bounce) with their
// own counter and ratio-tracked by k_shadow_tr.
int launch_trace_shadow_tr(krr_wf *wf, cudaStream_t st) {
    static_assert(kMediumSampleCh >= kShadowCh, "tracked shadow rays need five planes");
    KRR_CUDA(cudaMemsetAsync(wf->shadow_tracked_count(), 0, sizeof(int32_t), st));
    KRR_TRY(launch_shadow_split(wf, st, false));
    return launch_shadow_tracker(wf, st);
}

// k_shadow_split over the shadow queue, or over the media-scene shadow rays
// of split routing; the rays it does not finish are appended to the
// tracker's queue.
int launch_shadow_split(krr_wf *wf, cudaStream_t st, bool media_candidates) {
    const Queue tracked = tracked_queue(wf);
    const Queue from = media_candidates ? Queue{wf->media_shadow, (int32_t)wf->qcap, wf->media_shadow_count()}
                                        : wf->q(Q_SHADOW);
    int *terr = wf->accel.d_scratch + 4;
    const InstancedView iv = wf->accel.levels == 2 ? instanced_view(&wf->accel) : InstancedView{};
#define KRR_SHADOW_SPLIT(F, LV)                                                                        \
    k_shadow_split<F, LV><<<wf->grid, wf->block, 0, st>>>(wf->scene, wf->accel.d_nodes, wf->accel.d_tris, iv, \
                                                          from, tracked, wf->ps, wf->err(), terr)
    const bool two = wf->accel.levels == 2, f1 = wf->accel.node_format == 1;
    if (two) { if (f1) KRR_SHADOW_SPLIT(1, 2); else KRR_SHADOW_SPLIT(0, 2); }
    else { if (f1) KRR_SHADOW_SPLIT(1, 1); else KRR_SHADOW_SPLIT(0, 1); }
#undef KRR_SHADOW_SPLIT
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

// Ratio tracking of the shadow rays in the tracker's queue.
int launch_shadow_tracker(krr_wf *wf, cudaStream_t st) {
    const Queue tracked = tracked_queue(wf);
    int *terr = wf->accel.d_scratch + 4;
    const InstancedView iv = wf->accel.levels == 2 ? instanced_view(&wf->accel) : InstancedView{};
    const int32_t *order = nullptr;
    KRR_TRY(work_order(wf, tracked, 1, st, &order));
#define KRR_SHADOW_TR(F, LV)                                                                           \
    k_shadow_tr<F, LV><<<wf->grid, wf->block, 0, st>>>(wf->scene, wf->accel.d_nodes, wf->accel.d_tris, iv,    \
                                                       tracked, wf->ps, order, wf->err(), terr)
    const bool two = wf->accel.levels == 2, f1 = wf->accel.node_format == 1;
    if (two) { if (f1) KRR_SHADOW_TR(1, 2); else KRR_SHADOW_TR(0, 2); }
    else { if (f1) KRR_SHADOW_TR(1, 1); else KRR_SHADOW_TR(0, 1); }
#undef KRR_SHADOW_TR
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}
}  // namespace krr
