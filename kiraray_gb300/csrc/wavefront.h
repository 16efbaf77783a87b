// Device-side data of the wavefront path tracer: scene, queues, pixel state.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kmath.cuh"

namespace krr {

struct DevMesh {
    const float *pos;       // float3, object space
    const float *nrm;       // float3
    const float *uv;        // float2 or nullptr
    const uint32_t *idx;    // uint3
    int32_t material;       // -1 = null material
    int32_t medium_inside, medium_outside;
    int32_t pad;
};

struct DevInstance {
    float xf[12];           // object -> world, row-major 3x4
    float nxf[9];           // inverse-transpose of the linear part (normals)
    int32_t mesh;
    uint32_t prim_offset;   // global id of the instance's first triangle
    int32_t light_offset;   // light-list index of its first triangle light, -1 if none
    float le[3];            // emission divided by le_scale (src/core/mesh.cpp:41-49)
    float le_scale;
};

struct DevMaterial {
    int32_t type;
    float diffuse[3];
    float spec_alpha;       // 1 - roughness, as stored by the scene importer
    float spec_trans;
    float eta;
    float anisotropic;
};

struct DevLight {
    int32_t kind;           // 0 = triangle area light, 1 = infinite light
    int32_t index;          // instance (area) or infinite-light index
    uint32_t prim;          // local triangle (area)
    int32_t pad;
};

struct DevInfinite {
    float tint[3];
    float scale;
    float rot[9];           // light -> world
    const float4 *image;    // [h][w] or nullptr
    int32_t w, h;
    float scene_radius;
    int32_t pad;
};

struct DevMedium {
    // half octets [nz][ny][nx][8]: voxel (x, y, z) and its seven neighbours
    // at +x, +y, +z (0 past the grid's last column, row or slice), so that a
    // trilinear lookup reads its eight corners with one 16-byte load;
    // nullptr = homogeneous
    const uint16_t *density;
    int32_t nx, ny, nz;
    float lo[3], hi[3];
    float sigma_t[3];
    float albedo[3];
    float g;
    float scale;
    int32_t mres[3];
    const float *majorant;     // [mz][my][mx]
    float idx_scale[3];        // n / (hi - lo) per axis: world to voxel index
};

// One scene of a pass that traces several scenes in one wavefront
// (krr_wf_set_scenes): its lights and infinite lights are ranges of the
// pass's lists; its meshes, instances, materials and media are ranges of
// the pass's arrays with the indices relocated; its triangles are a range
// of the global ids and its BVH a root of the pass's node array.
struct DevScenePart {
    int32_t light_begin, n_lights;     // light list [begin, begin + n): mesh lights, then infinite
    int32_t inf_begin, n_infinite;     // infinite lights
    float cache_offset[3];             // added to positions fed to the radiance cache
    int32_t has_media;                 // the scene's meshes bound a medium
    int32_t max_depth;                 // the scene's path depth (the pass's, or its own)
    int32_t pad;
};

constexpr int kMaxNullCollisions = 1 << 20;   // default bound of the tracking loops
constexpr int kMaxInterfaceCrossings = 64;    // default bound of the shadow segments

struct DevScene {
    const DevMesh *meshes;
    const DevInstance *instances;
    const DevMaterial *materials;
    const DevLight *lights;
    int32_t n_lights;
    const uint32_t *tri_instance;
    const DevInfinite *infinite;
    int32_t n_infinite;
    const DevMedium *media;
    int32_t n_media;
    // bounds of the tracking loops (krr_wf_set_loop_limits): null collisions
    // per majorant walk and interface crossings per shadow ray; running out
    // raises kErrLoopLimit and ends the walk
    int32_t max_null_collisions;
    int32_t max_interface_crossings;
    // scene parts (one for a single scene); pixel_part[pixel] picks the part
    // of a pixel's view, nullptr with a single part
    const DevScenePart *parts;
    const uint8_t *pixel_part;
    const uint32_t *part_roots;   // BVH root of each part (nullptr: one part, root 0)
    int32_t n_parts;
};

// BVH root node of a pixel's scene.
__device__ __forceinline__ uint32_t root_of(const DevScene &s, uint32_t pixel) {
    return s.part_roots ? s.part_roots[s.pixel_part[pixel]] : 0u;
}

__device__ __forceinline__ const DevScenePart &part_of(const DevScene &s, uint32_t pixel) {
    return s.parts[s.pixel_part ? s.pixel_part[pixel] : 0];
}

// A queue: `channels` float4 planes of `cap` items and an item counter.
struct Queue {
    float4 *base;
    int32_t cap;
    int32_t *count;
    KRR_HD float4 &at(int ch, int i) const { return base[(size_t)ch * cap + i]; }
};

// Channel layouts (x,y,z | w):
//  Ray / Miss:   0 o|tmin 1 d|tmax 2 ctx.p|medium 3 ctx.n|bsdfType 4 thp|depth
//                5 pu|pixel 6 pl|time
//  HitLight:     0 p|light 1 n|u 2 wo|v 3 ctx.p|bsdfType 4 ctx.n|depth 5 thp|pixel
//                6 pu|- 7 pl|-
//  Shadow:       0 o|tmin 1 d|tmax 2 Ld|pixel 3 pu|medium 4 pl|time
//  Scatter:      0 p|material 1 wo|depth 2 n|pixel 3 tangent|mesh 4 bitangent|u
//                5 thp|v 6 pu|time 7 medium|-|-|-
//  MediumSample: Ray channels 0-6, 7 hit (t, b1, b2, prim) with t = tMax
//  MediumScatter:0 p|medium 1 wo|depth 2 thp|pixel 3 pu|time
constexpr int kRayCh = 7, kMissCh = 7, kHitLightCh = 8, kShadowCh = 5, kScatterCh = 8,
              kMediumSampleCh = 8, kMediumScatterCh = 4;

struct PixelState {
    float4 *L;            // radiance xyz | lambda[0]
    float4 *pixel;        // accumulated RGB
    ulonglong2 *rng;      // PCG state, inc
};

struct WfConst {
    int32_t width, height;
    int32_t nee, max_depth, enable_medium, enable_clamp, spp;
    float rr, clamp_max;
};

}  // namespace krr
