// Compressed 8-wide BVH: layout shared by the builder and the traversal.
//
// Node (80 bytes = 5 x 16 B, one 16-byte aligned record per node):
//   q0: origin p.xyz (float) | word: ex | ey<<8 | ez<<16 | imask<<24
//       (e* = biased float exponent of the per-axis quantisation step)
//   q1: child_base | tri_base | meta[0..3] | meta[4..7]
//   q2: qlo_x[0..7] | qlo_y[0..7]      (8-bit quantised child bounds)
//   q3: qlo_z[0..7] | qhi_x[0..7]
//   q4: qhi_y[0..7] | qhi_z[0..7]
// meta byte per child slot: 0 = empty; otherwise (unary count << 5) | bit,
// where an internal child in slot s has count 1 and bit 24 + s, and a leaf
// has count 1..3 (unary 001/011/111) and bit = its first triangle's offset
// (0..23).  A hit child contributes (m >> 5) << (m & 31) to a 32-bit hit mask:
// triangles in bits 0..23, internal children in bits 24..31 (the traversal
// XORs the slot of internal children with the ray octant).
// Internal children are stored contiguously from child_base in slot order;
// the leaf triangles of all children contiguously from tri_base.
// Slot s holds the child that is nearest for rays whose direction octant is
// s (bit i set = negative along axis i), so visiting positions s ^ octant in
// increasing order is an approximate front-to-back order.
//
// Float node format (224 bytes = 14 x 16 B), the same tree without
// quantisation: q0..q1 lo_x[0..7], q2..q3 hi_x, q4..q5 lo_y, q6..q7 hi_y,
// q8..q9 lo_z, q10..q11 hi_z (empty slots: lo = +inf, hi = -inf),
// q12: child_base | tri_base | meta[0..3] | meta[4..7], q13: imask | 0 | 0 | 0.
// It spends 2.8x the node bytes to drop the per-plane byte extraction.
//
// Triangle (48 bytes, leaf order): v0.xyz | global id, v1.xyz | any-hit mask,
// v2.xyz | unused.
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include <stdint.h>

#include "internal.h"

namespace krr {
// One instance of a two-level structure, as the traversal reads it.
struct TraceInst {
    float inv[12];          // world -> object, row-major 3x4
    uint32_t blas_root;     // root node of the instance's geometry tree
    uint32_t id_delta;      // global triangle id = geometry-tree id + id_delta
    uint32_t mask;          // 0: any-hit rays pass through (null material)
    uint32_t pad;
};
}  // namespace krr

struct krr_accel {
    int64_t n_tris = 0;
    int64_t n_nodes = 0;
    int32_t max_depth = 0;
    double build_ms = 0.0;
    float4 *d_nodes = nullptr;   // 5 per node
    float4 *d_tris = nullptr;    // 3 per triangle
    uint32_t *d_leaf_of_prim = nullptr;  // global id -> leaf-order slot
    int *d_scratch = nullptr;    // 64 B: ints 0-1 ray counter, 4 error flags, 8-9 second counter
    float scene_lo[3] = {0, 0, 0}, scene_hi[3] = {0, 0, 0};
    int refill_below = 20;       // traversal tuning (krr_accel_set_tuning)
    int postpone_pct = 0;
    int stack_limit = 48;        // krr_accel_set_stack_limit (kTraversalStack by default)
    int node_format = 0;         // 0 compressed (80 B), 1 float (224 B)
    int max_leaf = 1;            // triangles per leaf child (1..3)
    int full_leaf = 1;           // triangles per leaf child of a full node (max_leaf..3)
    int builder = 0;             // binary tree: 0 radix tree, 1 PLOC, 2 radix tree on cubic cells
    int collapse = 0;            // wide nodes: 0 greedy, 1 cost-optimal
    int treelets = 0;            // treelet restructuring passes applied to the binary tree
    // host-buffer entry point (krr_accel_trace_closest_host): device staging
    // for rays (2 float4 each) and hits, grown on demand, and a second stream
    // with two events, kept across calls so that a call allocates nothing
    // refit (krr_accel_refit): first node of each tree level (level L holds
    // nodes [level_first[L-1], level_first[L])) and the refitted node bounds
    std::vector<int32_t> level_first;
    // several BVHs in one node array (accel_build_parts): the root node of
    // each part; rays pick their part's root.  Empty with one part (root 0).
    std::vector<uint32_t> roots;
    uint32_t *d_roots = nullptr;
    std::vector<float> part_bounds;    // per part: lo.xyz, hi.xyz (accel_build_parts)
    // two-level structure (accel_build_instanced): levels == 2, the instance
    // level and the geometry level as structures of their own, the instance
    // records on the device and their inputs on the host
    int levels = 1;
    krr_accel *tlas = nullptr;
    krr_accel *blas = nullptr;
    krr::TraceInst *d_inst = nullptr;
    std::vector<krr::TraceInst> h_inst;
    std::vector<int64_t> geom_begin;     // first triangle of each geometry (+ total)
    std::vector<int32_t> inst_geom;      // geometry of each instance
    std::vector<float> inst_xf;          // object -> world, 12 per instance
    std::vector<uint32_t> inst_mask;
    std::vector<int64_t> inst_first;     // global id of each instance's first triangle
    int64_t inst_triangles = 0;
    float4 *d_node_bounds = nullptr;   // 2 per node: lo, hi
    float4 *stage_rays = nullptr;
    float4 *stage_hits = nullptr;
    int64_t stage_cap = 0;
    cudaStream_t stage_aux = nullptr;
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
};

namespace krr {

constexpr int kTraversalStack = 48;
// best-hit marker of a ray whose traversal the stack limit cut off
constexpr uint32_t kCutRay = KRR_MISS - 1u;
constexpr int kNodeQuads[2] = {5, 14};   // float4 per node, by node format
// Process-wide node format used by builds (krr_set_bvh_node_format).
int default_node_format();
int default_max_leaf();   // krr_set_bvh_max_leaf
int default_full_leaf();  // krr_set_bvh_full_node_leaf
int default_builder();    // krr_set_bvh_builder
constexpr int kTraceThreads = 128;

// Build from device world-space vertices (float3 x 3 per triangle).
int accel_build(krr_accel *a, const float *d_vertices, int64_t n_tris, cudaStream_t stream);
// New positions for the same triangles (same count and order): boxes refitted
// bottom-up over the existing tree; the buffers keep their addresses.
int accel_refit(krr_accel *a, const float *d_vertices, int64_t n_tris, cudaStream_t stream);
void accel_free(krr_accel *a);
// Several BVHs, one per part of the triangles (part p holds the global ids
// [part_begin[p], part_begin[p + 1])), in one node and triangle array: part
// p's tree starts at a->roots[p].  Hits are those of a build per part.  One
// part builds as accel_build.
int accel_build_parts(krr_accel *a, const float *d_vertices, const int64_t *part_begin, int n_parts,
                      cudaStream_t stream);

struct TraceLaunch {
    const float4 *ray_o;      // origin.xyz, tmin
    const float4 *ray_d;      // direction.xyz, tmax
    int ray_stride;           // float4 stride between consecutive rays
    int64_t n;                // ray count if d_count == nullptr, else the queue capacity
    const int *d_count;       // device ray count (queue counter, read as min(*d_count, n)) or nullptr
    float4 *hits;             // closest: t, b1, b2, prim bits
    uint8_t *occluded;        // any-hit output
    int *counter;             // scratch work counter (zeroed by the launcher)
    int *err;                 // device error flags
    int refill_below;         // refill a warp's idle lanes when fewer lanes are busy
    int postpone_pct;         // postpone triangles when fewer % of busy lanes have some
    int stack_limit;          // traversal stack entries a ray may use (1..kTraversalStack)
    // Mixed launches only: an any-hit ray set traced in the same launch as
    // the closest-hit set above (same stride); its rays take indices
    // [0, *d_any_count) of the shared work counter.
    const float4 *any_o;
    const float4 *any_d;
    const int *d_any_count;
    // Several BVHs (accel_build_parts): ray i starts at roots[pixel_part[p]]
    // with p the pixel id in ray_pix[i * ray_stride].w (any_pix for the
    // any-hit set); roots == nullptr: every ray starts at node 0.
    const uint32_t *roots;
    const uint8_t *pixel_part;
    const float4 *ray_pix;
    const float4 *any_pix;
};

int launch_trace_closest(const krr_accel *a, const TraceLaunch &l, cudaStream_t s);
int launch_trace_any(const krr_accel *a, const TraceLaunch &l, cudaStream_t s);
// One launch for an any-hit set (any_o/any_d -> occluded) and a closest-hit
// set (ray_o/ray_d -> hits): the two sets share one persistent grid, so the
// latency tail of the longest ray is paid once.
int launch_trace_mixed(const krr_accel *a, const TraceLaunch &l, cudaStream_t s);
int traversal_grid_size();

// Two-level structures (instanced.cu).
struct InstancedView {
    const float4 *tlas_nodes, *tlas_tris, *blas_nodes, *blas_tris;
    const TraceInst *inst;
};
struct InstancedInput {
    const float *d_geom_vertices;      // object-space triangles of every geometry, 9 floats each
    const int64_t *geom_tri_begin;     // host, n_geoms + 1 entries
    int n_geoms;
    const int32_t *inst_geom;          // host, per instance
    const float *inst_xf;              // host, object -> world 3x4 per instance
    const uint8_t *inst_mask;          // host, per instance, or nullptr (all 1)
    int n_instances;
};
int accel_build_instanced(krr_accel *a, const InstancedInput &in, cudaStream_t s);
// New object -> world transforms (12 floats per instance): the instance
// level is rebuilt, the geometry trees are kept.
int accel_update_instances(krr_accel *a, const float *inst_xf, cudaStream_t s);
int launch_trace_instanced(const krr_accel *a, const TraceLaunch &l, int mode, cudaStream_t s);
InstancedView instanced_view(const krr_accel *a);
// Object-space triangles (9 floats) of n triangles of a mesh's arrays.
int geometry_triangles(const float *d_pos, const uint32_t *d_idx, int64_t n, float *d_out, cudaStream_t s);
// Reads and clears the traversal error flags (device int at d_err) after the
// stream's work; KRR_ERR_OVERFLOW if a ray was cut off by the stack limit.
int take_trace_errors(int *d_err, cudaStream_t s, uint32_t *out_flags);

}  // namespace krr
