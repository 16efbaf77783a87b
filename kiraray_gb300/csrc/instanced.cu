// Two-level acceleration structure: one BVH per mesh geometry in object
// space (the bottom level, all geometries' trees in one node array) and a
// BVH over the instances' world-space boxes (the top level), as the
// reference's OptiX scene builds a GAS per mesh and an IAS over instances
// with 3x4 transforms (src/core/device/optix.cpp:357-398) and updates only
// the instance level when instances move (optix.cpp:618-669).
//
// Traversal: the world ray walks the top level; at an
// instance leaf the ray is carried into the instance's object space by the
// instance's world-to-object 3x4 matrix (row by row, m0 x + m1 y + m2 z
// (+ m3), each operation rounded), the instance's tree is searched for the
// closest hit with t in (tmin, best t] (ties inside it to the smaller
// triangle id), and the result replaces the best hit if its t is smaller,
// or equal with a smaller global id.  The hit is therefore the smallest
// (t, global id) over all instances, whatever the traversal order; the CPU
// oracle computes the same instance by instance.  t is the parameter of the
// object-space ray, which equals the world ray's up to rounding.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "accel.h"
#include "accel_device.cuh"
#include "kmath.cuh"

namespace krr {

namespace {

constexpr int kInstThreads = 128;

// MODE 0 closest, 1 any, 2 mixed (any-hit set first), as the one-level
// kernels: persistent warps that refill idle lanes from a work counter, as
// the one-level kernel (accel.cu), with one loop over both levels.
// At an instance leaf the lane saves its pending top-level work (node group,
// remaining instance leaves) and a return marker on its stack, carries the
// ray into the instance's object space and walks the geometry tree there,
// comparing every triangle's (t, global id) with the best so far; popping
// the marker reloads the world ray.  Each instance leaf and each triangle is
// tested exactly as in trace_two_level, and the result is the smallest
// (t, global id) as there.
constexpr uint32_t kTriGroupBit = 0x80000000u;   // stack entry: pending leaf group
constexpr uint32_t kReturnBit = 0x40000000u;     // stack entry: back to the world ray

// Eight blocks per SM (64 registers, the mixed variant spills 96 bytes):
// 1.31 against 1.39 ms per 2.07M camera rays at six blocks (80 registers).
template <int MODE, int FMT>
__global__ void __launch_bounds__(kInstThreads, 8)
k_trace_two_level_p(InstancedView v, TraceLaunch L) {
    const int lane = threadIdx.x & 31;
    const int64_t n_any = MODE == 2 ? min((int64_t)*L.d_any_count, L.n) : 0;
    const int64_t n = (L.d_count ? min((int64_t)*L.d_count, L.n) : L.n) + n_any;
    bool any_ray = MODE == 1;
    uint2 stack[kTraversalStack];
    int sp = 0;
    bool active = false, exhausted = false, in_geom = false;
    int64_t ray_id = 0;
    RayPre r;
    V3 inv, oinv;
    int oct = 0;
    float tmax = 0.f, tmin0 = 0.f;
    uint2 ng = make_uint2(0, 0), tg = make_uint2(0, 0);
    float best_b1 = 0.f, best_b2 = 0.f;
    uint32_t best_prim = KRR_MISS, id_delta = 0;

    auto world_ray = [&](V3 &o, V3 &d) {
        const float4 *po = (MODE == 2 && any_ray) ? L.any_o : L.ray_o;
        const float4 *pd = (MODE == 2 && any_ray) ? L.any_d : L.ray_d;
        const float4 ro = po[ray_id * L.ray_stride], rd = pd[ray_id * L.ray_stride];
        o = f3(ro);
        d = f3(rd);
        tmin0 = ro.w;
    };
    // Box tests need only the ray's origin, inverse direction and octant; the
    // triangle test's shear and axis permutation (ray_pre, three correctly
    // rounded divisions) are computed when a geometry tree first hands the
    // ray a triangle, so the world ray (instance boxes only) and instances
    // whose triangles are never reached skip them.
    bool tri_ready = false;
    auto set_ray = [&](V3 o, V3 d) {
        r.o = o;
        r.d = d;
        r.tmin = tmin0 > 0.f ? tmin0 : 0.f;
        tri_ready = false;
        inv = box_inverse(d);
        oinv = V3{-o.x * inv.x, -o.y * inv.y, -o.z * inv.z};
        oct = (inv.x < 0.f ? 1 : 0) | (inv.y < 0.f ? 2 : 0) | (inv.z < 0.f ? 4 : 0);
    };

    while (true) {
        unsigned act = __ballot_sync(0xffffffffu, active);
        if (__popc(act) < L.refill_below && !exhausted) {
            unsigned need = ~act;
            int leader = __ffs(need) - 1;
            long long base = 0;
            if (lane == leader) base = atomicAdd(reinterpret_cast<unsigned long long *>(L.counter),
                                                 (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + __popc(need) >= n) exhausted = true;
            if (!active) {
                int64_t idx = base + __popc(need & ((1u << lane) - 1));
                if (idx < n) {
                    if (MODE == 2) {
                        any_ray = idx < n_any;
                        if (!any_ray) idx -= n_any;
                    }
                    ray_id = idx;
                    V3 o, d;
                    world_ray(o, d);
                    tmax = ((MODE == 2 && any_ray) ? L.any_d : L.ray_d)[ray_id * L.ray_stride].w;
                    set_ray(o, d);
                    ng = make_uint2(0u, (1u << oct) | (1u << 8));
                    tg = make_uint2(0u, 0u);
                    sp = 0;
                    in_geom = false;
                    best_prim = KRR_MISS;
                    active = true;
                }
            }
            act = __ballot_sync(0xffffffffu, active);
        }
        if (act == 0) break;

        bool done = false;
        if (active && (ng.y & 0xffu)) {
            int p = __ffs(ng.y & 0xffu) - 1;
            ng.y &= ~(1u << p);
            int slot = p ^ oct;
            uint32_t imask = ng.y >> 8;
            uint32_t child = ng.x + __popc(imask & ((1u << slot) - 1u));
            if (ng.y & 0xffu) {
                if (sp < L.stack_limit) stack[sp++] = ng;
                else { atomicOr(L.err, (int)kErrStackOverflow); done = true; best_prim = kCutRay; }
            }
            visit<FMT>(in_geom ? v.blas_nodes : v.tlas_nodes, child, r, inv, oinv, oct, tmax, ng, tg);
        }
        // instance leaves: enter the first one not masked off (the remaining
        // ones wait on the stack); the step ends with no leaf group pending
        while (active && !done && tg.y && !in_geom) {
            const int b = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const uint32_t k = __float_as_uint(__ldg(v.tlas_tris + 3 * (size_t)(tg.x + b)).w);
            const TraceInst I = v.inst[k];
            if (any_ray && !I.mask) continue;
            const int need_slots = ((ng.y & 0xffu) ? 1 : 0) + (tg.y ? 1 : 0) + 1;
            if (sp + need_slots > L.stack_limit) {
                atomicOr(L.err, (int)kErrStackOverflow);
                done = true;
                best_prim = kCutRay;
                break;
            }
            if (ng.y & 0xffu) stack[sp++] = ng;
            if (tg.y) stack[sp++] = make_uint2(tg.x, tg.y | kTriGroupBit);
            stack[sp++] = make_uint2(0u, kReturnBit);
            V3 o, d;
            world_ray(o, d);
            set_ray(inst_point(I.inv, o), inst_vector(I.inv, d));
            ng = make_uint2(I.blas_root, (1u << oct) | (1u << 8));
            tg = make_uint2(0u, 0u);
            id_delta = I.id_delta;
            in_geom = true;
        }
        if (active && in_geom && tg.y && !done && !tri_ready) {
            r = ray_pre(r.o, r.d, tmin0);
            tri_ready = true;
        }
        while (active && in_geom && tg.y && !done) {
            const int b = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const float4 *tp = v.blas_tris + 3 * (size_t)(tg.x + b);
            const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
            float b1, b2;
            const float t = tri_test(r, v0, v1, v2, b1, b2);
            const uint32_t gid = __float_as_uint(v0.w) + id_delta;
            if (any_ray) {
                if (t > r.tmin && t <= tmax) { best_prim = gid; done = true; }
            } else if (t > r.tmin && (t < tmax || (t == tmax && gid < best_prim))) {
                tmax = t; best_b1 = b1; best_b2 = b2; best_prim = gid;
            }
        }
        if (active && !done && !(ng.y & 0xffu) && tg.y == 0u) {
            if (sp > 0) {
                const uint2 e = stack[--sp];
                if (e.y & kReturnBit) {
                    V3 o, d;
                    world_ray(o, d);
                    set_ray(o, d);
                    in_geom = false;
                    ng = make_uint2(0u, 0u);
                } else if (e.y & kTriGroupBit) {
                    tg = make_uint2(e.x, e.y & 0x00ffffffu);
                } else {
                    ng = e;
                }
            } else {
                done = true;
            }
        }
        if (!active) continue;
        if (done) {
            if (any_ray) {
                L.occluded[ray_id] = best_prim == kCutRay ? 0xFF : (best_prim != KRR_MISS ? 1 : 0);
            } else {
                L.hits[ray_id] = best_prim < kCutRay
                                     ? make_float4(tmax, best_b1, best_b2, __uint_as_float(best_prim))
                                     : make_float4(best_prim == kCutRay ? __int_as_float(0x7fffffff) : INFINITY,
                                                   0.f, 0.f, __uint_as_float(KRR_MISS));
            }
            active = false;
        }
    }
}

// Object-space triangles of geometry g (mesh arrays) in [begin, end).
__global__ void k_geometry_triangles(const float *__restrict__ pos, const uint32_t *__restrict__ idx,
                                     int64_t n, float *out) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = idx[3 * t + k];
        for (int c = 0; c < 3; ++c) out[9 * t + 3 * k + c] = pos[3 * vi + c];
    }
}

}  // namespace

InstancedView instanced_view(const krr_accel *a) {
    InstancedView v{};
    v.tlas_nodes = a->tlas->d_nodes;
    v.tlas_tris = a->tlas->d_tris;
    v.inst = a->d_inst;
    if (a->blas) {
        v.blas_nodes = a->blas->d_nodes;
        v.blas_tris = a->blas->d_tris;
    }
    return v;
}

// 3x4 object->world to world->object, in double, rounded once.
static void invert_3x4(const float *m, float *out) {
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double A = e * i - f * h, B = -(d * i - f * g), Cc = d * h - e * g;
    const double det = a * A + b * B + c * Cc;
    const double id = det != 0.0 ? 1.0 / det : 0.0;
    const double inv[9] = {A * id, -(b * i - c * h) * id, (b * f - c * e) * id,
                           B * id, (a * i - c * g) * id, -(a * f - c * d) * id,
                           Cc * id, -(a * h - b * g) * id, (a * e - b * d) * id};
    const double t[3] = {m[3], m[7], m[11]};
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) out[4 * r + k] = (float)inv[3 * r + k];
        out[4 * r + 3] = (float)(-(inv[3 * r] * t[0] + inv[3 * r + 1] * t[1] + inv[3 * r + 2] * t[2]));
    }
}

// The top level over the instances' world boxes (each box given to the
// builder as the degenerate triangle lo, hi, hi; the builder stores the
// instance index as the triangle id).  Instance records alongside.
static int build_top_level(krr_accel *a, cudaStream_t s) {
    const int n = (int)a->inst_geom.size();
    std::vector<float> boxes(9 * (size_t)n);
    a->h_inst.assign(n, TraceInst{});
    for (int i = 0; i < n; ++i) {
        const int g = a->inst_geom[i];
        const float *m = &a->inst_xf[12 * (size_t)i];
        const float *b = &a->blas->part_bounds[6 * (size_t)g];
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        const bool empty = a->geom_begin[g + 1] == a->geom_begin[g];
        for (int c = 0; c < 8 && !empty; ++c) {
            const double p[3] = {b[(c & 1) ? 3 : 0], b[(c & 2) ? 4 : 1], b[(c & 4) ? 5 : 2]};
            for (int r = 0; r < 3; ++r) {
                const double w = m[4 * r] * p[0] + m[4 * r + 1] * p[1] + m[4 * r + 2] * p[2] + m[4 * r + 3];
                lo[r] = std::min(lo[r], (float)w);
                hi[r] = std::max(hi[r], (float)w);
            }
        }
        if (empty) for (int r = 0; r < 3; ++r) lo[r] = hi[r] = 0.f;
        // widen by a few ulps of the box's magnitude (the rounding of the
        // corners above); the builder widens every leaf box again
        for (int r = 0; r < 3; ++r) {
            const float mag = std::max(std::fabs(lo[r]), std::fabs(hi[r]));
            lo[r] -= std::ldexp(mag, -20);
            hi[r] += std::ldexp(mag, -20);
        }
        float *t = &boxes[9 * (size_t)i];
        for (int r = 0; r < 3; ++r) { t[r] = lo[r]; t[3 + r] = hi[r]; t[6 + r] = hi[r]; }
        TraceInst &I = a->h_inst[i];
        invert_3x4(m, I.inv);
        I.blas_root = a->blas->roots.empty() ? 0u : a->blas->roots[g];
        I.id_delta = (uint32_t)(a->inst_first[i] - a->geom_begin[g]);
        I.mask = empty ? 0u : a->inst_mask[i];
    }
    float *d_boxes = nullptr;
    KRR_CUDA(cudaMalloc(&d_boxes, std::max<size_t>(boxes.size(), 9) * sizeof(float)));
    int st = cuda_status(cudaMemcpyAsync(d_boxes, boxes.data(), boxes.size() * sizeof(float),
                                         cudaMemcpyHostToDevice, s), "cudaMemcpyAsync", __FILE__, __LINE__);
    if (st == KRR_OK) st = accel_build(a->tlas, d_boxes, n, s);
    cudaStreamSynchronize(s);
    cudaFree(d_boxes);
    if (st != KRR_OK) return st;
    if (!a->d_inst) KRR_CUDA(cudaMalloc(&a->d_inst, std::max(1, n) * sizeof(TraceInst)));
    KRR_CUDA(cudaMemcpyAsync(a->d_inst, a->h_inst.data(), n * sizeof(TraceInst), cudaMemcpyHostToDevice, s));
    KRR_CUDA(cudaStreamSynchronize(s));
    return KRR_OK;
}

int accel_build_instanced(krr_accel *a, const InstancedInput &in, cudaStream_t s) {
    KRR_CHECK_ARG(in.n_geoms >= 1 && in.n_instances >= 0, "bad instanced input");
    accel_free(a);
    a->levels = 2;
    a->blas = new krr_accel();
    a->tlas = new krr_accel();
    a->geom_begin.assign(in.geom_tri_begin, in.geom_tri_begin + in.n_geoms + 1);
    a->inst_geom.assign(in.inst_geom, in.inst_geom + in.n_instances);
    a->inst_xf.assign(in.inst_xf, in.inst_xf + 12 * (size_t)in.n_instances);
    a->inst_mask.assign(in.n_instances, 1u);
    if (in.inst_mask)
        for (int i = 0; i < in.n_instances; ++i) a->inst_mask[i] = in.inst_mask[i] ? 1u : 0u;
    a->inst_first.assign(in.n_instances, 0);
    int64_t total = 0;
    for (int i = 0; i < in.n_instances; ++i) {
        const int g = in.inst_geom[i];
        KRR_CHECK_ARG(g >= 0 && g < in.n_geoms, "instance geometry out of range");
        a->inst_first[i] = total;
        total += a->geom_begin[g + 1] - a->geom_begin[g];
    }
    KRR_CHECK_ARG(total < (int64_t)0x7fffffff, "too many instanced triangles");
    a->inst_triangles = total;
    KRR_TRY(accel_build_parts(a->blas, in.d_geom_vertices, a->geom_begin.data(), in.n_geoms, s));
    if (a->blas->roots.empty()) a->blas->roots.assign(1, 0u);   // one geometry: root 0
    KRR_TRY(build_top_level(a, s));
    // the combined structure: its own work counter and error flags, sizes
    // and bounds for the statistics
    KRR_CUDA(cudaMalloc(&a->d_scratch, 64));
    KRR_CUDA(cudaMemsetAsync(a->d_scratch, 0, 64, s));
    a->n_tris = total;
    a->n_nodes = a->tlas->n_nodes + a->blas->n_nodes;
    a->max_depth = a->tlas->max_depth + a->blas->max_depth;
    a->build_ms = a->tlas->build_ms + a->blas->build_ms;
    a->node_format = a->blas->node_format;
    for (int k = 0; k < 3; ++k) { a->scene_lo[k] = a->tlas->scene_lo[k]; a->scene_hi[k] = a->tlas->scene_hi[k]; }
    KRR_CUDA(cudaStreamSynchronize(s));
    return KRR_OK;
}

int accel_update_instances(krr_accel *a, const float *inst_xf, cudaStream_t s) {
    KRR_CHECK_ARG(a && a->levels == 2, "not a two-level structure");
    std::memcpy(a->inst_xf.data(), inst_xf, a->inst_xf.size() * sizeof(float));
    KRR_TRY(build_top_level(a, s));
    for (int k = 0; k < 3; ++k) { a->scene_lo[k] = a->tlas->scene_lo[k]; a->scene_hi[k] = a->tlas->scene_hi[k]; }
    return KRR_OK;
}

int launch_trace_instanced(const krr_accel *a, const TraceLaunch &l, int mode, cudaStream_t s) {
    const InstancedView v = instanced_view(a);
    const bool fmt1 = a->node_format == 1;
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_two_level_p<0, 0>, kInstThreads, 0);
        grid = std::max(1, sms) * std::max(1, per_sm);
    }
    KRR_CHECK_ARG(l.counter != nullptr, "the two-level traversal needs a work counter");
    KRR_CUDA(cudaMemsetAsync(l.counter, 0, sizeof(unsigned long long), s));
    switch (mode) {
        case 0: fmt1 ? k_trace_two_level_p<0, 1><<<grid, kInstThreads, 0, s>>>(v, l)
                     : k_trace_two_level_p<0, 0><<<grid, kInstThreads, 0, s>>>(v, l); break;
        case 1: fmt1 ? k_trace_two_level_p<1, 1><<<grid, kInstThreads, 0, s>>>(v, l)
                     : k_trace_two_level_p<1, 0><<<grid, kInstThreads, 0, s>>>(v, l); break;
        default: fmt1 ? k_trace_two_level_p<2, 1><<<grid, kInstThreads, 0, s>>>(v, l)
                      : k_trace_two_level_p<2, 0><<<grid, kInstThreads, 0, s>>>(v, l); break;
    }
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

int geometry_triangles(const float *d_pos, const uint32_t *d_idx, int64_t n, float *d_out, cudaStream_t s) {
    if (n == 0) return KRR_OK;
    k_geometry_triangles<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_pos, d_idx, n, d_out);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

}  // namespace krr

using namespace krr;

extern "C" int krr_accel_create_instanced(const float *h_geom_vertices, const int64_t *h_geom_tri_begin,
                                          int32_t n_geoms, const krr_instance_desc *h_instances,
                                          int32_t n_instances, const uint8_t *h_instance_mask,
                                          krr_accel **out, void *stream) {
    KRR_CHECK_ARG(out && h_geom_tri_begin && n_geoms >= 1 && n_instances >= 0 &&
                      (n_instances == 0 || h_instances),
                  "bad argument");
    for (int g = 0; g < n_geoms; ++g)
        KRR_CHECK_ARG(h_geom_tri_begin[g + 1] >= h_geom_tri_begin[g], "geometry ranges must not decrease");
    KRR_CHECK_ARG(h_geom_tri_begin[0] == 0, "the first geometry starts at triangle 0");
    const int64_t n_tris = h_geom_tri_begin[n_geoms];
    KRR_CHECK_ARG(n_tris == 0 || h_geom_vertices, "vertices are NULL");
    cudaStream_t s = as_stream(stream);
    float *d_v = nullptr;
    const size_t bytes = sizeof(float) * 9 * (size_t)n_tris;
    KRR_CUDA(cudaMalloc(&d_v, std::max<size_t>(bytes, 4)));
    cudaError_t e = cudaMemcpyAsync(d_v, h_geom_vertices, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { cudaFree(d_v); return cuda_status(e, "cudaMemcpyAsync", __FILE__, __LINE__); }
    std::vector<int32_t> geom(n_instances);
    std::vector<float> xf(12 * (size_t)n_instances);
    for (int i = 0; i < n_instances; ++i) {
        geom[i] = h_instances[i].mesh;
        std::memcpy(&xf[12 * (size_t)i], h_instances[i].transform, 12 * sizeof(float));
    }
    InstancedInput in{d_v, h_geom_tri_begin, n_geoms, geom.data(), xf.data(), h_instance_mask, n_instances};
    krr_accel *a = new krr_accel();
    int st = accel_build_instanced(a, in, s);
    cudaStreamSynchronize(s);
    cudaFree(d_v);
    if (st != KRR_OK) { accel_free(a); delete a; return st; }
    *out = a;
    return KRR_OK;
}

extern "C" int krr_accel_update_instances(krr_accel *a, const float *h_transforms, void *stream) {
    KRR_CHECK_ARG(a && h_transforms, "NULL argument");
    KRR_CHECK_ARG(a->levels == 2, "krr_accel_update_instances takes a two-level structure");
    const int st = accel_update_instances(a, h_transforms, as_stream(stream));
    cudaStreamSynchronize(as_stream(stream));
    return st;
}

extern "C" int krr_accel_instance_inverse(const krr_accel *a, float *h_out, int32_t n) {
    KRR_CHECK_ARG(a && h_out, "NULL argument");
    KRR_CHECK_ARG(a->levels == 2, "not a two-level structure");
    KRR_CHECK_ARG(n == (int32_t)a->h_inst.size(), "instance count differs");
    for (int i = 0; i < n; ++i) std::memcpy(h_out + 12 * (size_t)i, a->h_inst[i].inv, 12 * sizeof(float));
    return KRR_OK;
}
