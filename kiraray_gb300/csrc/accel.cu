// GPU BVH builder and traversal.
//
// Replaces the OptiX acceleration structures of the reference
// (OptixScene::buildTriangleMeshGAS / buildASFromInputs,
// src/core/device/optix.cpp:143-250, and the single-level IAS at :357-398)
// and the closest-hit / any-hit programs (src/render/wavefront/device.cu:43-100).
// The reference has no software triangle test (OptiX does it in hardware); the
// test here is the watertight test of Woop, Benthin and Wald (JCGT 2013).
//
// Build: per-triangle bounds -> 63-bit Morton codes of centroids -> radix
// sort -> Karras (HPG 2012) binary radix tree -> bottom-up bounds -> greedy
// top-down collapse into compressed 8-wide nodes (Ylitie, Karras, Laine,
// HPG 2017 layout, own collapse heuristic) -> triangles gathered in leaf order.
//
// Traversal: persistent warps that refill idle lanes from a global ray
// counter, one ray per lane, node groups / triangle groups on a per-lane
// stack, octant-ordered child visits.  Box tests are conservative (children
// are widened by a margin before quantisation and compared with a small
// slack), so the hit set equals brute force; ties in t go to the smaller
// global triangle id, which makes the closest hit independent of the
// traversal order.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "accel.h"
#include "accel_device.cuh"
#include "kmath.cuh"

namespace krr {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kBuildThreads = 256;

__device__ __forceinline__ void atomic_min_f(float *addr, float v) {
    if (v >= 0.f) atomicMin(reinterpret_cast<int *>(addr), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned *>(addr), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float *addr, float v) {
    if (v >= 0.f) atomicMax(reinterpret_cast<int *>(addr), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned *>(addr), __float_as_uint(v));
}

__device__ __forceinline__ V3 ld3(const float *p) { return V3{p[0], p[1], p[2]}; }

// ---------------------------------------------------------------- bounds
// bounds[0..2] = centroid min, [3..5] = centroid max, [6..8] = geometry min,
// [9..11] = geometry max.
__global__ void k_scene_bounds(const float *__restrict__ v, int64_t n, float *bounds) {
    V3 cmin = v3(INFINITY), cmax = v3(-INFINITY), gmin = v3(INFINITY), gmax = v3(-INFINITY);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        V3 a = ld3(v + 9 * i), b = ld3(v + 9 * i + 3), c = ld3(v + 9 * i + 6);
        V3 lo = vmin(a, vmin(b, c)), hi = vmax(a, vmax(b, c));
        V3 ce = (lo + hi) * 0.5f;
        cmin = vmin(cmin, ce); cmax = vmax(cmax, ce);
        gmin = vmin(gmin, lo); gmax = vmax(gmax, hi);
    }
    float vals[12] = {cmin.x, cmin.y, cmin.z, cmax.x, cmax.y, cmax.z,
                      gmin.x, gmin.y, gmin.z, gmax.x, gmax.y, gmax.z};
    for (int k = 0; k < 12; ++k) {
        float x = vals[k];
        bool is_min = (k % 6) < 3;
        for (int off = 16; off > 0; off >>= 1) {
            float y = __shfl_xor_sync(0xffffffffu, x, off);
            x = is_min ? fminf(x, y) : fmaxf(x, y);
        }
        if ((threadIdx.x & 31) == 0) {
            if (is_min) atomic_min_f(bounds + k, x);
            else atomic_max_f(bounds + k, x);
        }
    }
}

__device__ __forceinline__ uint64_t spread21(uint32_t x) {
    uint64_t v = x & 0x1fffffu;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// Morton codes of centroids and margin-widened leaf boxes.
// cubic: one cell size on all three axes (the largest centroid extent), so
// that the code's splits follow the scene's proportions; otherwise each axis
// is normalised by its own extent.
__global__ void k_leaf_setup(const float *__restrict__ v, int64_t n, const float *bounds,
                             float margin, int cubic, uint64_t *keys, uint32_t *vals,
                             float4 *leaf_lo, float4 *leaf_hi) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 a = ld3(v + 9 * i), b = ld3(v + 9 * i + 3), c = ld3(v + 9 * i + 6);
    V3 lo = vmin(a, vmin(b, c)), hi = vmax(a, vmax(b, c));
    V3 ce = (lo + hi) * 0.5f;
    V3 cmin = ld3(bounds), cmax = ld3(bounds + 3);
    V3 ext = cmax - cmin;
    const float emax = fmaxf(ext.x, fmaxf(ext.y, ext.z));
    float q[3];
    for (int k = 0; k < 3; ++k) {
        float e = cubic ? emax : get(ext, k);
        float t = e > 0.f ? (get(ce, k) - get(cmin, k)) / e : 0.5f;
        q[k] = fminf(fmaxf(t * 2097152.f, 0.f), 2097151.f);
    }
    keys[i] = (spread21((uint32_t)q[0]) << 2) | (spread21((uint32_t)q[1]) << 1) |
              spread21((uint32_t)q[2]);
    vals[i] = (uint32_t)i;
    leaf_lo[i] = make_float4(lo.x - margin, lo.y - margin, lo.z - margin, 0.f);
    leaf_hi[i] = make_float4(hi.x + margin, hi.y + margin, hi.z + margin, 0.f);
}

__device__ __forceinline__ int delta_fn(const uint64_t *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz((uint32_t)(i ^ j));
    return __clzll(a ^ b);
}

// Karras 2012 radix tree: internal node i covers the sorted leaves [first, last]
// (count = last - first + 1 of them).
__global__ void k_karras(const uint64_t *__restrict__ keys, int n, uint32_t *left,
                         uint32_t *right, int *count, int *parent_int, int *parent_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta_fn(keys, n, i, i + 1) - delta_fn(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta_fn(keys, n, i, i - d);
    int lmax = 2;
    while (delta_fn(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta_fn(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta_fn(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta_fn(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    count[i] = hi - lo + 1;
    if (lo == gamma) { left[i] = kLeafBit | gamma; parent_leaf[gamma] = i; }
    else { left[i] = gamma; parent_int[gamma] = i; }
    if (hi == gamma + 1) { right[i] = kLeafBit | (gamma + 1); parent_leaf[gamma + 1] = i; }
    else { right[i] = gamma + 1; parent_int[gamma + 1] = i; }
    if (i == 0) parent_int[0] = -1;
}

// Leaf boxes are indexed by sorted position; internal boxes by node index.
__global__ void k_gather_leaf_boxes(const uint32_t *__restrict__ sorted_idx, int n,
                                    const float4 *__restrict__ lo_in,
                                    const float4 *__restrict__ hi_in, float4 *lo_out,
                                    float4 *hi_out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = sorted_idx[i];
    lo_out[i] = lo_in[p];
    hi_out[i] = hi_in[p];
}

__global__ void k_bottom_up(int n, const uint32_t *__restrict__ left,
                            const uint32_t *__restrict__ right, const int *__restrict__ parent_int,
                            const int *__restrict__ parent_leaf, const float4 *leaf_lo,
                            const float4 *leaf_hi, float4 *int_lo, float4 *int_hi, int *flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = parent_leaf[i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;
        __threadfence();
        uint32_t l = left[node], r = right[node];
        float4 llo = (l & kLeafBit) ? leaf_lo[l & ~kLeafBit] : __ldcg(int_lo + l);
        float4 lhi = (l & kLeafBit) ? leaf_hi[l & ~kLeafBit] : __ldcg(int_hi + l);
        float4 rlo = (r & kLeafBit) ? leaf_lo[r & ~kLeafBit] : __ldcg(int_lo + r);
        float4 rhi = (r & kLeafBit) ? leaf_hi[r & ~kLeafBit] : __ldcg(int_hi + r);
        float4 lo = make_float4(fminf(llo.x, rlo.x), fminf(llo.y, rlo.y), fminf(llo.z, rlo.z), 0.f);
        float4 hi = make_float4(fmaxf(lhi.x, rhi.x), fmaxf(lhi.y, rhi.y), fmaxf(lhi.z, rhi.z), 0.f);
        __stcg(int_lo + node, lo);
        __stcg(int_hi + node, hi);
        node = parent_int[node];
    }
}

// ------------------------------------------------------------- collapse
struct CollapseItem {
    uint32_t bref;    // binary node ref (kLeafBit | sorted leaf) or internal index
    uint32_t wnode;   // destination 8-wide node
    int depth;
};

// Binary tree handed to the collapse (LBVH or PLOC): internal node i has
// children left[i], right[i] (kLeafBit | sorted leaf, or an internal index),
// bounds int_lo/int_hi[i] and count[i] leaves below it.
struct BinTree {
    const uint32_t *left, *right;
    const int *count;
    const float4 *int_lo, *int_hi, *leaf_lo, *leaf_hi;
    const uint32_t *sorted_idx;
};

__device__ __forceinline__ void ref_info(const BinTree &t, uint32_t ref, V3 &lo, V3 &hi, int &count) {
    if (ref & kLeafBit) {
        uint32_t k = ref & ~kLeafBit;
        lo = f3(t.leaf_lo[k]); hi = f3(t.leaf_hi[k]);
        count = 1;
    } else {
        lo = f3(t.int_lo[ref]); hi = f3(t.int_hi[ref]);
        count = t.count[ref];
    }
}

// Triangles (original ids) under a subtree of at most three leaves.
__device__ __forceinline__ int subtree_leaves(const BinTree &t, uint32_t ref, uint32_t out[3]) {
    uint32_t st[4];
    int sp = 0, n = 0;
    st[sp++] = ref;
    while (sp > 0 && n < 3) {
        uint32_t r = st[--sp];
        if (r & kLeafBit) { out[n++] = t.sorted_idx[r & ~kLeafBit]; continue; }
        if (sp + 2 > 4) break;
        st[sp++] = t.right[r];
        st[sp++] = t.left[r];
    }
    return n;
}

__device__ __forceinline__ float half_area(V3 lo, V3 hi) {
    V3 e = hi - lo;
    return e.x * e.y + e.y * e.z + e.z * e.x;
}

// ------------------------------------------------------- treelet restructuring
// Treelet restructuring (Karras and Aila, "Fast Parallel Construction of
// High-Quality Bounding Volume Hierarchies", HPG 2013) of the binary tree
// before the collapse.  Nodes are visited bottom-up (a node is taken by the
// second of its children's walks, as in k_bottom_up); at each node with at
// least `min_count` triangles below it, the treelet of up to seven leaves
// grown by opening the largest-area leaf is rebuilt as the binary topology
// of least total internal surface area, found by dynamic programming over
// the 127 subsets of its leaves.  The treelet's internal nodes keep their
// indices (reassigned within the treelet); a topology no better than the
// current one by a relative 1e-5 is left alone, so ties (coincident
// triangles) never rearrange a balanced subtree into a chain.  All reads of
// the tree go through L2 (__ldcg): other threads rewrote the subtree.
constexpr int kTreeletLeaves = 7;
constexpr int kTreeletMinCount = 8;   // smaller subtrees are left as built

__device__ __forceinline__ void treelet_ref(const uint32_t ref, const float4 *int_lo,
                                            const float4 *int_hi, const float4 *leaf_lo,
                                            const float4 *leaf_hi, const int *count, V3 &lo,
                                            V3 &hi, int &n) {
    if (ref & kLeafBit) {
        lo = f3(leaf_lo[ref & ~kLeafBit]);
        hi = f3(leaf_hi[ref & ~kLeafBit]);
        n = 1;
    } else {
        lo = f3(__ldcg(int_lo + ref));
        hi = f3(__ldcg(int_hi + ref));
        n = __ldcg(count + ref);
    }
}

__device__ void restructure_treelet(uint32_t root, uint32_t *left, uint32_t *right, int *count,
                                    float4 *int_lo, float4 *int_hi, const float4 *leaf_lo,
                                    const float4 *leaf_hi) {
    uint32_t ref[kTreeletLeaves], inner[kTreeletLeaves - 2];
    V3 lo[kTreeletLeaves], hi[kTreeletLeaves];
    int cnt[kTreeletLeaves];
    float area[kTreeletLeaves];
    ref[0] = __ldcg(left + root);
    ref[1] = __ldcg(right + root);
    for (int k = 0; k < 2; ++k) {
        treelet_ref(ref[k], int_lo, int_hi, leaf_lo, leaf_hi, count, lo[k], hi[k], cnt[k]);
        area[k] = half_area(lo[k], hi[k]);
    }
    int nl = 2, ni = 0;
    float current = 0.f;   // internal area of the treelet below its root
    while (nl < kTreeletLeaves) {
        int pick = -1;
        float best = -1.f;
        for (int k = 0; k < nl; ++k)
            if (!(ref[k] & kLeafBit) && area[k] > best) { best = area[k]; pick = k; }
        if (pick < 0) break;
        const uint32_t open = ref[pick];
        inner[ni++] = open;
        current += area[pick];
        ref[pick] = __ldcg(left + open);
        ref[nl] = __ldcg(right + open);
        for (int k : {pick, nl}) {
            treelet_ref(ref[k], int_lo, int_hi, leaf_lo, leaf_hi, count, lo[k], hi[k], cnt[k]);
            area[k] = half_area(lo[k], hi[k]);
        }
        ++nl;
    }
    if (ni == 0) return;
    // cost[s]: least internal area of a binary tree over the leaf subset s
    // (its own root included); split[s]: the part of s holding s's lowest
    // leaf in that tree
    float cost[1 << kTreeletLeaves];
    uint8_t split[1 << kTreeletLeaves];
    const int full = (1 << nl) - 1;
    for (int s = 1; s <= full; ++s) {
        if ((s & (s - 1)) == 0) { cost[s] = 0.f; continue; }
        V3 slo = lo[__ffs(s) - 1], shi = hi[__ffs(s) - 1];
        for (int k = __ffs(s); k < nl; ++k)
            if (s >> k & 1) { slo = vmin(slo, lo[k]); shi = vmax(shi, hi[k]); }
        const int low = s & -s;
        float best = INFINITY;
        int arg = low;
        for (int p = (s - 1) & s; p; p = (p - 1) & s) {
            if (!(p & low)) continue;
            const float c = cost[p] + cost[s ^ p];
            if (c < best) { best = c; arg = p; }
        }
        cost[s] = half_area(slo, shi) + best;
        split[s] = (uint8_t)arg;
    }
    V3 rlo = lo[0], rhi = hi[0];
    for (int k = 1; k < nl; ++k) { rlo = vmin(rlo, lo[k]); rhi = vmax(rhi, hi[k]); }
    const float optimal = cost[full] - half_area(rlo, rhi);
    if (!(optimal < current * (1.f - 1e-5f))) return;
    // rewrite the treelet top-down from its root
    uint32_t st_node[kTreeletLeaves];
    int st_set[kTreeletLeaves];
    int sp = 0, na = ni;
    st_node[sp] = root;
    st_set[sp++] = full;
    while (sp > 0) {
        const uint32_t node = st_node[--sp];
        const int s = st_set[sp];
        const int parts[2] = {split[s], s ^ split[s]};
        uint32_t child[2];
        for (int h = 0; h < 2; ++h) {
            const int q = parts[h];
            if ((q & (q - 1)) == 0) {
                child[h] = ref[__ffs(q) - 1];
            } else {
                child[h] = inner[--na];
                st_node[sp] = child[h];
                st_set[sp++] = q;
            }
        }
        V3 slo = rlo, shi = rhi;
        int n = 0;
        bool first = true;
        for (int k = 0; k < nl; ++k) {
            if (!(s >> k & 1)) continue;
            slo = first ? lo[k] : vmin(slo, lo[k]);
            shi = first ? hi[k] : vmax(shi, hi[k]);
            first = false;
            n += cnt[k];
        }
        __stcg(left + node, child[0]);
        __stcg(right + node, child[1]);
        __stcg(count + node, n);
        __stcg(int_lo + node, make_float4(slo.x, slo.y, slo.z, 0.f));
        __stcg(int_hi + node, make_float4(shi.x, shi.y, shi.z, 0.f));
    }
}

__global__ void k_treelet(int n, uint32_t *left, uint32_t *right, int *count,
                          const int *__restrict__ par_int, const int *__restrict__ par_leaf,
                          float4 *int_lo, float4 *int_hi, const float4 *__restrict__ leaf_lo,
                          const float4 *__restrict__ leaf_hi, int *flags, int min_count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = par_leaf[i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;
        __threadfence();
        if (__ldcg(count + node) >= min_count)
            restructure_treelet((uint32_t)node, left, right, count, int_lo, int_hi, leaf_lo, leaf_hi);
        node = par_int[node];
    }
}

// ------------------------------------------------------------------ PLOC
// Parallel locally-ordered clustering (Meister and Bittner, IEEE TVCG 2018):
// the clusters stay in Morton order; each looks for the cluster within
// `radius` positions whose merged box has the smallest surface area, ties to
// the smallest i XOR j (the pair of least area and, among those, least XOR is
// mutual, so every round merges; coincident boxes pair up as (2k, 2k + 1)
// and give a balanced tree rather than a chain); mutual nearest neighbours
// merge into a new internal
// node at the smaller position, the other position drops out, and the
// survivors are compacted in order.  Higher-quality trees than the radix
// tree for the same Morton order.
struct Cluster {
    float4 lo;   // box min | ref bits (kLeafBit | sorted leaf, or internal node)
    float4 hi;   // box max | unused
};
constexpr int kPlocRadius = 16;
constexpr int kPlocThreads = 256;

__global__ void k_ploc_init(int n, const float4 *__restrict__ leaf_lo,
                            const float4 *__restrict__ leaf_hi, Cluster *c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 lo = leaf_lo[i];
    lo.w = __uint_as_float(kLeafBit | (uint32_t)i);
    c[i] = Cluster{lo, leaf_hi[i]};
}

__global__ void __launch_bounds__(kPlocThreads)
k_ploc_nn(const Cluster *__restrict__ c, int n, int r, uint32_t *__restrict__ nn) {
    __shared__ float4 slo[kPlocThreads + 2 * kPlocRadius], shi[kPlocThreads + 2 * kPlocRadius];
    const int base = blockIdx.x * kPlocThreads;
    for (int k = threadIdx.x; k < kPlocThreads + 2 * r; k += blockDim.x) {
        const int g = base - r + k;
        if (g >= 0 && g < n) { slo[k] = c[g].lo; shi[k] = c[g].hi; }
    }
    __syncthreads();
    const int i = base + threadIdx.x;
    if (i >= n) return;
    const V3 lo = f3(slo[threadIdx.x + r]), hi = f3(shi[threadIdx.x + r]);
    unsigned long long best = ~0ull;
    const int jlo = max(i - r, 0), jhi = min(i + r, n - 1);
    for (int j = jlo; j <= jhi; ++j) {
        if (j == i) continue;
        const int k = j - base + r;
        const float a = half_area(vmin(lo, f3(slo[k])), vmax(hi, f3(shi[k])));
        best = min(best, ((unsigned long long)__float_as_uint(a) << 32) | (uint32_t)(i ^ j));
    }
    nn[i] = (uint32_t)i ^ (uint32_t)best;
}

__global__ void k_ploc_merge(const Cluster *__restrict__ c, const uint32_t *__restrict__ nn, int n,
                             Cluster *out, uint8_t *keep, uint32_t *left, uint32_t *right,
                             int *count, float4 *int_lo, float4 *int_hi, int *node_counter) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = nn[i];
    const Cluster ci = c[i];
    if (nn[j] != (uint32_t)i) {
        out[i] = ci;
        keep[i] = 1;
        return;
    }
    if ((uint32_t)i > j) {
        keep[i] = 0;
        return;
    }
    const Cluster cj = c[j];
    const uint32_t ri = __float_as_uint(ci.lo.w), rj = __float_as_uint(cj.lo.w);
    const int node = atomicAdd(node_counter, 1);
    left[node] = ri;
    right[node] = rj;
    count[node] = ((ri & kLeafBit) ? 1 : count[ri]) + ((rj & kLeafBit) ? 1 : count[rj]);
    const float4 lo = make_float4(fminf(ci.lo.x, cj.lo.x), fminf(ci.lo.y, cj.lo.y),
                                  fminf(ci.lo.z, cj.lo.z), 0.f);
    const float4 hi = make_float4(fmaxf(ci.hi.x, cj.hi.x), fmaxf(ci.hi.y, cj.hi.y),
                                  fmaxf(ci.hi.z, cj.hi.z), 0.f);
    int_lo[node] = lo;
    int_hi[node] = hi;
    out[i] = Cluster{make_float4(lo.x, lo.y, lo.z, __uint_as_float((uint32_t)node)), hi};
    keep[i] = 1;
}

__device__ __forceinline__ int quant_exponent(float ext) {
    // smallest k with 2^k * 255 >= ext
    float s = ext * (1.0f + 1.0f / 1048576.f) / 255.f;
    int e;
    float m = frexpf(s, &e);   // s = m * 2^e, m in [0.5, 1)
    int k = (m == 0.5f) ? e - 1 : e;
    return max(min(k, 127), -126);
}

// Child boxes of one 8-wide node, by slot (empty slots have slot_box_lo.x =
// +inf): writes the quantisation frame and the quantised boxes (format 0:
// node quads 0 and 2-4, quad 1 left to the caller; format 1: the float planes,
// quads 0-11) and returns the node's bounds.  Used by the collapse and by the
// refit, so that both quantise alike: every quantised box contains its child
// box (floor/ceil, then stepped outwards while rounding left it inside).  An
// empty slot gets the inverted box lo = 255, hi = 0 on every axis, which no
// ray enters (its entry distance exceeds its exit distance by 255 steps).
__device__ void write_node_boxes(float4 *np, int format, const V3 *slo, const V3 *shi, uint32_t imask,
                                 V3 &out_lo, V3 &out_hi) {
    V3 lo = v3(INFINITY), hi = v3(-INFINITY);
    for (int s = 0; s < 8; ++s)
        if (slo[s].x != INFINITY) { lo = vmin(lo, slo[s]); hi = vmax(hi, shi[s]); }
    out_lo = lo;
    out_hi = hi;
    if (format == 1) {
        for (int k = 0; k < 3; ++k) {
            float b0[8], b1[8];
            for (int s = 0; s < 8; ++s) {
                const bool used = slo[s].x != INFINITY;
                b0[s] = used ? get(slo[s], k) : INFINITY;
                b1[s] = used ? get(shi[s], k) : -INFINITY;
            }
            np[4 * k + 0] = make_float4(b0[0], b0[1], b0[2], b0[3]);
            np[4 * k + 1] = make_float4(b0[4], b0[5], b0[6], b0[7]);
            np[4 * k + 2] = make_float4(b1[0], b1[1], b1[2], b1[3]);
            np[4 * k + 3] = make_float4(b1[4], b1[5], b1[6], b1[7]);
        }
        return;
    }
    int ek[3];
    float escale[3];
    for (int k = 0; k < 3; ++k) {
        ek[k] = quant_exponent(get(hi, k) - get(lo, k));
        escale[k] = ldexpf(1.f, ek[k]);
    }
    uint32_t qlo[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    uint32_t qhi[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int s = 0; s < 8; ++s) {
        if (slo[s].x == INFINITY) {
            for (int k = 0; k < 3; ++k) qlo[k][s >> 2] |= 0xffu << (8 * (s & 3));
            continue;
        }
        for (int k = 0; k < 3; ++k) {
            float p = get(lo, k), e = escale[k];
            float a = floorf((get(slo[s], k) - p) / e);
            float b = ceilf((get(shi[s], k) - p) / e);
            a = fminf(fmaxf(a, 0.f), 255.f);
            b = fminf(fmaxf(b, 0.f), 255.f);
            while (a > 0.f && fmaf(a, e, p) > get(slo[s], k)) a -= 1.f;
            while (b < 255.f && fmaf(b, e, p) < get(shi[s], k)) b += 1.f;
            qlo[k][s >> 2] |= (uint32_t)a << (8 * (s & 3));
            qhi[k][s >> 2] |= (uint32_t)b << (8 * (s & 3));
        }
    }
    uint32_t ew = (uint32_t)(ek[0] + 127) | ((uint32_t)(ek[1] + 127) << 8) |
                  ((uint32_t)(ek[2] + 127) << 16) | (imask << 24);
    np[0] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(ew));
    np[2] = make_float4(__uint_as_float(qlo[0][0]), __uint_as_float(qlo[0][1]),
                        __uint_as_float(qlo[1][0]), __uint_as_float(qlo[1][1]));
    np[3] = make_float4(__uint_as_float(qlo[2][0]), __uint_as_float(qlo[2][1]),
                        __uint_as_float(qhi[0][0]), __uint_as_float(qhi[0][1]));
    np[4] = make_float4(__uint_as_float(qhi[1][0]), __uint_as_float(qhi[1][1]),
                        __uint_as_float(qhi[2][0]), __uint_as_float(qhi[2][1]));
}

// ------------------------------------------------ cost-optimal collapse
// The 8-wide tree that minimises the surface-area cost over all ways of
// cutting the binary tree into wide nodes (Ylitie, Karras and Laine, "Efficient
// incoherent ray traversal on GPUs through compressed wide BVHs", HPG 2017,
// section 3.1), for one-triangle leaves.  With one triangle per leaf every
// triangle is tested when its own box is hit, whatever the cut, so the cost
// left to minimise is the wide nodes' visits: the sum of their areas.  For a
// binary node n and i = 1..8, C(n, i) is the least total area of the wide
// nodes when n's subtree is represented as at most i roots (wide nodes or
// triangles) plus everything below them:
//   triangle n:  C(n, i) = 0
//   internal n:  D(n, i) = min over 1 <= k < i of C(left, k) + C(right, i - k)
//                C(n, 1) = A(n) + D(n, 8)             (n becomes a wide node)
//                C(n, i) = min(C(n, i - 1), D(n, i))  (i >= 2)
// with A the half surface area.  A binary node's table needs only its
// children's, so the tables are filled bottom-up in one pass; each node keeps
// the split k of D(n, 8) (byte 0 of its choice word) and, for i = 2..8, the
// split taken by C(n, i) or 0 where C(n, i) = C(n, i - 1) (byte i - 1).  The
// collapse then reads a wide node's children off those choices.
__global__ void k_parents(int ni, const uint32_t *__restrict__ left, const uint32_t *__restrict__ right,
                          int *par_int, int *par_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni) return;
    for (uint32_t c : {left[i], right[i]}) {
        if (c & kLeafBit) par_leaf[c & ~kLeafBit] = i;
        else par_int[c] = i;
    }
}

__device__ __forceinline__ void cost_table(const BinTree &t, uint32_t ref, const float4 *cost, float out[8]) {
    if (ref & kLeafBit) {
        for (int i = 0; i < 8; ++i) out[i] = 0.f;
        return;
    }
    const float4 c0 = __ldcg(cost + 2 * (size_t)ref), c1 = __ldcg(cost + 2 * (size_t)ref + 1);
    out[0] = c0.x; out[1] = c0.y; out[2] = c0.z; out[3] = c0.w;
    out[4] = c1.x; out[5] = c1.y; out[6] = c1.z; out[7] = c1.w;
}

__global__ void k_collapse_cost(int n, BinTree t, const int *__restrict__ par_int,
                                const int *__restrict__ par_leaf, float4 *cost, uint2 *choice, int *flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = par_leaf[i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;
        __threadfence();
        float cl[8], cr[8], d[9], c[8];
        int arg[9];
        cost_table(t, t.left[node], cost, cl);
        cost_table(t, t.right[node], cost, cr);
        for (int w = 2; w <= 8; ++w) {
            d[w] = INFINITY;
            arg[w] = 1;
            for (int k = 1; k < w; ++k) {
                const float v = cl[k - 1] + cr[w - k - 1];
                if (v < d[w]) { d[w] = v; arg[w] = k; }
            }
        }
        c[0] = half_area(f3(t.int_lo[node]), f3(t.int_hi[node])) + d[8];
        uint32_t word[2] = {(uint32_t)arg[8], 0u};
        for (int w = 2; w <= 8; ++w) {
            uint32_t k = 0;
            if (d[w] < c[w - 2]) { c[w - 1] = d[w]; k = (uint32_t)arg[w]; }
            else c[w - 1] = c[w - 2];
            word[(w - 1) >> 2] |= k << (8 * ((w - 1) & 3));
        }
        __stcg(cost + 2 * (size_t)node, make_float4(c[0], c[1], c[2], c[3]));
        __stcg(cost + 2 * (size_t)node + 1, make_float4(c[4], c[5], c[6], c[7]));
        choice[node] = make_uint2(word[0], word[1]);
        node = par_int[node];
    }
}

__device__ __forceinline__ uint32_t choice_byte(uint2 w, int b) {
    return ((b < 4 ? w.x : w.y) >> (8 * (b & 3))) & 0xffu;
}

__global__ void k_collapse(BinTree t, const CollapseItem *__restrict__ in, const int *n_in,
                           CollapseItem *out, int *n_out, float4 *nodes, int *node_counter,
                           uint32_t *leaf_order, int *tri_counter, int *max_depth, int format,
                           int max_leaf, int full_leaf, const uint2 *__restrict__ choice) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= *n_in) return;
    CollapseItem item = in[w];

    uint32_t ref[8];
    V3 clo[8], chi[8];
    int ccount[8];
    int nc = 1;
    ref[0] = item.bref;
    ref_info(t, ref[0], clo[0], chi[0], ccount[0]);
    if (choice && !(item.bref & kLeafBit)) {
        // cost-optimal children: D(n, 8) of the node, expanded through the
        // children's choices (the i of the stacked entries sum to at most 8,
        // so at most eight roots come out)
        uint32_t st_ref[8];
        int st_i[8], sp = 0;
        const int k8 = min(max((int)choice_byte(choice[item.bref], 0), 1), 7);
        st_ref[sp] = t.right[item.bref]; st_i[sp++] = 8 - k8;
        st_ref[sp] = t.left[item.bref]; st_i[sp++] = k8;
        nc = 0;
        while (sp > 0) {
            const uint32_t m = st_ref[--sp];
            int i = st_i[sp];
            int k = 0;
            if (!(m & kLeafBit)) {
                const uint2 cw = choice[m];
                while (i > 1 && (k = (int)choice_byte(cw, i - 1)) == 0) --i;
            }
            if (k == 0 || k >= i || nc + sp >= 7) {
                ref[nc] = m;
                ref_info(t, m, clo[nc], chi[nc], ccount[nc]);
                ++nc;
            } else {
                st_ref[sp] = t.right[m]; st_i[sp++] = i - k;
                st_ref[sp] = t.left[m]; st_i[sp++] = k;
            }
        }
    }
    // Greedily open the largest child that cannot be a leaf (more than three
    // triangles) or, once all can be leaves, the largest internal one while
    // slots remain.
    while (!choice && nc < 8) {
        int best = -1;
        float best_area = -1.f;
        bool best_must = false;
        for (int c = 0; c < nc; ++c) {
            if (ref[c] & kLeafBit) continue;
            bool must = ccount[c] > max_leaf;
            float a = half_area(clo[c], chi[c]);
            if ((must && !best_must) || (must == best_must && a > best_area)) {
                best = c; best_area = a; best_must = must;
            }
        }
        if (best < 0 || !best_must) break;
        uint32_t r = ref[best];
        ref[best] = t.left[r];
        ref_info(t, ref[best], clo[best], chi[best], ccount[best]);
        ref[nc] = t.right[r];
        ref_info(t, ref[nc], clo[nc], chi[nc], ccount[nc]);
        ++nc;
    }
    // A child that stays internal becomes a node of its own; in a full node a
    // child of at most `full_leaf` triangles becomes a leaf instead (eight
    // leaves of three triangles still fit the 24-bit triangle mask).
    bool internal[8];
    const int leaf_max = nc == 8 ? full_leaf : max_leaf;
    for (int c = 0; c < nc; ++c) internal[c] = ccount[c] > leaf_max;

    // Node bounds.
    V3 lo = clo[0], hi = chi[0];
    for (int c = 1; c < nc; ++c) { lo = vmin(lo, clo[c]); hi = vmax(hi, chi[c]); }

    // Octant slot assignment: slot s gets the child nearest for direction
    // octant s (greedy on dot(child centre - node centre, dir_s)).  A node of
    // at most four children that are all leaves takes slots 0-3 in child
    // order instead: the order of its children does not matter (every hit
    // triangle is tested), and with slots 4-7 empty the traversal skips
    // their box tests.
    V3 pc = (lo + hi) * 0.5f;
    int slot_of[8];
    int child_in_slot[8];
    for (int s = 0; s < 8; ++s) child_in_slot[s] = -1;
    for (int c = 0; c < nc; ++c) slot_of[c] = -1;
    bool any_internal = false;
    for (int c = 0; c < nc; ++c) any_internal |= internal[c];
    const bool packed = !any_internal && nc <= 4;
    if (packed) {
        for (int c = 0; c < nc; ++c) { slot_of[c] = c; child_in_slot[c] = c; }
    }
    for (int it = 0; it < nc && !packed; ++it) {
        float best = INFINITY;
        int bc = -1, bs = -1;
        for (int c = 0; c < nc; ++c) {
            if (slot_of[c] >= 0) continue;
            V3 d = (clo[c] + chi[c]) * 0.5f - pc;
            for (int s = 0; s < 8; ++s) {
                if (child_in_slot[s] >= 0) continue;
                float cost = ((s & 1) ? -d.x : d.x) + ((s & 2) ? -d.y : d.y) + ((s & 4) ? -d.z : d.z);
                if (cost < best) { best = cost; bc = c; bs = s; }
            }
        }
        if (bc < 0) break;
        slot_of[bc] = bs;
        child_in_slot[bs] = bc;
    }

    // Allocate internal children and leaf triangles.
    int n_int = 0, n_tri = 0;
    for (int c = 0; c < nc; ++c) {
        if (internal[c]) ++n_int;
        else n_tri += ccount[c];
    }
    int child_base = n_int ? atomicAdd(node_counter, n_int) : 0;
    int tri_base = n_tri ? atomicAdd(tri_counter, n_tri) : 0;
    if (n_int) atomicMax(max_depth, item.depth + 1);

    uint32_t meta[2] = {0, 0};
    uint32_t imask = 0;
    int int_rank = 0, tri_off = 0;
    V3 slo[8], shi[8];
    for (int s = 0; s < 8; ++s) {
        int c = child_in_slot[s];
        slo[s] = c >= 0 ? clo[c] : v3(INFINITY);
        shi[s] = c >= 0 ? chi[c] : v3(-INFINITY);
        if (c < 0) continue;
        uint32_t m;
        if (internal[c]) {
            m = 0x20u | (24u + (uint32_t)s);
            imask |= 1u << s;
        } else {
            m = (((1u << ccount[c]) - 1u) << 5) | (uint32_t)tri_off;
            uint32_t tri[3];
            const int nl = subtree_leaves(t, ref[c], tri);
            for (int k = 0; k < nl; ++k) leaf_order[tri_base + tri_off + k] = tri[k];
            tri_off += ccount[c];
        }
        meta[s >> 2] |= m << (8 * (s & 3));
    }
    // internal children in slot order
    for (int s = 0; s < 8; ++s) {
        int c = child_in_slot[s];
        if (c < 0 || !internal[c]) continue;
        int slot = atomicAdd(n_out, 1);
        out[slot] = CollapseItem{ref[c], (uint32_t)(child_base + int_rank), item.depth + 1};
        ++int_rank;
    }

    V3 blo, bhi;
    if (format == 1) {
        float4 *np = nodes + 14 * (size_t)item.wnode;
        write_node_boxes(np, 1, slo, shi, imask, blo, bhi);
        np[12] = make_float4(__uint_as_float((uint32_t)child_base), __uint_as_float((uint32_t)tri_base),
                             __uint_as_float(meta[0]), __uint_as_float(meta[1]));
        np[13] = make_float4(__uint_as_float(imask), 0.f, 0.f, 0.f);
        return;
    }
    float4 *np = nodes + 5 * (size_t)item.wnode;
    write_node_boxes(np, 0, slo, shi, imask, blo, bhi);
    np[1] = make_float4(__uint_as_float((uint32_t)child_base), __uint_as_float((uint32_t)tri_base),
                        __uint_as_float(meta[0]), __uint_as_float(meta[1]));
}

__global__ void k_gather_tris(const float *__restrict__ v, const uint32_t *__restrict__ leaf_order,
                              int64_t n, float4 *tris, uint32_t *leaf_of_prim) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t p = leaf_order[k];
    const float *s = v + 9 * (size_t)p;
    tris[3 * k + 0] = make_float4(s[0], s[1], s[2], __uint_as_float(p));
    tris[3 * k + 1] = make_float4(s[3], s[4], s[5], __uint_as_float(1u));
    tris[3 * k + 2] = make_float4(s[6], s[7], s[8], 0.f);
    leaf_of_prim[p] = (uint32_t)k;
}

__global__ void k_set_mask(float4 *tris, const uint32_t *leaf_of_prim, const uint8_t *mask,
                           int64_t n) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t k = leaf_of_prim[p];
    tris[3 * (size_t)k + 1].w = __uint_as_float(mask ? (uint32_t)(mask[p] != 0) : 1u);
}

// MODE 0: closest hit, 1: any hit, 2: mixed (any-hit set, then closest set).
template <int MODE, bool STATS, int FMT>
__device__ __forceinline__ void trace_body(const float4 *__restrict__ nodes,
                                           const float4 *__restrict__ tris, const TraceLaunch &L,
                                           unsigned long long *stats) {
    const int lane = threadIdx.x & 31;
    // queue counts are clamped to the queue capacity (a queue that overflowed
    // has its flag raised and a count above its storage)
    const int64_t n_any = MODE == 2 ? min((int64_t)*L.d_any_count, L.n) : 0;
    const int64_t n = (L.d_count ? min((int64_t)*L.d_count, L.n) : L.n) + n_any;
    bool any_ray = MODE == 1;
    uint2 stack[kTraversalStack];
    int sp = 0;
    bool active = false, exhausted = false;
    int64_t ray_id = 0;
    RayPre r;
    V3 inv, oinv;
    int oct = 0;
    float tmax = 0.f;
    uint2 ng = make_uint2(0, 0), tg = make_uint2(0, 0);
    float best_b1 = 0.f, best_b2 = 0.f;
    uint32_t best_prim = KRR_MISS;
    unsigned long long n_nodes = 0, n_tris = 0;

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
                    const float4 *po = L.ray_o, *pd = L.ray_d;
                    if (MODE == 2) {
                        any_ray = idx < n_any;
                        if (any_ray) { po = L.any_o; pd = L.any_d; }
                        else idx -= n_any;
                    }
                    ray_id = idx;
                    uint32_t root = 0;
                    if (L.roots) {
                        const float4 *pp = (MODE == 2 && any_ray) ? L.any_pix : L.ray_pix;
                        root = L.roots[L.pixel_part[__float_as_uint(pp[idx * L.ray_stride].w)]];
                    }
                    float4 ro = po[idx * L.ray_stride];
                    float4 rd = pd[idx * L.ray_stride];
                    V3 o = f3(ro), d = f3(rd);
                    r = ray_pre(o, d, ro.w);
                    tmax = rd.w;
                    inv = box_inverse(d);
                    oinv = V3{-o.x * inv.x, -o.y * inv.y, -o.z * inv.z};
                    oct = (inv.x < 0.f ? 1 : 0) | (inv.y < 0.f ? 2 : 0) | (inv.z < 0.f ? 4 : 0);
                    ng = make_uint2(root, (1u << oct) | (1u << 8));
                    tg = make_uint2(0u, 0u);
                    sp = 0;
                    best_prim = KRR_MISS;
                    active = true;
                }
            }
            act = __ballot_sync(0xffffffffu, active);
        }
        if (act == 0) break;

        // ---- one traversal step, all lanes together: optional node visit,
        // triangles (possibly postponed), pop
        bool done = false, fresh = false;
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
            if (STATS) ++n_nodes;
            visit<FMT>(nodes, child, r, inv, oinv, oct, tmax, ng, tg);
            fresh = true;
        }
        // Postpone a fresh triangle group onto the stack while too few lanes
        // of the warp have triangles to test (keeps the warp on node work).
        if (L.postpone_pct > 0) {
            unsigned tri_lanes = __ballot_sync(0xffffffffu, active && tg.y != 0u);
            if (active && fresh && tg.y && __popc(tri_lanes) * 100 < L.postpone_pct * __popc(act) &&
                (ng.y & 0xffu) && sp < L.stack_limit) {
                stack[sp++] = make_uint2(tg.x, tg.y | 0x80000000u);
                tg.y = 0;
            }
        }
        while (active && tg.y && !done) {
            int b = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const float4 *tp = tris + 3 * (size_t)(tg.x + b);
            float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
            if (STATS) ++n_tris;
            float b1, b2;
            float t = tri_test(r, v0, v1, v2, b1, b2);
            uint32_t gid = __float_as_uint(v0.w);
            if (any_ray) {
                if (t > r.tmin && t <= tmax && __float_as_uint(v1.w) != 0u) {
                    best_prim = gid;
                    done = true;
                }
            } else {
                if (t > r.tmin && (t < tmax || (t == tmax && gid < best_prim))) {
                    tmax = t; best_b1 = b1; best_b2 = b2; best_prim = gid;
                }
            }
        }
        if (active && !done && !(ng.y & 0xffu) && tg.y == 0u) {
            if (sp > 0) {
                uint2 e = stack[--sp];
                if (e.y & 0x80000000u) tg = make_uint2(e.x, e.y & 0x00ffffffu);
                else ng = e;
            } else {
                done = true;
            }
        }
        if (!active) continue;
        if (done) {
            // a ray cut off by the stack limit: occluded = 0xFF (counted as
            // blocked), or a miss record with t = NaN
            if (any_ray) {
                L.occluded[ray_id] = best_prim == kCutRay ? 0xFF : (best_prim != KRR_MISS ? 1 : 0);
            } else {
                float4 h = best_prim < kCutRay
                               ? make_float4(tmax, best_b1, best_b2, __uint_as_float(best_prim))
                               : make_float4(best_prim == kCutRay ? __int_as_float(0x7fffffff) : INFINITY,
                                             0.f, 0.f, __uint_as_float(KRR_MISS));
                L.hits[ray_id] = h;
            }
            active = false;
        }
    }
    if (STATS) {
        atomicAdd(stats, n_nodes);
        atomicAdd(stats + 1, n_tris);
    }
}

// FMT: 0 compressed nodes, 1 float nodes, 2 compressed nodes whose leaf
// children all hold one triangle (the default build; a simpler child mask).
// Compressed nodes: eight blocks per SM (64 registers, no spills); the float
// node format keeps the compiler's register choice.
template <int MODE, bool STATS, int FMT>
__global__ void __launch_bounds__(kTraceThreads, FMT != 1 ? 8 : 1)
k_trace(const float4 *__restrict__ nodes, const float4 *__restrict__ tris, TraceLaunch L,
        unsigned long long *stats) {
    trace_body<MODE, STATS, FMT>(nodes, tris, L, stats);
}

// The mixed launch is held to the closest-hit kernel's 8 blocks per SM (the
// grid is sized for that occupancy).
template <int FMT>
__global__ void __launch_bounds__(kTraceThreads, FMT != 1 ? 8 : 1)
k_trace_mixed(const float4 *__restrict__ nodes, const float4 *__restrict__ tris, TraceLaunch L) {
    trace_body<2, false, FMT>(nodes, tris, L, nullptr);
}

int g_grid_size = 0;

// An empty scene: every ray misses (MODE as k_trace).
__global__ void k_all_miss(TraceLaunch L, int mode) {
    const int64_t n_any = mode == 2 ? min((int64_t)*L.d_any_count, L.n) : 0;
    const int64_t n = (L.d_count ? min((int64_t)*L.d_count, L.n) : L.n) + n_any;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bool any = mode == 1 || (mode == 2 && i < n_any);
        if (any) L.occluded[i] = 0;
        else L.hits[mode == 2 ? i - n_any : i] = make_float4(INFINITY, 0.f, 0.f, __uint_as_float(KRR_MISS));
    }
}

}  // namespace

int traversal_grid_size() {
    if (g_grid_size) return g_grid_size;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<0, false, 2>, kTraceThreads, 0);
    if (per_sm < 1) per_sm = 1;
    g_grid_size = sms * per_sm;
    return g_grid_size;
}

template <int MODE, bool STATS>
static int launch_trace(const krr_accel *a, const TraceLaunch &l, cudaStream_t s,
                        unsigned long long *stats = nullptr) {
    if (!a || !a->d_scratch) return fail(KRR_ERR_NOT_READY, "acceleration structure not built");
    KRR_CUDA(cudaMemsetAsync(l.counter, 0, sizeof(unsigned long long), s));
    if (a->n_tris == 0) {
        k_all_miss<<<traversal_grid_size(), kTraceThreads, 0, s>>>(l, MODE);
        KRR_CUDA(cudaGetLastError());
        return KRR_OK;
    }
    TraceLaunch lt = l;
    lt.refill_below = a->refill_below;
    lt.postpone_pct = a->postpone_pct;
    lt.stack_limit = a->stack_limit;
    if (a->levels == 2) {
        KRR_CHECK_ARG(!STATS, "the counter replay takes a one-level structure");
        return launch_trace_instanced(a, lt, MODE, s);
    }
    const int grid = traversal_grid_size();
    const bool single = a->max_leaf == 1 && a->full_leaf == 1;
    if constexpr (MODE == 2) {
        if (a->node_format == 1)
            k_trace_mixed<1><<<grid, kTraceThreads, 0, s>>>(a->d_nodes, a->d_tris, lt);
        else if (single)
            k_trace_mixed<2><<<grid, kTraceThreads, 0, s>>>(a->d_nodes, a->d_tris, lt);
        else
            k_trace_mixed<0><<<grid, kTraceThreads, 0, s>>>(a->d_nodes, a->d_tris, lt);
    } else {
        if (a->node_format == 1)
            k_trace<MODE, STATS, 1><<<grid, kTraceThreads, 0, s>>>(a->d_nodes, a->d_tris, lt, stats);
        else if (single)
            k_trace<MODE, STATS, 2><<<grid, kTraceThreads, 0, s>>>(a->d_nodes, a->d_tris, lt, stats);
        else
            k_trace<MODE, STATS, 0><<<grid, kTraceThreads, 0, s>>>(a->d_nodes, a->d_tris, lt, stats);
    }
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

int launch_trace_closest(const krr_accel *a, const TraceLaunch &l, cudaStream_t s) {
    return launch_trace<0, false>(a, l, s);
}
int launch_trace_any(const krr_accel *a, const TraceLaunch &l, cudaStream_t s) {
    return launch_trace<1, false>(a, l, s);
}
int launch_trace_mixed(const krr_accel *a, const TraceLaunch &l, cudaStream_t s) {
    return launch_trace<2, false>(a, l, s);
}
int launch_trace_stats(const krr_accel *a, const TraceLaunch &l, bool any,
                       unsigned long long *d_stats, cudaStream_t s) {
    return any ? launch_trace<1, true>(a, l, s, d_stats) : launch_trace<0, true>(a, l, s, d_stats);
}

void accel_free(krr_accel *a) {
    if (!a) return;
    cudaFree(a->d_nodes);
    cudaFree(a->d_tris);
    cudaFree(a->d_leaf_of_prim);
    cudaFree(a->d_scratch);
    cudaFree(a->stage_rays);
    cudaFree(a->stage_hits);
    cudaFree(a->d_node_bounds);
    cudaFree(a->d_roots);
    cudaFree(a->d_inst);
    a->d_inst = nullptr;
    for (krr_accel *sub : {a->tlas, a->blas})
        if (sub) { accel_free(sub); delete sub; }
    a->tlas = a->blas = nullptr;
    a->levels = 1;
    a->h_inst.clear();
    a->geom_begin.clear();
    a->inst_geom.clear();
    a->inst_xf.clear();
    a->inst_mask.clear();
    a->inst_first.clear();
    a->inst_triangles = 0;
    a->d_node_bounds = nullptr;
    a->d_roots = nullptr;
    a->roots.clear();
    a->part_bounds.clear();
    a->level_first.clear();
    if (a->stage_aux) cudaStreamDestroy(a->stage_aux);
    for (cudaEvent_t &e : a->stage_ev)
        if (e) cudaEventDestroy(e);
    a->d_nodes = nullptr;
    a->d_tris = nullptr;
    a->d_leaf_of_prim = nullptr;
    a->d_scratch = nullptr;
    a->stage_rays = a->stage_hits = nullptr;
    a->stage_cap = 0;
    a->stage_aux = nullptr;
    a->stage_ev[0] = a->stage_ev[1] = nullptr;
}

namespace {
template <typename T>
struct DevBuf {
    T *p = nullptr;
    ~DevBuf() { cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};
inline unsigned blocks_for(int64_t n, int t = kBuildThreads) { return (unsigned)((n + t - 1) / t); }
}  // namespace

// New vertex positions into the leaf-ordered triangle records (the id and
// mask words are kept).
__global__ void k_refit_tris(const float *__restrict__ v, int64_t n,
                             const uint32_t *__restrict__ leaf_of_prim, float4 *tris) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float *s = v + 9 * (size_t)p;
    float4 *t = tris + 3 * (size_t)leaf_of_prim[p];
    for (int j = 0; j < 3; ++j) {
        float4 q = t[j];
        q.x = s[3 * j]; q.y = s[3 * j + 1]; q.z = s[3 * j + 2];
        t[j] = q;
    }
}

// Refit of the nodes [first, first + count) of one tree level, children
// refitted before: a leaf child's box is the box of its triangles widened by
// `margin` (as the build's leaf boxes), an internal child's box the bounds of
// its node; quantised by write_node_boxes as the build does.  Topology,
// slots and child/triangle offsets are kept.
template <int FMT>
__global__ void k_refit_level(float4 *nodes, const float4 *__restrict__ tris, float4 *bounds,
                              int first, int count, float margin) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int w = first + i;
    float4 *np = nodes + (FMT == 1 ? 14 : 5) * (size_t)w;
    uint32_t child_base, tri_base, meta0, meta1, imask;
    if (FMT == 1) {
        const float4 q12 = np[12], q13 = np[13];
        child_base = __float_as_uint(q12.x); tri_base = __float_as_uint(q12.y);
        meta0 = __float_as_uint(q12.z); meta1 = __float_as_uint(q12.w);
        imask = __float_as_uint(q13.x);
    } else {
        const float4 q0 = np[0], q1 = np[1];
        child_base = __float_as_uint(q1.x); tri_base = __float_as_uint(q1.y);
        meta0 = __float_as_uint(q1.z); meta1 = __float_as_uint(q1.w);
        imask = __float_as_uint(q0.w) >> 24;
    }
    V3 slo[8], shi[8];
    for (int s = 0; s < 8; ++s) {
        const uint32_t m = ((s < 4 ? meta0 : meta1) >> (8 * (s & 3))) & 0xffu;
        slo[s] = v3(INFINITY);
        shi[s] = v3(-INFINITY);
        if (imask & (1u << s)) {
            const uint32_t c = child_base + __popc(imask & ((1u << s) - 1u));
            slo[s] = f3(bounds[2 * (size_t)c]);
            shi[s] = f3(bounds[2 * (size_t)c + 1]);
        } else if (m) {
            const uint32_t cnt = __popc(m >> 5), off = m & 31u;
            V3 lo = v3(INFINITY), hi = v3(-INFINITY);
            for (uint32_t k = 0; k < cnt; ++k) {
                const float4 *t = tris + 3 * (size_t)(tri_base + off + k);
                for (int j = 0; j < 3; ++j) {
                    V3 p = f3(t[j]);
                    lo = vmin(lo, p);
                    hi = vmax(hi, p);
                }
            }
            slo[s] = lo - v3(margin);
            shi[s] = hi + v3(margin);
        }
    }
    V3 lo, hi;
    write_node_boxes(np, FMT, slo, shi, imask, lo, hi);
    bounds[2 * (size_t)w] = make_float4(lo.x, lo.y, lo.z, 0.f);
    bounds[2 * (size_t)w + 1] = make_float4(hi.x, hi.y, hi.z, 0.f);
}

// Scene bounds of device vertices (into a->scene_lo/hi) and the margin that
// keeps quantised boxes conservative: a few float ulps of the largest
// coordinate magnitude and of the scene extent.
static int scene_bounds_margin(krr_accel *a, const float *d_v, int64_t n, cudaStream_t s,
                               DevBuf<float> &bounds, float *margin) {
    KRR_CUDA(bounds.alloc(12));
    float init[12] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY,
                      INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    KRR_CUDA(cudaMemcpyAsync(bounds.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
    k_scene_bounds<<<std::min<unsigned>(blocks_for(n), 4096), kBuildThreads, 0, s>>>(d_v, n, bounds.p);
    KRR_CUDA(cudaGetLastError());
    float hb[12];
    KRR_CUDA(cudaMemcpyAsync(hb, bounds.p, sizeof(hb), cudaMemcpyDeviceToHost, s));
    KRR_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < 3; ++k) { a->scene_lo[k] = hb[6 + k]; a->scene_hi[k] = hb[9 + k]; }
    for (int k = 6; k < 12; ++k)
        if (!std::isfinite(hb[k])) return fail(KRR_ERR_INVALID_ARGUMENT, "triangle vertices are not finite");
    float mag = 0.f, ext = 0.f;
    for (int k = 0; k < 3; ++k) {
        mag = std::max(mag, std::max(std::fabs(hb[6 + k]), std::fabs(hb[9 + k])));
        ext = std::max(ext, hb[9 + k] - hb[6 + k]);
    }
    *margin = std::ldexp(mag + ext, -19) + 1e-30f;
    return KRR_OK;
}

int accel_refit(krr_accel *a, const float *d_v, int64_t n, cudaStream_t s) {
    KRR_CHECK_ARG(a && a->d_scratch, "acceleration structure not built");
    KRR_CHECK_ARG(n == a->n_tris, "a refit keeps the triangle count of the build");
    KRR_CHECK_ARG(a->roots.empty(), "a structure of several scenes is rebuilt, not refitted");
    KRR_CHECK_ARG(a->levels == 1, "a two-level structure updates its instances instead");
    if (n == 0) return KRR_OK;
    KRR_CHECK_ARG(d_v != nullptr, "vertices are NULL");
    float margin = 0.f;
    DevBuf<float> bounds;
    KRR_TRY(scene_bounds_margin(a, d_v, n, s, bounds, &margin));
    if (!a->d_node_bounds) KRR_CUDA(cudaMalloc(&a->d_node_bounds, 2 * sizeof(float4) * a->n_nodes));
    k_refit_tris<<<blocks_for(n), kBuildThreads, 0, s>>>(d_v, n, a->d_leaf_of_prim, a->d_tris);
    KRR_CUDA(cudaGetLastError());
    const std::vector<int32_t> &lf = a->level_first;
    for (int L = (int)lf.size() - 1; L >= 1; --L) {
        const int first = lf[L - 1], count = lf[L] - lf[L - 1];
        if (count <= 0) continue;
        if (a->node_format == 1)
            k_refit_level<1><<<blocks_for(count, 128), 128, 0, s>>>(a->d_nodes, a->d_tris, a->d_node_bounds,
                                                                     first, count, margin);
        else
            k_refit_level<0><<<blocks_for(count, 128), 128, 0, s>>>(a->d_nodes, a->d_tris, a->d_node_bounds,
                                                                     first, count, margin);
        KRR_CUDA(cudaGetLastError());
    }
    return KRR_OK;
}

// krr_set_bvh_collapse: how the binary tree becomes 8-wide nodes (0 greedy,
// 1 cost-optimal).
static int g_collapse = 0;

// PLOC rounds over the Morton-ordered leaves until one cluster is left (its
// ref is the root).  Internal nodes are numbered in creation order.
static int build_ploc(int n, const float4 *leaf_lo, const float4 *leaf_hi, uint32_t *left,
                      uint32_t *right, int *count, float4 *int_lo, float4 *int_hi,
                      uint32_t *root_ref, cudaStream_t s) {
    DevBuf<Cluster> ca, cb;
    DevBuf<uint32_t> nn;
    DevBuf<uint8_t> keep;
    DevBuf<int> counters;   // [0] node counter, [1] clusters kept
    KRR_CUDA(ca.alloc(n)); KRR_CUDA(cb.alloc(n)); KRR_CUDA(nn.alloc(n)); KRR_CUDA(keep.alloc(n));
    KRR_CUDA(counters.alloc(2));
    KRR_CUDA(cudaMemsetAsync(counters.p, 0, 2 * sizeof(int), s));
    size_t tmp_bytes = 0;
    KRR_CUDA(cub::DeviceSelect::Flagged(nullptr, tmp_bytes, cb.p, keep.p, ca.p, counters.p + 1, n, s));
    DevBuf<uint8_t> tmp;
    KRR_CUDA(tmp.alloc(tmp_bytes));
    k_ploc_init<<<blocks_for(n), kBuildThreads, 0, s>>>(n, leaf_lo, leaf_hi, ca.p);
    KRR_CUDA(cudaGetLastError());
    int m = n, rounds = 0;
    while (m > 1) {
        const int r = std::min(kPlocRadius, m - 1);
        k_ploc_nn<<<blocks_for(m, kPlocThreads), kPlocThreads, 0, s>>>(ca.p, m, r, nn.p);
        k_ploc_merge<<<blocks_for(m), kBuildThreads, 0, s>>>(ca.p, nn.p, m, cb.p, keep.p, left, right,
                                                            count, int_lo, int_hi, counters.p);
        KRR_CUDA(cudaGetLastError());
        KRR_CUDA(cub::DeviceSelect::Flagged(tmp.p, tmp_bytes, cb.p, keep.p, ca.p, counters.p + 1, m, s));
        int kept = m;
        KRR_CUDA(cudaMemcpyAsync(&kept, counters.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        KRR_CUDA(cudaStreamSynchronize(s));
        if (kept >= m || kept < 1 || ++rounds > 100000)
            return fail(KRR_ERR_OVERFLOW, "PLOC clustering made no progress (%d clusters)", m);
        m = kept;
    }
    Cluster root{};
    KRR_CUDA(cudaMemcpyAsync(&root, ca.p, sizeof(Cluster), cudaMemcpyDeviceToHost, s));
    KRR_CUDA(cudaStreamSynchronize(s));
    std::memcpy(root_ref, &root.lo.w, sizeof(uint32_t));
    return KRR_OK;
}

static int build_tree(krr_accel *a, const float *d_v, int64_t n, cudaStream_t s, int treelets) {
    KRR_CHECK_ARG(n >= 0 && n < (int64_t)0x7fffffff, "triangle count out of range");
    accel_free(a);
    a->node_format = default_node_format();
    a->max_leaf = default_max_leaf();
    a->full_leaf = std::max(a->max_leaf, default_full_leaf());
    a->n_tris = n;
    a->n_nodes = 0;
    a->max_depth = 0;
    KRR_CUDA(cudaMalloc(&a->d_scratch, 64));
    KRR_CUDA(cudaMemsetAsync(a->d_scratch, 0, 64, s));
    if (n == 0) return KRR_OK;

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);

    // scene bounds (centroid bounds first, for the Morton codes) and the
    // conservative-box margin
    float margin = 0.f;
    DevBuf<float> bounds;
    KRR_TRY(scene_bounds_margin(a, d_v, n, s, bounds, &margin));

    DevBuf<uint64_t> keys, keys2;
    DevBuf<uint32_t> vals, vals2;
    DevBuf<float4> tlo, thi, llo, lhi, ilo, ihi;
    KRR_CUDA(keys.alloc(n)); KRR_CUDA(keys2.alloc(n));
    KRR_CUDA(vals.alloc(n)); KRR_CUDA(vals2.alloc(n));
    KRR_CUDA(tlo.alloc(n)); KRR_CUDA(thi.alloc(n));
    a->builder = default_builder();
    k_leaf_setup<<<blocks_for(n), kBuildThreads, 0, s>>>(d_v, n, bounds.p, margin, a->builder != 0,
                                                          keys.p, vals.p, tlo.p, thi.p);
    KRR_CUDA(cudaGetLastError());

    // sort by Morton code
    {
        size_t tmp_bytes = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.p, keys2.p, vals.p, vals2.p, (int)n,
                                        0, 63, s);
        DevBuf<uint8_t> tmp;
        KRR_CUDA(tmp.alloc(tmp_bytes));
        KRR_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.p, keys2.p, vals.p, vals2.p,
                                                 (int)n, 0, 63, s));
    }
    const uint64_t *skeys = keys2.p;
    const uint32_t *sidx = vals2.p;

    KRR_CUDA(llo.alloc(n)); KRR_CUDA(lhi.alloc(n));
    k_gather_leaf_boxes<<<blocks_for(n), kBuildThreads, 0, s>>>(sidx, (int)n, tlo.p, thi.p, llo.p, lhi.p);
    KRR_CUDA(cudaGetLastError());

    int64_t ni = std::max<int64_t>(n - 1, 1);
    DevBuf<uint32_t> left, right;
    DevBuf<int> count;
    KRR_CUDA(left.alloc(ni)); KRR_CUDA(right.alloc(ni)); KRR_CUDA(count.alloc(ni));
    KRR_CUDA(ilo.alloc(ni)); KRR_CUDA(ihi.alloc(ni));
    uint32_t root_ref = kLeafBit | 0u;
    if (n > 1 && a->builder == 1) {
        KRR_TRY(build_ploc((int)n, llo.p, lhi.p, left.p, right.p, count.p, ilo.p, ihi.p, &root_ref, s));
    } else if (n > 1) {
        DevBuf<int> par_int, par_leaf, flags;
        KRR_CUDA(par_int.alloc(ni)); KRR_CUDA(par_leaf.alloc(n)); KRR_CUDA(flags.alloc(ni));
        KRR_CUDA(cudaMemsetAsync(flags.p, 0, ni * sizeof(int), s));
        k_karras<<<blocks_for(n - 1), kBuildThreads, 0, s>>>(skeys, (int)n, left.p, right.p, count.p,
                                                              par_int.p, par_leaf.p);
        KRR_CUDA(cudaGetLastError());
        k_bottom_up<<<blocks_for(n), kBuildThreads, 0, s>>>((int)n, left.p, right.p, par_int.p,
                                                             par_leaf.p, llo.p, lhi.p, ilo.p, ihi.p,
                                                             flags.p);
        KRR_CUDA(cudaGetLastError());
        root_ref = 0;
        KRR_CUDA(cudaStreamSynchronize(s));   // the scratch above is freed on return
    }

    // treelet restructuring passes over the binary tree
    a->treelets = n > 2 ? treelets : 0;
    if (a->treelets > 0) {
        DevBuf<int> par_int, par_leaf, flags;
        KRR_CUDA(par_int.alloc(ni)); KRR_CUDA(par_leaf.alloc(n)); KRR_CUDA(flags.alloc(ni));
        for (int pass = 0; pass < a->treelets; ++pass) {
            KRR_CUDA(cudaMemsetAsync(flags.p, 0, ni * sizeof(int), s));
            KRR_CUDA(cudaMemsetAsync(par_int.p, 0xff, ni * sizeof(int), s));   // the root's parent: -1
            k_parents<<<blocks_for(n - 1), kBuildThreads, 0, s>>>((int)(n - 1), left.p, right.p,
                                                                   par_int.p, par_leaf.p);
            k_treelet<<<blocks_for(n), kBuildThreads, 0, s>>>((int)n, left.p, right.p, count.p, par_int.p,
                                                               par_leaf.p, ilo.p, ihi.p, llo.p, lhi.p,
                                                               flags.p, kTreeletMinCount);
            KRR_CUDA(cudaGetLastError());
        }
        KRR_CUDA(cudaStreamSynchronize(s));   // the scratch above is freed on return
    }

    BinTree bt{left.p, right.p, count.p, ilo.p, ihi.p, llo.p, lhi.p, sidx};
    // cost tables of the cost-optimal collapse (one-triangle leaves only)
    DevBuf<uint2> choice;
    a->collapse = g_collapse == 1 && a->max_leaf == 1 && a->full_leaf == 1 && n > 1 ? 1 : 0;
    if (a->collapse) {
        DevBuf<int> par_int, par_leaf, flags;
        DevBuf<float4> cost;
        KRR_CUDA(par_int.alloc(ni)); KRR_CUDA(par_leaf.alloc(n)); KRR_CUDA(flags.alloc(ni));
        KRR_CUDA(cost.alloc(2 * ni)); KRR_CUDA(choice.alloc(ni));
        KRR_CUDA(cudaMemsetAsync(flags.p, 0, ni * sizeof(int), s));
        KRR_CUDA(cudaMemsetAsync(par_int.p, 0xff, ni * sizeof(int), s));   // the root's parent: -1
        k_parents<<<blocks_for(n - 1), kBuildThreads, 0, s>>>((int)(n - 1), left.p, right.p, par_int.p,
                                                               par_leaf.p);
        k_collapse_cost<<<blocks_for(n), kBuildThreads, 0, s>>>((int)n, bt, par_int.p, par_leaf.p, cost.p,
                                                                 choice.p, flags.p);
        KRR_CUDA(cudaGetLastError());
        KRR_CUDA(cudaStreamSynchronize(s));   // the scratch above is freed on return
    }

    // collapse, level by level
    int64_t max_nodes = std::max<int64_t>(n, 2);
    DevBuf<float4> nodes_tmp;
    DevBuf<uint32_t> leaf_order;
    DevBuf<CollapseItem> qa, qb;
    DevBuf<int> counters;   // [0] node counter, [1] tri counter, [2] max depth, [3] n_in, [4] n_out
    const int fmt = a->node_format;
    const int quads = kNodeQuads[fmt];
    KRR_CUDA(nodes_tmp.alloc(quads * max_nodes));
    KRR_CUDA(leaf_order.alloc(n));
    KRR_CUDA(qa.alloc(max_nodes)); KRR_CUDA(qb.alloc(max_nodes));
    KRR_CUDA(counters.alloc(8));
    int hc[8];
    for (int attempt = 0;; ++attempt) {
        const int init[8] = {1, 0, 0, 1, 0, 0, 0, 0};
        std::memcpy(hc, init, sizeof(hc));
        KRR_CUDA(cudaMemcpyAsync(counters.p, hc, sizeof(hc), cudaMemcpyHostToDevice, s));
        CollapseItem root{root_ref, 0u, 1};
        KRR_CUDA(cudaMemcpyAsync(qa.p, &root, sizeof(root), cudaMemcpyHostToDevice, s));
        int n_in = 1;
        a->level_first.assign({0, 1});
        CollapseItem *qin = qa.p, *qout = qb.p;
        int *c_in = counters.p + 3, *c_out = counters.p + 4;
        int levels = 0;
        while (n_in > 0) {
            KRR_CUDA(cudaMemsetAsync(c_out, 0, sizeof(int), s));
            k_collapse<<<blocks_for(n_in, 128), 128, 0, s>>>(bt, qin, c_in, qout, c_out, nodes_tmp.p,
                                                             counters.p, leaf_order.p, counters.p + 1,
                                                             counters.p + 2, fmt, a->max_leaf, a->full_leaf,
                                                             a->collapse ? choice.p : nullptr);
            KRR_CUDA(cudaGetLastError());
            int allocated = 0;
            KRR_CUDA(cudaMemcpyAsync(&n_in, c_out, sizeof(int), cudaMemcpyDeviceToHost, s));
            KRR_CUDA(cudaMemcpyAsync(&allocated, counters.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            KRR_CUDA(cudaMemcpyAsync(c_in, c_out, sizeof(int), cudaMemcpyDeviceToDevice, s));
            KRR_CUDA(cudaStreamSynchronize(s));
            if (n_in > 0) a->level_first.push_back(allocated);   // the next level's nodes end here
            std::swap(qin, qout);
            if (++levels > 4096) return fail(KRR_ERR_OVERFLOW, "BVH collapse did not terminate");
        }
        KRR_CUDA(cudaMemcpyAsync(hc, counters.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
        KRR_CUDA(cudaStreamSynchronize(s));
        // a cost-optimal tree deeper than the traversal stack (possible on
        // degenerate input, where nodes of two children can chain) is
        // replaced by the greedy collapse, whose nodes open three levels
        if (a->collapse && hc[2] > kTraversalStack && attempt == 0) {
            a->collapse = 0;
            continue;
        }
        break;
    }
    a->n_nodes = hc[0];
    a->max_depth = hc[2];
    if (hc[1] != n) return fail(KRR_ERR_OVERFLOW, "BVH collapse emitted %d of %lld triangles", hc[1], (long long)n);
    if (a->max_depth > kTraversalStack)
        return fail(KRR_ERR_OVERFLOW, "BVH depth %d exceeds the traversal stack (%d)", a->max_depth,
                    kTraversalStack);

    KRR_CUDA(cudaMalloc(&a->d_nodes, quads * sizeof(float4) * a->n_nodes));
    KRR_CUDA(cudaMemcpyAsync(a->d_nodes, nodes_tmp.p, quads * sizeof(float4) * a->n_nodes,
                             cudaMemcpyDeviceToDevice, s));
    KRR_CUDA(cudaMalloc(&a->d_tris, 3 * sizeof(float4) * n));
    KRR_CUDA(cudaMalloc(&a->d_leaf_of_prim, sizeof(uint32_t) * n));
    k_gather_tris<<<blocks_for(n), kBuildThreads, 0, s>>>(d_v, leaf_order.p, n, a->d_tris,
                                                           a->d_leaf_of_prim);
    KRR_CUDA(cudaGetLastError());
    cudaEventRecord(e1, s);
    KRR_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    a->build_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return KRR_OK;
}

// Treelet passes of the BVHs built from now on (krr_set_bvh_treelets).
static int g_treelets = 0;

int accel_build(krr_accel *a, const float *d_v, int64_t n, cudaStream_t s) {
    int st = build_tree(a, d_v, n, s, g_treelets);
    // a restructured tree deeper than the traversal stack (possible on
    // degenerate input) is built again without restructuring
    if (st == KRR_ERR_OVERFLOW && g_treelets > 0 && a->max_depth > kTraversalStack)
        st = build_tree(a, d_v, n, s, 0);
    return st;
}

// Relocation of one part's tree into the combined arrays: child and
// triangle base indices move by the part's node and triangle offsets, the
// triangle ids by the part's first global id.
__global__ void k_relocate_nodes(float4 *nodes, int64_t n, int quads, int ref_quad, uint32_t node_off,
                                 uint32_t tri_off) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 *q = nodes + quads * (size_t)i + ref_quad;
    float4 v = *q;
    v.x = __uint_as_float(__float_as_uint(v.x) + node_off);
    v.y = __uint_as_float(__float_as_uint(v.y) + tri_off);
    *q = v;
}

__global__ void k_relocate_tris(float4 *tris, uint32_t *leaf_of_prim, int64_t n, uint32_t id_off) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    float4 v0 = tris[3 * (size_t)k];
    v0.w = __uint_as_float(__float_as_uint(v0.w) + id_off);
    tris[3 * (size_t)k] = v0;
    leaf_of_prim[k] += id_off;   // the part's local slot -> combined slot (same offset)
}

// A node with every slot empty (inverted boxes): the root of a part without
// triangles, which every ray misses.
__global__ void k_empty_node(float4 *np, int format) {
    V3 slo[8], shi[8];
    for (int k = 0; k < 8; ++k) { slo[k] = v3(INFINITY); shi[k] = v3(-INFINITY); }
    V3 lo, hi;
    write_node_boxes(np, format, slo, shi, 0u, lo, hi);
    const float4 refs = make_float4(0.f, 0.f, 0.f, 0.f);
    if (format == 1) { np[12] = refs; np[13] = refs; }
    else {
        np[0] = make_float4(0.f, 0.f, 0.f, __uint_as_float(127u | (127u << 8) | (127u << 16)));
        np[1] = refs;
    }
}

int accel_set_mask(krr_accel *a, const uint8_t *d_mask, cudaStream_t s) {
    if (a->n_tris == 0) return KRR_OK;
    k_set_mask<<<blocks_for(a->n_tris), kBuildThreads, 0, s>>>(a->d_tris, a->d_leaf_of_prim, d_mask,
                                                               a->n_tris);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

int accel_build_parts(krr_accel *a, const float *d_v, const int64_t *part_begin, int n_parts,
                      cudaStream_t s) {
    KRR_CHECK_ARG(n_parts >= 1 && n_parts <= 255, "1..255 scene parts");
    const int64_t n = part_begin[n_parts] - part_begin[0];
    if (n_parts == 1) {
        KRR_TRY(accel_build(a, d_v, n, s));
        a->part_bounds.assign({a->scene_lo[0], a->scene_lo[1], a->scene_lo[2], a->scene_hi[0],
                               a->scene_hi[1], a->scene_hi[2]});
        return KRR_OK;
    }
    std::vector<krr_accel> parts(n_parts);
    int st = KRR_OK;
    for (int p = 0; p < n_parts && st == KRR_OK; ++p)
        st = accel_build(&parts[p], d_v + 9 * (size_t)part_begin[p], part_begin[p + 1] - part_begin[p], s);
    auto release = [&]() { for (auto &q : parts) accel_free(&q); };
    if (st != KRR_OK) { release(); return st; }
    accel_free(a);
    a->node_format = parts[0].node_format;
    a->max_leaf = parts[0].max_leaf;
    a->full_leaf = parts[0].full_leaf;
    a->builder = parts[0].builder;
    const int quads = kNodeQuads[a->node_format];
    int64_t n_nodes = 0;
    a->roots.assign(n_parts, 0);
    for (int p = 0; p < n_parts; ++p) {
        a->roots[p] = (uint32_t)n_nodes;
        n_nodes += parts[p].n_tris ? parts[p].n_nodes : 1;   // an empty part gets an empty node
    }
    a->n_tris = n;
    a->n_nodes = n_nodes;
    a->max_depth = 0;
    a->build_ms = 0.0;
    for (int k = 0; k < 3; ++k) { a->scene_lo[k] = INFINITY; a->scene_hi[k] = -INFINITY; }
    a->part_bounds.assign(6 * (size_t)n_parts, 0.f);
    for (int p = 0; p < n_parts; ++p)
        if (parts[p].n_tris)
            for (int k = 0; k < 3; ++k) {
                a->part_bounds[6 * p + k] = parts[p].scene_lo[k];
                a->part_bounds[6 * p + 3 + k] = parts[p].scene_hi[k];
            }
    auto check = [&](cudaError_t e, const char *what) {
        if (st == KRR_OK && e != cudaSuccess) st = cuda_status(e, what, __FILE__, __LINE__);
    };
    check(cudaMalloc(&a->d_scratch, 64), "cudaMalloc");
    if (st == KRR_OK) check(cudaMemsetAsync(a->d_scratch, 0, 64, s), "cudaMemsetAsync");
    check(cudaMalloc(&a->d_nodes, quads * sizeof(float4) * (size_t)n_nodes), "cudaMalloc");
    check(cudaMalloc(&a->d_tris, 3 * sizeof(float4) * (size_t)std::max<int64_t>(n, 1)), "cudaMalloc");
    check(cudaMalloc(&a->d_leaf_of_prim, sizeof(uint32_t) * (size_t)std::max<int64_t>(n, 1)), "cudaMalloc");
    check(cudaMalloc(&a->d_roots, sizeof(uint32_t) * n_parts), "cudaMalloc");
    for (int p = 0; p < n_parts && st == KRR_OK; ++p) {
        const krr_accel &q = parts[p];
        const int64_t tri0 = part_begin[p] - part_begin[0];
        float4 *nodes = a->d_nodes + quads * (size_t)a->roots[p];
        a->max_depth = std::max(a->max_depth, q.max_depth);
        a->build_ms += q.build_ms;
        if (q.n_tris == 0) {
            k_empty_node<<<1, 1, 0, s>>>(nodes, a->node_format);
            check(cudaGetLastError(), "k_empty_node");
            continue;
        }
        for (int k = 0; k < 3; ++k) {
            a->scene_lo[k] = std::min(a->scene_lo[k], q.scene_lo[k]);
            a->scene_hi[k] = std::max(a->scene_hi[k], q.scene_hi[k]);
        }
        check(cudaMemcpyAsync(nodes, q.d_nodes, quads * sizeof(float4) * (size_t)q.n_nodes,
                              cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        check(cudaMemcpyAsync(a->d_tris + 3 * (size_t)tri0, q.d_tris, 3 * sizeof(float4) * (size_t)q.n_tris,
                              cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        check(cudaMemcpyAsync(a->d_leaf_of_prim + tri0, q.d_leaf_of_prim, sizeof(uint32_t) * (size_t)q.n_tris,
                              cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        k_relocate_nodes<<<blocks_for(q.n_nodes), kBuildThreads, 0, s>>>(
            nodes, q.n_nodes, quads, a->node_format == 1 ? 12 : 1, a->roots[p], (uint32_t)tri0);
        k_relocate_tris<<<blocks_for(q.n_tris), kBuildThreads, 0, s>>>(a->d_tris + 3 * (size_t)tri0,
                                                                        a->d_leaf_of_prim + tri0, q.n_tris,
                                                                        (uint32_t)tri0);
        check(cudaGetLastError(), "relocate");
    }
    if (st == KRR_OK)
        check(cudaMemcpyAsync(a->d_roots, a->roots.data(), sizeof(uint32_t) * n_parts, cudaMemcpyHostToDevice, s),
              "cudaMemcpyAsync");
    if (st == KRR_OK) check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    release();
    a->level_first.clear();   // no refit of a multi-part structure
    return st;
}

}  // namespace krr

// ------------------------------------------------------------------ C ABI
using namespace krr;

extern "C" int krr_accel_create_from_triangles(const float *h_vertices, int64_t n_triangles,
                                               krr_accel **out, void *stream) {
    KRR_CHECK_ARG(out != nullptr, "out is NULL");
    KRR_CHECK_ARG(n_triangles == 0 || h_vertices != nullptr, "vertices are NULL");
    cudaStream_t s = as_stream(stream);
    float *d_v = nullptr;
    size_t bytes = sizeof(float) * 9 * (size_t)n_triangles;
    KRR_CUDA(cudaMalloc(&d_v, std::max<size_t>(bytes, 4)));
    cudaError_t e = cudaMemcpyAsync(d_v, h_vertices, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { cudaFree(d_v); return cuda_status(e, "cudaMemcpyAsync", __FILE__, __LINE__); }
    krr_accel *a = new krr_accel();
    int st = accel_build(a, d_v, n_triangles, s);
    cudaStreamSynchronize(s);
    cudaFree(d_v);
    if (st != KRR_OK) { accel_free(a); delete a; return st; }
    *out = a;
    return KRR_OK;
}

extern "C" int krr_accel_refit_triangles(krr_accel *a, const float *h_vertices, int64_t n_triangles,
                                         void *stream) {
    KRR_CHECK_ARG(a != nullptr, "accel is NULL");
    KRR_CHECK_ARG(n_triangles == 0 || h_vertices != nullptr, "vertices are NULL");
    KRR_CHECK_ARG(n_triangles == a->n_tris, "a refit keeps the triangle count of the build");
    if (n_triangles == 0) return KRR_OK;
    cudaStream_t s = as_stream(stream);
    DevBuf<float> d_v;
    const size_t bytes = sizeof(float) * 9 * (size_t)n_triangles;
    KRR_CUDA(d_v.alloc(9 * (size_t)n_triangles));
    KRR_CUDA(cudaMemcpyAsync(d_v.p, h_vertices, bytes, cudaMemcpyHostToDevice, s));
    int st = accel_refit(a, d_v.p, n_triangles, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (st != KRR_OK) return st;
    return cuda_status(e, "cudaStreamSynchronize", __FILE__, __LINE__);
}

// The radix tree on cubic Morton cells is the default: on the 10.9M-triangle
// bench scene it visits 5-6 % fewer nodes per ray than per-axis cells (the
// scene is 100 x 20 x 100 units, so per-axis cells split the thin axis as
// often as the wide ones), and PLOC's tree, collapsed the same way, visits
// more.
static int g_builder = 2;
int krr::default_builder() { return g_builder; }

extern "C" int krr_set_bvh_collapse(int32_t mode) {
    KRR_CHECK_ARG(mode == 0 || mode == 1, "collapse must be 0 (greedy) or 1 (cost-optimal)");
    g_collapse = mode;
    return KRR_OK;
}

extern "C" int krr_set_bvh_treelets(int32_t passes) {
    KRR_CHECK_ARG(passes >= 0 && passes <= 3, "treelet passes must be 0..3");
    g_treelets = passes;
    return KRR_OK;
}

extern "C" int krr_set_bvh_builder(int32_t builder) {
    KRR_CHECK_ARG(builder >= 0 && builder <= 2,
                  "builder must be 0 (radix tree), 1 (PLOC) or 2 (radix tree, cubic Morton cells)");
    g_builder = builder;
    return KRR_OK;
}

static int g_node_format = 0;
static int g_max_leaf = 1;
int krr::default_node_format() { return g_node_format; }
int krr::default_max_leaf() { return g_max_leaf; }

extern "C" int krr_set_bvh_max_leaf(int32_t triangles) {
    KRR_CHECK_ARG(triangles >= 1 && triangles <= 3, "leaf size must be 1, 2 or 3 triangles");
    g_max_leaf = triangles;
    return KRR_OK;
}

static int g_full_leaf = 1;
int krr::default_full_leaf() { return g_full_leaf; }

extern "C" int krr_set_bvh_full_node_leaf(int32_t triangles) {
    KRR_CHECK_ARG(triangles >= 1 && triangles <= 3, "leaf size must be 1, 2 or 3 triangles");
    g_full_leaf = triangles;
    return KRR_OK;
}

extern "C" int krr_set_bvh_node_format(int32_t format) {
    KRR_CHECK_ARG(format == 0 || format == 1, "node format must be 0 (compressed) or 1 (float)");
    g_node_format = format;
    return KRR_OK;
}

extern "C" int krr_accel_stats_get(const krr_accel *a, krr_accel_stats *out) {
    KRR_CHECK_ARG(a && out, "NULL argument");
    out->n_triangles = a->n_tris;
    out->n_nodes = a->n_nodes;
    out->max_depth = a->max_depth;
    out->build_ms = a->build_ms;
    out->node_bytes = 16.0 * kNodeQuads[a->node_format] * (double)a->n_nodes;
    out->reserved = a->node_format;
    out->triangle_bytes = 48.0 * (double)a->n_tris;
    if (a->levels == 2) {   // each geometry once, plus the instance records
        out->triangle_bytes = 48.0 * (double)(a->blas->n_tris + a->tlas->n_tris) +
                              sizeof(TraceInst) * (double)a->h_inst.size();
    }
    return KRR_OK;
}

extern "C" int krr_accel_destroy(krr_accel *a) {
    if (!a) return KRR_OK;
    accel_free(a);
    delete a;
    return KRR_OK;
}

extern "C" int krr_accel_set_mask(krr_accel *a, const uint8_t *h_mask) {
    KRR_CHECK_ARG(a != nullptr, "accel is NULL");
    if (a->n_tris == 0) return KRR_OK;
    uint8_t *d = nullptr;
    if (h_mask) {
        KRR_CUDA(cudaMalloc(&d, a->n_tris));
        KRR_CUDA(cudaMemcpy(d, h_mask, a->n_tris, cudaMemcpyHostToDevice));
    }
    int st = accel_set_mask(a, d, 0);
    cudaDeviceSynchronize();
    cudaFree(d);
    return st;
}

static TraceLaunch aos_launch(const krr_accel *a, const krr_ray *d_rays, int64_t n) {
    TraceLaunch l{};
    l.ray_o = reinterpret_cast<const float4 *>(d_rays);
    l.ray_d = reinterpret_cast<const float4 *>(d_rays) + 1;
    l.ray_stride = 2;
    l.n = n;
    l.d_count = nullptr;
    l.counter = a->d_scratch;
    l.err = a->d_scratch + 4;
    return l;
}

// Reads and clears the traversal error flags at d_err (device) after the
// stream's work; a raised stack-overflow flag becomes KRR_ERR_OVERFLOW.
int krr::take_trace_errors(int *d_err, cudaStream_t s, uint32_t *out_flags) {
    uint32_t flags = 0;
    KRR_CUDA(cudaMemcpyAsync(&flags, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    KRR_CUDA(cudaMemsetAsync(d_err, 0, sizeof(uint32_t), s));
    KRR_CUDA(cudaStreamSynchronize(s));
    if (out_flags) *out_flags = flags;
    if (flags & kErrStackOverflow)
        return fail(KRR_ERR_OVERFLOW, "traversal stack limit reached: rays were cut off (t = NaN / occluded = 0xFF)");
    return KRR_OK;
}

extern "C" int krr_accel_device_errors(const krr_accel *a, uint32_t *out_flags, void *stream) {
    KRR_CHECK_ARG(a && out_flags, "NULL argument");
    *out_flags = 0;
    if (!a->d_scratch) return KRR_OK;
    int st = take_trace_errors(a->d_scratch + 4, as_stream(stream), out_flags);
    return st == KRR_ERR_OVERFLOW ? KRR_OK : st;
}

extern "C" int krr_accel_set_stack_limit(krr_accel *a, int32_t entries) {
    KRR_CHECK_ARG(a != nullptr, "accel is NULL");
    KRR_CHECK_ARG(entries >= 1 && entries <= kTraversalStack, "stack limit must be 1..48 entries");
    a->stack_limit = entries;
    return KRR_OK;
}

extern "C" int krr_accel_trace_closest(const krr_accel *a, const krr_ray *d_rays, int64_t n,
                                       krr_hit *d_hits, void *stream) {
    KRR_CHECK_ARG(a && (n == 0 || (d_rays && d_hits)), "NULL argument");
    KRR_CHECK_ARG(n >= 0, "negative ray count");
    if (n == 0) return KRR_OK;
    TraceLaunch l = aos_launch(a, d_rays, n);
    l.hits = reinterpret_cast<float4 *>(d_hits);
    return launch_trace_closest(a, l, as_stream(stream));   // no triangles: every ray misses
}

extern "C" int krr_accel_trace_any(const krr_accel *a, const krr_ray *d_rays, int64_t n,
                                   uint8_t *d_occluded, void *stream) {
    KRR_CHECK_ARG(a && (n == 0 || (d_rays && d_occluded)), "NULL argument");
    KRR_CHECK_ARG(n >= 0, "negative ray count");
    if (n == 0) return KRR_OK;
    TraceLaunch l = aos_launch(a, d_rays, n);
    l.occluded = d_occluded;
    return launch_trace_any(a, l, as_stream(stream));
}

extern "C" int krr_accel_trace_stats(const krr_accel *a, const krr_ray *d_rays, int64_t n,
                                     int32_t any_hit, unsigned long long *h_counts, void *stream) {
    KRR_CHECK_ARG(a && d_rays && h_counts && n > 0, "bad argument");
    if (a->n_tris == 0) return fail(KRR_ERR_NOT_READY, "empty acceleration structure");
    cudaStream_t s = as_stream(stream);
    TraceLaunch l = aos_launch(a, d_rays, n);
    float4 *hits = nullptr;
    uint8_t *occ = nullptr;
    unsigned long long *d_counts = nullptr;
    KRR_CUDA(cudaMalloc(&d_counts, 2 * sizeof(unsigned long long)));
    KRR_CUDA(cudaMemsetAsync(d_counts, 0, 2 * sizeof(unsigned long long), s));
    if (any_hit) { KRR_CUDA(cudaMalloc(&occ, n)); l.occluded = occ; }
    else { KRR_CUDA(cudaMalloc(&hits, n * sizeof(float4))); l.hits = hits; }
    int st = launch_trace_stats(a, l, any_hit != 0, d_counts, s);
    if (st == KRR_OK) {
        KRR_CUDA(cudaMemcpyAsync(h_counts, d_counts, 2 * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, s));
        st = take_trace_errors(l.err, s, nullptr);
    }
    cudaFree(d_counts);
    cudaFree(hits);
    cudaFree(occ);
    return st;
}

// Host buffers in and out.  The rays go in chunks over two streams (the
// caller's and a helper), so that the copies of one chunk overlap the
// traversal of another; each stream has its own work counter in the scratch
// block (ints 0-1 and 8-9).
extern "C" int krr_accel_trace_closest_host(const krr_accel *a, const krr_ray *h_rays, int64_t n,
                                            krr_hit *h_hits, void *stream) {
    KRR_CHECK_ARG(a && (n == 0 || (h_rays && h_hits)), "NULL argument");
    KRR_CHECK_ARG(n >= 0, "negative ray count");
    if (n == 0) return KRR_OK;
    if (!a->d_scratch) return fail(KRR_ERR_NOT_READY, "acceleration structure not built");
    // the staging buffers, stream and events are cached on the handle (the
    // handle is not const in storage; callers already may not trace on one
    // handle from two threads at once, since the work counters are shared)
    krr_accel *m = const_cast<krr_accel *>(a);
    cudaStream_t s = as_stream(stream);
    // Page-locked host buffers on a GPU that reaches host memory coherently
    // through the host's page tables (Grace's NVLink-C2C): the persistent
    // kernel reads the rays and writes the hits in host memory directly, so
    // the transfers overlap the traversal with no staging and no chunking.
    {
        static int coherent = -1;
        if (coherent < 0) {
            int dev = 0, v = 0;
            cudaGetDevice(&dev);
            coherent = cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
                               cudaSuccess && v ? 1 : 0;
            cudaGetLastError();
        }
        cudaPointerAttributes pr{}, ph{};
        const bool ok = coherent && cudaPointerGetAttributes(&pr, h_rays) == cudaSuccess &&
                        cudaPointerGetAttributes(&ph, h_hits) == cudaSuccess;
        cudaGetLastError();
        if (ok && pr.type == cudaMemoryTypeHost && ph.type == cudaMemoryTypeHost && pr.devicePointer &&
            ph.devicePointer && ((uintptr_t)pr.devicePointer & 15u) == 0 &&
            ((uintptr_t)ph.devicePointer & 15u) == 0) {
            TraceLaunch l = aos_launch(a, reinterpret_cast<const krr_ray *>(pr.devicePointer), n);
            l.hits = reinterpret_cast<float4 *>(ph.devicePointer);
            KRR_TRY(launch_trace_closest(a, l, s));
            return take_trace_errors(l.err, s, nullptr);
        }
    }
    // Otherwise (pageable memory, or no coherent link): chunks of rays are
    // copied in, traced and copied out over two streams.
    if (!m->stage_aux) {
        KRR_CUDA(cudaStreamCreateWithFlags(&m->stage_aux, cudaStreamNonBlocking));
        KRR_CUDA(cudaEventCreateWithFlags(&m->stage_ev[0], cudaEventDisableTiming));
        KRR_CUDA(cudaEventCreateWithFlags(&m->stage_ev[1], cudaEventDisableTiming));
    }
    if (m->stage_cap < n) {
        KRR_CUDA(cudaStreamSynchronize(s));
        cudaFree(m->stage_rays);
        cudaFree(m->stage_hits);
        m->stage_rays = m->stage_hits = nullptr;
        m->stage_cap = 0;
        KRR_CUDA(cudaMalloc(&m->stage_rays, (size_t)n * sizeof(krr_ray)));
        KRR_CUDA(cudaMalloc(&m->stage_hits, (size_t)n * sizeof(krr_hit)));
        m->stage_cap = n;
    }
    static_assert(sizeof(krr_ray) == 2 * sizeof(float4) && sizeof(krr_hit) == sizeof(float4),
                  "ray and hit records");
    krr_ray *d_rays = reinterpret_cast<krr_ray *>(m->stage_rays);
    krr_hit *d_hits = reinterpret_cast<krr_hit *>(m->stage_hits);
    cudaStream_t aux = m->stage_aux;
    int st = KRR_OK;
    auto check = [&](cudaError_t e, const char *what) {
        if (st == KRR_OK && e != cudaSuccess) st = cuda_status(e, what, __FILE__, __LINE__);
    };
    check(cudaEventRecord(m->stage_ev[0], s), "cudaEventRecord");
    check(cudaStreamWaitEvent(aux, m->stage_ev[0], 0), "cudaStreamWaitEvent");
    const int64_t chunk = std::max<int64_t>(int64_t(1) << 18, (n + 3) / 4);
    int k = 0;
    for (int64_t off = 0; off < n && st == KRR_OK; off += chunk, ++k) {
        const int64_t c = std::min(chunk, n - off);
        cudaStream_t sk = (k & 1) ? aux : s;
        check(cudaMemcpyAsync(d_rays + off, h_rays + off, c * sizeof(krr_ray), cudaMemcpyHostToDevice, sk),
              "cudaMemcpyAsync");
        if (st != KRR_OK) break;
        TraceLaunch l = aos_launch(a, d_rays + off, c);
        l.hits = reinterpret_cast<float4 *>(d_hits + off);
        l.counter = a->d_scratch + ((k & 1) ? 8 : 0);
        st = launch_trace_closest(a, l, sk);
        if (st != KRR_OK) break;
        check(cudaMemcpyAsync(h_hits + off, d_hits + off, c * sizeof(krr_hit), cudaMemcpyDeviceToHost, sk),
              "cudaMemcpyAsync");
    }
    cudaEventRecord(m->stage_ev[1], aux);
    cudaStreamWaitEvent(s, m->stage_ev[1], 0);
    check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (st == KRR_OK) st = take_trace_errors(a->d_scratch + 4, s, nullptr);
    return st;
}

extern "C" int krr_accel_set_tuning(krr_accel *a, int32_t refill_below, int32_t postpone_pct) {
    KRR_CHECK_ARG(a != nullptr, "accel is NULL");
    KRR_CHECK_ARG(refill_below >= 1 && refill_below <= 32, "refill_below must be 1..32");
    KRR_CHECK_ARG(postpone_pct >= 0 && postpone_pct <= 100, "postpone_pct must be 0..100");
    a->refill_below = refill_below;
    a->postpone_pct = postpone_pct;
    return KRR_OK;
}

// Times the closest-hit kernel on the given rays for each candidate setting
// (refill threshold x triangle-postponing threshold) and keeps the fastest.
extern "C" int krr_accel_autotune(krr_accel *a, const krr_ray *d_rays, int64_t n, int32_t repeats,
                                  int32_t *out_refill, int32_t *out_postpone, float *out_ms,
                                  void *stream) {
    KRR_CHECK_ARG(a && d_rays && n > 0, "bad argument");
    if (a->n_tris == 0) return fail(KRR_ERR_NOT_READY, "empty acceleration structure");
    cudaStream_t s = as_stream(stream);
    float4 *hits = nullptr;
    KRR_CUDA(cudaMalloc(&hits, n * sizeof(float4)));
    TraceLaunch l = aos_launch(a, d_rays, n);
    l.hits = hits;
    const int refills[] = {12, 16, 20, 24, 28};
    const int postpones[] = {0, 10, 20, 35};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int br = a->refill_below, bp = a->postpone_pct;
    int st = KRR_OK;
    for (int rf : refills) {
        for (int pp : postpones) {
            a->refill_below = rf;
            a->postpone_pct = pp;
            st = launch_trace_closest(a, l, s);   // warm-up
            if (st != KRR_OK) break;
            cudaEventRecord(e0, s);
            for (int k = 0; k < std::max(1, repeats); ++k) st = launch_trace_closest(a, l, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= std::max(1, repeats);
            if (ms < best) { best = ms; br = rf; bp = pp; }
        }
        if (st != KRR_OK) break;
    }
    a->refill_below = br;
    a->postpone_pct = bp;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(hits);
    if (out_refill) *out_refill = br;
    if (out_postpone) *out_postpone = bp;
    if (out_ms) *out_ms = best;
    return st;
}
