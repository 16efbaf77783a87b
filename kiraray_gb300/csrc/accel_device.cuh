// Device-side traversal building blocks shared by the persistent trace kernel
// (accel.cu) and kernels that trace inside their own loops (media.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "accel.h"
#include "kmath.cuh"

namespace krr {

struct RayPre {
    V3 o, d;
    float tmin;
    int kx, ky, kz;
    float sx, sy, sz;
};

__device__ __forceinline__ RayPre ray_pre(V3 o, V3 d, float tmin) {
    RayPre r;
    r.o = o; r.d = d;
    r.tmin = tmin > 0.f ? tmin : 0.f;   // negative (and -0) tmin act as +0
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (get(d, kz) < 0.f) { int tmp = kx; kx = ky; ky = tmp; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    float dz = get(d, kz);
    r.sx = __fdiv_rn(get(d, kx), dz);
    r.sy = __fdiv_rn(get(d, ky), dz);
    r.sz = __fdiv_rn(1.0f, dz);
    return r;
}

__device__ __forceinline__ float sel3(float a, float b, float c, int k) {
    return k == 0 ? a : (k == 1 ? b : c);
}

// Watertight ray/triangle test; returns t (NaN on a miss, so that a miss fails
// every comparison including the tie rule at t == tmax == inf) and (b1, b2).
// Every operation is explicitly rounded so that the CPU restatement of the
// same steps gives bit-identical results.
__device__ __forceinline__ float tri_test(const RayPre &r, float4 v0, float4 v1, float4 v2,
                                          float &b1, float &b2) {
    float Ax_ = __fsub_rn(v0.x, r.o.x), Ay_ = __fsub_rn(v0.y, r.o.y), Az_ = __fsub_rn(v0.z, r.o.z);
    float Bx_ = __fsub_rn(v1.x, r.o.x), By_ = __fsub_rn(v1.y, r.o.y), Bz_ = __fsub_rn(v1.z, r.o.z);
    float Cx_ = __fsub_rn(v2.x, r.o.x), Cy_ = __fsub_rn(v2.y, r.o.y), Cz_ = __fsub_rn(v2.z, r.o.z);
    float Akx = sel3(Ax_, Ay_, Az_, r.kx), Aky = sel3(Ax_, Ay_, Az_, r.ky), Akz = sel3(Ax_, Ay_, Az_, r.kz);
    float Bkx = sel3(Bx_, By_, Bz_, r.kx), Bky = sel3(Bx_, By_, Bz_, r.ky), Bkz = sel3(Bx_, By_, Bz_, r.kz);
    float Ckx = sel3(Cx_, Cy_, Cz_, r.kx), Cky = sel3(Cx_, Cy_, Cz_, r.ky), Ckz = sel3(Cx_, Cy_, Cz_, r.kz);
    float Ax = __fmaf_rn(-r.sx, Akz, Akx), Ay = __fmaf_rn(-r.sy, Akz, Aky);
    float Bx = __fmaf_rn(-r.sx, Bkz, Bkx), By = __fmaf_rn(-r.sy, Bkz, Bky);
    float Cx = __fmaf_rn(-r.sx, Ckz, Ckx), Cy = __fmaf_rn(-r.sy, Ckz, Cky);
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
        V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
        W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return __int_as_float(0x7fffffff);
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.f) return __int_as_float(0x7fffffff);
    float Az = __fmul_rn(r.sz, Akz), Bz = __fmul_rn(r.sz, Bkz), Cz = __fmul_rn(r.sz, Ckz);
    float T = __fmaf_rn(U, Az, __fmaf_rn(V, Bz, __fmul_rn(W, Cz)));
    float rcp = __frcp_rn(det);
    float t = __fmul_rn(T, rcp);
    b1 = __fmul_rn(V, rcp);
    b2 = __fmul_rn(W, rcp);
    return t;
}


// 8-bit quantised plane k of a packed word as the float 2^23 + 256 q
// (exact): one byte permute into 0x4B00qq00.
__device__ __forceinline__ float plane256(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7404u | ((uint32_t)k << 4)));
}

// Visits one 8-wide node: returns the next node group (child base, hit
// positions | internal mask << 8) and the triangle group (base, bits).
// Entry/exit distances are compared as integers: with tmin >= +0 the
// maximum of the entry distances is a non-negative float, and the ordering
// of non-negative floats is the ordering of their bit patterns; a negative
// exit distance is a negative integer and fails the test, as it should.
// SINGLE: every leaf child holds one triangle, so a child's bit is one shift
// of 1 by its meta byte's position field (empty slots never hit: their boxes
// are inverted).
template <bool SINGLE>
__device__ __forceinline__ void visit_node(const float4 *__restrict__ nodes, uint32_t child,
                                           const RayPre &r, V3 inv, int oct, float tmax,
                                           uint2 &ng, uint2 &tg) {
    const float4 *np = nodes + 5 * (size_t)child;
    float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3),
           q4 = __ldg(np + 4);
    uint32_t ew = __float_as_uint(q0.w);
    float ex = __uint_as_float((ew & 0xffu) << 23);
    float ey = __uint_as_float(((ew >> 8) & 0xffu) << 23);
    float ez = __uint_as_float(((ew >> 16) & 0xffu) << 23);
    float adx = ex * inv.x, ady = ey * inv.y, adz = ez * inv.z;
    float orx = (q0.x - r.o.x) * inv.x, ory = (q0.y - r.o.y) * inv.y, orz = (q0.z - r.o.z) * inv.z;
    // A plane at q steps is t = q ad + or = (2^23 + 256 q) (ad / 256) + (or - 2^15 ad): one FMA
    // on the permuted byte.  Rounding the offset or - 2^15 ad errs by at most 2^-9 |ad| (half an
    // ulp of 2^15 |ad|) plus half an ulp of or; entry planes are moved down and exit planes up
    // by |ad| / 64 (1/64 of a quantisation step), which covers that with room to spare, so the
    // test stays conservative.
    const float dx = adx * 0.00390625f, dy = ady * 0.00390625f, dz = adz * 0.00390625f;
    const float cx = fmaf(-32768.f, adx, orx), cy = fmaf(-32768.f, ady, ory), cz = fmaf(-32768.f, adz, orz);
    const float sx = fabsf(adx) * 0.015625f, sy = fabsf(ady) * 0.015625f, sz = fabsf(adz) * 0.015625f;
    const float nox = cx - sx, noy = cy - sy, noz = cz - sz;
    const float fox = cx + sx, foy = cy + sy, foz = cz + sz;
    uint32_t lox0 = __float_as_uint(q2.x), lox1 = __float_as_uint(q2.y);
    uint32_t loy0 = __float_as_uint(q2.z), loy1 = __float_as_uint(q2.w);
    uint32_t loz0 = __float_as_uint(q3.x), loz1 = __float_as_uint(q3.y);
    uint32_t hix0 = __float_as_uint(q3.z), hix1 = __float_as_uint(q3.w);
    uint32_t hiy0 = __float_as_uint(q4.x), hiy1 = __float_as_uint(q4.y);
    uint32_t hiz0 = __float_as_uint(q4.z), hiz1 = __float_as_uint(q4.w);
    uint32_t nx0 = (oct & 1) ? hix0 : lox0, nx1 = (oct & 1) ? hix1 : lox1;
    uint32_t fx0 = (oct & 1) ? lox0 : hix0, fx1 = (oct & 1) ? lox1 : hix1;
    uint32_t ny0 = (oct & 2) ? hiy0 : loy0, ny1 = (oct & 2) ? hiy1 : loy1;
    uint32_t fy0 = (oct & 2) ? loy0 : hiy0, fy1 = (oct & 2) ? loy1 : hiy1;
    uint32_t nz0 = (oct & 4) ? hiz0 : loz0, nz1 = (oct & 4) ? hiz1 : loz1;
    uint32_t fz0 = (oct & 4) ? loz0 : hiz0, fz1 = (oct & 4) ? loz1 : hiz1;
    // internal children: XOR the ray octant into their bit index (24 + slot)
    uint32_t meta0 = __float_as_uint(q1.z), meta1 = __float_as_uint(q1.w);
    meta0 ^= ((meta0 & (meta0 << 1) & 0x10101010u) >> 4) * (uint32_t)oct;
    meta1 ^= ((meta1 & (meta1 << 1) & 0x10101010u) >> 4) * (uint32_t)oct;
    const float tlimit = tmax + fabsf(tmax) * 5e-7f;
    const int tmin_i = __float_as_int(r.tmin), tlim_i = __float_as_int(tlimit);
    uint32_t hitmask = 0;
    // children in slots 0-3, then 4-7 unless all four are empty (meta bytes
    // 0: nodes of at most four leaf children keep their slots 4-7 empty)
    auto test_child = [&](uint32_t meta, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t fx, uint32_t fy,
                          uint32_t fz, int k) {
        uint32_t m = __byte_perm(meta, 0u, 0x4440u + (uint32_t)k);
        int tnx = __float_as_int(fmaf(plane256(nx, k), dx, nox));
        int tny = __float_as_int(fmaf(plane256(ny, k), dy, noy));
        int tnz = __float_as_int(fmaf(plane256(nz, k), dz, noz));
        int tfx = __float_as_int(fmaf(plane256(fx, k), dx, fox));
        int tfy = __float_as_int(fmaf(plane256(fy, k), dy, foy));
        int tfz = __float_as_int(fmaf(plane256(fz, k), dz, foz));
        int t0 = __vimax3_s32(tnx, tny, max(tnz, tmin_i));
        int t1 = __vimin3_s32(tfx, tfy, min(tfz, tlim_i));
        uint32_t bits = SINGLE ? __funnelshift_l(0u, 1u, m) : (m >> 5) << (m & 31u);
        hitmask |= (t0 <= t1) ? bits : 0u;
    };
#pragma unroll
    for (int k = 0; k < 4; ++k) test_child(meta0, nx0, ny0, nz0, fx0, fy0, fz0, k);
    if (meta1 != 0u) {
#pragma unroll
        for (int k = 0; k < 4; ++k) test_child(meta1, nx1, ny1, nz1, fx1, fy1, fz1, k);
    }
    uint32_t cimask = ew >> 24;
    ng = make_uint2(__float_as_uint(q1.x), (hitmask >> 24) | (cimask << 8));
    tg = make_uint2(__float_as_uint(q1.y), hitmask & 0x00ffffffu);
}

// Float node format: near/far planes are picked per ray by address (no
// per-child selects); t = b * inv + (-o * inv) with one FMA per plane.
__device__ __forceinline__ void visit_node_f(const float4 *__restrict__ nodes, uint32_t child,
                                             const RayPre &r, V3 inv, V3 oinv, int oct, float tmax,
                                             uint2 &ng, uint2 &tg) {
    const float4 *np = nodes + 14 * (size_t)child;
    const int nxo = (oct & 1) ? 2 : 0, nyo = (oct & 2) ? 6 : 4, nzo = (oct & 4) ? 10 : 8;
    const float4 nxa = __ldg(np + nxo), nxb = __ldg(np + nxo + 1);
    const float4 fxa = __ldg(np + (nxo ^ 2)), fxb = __ldg(np + (nxo ^ 2) + 1);
    const float4 nya = __ldg(np + nyo), nyb = __ldg(np + nyo + 1);
    const float4 fya = __ldg(np + (nyo ^ 2)), fyb = __ldg(np + (nyo ^ 2) + 1);
    const float4 nza = __ldg(np + nzo), nzb = __ldg(np + nzo + 1);
    const float4 fza = __ldg(np + (nzo ^ 2)), fzb = __ldg(np + (nzo ^ 2) + 1);
    const float4 q12 = __ldg(np + 12), q13 = __ldg(np + 13);
    uint32_t meta0 = __float_as_uint(q12.z), meta1 = __float_as_uint(q12.w);
    meta0 ^= ((meta0 & (meta0 << 1) & 0x10101010u) >> 4) * (uint32_t)oct;
    meta1 ^= ((meta1 & (meta1 << 1) & 0x10101010u) >> 4) * (uint32_t)oct;
    const float tlimit = tmax + fabsf(tmax) * 5e-7f;
    const int tmin_i = __float_as_int(r.tmin), tlim_i = __float_as_int(tlimit);
    const float nx[8] = {nxa.x, nxa.y, nxa.z, nxa.w, nxb.x, nxb.y, nxb.z, nxb.w};
    const float fx[8] = {fxa.x, fxa.y, fxa.z, fxa.w, fxb.x, fxb.y, fxb.z, fxb.w};
    const float ny[8] = {nya.x, nya.y, nya.z, nya.w, nyb.x, nyb.y, nyb.z, nyb.w};
    const float fy[8] = {fya.x, fya.y, fya.z, fya.w, fyb.x, fyb.y, fyb.z, fyb.w};
    const float nz[8] = {nza.x, nza.y, nza.z, nza.w, nzb.x, nzb.y, nzb.z, nzb.w};
    const float fz[8] = {fza.x, fza.y, fza.z, fza.w, fzb.x, fzb.y, fzb.z, fzb.w};
    uint32_t hitmask = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint32_t m = __byte_perm(c < 4 ? meta0 : meta1, 0u, 0x4440u + (uint32_t)(c & 3));
        int tnx = __float_as_int(fmaf(nx[c], inv.x, oinv.x));
        int tny = __float_as_int(fmaf(ny[c], inv.y, oinv.y));
        int tnz = __float_as_int(fmaf(nz[c], inv.z, oinv.z));
        int tfx = __float_as_int(fmaf(fx[c], inv.x, oinv.x));
        int tfy = __float_as_int(fmaf(fy[c], inv.y, oinv.y));
        int tfz = __float_as_int(fmaf(fz[c], inv.z, oinv.z));
        int t0 = __vimax3_s32(tnx, tny, max(tnz, tmin_i));
        int t1 = __vimin3_s32(tfx, tfy, min(tfz, tlim_i));
        uint32_t bits = (m >> 5) << (m & 31u);
        hitmask |= (t0 <= t1) ? bits : 0u;
    }
    uint32_t cimask = __float_as_uint(q13.x);
    ng = make_uint2(__float_as_uint(q12.x), (hitmask >> 24) | (cimask << 8));
    tg = make_uint2(__float_as_uint(q12.y), hitmask & 0x00ffffffu);
}

template <int FMT>
__device__ __forceinline__ void visit(const float4 *__restrict__ nodes, uint32_t child,
                                      const RayPre &r, V3 inv, V3 oinv, int oct, float tmax,
                                      uint2 &ng, uint2 &tg) {
    if (FMT == 1) visit_node_f(nodes, child, r, inv, oinv, oct, tmax, ng, tg);
    else visit_node<FMT == 2>(nodes, child, r, inv, oct, tmax, ng, tg);
}

__device__ __forceinline__ V3 box_inverse(V3 d) {
    float dx = fabsf(d.x) < 1e-20f ? copysignf(1e-20f, d.x) : d.x;
    float dy = fabsf(d.y) < 1e-20f ? copysignf(1e-20f, d.y) : d.y;
    float dz = fabsf(d.z) < 1e-20f ? copysignf(1e-20f, d.z) : d.z;
    return V3{1.f / dx, 1.f / dy, 1.f / dz};
}

// Single-ray traversal for kernels that trace inside their own loops, from
// node `root` (a part's tree in a multi-part node array).
// Closest hit: returns (t, b1, b2, id bits) or id KRR_MISS; any hit: the id
// of some blocking triangle (mask != 0, or any triangle when !MASKED) or
// KRR_MISS.  Same hit as the persistent kernel (the result does not depend
// on traversal order).
template <bool ANY, int FMT, bool MASKED = true>
__device__ float4 traverse_ray(const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
                               V3 o, V3 d, float tmin, float tmax, int *err, uint32_t root = 0) {
    RayPre r = ray_pre(o, d, tmin);
    V3 inv = box_inverse(d);
    V3 oinv = V3{-o.x * inv.x, -o.y * inv.y, -o.z * inv.z};
    int oct = (inv.x < 0.f ? 1 : 0) | (inv.y < 0.f ? 2 : 0) | (inv.z < 0.f ? 4 : 0);
    uint2 stack[kTraversalStack];
    int sp = 0;
    uint2 ng = make_uint2(root, (1u << oct) | (1u << 8)), tg = make_uint2(0u, 0u);
    float b1b = 0.f, b2b = 0.f;
    uint32_t best = KRR_MISS;
    while (true) {
        if (ng.y & 0xffu) {
            int p = __ffs(ng.y & 0xffu) - 1;
            ng.y &= ~(1u << p);
            int slot = p ^ oct;
            uint32_t imask = ng.y >> 8;
            uint32_t child = ng.x + __popc(imask & ((1u << slot) - 1u));
            if (ng.y & 0xffu) {
                if (sp < kTraversalStack) stack[sp++] = ng;
                else { atomicOr(err, (int)kErrStackOverflow); break; }
            }
            visit<FMT>(nodes, child, r, inv, oinv, oct, tmax, ng, tg);
        }
        while (tg.y) {
            int b = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const float4 *tp = tris + 3 * (size_t)(tg.x + b);
            float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
            float b1, b2;
            float t = tri_test(r, v0, v1, v2, b1, b2);
            uint32_t gid = __float_as_uint(v0.w);
            if (ANY) {
                if (t > r.tmin && t <= tmax && (!MASKED || __float_as_uint(v1.w) != 0u))
                    return make_float4(t, b1, b2, __uint_as_float(gid));
            } else if (t > r.tmin && (t < tmax || (t == tmax && gid < best))) {
                tmax = t; b1b = b1; b2b = b2; best = gid;
            }
        }
        if (!(ng.y & 0xffu)) {
            if (sp > 0) ng = stack[--sp];
            else break;
        }
    }
    if (best == KRR_MISS) return make_float4(INFINITY, 0.f, 0.f, __uint_as_float(KRR_MISS));
    return make_float4(tmax, b1b, b2b, __uint_as_float(best));
}

// Two-level structures (instanced.cu): the world ray walks the instance
// tree; at an instance leaf it is carried into the instance's object space
// by the instance's world-to-object 3x4 matrix, row by row, each operation
// rounded, and the instance's geometry tree gives the closest hit with t in
// (tmin, best t]; it replaces the best hit if its t is smaller, or equal
// with a smaller global id.  The result is the smallest (t, global id) over
// all instances whatever the order, as the CPU oracle computes it.
// world -> object: rows of a 3x4 row-major matrix, operation by operation
__device__ __forceinline__ V3 inst_point(const float *m, V3 p) {
    V3 r;
    float *o = &r.x;
    for (int k = 0; k < 3; ++k) {
        const float *row = m + 4 * k;
        float acc = __fmul_rn(row[0], p.x);
        acc = __fadd_rn(acc, __fmul_rn(row[1], p.y));
        acc = __fadd_rn(acc, __fmul_rn(row[2], p.z));
        o[k] = __fadd_rn(acc, row[3]);
    }
    return r;
}

__device__ __forceinline__ V3 inst_vector(const float *m, V3 d) {
    V3 r;
    float *o = &r.x;
    for (int k = 0; k < 3; ++k) {
        const float *row = m + 4 * k;
        float acc = __fmul_rn(row[0], d.x);
        acc = __fadd_rn(acc, __fmul_rn(row[1], d.y));
        o[k] = __fadd_rn(acc, __fmul_rn(row[2], d.z));
    }
    return r;
}

// Closest (ANY: any masked) hit of one world ray over the two levels.
template <bool ANY, int FMT, bool MASKED = true>
__device__ float4 trace_two_level(const InstancedView &v, V3 o, V3 d, float tmin, float tmax, int *err) {
    // the instance tree holds no triangles: the world ray needs only what the
    // box tests read (origin and tmin), not the triangle test's shear
    RayPre r;
    r.o = o;
    r.d = d;
    r.tmin = tmin > 0.f ? tmin : 0.f;
    V3 inv = box_inverse(d);
    V3 oinv = V3{-o.x * inv.x, -o.y * inv.y, -o.z * inv.z};
    int oct = (inv.x < 0.f ? 1 : 0) | (inv.y < 0.f ? 2 : 0) | (inv.z < 0.f ? 4 : 0);
    uint2 stack[kTraversalStack];
    int sp = 0;
    uint2 ng = make_uint2(0u, (1u << oct) | (1u << 8)), tg = make_uint2(0u, 0u);
    float bt = tmax, bb1 = 0.f, bb2 = 0.f;
    uint32_t best = KRR_MISS;
    while (true) {
        if (ng.y & 0xffu) {
            int p = __ffs(ng.y & 0xffu) - 1;
            ng.y &= ~(1u << p);
            int slot = p ^ oct;
            uint32_t imask = ng.y >> 8;
            uint32_t child = ng.x + __popc(imask & ((1u << slot) - 1u));
            if (ng.y & 0xffu) {
                if (sp < kTraversalStack) stack[sp++] = ng;
                else { atomicOr(err, (int)kErrStackOverflow); break; }
            }
            visit<FMT>(v.tlas_nodes, child, r, inv, oinv, oct, bt, ng, tg);
        }
        while (tg.y) {
            int b = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const uint32_t k = __float_as_uint(__ldg(v.tlas_tris + 3 * (size_t)(tg.x + b)).w);
            const TraceInst I = v.inst[k];
            if (ANY && MASKED && !I.mask) continue;
            const V3 io = inst_point(I.inv, o), id = inst_vector(I.inv, d);
            const float4 h = traverse_ray<ANY, FMT, false>(v.blas_nodes, v.blas_tris, io, id, tmin, bt,
                                                           err, I.blas_root);
            const uint32_t local = __float_as_uint(h.w);
            if (local == KRR_MISS) continue;
            const uint32_t gid = local + I.id_delta;
            if (ANY) return make_float4(h.x, h.y, h.z, __uint_as_float(gid));
            if (h.x < bt || (h.x == bt && gid < best)) {
                bt = h.x; bb1 = h.y; bb2 = h.z; best = gid;
            }
        }
        if (!(ng.y & 0xffu)) {
            if (sp > 0) ng = stack[--sp];
            else break;
        }
    }
    if (best == KRR_MISS) return make_float4(INFINITY, 0.f, 0.f, __uint_as_float(KRR_MISS));
    return make_float4(bt, bb1, bb2, __uint_as_float(best));
}

}  // namespace krr
