// CPU closest-hit / any-hit oracle (test infrastructure only).
//
// The reference traces with OptiX (src/render/wavefront/device.cu:12-22,
// src/core/device/optix.cpp:143-250) and contains no ray/triangle code, so
// this restates the watertight test of Woop, Benthin and Wald (JCGT 2013)
// with the operation order spelled out, plus a binned-SAH binary BVH whose
// box tests are made conservative (margin-widened boxes, slab slack) so that
// the hit set equals brute force.  Ties in t go to the smaller triangle id.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

constexpr uint32_t kMiss = 0xFFFFFFFFu;

struct RayPre {
    float o[3], d[3];
    float tmin, tmax;
    int kx, ky, kz;
    float sx, sy, sz;
    float inv[3];
};

RayPre make_ray(const float *r) {
    RayPre p;
    for (int k = 0; k < 3; ++k) { p.o[k] = r[k]; p.d[k] = r[4 + k]; }
    p.tmin = r[3] > 0.f ? r[3] : 0.f;   // negative (and -0) tmin act as +0
    p.tmax = r[7];
    float ax = std::fabs(p.d[0]), ay = std::fabs(p.d[1]), az = std::fabs(p.d[2]);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (p.d[kz] < 0.f) std::swap(kx, ky);
    p.kx = kx; p.ky = ky; p.kz = kz;
    p.sx = p.d[kx] / p.d[kz];
    p.sy = p.d[ky] / p.d[kz];
    p.sz = 1.0f / p.d[kz];
    for (int k = 0; k < 3; ++k) {
        float dd = std::fabs(p.d[k]) < 1e-20f ? std::copysign(1e-20f, p.d[k]) : p.d[k];
        p.inv[k] = 1.0f / dd;
    }
    return p;
}

// Woop-Benthin-Wald watertight test.  Returns NaN on a miss (NaN fails every
// comparison, so a miss never passes the t-window or the tie rule).
float tri_test(const RayPre &r, const float *v0, const float *v1, const float *v2, float &b1,
               float &b2) {
    float A[3] = {v0[0] - r.o[0], v0[1] - r.o[1], v0[2] - r.o[2]};
    float B[3] = {v1[0] - r.o[0], v1[1] - r.o[1], v1[2] - r.o[2]};
    float C[3] = {v2[0] - r.o[0], v2[1] - r.o[1], v2[2] - r.o[2]};
    float Ax = std::fma(-r.sx, A[r.kz], A[r.kx]), Ay = std::fma(-r.sy, A[r.kz], A[r.ky]);
    float Bx = std::fma(-r.sx, B[r.kz], B[r.kx]), By = std::fma(-r.sy, B[r.kz], B[r.ky]);
    float Cx = std::fma(-r.sx, C[r.kz], C[r.kx]), Cy = std::fma(-r.sy, C[r.kz], C[r.ky]);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return NAN;
    float det = (U + V) + W;
    if (det == 0.f) return NAN;
    float Az = r.sz * A[r.kz], Bz = r.sz * B[r.kz], Cz = r.sz * C[r.kz];
    float T = std::fma(U, Az, std::fma(V, Bz, W * Cz));
    float rcp = 1.0f / det;
    float t = T * rcp;
    b1 = V * rcp;
    b2 = W * rcp;
    return t;
}

struct Node {
    float lo[3], hi[3];
    int32_t index;   // leaf: first triangle; inner: right child (left = this + 1)
    int32_t count;   // > 0 for leaves
};

}  // namespace

struct oracle_bvh {
    std::vector<Node> nodes;
    std::vector<float> tris;       // 9 floats per triangle, BVH order
    std::vector<uint32_t> ids;     // original triangle id per BVH slot
    std::vector<uint8_t> mask;     // per original id, any-hit mask
};

namespace {

struct BuildCtx {
    const float *v;
    std::vector<uint32_t> idx;
    std::vector<float> clo, chi, cen;   // per triangle
    float margin;
};

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float *l, const float *h) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], l[k]); hi[k] = std::max(hi[k], h[k]); }
    }
    float area() const {
        if (lo[0] > hi[0]) return 0.f;
        float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
        return e0 * e1 + e1 * e2 + e2 * e0;
    }
};

// Builds the subtree for idx[b, e) into `out` (pre-order, left child next).
void build_rec(BuildCtx &c, uint32_t b, uint32_t e, std::vector<Node> &out) {
    Box box, cbox;
    for (uint32_t i = b; i < e; ++i) {
        uint32_t t = c.idx[i];
        box.grow(&c.clo[3 * t], &c.chi[3 * t]);
        cbox.grow(&c.cen[3 * t], &c.cen[3 * t]);
    }
    size_t me = out.size();
    out.push_back(Node{});
    for (int k = 0; k < 3; ++k) { out[me].lo[k] = box.lo[k]; out[me].hi[k] = box.hi[k]; }
    uint32_t n = e - b;
    if (n <= 4) {
        out[me].index = (int32_t)b;
        out[me].count = (int32_t)n;
        return;
    }
    constexpr int kBins = 16;
    int best_axis = -1, best_split = 0;
    float best_cost = INFINITY;
    for (int k = 0; k < 3; ++k) {
        float ext = cbox.hi[k] - cbox.lo[k];
        if (!(ext > 0.f)) continue;
        Box bins[kBins];
        uint32_t cnt[kBins] = {};
        for (uint32_t i = b; i < e; ++i) {
            uint32_t t = c.idx[i];
            int bi = (int)((c.cen[3 * t + k] - cbox.lo[k]) / ext * kBins);
            bi = std::min(std::max(bi, 0), kBins - 1);
            cnt[bi]++;
            bins[bi].grow(&c.clo[3 * t], &c.chi[3 * t]);
        }
        float right_area[kBins];
        uint32_t right_cnt[kBins];
        Box acc;
        uint32_t ac = 0;
        for (int i = kBins - 1; i > 0; --i) {
            acc.grow(bins[i].lo, bins[i].hi);
            ac += cnt[i];
            right_area[i] = acc.area();
            right_cnt[i] = ac;
        }
        Box lacc;
        uint32_t lc = 0;
        for (int i = 0; i < kBins - 1; ++i) {
            lacc.grow(bins[i].lo, bins[i].hi);
            lc += cnt[i];
            if (lc == 0 || right_cnt[i + 1] == 0) continue;
            float cost = lacc.area() * lc + right_area[i + 1] * right_cnt[i + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = k; best_split = i + 1; }
        }
    }
    uint32_t mid;
    if (best_axis < 0) {
        mid = b + n / 2;
    } else {
        float ext = cbox.hi[best_axis] - cbox.lo[best_axis];
        auto it = std::partition(c.idx.begin() + b, c.idx.begin() + e, [&](uint32_t t) {
            int bi = (int)((c.cen[3 * t + best_axis] - cbox.lo[best_axis]) / ext * kBins);
            bi = std::min(std::max(bi, 0), kBins - 1);
            return bi < best_split;
        });
        mid = (uint32_t)(it - c.idx.begin());
        if (mid == b || mid == e) mid = b + n / 2;
    }
    out[me].count = 0;
    build_rec(c, b, mid, out);
    out[me].index = (int32_t)out.size();
    build_rec(c, mid, e, out);
}

inline bool slab(const Node &nd, const RayPre &r, float tmax, float &tnear) {
    float t0 = r.tmin, t1 = tmax + std::fabs(tmax) * 5e-7f;
    for (int k = 0; k < 3; ++k) {
        float ta = (nd.lo[k] - r.o[k]) * r.inv[k];
        float tb = (nd.hi[k] - r.o[k]) * r.inv[k];
        if (ta > tb) std::swap(ta, tb);
        tb = tb + std::fabs(tb) * 4e-7f;
        t0 = ta > t0 ? ta : t0;
        t1 = tb < t1 ? tb : t1;
    }
    tnear = t0;
    return t0 <= t1;
}

template <bool ANY>
void trace_one(const oracle_bvh &bvh, const float *ray, float *hit, uint8_t *occ) {
    RayPre r = make_ray(ray);
    float tmax = r.tmax, bb1 = 0.f, bb2 = 0.f;
    uint32_t best = kMiss;
    int stack[128];
    int sp = 0;
    float tn;
    if (!bvh.nodes.empty() && slab(bvh.nodes[0], r, tmax, tn)) stack[sp++] = 0;
    while (sp > 0) {
        const Node &nd = bvh.nodes[stack[--sp]];
        if (nd.count > 0) {
            for (int i = 0; i < nd.count; ++i) {
                uint32_t slot = (uint32_t)nd.index + i;
                const float *v = &bvh.tris[9 * (size_t)slot];
                float b1, b2;
                float t = tri_test(r, v, v + 3, v + 6, b1, b2);
                uint32_t gid = bvh.ids[slot];
                if (ANY) {
                    if (t > r.tmin && t <= tmax && (bvh.mask.empty() || bvh.mask[gid])) {
                        *occ = 1;
                        return;
                    }
                } else if (t > r.tmin && (t < tmax || (t == tmax && gid < best))) {
                    tmax = t; bb1 = b1; bb2 = b2; best = gid;
                }
            }
            continue;
        }
        int l = (int)(&nd - bvh.nodes.data()) + 1, rr = nd.index;
        float tl, tr;
        bool hl = slab(bvh.nodes[l], r, tmax, tl), hr = slab(bvh.nodes[rr], r, tmax, tr);
        if (sp + 2 > 128) { sp = 0; break; }
        if (hl && hr) {
            if (tl <= tr) { stack[sp++] = rr; stack[sp++] = l; }
            else { stack[sp++] = l; stack[sp++] = rr; }
        } else if (hl) stack[sp++] = l;
        else if (hr) stack[sp++] = rr;
    }
    if (ANY) { *occ = 0; return; }
    uint32_t bits = best;
    hit[0] = best == kMiss ? INFINITY : tmax;
    hit[1] = best == kMiss ? 0.f : bb1;
    hit[2] = best == kMiss ? 0.f : bb2;
    std::memcpy(&hit[3], &bits, 4);
}

template <typename F>
void parallel_for(int64_t n, int threads, F f) {
    if (threads <= 1 || n < 1024) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (;;) {
                int64_t s = next.fetch_add(256);
                if (s >= n) break;
                int64_t e = std::min<int64_t>(s + 256, n);
                for (int64_t i = s; i < e; ++i) f(i);
            }
        });
    for (auto &th : pool) th.join();
}

}  // namespace

extern "C" int oracle_bvh_build(const float *v, int64_t n, int threads, oracle_bvh **out) {
    (void)threads;
    auto *bvh = new oracle_bvh();
    BuildCtx c;
    c.v = v;
    c.idx.resize(n);
    c.clo.resize(3 * n);
    c.chi.resize(3 * n);
    c.cen.resize(3 * n);
    float mag = 0.f, lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; ++i) {
        c.idx[i] = (uint32_t)i;
        for (int k = 0; k < 3; ++k) {
            float a = v[9 * i + k], b = v[9 * i + 3 + k], d = v[9 * i + 6 + k];
            float l = std::min(a, std::min(b, d)), h = std::max(a, std::max(b, d));
            c.clo[3 * i + k] = l;
            c.chi[3 * i + k] = h;
            c.cen[3 * i + k] = (l + h) * 0.5f;
            lo[k] = std::min(lo[k], l);
            hi[k] = std::max(hi[k], h);
            mag = std::max(mag, std::max(std::fabs(l), std::fabs(h)));
        }
    }
    float ext = 0.f;
    for (int k = 0; k < 3; ++k) ext = std::max(ext, hi[k] - lo[k]);
    c.margin = std::ldexp(n ? mag + ext : 0.f, -19) + 1e-30f;
    for (int64_t i = 0; i < 3 * n; ++i) { c.clo[i] -= c.margin; c.chi[i] += c.margin; }
    if (n > 0) {
        bvh->nodes.reserve(2 * n / 2 + 16);
        build_rec(c, 0, (uint32_t)n, bvh->nodes);
    }
    bvh->tris.resize(9 * n);
    bvh->ids.resize(n);
    for (int64_t s = 0; s < n; ++s) {
        uint32_t t = c.idx[s];
        bvh->ids[s] = t;
        std::memcpy(&bvh->tris[9 * s], v + 9 * (size_t)t, 9 * sizeof(float));
    }
    *out = bvh;
    return 0;
}

extern "C" void oracle_bvh_free(oracle_bvh *bvh) { delete bvh; }

extern "C" void oracle_bvh_set_mask(oracle_bvh *bvh, const uint8_t *mask) {
    if (!mask) { bvh->mask.clear(); return; }
    bvh->mask.assign(mask, mask + bvh->ids.size());
}

extern "C" int oracle_trace_closest(const oracle_bvh *bvh, const float *rays, int64_t n,
                                    float *hits, int threads) {
    parallel_for(n, threads, [&](int64_t i) { trace_one<false>(*bvh, rays + 8 * i, hits + 4 * i, nullptr); });
    return 0;
}

extern "C" int oracle_trace_any(const oracle_bvh *bvh, const float *rays, int64_t n,
                                uint8_t *occluded, int threads) {
    parallel_for(n, threads, [&](int64_t i) { trace_one<true>(*bvh, rays + 8 * i, nullptr, occluded + i); });
    return 0;
}

// Two-level tracing: instance i draws geometry inst_geom[i] (object-space
// triangles [geom_begin[g], geom_begin[g + 1]) of v) through the
// world-to-object matrix inst_inv[12 i..]; the ray is carried into object
// space row by row (m0 x + m1 y + m2 z (+ m3), each operation rounded as
// written), the geometry's BVH gives the closest hit with t in (tmin, best
// t], and it replaces the best hit if its t is smaller or equal with a
// smaller global id (inst_first[i] + its index in the geometry).  Any-hit:
// some instance with a non-zero mask has a hit in (tmin, tmax].
extern "C" int oracle_trace_instanced(const float *v, const int64_t *geom_begin, int n_geoms,
                                      const int32_t *inst_geom, const float *inst_inv,
                                      const int64_t *inst_first, const uint8_t *inst_mask,
                                      int n_inst, const float *rays, int64_t n, float *hits,
                                      uint8_t *occluded, int threads) {
    std::vector<oracle_bvh *> geoms(n_geoms, nullptr);
    for (int g = 0; g < n_geoms; ++g)
        oracle_bvh_build(v + 9 * (size_t)geom_begin[g], geom_begin[g + 1] - geom_begin[g], 1, &geoms[g]);
    parallel_for(n, threads, [&](int64_t q) {
        const float *ray = rays + 8 * q;
        float best_t = ray[7], bb1 = 0.f, bb2 = 0.f;
        uint32_t best = kMiss;
        bool occ = false;
        for (int i = 0; i < n_inst && !occ; ++i) {
            if (occluded && inst_mask && !inst_mask[i]) continue;
            const float *m = inst_inv + 12 * (size_t)i;
            float oray[8];
            for (int r = 0; r < 3; ++r) {
                const float *row = m + 4 * r;
                float acc = row[0] * ray[0];
                acc = acc + row[1] * ray[1];
                acc = acc + row[2] * ray[2];
                oray[r] = acc + row[3];
                float dacc = row[0] * ray[4];
                dacc = dacc + row[1] * ray[5];
                oray[4 + r] = dacc + row[2] * ray[6];
            }
            oray[3] = ray[3];
            oray[7] = best_t;
            const oracle_bvh &g = *geoms[inst_geom[i]];
            if (occluded) {
                uint8_t o = 0;
                trace_one<true>(g, oray, nullptr, &o);
                occ = o != 0;
                continue;
            }
            float h[4];
            trace_one<false>(g, oray, h, nullptr);
            uint32_t local;
            std::memcpy(&local, &h[3], 4);
            if (local == kMiss) continue;
            const uint32_t gid = (uint32_t)inst_first[i] + local;
            if (h[0] < best_t || (h[0] == best_t && gid < best)) {
                best_t = h[0]; bb1 = h[1]; bb2 = h[2]; best = gid;
            }
        }
        if (occluded) { occluded[q] = occ ? 1 : 0; return; }
        float *hit = hits + 4 * q;
        hit[0] = best == kMiss ? INFINITY : best_t;
        hit[1] = best == kMiss ? 0.f : bb1;
        hit[2] = best == kMiss ? 0.f : bb2;
        std::memcpy(&hit[3], &best, 4);
    });
    for (auto *g : geoms) oracle_bvh_free(g);
    return 0;
}

extern "C" int oracle_trace_closest_brute(const float *v, int64_t n_tris, const float *rays,
                                          int64_t n, float *hits) {
    for (int64_t i = 0; i < n; ++i) {
        RayPre r = make_ray(rays + 8 * i);
        float tmax = r.tmax, bb1 = 0.f, bb2 = 0.f;
        uint32_t best = kMiss;
        for (int64_t t = 0; t < n_tris; ++t) {
            float b1, b2;
            const float *p = v + 9 * t;
            float th = tri_test(r, p, p + 3, p + 6, b1, b2);
            if (th > r.tmin && (th < tmax || (th == tmax && (uint32_t)t < best))) {
                tmax = th; bb1 = b1; bb2 = b2; best = (uint32_t)t;
            }
        }
        hits[4 * i + 0] = best == kMiss ? INFINITY : tmax;
        hits[4 * i + 1] = best == kMiss ? 0.f : bb1;
        hits[4 * i + 2] = best == kMiss ? 0.f : bb2;
        std::memcpy(&hits[4 * i + 3], &best, 4);
    }
    return 0;
}
