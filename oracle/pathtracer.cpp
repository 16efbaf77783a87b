// CPU restatement of the reference's WavefrontPathTracer (test infrastructure
// only; the checker for the CUDA path).
//
// Every stage of the wavefront (src/render/wavefront/integrator.cpp:50-267)
// touches only the state of the pixel that owns the queue item, and the
// stages run in a fixed order, so running one pixel's path through the same
// stages in the same order reproduces the wavefront result exactly: the
// per-pixel sampler stream sees the same draws, and radiance is added to
// L[pixel] in the same sequence (emission/miss of a bounce, then its shadow
// ray).  Media follow src/render/wavefront/medium.cpp and wavefront.h:34-139.
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/krr_gb300.h"
#include "oracle.h"
#include "pcg.h"
#include "shading.h"

using namespace oracle;

namespace {

struct Mesh {
    const float *pos, *nrm, *uv;
    const uint32_t *idx;
    int64_t n_tris;
    int32_t material, medium_inside, medium_outside;
};
struct Instance {
    float xf[12], nxf[9];
    int32_t mesh;
    uint32_t prim_offset;
    int32_t light_offset;
    float le[3], le_scale;
};
struct Material {
    int32_t type;
    float diffuse[3], spec_alpha, spec_trans, eta, anisotropic;
};
struct Light {
    int32_t kind, index;
    uint32_t prim;
};
struct Infinite {
    float tint[3], scale, rot[9];
    std::vector<float> image;
    int32_t w, h;
    float scene_radius;
};
struct Medium {
    std::vector<uint16_t> density;
    int32_t nx, ny, nz;
    float lo[3], hi[3], sigma_t[3], albedo[3], g, scale;
    int32_t mres[3];
    std::vector<float> majorant;
};

void inverse_transpose(const float *m, float *out) {
    double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    double D = -(b * i - c * h), E = a * i - c * g, F = -(a * h - b * g);
    double G = b * f - c * e, H = -(a * f - c * d), I = a * e - b * d;
    double det = a * A + b * B + c * C;
    double cof[9] = {A, B, C, D, E, F, G, H, I};
    for (int k = 0; k < 9; ++k) out[k] = (float)(cof[k] / det);
}

}  // namespace

struct oracle_pt {
    std::vector<Mesh> meshes;
    std::vector<Instance> instances;
    std::vector<Material> materials;
    std::vector<Light> lights;
    std::vector<Infinite> infinite;
    std::vector<Medium> media;
    std::vector<uint32_t> tri_instance;
    std::vector<float> world;
    oracle_bvh *bvh = nullptr;
    float scene_radius = 1.f;
    ~oracle_pt() { oracle_bvh_free(bvh); }
};

namespace {

struct Ray {
    V3 o, d;
    float tmax;
};

struct Hit {
    float t, b1, b2;
    uint32_t prim;
};

Hit trace(const oracle_pt &s, const Ray &r) {
    float ray[8] = {r.o.x, r.o.y, r.o.z, 0.f, r.d.x, r.d.y, r.d.z, r.tmax};
    float h[4];
    oracle_trace_closest(s.bvh, ray, 1, h, 1);
    Hit out;
    out.t = h[0];
    out.b1 = h[1];
    out.b2 = h[2];
    std::memcpy(&out.prim, &h[3], 4);
    return out;
}

bool occluded(const oracle_pt &s, V3 o, V3 d, float tmax) {
    float ray[8] = {o.x, o.y, o.z, 0.f, d.x, d.y, d.z, tmax};
    uint8_t occ = 0;
    oracle_trace_any(s.bvh, ray, 1, &occ, 1);
    return occ != 0;
}

struct Surf {
    V3 p, wo, n, t, b;
    float u, v;
    int32_t material, mesh, light, interface_in, interface_out;
};

// prepareSurfaceInteraction, src/render/shading.h:115-226
Surf prepare_surface(const oracle_pt &s, float b1, float b2, uint32_t gid, V3 ray_dir) {
    Surf o;
    const Instance &I = s.instances[s.tri_instance[gid]];
    const Mesh &M = s.meshes[I.mesh];
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
    o.u = o.v = 0.f;
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

// offsetRayOrigin, raytracing.h:106-111
V3 offset_ray_origin(V3 p, V3 n, V3 w) {
    V3 off = n * kRayEps;
    if (dot(n, w) < 0.f) off = -off;
    return p + off;
}

int32_t medium_towards(int32_t in, int32_t out, int32_t medium, V3 n, V3 w) {
    if (in != -2) return dot(w, n) > 0 ? out : in;
    return medium;
}

ShadingData shading_data(const oracle_pt &s, int32_t material) {
    const Material &m = s.materials[material];
    ShadingData sd;
    sd.type = m.type;
    sd.diffuse = V3{m.diffuse[0], m.diffuse[1], m.diffuse[2]};
    sd.roughness = 1.f - m.spec_alpha;
    sd.spec_trans = m.spec_trans;
    sd.ior = m.eta;
    sd.anisotropic = m.anisotropic;
    return sd;
}

void light_triangle(const oracle_pt &s, const Light &l, V3 &p0, V3 &p1, V3 &p2, uint32_t &i0,
                    uint32_t &i1, uint32_t &i2, const Instance *&I, const Mesh *&M) {
    I = &s.instances[l.index];
    M = &s.meshes[I->mesh];
    i0 = M->idx[3 * l.prim];
    i1 = M->idx[3 * l.prim + 1];
    i2 = M->idx[3 * l.prim + 2];
    p0 = V3{M->pos[3 * i0], M->pos[3 * i0 + 1], M->pos[3 * i0 + 2]};
    p1 = V3{M->pos[3 * i1], M->pos[3 * i1 + 1], M->pos[3 * i1 + 2]};
    p2 = V3{M->pos[3 * i2], M->pos[3 * i2 + 1], M->pos[3 * i2 + 2]};
}

// Triangle::area, shape.h:29-38
float tri_area(const Instance &I, V3 p0, V3 p1, V3 p2) {
    V3 w0 = xform_point(I.xf, p0), w1 = xform_point(I.xf, p1), w2 = xform_point(I.xf, p2);
    return 0.5f * length(cross(w1 - w0, w2 - w0));
}

// DiffuseAreaLight::L, light.h:182-188
V3 area_L(const Instance &I, V3 n, V3 w) {
    if (dot(n, w) < 0.f) return v3(0.f);
    return I.le_scale * V3{I.le[0], I.le[1], I.le[2]};
}

// Triangle::pdf(sample, ctx), shape.h:114-123
float area_pdf(const oracle_pt &s, const Light &l, V3 sp, V3 sn, V3 cp) {
    V3 p0, p1, p2;
    uint32_t i0, i1, i2;
    const Instance *I;
    const Mesh *M;
    light_triangle(s, l, p0, p1, p2, i0, i1, i2, I, M);
    V3 wi = normalize(sp - cp);
    float pdf = (1 / tri_area(*I, p0, p1, p2)) / (std::fabs(dot(sn, -wi)) / length_sq(cp - sp));
    if (length(wi) == 0 || std::isinf(pdf)) pdf = 0;
    return pdf;
}

// bilinear, wrap, normalised coordinates (texture.cpp:237-243)
V3 env_lookup(const Infinite &e, float u, float v) {
    float x = u * (float)e.w - 0.5f, y = v * (float)e.h - 0.5f;
    float fx0 = std::floor(x), fy0 = std::floor(y);
    float fx = x - fx0, fy = y - fy0;
    int x0 = (int)fx0, y0 = (int)fy0;
    int xa = ((x0 % e.w) + e.w) % e.w, xb = (((x0 + 1) % e.w) + e.w) % e.w;
    int ya = ((y0 % e.h) + e.h) % e.h, yb = (((y0 + 1) % e.h) + e.h) % e.h;
    auto px = [&](int yy, int xx) {
        const float *c = &e.image[4 * ((size_t)yy * e.w + xx)];
        return V3{c[0], c[1], c[2]};
    };
    V3 top = px(ya, xa) * (1.f - fx) + px(ya, xb) * fx;
    V3 bot = px(yb, xa) * (1.f - fx) + px(yb, xb) * fx;
    return top * (1.f - fy) + bot * fy;
}

// InfiniteLight::Li, light.h:242-247
V3 env_Li(const Infinite &e, V3 wi) {
    float u, v;
    world_to_latlong(mat3_mul_transposed(e.rot, wi), u, v);
    V3 tint{e.tint[0], e.tint[1], e.tint[2]};
    V3 L = e.image.empty() ? tint : tint * env_lookup(e, u, v);
    return e.scale * L;
}

struct LightSample {
    V3 p, n, L;
    float pdf;
};

// Light::sampleLi (light.h:167-180, 222-231; shape.h:54-108)
LightSample sample_li(const oracle_pt &s, const Light &l, float u0, float u1, V3 cp) {
    LightSample ls;
    if (l.kind == 1) {
        const Infinite &e = s.infinite[l.index];
        V3 wi = uniform_sample_sphere(u0, u1);
        ls.p = cp + wi * 2 * e.scene_radius;
        ls.n = v3(0.f);
        ls.L = env_Li(e, wi);
        ls.pdf = kInv4Pi;
        return ls;
    }
    V3 p0, p1, p2;
    uint32_t i0, i1, i2;
    const Instance *I;
    const Mesh *M;
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
    pdf = pdf / (std::fabs(dot(n, wi)) / length_sq(cp - p));
    if (length(wi) == 0 || std::isinf(pdf)) pdf = 0;
    ls.p = p;
    ls.n = n;
    ls.L = area_L(*I, n, normalize(cp - p));
    ls.pdf = pdf;
    return ls;
}


// ------------------------------------------------------------------ media
// Dense-grid restatement of NanoVDBMedium<float> (media.h:144-227),
// MajorantIterator (media.h:41-106), sampleT_maj (wavefront.h:34-78),
// initializeMajorantGrid (media.cpp:18-75) and HGPhaseFunction (media.cpp:83-111).
struct MediumProps {
    V3 sigma_a, sigma_s;
};

float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h >> 15) << 31, exp = (h >> 10) & 0x1f, man = h & 0x3ff, bits;
    if (exp == 0) {
        if (man == 0) bits = sign;
        else {   // subnormal half -> normal float
            int e = -1;
            do { ++e; man <<= 1; } while (!(man & 0x400));
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3ff) << 13);
        }
    } else if (exp == 31) bits = sign | 0x7f800000u | (man << 13);
    else bits = sign | ((exp - 15 + 127) << 23) | (man << 13);
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// Index-space point: offset, then a multiply by the voxels per unit length
// (an affine world-to-index map, as NanoVDB's worldToIndexF).
float density_at(const Medium &m, V3 p) {
    float fx = (p.x - m.lo[0]) * ((float)m.nx / (m.hi[0] - m.lo[0])) - 0.5f;
    float fy = (p.y - m.lo[1]) * ((float)m.ny / (m.hi[1] - m.lo[1])) - 0.5f;
    float fz = (p.z - m.lo[2]) * ((float)m.nz / (m.hi[2] - m.lo[2])) - 0.5f;
    float ix = std::floor(fx), iy = std::floor(fy), iz = std::floor(fz);
    float u = fx - ix, v = fy - iy, w = fz - iz;
    int x0 = (int)ix, y0 = (int)iy, z0 = (int)iz;
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int e = 0; e < 2; ++e) {
                int x = x0 + a, y = y0 + b, z = z0 + e;
                bool in = x >= 0 && y >= 0 && z >= 0 && x < m.nx && y < m.ny && z < m.nz;
                c[a][b][e] = in ? half_to_float(m.density[((size_t)z * m.ny + y) * m.nx + x]) : 0.f;
            }
    auto lerp = [](float a, float b, float t) { return a + t * (b - a); };
    return lerp(lerp(lerp(c[0][0][0], c[0][0][1], w), lerp(c[0][1][0], c[0][1][1], w), v),
                lerp(lerp(c[1][0][0], c[1][0][1], w), lerp(c[1][1][0], c[1][1][1], w), v), u);
}

MediumProps sample_point(const Medium &m, V3 p) {
    V3 st{m.sigma_t[0], m.sigma_t[1], m.sigma_t[2]};
    V3 sigma_t = !m.density.empty() ? (density_at(m, p) * m.scale) * st : st;
    V3 sigma_s = sigma_t * V3{m.albedo[0], m.albedo[1], m.albedo[2]};
    return MediumProps{sigma_t - sigma_s, sigma_s};
}

bool box_intersect(const float *lo, const float *hi, V3 o, V3 d, float tmax, float &t0, float &t1) {
    t0 = 0.f;
    t1 = tmax;
    for (int i = 0; i < 3; ++i) {
        float inv = 1 / get(d, i);
        float tn = (lo[i] - get(o, i)) * inv;
        float tf = (hi[i] - get(o, i)) * inv;
        if (tn > tf) std::swap(tn, tf);
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return false;
    }
    return true;
}

struct MajorantSeg {
    float tmin, tmax;
    V3 sigma_maj;
};

struct MajorantIter {
    float tmin = 3.402823466e38f, tmax = 1.175494351e-38f;
    V3 sigma_t{0, 0, 0};
    const Medium *m = nullptr;
    float next_cross[3], delta_t[3];
    int step[3], limit[3], voxel[3];

    void init(const Medium &med, V3 o, V3 d, float ray_tmax) {
        V3 st{med.sigma_t[0], med.sigma_t[1], med.sigma_t[2]};
        if (med.density.empty()) {
            tmin = 0.f;
            tmax = ray_tmax;
            sigma_t = st;
            return;
        }
        float t0, t1;
        if (!box_intersect(med.lo, med.hi, o, d, ray_tmax, t0, t1)) return;
        tmin = t0;
        tmax = t1;
        sigma_t = med.scale * st;
        m = &med;
        float diag[3] = {med.hi[0] - med.lo[0], med.hi[1] - med.lo[1], med.hi[2] - med.lo[2]};
        float go[3], gd[3];
        for (int a = 0; a < 3; ++a) {
            go[a] = (get(o, a) - med.lo[a]) / (diag[a] == 0.f ? 1.f : diag[a]);
            gd[a] = get(d, a) / diag[a];
        }
        for (int a = 0; a < 3; ++a) {
            float gi = go[a] + gd[a] * tmin;
            float res = (float)med.mres[a];
            voxel[a] = (int)std::fmin(std::fmax(gi * res, 0.f), res - 1.f);
            delta_t[a] = 1.f / (std::fabs(gd[a]) * res);
            if (gd[a] == -0.f) gd[a] = 0.f;
            if (gd[a] >= 0) {
                float nvp = (float)(voxel[a] + 1) / res;
                next_cross[a] = tmin + (nvp - gi) / gd[a];
                step[a] = 1;
                limit[a] = med.mres[a];
            } else {
                float nvp = (float)voxel[a] / res;
                next_cross[a] = tmin + (nvp - gi) / gd[a];
                step[a] = -1;
                limit[a] = -1;
            }
        }
    }

    bool next(MajorantSeg &seg) {
        if (tmin >= tmax) return false;
        if (!m) {
            seg = MajorantSeg{tmin, tmax, sigma_t};
            tmin = tmax;
            return true;
        }
        int bits = ((next_cross[0] < next_cross[1]) << 2) + ((next_cross[0] < next_cross[2]) << 1) +
                   (next_cross[1] < next_cross[2]);
        const int cmp_to_axis[8] = {2, 1, 2, 1, 2, 2, 0, 0};
        int ax = cmp_to_axis[bits];
        float exit = std::fmin(tmax, next_cross[ax]);
        float maj = m->majorant[voxel[0] + m->mres[0] * (voxel[1] + m->mres[1] * voxel[2])];
        seg = MajorantSeg{tmin, exit, sigma_t * maj};
        tmin = exit;
        if (next_cross[ax] > tmax) tmin = tmax;
        voxel[ax] += step[ax];
        if (voxel[ax] == limit[ax]) tmin = tmax;
        next_cross[ax] += delta_t[ax];
        return true;
    }
};

void build_majorant(Medium &m) {
    size_t n = (size_t)m.mres[0] * m.mres[1] * m.mres[2];
    m.majorant.assign(n, 0.f);
    int dims[3] = {m.nx, m.ny, m.nz};
    for (size_t idx = 0; idx < n; ++idx) {
        int c[3] = {(int)(idx % m.mres[0]), (int)((idx / m.mres[0]) % m.mres[1]),
                    (int)(idx / ((size_t)m.mres[0] * m.mres[1]))};
        int r0[3], r1[3];
        for (int a = 0; a < 3; ++a) {
            float diag = m.hi[a] - m.lo[a];
            float cl = m.lo[a] + ((float)c[a] / (float)m.mres[a]) * diag;
            float ch = m.lo[a] + ((float)(c[a] + 1) / (float)m.mres[a]) * diag;
            float i0 = (cl - m.lo[a]) / diag * (float)dims[a] - 0.5f;
            float i1 = (ch - m.lo[a]) / diag * (float)dims[a] - 0.5f;
            r0[a] = std::max((int)(i0 - 1.f), 0);
            r1[a] = std::min((int)(i1 + 1.f), dims[a] - 1);
        }
        float mx = 0.f;
        for (int k = r0[2]; k <= r1[2]; ++k)
            for (int j = r0[1]; j <= r1[1]; ++j)
                for (int i = r0[0]; i <= r1[0]; ++i)
                    mx = std::fmax(mx, half_to_float(m.density[((size_t)k * m.ny + j) * m.nx + i]));
        m.majorant[idx] = mx;
    }
}

int main_index(float lambda0) {
    int c = (int)((lambda0 - 360.f) / (830.f - 360.f) * 3);
    return c < 0 ? 0 : (c > 2 ? 2 : c);
}

float next_float_down(float v) {
    if (std::isinf(v) && v < 0.f) return v;
    if (v == 0.f) v = -0.f;
    uint32_t ui;
    std::memcpy(&ui, &v, 4);
    if (v > 0) --ui;
    else ++ui;
    std::memcpy(&v, &ui, 4);
    return v;
}

int sample_discrete3(float w0, float w1, float w2, float u) {
    float w[3] = {w0, w1, w2};
    float sum = 0;
    for (int i = 0; i < 3; ++i) sum += w[i];
    float up = u * sum;
    if (up == sum) up = next_float_down(up);
    int off = 0;
    float acc = 0;
    while (off < 2 && acc + w[off] <= up) acc += w[off++];
    return off;
}

float hg_p(float g, V3 wo, V3 wi) {
    g = std::fmin(std::fmax(g, -.99f), .99f);
    float denom = 1 + g * g + 2 * g * dot(wo, wi);
    return kInv4Pi * (1 - g * g) / (denom * std::sqrt(std::fmax(0.f, denom)));
}

V3 hg_sample(float g0, V3 wo, float u0, float u1, float &pdf) {
    float g = std::fmin(std::fmax(g0, -.99f), .99f);
    float cos_t;
    if (std::fabs(g) < 1e-3f) cos_t = 1 - 2 * u0;
    else {
        float q = (1 - g * g) / (1 + g - 2 * g * u0);
        cos_t = -1 / (2 * g) * (1 + g * g - q * q);
    }
    float sin_t = std::sqrt(std::fmax(0.f, 1 - cos_t * cos_t));
    float phi = k2Pi * u1;
    V3 n = normalize(wo);
    V3 t = get_perpendicular(n);
    V3 b = normalize(cross(n, t));
    V3 v{sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t};
    V3 wi = t * v.x + b * v.y + n * v.z;
    pdf = hg_p(g0, normalize(wo), wi);
    return wi;
}

template <typename F>
V3 sample_t_maj(const Medium &m, V3 o, V3 d, float tmax, Pcg &rng, int ch, bool &aborted, F &&cb) {
    aborted = false;
    tmax *= length(d);
    d = normalize(d);
    V3 T_maj = v3(1.f);
    MajorantIter it;
    it.init(m, o, d, tmax);
    int guard = 0;
    while (true) {
        MajorantSeg seg;
        if (!it.next(seg)) return T_maj;
        if (get(seg.sigma_maj, ch) == 0.f) {
            float dt = seg.tmax - seg.tmin;
            if (std::isinf(dt)) dt = 3.402823466e38f;
            T_maj = T_maj * vexp(-dt * seg.sigma_maj);
            continue;
        }
        float tmin = seg.tmin;
        while (true) {
            if (++guard > (1 << 20)) { aborted = true; return v3(1.f); }
            float u = rng.get1d();
            float t = tmin + (-std::log(1 - u) / get(seg.sigma_maj, ch));
            if (t < seg.tmax) {
                T_maj = T_maj * vexp(-(t - tmin) * seg.sigma_maj);
                V3 p = o + d * t;
                MediumProps mp = sample_point(m, p);
                if (!cb(p, mp, seg.sigma_maj, T_maj)) return v3(1.f);
                T_maj = v3(1.f);
                tmin = t;
            } else {
                float dt = seg.tmax - tmin;
                if (std::isinf(dt)) dt = 3.402823466e38f;
                T_maj = T_maj * vexp(-dt * seg.sigma_maj);
                break;
            }
        }
    }
}

struct PathState {
    Ray ray;
    V3 ctx_p, ctx_n, thp, pu, pl;
    uint32_t bsdf_type, depth;
    int32_t medium;
    float time;
};

struct Camera {
    V3 pos;
    float rot[9];
    float tan_fov, aspect, shutter_open, shutter_time;
    int32_t medium;
};

// Transmittance of one shadow ray (traceTransmittance, wavefront.h:80-139).
V3 shadow_transmittance(const oracle_pt &s, V3 o, V3 d, float tmax, int32_t medium, Pcg &rng, int ch,
                        V3 &pu, V3 &pl) {
    V3 p_light = o + d * tmax;
    V3 T_ray = v3(1.f);
    pu = v3(1.f);
    pl = v3(1.f);
    int crossings = 0;
    while (std::fabs(d.x) > kRayEps * 2 || std::fabs(d.y) > kRayEps * 2 || std::fabs(d.z) > kRayEps * 2) {
        Hit h = trace(s, Ray{o, d, tmax});
        bool visible = h.prim == 0xFFFFFFFFu;
        Surf sf{};
        if (!visible) {
            sf = prepare_surface(s, h.b1, h.b2, h.prim, d);
            if (sf.material >= 0) { T_ray = v3(0.f); break; }
        }
        if (medium >= 0) {
            float t_end = visible ? tmax : length(sf.p - o) / length(d);
            bool aborted;
            V3 T_maj = sample_t_maj(s.media[medium], o, d, t_end, rng, ch, aborted,
                [&](V3, const MediumProps &mp, V3 sigma_maj, V3 Tm) -> bool {
                    V3 sigma_n = vmax(sigma_maj - mp.sigma_a - mp.sigma_s, v3(0.f));
                    float pr = get(Tm, ch) * get(sigma_maj, ch);
                    T_ray = T_ray * (Tm * sigma_n / pr);
                    pl = pl * (Tm * sigma_maj / pr);
                    pu = pu * (Tm * sigma_n / pr);
                    V3 Tr = T_ray / mean(pu + pl);
                    if (max_coeff(Tr) < 0.05f) {
                        if (rng.get1d() < 0.75f) T_ray = v3(0.f);
                        else T_ray = T_ray / 0.25f;
                    }
                    return any(T_ray);
                });
            if (aborted) T_ray = v3(0.f);
            V3 r = T_maj / get(T_maj, ch);
            T_ray = T_ray * r;
            pu = pu * r;
            pl = pl * r;
        }
        if (visible || !any(T_ray)) break;
        V3 po = offset_ray_origin(sf.p, sf.n, p_light - sf.p);
        V3 nd = p_light - po;
        medium = medium_towards(sf.interface_in, sf.interface_out, medium, sf.n, nd);
        o = po;
        d = nd;
        if (++crossings > 64) { T_ray = v3(0.f); break; }
    }
    return T_ray;
}

struct ScatterItem {
    Surf sf;
    V3 thp, pu;
    uint32_t depth;
    int32_t medium;
    float time;
};

// One pixel through the wavefront stages; returns L (the reference's
// PixelState::L after the frame) and accumulates `pixel`.
void render_pixel(const oracle_pt &s, const krr_wf_params &prm, const Camera &cam, int w, int h,
                  int64_t pixel_id, uint32_t sample_index, V3 &L_out, V3 &pixel_out) {
    uint32_t x = (uint32_t)(pixel_id % w), y = (uint32_t)(pixel_id / w);
    Pcg rng;
    rng.set_seed(interleave_32bit(x, y), sample_index);
    rng.advance(256 * pixel_id);
    float ul = rng.get1d();
    float lambda0 = (1.f - ul) * 360.f + ul * 830.f;
    const int ch = main_index(lambda0);
    const bool media_on = prm.enable_medium && !s.media.empty();
    V3 L = v3(0.f), pixel = v3(0.f);
    const float lsel_pdf = 1.f / (float)s.lights.size();
    for (int spp = 0; spp < prm.spp; ++spp) {
        // generateCameraRays
        float fx = rng.get1d(), fy = rng.get1d();
        rng.get1d();
        rng.get1d();
        float tm = rng.get1d();
        float px = (float)x + 0.5f + fx, py = (float)y + 0.5f + fy;
        float ndcx = (2 * px) / (float)w + (-1.f);
        float ndcy = (2 * py) / (float)h + (-1.f);
        V3 fd = normalize(V3{cam.tan_fov * cam.aspect * ndcx, cam.tan_fov * ndcy, -1.f});
        PathState ps;
        ps.ray = Ray{cam.pos, mat3_mul(cam.rot, fd), INFINITY};
        ps.ctx_p = ps.ctx_n = v3(0.f);
        ps.thp = ps.pu = ps.pl = v3(1.f);
        ps.bsdf_type = 0;
        ps.depth = 0;
        ps.medium = cam.medium;
        ps.time = cam.shutter_open + cam.shutter_time * tm;
        for (int depth = 0;; ++depth) {
            Hit hit = trace(s, ps.ray);
            bool has_scatter = false, has_mscatter = false, has_hitl = false, has_miss = false;
            bool next_pending = false;
            ScatterItem sc{};
            PathState next{}, hl{}, ms{};
            Surf hl_sf{};
            V3 msc_p{}, msc_wo{}, msc_thp{}, msc_pu{};
            int32_t msc_medium = -1;
            uint32_t msc_depth = 0;
            if (media_on && ps.medium >= 0) {
                // sampleMediumInteraction
                const Medium &m = s.media[ps.medium];
                V3 thp = ps.thp, pu = ps.pu, pl = ps.pl;
                bool scattered = false, aborted;
                float tmax_hit = hit.prim == 0xFFFFFFFFu ? INFINITY : hit.t;
                V3 T_maj = sample_t_maj(m, ps.ray.o, ps.ray.d, tmax_hit, rng, ch, aborted,
                    [&](V3 p, const MediumProps &mp, V3 sigma_maj, V3 Tm) -> bool {
                        float pa = get(mp.sigma_a, ch) / get(sigma_maj, ch);
                        float pscat = get(mp.sigma_s, ch) / get(sigma_maj, ch);
                        float pn = std::fmax(0.f, 1.f - pa - pscat);
                        int mode = sample_discrete3(pa, pscat, pn, rng.get1d());
                        if (mode == 0) { thp = v3(0.f); return false; }
                        if (mode == 1) {
                            float pr = get(Tm, ch) * get(mp.sigma_s, ch);
                            thp = thp * (Tm * mp.sigma_s / pr);
                            pu = pu * (Tm * mp.sigma_s / pr);
                            if (any(thp) && any(pu)) {
                                has_mscatter = true;
                                msc_p = p; msc_wo = -ps.ray.d; msc_thp = thp; msc_pu = pu;
                                msc_medium = ps.medium; msc_depth = ps.depth;
                            }
                            scattered = true;
                            return false;
                        }
                        V3 sigma_n = vmax(sigma_maj - mp.sigma_a - mp.sigma_s, v3(0.f));
                        float pr = get(Tm, ch) * get(sigma_n, ch);
                        thp = thp * (Tm * sigma_n / pr);
                        if (pr == 0) thp = v3(0.f);
                        pu = pu * (Tm * sigma_n / pr);
                        pl = pl * (Tm * sigma_maj / pr);
                        return any(thp) && any(pu);
                    });
                if (aborted) thp = v3(0.f);
                if (!scattered && any(thp)) {
                    V3 r = T_maj / get(T_maj, ch);
                    thp = thp * r;
                    pu = pu * r;
                    pl = pl * r;
                }
                if (!(scattered || !any(thp) || !any(pu) || (int)ps.depth == prm.max_depth)) {
                    PathState cur = ps;
                    cur.thp = thp; cur.pu = pu; cur.pl = pl;
                    if (std::isinf(tmax_hit)) {
                        has_miss = true;
                        ms = cur;
                    } else {
                        Surf sf = prepare_surface(s, hit.b1, hit.b2, hit.prim, ps.ray.d);
                        if (sf.material < 0) {
                            next = cur;
                            next.ray = Ray{offset_ray_origin(sf.p, sf.n, ps.ray.d), ps.ray.d, INFINITY};
                            next.medium = medium_towards(sf.interface_in, sf.interface_out, ps.medium, sf.n, ps.ray.d);
                            next_pending = true;
                        } else {
                            if (sf.light >= 0) { has_hitl = true; hl = cur; hl_sf = sf; }
                            has_scatter = true;
                            sc = ScatterItem{sf, thp, pu, ps.depth, ps.medium, ps.time};
                        }
                    }
                }
            } else if (hit.prim == 0xFFFFFFFFu) {
                has_miss = true;
                ms = ps;
            } else {
                Surf sf = prepare_surface(s, hit.b1, hit.b2, hit.prim, ps.ray.d);
                if (sf.material < 0) {
                    next = ps;
                    next.ray = Ray{offset_ray_origin(sf.p, sf.n, ps.ray.d), ps.ray.d, INFINITY};
                    next.medium = medium_towards(sf.interface_in, sf.interface_out, ps.medium, sf.n, ps.ray.d);
                    next_pending = true;
                } else {
                    if (sf.light >= 0) { has_hitl = true; hl = ps; hl_sf = sf; }
                    if (any(ps.thp)) {
                        has_scatter = true;
                        sc = ScatterItem{sf, ps.thp, ps.pu, ps.depth, ps.medium, ps.time};
                    }
                }
            }
            // handleHit
            if (has_hitl) {
                const Light &l = s.lights[hl_sf.light];
                const Instance &I = s.instances[l.index];
                V3 Le = area_L(I, hl_sf.n, hl_sf.wo) * hl.thp;
                if (prm.nee && hl.depth && !(hl.bsdf_type & BSDF_DELTA)) {
                    float light_pdf = area_pdf(s, l, hl_sf.p, hl_sf.n, hl.ctx_p) * lsel_pdf;
                    Le = Le / mean(hl.pl * light_pdf + hl.pu);
                } else {
                    Le = Le / mean(hl.pu);
                }
                L = Le + L;
            }
            // handleMiss
            if (has_miss && !s.infinite.empty()) {
                V3 Lm = v3(0.f);
                for (const Infinite &e : s.infinite) {
                    if (prm.nee && ms.depth && !(ms.bsdf_type & BSDF_DELTA)) {
                        float light_pdf = kInv4Pi * lsel_pdf;
                        Lm = Lm + env_Li(e, ms.ray.d) / mean(ms.pu + ms.pl * light_pdf);
                    } else {
                        Lm = Lm + env_Li(e, ms.ray.d) / mean(ms.pu);
                    }
                }
                L = ms.thp * Lm + L;
            }
            if (depth == prm.max_depth) break;
            bool shadow_pending = false;
            V3 sh_o{}, sh_d{}, sh_Ld{}, sh_pu{}, sh_pl{};
            int32_t sh_medium = -1;
            if (has_mscatter) {
                // sampleMediumScattering
                float g = s.media[msc_medium].g;
                if (prm.nee && !s.lights.empty()) {
                    float u = rng.get1d();
                    uint32_t lid = (uint32_t)(u * (float)s.lights.size());
                    float u0 = rng.get1d();
                    float u1 = rng.get1d();
                    LightSample ls = sample_li(s, s.lights[lid], u0, u1, msc_p);
                    V3 to = offset_ray_origin(ls.p, ls.n, msc_p - ls.p);
                    V3 d = to - msc_p;
                    V3 wi = normalize(d);
                    V3 thp = msc_thp * hg_p(g, msc_wo, wi);
                    float light_pdf = lsel_pdf * ls.pdf;
                    float phase_pdf = hg_p(g, msc_wo, wi);
                    V3 Ld = thp * ls.L;
                    if (any(Ld) && light_pdf > 0) {
                        shadow_pending = true;
                        sh_o = msc_p; sh_d = d; sh_Ld = Ld;
                        sh_pu = msc_pu * phase_pdf;
                        sh_pl = msc_pu * light_pdf;
                        sh_medium = msc_medium;
                    }
                }
                float u0 = rng.get1d();
                float u1 = rng.get1d();
                float pdf;
                V3 wi = hg_sample(g, msc_wo, u0, u1, pdf);
                V3 thp = msc_thp * pdf / pdf;
                float rr = max_coeff(thp / mean(msc_pu));
                bool killed = false;
                if (msc_depth >= 1 && rr < 1) {
                    if (rng.get1d() >= rr) killed = true;
                    else thp = thp / rr;
                }
                bool nan = std::isnan(thp.x) || std::isnan(thp.y) || std::isnan(thp.z);
                if (!killed && any(thp) && !nan) {
                    next.ray = Ray{msc_p, wi, INFINITY};
                    next.ctx_p = msc_p;
                    next.ctx_n = v3(0.f);
                    next.thp = thp;
                    next.pu = msc_pu;
                    next.pl = msc_pu / pdf;
                    next.bsdf_type = BSDF_SMOOTH;
                    next.depth = msc_depth + 1;
                    next.medium = msc_medium;
                    next.time = ps.time;
                    next_pending = true;
                }
            }
            if (has_scatter) {
                // generateScatterRays
                const Surf &sf = sc.sf;
                if (rng.get1d() < prm.rr) {
                    V3 thp = sc.thp / prm.rr;
                    auto to_local = [&](V3 v) { return V3{dot(sf.t, v), dot(sf.b, v), dot(sf.n, v)}; };
                    V3 wo_local = to_local(sf.wo);
                    ShadingData sd = shading_data(s, sf.material);
                    uint32_t bt = bsdf_type_of(sd);
                    Bsdf bsdf = Bsdf::setup(sd);
                    if (prm.nee && (bt & BSDF_SMOOTH) && !s.lights.empty()) {
                        float u = rng.get1d();
                        uint32_t lid = (uint32_t)(u * (float)s.lights.size());
                        float u0 = rng.get1d();
                        float u1 = rng.get1d();
                        LightSample ls = sample_li(s, s.lights[lid], u0, u1, sf.p);
                        V3 to = offset_ray_origin(ls.p, ls.n, sf.p - ls.p);
                        V3 po = offset_ray_origin(sf.p, sf.n, to - sf.p);
                        V3 d = to - po;
                        V3 wi_local = to_local(normalize(d));
                        float light_pdf = lsel_pdf * ls.pdf;
                        V3 fv = bsdf.f(wo_local, wi_local);
                        float bsdf_pdf = bsdf.pdf(wo_local, wi_local);
                        if (light_pdf > 0 && any(fv)) {
                            V3 Ld = ls.L * thp * fv * std::fabs(wi_local.z);
                            if (any(Ld)) {
                                shadow_pending = true;
                                sh_o = po; sh_d = d; sh_Ld = Ld;
                                sh_pu = sc.pu * bsdf_pdf;
                                sh_pl = sc.pu * light_pdf;
                                sh_medium = medium_towards(sf.interface_in, sf.interface_out, sc.medium, sf.n, d);
                            }
                        }
                    }
                    BsdfSample bs = bsdf.sample(wo_local, [&]() { return rng.get1d(); });
                    if (bs.pdf != 0 && any(bs.f)) {
                        V3 wi_world = sf.t * bs.wi.x + sf.b * bs.wi.y + sf.n * bs.wi.z;
                        V3 nthp = thp * bs.f * std::fabs(bs.wi.z) / bs.pdf;
                        if (any(nthp)) {
                            next.ray = Ray{offset_ray_origin(sf.p, sf.n, wi_world), wi_world, INFINITY};
                            next.ctx_p = sf.p;
                            next.ctx_n = sf.n;
                            next.thp = nthp;
                            next.pu = sc.pu;
                            next.pl = sc.pu / bs.pdf;
                            next.bsdf_type = bs.flags;
                            next.depth = sc.depth + 1;
                            next.medium = medium_towards(sf.interface_in, sf.interface_out, sc.medium, sf.n, wi_world);
                            next.time = sc.time;
                            next_pending = true;
                        }
                    }
                }
            }
            // traceShadow
            if (shadow_pending && prm.nee) {
                if (media_on) {
                    V3 tpu, tpl;
                    V3 T = shadow_transmittance(s, sh_o, sh_d, 1.f, sh_medium, rng, ch, tpu, tpl);
                    if (any(T)) L = sh_Ld * T / mean(sh_pu * tpu + sh_pl * tpl) + L;
                } else if (!occluded(s, sh_o, sh_d, 1.f)) {
                    L = sh_Ld / mean(sh_pl + sh_pu) + L;
                }
            }
            if (!next_pending) break;
            ps = next;
        }
        pixel = pixel + L;
        // the reference keeps L across the samples of a frame
        // (integrator.cpp:205-221, 255-258); independent_samples clears it
        if (prm.independent_samples && spp + 1 < prm.spp) L = v3(0.f);
    }
    L_out = L;
    pixel_out = pixel;
}

}  // namespace

extern "C" int oracle_pt_create(const krr_scene_desc *sd, int threads, oracle_pt **out) {
    auto *s = new oracle_pt();
    for (int i = 0; i < sd->n_meshes; ++i) {
        const krr_mesh_desc &m = sd->meshes[i];
        s->meshes.push_back(Mesh{m.h_positions, m.h_normals, m.h_texcoords, m.h_indices,
                                 m.n_triangles, m.material, m.medium_inside, m.medium_outside});
    }
    for (int i = 0; i < sd->n_materials; ++i) {
        const krr_material_desc &m = sd->materials[i];
        Material d;
        d.type = m.type;
        for (int k = 0; k < 3; ++k) d.diffuse[k] = m.diffuse[k];
        d.spec_alpha = 1.f - m.roughness;
        d.spec_trans = m.specular_transmission;
        d.eta = m.eta;
        d.anisotropic = m.anisotropic;
        s->materials.push_back(d);
    }
    uint32_t n_tris = 0;
    for (int i = 0; i < sd->n_instances; ++i) {
        const krr_instance_desc &in = sd->instances[i];
        const krr_mesh_desc &m = sd->meshes[in.mesh];
        Instance d{};
        std::memcpy(d.xf, in.transform, sizeof(d.xf));
        inverse_transpose(in.transform, d.nxf);
        d.mesh = in.mesh;
        d.prim_offset = n_tris;
        d.light_offset = -1;
        if (m.emission[0] > 0.f || m.emission[1] > 0.f || m.emission[2] > 0.f) {
            float scale = std::max(m.emission[0], std::max(m.emission[1], m.emission[2]));
            for (int k = 0; k < 3; ++k) d.le[k] = m.emission[k] / scale;
            d.le_scale = scale;
            d.light_offset = (int32_t)s->lights.size();
            for (int64_t t = 0; t < m.n_triangles; ++t) s->lights.push_back(Light{0, i, (uint32_t)t});
        }
        s->instances.push_back(d);
        for (int64_t t = 0; t < m.n_triangles; ++t) s->tri_instance.push_back((uint32_t)i);
        n_tris += (uint32_t)m.n_triangles;
    }
    // world-space triangles: m0*x + m1*y + m2*z + m3 per row, unfused
    s->world.resize(9 * (size_t)n_tris);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t g = 0; g < n_tris; ++g) {
        const Instance &I = s->instances[s->tri_instance[g]];
        const Mesh &M = s->meshes[I.mesh];
        uint32_t prim = g - I.prim_offset;
        for (int k = 0; k < 3; ++k) {
            uint32_t vi = M.idx[3 * prim + k];
            float x = M.pos[3 * vi], y = M.pos[3 * vi + 1], z = M.pos[3 * vi + 2];
            for (int r = 0; r < 3; ++r) {
                const float *m = I.xf + 4 * r;
                float acc = m[0] * x;
                acc = acc + m[1] * y;
                acc = acc + m[2] * z;
                float v = acc + m[3];
                s->world[9 * (size_t)g + 3 * k + r] = v;
                lo[r] = std::min(lo[r], v);
                hi[r] = std::max(hi[r], v);
            }
        }
    }
    oracle_bvh_build(s->world.data(), n_tris, threads, &s->bvh);
    std::vector<uint8_t> mask(n_tris);
    for (uint32_t g = 0; g < n_tris; ++g)
        mask[g] = s->meshes[s->instances[s->tri_instance[g]].mesh].material >= 0 ? 1 : 0;
    oracle_bvh_set_mask(s->bvh, mask.data());
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    s->scene_radius = std::sqrt(dx * dx + dy * dy + dz * dz);
    for (int i = 0; i < sd->n_infinite_lights; ++i) {
        const krr_infinite_light_desc &l = sd->infinite_lights[i];
        Infinite e;
        for (int k = 0; k < 3; ++k) e.tint[k] = l.tint[k];
        e.scale = l.scale;
        std::memcpy(e.rot, l.rotation, sizeof(e.rot));
        e.w = l.width;
        e.h = l.height;
        if (l.h_image) e.image.assign(l.h_image, l.h_image + 4 * (size_t)l.width * l.height);
        e.scene_radius = s->scene_radius;
        s->infinite.push_back(std::move(e));
        s->lights.push_back(Light{1, i, 0});
    }
    for (int i = 0; i < sd->n_media; ++i) {
        const krr_medium_desc &m = sd->media[i];
        Medium d;
        d.nx = m.nx; d.ny = m.ny; d.nz = m.nz;
        for (int k = 0; k < 3; ++k) {
            d.lo[k] = m.bounds_min[k]; d.hi[k] = m.bounds_max[k];
            d.sigma_t[k] = m.sigma_t[k]; d.albedo[k] = m.albedo[k];
            d.mres[k] = std::max(1, m.majorant_res[k]);
        }
        d.g = m.g;
        d.scale = m.scale;
        if (m.h_density) {
            d.density.assign(m.h_density, m.h_density + (size_t)m.nx * m.ny * m.nz);
            build_majorant(d);
        }
        s->media.push_back(std::move(d));
    }
    *out = s;
    return 0;
}

extern "C" void oracle_pt_free(oracle_pt *s) { delete s; }

// Light sampling of the restatement (known-answer tests): n samples of light
// `light` seen from cp, from u[n][2]; out[n][8] = p xyz, L rgb, solid-angle
// pdf, and the pdf that area_pdf() gives the same point (MIS side).
extern "C" int oracle_light_sample(const oracle_pt *s, int32_t light, const float *cp, const float *u,
                                   int64_t n, float *out) {
    if (light < 0 || light >= (int32_t)s->lights.size()) return 1;
    const Light &l = s->lights[light];
    const V3 c{cp[0], cp[1], cp[2]};
    for (int64_t i = 0; i < n; ++i) {
        const LightSample ls = sample_li(*s, l, u[2 * i], u[2 * i + 1], c);
        float *r = out + 8 * i;
        r[0] = ls.p.x; r[1] = ls.p.y; r[2] = ls.p.z;
        r[3] = ls.L.x; r[4] = ls.L.y; r[5] = ls.L.z;
        r[6] = ls.pdf;
        r[7] = l.kind == 0 ? area_pdf(*s, l, ls.p, ls.n, c) : kInv4Pi;
    }
    return 0;
}

extern "C" int32_t oracle_light_count(const oracle_pt *s) { return (int32_t)s->lights.size(); }

// Henyey-Greenstein phase function of the restatement (known-answer tests).
extern "C" float oracle_hg_p(float g, const float *wo, const float *wi) {
    return hg_p(g, V3{wo[0], wo[1], wo[2]}, V3{wi[0], wi[1], wi[2]});
}

// n samples of the HG phase function around wo; out[n][4] = wi xyz, pdf
extern "C" void oracle_hg_sample(float g, const float *wo, const float *u, int64_t n, float *out) {
    const V3 o{wo[0], wo[1], wo[2]};
    for (int64_t i = 0; i < n; ++i) {
        float pdf = 0.f;
        const V3 wi = hg_sample(g, o, u[2 * i], u[2 * i + 1], pdf);
        out[4 * i] = wi.x; out[4 * i + 1] = wi.y; out[4 * i + 2] = wi.z; out[4 * i + 3] = pdf;
    }
}

// Mean of the ratio-tracking transmittance estimator along one segment inside
// medium 0 of the scene (no surfaces), over n independent PCG streams.
extern "C" double oracle_medium_transmittance(const oracle_pt *s, const float *o, const float *d,
                                              float tmax, int n, uint32_t seed) {
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
        Pcg rng;
        rng.set_seed((uint64_t)i, seed);
        V3 T_ray = v3(1.f), pu = v3(1.f), pl = v3(1.f);
        bool aborted;
        V3 T_maj = sample_t_maj(s->media[0], V3{o[0], o[1], o[2]}, V3{d[0], d[1], d[2]}, tmax, rng, 1,
                                aborted, [&](V3, const MediumProps &mp, V3 sigma_maj, V3 Tm) -> bool {
                                    V3 sigma_n = vmax(sigma_maj - mp.sigma_a - mp.sigma_s, v3(0.f));
                                    float pr = get(Tm, 1) * get(sigma_maj, 1);
                                    T_ray = T_ray * (Tm * sigma_n / pr);
                                    pl = pl * (Tm * sigma_maj / pr);
                                    pu = pu * (Tm * sigma_n / pr);
                                    return any(T_ray);
                                });
        V3 r = T_maj / get(T_maj, 1);
        T_ray = T_ray * r;
        pu = pu * r;
        pl = pl * r;
        // ratio-tracking estimate of T: T_ray over the light-sampling path pdf
        if (any(T_ray)) acc += (double)get(T_ray, 1) / (double)get(pl, 1);
    }
    return acc / n;
}

extern "C" int oracle_pt_render(const oracle_pt *s, const krr_wf_params *prm,
                                const krr_camera_desc *c, int32_t w, int32_t h, int64_t frame_index,
                                int64_t px_begin, int64_t px_end, float *out_L, float *out_pixel,
                                int threads) {
    Camera cam;
    cam.pos = V3{c->position[0], c->position[1], c->position[2]};
    std::memcpy(cam.rot, c->rotation, sizeof(cam.rot));
    float fov = std::atan2(c->film_size[1] * 0.5f, c->focal_length);
    cam.tan_fov = std::tan(fov);
    cam.aspect = c->aspect_ratio;
    cam.shutter_open = c->shutter_open;
    cam.shutter_time = c->shutter_time;
    cam.medium = c->medium;
    uint32_t sample_index = (uint32_t)(frame_index * prm->spp + prm->seed);
    int64_t n = px_end - px_begin;
    std::atomic<int64_t> next{0};
    auto work = [&] {
        for (;;) {
            int64_t s0 = next.fetch_add(64);
            if (s0 >= n) break;
            int64_t s1 = std::min<int64_t>(s0 + 64, n);
            for (int64_t i = s0; i < s1; ++i) {
                V3 L, pix;
                render_pixel(*s, *prm, cam, w, h, px_begin + i, sample_index, L, pix);
                out_L[3 * i] = L.x; out_L[3 * i + 1] = L.y; out_L[3 * i + 2] = L.z;
                if (out_pixel) {
                    out_pixel[3 * i] = pix.x; out_pixel[3 * i + 1] = pix.y; out_pixel[3 * i + 2] = pix.z;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < std::max(1, threads); ++t) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    return 0;
}
