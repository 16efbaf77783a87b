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

// One pixel through the wavefront stages; returns L (the reference's
// PixelState::L after the frame) and accumulates `pixel`.
void render_pixel(const oracle_pt &s, const krr_wf_params &prm, const Camera &cam, int w, int h,
                  int64_t pixel_id, uint32_t sample_index, V3 &L_out, V3 &pixel_out) {
    (void)h;
    uint32_t x = (uint32_t)(pixel_id % w), y = (uint32_t)(pixel_id / w);
    Pcg rng;
    rng.set_seed(interleave_32bit(x, y), sample_index);
    rng.advance(256 * pixel_id);
    float ul = rng.get1d();
    float lambda0 = (1.f - ul) * 360.f + ul * 830.f;
    (void)lambda0;
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
        bool alive = true;
        for (int depth = 0; alive; ++depth) {
            Hit hit = trace(s, ps.ray);
            bool scatter_pending = false;
            Surf sf{};
            PathState next{};
            bool next_pending = false;
            if (hit.prim == 0xFFFFFFFFu) {
                // handleMiss
                V3 Lm = v3(0.f);
                for (const Infinite &e : s.infinite) {
                    if (prm.nee && ps.depth && !(ps.bsdf_type & BSDF_DELTA)) {
                        float light_pdf = kInv4Pi * lsel_pdf;
                        Lm = Lm + env_Li(e, ps.ray.d) / mean(ps.pu + ps.pl * light_pdf);
                    } else {
                        Lm = Lm + env_Li(e, ps.ray.d) / mean(ps.pu);
                    }
                }
                if (!s.infinite.empty()) L = ps.thp * Lm + L;
            } else {
                sf = prepare_surface(s, hit.b1, hit.b2, hit.prim, ps.ray.d);
                if (sf.material < 0) {
                    next = ps;
                    next.ray = Ray{offset_ray_origin(sf.p, sf.n, ps.ray.d), ps.ray.d, INFINITY};
                    next.medium = medium_towards(sf.interface_in, sf.interface_out, ps.medium, sf.n, ps.ray.d);
                    next_pending = true;
                } else {
                    if (sf.light >= 0) {
                        // handleHit
                        const Light &l = s.lights[sf.light];
                        const Instance &I = s.instances[l.index];
                        V3 Le = area_L(I, sf.n, sf.wo) * ps.thp;
                        if (prm.nee && ps.depth && !(ps.bsdf_type & BSDF_DELTA)) {
                            float light_pdf = area_pdf(s, l, sf.p, sf.n, ps.ctx_p) * lsel_pdf;
                            Le = Le / mean(ps.pl * light_pdf + ps.pu);
                        } else {
                            Le = Le / mean(ps.pu);
                        }
                        L = Le + L;
                    }
                    scatter_pending = any(ps.thp);
                }
            }
            if (depth == prm.max_depth) break;
            bool shadow_pending = false;
            V3 sh_o, sh_d, sh_Ld, sh_pu, sh_pl;
            if (scatter_pending) {
                // generateScatterRays
                if (rng.get1d() >= prm.rr) {
                    scatter_pending = false;
                } else {
                    V3 thp = ps.thp / prm.rr;
                    auto to_local = [&](V3 v) { return V3{dot(sf.t, v), dot(sf.b, v), dot(sf.n, v)}; };
                    V3 wo_local = to_local(sf.wo);
                    ShadingData sd = shading_data(s, sf.material);
                    uint32_t bt = bsdf_type_of(sd);
                    Bsdf bsdf = Bsdf::setup(sd);
                    if (prm.nee && (bt & BSDF_SMOOTH)) {
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
                                sh_pu = ps.pu * bsdf_pdf;
                                sh_pl = ps.pu * light_pdf;
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
                            next.pu = ps.pu;
                            next.pl = ps.pu / bs.pdf;
                            next.bsdf_type = bs.flags;
                            next.depth = ps.depth + 1;
                            next.medium = medium_towards(sf.interface_in, sf.interface_out, ps.medium, sf.n, wi_world);
                            next.time = ps.time;
                            next_pending = true;
                        }
                    }
                }
            }
            if (shadow_pending && prm.nee) {
                if (!occluded(s, sh_o, sh_d, 1.f)) L = sh_Ld / mean(sh_pl + sh_pu) + L;
            }
            if (!next_pending) break;
            ps = next;
        }
        pixel = pixel + L;
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
    *out = s;
    return 0;
}

extern "C" void oracle_pt_free(oracle_pt *s) { delete s; }

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
