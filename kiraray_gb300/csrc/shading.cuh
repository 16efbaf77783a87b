// Device-side sampling, BSDF and light code of the wavefront path tracer.
//
// Each function follows the reference routine cited beside it (RGB build:
// Spectrum = RGB, src/render/color.h:24-28), with the same operation order
// and the same sampler-draw order, so that per-pixel paths match the CPU
// restatement in oracle/.
#pragma once
#include <stdint.h>

#include "kmath.cuh"

namespace krr {

// BSDFType bits, src/render/materials/bxdf.h:29-48
enum : uint32_t {
    BSDF_UNSET = 0,
    BSDF_NULL = 1u << 0,
    BSDF_REFLECTION = 1u << 1,
    BSDF_TRANSMISSION = 1u << 2,
    BSDF_DIFFUSE = 1u << 3,
    BSDF_GLOSSY = 1u << 4,
    BSDF_SPECULAR = 1u << 5,
    BSDF_DIFFUSE_REFLECTION = BSDF_DIFFUSE | BSDF_REFLECTION,
    BSDF_SPECULAR_REFLECTION = BSDF_SPECULAR | BSDF_REFLECTION,
    BSDF_GLOSSY_REFLECTION = BSDF_GLOSSY | BSDF_REFLECTION,
    BSDF_SPECULAR_TRANSMISSION = BSDF_SPECULAR | BSDF_TRANSMISSION,
    BSDF_GLOSSY_TRANSMISSION = BSDF_GLOSSY | BSDF_TRANSMISSION,
    BSDF_SMOOTH = BSDF_DIFFUSE | BSDF_GLOSSY,
    BSDF_DELTA = BSDF_SPECULAR | BSDF_NULL,
};

enum : int32_t { MAT_NULL = 0, MAT_DIFFUSE = 1, MAT_DIELECTRIC = 2, MAT_CONDUCTOR = 3 };

// ------------------------------------------------------------- sampler
// PCGSampler, src/core/sampler.h:13-91; interleave_32bit, src/util/hash.h:12-27
KRR_HD uint32_t interleave_32bit(uint32_t x, uint32_t y) {
    x &= 0x0000ffffu;
    y &= 0x0000ffffu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    y = (y | (y << 8)) & 0x00FF00FFu;
    y = (y | (y << 4)) & 0x0F0F0F0Fu;
    y = (y | (y << 2)) & 0x33333333u;
    y = (y | (y << 1)) & 0x55555555u;
    return x | (y << 1);
}

struct Pcg {
    uint64_t state, inc;
    static constexpr uint64_t kMult = 0x5851f42d4c957f2dULL;

    KRR_HD uint32_t next_u32() {
        uint64_t old = state;
        state = old * kMult + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((~rot + 1u) & 31));
    }
    KRR_HD void set_seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next_u32();
        state += initstate;
        next_u32();
    }
    KRR_HD void advance(int64_t delta) {
        uint64_t cur_mult = kMult, cur_plus = inc, acc_mult = 1u, acc_plus = 0u;
        while (delta > 0) {
            if (delta & 1) {
                acc_mult *= cur_mult;
                acc_plus = acc_plus * cur_mult + cur_plus;
            }
            cur_plus = (cur_mult + 1) * cur_plus;
            cur_mult *= cur_mult;
            delta /= 2;
        }
        state = acc_mult * state + acc_plus;
    }
    KRR_D float get1d() { return __uint_as_float((next_u32() >> 9) | 0x3f800000u) - 1.0f; }
};

// ------------------------------------------------------------ sampling
// src/render/sampling.h:30-83
KRR_D V3 uniform_sample_sphere(float u0, float u1) {
    float z = 1.0f - 2.0f * u0;
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float phi = k2Pi * u1;
    return {r * cosf(phi), r * sinf(phi), z};
}

KRR_D void uniform_sample_disk(float u0, float u1, float &x, float &y) {
    float ox = 2.f * u0 - 1.f, oy = 2.f * u1 - 1.f;
    if (ox == 0.f && oy == 0.f) { x = 0.f; y = 0.f; return; }
    float theta, r;
    if (fabsf(ox) > fabsf(oy)) {
        r = ox;
        theta = (kPi / 4) * (oy / ox);
    } else {
        r = oy;
        theta = kPi / 2 - (kPi / 4) * (ox / oy);
    }
    x = r * cosf(theta);
    y = r * sinf(theta);
}

KRR_D V3 cosine_sample_hemisphere(float u0, float u1) {
    float dx, dy;
    uniform_sample_disk(u0, u1, dx, dy);
    float z = sqrtf(fmaxf(0.f, 1 - dx * dx - dy * dy));
    return {dx, dy, z};
}

KRR_D V3 uniform_sample_triangle(float u0, float u1) {
    float b0, b1;
    if (u0 < u1) {
        b0 = u0 / 2;
        b1 = u1 - b0;
    } else {
        b1 = u1 / 2;
        b0 = u0 - b1;
    }
    return {b0, b1, 1 - b0 - b1};
}

// getPerpendicular, src/util/math_utils.h:120-130
KRR_D V3 get_perpendicular(V3 u) {
    V3 a = vabs(u);
    uint32_t uyx = (a.x - a.y) < 0 ? 1 : 0;
    uint32_t uzx = (a.x - a.z) < 0 ? 1 : 0;
    uint32_t uzy = (a.y - a.z) < 0 ? 1 : 0;
    uint32_t xm = uyx & uzx;
    uint32_t ym = (1 ^ xm) & uzy;
    uint32_t zm = 1 ^ (xm | ym);
    return normalize(cross(u, V3{(float)xm, (float)ym, (float)zm}));
}

// worldToLatLong, src/util/math_utils.h:133-139
KRR_D void world_to_latlong(V3 dir, float &u, float &v) {
    V3 p = normalize(dir);
    u = atan2f(p.x, -p.z) * kInv2Pi + 0.5f;
    v = acosf(p.y) * kInvPi;
}

// ------------------------------------------------------------ microfacet
// matutils.h:13-63
KRR_D bool same_hemisphere(V3 w, V3 wp) { return w.z * wp.z > 0; }
KRR_D float cos2_theta(V3 w) { return w.z * w.z; }
KRR_D float abs_cos_theta(V3 w) { return fabsf(w.z); }
KRR_D float sin2_theta(V3 w) { return fmaxf(0.f, 1.f - cos2_theta(w)); }
KRR_D float sin_theta(V3 w) { return sqrtf(sin2_theta(w)); }
KRR_D float tan_theta(V3 w) { return sin_theta(w) / w.z; }
KRR_D float tan2_theta(V3 w) { return sin2_theta(w) / cos2_theta(w); }
KRR_D float cos_phi(V3 w) {
    float s = sin_theta(w);
    return (s == 0) ? 1.f : fminf(fmaxf(w.x / s, -1.f), 1.f);
}
KRR_D float sin_phi(V3 w) {
    float s = sin_theta(w);
    return (s == 0) ? 0.f : fminf(fmaxf(w.y / s, -1.f), 1.f);
}
KRR_D V3 face_forward(V3 w, V3 wp) { return dot(w, wp) > 0 ? w : -w; }
KRR_D V3 reflect(V3 wo, V3 n) { return -wo + 2 * dot(wo, n) * n; }
// Refract with orientation flip, matutils.h:86-100
KRR_D bool refract(V3 wi, V3 n, float eta, float *etap, V3 *wt) {
    float cos_i = dot(n, wi);
    if (wi.z < 0) eta = 1 / eta;
    float sin2_i = fmaxf(0.f, 1.f - cos_i * cos_i);
    float sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= 1) return false;
    float cos_t = sqrtf(1 - sin2_t);
    *wt = -wi / eta + (cos_i / eta - cos_t) * n;
    if (etap) *etap = eta;
    return true;
}

// GGXMicrofacetDistribution, microfacet.h:17-70
struct Ggx {
    float ax, ay;
    KRR_D static Ggx make(float alphax, float alphay) {
        return Ggx{fmaxf(1e-3f, alphax), fmaxf(1e-3f, alphay)};
    }
    KRR_D bool is_delta() const { return fmaxf(ax, ay) <= 1e-3f; }
    KRR_D float lambda(V3 w) const {
        float abs_tan = fabsf(tan_theta(w));
        if (isinf(abs_tan)) return 0.f;
        float c = cos_phi(w), s = sin_phi(w);
        float alpha = sqrtf(c * c * ax * ax + s * s * ay * ay);
        float a2t2 = (alpha * abs_tan) * (alpha * abs_tan);
        return (-1 + sqrtf(1.f + a2t2)) / 2;
    }
    KRR_D float g1(V3 w) const { return 1 / (1 + lambda(w)); }
    KRR_D float g(V3 wo, V3 wi) const { return 1 / (1 + lambda(wo) + lambda(wi)); }
    KRR_D float d(V3 wh) const {
        float t2 = tan2_theta(wh);
        if (isinf(t2)) return 0.f;
        float c2 = cos2_theta(wh);
        float cos4 = c2 * c2;
        float cp = cos_phi(wh) / ax, sp = sin_phi(wh) / ay;
        float e = (cp * cp + sp * sp) * t2;
        return 1 / (kPi * ax * ay * cos4 * ((1 + e) * (1 + e)));
    }
    KRR_D float pdf(V3 wo, V3 wh) const { return d(wh) * g1(wo) * fabsf(dot(wo, wh)) / abs_cos_theta(wo); }
    KRR_D V3 sample(V3 wo, float u0, float u1) const;
};

// GGXSample11 / GGXSample (legacy stretched sampling), microfacet.h:86-154
KRR_D void ggx_sample11(float cos_theta, float u1, float u2, float *sx, float *sy) {
    if (cos_theta > .9999f) {
        float r = sqrtf(u1 / (1 - u1));
        float phi = k2Pi * u2;
        *sx = r * cosf(phi);
        *sy = r * sinf(phi);
        return;
    }
    float sin_t = sqrtf(fmaxf(0.f, 1.f - cos_theta * cos_theta));
    float tan_t = sin_t / cos_theta;
    float a = 1 / tan_t;
    float G1 = 2 / (1 + sqrtf(1.f + 1.f / (a * a)));
    float A = 2 * u1 / G1 - 1;
    float tmp = 1.f / (A * A - 1.f);
    if (tmp > 1e10f) tmp = 1e10f;
    float B = tan_t;
    float D = sqrtf(fmaxf(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.f));
    float s1 = B * tmp - D;
    float s2 = B * tmp + D;
    *sx = (A < 0 || s2 > 1.f / tan_t) ? s1 : s2;
    float S;
    if (u2 > 0.5f) {
        S = 1.f;
        u2 = 2.f * (u2 - .5f);
    } else {
        S = -1.f;
        u2 = 2.f * (.5f - u2);
    }
    float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
              (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    *sy = S * z * sqrtf(1.f + *sx * *sx);
}

KRR_D V3 ggx_sample(V3 wi, float ax, float ay, float u1, float u2) {
    V3 ws = normalize(V3{ax * wi.x, ay * wi.y, wi.z});
    float sx, sy;
    ggx_sample11(ws.z, u1, u2, &sx, &sy);
    float cp = cos_phi(ws), sp = sin_phi(ws);
    float tmp = cp * sx - sp * sy;
    sy = sp * sx + cp * sy;
    sx = tmp;
    sx = ax * sx;
    sy = ay * sy;
    return normalize(V3{-sx, -sy, 1.f});
}

KRR_D V3 Ggx::sample(V3 wo, float u0, float u1) const {
    bool flip = wo.z < 0;
    V3 wh = ggx_sample(flip ? -wo : wo, ax, ay, u0, u1);
    return flip ? -wh : wh;
}

// FrDielectric / FrComplex, src/render/materials/fresnel.h:21-63
KRR_D float fr_dielectric(float cos_i, float eta) {
    cos_i = fminf(fmaxf(cos_i, -1.f), 1.f);
    if (cos_i < 0) {
        eta = 1 / eta;
        cos_i = -cos_i;
    }
    float sin2_i = 1 - cos_i * cos_i;
    float sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= 1) return 1.f;
    float cos_t = sqrtf(fmaxf(1 - sin2_t, 0.f));
    float r_parl = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    float r_perp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return (r_parl * r_parl + r_perp * r_perp) / 2;
}

struct Cx {
    float re, im;
};
KRR_D Cx cx_add(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
KRR_D Cx cx_sub(Cx a, Cx b) { return {a.re - b.re, a.im - b.im}; }
KRR_D Cx cx_mul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
KRR_D Cx cx_div(Cx a, Cx b) {
    float scale = 1 / (b.re * b.re + b.im * b.im);
    return {scale * (a.re * b.re + a.im * b.im), scale * (a.im * b.re - a.re * b.im)};
}
KRR_D float cx_norm(Cx a) { return a.re * a.re + a.im * a.im; }
KRR_D Cx cx_sqrt(Cx z) {
    // Complex<T>::sqrt, src/core/math/include/krrmath/complex.h
    float n = sqrtf(cx_norm(z)), t1 = sqrtf(.5f * (n + fabsf(z.re))), t2 = .5f * z.im / t1;
    if (n == 0) return {0, 0};
    if (z.re >= 0) return {t1, t2};
    return {fabsf(t2), copysignf(t1, z.im)};
}

KRR_D float fr_complex(float cos_i, Cx eta) {
    cos_i = fminf(fmaxf(cos_i, 0.f), 1.f);
    float sin2_i = 1 - cos_i * cos_i;
    Cx sin2_t = cx_div(Cx{sin2_i, 0}, cx_mul(eta, eta));
    Cx cos_t = cx_sqrt(cx_sub(Cx{1, 0}, sin2_t));
    Cx ec = cx_mul(eta, Cx{cos_i, 0});
    Cx r_parl = cx_div(cx_sub(ec, cos_t), cx_add(ec, cos_t));
    Cx ect = cx_mul(eta, cos_t);
    Cx r_perp = cx_div(cx_sub(Cx{cos_i, 0}, ect), cx_add(Cx{cos_i, 0}, ect));
    return (cx_norm(r_parl) + cx_norm(r_perp)) / 2;
}

KRR_D V3 fr_complex3(float cos_i, V3 eta, V3 k) {
    return {fr_complex(cos_i, Cx{eta.x, k.x}), fr_complex(cos_i, Cx{eta.y, k.y}),
            fr_complex(cos_i, Cx{eta.z, k.z})};
}

// --------------------------------------------------------------- BSDF
struct BsdfSample {
    V3 f;
    V3 wi;
    float pdf;
    uint32_t flags;
};

// Per-hit shading data (BSDFData, src/render/shared.h:35-74)
struct ShadingData {
    int32_t type;
    V3 diffuse;
    float roughness;
    float spec_trans;
    float ior;
    float anisotropic;
};

KRR_D uint32_t bsdf_type_of(const ShadingData &sd) {
    switch (sd.type) {
        case MAT_NULL: return BSDF_NULL;
        case MAT_DIFFUSE: return BSDF_DIFFUSE_REFLECTION;
        case MAT_DIELECTRIC:
            return (sd.roughness <= 1e-3f ? BSDF_SPECULAR : BSDF_GLOSSY) | BSDF_REFLECTION |
                   BSDF_TRANSMISSION;
        case MAT_CONDUCTOR:
            return BSDF_REFLECTION | (sd.roughness <= 1e-3f ? BSDF_SPECULAR : BSDF_GLOSSY);
        default: return BSDF_UNSET;
    }
}

// The BSDF variant set up from the shading data (BSDF::setup, src/render/bsdf.h:25-29).
struct Bsdf {
    int32_t type;
    V3 color;       // diffuse: reflectance; dielectric: base colour; conductor: reflectance
    V3 eta3, k3;    // conductor
    float eta;      // dielectric
    Ggx dist;

    KRR_D static Bsdf setup(const ShadingData &sd) {
        Bsdf b;
        b.type = sd.type;
        b.eta = 1.f;
        b.dist = Ggx{1e-3f, 1e-3f};
        if (sd.type == MAT_DIFFUSE) {
            b.color = sd.diffuse;   // diffuse.h:27-29
        } else if (sd.type == MAT_CONDUCTOR) {
            // conductor.h:12-33
            b.color = vmin(sd.diffuse, v3(0.9999f));
            float aspect = sqrtf(1 - sd.anisotropic * .9f);
            float r2 = sd.roughness * sd.roughness;
            float ax = fmaxf(.001f, r2 / aspect);
            float ay = fmaxf(.001f, r2 * aspect);
            b.dist = Ggx::make(ax, ay);
            b.eta3 = v3(sd.ior);
            V3 one_minus = vmax(v3(1.f) - b.color, v3(0.f));
            b.k3 = 2 * vsqrt(b.color) / vsqrt(one_minus);
        } else if (sd.type == MAT_DIELECTRIC) {
            // dielectric.h:87-92
            b.color = sd.diffuse * sd.spec_trans;
            b.eta = sd.ior;
            float alpha = sd.roughness * sd.roughness;
            b.dist = Ggx::make(alpha, alpha);
        }
        return b;
    }

    // f(), TransportMode::Radiance
    KRR_D V3 f(V3 wo, V3 wi) const {
        if (type == MAT_DIFFUSE) {
            if (!same_hemisphere(wo, wi)) return v3(0.f);
            return color * kInvPi;
        }
        if (type == MAT_CONDUCTOR) {
            if (!same_hemisphere(wo, wi)) return v3(0.f);
            if (dist.is_delta()) return v3(0.f);
            float co = abs_cos_theta(wo), ci = abs_cos_theta(wi);
            if (ci == 0 || co == 0) return v3(0.f);
            V3 wm = wi + wo;
            if (length_sq(wm) == 0) return v3(0.f);
            wm = normalize(wm);
            V3 F = fr_complex3(fabsf(dot(wo, wm)), eta3, k3);
            return dist.d(wm) * F * dist.g(wo, wi) / (4 * ci * co);
        }
        if (type == MAT_DIELECTRIC) {
            if (eta == 1 || dist.is_delta()) return v3(0.f);
            float co = wo.z, ci = wi.z;
            bool refl = ci * co > 0;
            float etap = 1;
            if (!refl) etap = co > 0 ? eta : (1 / eta);
            V3 wm = wi * etap + wo;
            if (ci == 0 || co == 0 || !any(wm)) return v3(0.f);
            wm = face_forward(normalize(wm), V3{0, 0, 1});
            if (dot(wm, wi) * ci < 0 || dot(wm, wo) * co < 0) return v3(0.f);
            float F = fr_dielectric(copysignf(dot(wo, wm), wo.z), eta);
            V3 R = color * F, T = color * (1 - F);
            if (refl) return dist.d(wm) * dist.g(wo, wi) * R / fabsf(4 * ci * co);
            float dwi = dot(wi, wm) + dot(wo, wm) / etap;
            float denom = dwi * dwi * ci * co;
            V3 ft = T * dist.d(wm) * dist.g(wo, wi) * fabsf(dot(wi, wm) * dot(wo, wm) / denom);
            ft = ft / (etap * etap);
            return ft;
        }
        return v3(0.f);
    }

    KRR_D float pdf(V3 wo, V3 wi) const {
        if (type == MAT_DIFFUSE) {
            if (!same_hemisphere(wo, wi)) return 0.f;
            return fabsf(wi.z) * kInvPi;
        }
        if (type == MAT_CONDUCTOR) {
            if (!same_hemisphere(wo, wi)) return 0.f;
            if (dist.is_delta()) return 0.f;
            V3 wm = wo + wi;
            if (is_zero(wm)) return 0.f;
            wm = face_forward(normalize(wm), V3{0, 0, 1});
            return dist.pdf(wo, wm) / (4 * fabsf(dot(wo, wm)));
        }
        if (type == MAT_DIELECTRIC) {
            if (eta == 1 || dist.is_delta()) return 0.f;
            float co = wo.z, ci = wi.z;
            bool refl = ci * co > 0;
            float etap = 1;
            if (!refl) etap = co > 0 ? eta : (1 / eta);
            V3 wm = wi * etap + wo;
            if (ci == 0 || co == 0 || length_sq(wm) == 0) return 0.f;
            wm = face_forward(normalize(wm), V3{0, 0, 1});
            if (dot(wm, wi) * ci < 0 || dot(wm, wo) * co < 0) return 0.f;
            float F = fr_dielectric(wo.z, eta);
            V3 R = color * F, T = color * (1 - F);
            float pr = mean(R), pt = mean(T);
            if (pr == 0 && pt == 0) return 0.f;
            if (refl) return dist.pdf(wo, wm) / (4 * fabsf(dot(wo, wm))) * pr / (pr + pt);
            float dwi = dot(wi, wm) + dot(wo, wm) / etap;
            float denom = dwi * dwi;
            float dwm_dwi = fabsf(dot(wi, wm)) / denom;
            return dist.pdf(wo, wm) * dwm_dwi * pt / (pr + pt);
        }
        return 0.f;
    }

    template <typename Draw>
    KRR_D BsdfSample sample(V3 wo, Draw &&draw) const {
        BsdfSample s{v3(0.f), v3(0.f), 0.f, BSDF_UNSET};
        if (type == MAT_DIFFUSE) {
            // diffuse.h:33-43
            float u0 = draw(), u1 = draw();
            V3 wi = cosine_sample_hemisphere(u0, u1);
            wi.z = wi.z * wo.z > 0 ? wi.z : -wi.z;   // ToSameHemisphere
            s.wi = wi;
            s.f = f(wo, wi);
            s.pdf = pdf(wo, wi);
            s.flags = BSDF_DIFFUSE_REFLECTION;
            return s;
        }
        if (type == MAT_CONDUCTOR) {
            // conductor.h:51-77
            if (dist.is_delta()) {
                V3 wi{-wo.x, -wo.y, wo.z};
                s.f = fr_complex3(abs_cos_theta(wi), eta3, k3) / abs_cos_theta(wi);
                s.wi = wi;
                s.pdf = 1;
                s.flags = BSDF_SPECULAR_REFLECTION;
                return s;
            }
            if (wo.z == 0) return s;
            float u0 = draw(), u1 = draw();
            V3 wm = dist.sample(wo, u0, u1);
            V3 wi = reflect(wo, wm);
            if (!same_hemisphere(wo, wi)) return s;
            float p = dist.pdf(wo, wm) / (4 * fabsf(dot(wo, wm)));
            float co = abs_cos_theta(wo), ci = abs_cos_theta(wi);
            if (ci == 0 || co == 0) return s;
            V3 F = fr_complex3(fabsf(dot(wo, wm)), eta3, k3);
            s.f = dist.d(wm) * F * dist.g(wo, wi) / (4 * ci * co);
            s.wi = wi;
            s.pdf = p;
            s.flags = BSDF_GLOSSY_REFLECTION;
            return s;
        }
        if (type == MAT_DIELECTRIC) {
            // dielectric.h:130-206
            if (eta == 1 || dist.is_delta()) {
                float F = fr_dielectric(wo.z, eta);
                V3 R = color * F, T = color * (1 - F);
                float pr = mean(R), pt = mean(T);
                if (pr == 0 && pt == 0) return s;
                if (draw() < pr / (pr + pt)) {
                    V3 wi{-wo.x, -wo.y, wo.z};
                    s.f = R / abs_cos_theta(wi);
                    s.wi = wi;
                    s.pdf = pr / (pr + pt);
                    s.flags = BSDF_SPECULAR_REFLECTION;
                    return s;
                }
                V3 wi;
                float etap;
                if (!refract(wo, V3{0, 0, copysignf(1.f, wo.z)}, eta, &etap, &wi)) return s;
                V3 ft = T / abs_cos_theta(wi);
                ft = ft / (etap * etap);
                s.f = ft;
                s.wi = wi;
                s.pdf = pt / (pr + pt);
                s.flags = BSDF_SPECULAR_TRANSMISSION;
                return s;
            }
            float u0 = draw(), u1 = draw();
            V3 wm = dist.sample(wo, u0, u1);
            float F = fr_dielectric(copysignf(dot(wo, wm), wo.z), eta);
            V3 R = color * F, T = color * (1 - F);
            float pr = mean(R), pt = mean(T);
            if (pr == 0 && pt == 0) return s;
            if (draw() < pr / (pr + pt)) {
                V3 wi = reflect(wo, wm);
                if (!same_hemisphere(wo, wi)) return s;
                float p = dist.pdf(wo, wm) / (4 * fabsf(dot(wo, wm))) * pr / (pr + pt);
                s.f = dist.d(wm) * dist.g(wo, wi) * R / (4 * wi.z * wo.z);
                s.wi = wi;
                s.pdf = p;
                s.flags = BSDF_GLOSSY_REFLECTION;
                return s;
            }
            float etap;
            V3 wi;
            bool tir = !refract(wo, wm, eta, &etap, &wi);
            if (same_hemisphere(wo, wi) || wi.z == 0 || tir) return s;
            float dd = dot(wi, wm) + dot(wo, wm) / etap;
            float denom = dd * dd;
            float dwm_dwi = fabsf(dot(wi, wm)) / denom;
            float p = dist.pdf(wo, wm) * dwm_dwi * pt / (pr + pt);
            V3 ft = T * dist.d(wm) * dist.g(wo, wi) *
                    fabsf(dot(wi, wm) * dot(wo, wm) / (wi.z * wo.z * denom));
            ft = ft / (etap * etap);
            s.f = ft;
            s.wi = wi;
            s.pdf = p;
            s.flags = BSDF_GLOSSY_TRANSMISSION;
            return s;
        }
        // NullBsdf::sample, null.h:30-38
        s.wi = -wo;
        s.pdf = 1;
        s.f = v3(1.f) / abs_cos_theta(wo);
        s.flags = BSDF_NULL;
        return s;
    }
};

}  // namespace krr
