// CPU restatement of the reference's sampling, BSDF, Fresnel and microfacet
// code (RGB build).  Test infrastructure only: the checker for the CUDA path.
// Each routine cites the reference routine it follows.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>

namespace oracle {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInv2Pi = 0.15915494309189533577f;
constexpr float kInv4Pi = 0.07957747154594766788f;
constexpr float k2Pi = 6.28318530717958647692f;
constexpr float kRayEps = 1e-4f;   // KRR_RAY_EPS, src/core/raytracing.h:10

struct V3 {
    float x, y, z;
};
inline V3 v3(float s) { return {s, s, s}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length_sq(V3 a) { return dot(a, a); }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a / length(a); }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline V3 vmin(V3 a, V3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline V3 vsqrt(V3 a) { return {std::sqrt(a.x), std::sqrt(a.y), std::sqrt(a.z)}; }
inline V3 vexp(V3 a) { return {std::exp(a.x), std::exp(a.y), std::exp(a.z)}; }
inline bool any(V3 a) { return a.x != 0.f || a.y != 0.f || a.z != 0.f; }
inline float mean(V3 a) { return (a.x + a.y + a.z) / 3.f; }
inline float max_coeff(V3 a) { return std::fmax(a.x, std::fmax(a.y, a.z)); }
inline float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

inline V3 xform_point(const float *m, V3 p) {
    return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
inline V3 mat3_mul(const float *m, V3 v) {
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
inline V3 mat3_mul_transposed(const float *m, V3 v) {
    return {m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
            m[2] * v.x + m[5] * v.y + m[8] * v.z};
}

enum : uint32_t {
    BSDF_UNSET = 0, BSDF_NULL = 1, BSDF_REFLECTION = 2, BSDF_TRANSMISSION = 4, BSDF_DIFFUSE = 8,
    BSDF_GLOSSY = 16, BSDF_SPECULAR = 32,
    BSDF_SMOOTH = BSDF_DIFFUSE | BSDF_GLOSSY, BSDF_DELTA = BSDF_SPECULAR | BSDF_NULL,
};
enum : int32_t { MAT_NULL = 0, MAT_DIFFUSE = 1, MAT_DIELECTRIC = 2, MAT_CONDUCTOR = 3 };

// sampling.h:30-83
inline V3 uniform_sample_sphere(float u0, float u1) {
    float z = 1.0f - 2.0f * u0;
    float r = std::sqrt(std::fmax(0.0f, 1.0f - z * z));
    float phi = k2Pi * u1;
    return {r * std::cos(phi), r * std::sin(phi), z};
}
inline void uniform_sample_disk(float u0, float u1, float &x, float &y) {
    float ox = 2.f * u0 - 1.f, oy = 2.f * u1 - 1.f;
    if (ox == 0.f && oy == 0.f) { x = 0.f; y = 0.f; return; }
    float theta, r;
    if (std::fabs(ox) > std::fabs(oy)) { r = ox; theta = (kPi / 4) * (oy / ox); }
    else { r = oy; theta = kPi / 2 - (kPi / 4) * (ox / oy); }
    x = r * std::cos(theta);
    y = r * std::sin(theta);
}
inline V3 cosine_sample_hemisphere(float u0, float u1) {
    float dx, dy;
    uniform_sample_disk(u0, u1, dx, dy);
    return {dx, dy, std::sqrt(std::fmax(0.f, 1 - dx * dx - dy * dy))};
}
inline V3 uniform_sample_triangle(float u0, float u1) {
    float b0, b1;
    if (u0 < u1) { b0 = u0 / 2; b1 = u1 - b0; }
    else { b1 = u1 / 2; b0 = u0 - b1; }
    return {b0, b1, 1 - b0 - b1};
}
// math_utils.h:120-130
inline V3 get_perpendicular(V3 u) {
    V3 a = vabs(u);
    uint32_t uyx = (a.x - a.y) < 0 ? 1 : 0, uzx = (a.x - a.z) < 0 ? 1 : 0, uzy = (a.y - a.z) < 0 ? 1 : 0;
    uint32_t xm = uyx & uzx, ym = (1 ^ xm) & uzy, zm = 1 ^ (xm | ym);
    return normalize(cross(u, V3{(float)xm, (float)ym, (float)zm}));
}
// math_utils.h:133-139
inline void world_to_latlong(V3 dir, float &u, float &v) {
    V3 p = normalize(dir);
    u = std::atan2(p.x, -p.z) * kInv2Pi + 0.5f;
    v = std::acos(p.y) * kInvPi;
}

// matutils.h:13-100
inline bool same_hemisphere(V3 w, V3 wp) { return w.z * wp.z > 0; }
inline float cos2_theta(V3 w) { return w.z * w.z; }
inline float abs_cos_theta(V3 w) { return std::fabs(w.z); }
inline float sin2_theta(V3 w) { return std::fmax(0.f, 1.f - cos2_theta(w)); }
inline float sin_theta(V3 w) { return std::sqrt(sin2_theta(w)); }
inline float tan_theta(V3 w) { return sin_theta(w) / w.z; }
inline float tan2_theta(V3 w) { return sin2_theta(w) / cos2_theta(w); }
inline float cos_phi(V3 w) {
    float s = sin_theta(w);
    return (s == 0) ? 1.f : std::fmin(std::fmax(w.x / s, -1.f), 1.f);
}
inline float sin_phi(V3 w) {
    float s = sin_theta(w);
    return (s == 0) ? 0.f : std::fmin(std::fmax(w.y / s, -1.f), 1.f);
}
inline V3 face_forward(V3 w, V3 wp) { return dot(w, wp) > 0 ? w : -w; }
inline V3 reflect(V3 wo, V3 n) { return -wo + 2 * dot(wo, n) * n; }
inline bool refract(V3 wi, V3 n, float eta, float *etap, V3 *wt) {
    float cos_i = dot(n, wi);
    if (wi.z < 0) eta = 1 / eta;
    float sin2_i = std::fmax(0.f, 1.f - cos_i * cos_i);
    float sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= 1) return false;
    float cos_t = std::sqrt(1 - sin2_t);
    *wt = -wi / eta + (cos_i / eta - cos_t) * n;
    if (etap) *etap = eta;
    return true;
}

// microfacet.h:17-70
struct Ggx {
    float ax, ay;
    static Ggx make(float a, float b) { return {std::fmax(1e-3f, a), std::fmax(1e-3f, b)}; }
    bool is_delta() const { return std::fmax(ax, ay) <= 1e-3f; }
    float lambda(V3 w) const {
        float abs_tan = std::fabs(tan_theta(w));
        if (std::isinf(abs_tan)) return 0.f;
        float c = cos_phi(w), s = sin_phi(w);
        float alpha = std::sqrt(c * c * ax * ax + s * s * ay * ay);
        float a2t2 = (alpha * abs_tan) * (alpha * abs_tan);
        return (-1 + std::sqrt(1.f + a2t2)) / 2;
    }
    float g1(V3 w) const { return 1 / (1 + lambda(w)); }
    float g(V3 wo, V3 wi) const { return 1 / (1 + lambda(wo) + lambda(wi)); }
    float d(V3 wh) const {
        float t2 = tan2_theta(wh);
        if (std::isinf(t2)) return 0.f;
        float c2 = cos2_theta(wh);
        float cos4 = c2 * c2;
        float cp = cos_phi(wh) / ax, sp = sin_phi(wh) / ay;
        float e = (cp * cp + sp * sp) * t2;
        return 1 / (kPi * ax * ay * cos4 * ((1 + e) * (1 + e)));
    }
    float pdf(V3 wo, V3 wh) const { return d(wh) * g1(wo) * std::fabs(dot(wo, wh)) / abs_cos_theta(wo); }
    V3 sample(V3 wo, float u0, float u1) const;
};

// microfacet.h:86-131
inline void ggx_sample11(float cos_theta, float u1, float u2, float *sx, float *sy) {
    if (cos_theta > .9999f) {
        float r = std::sqrt(u1 / (1 - u1));
        float phi = k2Pi * u2;
        *sx = r * std::cos(phi);
        *sy = r * std::sin(phi);
        return;
    }
    float sin_t = std::sqrt(std::fmax(0.f, 1.f - cos_theta * cos_theta));
    float tan_t = sin_t / cos_theta;
    float a = 1 / tan_t;
    float G1 = 2 / (1 + std::sqrt(1.f + 1.f / (a * a)));
    float A = 2 * u1 / G1 - 1;
    float tmp = 1.f / (A * A - 1.f);
    if (tmp > 1e10f) tmp = 1e10f;
    float B = tan_t;
    float D = std::sqrt(std::fmax(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.f));
    float s1 = B * tmp - D, s2 = B * tmp + D;
    *sx = (A < 0 || s2 > 1.f / tan_t) ? s1 : s2;
    float S;
    if (u2 > 0.5f) { S = 1.f; u2 = 2.f * (u2 - .5f); }
    else { S = -1.f; u2 = 2.f * (.5f - u2); }
    float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
              (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    *sy = S * z * std::sqrt(1.f + *sx * *sx);
}
// microfacet.h:133-154
inline V3 ggx_sample(V3 wi, float ax, float ay, float u1, float u2) {
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
// microfacet.h:157-164 (KRR_GGX_SAMPLE_LEGACY)
inline V3 Ggx::sample(V3 wo, float u0, float u1) const {
    bool flip = wo.z < 0;
    V3 wh = ggx_sample(flip ? -wo : wo, ax, ay, u0, u1);
    return flip ? -wh : wh;
}

// fresnel.h:21-41
inline float fr_dielectric(float cos_i, float eta) {
    cos_i = std::fmin(std::fmax(cos_i, -1.f), 1.f);
    if (cos_i < 0) { eta = 1 / eta; cos_i = -cos_i; }
    float sin2_i = 1 - cos_i * cos_i;
    float sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= 1) return 1.f;
    float cos_t = std::sqrt(std::fmax(1 - sin2_t, 0.f));
    float r_parl = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    float r_perp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return (r_parl * r_parl + r_perp * r_perp) / 2;
}

// Complex<float> (src/core/math/include/krrmath/complex.h) and FrComplex
// (fresnel.h:43-55)
struct Cx {
    float re, im;
};
inline Cx cx_add(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
inline Cx cx_sub(Cx a, Cx b) { return {a.re - b.re, a.im - b.im}; }
inline Cx cx_mul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cx cx_div(Cx a, Cx b) {
    float scale = 1 / (b.re * b.re + b.im * b.im);
    return {scale * (a.re * b.re + a.im * b.im), scale * (a.im * b.re - a.re * b.im)};
}
inline float cx_norm(Cx a) { return a.re * a.re + a.im * a.im; }
inline Cx cx_sqrt(Cx z) {
    float n = std::sqrt(cx_norm(z)), t1 = std::sqrt(.5f * (n + std::fabs(z.re))), t2 = .5f * z.im / t1;
    if (n == 0) return {0, 0};
    if (z.re >= 0) return {t1, t2};
    return {std::fabs(t2), std::copysign(t1, z.im)};
}
inline float fr_complex(float cos_i, Cx eta) {
    cos_i = std::fmin(std::fmax(cos_i, 0.f), 1.f);
    float sin2_i = 1 - cos_i * cos_i;
    Cx sin2_t = cx_div(Cx{sin2_i, 0}, cx_mul(eta, eta));
    Cx cos_t = cx_sqrt(cx_sub(Cx{1, 0}, sin2_t));
    Cx ec = cx_mul(eta, Cx{cos_i, 0});
    Cx r_parl = cx_div(cx_sub(ec, cos_t), cx_add(ec, cos_t));
    Cx ect = cx_mul(eta, cos_t);
    Cx r_perp = cx_div(cx_sub(Cx{cos_i, 0}, ect), cx_add(Cx{cos_i, 0}, ect));
    return (cx_norm(r_parl) + cx_norm(r_perp)) / 2;
}
inline V3 fr_complex3(float cos_i, V3 eta, V3 k) {
    return {fr_complex(cos_i, Cx{eta.x, k.x}), fr_complex(cos_i, Cx{eta.y, k.y}),
            fr_complex(cos_i, Cx{eta.z, k.z})};
}

struct ShadingData {
    int32_t type;
    V3 diffuse;
    float roughness, spec_trans, ior, anisotropic;
};

// BSDFData::getBsdfType, src/render/shared.h:46-73
inline uint32_t bsdf_type_of(const ShadingData &sd) {
    switch (sd.type) {
        case MAT_NULL: return BSDF_NULL;
        case MAT_DIFFUSE: return BSDF_DIFFUSE | BSDF_REFLECTION;
        case MAT_DIELECTRIC:
            return (sd.roughness <= 1e-3f ? BSDF_SPECULAR : BSDF_GLOSSY) | BSDF_REFLECTION | BSDF_TRANSMISSION;
        case MAT_CONDUCTOR: return BSDF_REFLECTION | (sd.roughness <= 1e-3f ? BSDF_SPECULAR : BSDF_GLOSSY);
        default: return BSDF_UNSET;
    }
}

struct BsdfSample {
    V3 f, wi;
    float pdf;
    uint32_t flags;
};

// DiffuseBrdf (diffuse.h:18-57), ConductorBsdf (conductor.h:6-99),
// DielectricBsdf (dielectric.h:75-261), NullBsdf (null.h:18-47)
struct Bsdf {
    int32_t type;
    V3 color, eta3, k3;
    float eta;
    Ggx dist;

    static Bsdf setup(const ShadingData &sd) {
        Bsdf b{};
        b.type = sd.type;
        b.eta = 1.f;
        b.dist = Ggx{1e-3f, 1e-3f};
        if (sd.type == MAT_DIFFUSE) {
            b.color = sd.diffuse;
        } else if (sd.type == MAT_CONDUCTOR) {
            b.color = vmin(sd.diffuse, v3(0.9999f));
            float aspect = std::sqrt(1 - sd.anisotropic * .9f);
            float r2 = sd.roughness * sd.roughness;
            b.dist = Ggx::make(std::fmax(.001f, r2 / aspect), std::fmax(.001f, r2 * aspect));
            b.eta3 = v3(sd.ior);
            b.k3 = 2 * vsqrt(b.color) / vsqrt(vmax(v3(1.f) - b.color, v3(0.f)));
        } else if (sd.type == MAT_DIELECTRIC) {
            b.color = sd.diffuse * sd.spec_trans;
            b.eta = sd.ior;
            float alpha = sd.roughness * sd.roughness;
            b.dist = Ggx::make(alpha, alpha);
        }
        return b;
    }

    V3 f(V3 wo, V3 wi) const {
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
            V3 F = fr_complex3(std::fabs(dot(wo, wm)), eta3, k3);
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
            float F = fr_dielectric(std::copysign(dot(wo, wm), wo.z), eta);
            V3 R = color * F, T = color * (1 - F);
            if (refl) return dist.d(wm) * dist.g(wo, wi) * R / std::fabs(4 * ci * co);
            float dwi = dot(wi, wm) + dot(wo, wm) / etap;
            float denom = dwi * dwi * ci * co;
            V3 ft = T * dist.d(wm) * dist.g(wo, wi) * std::fabs(dot(wi, wm) * dot(wo, wm) / denom);
            return ft / (etap * etap);
        }
        return v3(0.f);
    }

    float pdf(V3 wo, V3 wi) const {
        if (type == MAT_DIFFUSE) {
            if (!same_hemisphere(wo, wi)) return 0.f;
            return std::fabs(wi.z) * kInvPi;
        }
        if (type == MAT_CONDUCTOR) {
            if (!same_hemisphere(wo, wi)) return 0.f;
            if (dist.is_delta()) return 0.f;
            V3 wm = wo + wi;
            if (!any(wm)) return 0.f;
            wm = face_forward(normalize(wm), V3{0, 0, 1});
            return dist.pdf(wo, wm) / (4 * std::fabs(dot(wo, wm)));
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
            if (refl) return dist.pdf(wo, wm) / (4 * std::fabs(dot(wo, wm))) * pr / (pr + pt);
            float dwi = dot(wi, wm) + dot(wo, wm) / etap;
            float denom = dwi * dwi;
            float dwm_dwi = std::fabs(dot(wi, wm)) / denom;
            return dist.pdf(wo, wm) * dwm_dwi * pt / (pr + pt);
        }
        return 0.f;
    }

    template <typename Draw>
    BsdfSample sample(V3 wo, Draw &&draw) const {
        BsdfSample s{v3(0.f), v3(0.f), 0.f, BSDF_UNSET};
        if (type == MAT_DIFFUSE) {
            float u0 = draw();
            float u1 = draw();
            V3 wi = cosine_sample_hemisphere(u0, u1);
            wi.z = wi.z * wo.z > 0 ? wi.z : -wi.z;
            s.wi = wi;
            s.f = f(wo, wi);
            s.pdf = pdf(wo, wi);
            s.flags = BSDF_DIFFUSE | BSDF_REFLECTION;
            return s;
        }
        if (type == MAT_CONDUCTOR) {
            if (dist.is_delta()) {
                V3 wi{-wo.x, -wo.y, wo.z};
                s.f = fr_complex3(abs_cos_theta(wi), eta3, k3) / abs_cos_theta(wi);
                s.wi = wi;
                s.pdf = 1;
                s.flags = BSDF_SPECULAR | BSDF_REFLECTION;
                return s;
            }
            if (wo.z == 0) return s;
            float u0 = draw();
            float u1 = draw();
            V3 wm = dist.sample(wo, u0, u1);
            V3 wi = reflect(wo, wm);
            if (!same_hemisphere(wo, wi)) return s;
            float p = dist.pdf(wo, wm) / (4 * std::fabs(dot(wo, wm)));
            float co = abs_cos_theta(wo), ci = abs_cos_theta(wi);
            if (ci == 0 || co == 0) return s;
            V3 F = fr_complex3(std::fabs(dot(wo, wm)), eta3, k3);
            s.f = dist.d(wm) * F * dist.g(wo, wi) / (4 * ci * co);
            s.wi = wi;
            s.pdf = p;
            s.flags = BSDF_GLOSSY | BSDF_REFLECTION;
            return s;
        }
        if (type == MAT_DIELECTRIC) {
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
                    s.flags = BSDF_SPECULAR | BSDF_REFLECTION;
                    return s;
                }
                V3 wi;
                float etap;
                if (!refract(wo, V3{0, 0, std::copysign(1.f, wo.z)}, eta, &etap, &wi)) return s;
                s.f = (T / abs_cos_theta(wi)) / (etap * etap);
                s.wi = wi;
                s.pdf = pt / (pr + pt);
                s.flags = BSDF_SPECULAR | BSDF_TRANSMISSION;
                return s;
            }
            float u0 = draw();
            float u1 = draw();
            V3 wm = dist.sample(wo, u0, u1);
            float F = fr_dielectric(std::copysign(dot(wo, wm), wo.z), eta);
            V3 R = color * F, T = color * (1 - F);
            float pr = mean(R), pt = mean(T);
            if (pr == 0 && pt == 0) return s;
            if (draw() < pr / (pr + pt)) {
                V3 wi = reflect(wo, wm);
                if (!same_hemisphere(wo, wi)) return s;
                float p = dist.pdf(wo, wm) / (4 * std::fabs(dot(wo, wm))) * pr / (pr + pt);
                s.f = dist.d(wm) * dist.g(wo, wi) * R / (4 * wi.z * wo.z);
                s.wi = wi;
                s.pdf = p;
                s.flags = BSDF_GLOSSY | BSDF_REFLECTION;
                return s;
            }
            float etap;
            V3 wi;
            bool tir = !refract(wo, wm, eta, &etap, &wi);
            if (same_hemisphere(wo, wi) || wi.z == 0 || tir) return s;
            float dd = dot(wi, wm) + dot(wo, wm) / etap;
            float denom = dd * dd;
            float dwm_dwi = std::fabs(dot(wi, wm)) / denom;
            float p = dist.pdf(wo, wm) * dwm_dwi * pt / (pr + pt);
            V3 ft = T * dist.d(wm) * dist.g(wo, wi) *
                    std::fabs(dot(wi, wm) * dot(wo, wm) / (wi.z * wo.z * denom));
            s.f = ft / (etap * etap);
            s.wi = wi;
            s.pdf = p;
            s.flags = BSDF_GLOSSY | BSDF_TRANSMISSION;
            return s;
        }
        s.wi = -wo;
        s.pdf = 1;
        s.f = v3(1.f) / abs_cos_theta(wo);
        s.flags = BSDF_NULL;
        return s;
    }
};

}  // namespace oracle
