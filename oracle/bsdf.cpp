// C entry points for the known-answer tests of the BSDF restatement in
// shading.h (test infrastructure only): Fresnel, evaluation and sampling of
// the diffuse, conductor and dielectric BSDFs in the local shading frame.
#include <cstdint>

#include "shading.h"

using namespace oracle;

namespace {
// mat: type, diffuse r, g, b, roughness, specular transmission, ior, anisotropic
Bsdf make_bsdf(const float *mat) {
    ShadingData sd{};
    sd.type = (int32_t)mat[0];
    sd.diffuse = V3{mat[1], mat[2], mat[3]};
    sd.roughness = mat[4];
    sd.spec_trans = mat[5];
    sd.ior = mat[6];
    sd.anisotropic = mat[7];
    return Bsdf::setup(sd);
}
}  // namespace

extern "C" float oracle_fr_dielectric(float cos_i, float eta) { return fr_dielectric(cos_i, eta); }

// f (rgb) and pdf of n direction pairs (wo[3 n], wi[3 n]) -> out[4 n]
extern "C" void oracle_bsdf_eval(const float *mat, const float *wo, const float *wi, int64_t n, float *out) {
    const Bsdf b = make_bsdf(mat);
    for (int64_t i = 0; i < n; ++i) {
        const V3 o{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]}, w{wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]};
        const V3 f = b.f(o, w);
        out[4 * i] = f.x;
        out[4 * i + 1] = f.y;
        out[4 * i + 2] = f.z;
        out[4 * i + 3] = b.pdf(o, w);
    }
}

// n samples for one wo, each drawing from its own row of u[n][3] uniforms;
// out[n][8] = f rgb, wi xyz, pdf, flags
extern "C" void oracle_bsdf_sample(const float *mat, const float *wo, const float *u, int64_t n, float *out) {
    const Bsdf b = make_bsdf(mat);
    const V3 o{wo[0], wo[1], wo[2]};
    for (int64_t i = 0; i < n; ++i) {
        int k = 0;
        const float *ui = u + 3 * i;
        BsdfSample s = b.sample(o, [&]() { return ui[k < 3 ? k++ : 2]; });
        float *r = out + 8 * i;
        r[0] = s.f.x; r[1] = s.f.y; r[2] = s.f.z;
        r[3] = s.wi.x; r[4] = s.wi.y; r[5] = s.wi.z;
        r[6] = s.pdf;
        r[7] = (float)s.flags;
    }
}
