// Participating media of the wavefront path tracer (included by wavefront.cu).
//
// Dense FP16 density grid with a majorant grid (the reference's
// NanoVDBMedium<float>, src/render/media.h:144-227, on a dense grid instead of
// a NanoVDB tree), the majorant DDA (MajorantIterator, media.h:41-106), the
// majorant sampling loop sampleT_maj (src/render/wavefront/wavefront.h:34-78),
// delta tracking (sampleMediumInteraction, medium.cpp:13-103), HG phase
// scattering with NEE (sampleMediumScattering, medium.cpp:105-153) and
// ratio-tracked shadow transmittance (traceTransmittance, wavefront.h:80-139).
#pragma once

namespace krr {


struct MediumProps {
    V3 sigma_a, sigma_s;
};

struct MajorantSeg {
    float tmin, tmax;
    V3 sigma_maj;
};

__device__ __forceinline__ float half_to_float(uint16_t h) {
    return __half2float(__ushort_as_half(h));
}

// Density at world point p: trilinear interpolation with voxel centres at
// integer index coordinates, zero outside the grid (NanoVDB's
// SampleFromVoxels<1> on the index-space point worldToIndexF(p), an affine
// map: offset, then a multiply by the voxels per unit length).
__device__ __forceinline__ float density_at(const DevMedium &m, V3 p) {
    float fx = (p.x - m.lo[0]) * m.idx_scale[0] - 0.5f;
    float fy = (p.y - m.lo[1]) * m.idx_scale[1] - 0.5f;
    float fz = (p.z - m.lo[2]) * m.idx_scale[2] - 0.5f;
    float ix = floorf(fx), iy = floorf(fy), iz = floorf(fz);
    float u = fx - ix, v = fy - iy, w = fz - iz;
    int x0 = (int)ix, y0 = (int)iy, z0 = (int)iz;
    // the octet of corner (x0 + sx, y0 + sy, z0 + sz): sx = 1 when x0 = -1
    // (column -1 lies outside, column 0 is the octet's first), likewise sy, sz
    const int sx = x0 == -1 ? 1 : 0, sy = y0 == -1 ? 1 : 0, sz = z0 == -1 ? 1 : 0;
    float o[2][2][2] = {{{0.f, 0.f}, {0.f, 0.f}}, {{0.f, 0.f}, {0.f, 0.f}}};   // o[i][j][k]: +i x, +j y, +k z
    if (x0 >= -1 && x0 < m.nx && y0 >= -1 && y0 < m.ny && z0 >= -1 && z0 < m.nz) {
        const uint4 q = __ldg(reinterpret_cast<const uint4 *>(m.density) +
                              ((size_t)(z0 + sz) * m.ny + (y0 + sy)) * m.nx + (x0 + sx));
        const uint32_t wd[4] = {q.x, q.y, q.z, q.w};   // word 2k + j: (x, x+1) at +j y, +k z
#pragma unroll
        for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                o[0][j][k] = half_to_float((uint16_t)(wd[2 * k + j] & 0xffffu));
                o[1][j][k] = half_to_float((uint16_t)(wd[2 * k + j] >> 16));
            }
    }
    float c[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int e = 0; e < 2; ++e)
                c[a][b][e] = (a >= sx && b >= sy && e >= sz) ? o[a - sx][b - sy][e - sz] : 0.f;
    auto lerp = [](float a, float b, float t) { return a + t * (b - a); };
    return lerp(lerp(lerp(c[0][0][0], c[0][0][1], w), lerp(c[0][1][0], c[0][1][1], w), v),
                lerp(lerp(c[1][0][0], c[1][0][1], w), lerp(c[1][1][0], c[1][1][1], w), v), u);
}

// Spectra of a grey medium keep three equal channels through the tracking
// loops; an operation on such a spectrum is done once and broadcast, which
// gives the same bits as three per-channel operations.
__device__ __forceinline__ bool grey(V3 a) {
    return __float_as_uint(a.x) == __float_as_uint(a.y) && __float_as_uint(a.y) == __float_as_uint(a.z);
}
__device__ __forceinline__ V3 div_g(V3 a, float b) {
    if (grey(a)) {
        float q = a.x / b;
        return V3{q, q, q};
    }
    return a / b;
}
__device__ __forceinline__ V3 exp_g(V3 a) {
    if (grey(a)) {
        float e = expf(a.x);
        return V3{e, e, e};
    }
    return vexp(a);
}

// Medium::samplePoint (media.h:121-126 homogeneous, :161-172 grid)
__device__ __forceinline__ MediumProps sample_point(const DevMedium &m, V3 p) {
    V3 st{m.sigma_t[0], m.sigma_t[1], m.sigma_t[2]};
    V3 sigma_t = m.density ? (density_at(m, p) * m.scale) * st : st;
    V3 sigma_s = sigma_t * V3{m.albedo[0], m.albedo[1], m.albedo[2]};
    return MediumProps{sigma_t - sigma_s, sigma_s};
}

// AABB::intersect, krrmath/aabb.h:58-76
__device__ __forceinline__ bool box_intersect(const float *lo, const float *hi, V3 o, V3 d, float tmax,
                                              float &t0, float &t1) {
    t0 = 0.f;
    t1 = tmax;
    for (int i = 0; i < 3; ++i) {
        float inv = 1 / get(d, i);
        float tn = (lo[i] - get(o, i)) * inv;
        float tf = (hi[i] - get(o, i)) * inv;
        if (tn > tf) { float tmp = tn; tn = tf; tf = tmp; }
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return false;
    }
    return true;
}

struct MajorantIter {
    float tmin, tmax;
    V3 sigma_t;
    const DevMedium *m;
    float next_cross[3], delta_t[3];
    int step[3], limit[3], voxel[3];

    // Medium::sampleRay + MajorantIterator constructor (media.h:45-70, 174-185)
    __device__ void init(const DevMedium &med, V3 o, V3 d, float ray_tmax) {
        tmin = 3.402823466e38f;
        tmax = 1.175494351e-38f;
        m = nullptr;
        V3 st{med.sigma_t[0], med.sigma_t[1], med.sigma_t[2]};
        if (!med.density) {   // homogeneous: one segment, no bounds
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
            voxel[a] = (int)fminf(fmaxf(gi * res, 0.f), res - 1.f);
            delta_t[a] = 1.f / (fabsf(gd[a]) * res);
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

    // MajorantIterator::next, media.h:72-98
    __device__ bool next(MajorantSeg &seg) {
        if (tmin >= tmax) return false;
        if (!m) {
            seg = MajorantSeg{tmin, tmax, sigma_t};
            tmin = tmax;
            return true;
        }
        int bits = ((next_cross[0] < next_cross[1]) << 2) + ((next_cross[0] < next_cross[2]) << 1) +
                   (next_cross[1] < next_cross[2]);
        // cmp -> axis {2, 1, 2, 1, 2, 2, 0, 0}, two bits per entry (no table in local memory)
        int ax = (0xA66 >> (2 * bits)) & 3;
        float exit = fminf(tmax, next_cross[ax]);
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

// SampledWavelengths::mainIndex in the RGB build (spectrum.h:76-81)
__device__ __forceinline__ int main_index(float lambda0) {
    int c = (int)((lambda0 - 360.f) / (830.f - 360.f) * 3);
    return c < 0 ? 0 : (c > 2 ? 2 : c);
}

__device__ __forceinline__ float next_float_down(float v) {
    if (isinf(v) && v < 0.f) return v;
    if (v == 0.f) v = -0.f;
    uint32_t ui = __float_as_uint(v);
    if (v > 0) --ui;
    else ++ui;
    return __uint_as_float(ui);
}

// sampleDiscrete over three weights (sampling.h:90-105)
__device__ __forceinline__ int sample_discrete3(float w0, float w1, float w2, float u) {
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

// HGPhaseFunction, media.cpp:83-111
__device__ __forceinline__ float hg_p(float g, V3 wo, V3 wi) {
    g = fminf(fmaxf(g, -.99f), .99f);
    float denom = 1 + g * g + 2 * g * dot(wo, wi);
    return kInv4Pi * (1 - g * g) / (denom * sqrtf(fmaxf(0.f, denom)));
}

__device__ __forceinline__ V3 hg_sample(float g0, V3 wo, float u0, float u1, float &pdf) {
    float g = fminf(fmaxf(g0, -.99f), .99f);
    float cos_t;
    if (fabsf(g) < 1e-3f) cos_t = 1 - 2 * u0;
    else {
        float q = (1 - g * g) / (1 + g - 2 * g * u0);
        cos_t = -1 / (2 * g) * (1 + g * g - q * q);
    }
    float sin_t = sqrtf(fmaxf(0.f, 1 - cos_t * cos_t));
    float phi = k2Pi * u1;
    V3 n = normalize(wo);
    V3 t = get_perpendicular(n);
    V3 b = normalize(cross(n, t));
    V3 v{sin_t * cosf(phi), sin_t * sinf(phi), cos_t};
    V3 wi = t * v.x + b * v.y + n * v.z;
    pdf = hg_p(g0, normalize(wo), wi);
    return wi;
}

// sampleT_maj, wavefront.h:34-78.  `cb` returns false to stop.  The loop
// over null collisions is bounded; running out sets an error flag and stops.
template <typename F>
__device__ V3 sample_t_maj(const DevMedium &m, V3 o, V3 d, float tmax, Pcg &rng, int ch,
                           int max_null, uint32_t *err, bool &aborted, F &&cb) {
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
            if (isinf(dt)) dt = 3.402823466e38f;
            T_maj *= exp_g(-dt * seg.sigma_maj);
            continue;
        }
        float tmin = seg.tmin;
        while (true) {
            if (++guard > max_null) {
                atomicOr(err, (uint32_t)kErrLoopLimit);
                aborted = true;
                return v3(1.f);
            }
            float u = rng.get1d();
            float t = tmin + (-logf(1 - u) / get(seg.sigma_maj, ch));
            if (t < seg.tmax) {
                T_maj *= exp_g(-(t - tmin) * seg.sigma_maj);
                V3 p = o + d * t;
                MediumProps mp = sample_point(m, p);
                if (!cb(p, mp, seg.sigma_maj, T_maj)) return v3(1.f);
                T_maj = v3(1.f);
                tmin = t;
            } else {
                float dt = seg.tmax - tmin;
                if (isinf(dt)) dt = 3.402823466e38f;
                T_maj *= exp_g(-dt * seg.sigma_maj);
                break;
            }
        }
    }
}

// x-fastest densities [nz][ny][nx] -> octets (voxel and its neighbours at
// +x, +y, +z, 0 past the last column, row or slice).
__global__ void k_octet_density(const uint16_t *__restrict__ lin, int nx, int ny, int nz, int64_t n,
                                uint4 *octets) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
        uint32_t w[4];
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 2; ++j) {
                uint32_t v[2];
                for (int a = 0; a < 2; ++a) {
                    const bool in = x + a < nx && y + j < ny && z + k < nz;
                    v[a] = in ? lin[i + a + (int64_t)j * nx + (int64_t)k * nx * ny] : 0u;
                }
                w[2 * k + j] = v[0] | (v[1] << 16);
            }
        octets[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// initializeMajorantGrid, media.cpp:18-75 (dense grid, filter slop 1 voxel)
__global__ void k_build_majorant(DevMedium m, float *out) {
    int n = m.mres[0] * m.mres[1] * m.mres[2];
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        int x = idx % m.mres[0], y = (idx / m.mres[0]) % m.mres[1], z = idx / (m.mres[0] * m.mres[1]);
        float cl[3], ch[3];
        int c[3] = {x, y, z};
        int dims[3] = {m.nx, m.ny, m.nz};
        int r0[3], r1[3];
        for (int a = 0; a < 3; ++a) {
            float diag = m.hi[a] - m.lo[a];
            cl[a] = m.lo[a] + ((float)c[a] / (float)m.mres[a]) * diag;
            ch[a] = m.lo[a] + ((float)(c[a] + 1) / (float)m.mres[a]) * diag;
            float i0 = (cl[a] - m.lo[a]) / diag * (float)dims[a] - 0.5f;
            float i1 = (ch[a] - m.lo[a]) / diag * (float)dims[a] - 0.5f;
            r0[a] = max((int)(i0 - 1.f), 0);
            r1[a] = min((int)(i1 + 1.f), dims[a] - 1);
        }
        float mx = 0.f;
        for (int k = r0[2]; k <= r1[2]; ++k)
            for (int j = r0[1]; j <= r1[1]; ++j)
                for (int i = r0[0]; i <= r1[0]; ++i)
                    mx = fmaxf(mx, half_to_float(m.density[8 * (((size_t)k * m.ny + j) * m.nx + i)]));
        out[idx] = mx;
    }
}

}  // namespace krr
