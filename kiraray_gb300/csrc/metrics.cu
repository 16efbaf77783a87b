// Image passes on the GPU: accumulation in FP64, error metrics, tone mapping.
//
// The reference accumulates frames in its AccumulatePass with a "double"
// precision mode (src/render/passes/accumulate/accumulate.cu:30-79) and
// measures convergence with ErrorMeasurePass (src/render/passes/errormeasure/
// metrics.cu:64-128): per pixel relMSE = mean over channels of
// (|y - ref| / ref)^2 with channels whose reference is 0 contributing 0
// (ERROR_EPS = 0), clamped at 100 per pixel, averaged over pixels.  Here the
// reduction is done in FP64 (the reference reduces in float with thrust).
#include <algorithm>

#include "internal.h"

namespace {

constexpr int kThreads = 256;

__global__ void k_accumulate_f64(const float4 *__restrict__ rgba, double *__restrict__ acc,
                                 int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 c = rgba[i];
        acc[3 * i + 0] += (double)c.x;
        acc[3 * i + 1] += (double)c.y;
        acc[3 * i + 2] += (double)c.z;
    }
}

// Per-block partial sums of the clamped per-pixel metric; `scale` turns the
// accumulated sums into the image estimate (1 / frames).
template <int METRIC>
__global__ void k_metric_partial(const double *__restrict__ acc, double scale,
                                 const float *__restrict__ ref, int64_t n, double *partial) {
    __shared__ double sh[kThreads / 32];
    double sum = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double e = 0.0;
        for (int c = 0; c < 3; ++c) {
            double y = acc[3 * i + c] * scale;
            double r = (double)ref[4 * i + c];
            double d = fabs(y - r);
            if (METRIC == 0) e += (r == 0.0) ? 0.0 : (d / r) * (d / r);   // relMSE
            else e += d * d;                                              // MSE
        }
        e /= 3.0;
        sum += e < 100.0 ? e : 100.0;   // CLAMP_PIXEL_ERROR_THRESHOLD
    }
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
        partial[blockIdx.x] = t;
    }
}

__global__ void k_sum_partials(const double *partial, int n, double *out) {
    __shared__ double sh[kThreads];
    double t = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) t += partial[i];
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// ToneMappingPass::render (src/render/passes/tonemapping/tonemapping.cu:
// 60-88): exposure scale, operator, optional gamma 1/2.2, alpha 1.
__device__ __forceinline__ float tm_lum(float r, float g, float b) {
    return r * 0.299f + g * 0.587f + b * 0.114f;   // luminance(), spectrum.h:545-547
}

__device__ __forceinline__ float tm_aces(float c) {   // toneMapAces, tonemapping.cu:11-20
    c *= 0.6f;
    const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
    float v = (c * (a * c + b)) / (c * (cc * c + d) + e);
    return fminf(fmaxf(v, 0.f), 1.f);
}

__device__ __forceinline__ float tm_uc2(float c) {    // toneMapUC2, tonemapping.cu:28-37
    const float A = 0.22f, B = 0.3f, C = 0.1f, D = 0.2f, E = 0.01f, F = 0.3f;
    return ((c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * F)) - (E / F);
}

__device__ __forceinline__ float tm_heji(float c) {   // toneMapHejiHableAlu, tonemapping.cu:39-44
    c = fmaxf(c - 0.004f, 0.f);
    c = (c * (6.2f * c + 0.5f)) / (c * (6.2f * c + 1.7f) + 0.06f);
    return powf(c, 2.2f);
}

__global__ void k_tonemap(const float4 *__restrict__ in, float4 *__restrict__ out, int64_t n, int op,
                          float exposure, int gamma) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 p = in[i];
        float c[3] = {p.x * exposure, p.y * exposure, p.z * exposure};
        if (op == 1) {   // Reinhard on luminance
            float lum = tm_lum(c[0], c[1], c[2]);
            float r = lum / (lum + 1.f);
            for (int k = 0; k < 3; ++k) c[k] = lum == 0.f ? 0.f : (c[k] * r) / lum;
        } else if (op == 2) {
            for (int k = 0; k < 3; ++k) c[k] = tm_aces(c[k]);
        } else if (op == 3) {
            for (int k = 0; k < 3; ++k) c[k] = tm_uc2(c[k]);
        } else if (op == 4) {
            for (int k = 0; k < 3; ++k) c[k] = tm_heji(c[k]);
        }
        if (gamma)
            for (int k = 0; k < 3; ++k) c[k] = powf(c[k], 0.45454545f);
        out[i] = make_float4(c[0], c[1], c[2], 1.f);
    }
}

int grid_for(int64_t n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t g = (n + kThreads - 1) / kThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)std::max(sms, 1) * 4));
}

}  // namespace

using namespace krr;

extern "C" int krr_accumulate_f64(const float *d_rgba, double *d_accum, int64_t n_pixels,
                                  void *stream) {
    KRR_CHECK_ARG(d_rgba && d_accum && n_pixels >= 0, "bad argument");
    if (n_pixels == 0) return KRR_OK;
    k_accumulate_f64<<<grid_for(n_pixels), kThreads, 0, as_stream(stream)>>>(
        reinterpret_cast<const float4 *>(d_rgba), d_accum, n_pixels);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_tonemap(const float *d_in_rgba, float *d_out_rgba, int64_t n_pixels, int32_t op,
                           float exposure, int32_t gamma, void *stream) {
    KRR_CHECK_ARG(d_in_rgba && d_out_rgba && n_pixels >= 0, "bad argument");
    KRR_CHECK_ARG(op >= 0 && op <= 4, "operator must be 0 linear, 1 reinhard, 2 aces, 3 uncharted2, 4 hejihable");
    if (n_pixels == 0) return KRR_OK;
    k_tonemap<<<grid_for(n_pixels), kThreads, 0, as_stream(stream)>>>(
        reinterpret_cast<const float4 *>(d_in_rgba), reinterpret_cast<float4 *>(d_out_rgba), n_pixels, op,
        exposure, gamma);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

extern "C" int krr_image_error(const double *d_accum, double scale, const float *d_ref_rgba,
                               int64_t n_pixels, int32_t metric, double *h_out, void *stream) {
    KRR_CHECK_ARG(d_accum && d_ref_rgba && h_out && n_pixels > 0, "bad argument");
    KRR_CHECK_ARG(metric == 0 || metric == 1, "metric must be 0 (relMSE) or 1 (MSE)");
    cudaStream_t s = as_stream(stream);
    int grid = grid_for(n_pixels);
    double *partial = nullptr;
    KRR_CUDA(cudaMallocAsync(&partial, (grid + 1) * sizeof(double), s));
    if (metric == 0)
        k_metric_partial<0><<<grid, kThreads, 0, s>>>(d_accum, scale, d_ref_rgba, n_pixels, partial);
    else
        k_metric_partial<1><<<grid, kThreads, 0, s>>>(d_accum, scale, d_ref_rgba, n_pixels, partial);
    k_sum_partials<<<1, kThreads, 0, s>>>(partial, grid, partial + grid);
    double total = 0.0;
    cudaError_t e = cudaMemcpyAsync(&total, partial + grid, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(partial, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "krr_image_error", __FILE__, __LINE__);
    *h_out = total / (double)n_pixels;
    return KRR_OK;
}
