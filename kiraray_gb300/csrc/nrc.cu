// Neural radiance cache (no counterpart in the reference; its learned-method
// hook is PPG's per-vertex radiance records, src/misc/render/ppg/
// guideditem.h:119-166).
//
// Encoding: multiresolution hash grid (16 levels x 2 features, 2^19 entries
// per hashed level, resolutions 16..2048 in a geometric series; coarse
// levels that fit are indexed densely), trilinear interpolation, features
// stored in BF16.  Inputs of the MLP: the 32 grid features, the normal
// mapped to [0,1], roughness and albedo, zero-padded to 64.  MLP: 5 hidden
// layers of width 64 with ReLU and a linear RGB output.  Activations and
// weights are rounded to BF16 at every layer input, products accumulate in
// FP32.  Loss: relative L2, (y - t)^2 / (sg(y)^2 + 0.01), scaled by a
// constant loss scale during the backward pass.  Optimiser: Adam on FP32
// master copies of the weights and of the hash table.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "nrc.h"

using namespace krr;

struct krr_nrc {
    krr_nrc_config cfg{};
    NrcGrid grid{};
    NrcMlp mlp{};
    uint32_t n_entries = 0;                  // total table entries
    // parameters: FP32 master, BF16 copy, Adam moments, gradient
    float *table_master = nullptr, *table_m = nullptr, *table_v = nullptr, *table_grad = nullptr;
    __nv_bfloat16 *table = nullptr;
    float *w_master = nullptr, *w_m = nullptr, *w_v = nullptr, *w_grad = nullptr;
    __nv_bfloat16 *weights = nullptr;
    // Adam step counter and bias corrections live on the device so that a
    // captured frame graph advances them on every replay: {int64 step,
    // float 1 - beta1^step, float 1 - beta2^step}.
    int64_t *step = nullptr;
    // activation buffers: [layers][cap][64] bf16, gradients float
    int64_t cap = 0;
    __nv_bfloat16 *act = nullptr;
    float *out = nullptr;                    // [cap][16]
    float *dA = nullptr, *dB = nullptr;      // [cap][64]
    float *loss = nullptr;                   // device loss accumulator
    int32_t *count_buf = nullptr;
    uint8_t *packed = nullptr;               // weights in tcgen05 canonical tiles
    uint8_t *packed_t = nullptr;             // transposed weights (backward)
    uint32_t *err = nullptr;                 // device error flags
    // inference copy (ema_decay > 0): exponential moving average of the
    // parameters after each Adam step, FP32 and BF16, and its packed tiles;
    // queries read it, training reads the parameters themselves
    float *ema_w = nullptr, *ema_table = nullptr;
    __nv_bfloat16 *ema_weights = nullptr, *ema_table_bf = nullptr;
    uint8_t *ema_packed = nullptr;
};

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Level-l grid index of integer corner (x, y, z).
__device__ __forceinline__ uint32_t grid_index(const NrcGrid &g, int l, uint32_t x, uint32_t y,
                                               uint32_t z) {
    uint32_t n1 = (uint32_t)g.res[l] + 1u;
    if (g.dense_mask & (1u << l)) return x + n1 * (y + n1 * z);
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (g.table_size - 1u);
}

struct Corner {
    uint32_t idx[8];
    float w[8];
};

__device__ __forceinline__ void corners(const NrcGrid &g, int l, const float p[3], Corner &c) {
    float fr[3];
    uint32_t base[3];
    for (int a = 0; a < 3; ++a) {
        float s = p[a] * (float)g.res[l];
        float fl = floorf(s);
        fl = fminf(fmaxf(fl, 0.f), (float)(g.res[l] - 1));
        base[a] = (uint32_t)fl;
        fr[a] = fminf(fmaxf(s - fl, 0.f), 1.f);
    }
    for (int k = 0; k < 8; ++k) {
        uint32_t x = base[0] + (k & 1), y = base[1] + ((k >> 1) & 1), z = base[2] + ((k >> 2) & 1);
        c.idx[k] = g.offset[l] + grid_index(g, l, x, y, z);
        c.w[k] = ((k & 1) ? fr[0] : 1.f - fr[0]) * (((k >> 1) & 1) ? fr[1] : 1.f - fr[1]) *
                 (((k >> 2) & 1) ? fr[2] : 1.f - fr[2]);
    }
}

__device__ __forceinline__ void normalise_position(const NrcGrid &g, const float *in, float p[3]) {
    for (int a = 0; a < 3; ++a) p[a] = fminf(fmaxf((in[a] - g.lo[a]) * g.inv_extent[a], 0.f), 1.f);
}

__device__ __forceinline__ int64_t live_count(const int32_t *d_count, int64_t cap) {
    return d_count ? min((int64_t)*d_count, cap) : cap;
}

// Encoded MLP input (bf16 values) for each query.
__global__ void k_encode(NrcGrid g, const float *__restrict__ in, const int32_t *d_count,
                         int64_t cap, const __nv_bfloat16 *__restrict__ table,
                         __nv_bfloat16 *__restrict__ X) {
    int64_t n = live_count(d_count, cap);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float *q = in + kNrcInputs * i;
        float p[3];
        normalise_position(g, q, p);
        __nv_bfloat16 *x = X + kNrcIn * i;
        for (int l = 0; l < g.levels; ++l) {
            Corner c;
            corners(g, l, p, c);
            float f0 = 0.f, f1 = 0.f;
            for (int k = 0; k < 8; ++k) {
                __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162 *>(table + 2 * (size_t)c.idx[k]);
                f0 += c.w[k] * __bfloat162float(v.x);
                f1 += c.w[k] * __bfloat162float(v.y);
            }
            x[2 * l] = __float2bfloat16_rn(f0);
            x[2 * l + 1] = __float2bfloat16_rn(f1);
        }
        int o = 2 * g.levels;
        float e[kNrcExtra];
        nrc_encode_extras(q, e);
        for (int a = 0; a < kNrcExtra; ++a) x[o + a] = __float2bfloat16_rn(e[a]);
        for (int k = o + kNrcExtra; k < kNrcIn; ++k) x[k] = __float2bfloat16_rn(0.f);
    }
}

// Y[i][0..N) = act(X[i] . W[j]) for 128-row tiles; W is [N][64].
template <int N, bool RELU, bool OUT_F32>
__global__ void __launch_bounds__(kThreads)
k_dense_fwd(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ W,
            const int32_t *d_count, int64_t cap, __nv_bfloat16 *__restrict__ Yb,
            float *__restrict__ Yf) {
    __shared__ float Ws[kNrcIn][N + 1];
    __shared__ float Xs[128][kNrcIn + 1];
    for (int e = threadIdx.x; e < N * kNrcIn; e += blockDim.x)
        Ws[e % kNrcIn][e / kNrcIn] = __bfloat162float(W[e]);
    int64_t n = live_count(d_count, cap);
    constexpr int kCols = N * 128 / kThreads;   // outputs per thread
    constexpr int kThreadsPerRow = N / kCols;
    for (int64_t t0 = (int64_t)blockIdx.x * 128; t0 < n; t0 += (int64_t)gridDim.x * 128) {
        __syncthreads();
        for (int e = threadIdx.x; e < 128 * kNrcIn; e += blockDim.x) {
            int64_t r = t0 + e / kNrcIn;
            Xs[e / kNrcIn][e % kNrcIn] = r < n ? __bfloat162float(X[r * kNrcIn + e % kNrcIn]) : 0.f;
        }
        __syncthreads();
        int row = threadIdx.x / kThreadsPerRow;
        int c0 = (threadIdx.x % kThreadsPerRow) * kCols;
        float acc[kCols];
#pragma unroll
        for (int j = 0; j < kCols; ++j) acc[j] = 0.f;
        for (int k = 0; k < kNrcIn; ++k) {
            float x = Xs[row][k];
#pragma unroll
            for (int j = 0; j < kCols; ++j) acc[j] = fmaf(x, Ws[k][c0 + j], acc[j]);
        }
        int64_t r = t0 + row;
        if (r < n) {
#pragma unroll
            for (int j = 0; j < kCols; ++j) {
                float v = RELU ? fmaxf(acc[j], 0.f) : acc[j];
                if (OUT_F32) Yf[r * N + c0 + j] = v;
                else Yb[r * N + c0 + j] = __float2bfloat16_rn(v);
            }
        }
    }
}

// dX[i][k] = sum_j dY[i][j] W[j][k], masked by the ReLU of the layer input
// (X > 0) when MASK; dY is [n][N] float, W is [N][64].
template <int N, bool MASK>
__global__ void __launch_bounds__(kThreads)
k_dense_bwd(const float *__restrict__ dY, const __nv_bfloat16 *__restrict__ W,
            const __nv_bfloat16 *__restrict__ Xin, const int32_t *d_count, int64_t cap,
            float *__restrict__ dX) {
    __shared__ float Ws[N][kNrcIn + 1];
    __shared__ float Ds[128][N + 1];
    for (int e = threadIdx.x; e < N * kNrcIn; e += blockDim.x)
        Ws[e / kNrcIn][e % kNrcIn] = __bfloat162float(W[e]);
    int64_t n = live_count(d_count, cap);
    constexpr int kCols = kNrcIn * 128 / kThreads;
    constexpr int kThreadsPerRow = kNrcIn / kCols;
    for (int64_t t0 = (int64_t)blockIdx.x * 128; t0 < n; t0 += (int64_t)gridDim.x * 128) {
        __syncthreads();
        for (int e = threadIdx.x; e < 128 * N; e += blockDim.x) {
            int64_t r = t0 + e / N;
            Ds[e / N][e % N] = r < n ? bf(dY[r * N + e % N]) : 0.f;
        }
        __syncthreads();
        int row = threadIdx.x / kThreadsPerRow;
        int c0 = (threadIdx.x % kThreadsPerRow) * kCols;
        float acc[kCols];
#pragma unroll
        for (int j = 0; j < kCols; ++j) acc[j] = 0.f;
        for (int k = 0; k < N; ++k) {
            float d = Ds[row][k];
#pragma unroll
            for (int j = 0; j < kCols; ++j) acc[j] = fmaf(d, Ws[k][c0 + j], acc[j]);
        }
        int64_t r = t0 + row;
        if (r < n) {
#pragma unroll
            for (int j = 0; j < kCols; ++j) {
                float v = acc[j];
                if (MASK && !(__bfloat162float(Xin[r * kNrcIn + c0 + j]) > 0.f)) v = 0.f;
                dX[r * kNrcIn + c0 + j] = v;
            }
        }
    }
}

// dW[j][k] += sum_i dY[i][j] X[i][k] over a chunk of rows per block.
template <int N>
__global__ void __launch_bounds__(kThreads)
k_dense_wgrad(const float *__restrict__ dY, const __nv_bfloat16 *__restrict__ X,
              const int32_t *d_count, int64_t cap, float *__restrict__ dW) {
    constexpr int kRows = 64;
    __shared__ float Ds[kRows][N + 1];
    __shared__ float Xs[kRows][kNrcIn + 1];
    constexpr int kOut = N * kNrcIn / kThreads;   // outputs per thread
    int64_t n = live_count(d_count, cap);
    float acc[kOut];
#pragma unroll
    for (int j = 0; j < kOut; ++j) acc[j] = 0.f;
    int o0 = threadIdx.x * kOut;
    for (int64_t t0 = (int64_t)blockIdx.x * kRows; t0 < n; t0 += (int64_t)gridDim.x * kRows) {
        __syncthreads();
        for (int e = threadIdx.x; e < kRows * N; e += blockDim.x) {
            int64_t r = t0 + e / N;
            Ds[e / N][e % N] = r < n ? bf(dY[r * N + e % N]) : 0.f;
        }
        for (int e = threadIdx.x; e < kRows * kNrcIn; e += blockDim.x) {
            int64_t r = t0 + e / kNrcIn;
            Xs[e / kNrcIn][e % kNrcIn] = r < n ? __bfloat162float(X[r * kNrcIn + e % kNrcIn]) : 0.f;
        }
        __syncthreads();
        for (int r = 0; r < kRows; ++r) {
#pragma unroll
            for (int j = 0; j < kOut; ++j) {
                int o = o0 + j;
                acc[j] = fmaf(Ds[r][o / kNrcIn], Xs[r][o % kNrcIn], acc[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kOut; ++j) atomicAdd(dW + o0 + j, acc[j]);
}

// Relative L2 loss gradient (scaled) and loss sum.
__global__ void k_loss(const float *__restrict__ Y, const float *__restrict__ T, const int32_t *d_count,
                       int64_t cap, float scale, float *__restrict__ dY, float *loss) {
    int64_t n = live_count(d_count, cap);
    float inv = 1.f / (float)(max(n, (int64_t)1) * 3);
    float lsum = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < kNrcOutPad; ++c) {
            float g = 0.f;
            if (c < 3) {
                float y = Y[i * kNrcOutPad + c], t = T[3 * i + c];
                float den = y * y + 0.01f;
                lsum += (y - t) * (y - t) / den;
                g = 2.f * (y - t) / den * inv * scale;
            }
            dY[i * kNrcOutPad + c] = g;
        }
    }
    for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum * inv);
}

// Scatter the gradient of the 32 grid features into the table gradient.
__global__ void k_encode_bwd(NrcGrid g, const float *__restrict__ in, const float *__restrict__ dX,
                             const int32_t *d_count, int64_t cap, float *__restrict__ tgrad) {
    int64_t n = live_count(d_count, cap);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float p[3];
        normalise_position(g, in + kNrcInputs * i, p);
        for (int l = 0; l < g.levels; ++l) {
            float d0 = dX[i * kNrcIn + 2 * l], d1 = dX[i * kNrcIn + 2 * l + 1];
            if (d0 == 0.f && d1 == 0.f) continue;
            Corner c;
            corners(g, l, p, c);
            // one 8-byte vector atomic per corner (both features of the entry)
            for (int k = 0; k < 8; ++k)
                atomicAdd(reinterpret_cast<float2 *>(tgrad) + c.idx[k],
                          make_float2(c.w[k] * d0, c.w[k] * d1));
        }
    }
}

// Adam on an FP32 master array; writes the BF16 copy and clears the gradient.
// Advances the device step counter and stores the bias corrections.
// A loss that is not finite marks the cache as diverged (err[1]); a diverged
// cache takes no further steps.
__global__ void k_adam_step(int64_t *step, double b1, double b2, const float *loss, uint32_t *err) {
    if (!isfinite(*loss)) err[1] = 1u;
    if (err[1]) return;
    int64_t t = *step + 1;
    *step = t;
    float *bc = reinterpret_cast<float *>(step + 1);
    bc[0] = (float)(1.0 - pow(b1, (double)t));
    bc[1] = (float)(1.0 - pow(b2, (double)t));
}

struct AdamArgs {
    float lr, b1, b2, eps, grad_scale, bc1, bc2;
};

// One Adam update; a non-finite gradient leaves the parameter and its moments
// unchanged.  Returns the new FP32 master weight.
__device__ __forceinline__ float adam_one(const AdamArgs &a, float g, float &m, float &v, float w) {
    float gr = g * a.grad_scale;
    if (!isfinite(gr)) return w;
    m = a.b1 * m + (1.f - a.b1) * gr;
    v = a.b2 * v + (1.f - a.b2) * gr * gr;
    return w - a.lr * (m / a.bc1) / (sqrtf(v / a.bc2) + a.eps);
}

// Adam over n parameters (FP32 masters w, moments m and v, gradient grad which
// is cleared, BF16 copy wb).  A thread streams two groups of four parameters
// per step (16-byte accesses, all eight loads issued before the arithmetic):
// the kernel is bound by HBM bandwidth, 34 bytes per parameter.
__device__ __forceinline__ void adam4(const AdamArgs &a, float4 g, float4 &mm, float4 &vv, float4 &ww) {
    ww.x = adam_one(a, g.x, mm.x, vv.x, ww.x);
    ww.y = adam_one(a, g.y, mm.y, vv.y, ww.y);
    ww.z = adam_one(a, g.z, mm.z, vv.z, ww.z);
    ww.w = adam_one(a, g.w, mm.w, vv.w, ww.w);
}

__device__ __forceinline__ void store_bf16x4(__nv_bfloat16 *dst, int64_t i, float4 x) {
    __nv_bfloat162 lo = __floats2bfloat162_rn(x.x, x.y), hi = __floats2bfloat162_rn(x.z, x.w);
    reinterpret_cast<uint2 *>(dst)[i] =
        make_uint2(*reinterpret_cast<uint32_t *>(&lo), *reinterpret_cast<uint32_t *>(&hi));
}

__device__ __forceinline__ void adam_store4(float *m, float *v, float *w, float *grad,
                                            __nv_bfloat16 *wb, int64_t i, float4 mm, float4 vv,
                                            float4 ww) {
    reinterpret_cast<float4 *>(grad)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    reinterpret_cast<float4 *>(m)[i] = mm;
    reinterpret_cast<float4 *>(v)[i] = vv;
    reinterpret_cast<float4 *>(w)[i] = ww;
    store_bf16x4(wb, i, ww);
}

// ema <- d ema + (1 - d) w, FP32 and BF16
struct EmaArgs {
    float *e;
    __nv_bfloat16 *eb;
    float d;
};
__device__ __forceinline__ void ema_store4(const EmaArgs &x, int64_t i, float4 ww) {
    float4 e = reinterpret_cast<const float4 *>(x.e)[i];
    const float c = 1.f - x.d;
    e = make_float4(x.d * e.x + c * ww.x, x.d * e.y + c * ww.y, x.d * e.z + c * ww.z, x.d * e.w + c * ww.w);
    reinterpret_cast<float4 *>(x.e)[i] = e;
    store_bf16x4(x.eb, i, e);
}

__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       float *__restrict__ grad, __nv_bfloat16 *__restrict__ wb, int64_t n, float lr,
                       float b1, float b2, float eps, float grad_scale, const int64_t *__restrict__ step,
                       const uint32_t *__restrict__ diverged, EmaArgs ema) {
    if (*diverged) {   // keep the parameters; drop the gradient
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x)
            grad[i] = 0.f;
        return;
    }
    AdamArgs a{lr, b1, b2, eps, grad_scale, reinterpret_cast<const float *>(step + 1)[0],
               reinterpret_cast<const float *>(step + 1)[1]};
    const int64_t n4 = n >> 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += 2 * stride) {
        const int64_t j = i + stride;
        const bool two = j < n4;
        float4 g0 = reinterpret_cast<const float4 *>(grad)[i];
        float4 m0 = reinterpret_cast<const float4 *>(m)[i];
        float4 v0 = reinterpret_cast<const float4 *>(v)[i];
        float4 w0 = reinterpret_cast<const float4 *>(w)[i];
        float4 g1{}, m1{}, v1{}, w1{};
        if (two) {
            g1 = reinterpret_cast<const float4 *>(grad)[j];
            m1 = reinterpret_cast<const float4 *>(m)[j];
            v1 = reinterpret_cast<const float4 *>(v)[j];
            w1 = reinterpret_cast<const float4 *>(w)[j];
        }
        adam4(a, g0, m0, v0, w0);
        adam_store4(m, v, w, grad, wb, i, m0, v0, w0);
        if (ema.e) ema_store4(ema, i, w0);
        if (two) {
            adam4(a, g1, m1, v1, w1);
            adam_store4(m, v, w, grad, wb, j, m1, v1, w1);
            if (ema.e) ema_store4(ema, j, w1);
        }
    }
    for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        float g = grad[i], mm = m[i], vv = v[i];
        grad[i] = 0.f;
        float ww = adam_one(a, g, mm, vv, w[i]);
        m[i] = mm;
        v[i] = vv;
        w[i] = ww;
        wb[i] = __float2bfloat16_rn(ww);
        if (ema.e) {
            const float e = ema.d * ema.e[i] + (1.f - ema.d) * ww;
            ema.e[i] = e;
            ema.eb[i] = __float2bfloat16_rn(e);
        }
    }
}

__global__ void k_to_bf16(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

int grid_for(int64_t n, int per = kThreads) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t g = (n + per - 1) / per;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)std::max(sms, 1) * 8));
}

// Deterministic parameter initialisation (splitmix64).
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)((next() >> 40) * (1.0 / 16777216.0)); }
};

int ensure_capacity(krr_nrc *n, int64_t cap) {
    if (cap <= n->cap) return KRR_OK;
    cudaFree(n->act); cudaFree(n->out); cudaFree(n->dA); cudaFree(n->dB);
    n->act = nullptr; n->out = nullptr; n->dA = nullptr; n->dB = nullptr;
    int layers = n->mlp.layers;   // inputs of every layer: encoding + hidden outputs
    KRR_CUDA(cudaMalloc(&n->act, (size_t)layers * cap * kNrcIn * sizeof(__nv_bfloat16)));
    KRR_CUDA(cudaMalloc(&n->out, (size_t)cap * kNrcOutPad * sizeof(float)));
    KRR_CUDA(cudaMalloc(&n->dA, (size_t)cap * kNrcIn * sizeof(float)));
    KRR_CUDA(cudaMalloc(&n->dB, (size_t)cap * kNrcIn * sizeof(float)));
    n->cap = cap;
    return KRR_OK;
}

// Forward pass over `cap` rows (live count on the device); leaves the layer
// inputs in n->act and the output in n->out.
// inference = true: the inference copy of the parameters (the moving
// average when ema_decay > 0), for queries; false: the trained parameters.
int forward(krr_nrc *n, const float *d_inputs, const int32_t *d_count, int64_t cap, cudaStream_t s,
            bool keep_acts = true, bool inference = false) {
    KRR_TRY(ensure_capacity(n, cap));
    __nv_bfloat16 *A = n->act;
    const bool ema = inference && n->ema_w;
    const __nv_bfloat16 *table = ema ? n->ema_table_bf : n->table;
    const __nv_bfloat16 *weights = ema ? n->ema_weights : n->weights;
    if (n->cfg.tensor_cores)
        return nrc_forward_tc(n->grid, n->mlp, d_inputs, d_count, cap, table, ema ? n->ema_packed : n->packed,
                              n->out, keep_acts ? A : nullptr, n->err, s);
    k_encode<<<grid_for(cap), kThreads, 0, s>>>(n->grid, d_inputs, d_count, cap, table, A);
    KRR_CUDA(cudaGetLastError());
    int blocks = grid_for(cap, 128);
    for (int l = 0; l < n->mlp.layers; ++l) {
        const __nv_bfloat16 *X = A + (size_t)l * cap * kNrcIn;
        const __nv_bfloat16 *W = weights + n->mlp.w_offset[l];
        if (l + 1 < n->mlp.layers) {
            __nv_bfloat16 *Y = A + (size_t)(l + 1) * cap * kNrcIn;
            k_dense_fwd<kNrcWidth, true, false><<<blocks, kThreads, 0, s>>>(X, W, d_count, cap, Y, nullptr);
        } else {
            k_dense_fwd<kNrcOutPad, false, true><<<blocks, kThreads, 0, s>>>(X, W, d_count, cap, nullptr, n->out);
        }
        KRR_CUDA(cudaGetLastError());
    }
    return KRR_OK;
}

__global__ void k_write_rgb(const float *__restrict__ out, const int32_t *d_count, int64_t cap,
                            float *__restrict__ dst) {
    int64_t n = live_count(d_count, cap);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) dst[3 * i + c] = out[i * kNrcOutPad + c];
}

}  // namespace

namespace krr {

NrcView nrc_view(const krr_nrc *n) { return NrcView{n->grid, n->mlp, n->table, n->weights}; }
int64_t nrc_batch_size(const krr_nrc *n) { return n->cfg.batch_size; }
int32_t nrc_train_stride(const krr_nrc *n) { return n->cfg.train_pixel_stride; }
float nrc_termination_spread(const krr_nrc *n) { return n->cfg.termination_spread; }
const uint32_t *nrc_diverged_flag(const krr_nrc *n) { return n->err + 1; }
uint32_t *nrc_error_flags(krr_nrc *n) { return n->err; }

int nrc_query_device(krr_nrc *n, const float *d_inputs, const int32_t *d_count, int64_t cap,
                     float *d_out, cudaStream_t s) {
    if (cap <= 0) return KRR_OK;
    KRR_TRY(forward(n, d_inputs, d_count, cap, s, false, true));
    k_write_rgb<<<grid_for(cap), kThreads, 0, s>>>(n->out, d_count, cap, d_out);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

// Loss, MLP backward and hash-grid backward of the last forward pass (its
// activations in n->act): w_grad and table_grad receive the scaled gradients.
int backward(krr_nrc *n, const float *d_inputs, const float *d_targets, const int32_t *d_count,
             int64_t cap, cudaStream_t s) {
    const float scale = n->cfg.loss_scale;
    KRR_CUDA(cudaMemsetAsync(n->loss, 0, sizeof(float), s));
    k_loss<<<grid_for(cap), kThreads, 0, s>>>(n->out, d_targets, d_count, cap, scale, n->dA, n->loss);
    KRR_CUDA(cudaGetLastError());
    float *dY = n->dA, *dX = n->dB;
    if (n->cfg.tensor_cores) {
        // dX0 -> dB, dW += on the tensor cores
        KRR_TRY(nrc_backward_tc(n->mlp, n->dA, n->act, d_count, cap, n->packed_t, n->dB, n->w_grad,
                                n->err, s));
        dY = n->dB;
    } else {
        // backward through the layers: dY holds the gradient of layer l's output
        int blocks = grid_for(cap, 128);
        int wblocks = grid_for(cap, 64);
        for (int l = n->mlp.layers - 1; l >= 0; --l) {
            const __nv_bfloat16 *X = n->act + (size_t)l * cap * kNrcIn;
            const __nv_bfloat16 *W = n->weights + n->mlp.w_offset[l];
            float *dW = n->w_grad + n->mlp.w_offset[l];
            bool out_layer = l + 1 == n->mlp.layers;
            if (out_layer) k_dense_wgrad<kNrcOutPad><<<wblocks, kThreads, 0, s>>>(dY, X, d_count, cap, dW);
            else k_dense_wgrad<kNrcWidth><<<wblocks, kThreads, 0, s>>>(dY, X, d_count, cap, dW);
            KRR_CUDA(cudaGetLastError());
            if (l > 0) {
                if (out_layer) k_dense_bwd<kNrcOutPad, true><<<blocks, kThreads, 0, s>>>(dY, W, X, d_count, cap, dX);
                else k_dense_bwd<kNrcWidth, true><<<blocks, kThreads, 0, s>>>(dY, W, X, d_count, cap, dX);
            } else {
                if (out_layer) k_dense_bwd<kNrcOutPad, false><<<blocks, kThreads, 0, s>>>(dY, W, X, d_count, cap, dX);
                else k_dense_bwd<kNrcWidth, false><<<blocks, kThreads, 0, s>>>(dY, W, X, d_count, cap, dX);
            }
            KRR_CUDA(cudaGetLastError());
            std::swap(dY, dX);
        }
    }
    // dY now holds the gradient of the encoded input
    k_encode_bwd<<<grid_for(cap), kThreads, 0, s>>>(n->grid, d_inputs, dY, d_count, cap, n->table_grad);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

// Both weight layouts of the tensor-core kernels, from the BF16 weights, and
// the forward layout of the inference copy.
int pack_weights(krr_nrc *n, cudaStream_t s) {
    if (!n->cfg.tensor_cores) return KRR_OK;
    KRR_TRY(nrc_pack_weights(n->weights, n->mlp, n->packed, s));
    if (n->ema_w) KRR_TRY(nrc_pack_weights(n->ema_weights, n->mlp, n->ema_packed, s));
    return nrc_pack_weights_t(n->weights, n->mlp, n->packed_t, s);
}

// The inference copy restarts from the trained parameters.
int reset_ema(krr_nrc *n, cudaStream_t s) {
    if (!n->ema_w) return KRR_OK;
    const int64_t tn = (int64_t)n->n_entries * n->grid.features;
    KRR_CUDA(cudaMemcpyAsync(n->ema_w, n->w_master, n->mlp.n_params * 4, cudaMemcpyDeviceToDevice, s));
    KRR_CUDA(cudaMemcpyAsync(n->ema_table, n->table_master, tn * 4, cudaMemcpyDeviceToDevice, s));
    k_to_bf16<<<grid_for(n->mlp.n_params), kThreads, 0, s>>>(n->ema_w, n->ema_weights, n->mlp.n_params);
    k_to_bf16<<<grid_for(tn), kThreads, 0, s>>>(n->ema_table, n->ema_table_bf, tn);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

int nrc_train_device(krr_nrc *n, const float *d_inputs, const float *d_targets,
                     const int32_t *d_count, int64_t cap, cudaStream_t s) {
    if (cap <= 0) return KRR_OK;
    KRR_TRY(forward(n, d_inputs, d_count, cap, s));
    KRR_TRY(backward(n, d_inputs, d_targets, d_count, cap, s));
    const float scale = n->cfg.loss_scale;
    // Adam
    const krr_nrc_config &c = n->cfg;
    k_adam_step<<<1, 1, 0, s>>>(n->step, (double)c.beta1, (double)c.beta2, n->loss, n->err);
    const EmaArgs ew{n->ema_w, n->ema_weights, c.ema_decay}, et{n->ema_table, n->ema_table_bf, c.ema_decay};
    k_adam<<<grid_for(n->mlp.n_params), kThreads, 0, s>>>(n->w_master, n->w_m, n->w_v, n->w_grad,
                                                           n->weights, n->mlp.n_params, c.learning_rate,
                                                           c.beta1, c.beta2, c.epsilon, 1.f / scale,
                                                           n->step, n->err + 1, ew);
    int64_t tn = (int64_t)n->n_entries * n->grid.features;
    k_adam<<<grid_for(tn), kThreads, 0, s>>>(n->table_master, n->table_m, n->table_v, n->table_grad,
                                             n->table, tn, c.learning_rate, c.beta1, c.beta2,
                                             c.epsilon, 1.f / scale, n->step, n->err + 1, et);
    KRR_CUDA(cudaGetLastError());
    return pack_weights(n, s);
}

}  // namespace krr

// ------------------------------------------------------------------ C ABI
extern "C" void krr_nrc_config_default(krr_nrc_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->n_levels = 16;
    c->features_per_level = 2;
    c->log2_table_size = 19;
    c->base_resolution = 16;
    c->max_resolution = 2048;
    c->hidden_layers = 5;
    c->learning_rate = 1e-2f;
    c->beta1 = 0.9f;
    c->beta2 = 0.99f;
    c->epsilon = 1e-15f;
    c->loss_scale = 128.f;
    c->batch_size = 65536;
    c->train_pixel_stride = 16;
    c->seed = 3;
    c->tensor_cores = 1;
    c->termination_spread = 0.01f;
    for (int k = 0; k < 3; ++k) { c->scene_lo[k] = 0.f; c->scene_hi[k] = 1.f; }
}

extern "C" int krr_nrc_create(const krr_nrc_config *cfg, krr_nrc **out) {
    KRR_CHECK_ARG(cfg && out, "NULL argument");
    KRR_CHECK_ARG(cfg->n_levels >= 1 && cfg->n_levels <= kNrcMaxLevels, "n_levels must be 1..16");
    KRR_CHECK_ARG(cfg->features_per_level == 2, "features_per_level must be 2");
    KRR_CHECK_ARG(2 * cfg->n_levels + 7 <= kNrcIn, "encoded input wider than 64");
    KRR_CHECK_ARG(cfg->log2_table_size >= 8 && cfg->log2_table_size <= 24, "log2_table_size 8..24");
    KRR_CHECK_ARG(cfg->hidden_layers >= 1 && cfg->hidden_layers <= 7, "hidden_layers 1..7");
    KRR_CHECK_ARG(cfg->base_resolution >= 2 && cfg->max_resolution >= cfg->base_resolution,
                  "bad resolutions");
    KRR_CHECK_ARG(cfg->batch_size > 0, "batch_size must be positive");
    KRR_CHECK_ARG(cfg->ema_decay >= 0.f && cfg->ema_decay < 1.f, "ema_decay must be in [0, 1)");
    krr_nrc *n = new krr_nrc();
    n->cfg = *cfg;
    if (n->cfg.train_pixel_stride < 1) n->cfg.train_pixel_stride = 1;
    NrcGrid &g = n->grid;
    g.levels = cfg->n_levels;
    g.features = 2;
    g.table_size = 1u << cfg->log2_table_size;
    double b = cfg->n_levels > 1 ? std::exp((std::log((double)cfg->max_resolution) -
                                             std::log((double)cfg->base_resolution)) / (cfg->n_levels - 1))
                                 : 1.0;
    uint32_t off = 0;
    for (int l = 0; l < g.levels; ++l) {
        g.res[l] = (int)std::floor(cfg->base_resolution * std::pow(b, l) + 1e-6);
        uint64_t n1 = (uint64_t)g.res[l] + 1;
        uint64_t dense = n1 * n1 * n1;
        g.size[l] = dense <= g.table_size ? (uint32_t)dense : g.table_size;
        if (dense <= g.table_size) g.dense_mask |= 1u << l;
        g.offset[l] = off;
        off += g.size[l];
    }
    n->n_entries = off;
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = cfg->scene_lo[a];
        float e = cfg->scene_hi[a] - cfg->scene_lo[a];
        g.inv_extent[a] = e > 0.f ? 1.f / e : 1.f;
    }
    NrcMlp &m = n->mlp;
    m.layers = cfg->hidden_layers + 1;
    int o = 0;
    for (int l = 0; l < m.layers; ++l) {
        m.w_offset[l] = o;
        o += (l + 1 < m.layers ? kNrcWidth : kNrcOutPad) * kNrcIn;
    }
    m.n_params = o;
    // host initialisation
    Rng rng{0x6a09e667f3bcc908ULL ^ (uint64_t)cfg->seed};
    std::vector<float> w(m.n_params, 0.f);
    for (int l = 0; l < m.layers; ++l) {
        int rows = l + 1 < m.layers ? kNrcWidth : 3;
        int fan_in = l == 0 ? 2 * g.levels + kNrcExtra : kNrcWidth;
        float a = std::sqrt(6.f / (float)(fan_in + rows));
        for (int r = 0; r < rows; ++r)
            for (int k = 0; k < fan_in; ++k) w[m.w_offset[l] + r * kNrcIn + k] = (2.f * rng.uniform() - 1.f) * a;
    }
    size_t tn = (size_t)n->n_entries * 2;
    std::vector<float> t(tn);
    for (auto &x : t) x = (2.f * rng.uniform() - 1.f) * 1e-4f;
    int st = KRR_OK;
    auto alloc = [&](void **p, size_t bytes) {
        if (st != KRR_OK) return;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
        if (e != cudaSuccess) st = cuda_status(e, "cudaMalloc", __FILE__, __LINE__);
    };
    alloc((void **)&n->w_master, m.n_params * 4);
    alloc((void **)&n->w_m, m.n_params * 4);
    alloc((void **)&n->w_v, m.n_params * 4);
    alloc((void **)&n->w_grad, m.n_params * 4);
    alloc((void **)&n->weights, m.n_params * 2);
    alloc((void **)&n->table_master, tn * 4);
    alloc((void **)&n->table_m, tn * 4);
    alloc((void **)&n->table_v, tn * 4);
    alloc((void **)&n->table_grad, tn * 4);
    alloc((void **)&n->table, tn * 2);
    alloc((void **)&n->loss, 16);
    alloc((void **)&n->packed, (size_t)(m.layers - 1) * kNrcWidth * kNrcIn * 2 + kNrcOutPad * kNrcIn * 2);
    alloc((void **)&n->packed_t, (size_t)(m.layers - 1) * kNrcWidth * kNrcIn * 2 + kNrcIn * kNrcOutPad * 2);
    alloc((void **)&n->err, 16);
    alloc((void **)&n->step, 16);
    if (cfg->ema_decay > 0.f) {
        alloc((void **)&n->ema_w, m.n_params * 4);
        alloc((void **)&n->ema_weights, m.n_params * 2);
        alloc((void **)&n->ema_table, tn * 4);
        alloc((void **)&n->ema_table_bf, tn * 2);
        alloc((void **)&n->ema_packed, (size_t)(m.layers - 1) * kNrcWidth * kNrcIn * 2 + kNrcOutPad * kNrcIn * 2);
    }
    if (st == KRR_OK) {
        cudaMemcpy(n->w_master, w.data(), m.n_params * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(n->table_master, t.data(), tn * 4, cudaMemcpyHostToDevice);
        k_to_bf16<<<grid_for(m.n_params), kThreads>>>(n->w_master, n->weights, m.n_params);
        k_to_bf16<<<grid_for((int64_t)tn), kThreads>>>(n->table_master, n->table, (int64_t)tn);
        reset_ema(n, 0);
        pack_weights(n, 0);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_status(e, "krr_nrc_create", __FILE__, __LINE__);
    }
    if (st != KRR_OK) {
        krr_nrc_destroy(n);
        return st;
    }
    *out = n;
    return KRR_OK;
}

extern "C" int krr_nrc_destroy(krr_nrc *n) {
    if (!n) return KRR_OK;
    cudaDeviceSynchronize();
    for (void *p : {(void *)n->table_master, (void *)n->table_m, (void *)n->table_v,
                    (void *)n->table_grad, (void *)n->table, (void *)n->w_master, (void *)n->w_m,
                    (void *)n->w_v, (void *)n->w_grad, (void *)n->weights, (void *)n->act,
                    (void *)n->out, (void *)n->dA, (void *)n->dB, (void *)n->loss,
                    (void *)n->packed, (void *)n->packed_t, (void *)n->err, (void *)n->step,
                    (void *)n->ema_w, (void *)n->ema_weights, (void *)n->ema_table,
                    (void *)n->ema_table_bf, (void *)n->ema_packed})
        cudaFree(p);
    delete n;
    return KRR_OK;
}

extern "C" int krr_nrc_query(krr_nrc *n, const float *d_inputs, int64_t count, float *d_out,
                             void *stream) {
    KRR_CHECK_ARG(n && (count == 0 || (d_inputs && d_out)) && count >= 0, "bad argument");
    return nrc_query_device(n, d_inputs, nullptr, count, d_out, as_stream(stream));
}

extern "C" int krr_nrc_train_step(krr_nrc *n, const float *d_inputs, const float *d_targets,
                                  int64_t count, float *h_loss, void *stream) {
    KRR_CHECK_ARG(n && (count == 0 || (d_inputs && d_targets)) && count >= 0, "bad argument");
    cudaStream_t s = as_stream(stream);
    KRR_TRY(nrc_train_device(n, d_inputs, d_targets, nullptr, count, s));
    if (h_loss) {
        KRR_CUDA(cudaMemcpyAsync(h_loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        KRR_CUDA(cudaStreamSynchronize(s));
    }
    return KRR_OK;
}

extern "C" int krr_nrc_info(const krr_nrc *n, krr_nrc_info_t *info) {
    KRR_CHECK_ARG(n && info, "NULL argument");
    info->n_params_mlp = n->mlp.n_params;
    info->n_table_entries = (int64_t)n->n_entries;
    info->n_levels = n->grid.levels;
    for (int l = 0; l < n->grid.levels; ++l) {
        info->resolution[l] = n->grid.res[l];
        info->level_offset[l] = n->grid.offset[l];
        info->level_size[l] = n->grid.size[l];
    }
    int64_t step = 0;
    KRR_CUDA(cudaDeviceSynchronize());
    KRR_CUDA(cudaMemcpy(&step, n->step, sizeof(step), cudaMemcpyDeviceToHost));
    info->step = step;
    return KRR_OK;
}

// Parameter access for tests and checkpoints: which = 0 MLP weights (FP32
// master, [layer][out][64]), 1 hash table (FP32 master, [entry][2]); 2 and 3
// the same arrays of the inference copy (ema_decay > 0).
extern "C" int krr_nrc_get_params(const krr_nrc *n, int32_t which, float *h_dst, int64_t count) {
    KRR_CHECK_ARG(n && h_dst && which >= 0 && which <= 3, "bad argument");
    KRR_CHECK_ARG(which < 2 || n->ema_w, "the cache keeps no inference copy (ema_decay 0)");
    int64_t total = (which & 1) == 0 ? n->mlp.n_params : (int64_t)n->n_entries * 2;
    KRR_CHECK_ARG(count == total, "count does not match the parameter array");
    const float *src[4] = {n->w_master, n->table_master, n->ema_w, n->ema_table};
    KRR_CUDA(cudaDeviceSynchronize());
    KRR_CUDA(cudaMemcpy(h_dst, src[which], total * 4, cudaMemcpyDeviceToHost));
    return KRR_OK;
}

extern "C" int krr_nrc_set_params(krr_nrc *n, int32_t which, const float *h_src, int64_t count) {
    KRR_CHECK_ARG(n && h_src, "NULL argument");
    int64_t total = which == 0 ? n->mlp.n_params : (int64_t)n->n_entries * 2;
    KRR_CHECK_ARG(count == total, "count does not match the parameter array");
    float *dst = which == 0 ? n->w_master : n->table_master;
    __nv_bfloat16 *bdst = which == 0 ? n->weights : n->table;
    KRR_CUDA(cudaDeviceSynchronize());
    KRR_CUDA(cudaMemcpy(dst, h_src, total * 4, cudaMemcpyHostToDevice));
    k_to_bf16<<<grid_for(total), kThreads>>>(dst, bdst, total);
    KRR_TRY(reset_ema(n, 0));   // the inference copy restarts from the new parameters
    KRR_TRY(pack_weights(n, 0));
    KRR_CUDA(cudaMemset(n->err + 1, 0, sizeof(uint32_t)));   // new parameters: not diverged
    KRR_CUDA(cudaDeviceSynchronize());
    return KRR_OK;
}

extern "C" int krr_nrc_status(krr_nrc *n, uint32_t *out_flags, int32_t *out_diverged, void *stream) {
    KRR_CHECK_ARG(n != nullptr, "NULL argument");
    cudaStream_t s = as_stream(stream);
    uint32_t w[2] = {0, 0};
    KRR_CUDA(cudaMemcpyAsync(w, n->err, sizeof(w), cudaMemcpyDeviceToHost, s));
    KRR_CUDA(cudaMemsetAsync(n->err, 0, sizeof(uint32_t), s));
    KRR_CUDA(cudaStreamSynchronize(s));
    if (out_flags) *out_flags = w[0];
    if (out_diverged) *out_diverged = w[1] ? 1 : 0;
    return KRR_OK;
}

// Checkpoint file: a fixed header, then the FP32 arrays in this order: MLP
// weights, their Adam moments m and v, hash table, its moments m and v; with
// cfg.ema_decay > 0 then the inference copy's MLP weights and table.
namespace {
struct NrcFileHeader {
    char magic[8];              // "KRRNRC02"
    uint32_t header_bytes;      // sizeof(NrcFileHeader)
    uint32_t config_bytes;      // sizeof(krr_nrc_config)
    krr_nrc_config cfg;
    int64_t n_params;
    int64_t n_table_values;     // entries x 2
    int64_t step;
    float bias_correction[2];
    uint32_t diverged;
    uint32_t reserved;
};
constexpr char kNrcMagic[8] = {'K', 'R', 'R', 'N', 'R', 'C', '0', '2'};

bool same_structure(const krr_nrc_config &a, const krr_nrc_config &b) {
    return a.n_levels == b.n_levels && a.features_per_level == b.features_per_level &&
           a.log2_table_size == b.log2_table_size && a.base_resolution == b.base_resolution &&
           a.max_resolution == b.max_resolution && a.hidden_layers == b.hidden_layers;
}
}  // namespace

extern "C" int krr_nrc_save(const krr_nrc *n, const char *path) {
    KRR_CHECK_ARG(n && path, "NULL argument");
    KRR_CUDA(cudaDeviceSynchronize());
    NrcFileHeader h{};
    std::memcpy(h.magic, kNrcMagic, 8);
    h.header_bytes = sizeof(NrcFileHeader);
    h.config_bytes = sizeof(krr_nrc_config);
    h.cfg = n->cfg;
    h.n_params = n->mlp.n_params;
    h.n_table_values = (int64_t)n->n_entries * 2;
    unsigned char st[16];
    KRR_CUDA(cudaMemcpy(st, n->step, 16, cudaMemcpyDeviceToHost));
    std::memcpy(&h.step, st, 8);
    std::memcpy(h.bias_correction, st + 8, 8);
    uint32_t w[2];
    KRR_CUDA(cudaMemcpy(w, n->err, sizeof(w), cudaMemcpyDeviceToHost));
    h.diverged = w[1];
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(KRR_ERR_INVALID_ARGUMENT, "krr_nrc_save: cannot open %s", path);
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
    std::vector<float> buf;
    const float *arrays[8] = {n->w_master, n->w_m, n->w_v, n->table_master, n->table_m, n->table_v,
                              n->ema_w, n->ema_table};
    const int n_arrays = n->ema_w ? 8 : 6;
    for (int k = 0; k < n_arrays && ok; ++k) {
        const size_t cnt = (size_t)(k < 3 || k == 6 ? h.n_params : h.n_table_values);
        buf.resize(cnt);
        if (cudaMemcpy(buf.data(), arrays[k], cnt * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
            std::fclose(f);
            return fail(KRR_ERR_CUDA, "krr_nrc_save: device copy failed");
        }
        ok = std::fwrite(buf.data(), 4, cnt, f) == cnt;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(KRR_ERR_INVALID_ARGUMENT, "krr_nrc_save: write to %s failed", path);
    return KRR_OK;
}

extern "C" int krr_nrc_load(krr_nrc *n, const char *path) {
    KRR_CHECK_ARG(n && path, "NULL argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(KRR_ERR_INVALID_ARGUMENT, "krr_nrc_load: cannot open %s", path);
    NrcFileHeader h{};
    const bool hdr = std::fread(&h, sizeof(h), 1, f) == 1;
    if (!hdr || std::memcmp(h.magic, kNrcMagic, 8) != 0 || h.header_bytes != sizeof(NrcFileHeader) ||
        h.config_bytes != sizeof(krr_nrc_config)) {
        std::fclose(f);
        return fail(KRR_ERR_INVALID_ARGUMENT, "krr_nrc_load: %s is not a cache checkpoint", path);
    }
    if (!same_structure(h.cfg, n->cfg) || h.n_params != n->mlp.n_params ||
        h.n_table_values != (int64_t)n->n_entries * 2) {
        std::fclose(f);
        return fail(KRR_ERR_INVALID_ARGUMENT,
                    "krr_nrc_load: the checkpoint's encoding or network shape differs from the cache's");
    }
    KRR_CUDA(cudaDeviceSynchronize());
    std::vector<float> buf;
    // the inference copy is read into the cache's own when both keep one
    float *arrays[8] = {n->w_master, n->w_m, n->w_v, n->table_master, n->table_m, n->table_v,
                        n->ema_w, n->ema_table};
    const int n_arrays = h.cfg.ema_decay > 0.f ? 8 : 6;
    for (int k = 0; k < n_arrays; ++k) {
        const size_t cnt = (size_t)(k < 3 || k == 6 ? h.n_params : h.n_table_values);
        buf.resize(cnt);
        if (std::fread(buf.data(), 4, cnt, f) != cnt) {
            std::fclose(f);
            return fail(KRR_ERR_INVALID_ARGUMENT, "krr_nrc_load: %s is truncated", path);
        }
        if (arrays[k]) KRR_CUDA(cudaMemcpy(arrays[k], buf.data(), cnt * 4, cudaMemcpyHostToDevice));
    }
    std::fclose(f);
    // training settings (learning rate, batch, stride, ...) and the scene box
    // the table was trained over come with the checkpoint; whether the cache
    // keeps an inference copy stays the cache's own setting
    const float own_decay = n->cfg.ema_decay;
    n->cfg = h.cfg;
    n->cfg.ema_decay = n->ema_w ? (h.cfg.ema_decay > 0.f ? h.cfg.ema_decay : own_decay) : 0.f;
    if (n->cfg.train_pixel_stride < 1) n->cfg.train_pixel_stride = 1;
    for (int a = 0; a < 3; ++a) {
        n->grid.lo[a] = h.cfg.scene_lo[a];
        const float e = h.cfg.scene_hi[a] - h.cfg.scene_lo[a];
        n->grid.inv_extent[a] = e > 0.f ? 1.f / e : 1.f;
    }
    unsigned char st[16];
    std::memcpy(st, &h.step, 8);
    std::memcpy(st + 8, h.bias_correction, 8);
    KRR_CUDA(cudaMemcpy(n->step, st, 16, cudaMemcpyHostToDevice));
    uint32_t w[2] = {0, h.diverged};
    KRR_CUDA(cudaMemcpy(n->err, w, sizeof(w), cudaMemcpyHostToDevice));
    KRR_CUDA(cudaMemset(n->w_grad, 0, (size_t)h.n_params * 4));
    KRR_CUDA(cudaMemset(n->table_grad, 0, (size_t)h.n_table_values * 4));
    k_to_bf16<<<grid_for(h.n_params), kThreads>>>(n->w_master, n->weights, h.n_params);
    k_to_bf16<<<grid_for(h.n_table_values), kThreads>>>(n->table_master, n->table, h.n_table_values);
    if (n->ema_w && h.cfg.ema_decay > 0.f) {
        k_to_bf16<<<grid_for(h.n_params), kThreads>>>(n->ema_w, n->ema_weights, h.n_params);
        k_to_bf16<<<grid_for(h.n_table_values), kThreads>>>(n->ema_table, n->ema_table_bf, h.n_table_values);
    } else {
        KRR_TRY(reset_ema(n, 0));
    }
    KRR_TRY(pack_weights(n, 0));
    KRR_CUDA(cudaDeviceSynchronize());
    return KRR_OK;
}

// Gradients of the last train step before Adam consumed them are not kept;
// this computes them for one batch without updating (loss-scaled units are
// removed): which = 0 MLP, 1 table.
extern "C" int krr_nrc_gradients(krr_nrc *n, const float *d_inputs, const float *d_targets,
                                 int64_t count, float *h_grad_mlp, float *h_grad_table,
                                 float *h_loss) {
    KRR_CHECK_ARG(n && d_inputs && d_targets && count > 0, "bad argument");
    cudaStream_t s = 0;
    KRR_TRY(forward(n, d_inputs, nullptr, count, s));
    // the training path, stopped before Adam
    float scale = n->cfg.loss_scale;
    KRR_CUDA(cudaMemset(n->w_grad, 0, n->mlp.n_params * 4));
    KRR_CUDA(cudaMemset(n->table_grad, 0, (size_t)n->n_entries * 2 * 4));
    KRR_TRY(backward(n, d_inputs, d_targets, nullptr, count, s));
    KRR_CUDA(cudaDeviceSynchronize());
    std::vector<float> tmp;
    if (h_grad_mlp) {
        KRR_CUDA(cudaMemcpy(h_grad_mlp, n->w_grad, n->mlp.n_params * 4, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n->mlp.n_params; ++i) h_grad_mlp[i] /= scale;
    }
    if (h_grad_table) {
        size_t tn = (size_t)n->n_entries * 2;
        KRR_CUDA(cudaMemcpy(h_grad_table, n->table_grad, tn * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < tn; ++i) h_grad_table[i] /= scale;
    }
    if (h_loss) KRR_CUDA(cudaMemcpy(h_loss, n->loss, 4, cudaMemcpyDeviceToHost));
    KRR_CUDA(cudaMemset(n->w_grad, 0, n->mlp.n_params * 4));
    KRR_CUDA(cudaMemset(n->table_grad, 0, (size_t)n->n_entries * 2 * 4));
    return KRR_OK;
}
