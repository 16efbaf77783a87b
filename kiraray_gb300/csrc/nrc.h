// Neural radiance cache: device layout shared by nrc.cu and the wavefront
// integration (wavefront.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace krr {

constexpr int kNrcMaxLevels = 16;
constexpr int kNrcIn = 64;       // padded MLP input width
constexpr int kNrcWidth = 64;    // hidden width
constexpr int kNrcOutPad = 16;   // padded output rows (3 used)
constexpr int kNrcInputs = 13;   // query record: position 3, normal 3, roughness 1, albedo 3,
                                 // outgoing direction 3

// Inputs after the hash-grid features (the encoding of neural radiance
// caching, Mueller et al. 2021): normal and outgoing direction as spherical
// angles, and roughness as 1 - exp(-r), each in a one-blob encoding of 4
// bins (Gaussian bumps of width 1/4 centred at (i + 0.5)/4); albedo as is.
constexpr int kNrcBlobBins = 4;
constexpr int kNrcExtra = 5 * kNrcBlobBins + 3;

__host__ __device__ inline void nrc_one_blob(float s, float *x) {
    for (int i = 0; i < kNrcBlobBins; ++i) {
        float d = (s - ((float)i + 0.5f) / (float)kNrcBlobBins) * (float)kNrcBlobBins;
        x[i] = expf(-0.5f * d * d);
    }
}

__host__ __device__ inline void nrc_spherical(float x, float y, float z, float &theta, float &phi) {
    theta = acosf(fminf(fmaxf(z, -1.f), 1.f)) * 0.318309886183790672f;        // / pi
    phi = atan2f(y, x) * 0.159154943091895336f + 0.5f;                          // / (2 pi) + 1/2
}

// q: query record (position 3, normal 3, roughness 1, albedo 3, wo 3);
// writes kNrcExtra values.
__host__ __device__ inline void nrc_encode_extras(const float *q, float *x) {
    float t, p;
    nrc_spherical(q[3], q[4], q[5], t, p);
    nrc_one_blob(t, x);
    nrc_one_blob(p, x + kNrcBlobBins);
    nrc_spherical(q[10], q[11], q[12], t, p);
    nrc_one_blob(t, x + 2 * kNrcBlobBins);
    nrc_one_blob(p, x + 3 * kNrcBlobBins);
    nrc_one_blob(1.f - expf(-q[6]), x + 4 * kNrcBlobBins);
    x[5 * kNrcBlobBins + 0] = q[7];
    x[5 * kNrcBlobBins + 1] = q[8];
    x[5 * kNrcBlobBins + 2] = q[9];
}

// Hash-grid description passed by value to kernels.
struct NrcGrid {
    int32_t levels, features;         // features per level (2)
    uint32_t table_size;              // entries per hashed level (power of two)
    uint32_t dense_mask;              // bit l set: level l is indexed densely
    int32_t res[kNrcMaxLevels];       // cells per axis
    uint32_t offset[kNrcMaxLevels];   // first entry of each level
    uint32_t size[kNrcMaxLevels];     // entries of each level
    float lo[3], inv_extent[3];       // scene box -> [0,1]^3
};

// One MLP: layer l maps rows_in[l] -> rows_out[l]; weights row-major
// [out][in] at w_offset[l].
struct NrcMlp {
    int32_t layers;                   // hidden layers + output layer
    int32_t w_offset[8];
    int32_t n_params;
};

}  // namespace krr

struct krr_nrc;

namespace krr {
// Device views used by the wavefront hooks.
struct NrcView {
    NrcGrid grid;
    NrcMlp mlp;
    const __nv_bfloat16 *table;       // bf16 features, [entries][features]
    const __nv_bfloat16 *weights;     // bf16 weights
};
NrcView nrc_view(const krr_nrc *n);
int nrc_query_device(krr_nrc *n, const float *d_inputs, const int32_t *d_count, int64_t capacity,
                     float *d_out, cudaStream_t s);
int nrc_train_device(krr_nrc *n, const float *d_inputs, const float *d_targets,
                     const int32_t *d_count, int64_t capacity, cudaStream_t s);
int64_t nrc_batch_size(const krr_nrc *n);
// tcgen05 forward (nrc_tc.cu)
size_t nrc_tc_smem_bytes(int layers);
int nrc_pack_weights(const __nv_bfloat16 *w, const NrcMlp &mlp, uint8_t *packed, cudaStream_t s);
// tcgen05 backward (nrc_tc.cu): transposed weight tiles, then dX0 and dW.
size_t nrc_tc_bwd_smem_bytes(int layers);
int nrc_pack_weights_t(const __nv_bfloat16 *w, const NrcMlp &mlp, uint8_t *packed, cudaStream_t s);
int nrc_backward_tc(const NrcMlp &mlp, const float *d_dy_out, const __nv_bfloat16 *acts,
                    const int32_t *d_count, int64_t cap, const uint8_t *packed_wt, float *d_dx0,
                    float *d_dw, uint32_t *err, cudaStream_t s);
int nrc_forward_tc(const NrcGrid &g, const NrcMlp &mlp, const float *d_in, const int32_t *d_count,
                   int64_t cap, const __nv_bfloat16 *table, const uint8_t *packed, float *d_out,
                   __nv_bfloat16 *acts, uint32_t *err, cudaStream_t s);
int32_t nrc_train_stride(const krr_nrc *n);
// Device word that is non-zero once a training step's loss was not finite:
// the cache has diverged, takes no further Adam steps, and the pass runs the
// plain tracer (no path stops at it) until new parameters are loaded.
const uint32_t *nrc_diverged_flag(const krr_nrc *n);
// Device error flags of the cache's kernels (bounded tensor-core waits).
uint32_t *nrc_error_flags(krr_nrc *n);
float nrc_termination_spread(const krr_nrc *n);
constexpr int kNrcRecFloats = 20;   // training vertex: record 13 | throughput 3 | L 3 | pad
}  // namespace krr
