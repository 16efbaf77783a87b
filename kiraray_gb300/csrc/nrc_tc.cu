// Fused neural-radiance-cache forward pass on the 5th-generation tensor
// cores (tcgen05), two 128-row tiles of queries in flight per CTA.
//
// Per tile: four encoder warps encode the queries (hash grid, trilinear)
// into a 128x64 BF16 activation tile in shared memory while four MLP warps
// run the previous tile: for each of the six layers one elected thread
// issues four tcgen05.mma.kind::f16 (M=128, N=64 or 16, K=16, BF16 x BF16 ->
// FP32 in tensor memory), commits them to an mbarrier, and the 128 MLP
// threads read the accumulator rows back with tcgen05.ld, apply ReLU, round
// to BF16 and write the next activation tile (or the RGB output).  All
// weights (43 KB, BF16) stay resident in shared memory for the CTA's
// lifetime.  Waits on the mbarrier are bounded: a wait that gives up sets an
// error flag, and the CTA finishes without further tensor-core work and
// frees its tensor memory.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8x8-element core matrices of 128 contiguous bytes, core (i, j) of a tile
// with 64 columns at byte ((i * 8) + j) * 128, so the leading-dimension
// byte offset (next core along K) is 128 and the stride-dimension byte
// offset (next 8-row group) is 1024.
#include <algorithm>

#include "nrc.h"

namespace krr {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr uint32_t kTcCols = 64;                 // tensor-memory columns per CTA
constexpr int kLayerBytes = kNrcWidth * kNrcIn * 2;     // 8 KB
constexpr int kOutBytes = kNrcOutPad * kNrcIn * 2;      // 2 KB
constexpr uint32_t kWaitLimit = 1u << 26;

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading and
// stride byte offsets (all >> 4), descriptor version 1 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4
// at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ uint32_t mbar_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok;
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Byte offset of element (r, k) in a canonical K-major tile of 64 columns.
__host__ __device__ __forceinline__ uint32_t canon(uint32_t r, uint32_t k) {
    return (((r >> 3) * 8u + (k >> 3)) * 128u) + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Writes one row (64 values) of a canonical tile as eight 16-byte chunks.
__device__ __forceinline__ void store_row(uint8_t *tile, uint32_t r, const float *v) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        __nv_bfloat162 p0 = __floats2bfloat162_rn(v[8 * j + 0], v[8 * j + 1]);
        __nv_bfloat162 p1 = __floats2bfloat162_rn(v[8 * j + 2], v[8 * j + 3]);
        __nv_bfloat162 p2 = __floats2bfloat162_rn(v[8 * j + 4], v[8 * j + 5]);
        __nv_bfloat162 p3 = __floats2bfloat162_rn(v[8 * j + 6], v[8 * j + 7]);
        uint4 q;
        q.x = *reinterpret_cast<uint32_t *>(&p0);
        q.y = *reinterpret_cast<uint32_t *>(&p1);
        q.z = *reinterpret_cast<uint32_t *>(&p2);
        q.w = *reinterpret_cast<uint32_t *>(&p3);
        *reinterpret_cast<uint4 *>(tile + canon(r, 8 * j)) = q;
    }
}

// Packs the BF16 weights [layer][out][64] into canonical tiles.
__global__ void k_pack_weights(const __nv_bfloat16 *__restrict__ w, NrcMlp mlp, uint8_t *packed) {
    int total = mlp.n_params;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        int l = 0;
        while (l + 1 < mlp.layers && e >= mlp.w_offset[l + 1]) ++l;
        int local = e - mlp.w_offset[l];
        int r = local / kNrcIn, k = local % kNrcIn;
        *reinterpret_cast<__nv_bfloat16 *>(packed + (size_t)l * kLayerBytes + canon(r, k)) = w[e];
    }
}

// Hash-grid encoding of one query row.  The table gathers are the latency
// of the whole kernel, so the levels go in groups of four: the 32 corner
// loads of a group are issued before any of them is used (levels at or
// beyond g.levels load entry 0 and are discarded), which turns sixteen
// dependent round trips into four.  Per level the corner weights and the
// accumulation order are those of the CUDA-core encoder (nrc.cu).
constexpr int kEncGroup = 4;

__device__ __forceinline__ void encode_row(const NrcGrid &g, const float *q,
                                           const __nv_bfloat16 *__restrict__ table, float *x) {
    float p[3];
    for (int a = 0; a < 3; ++a) p[a] = fminf(fmaxf((q[a] - g.lo[a]) * g.inv_extent[a], 0.f), 1.f);
#pragma unroll 1
    for (int l0 = 0; l0 < kNrcMaxLevels; l0 += kEncGroup) {
        if (l0 >= g.levels) break;
        __nv_bfloat162 v[kEncGroup][8];
        float fr[kEncGroup][3];
#pragma unroll
        for (int j = 0; j < kEncGroup; ++j) {
            const int l = l0 + j;
            const bool valid = l < g.levels;
            uint32_t base[3];
            for (int a = 0; a < 3; ++a) {
                float s = p[a] * (float)g.res[l];
                float fl = fminf(fmaxf(floorf(s), 0.f), (float)(g.res[l] - 1));
                base[a] = (uint32_t)fl;
                fr[j][a] = fminf(fmaxf(s - fl, 0.f), 1.f);
            }
            uint32_t n1 = (uint32_t)g.res[l] + 1u;
            bool dense = g.dense_mask & (1u << l);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                uint32_t xx = base[0] + (k & 1), yy = base[1] + ((k >> 1) & 1), zz = base[2] + ((k >> 2) & 1);
                uint32_t idx = dense ? xx + n1 * (yy + n1 * zz)
                                     : (xx ^ (yy * 2654435761u) ^ (zz * 805459861u)) & (g.table_size - 1u);
                idx = valid ? idx + g.offset[l] : 0u;
                v[j][k] = *reinterpret_cast<const __nv_bfloat162 *>(table + 2 * (size_t)idx);
            }
        }
#pragma unroll
        for (int j = 0; j < kEncGroup; ++j) {
            if (l0 + j >= g.levels) break;
            float f0 = 0.f, f1 = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                float w = ((k & 1) ? fr[j][0] : 1.f - fr[j][0]) *
                          (((k >> 1) & 1) ? fr[j][1] : 1.f - fr[j][1]) *
                          (((k >> 2) & 1) ? fr[j][2] : 1.f - fr[j][2]);
                f0 += w * __bfloat162float(v[j][k].x);
                f1 += w * __bfloat162float(v[j][k].y);
            }
            x[2 * (l0 + j)] = f0;
            x[2 * (l0 + j) + 1] = f1;
        }
    }
    int o = 2 * g.levels;
    nrc_encode_extras(q, x + o);
    for (int k = o + kNrcExtra; k < kNrcIn; ++k) x[k] = 0.f;
}

__device__ __forceinline__ void bar_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Named barriers of the forward kernel (0 is __syncthreads): a tile buffer
// is full (encoders -> MLP warps), a tile buffer is free again (MLP warps
// -> encoders), and the MLP warps' own per-layer barrier.
constexpr int kBarFull = 1, kBarEmpty = 3, kBarMlp = 5;
constexpr int kFwThreads = 256;   // warps 0-3: MLP (tensor-memory lanes 0-127); 4-7: encoders

// out[i][0..3) for i < *count (or cap); optional per-layer activation dump
// (bf16 [layers][cap][64], row-major) for the training backward pass.
//
// Warp-specialised: warps 4-7 encode the rows of the CTA's next tile (the
// hash-grid gathers) into one of two activation buffers while warps 0-3 run
// the six layers of the current tile out of the other (one thread issues
// the MMAs, all 128 read the accumulator rows back, apply ReLU and write the
// next layer's input in place), so the gathers of tile k+1 overlap the MMA
// chain of tile k.  The groups hand the buffers over with named barriers;
// after a failed (bounded) accumulator wait the MLP warps skip the compute
// of the remaining tiles but keep handing buffers back, so no warp waits
// forever.
__global__ void __launch_bounds__(kFwThreads, 1)
k_nrc_forward_tc(NrcGrid g, int layers, const float *__restrict__ in, const int32_t *d_count,
                 int64_t cap, const __nv_bfloat16 *__restrict__ table,
                 const uint8_t *__restrict__ packed_w, float *__restrict__ out,
                 __nv_bfloat16 *__restrict__ acts, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sw = smem;                                              // weights
    uint8_t *sa0 = smem + (layers - 1) * kLayerBytes + kOutBytes;    // activation tiles
    sa0 = reinterpret_cast<uint8_t *>(((uintptr_t)sa0 + 1023) & ~(uintptr_t)1023);
    uint8_t *sa1 = sa0 + kTcRows * kNrcIn * 2;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sa1 + kTcRows * kNrcIn * 2);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
    uint32_t *fail_flag = tmem_slot + 1;
    const int tid = threadIdx.x, warp = tid >> 5;

    // weights -> shared memory (16-byte copies)
    int wbytes = (layers - 1) * kLayerBytes + kOutBytes;
    for (int e = tid; e < wbytes / 16; e += blockDim.x)
        reinterpret_cast<uint4 *>(sw)[e] = reinterpret_cast<const uint4 *>(packed_w)[e];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(smem_u32(mbar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    const int64_t n = d_count ? min((int64_t)*d_count, cap) : cap;
    const int64_t tiles = (n + kTcRows - 1) / kTcRows;
    if (warp >= 4) {
        // encoders: row r of each tile into the free buffer
        const int r = tid - 128;
        float x[kNrcIn];
        int k = 0;
        for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x, ++k) {
            uint8_t *sa = (k & 1) ? sa1 : sa0;
            if (k >= 2) bar_sync(kBarEmpty + (k & 1), kFwThreads);
            const int64_t row = t * kTcRows + r;
            if (row < n) encode_row(g, in + kNrcInputs * row, table, x);
            else
                for (int q = 0; q < kNrcIn; ++q) x[q] = 0.f;
            store_row(sa, (uint32_t)r, x);
            fence_proxy_async();   // the tensor cores read the tile through the async proxy
            bar_arrive(kBarFull + (k & 1), kFwThreads);
        }
    } else {
        const uint32_t my_lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        uint32_t phase = 0;
        bool failed = false;
        int k = 0;
        for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x, ++k) {
            uint8_t *sa = (k & 1) ? sa1 : sa0;
            bar_sync(kBarFull + (k & 1), kFwThreads);
            const int64_t row = t * kTcRows + tid;
            for (int l = 0; l < layers && !failed; ++l) {
                const bool last = l + 1 == layers;
                const int nrows = last ? kNrcOutPad : kNrcWidth;
                // the tile holds this layer's input X_l: dump it for the
                // backward pass while the MMAs read it (it is overwritten
                // only after the accumulator wait's barrier)
                if (acts) {
                    __nv_bfloat16 *dst = acts + (size_t)l * cap * kNrcIn;
                    for (int c = tid; c < kTcRows * 8; c += kTcRows) {
                        const int rr = c >> 3, j = c & 7;
                        if (t * kTcRows + rr < n)
                            reinterpret_cast<uint4 *>(dst + (t * kTcRows + rr) * kNrcIn)[j] =
                                *reinterpret_cast<const uint4 *>(sa + canon((uint32_t)rr, (uint32_t)(8 * j)));
                    }
                }
                if (tid == 0) {
                    fence_after_sync();
                    const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sw + l * kLayerBytes);
                    const uint32_t idesc = idesc_bf16(kTcRows, nrows);
#pragma unroll
                    for (int kk = 0; kk < kNrcIn / 16; ++kk)
                        tc_mma(tmem, smem_desc(a0 + 256u * kk, 128u, 1024u),
                               smem_desc(b0 + 256u * kk, 128u, 1024u), idesc, kk > 0 ? 1u : 0u);
                    tc_commit(smem_u32(mbar));
                    // bounded wait for the accumulator; the decision to stop
                    // is uniform across the MLP warps
                    uint32_t spins = 0, ok = 0;
                    while (!(ok = mbar_try_wait(smem_u32(mbar), phase)) && ++spins < kWaitLimit) {
                    }
                    *fail_flag = ok ? 0u : 1u;
                    if (!ok) atomicOr(err, (uint32_t)kErrLoopLimit);
                }
                bar_sync(kBarMlp, kTcRows);
                if (*fail_flag) {
                    failed = true;
                    break;
                }
                {
                    uint32_t spins = 0;   // already complete: returns at once
                    while (!mbar_try_wait(smem_u32(mbar), phase) && ++spins < kWaitLimit) {
                    }
                }
                phase ^= 1u;
                fence_after_sync();
                float v[kNrcIn];
                tmem_ld16(my_lane_addr + 0, v);
                if (!last) {
                    tmem_ld16(my_lane_addr + 16, v + 16);
                    tmem_ld16(my_lane_addr + 32, v + 32);
                    tmem_ld16(my_lane_addr + 48, v + 48);
                }
                tmem_wait_ld();
                if (!last) {
                    for (int q = 0; q < kNrcIn; ++q) v[q] = fmaxf(v[q], 0.f);
                    store_row(sa, (uint32_t)tid, v);
                    fence_proxy_async();
                } else if (row < n) {
                    out[row * kNrcOutPad + 0] = v[0];
                    out[row * kNrcOutPad + 1] = v[1];
                    out[row * kNrcOutPad + 2] = v[2];
                }
                fence_before_sync();
                bar_sync(kBarMlp, kTcRows);
            }
            bar_arrive(kBarEmpty + (k & 1), kFwThreads);   // the buffer is free
        }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
}

// ------------------------------------------------------------------ backward
//
// Per 128-row tile, from the output layer down: dX_l = dY_l . W_l (M=128,
// N=64, K=64 or 16) and dW_l += dY_l^T . X_l (M=128 with rows 64..127 of the
// A operand zero, N=64, K=128 rows of the tile).  The dX accumulator (64
// columns) is read back each layer, masked by ReLU'(X_l), rounded to BF16
// and becomes the next layer's dY tile (row-major and transposed copies);
// the dW_l accumulators (64 columns each) stay in tensor memory for all of
// the CTA's tiles and are added to the FP32 gradient once at the end.
// Operand rounding points match the CUDA-core kernels: dY, W and X in BF16,
// FP32 accumulation.

constexpr uint32_t kBwCols = 512;
constexpr int kT128Bytes = 128 * 128 * 2;   // [128][128] canonical tile, 32 KB
constexpr int kXtBytes = 64 * 128 * 2;      // [64][128], 16 KB
constexpr int kA64Bytes = 128 * 64 * 2;     // [128][64], 16 KB
constexpr int kA16Bytes = 128 * 16 * 2;     // [128][16], 4 KB
constexpr int kWtOutBytes = 64 * 16 * 2;    // W_out^T [64][16], 2 KB

// Byte offset of element (r, k) in a canonical K-major tile of `cols` columns.
__host__ __device__ __forceinline__ uint32_t canon_c(uint32_t r, uint32_t k, uint32_t cols) {
    return (((r >> 3) * (cols >> 3) + (k >> 3)) * 128u) + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Transposed weights: hidden layer l as W_l^T [64 in][64 out] at l * 8 KB,
// the output layer as W^T [64 in][16 out] after them.
__global__ void k_pack_weights_t(const __nv_bfloat16 *__restrict__ w, NrcMlp mlp, uint8_t *packed) {
    int total = mlp.n_params;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        int l = 0;
        while (l + 1 < mlp.layers && e >= mlp.w_offset[l + 1]) ++l;
        int local = e - mlp.w_offset[l];
        int r = local / kNrcIn, k = local % kNrcIn;   // W_l[r][k]
        size_t off = l + 1 < mlp.layers ? (size_t)l * kLayerBytes + canon_c(k, r, 64)
                                        : (size_t)l * kLayerBytes + canon_c(k, r, 16);
        *reinterpret_cast<__nv_bfloat16 *>(packed + off) = w[e];
    }
}

__device__ __forceinline__ void store_bf16(uint8_t *tile, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(tile + off) = __float2bfloat16_rn(v);
}

// Bounded wait on the CTA's mbarrier by thread 0, decision shared through
// shared memory; returns false (all threads) when the wait gave up.
__device__ __forceinline__ bool cta_wait(uint32_t mbar, uint32_t phase, uint32_t *fail_flag,
                                         uint32_t *err) {
    if (threadIdx.x == 0) {
        uint32_t spins = 0, ok = 0;
        while (!(ok = mbar_try_wait(mbar, phase)) && ++spins < kWaitLimit) {
        }
        *fail_flag = ok ? 0u : 1u;
        if (!ok) atomicOr(err, (uint32_t)kErrLoopLimit);
    }
    __syncthreads();
    if (*fail_flag) return false;
    uint32_t spins = 0;   // already complete: returns at once
    while (!mbar_try_wait(mbar, phase) && ++spins < kWaitLimit) {
    }
    return true;
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_nrc_backward_tc(int layers, const float *__restrict__ dy_out, const __nv_bfloat16 *__restrict__ acts,
                  const int32_t *d_count, int64_t cap, const uint8_t *__restrict__ packed_wt,
                  float *__restrict__ dx0, float *__restrict__ dw, NrcMlp mlp, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int wt_bytes = (layers - 1) * kLayerBytes + kWtOutBytes;
    uint8_t *swt = smem;
    uint8_t *at = smem + ((wt_bytes + 1023) & ~1023);   // dY_l^T, rows 64..127 zero
    uint8_t *at16 = at + kT128Bytes;                     // dY_out^T, rows 16..127 zero
    uint8_t *xt = at16 + kT128Bytes;                     // X_l^T
    uint8_t *a64 = xt + kXtBytes;                        // dY_l
    uint8_t *a16 = a64 + kA64Bytes;                      // dY_out
    uint64_t *mbar = reinterpret_cast<uint64_t *>(a16 + kA16Bytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
    uint32_t *fail_flag = tmem_slot + 1;
    const int tid = threadIdx.x, warp = tid >> 5;

    for (int e = tid; e < wt_bytes / 16; e += blockDim.x)
        reinterpret_cast<uint4 *>(swt)[e] = reinterpret_cast<const uint4 *>(packed_wt)[e];
    for (int e = tid; e < 2 * kT128Bytes / 16; e += blockDim.x)
        reinterpret_cast<uint4 *>(at)[e] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(kBwCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(smem_u32(mbar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t my_lanes = (uint32_t)(warp * 32) << 16;

    const int64_t n = d_count ? min((int64_t)*d_count, cap) : cap;
    const int64_t tiles = (n + kTcRows - 1) / kTcRows;
    uint32_t phase = 0;
    bool failed = false, any_tile = false;
    for (int64_t t = blockIdx.x; t < tiles && !failed; t += gridDim.x) {
        const int64_t row = t * kTcRows + tid;
        const bool live = row < n;
        // dY of the output layer: row-major [128][16] and transposed [16 of 128][128]
        {
            float d[kNrcOutPad];
            for (int c = 0; c < kNrcOutPad; ++c) d[c] = live ? dy_out[row * kNrcOutPad + c] : 0.f;
            for (int c = 0; c < kNrcOutPad; ++c) {
                store_bf16(a16, canon_c((uint32_t)tid, (uint32_t)c, 16), d[c]);
                store_bf16(at16, canon_c((uint32_t)c, (uint32_t)tid, 128), d[c]);
            }
        }
        for (int l = layers - 1; l >= 0 && !failed; --l) {
            const bool out_layer = l == layers - 1;
            // X_l^T and the ReLU mask of X_l
            uint64_t mask = 0;
            {
                const uint4 *src = reinterpret_cast<const uint4 *>(acts + ((size_t)l * cap + row) * kNrcIn);
                for (int j = 0; j < 8; ++j) {
                    uint4 q = live ? src[j] : make_uint4(0u, 0u, 0u, 0u);
                    const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
                    for (int i = 0; i < 8; ++i) {
                        const int k = 8 * j + i;
                        *reinterpret_cast<__nv_bfloat16 *>(xt + canon_c((uint32_t)k, (uint32_t)tid, 128)) = h[i];
                        if (__bfloat162float(h[i]) > 0.f) mask |= 1ull << k;
                    }
                }
            }
            fence_proxy_async();
            fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                fence_after_sync();
                // dW_l += dY_l^T . X_l   (K = the tile's 128 rows)
                const uint32_t a0 = smem_u32(out_layer ? at16 : at), b0 = smem_u32(xt);
                const uint32_t dcol = tmem + 64u + 64u * (uint32_t)l;
                const uint32_t idw = idesc_bf16(kTcRows, 64);
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    tc_mma(dcol, smem_desc(a0 + 256u * kk, 128u, 2048u), smem_desc(b0 + 256u * kk, 128u, 2048u),
                           idw, (any_tile || kk > 0) ? 1u : 0u);
                // dX = dY_l . W_l  (K = 16 for the output layer, 64 otherwise)
                const uint32_t wt = smem_u32(swt + l * kLayerBytes);
                if (out_layer) {
                    tc_mma(tmem, smem_desc(smem_u32(a16), 128u, 256u), smem_desc(wt, 128u, 256u),
                           idesc_bf16(kTcRows, 64), 0u);
                } else {
                    const uint32_t a1 = smem_u32(a64);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        tc_mma(tmem, smem_desc(a1 + 256u * kk, 128u, 1024u), smem_desc(wt + 256u * kk, 128u, 1024u),
                               idesc_bf16(kTcRows, 64), kk > 0 ? 1u : 0u);
                }
                tc_commit(smem_u32(mbar));
            }
            if (!cta_wait(smem_u32(mbar), phase, fail_flag, err)) {
                failed = true;
                break;
            }
            phase ^= 1u;
            fence_after_sync();
            float v[kNrcIn];
            tmem_ld16(tmem + my_lanes + 0, v);
            tmem_ld16(tmem + my_lanes + 16, v + 16);
            tmem_ld16(tmem + my_lanes + 32, v + 32);
            tmem_ld16(tmem + my_lanes + 48, v + 48);
            tmem_wait_ld();
            if (l > 0) {
                for (int k = 0; k < kNrcIn; ++k) {
                    const float d = ((mask >> k) & 1ull) ? v[k] : 0.f;
                    v[k] = d;
                    store_bf16(at, canon_c((uint32_t)k, (uint32_t)tid, 128), d);
                }
                store_row(a64, (uint32_t)tid, v);
                fence_proxy_async();
            } else if (live) {
                float4 *dst = reinterpret_cast<float4 *>(dx0 + row * kNrcIn);
                for (int k = 0; k < kNrcIn / 4; ++k)
                    dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            }
            fence_before_sync();
            __syncthreads();
        }
        any_tile = true;
    }
    // dW accumulators: rows 0..63 (out features) live in the lanes of warps 0-1
    if (!failed && any_tile && warp < 2) {
        fence_after_sync();
        const int m = tid;   // out-feature row of dW_l
        for (int l = 0; l < layers; ++l) {
            const int rows = l + 1 == layers ? kNrcOutPad : kNrcWidth;
            float v[kNrcIn];
            const uint32_t base = tmem + my_lanes + 64u + 64u * (uint32_t)l;
            tmem_ld16(base + 0, v);
            tmem_ld16(base + 16, v + 16);
            tmem_ld16(base + 32, v + 32);
            tmem_ld16(base + 48, v + 48);
            tmem_wait_ld();
            if (m < rows) {   // 16-byte vector atomics (the row offsets are multiples of 64 floats)
                float4 *dst = reinterpret_cast<float4 *>(dw + mlp.w_offset[l] + (size_t)m * kNrcIn);
                for (int k = 0; k < kNrcIn / 4; ++k)
                    atomicAdd(dst + k, make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBwCols));
}

}  // namespace

// Resident CTAs per SM of a tensor-memory kernel, from its registers, its
// shared memory (carveout at the maximum) and its tensor-memory columns.
// (The occupancy query does not count tensor memory and reported one CTA
// for this kernel, the carveout preference not yet applied.)
static int tc_ctas_per_sm(const void *fn, int threads, size_t smem, int dev) {
    cudaFuncAttributes fa{};
    int regs_sm = 0, smem_sm = 0, smem_reserved = 0, threads_sm = 0;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    const int by_regs = regs_sm / std::max(1, threads * std::max(1, fa.numRegs));
    const int by_smem = smem_sm / (int)std::max<size_t>(1, smem + fa.sharedSizeBytes + smem_reserved);
    const int by_threads = threads_sm / threads;
    const int by_tmem = 512 / (int)kTcCols;
    return std::max(1, std::min(std::min(by_regs, by_smem), std::min(by_threads, by_tmem)));
}

size_t nrc_tc_smem_bytes(int layers) {
    size_t w = (size_t)(layers - 1) * kLayerBytes + kOutBytes;
    size_t a = ((w + 1023) & ~(size_t)1023) + 2 * kTcRows * kNrcIn * 2;   // two tile buffers
    return a + 64 + 1024;   // mbarrier, tensor-memory slot, alignment slack
}

int nrc_pack_weights(const __nv_bfloat16 *w, const NrcMlp &mlp, uint8_t *packed, cudaStream_t s) {
    cudaMemsetAsync(packed, 0, (size_t)(mlp.layers - 1) * kLayerBytes + kOutBytes, s);
    k_pack_weights<<<64, 256, 0, s>>>(w, mlp, packed);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

size_t nrc_tc_bwd_smem_bytes(int layers) {
    size_t w = (size_t)(layers - 1) * kLayerBytes + kWtOutBytes;
    return ((w + 1023) & ~(size_t)1023) + 2 * kT128Bytes + kXtBytes + kA64Bytes + kA16Bytes + 64 + 1024;
}

int nrc_pack_weights_t(const __nv_bfloat16 *w, const NrcMlp &mlp, uint8_t *packed, cudaStream_t s) {
    cudaMemsetAsync(packed, 0, (size_t)(mlp.layers - 1) * kLayerBytes + kWtOutBytes, s);
    k_pack_weights_t<<<64, 256, 0, s>>>(w, mlp, packed);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

int nrc_backward_tc(const NrcMlp &mlp, const float *d_dy_out, const __nv_bfloat16 *acts,
                    const int32_t *d_count, int64_t cap, const uint8_t *packed_wt, float *d_dx0,
                    float *d_dw, uint32_t *err, cudaStream_t s) {
    static bool configured = false;
    size_t smem = nrc_tc_bwd_smem_bytes(mlp.layers);
    if (!configured) {
        KRR_CUDA(cudaFuncSetAttribute(k_nrc_backward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        configured = true;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t tiles = (cap + kTcRows - 1) / kTcRows;
    int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sms));
    k_nrc_backward_tc<<<grid, kTcThreads, smem, s>>>(mlp.layers, d_dy_out, acts, d_count, cap, packed_wt,
                                                     d_dx0, d_dw, mlp, err);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

int nrc_forward_tc(const NrcGrid &g, const NrcMlp &mlp, const float *d_in, const int32_t *d_count,
                   int64_t cap, const __nv_bfloat16 *table, const uint8_t *packed, float *d_out,
                   __nv_bfloat16 *acts, uint32_t *err, cudaStream_t s) {
    static bool configured = false;
    size_t smem = nrc_tc_smem_bytes(mlp.layers);
    if (!configured) {
        KRR_CUDA(cudaFuncSetAttribute(k_nrc_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        // the largest shared-memory carveout, so that several CTAs fit
        KRR_CUDA(cudaFuncSetAttribute(k_nrc_forward_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      cudaSharedmemCarveoutMaxShared));
        configured = true;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // several CTAs per SM, so that the hash gathers of one CTA's tile overlap
    // the MMA chains of the others: as many as registers, shared memory and
    // the 512 tensor-memory columns allow (3 for five hidden layers)
    static int per_sm = 0;
    if (!per_sm) per_sm = tc_ctas_per_sm((const void *)k_nrc_forward_tc, kFwThreads, smem, dev);
    int64_t tiles = (cap + kTcRows - 1) / kTcRows;
    int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sms * per_sm));
    k_nrc_forward_tc<<<grid, kFwThreads, smem, s>>>(g, mlp.layers, d_in, d_count, cap, table, packed,
                                                    d_out, acts, err);
    KRR_CUDA(cudaGetLastError());
    return KRR_OK;
}

}  // namespace krr
