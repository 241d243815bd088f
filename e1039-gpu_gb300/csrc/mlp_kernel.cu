// mlp_kernel.cu -- the learned tracklet scorer: a 16-64-64-1 MLP with BF16
// weights and activations, FP32 accumulation and a sigmoid output.
//
//   mlp_score_kernel   inference on the 5th-generation tensor cores: tiles
//                      of 128 tracklets; tcgen05.mma (kind::f16, BF16 x BF16
//                      -> FP32 in tensor memory) for both hidden layers,
//                      operands in shared memory in the no-swizzle K-major
//                      core-matrix layout, completion through an mbarrier,
//                      accumulators read back with tcgen05.ld; bias, ReLU
//                      and the 64 -> 1 output layer on the CUDA cores.
//   mlp_train_kernel   one mini-batch: forward and backward on the CUDA
//                      cores with the same rounding points (input and first
//                      hidden layer rounded to BF16, weights BF16, FP32
//                      sums), weighted binary cross-entropy; per-block
//                      partial gradients (no atomics: the Adam kernel sums
//                      them in block order, so training is deterministic).
//   mlp_adam_kernel    Adam on the FP32 master parameters, then the BF16
//                      copies the forward passes read.
#include <cuda_bf16.h>

#include "../../include/or_gb300.h"
#include "or_device.cuh"

namespace orgpu {

constexpr int MLP_IN = OR_NFEAT, MLP_H = OR_MLP_H;
constexpr uint32_t MLP_WAIT_LIMIT = 1u << 22;  // bounded mbarrier polls per wait

__device__ __forceinline__ float bf16_bits_to_float(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }
__device__ __forceinline__ uint16_t float_to_bf16_bits(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ float round_bf16(float f) { return bf16_bits_to_float(float_to_bf16_bits(f)); }

// ---------------------------------------------------------------------------
// tcgen05 helpers
// ---------------------------------------------------------------------------
// byte offset of element (row, k) of a K-major operand with K columns in the
// no-swizzle core-matrix layout: 8 rows x 16 bytes per core matrix, core
// matrices along K adjacent (128 B apart), row groups K/8 core matrices apart
__device__ __forceinline__ uint32_t cm_offset(int row, int k, int K) {
    return (uint32_t)(((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
// shared-memory matrix descriptor (no swizzle): start, leading-dimension
// (K direction) and stride-dimension (row-group) byte offsets, version 1
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

constexpr int MS_ROWS = 128;       // tracklets per tile = MMA M
constexpr int MS_TMEM_COLS = 128;  // D1 in columns 0-63, D2 in 64-127

struct __align__(1024) MlpSmem {
    uint8_t a1[MS_ROWS * MLP_IN * 2];  // x tile, K = 16
    uint8_t a2[MS_ROWS * MLP_H * 2];   // h1 tile, K = 64
    uint8_t b1[MLP_H * MLP_IN * 2];    // W1 [64][16]
    uint8_t b2[MLP_H * MLP_H * 2];     // W2 [64][64]
    float mean[MLP_IN], inv_std[MLP_IN], bias1[MLP_H], bias2[MLP_H], w3[MLP_H];
    float b3;
    uint32_t tmem_base;
    uint64_t bar;
};

__global__ void __launch_bounds__(MS_ROWS)
    mlp_score_kernel(const or_mlp_t *__restrict__ model, const float *__restrict__ feat, long max_rows,
                     const int32_t *__restrict__ n_rows_dev, float *__restrict__ score, uint32_t *__restrict__ errw) {
    // rows to score: max_rows, or fewer when the count is on the device
    const long n_rows = n_rows_dev ? min(max_rows, (long)*n_rows_dev) : max_rows;
    extern __shared__ __align__(1024) uint8_t ms_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(ms_raw);
    const int t = threadIdx.x, w = t >> 5;
    // weights into the B operand layouts, small vectors as floats
    for (int i = t; i < MLP_H * MLP_IN; i += MS_ROWS)
        *reinterpret_cast<uint16_t *>(S.b1 + cm_offset(i / MLP_IN, i % MLP_IN, MLP_IN)) = model->w1[i];
    for (int i = t; i < MLP_H * MLP_H; i += MS_ROWS)
        *reinterpret_cast<uint16_t *>(S.b2 + cm_offset(i / MLP_H, i % MLP_H, MLP_H)) = model->w2[i];
    if (t < MLP_IN) {
        S.mean[t] = model->mean[t];
        S.inv_std[t] = model->inv_std[t];
    }
    if (t < MLP_H) {
        S.bias1[t] = model->b1[t];
        S.bias2[t] = model->b2[t];
        S.w3[t] = model->w3[t];
    }
    if (t == 0) {
        S.b3 = model->b3;
        mbar_init(&S.bar, 1);
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(MS_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_proxy_async_smem();  // weights written by threads, read by the tensor core
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = (uint32_t)(32 * w) << 16;  // this warp's quarter of the 128 lanes
    const uint32_t sa1 = smem_u32(S.a1), sa2 = smem_u32(S.a2), sb1 = smem_u32(S.b1), sb2 = smem_u32(S.b2);
    const uint32_t id = idesc_bf16_f32(MS_ROWS, MLP_H);
    uint32_t phase = 0;
    bool timed_out = false;

    const long ntiles = (n_rows + MS_ROWS - 1) / MS_ROWS;
    for (long tile = blockIdx.x; tile < ntiles && !timed_out; tile += gridDim.x) {
        const long row = tile * MS_ROWS + t;
        // ---- x row -> A1 (normalised, BF16) ----------------------------------
        {
            float x[MLP_IN];
            if (row < n_rows) {
                const float4 *src = reinterpret_cast<const float4 *>(feat + row * MLP_IN);
#pragma unroll
                for (int q = 0; q < MLP_IN / 4; ++q) {
                    const float4 v = src[q];
                    x[4 * q] = v.x;
                    x[4 * q + 1] = v.y;
                    x[4 * q + 2] = v.z;
                    x[4 * q + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < MLP_IN; ++k) x[k] = S.mean[k];
            }
            uint32_t pk[MLP_IN / 2];
#pragma unroll
            for (int k = 0; k < MLP_IN; k += 2) {
                const uint16_t lo = float_to_bf16_bits((x[k] - S.mean[k]) * S.inv_std[k]);
                const uint16_t hi = float_to_bf16_bits((x[k + 1] - S.mean[k + 1]) * S.inv_std[k + 1]);
                pk[k / 2] = (uint32_t)lo | ((uint32_t)hi << 16);
            }
            *reinterpret_cast<uint4 *>(S.a1 + cm_offset(t, 0, MLP_IN)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            *reinterpret_cast<uint4 *>(S.a1 + cm_offset(t, 8, MLP_IN)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            umma_bf16(tmem, umma_desc(sa1, 128, 256), umma_desc(sb1, 128, 256), id, 0u);
            umma_commit(&S.bar);
        }
        bool ok = mbar_wait_bounded(&S.bar, phase, MLP_WAIT_LIMIT);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        tc_fence_after();
        // ---- D1 -> h1 = bf16(relu(D1 + b1)) -> A2 --------------------------
        {
            float d[MLP_H];
#pragma unroll
            for (int c = 0; c < MLP_H; c += 16) tmem_ld16(tmem + lane_base + (uint32_t)c, d + c);
            tmem_ld_wait();
#pragma unroll
            for (int c = 0; c < MLP_H; c += 8) {
                uint32_t pk[4];
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                    const uint16_t lo = float_to_bf16_bits(fmaxf(d[c + j] + S.bias1[c + j], 0.f));
                    const uint16_t hi = float_to_bf16_bits(fmaxf(d[c + j + 1] + S.bias1[c + j + 1], 0.f));
                    pk[j / 2] = (uint32_t)lo | ((uint32_t)hi << 16);
                }
                *reinterpret_cast<uint4 *>(S.a2 + cm_offset(t, c, MLP_H)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < MLP_H / 16; ++s)
                umma_bf16(tmem + MLP_H, umma_desc(sa2 + 256u * s, 128, 1024), umma_desc(sb2 + 256u * s, 128, 1024),
                          id, s > 0 ? 1u : 0u);
            umma_commit(&S.bar);
        }
        ok = mbar_wait_bounded(&S.bar, phase, MLP_WAIT_LIMIT);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        tc_fence_after();
        // ---- D2 -> h2 = relu(D2 + b2); z = w3 . h2 + b3; sigmoid -------------
        {
            float d[MLP_H];
#pragma unroll
            for (int c = 0; c < MLP_H; c += 16) tmem_ld16(tmem + lane_base + (uint32_t)(MLP_H + c), d + c);
            tmem_ld_wait();
            float z = S.b3;
#pragma unroll
            for (int j = 0; j < MLP_H; ++j) z += S.w3[j] * fmaxf(d[j] + S.bias2[j], 0.f);
            if (row < n_rows) score[row] = 1.f / (1.f + expf(-z));
        }
        tc_fence_before();
        __syncthreads();  // TMEM reads of this tile done before the next tile's MMAs
    }
    if (timed_out) {
        if (t == 0) atomicOr(errw, ERRW_TMA_TIMEOUT);
        // let the MMA in flight finish (bounded) before the columns are freed
        mbar_wait_bounded(&S.bar, phase ^ 1u, MLP_WAIT_LIMIT);
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(MS_TMEM_COLS)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// training
// ---------------------------------------------------------------------------
constexpr int TR_ROWS = 128;  // samples per block
constexpr int TR_LD = MLP_H + 1;

// parameter offsets in the FP32 vector
constexpr int P_W1 = 0, P_B1 = P_W1 + MLP_H * MLP_IN, P_W2 = P_B1 + MLP_H, P_B2 = P_W2 + MLP_H * MLP_H,
              P_W3 = P_B2 + MLP_H, P_B3 = P_W3 + MLP_H, P_N = P_B3 + 1;
static_assert(P_N == OR_MLP_NPARAM, "parameter vector layout");

struct TrainSmem {
    float w1[MLP_H * MLP_IN], w2[MLP_H * MLP_H], b1[MLP_H], b2[MLP_H], w3[MLP_H];
    float mean[MLP_IN], inv_std[MLP_IN];
    float b3;
    float x[TR_ROWS][MLP_IN + 1];
    float h1[TR_ROWS][TR_LD], dh1[TR_ROWS][TR_LD], dh2[TR_ROWS][TR_LD], h2dz[TR_ROWS][TR_LD];
    float dz[TR_ROWS];
    float loss[TR_ROWS];
};

__device__ __forceinline__ float softplus(float a) { return fmaxf(a, 0.f) + log1pf(expf(-fabsf(a))); }

// Forward (and backward when grad_part != nullptr) of the samples
// idx[blockIdx.x*128 ...] of one batch of `batch` samples.  Loss: mean over
// the batch of pos_weight*y*softplus(-z) + (1-y)*softplus(z).  prob
// (optional) receives the sigmoid output per batch position.
__global__ void __launch_bounds__(TR_ROWS)
    mlp_train_kernel(const or_mlp_t *__restrict__ model, const float *__restrict__ feat,
                     const uint8_t *__restrict__ label, const int64_t *__restrict__ idx, int batch, float pos_weight,
                     float *__restrict__ grad_part, float *__restrict__ loss_part, float *__restrict__ prob) {
    extern __shared__ __align__(16) uint8_t tr_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(tr_raw);
    const int t = threadIdx.x;
    for (int i = t; i < MLP_H * MLP_IN; i += TR_ROWS) S.w1[i] = bf16_bits_to_float(model->w1[i]);
    for (int i = t; i < MLP_H * MLP_H; i += TR_ROWS) S.w2[i] = bf16_bits_to_float(model->w2[i]);
    if (t < MLP_H) {
        S.b1[t] = model->b1[t];
        S.b2[t] = model->b2[t];
        S.w3[t] = model->w3[t];
    }
    if (t < MLP_IN) {
        S.mean[t] = model->mean[t];
        S.inv_std[t] = model->inv_std[t];
    }
    if (t == 0) S.b3 = model->b3;
    __syncthreads();
    const int pos = blockIdx.x * TR_ROWS + t;
    const bool valid = pos < batch;
    const long r = valid ? idx[pos] : 0;
    float x[MLP_IN], a1[MLP_H], h1[MLP_H], a2[MLP_H];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) x[k] = round_bf16((feat[r * MLP_IN + k] - S.mean[k]) * S.inv_std[k]);
    for (int j = 0; j < MLP_H; ++j) {
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < MLP_IN; ++k) sum += S.w1[j * MLP_IN + k] * x[k];
        a1[j] = sum + S.b1[j];
        h1[j] = round_bf16(fmaxf(a1[j], 0.f));
    }
    float z = S.b3;
    for (int j = 0; j < MLP_H; ++j) {
        float sum = 0.f;
        for (int k = 0; k < MLP_H; ++k) sum += S.w2[j * MLP_H + k] * h1[k];
        a2[j] = sum + S.b2[j];
        z += S.w3[j] * fmaxf(a2[j], 0.f);
    }
    const float p = 1.f / (1.f + expf(-z));
    if (prob && valid) prob[pos] = p;
    if (!grad_part) return;
    const float y = valid ? (float)label[r] : 0.f;
    const float inv_b = 1.f / (float)batch;
    const float dz = valid ? (p * (pos_weight * y + 1.f - y) - pos_weight * y) * inv_b : 0.f;
    S.loss[t] = valid ? (pos_weight * y * softplus(-z) + (1.f - y) * softplus(z)) * inv_b : 0.f;
    S.dz[t] = dz;
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) S.x[t][k] = valid ? x[k] : 0.f;
    for (int j = 0; j < MLP_H; ++j) {
        const float g2 = a2[j] > 0.f ? dz * S.w3[j] : 0.f;
        S.dh2[t][j] = g2;
        S.h2dz[t][j] = dz * fmaxf(a2[j], 0.f);
        S.h1[t][j] = h1[j];
    }
    for (int k = 0; k < MLP_H; ++k) {
        float sum = 0.f;
        if (a1[k] > 0.f)
            for (int j = 0; j < MLP_H; ++j) sum += S.w2[j * MLP_H + k] * S.dh2[t][j];
        S.dh1[t][k] = sum;
    }
    __syncthreads();
    float *gp = grad_part + (long)blockIdx.x * P_N;
    for (int q = t; q < P_N; q += TR_ROWS) {
        float g = 0.f;
        if (q < P_B1) {
            const int j = q / MLP_IN, k = q % MLP_IN;
            for (int i = 0; i < TR_ROWS; ++i) g += S.dh1[i][j] * S.x[i][k];
        } else if (q < P_W2) {
            const int j = q - P_B1;
            for (int i = 0; i < TR_ROWS; ++i) g += S.dh1[i][j];
        } else if (q < P_B2) {
            const int j = (q - P_W2) / MLP_H, k = (q - P_W2) % MLP_H;
            for (int i = 0; i < TR_ROWS; ++i) g += S.dh2[i][j] * S.h1[i][k];
        } else if (q < P_W3) {
            const int j = q - P_B2;
            for (int i = 0; i < TR_ROWS; ++i) g += S.dh2[i][j];
        } else if (q < P_B3) {
            const int j = q - P_W3;
            for (int i = 0; i < TR_ROWS; ++i) g += S.h2dz[i][j];
        } else {
            for (int i = 0; i < TR_ROWS; ++i) g += S.dz[i];
        }
        gp[q] = g;
    }
    if (t == 0) {
        float l = 0.f;
        for (int i = 0; i < TR_ROWS; ++i) l += S.loss[i];
        loss_part[blockIdx.x] = l;
    }
}

// Adam on the FP32 parameters (gradient = sum of the blocks' partials, in
// block order), then the model copy the forward passes read.
__global__ void mlp_adam_kernel(float *__restrict__ param, float *__restrict__ m1, float *__restrict__ m2,
                                const float *__restrict__ grad_part, int nblocks, int step, float lr, float beta1,
                                float beta2, float eps, or_mlp_t *__restrict__ model) {
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < P_N; q += gridDim.x * blockDim.x) {
        float g = 0.f;
        for (int b = 0; b < nblocks; ++b) g += grad_part[(long)b * P_N + q];
        const float a = beta1 * m1[q] + (1.f - beta1) * g;
        const float v = beta2 * m2[q] + (1.f - beta2) * g * g;
        m1[q] = a;
        m2[q] = v;
        const float w = param[q] - lr * (a / c1) / (sqrtf(v / c2) + eps);
        param[q] = w;
        if (q < P_B1) model->w1[q - P_W1] = float_to_bf16_bits(w);
        else if (q < P_W2) model->b1[q - P_B1] = w;
        else if (q < P_B2) model->w2[q - P_W2] = float_to_bf16_bits(w);
        else if (q < P_W3) model->b2[q - P_B2] = w;
        else if (q < P_B3) model->w3[q - P_W3] = w;
        else model->b3 = w;
    }
}

size_t mlp_score_smem() { return sizeof(MlpSmem) + 1024; }
size_t mlp_train_smem() { return sizeof(TrainSmem); }

cudaError_t launch_mlp_score(const or_mlp_t *model, const float *feat, long n_rows, const int32_t *n_rows_dev,
                             float *score, uint32_t *errw, cudaStream_t stream, int sm_count) {
    if (n_rows <= 0) return cudaSuccess;
    const size_t smem = mlp_score_smem();
    cudaError_t err = smem_attr_once((const void *)mlp_score_kernel, (int)smem);
    if (err != cudaSuccess) return err;
    const long ntiles = (n_rows + MS_ROWS - 1) / MS_ROWS;
    long blocks = ntiles;
    const long cap = (long)sm_count * 4;  // 4 x 128 TMEM columns fill an SM's 512
    if (blocks > cap) blocks = cap;
    mlp_score_kernel<<<(unsigned)blocks, MS_ROWS, smem, stream>>>(model, feat, n_rows, n_rows_dev, score, errw);
    return cudaGetLastError();
}

int mlp_train_blocks(int batch) { return (batch + TR_ROWS - 1) / TR_ROWS; }

cudaError_t launch_mlp_train(const or_mlp_t *model, const float *feat, const uint8_t *label, const int64_t *idx,
                             int batch, float pos_weight, float *grad_part, float *loss_part, float *prob,
                             cudaStream_t stream) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = mlp_train_smem();
    cudaError_t err = smem_attr_once((const void *)mlp_train_kernel, (int)smem);
    if (err != cudaSuccess) return err;
    mlp_train_kernel<<<(unsigned)mlp_train_blocks(batch), TR_ROWS, smem, stream>>>(model, feat, label, idx, batch,
                                                                                  pos_weight, grad_part, loss_part,
                                                                                  prob);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *param, float *m1, float *m2, const float *grad_part, int nblocks, int step,
                            float lr, float beta1, float beta2, float eps, or_mlp_t *model, cudaStream_t stream) {
    mlp_adam_kernel<<<(P_N + 255) / 256, 256, 0, stream>>>(param, m1, m2, grad_part, nblocks, step, lr, beta1, beta2,
                                                          eps, model);
    return cudaGetLastError();
}

}  // namespace orgpu
