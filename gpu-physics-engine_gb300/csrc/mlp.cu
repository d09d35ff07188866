// mlp.cu — the warm-start network: parameters, pair set, training on the tensor cores, inference entry.
//
// Training step (one launch per minibatch, then one AdamW launch). Each CTA (128 threads, one per SM) takes
// tiles of 128 pairs; thread r owns pair r of the tile. Per tile, on the tensor cores (tcgen05.mma, M = 128,
// BF16 operands in shared memory, FP32 accumulators in TMEM):
//   Z1  = X  W1^T            (K = 16)    TMEM cols   0..63
//   Z2  = A1 W2^T            (K = 64)    TMEM cols  64..127     A1 = relu(Z1 + b1)
//   dA1 = dZ2 W2             (K = 64)    TMEM cols   0..63      dZ2 = dy w3 [Z2 + b2 > 0]
//   G  += [dZ2^T; dZ1^T] [A1^T; X^T; 1]^T  (K = 128 pairs, N = 80)  TMEM cols 128..207, summed over tiles
// so G holds dW2 (rows 0-63, cols 0-63), db2 (rows 0-63, col 76), dW1 (rows 64-127, cols 64-75) and db1
// (rows 64-127, col 76); the 64 -> 1 output layer and its gradient are FP32 on the CUDA cores. At the end the
// CTA adds G into the global gradient with atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gpe_internal.h"
#include "mlp.cuh"

struct gpe_mlp {
    int device = 0;
    gpe::MlpDev* dev = nullptr; // network image read by the kernels
    float* master    = nullptr; // FP32 parameter vector (GPE_MLP_NUM_WEIGHTS)
    float* grad      = nullptr; // gradient accumulator, [NW] = loss sum, [NW+1] = epoch loss sum
    float* adam_m    = nullptr;
    float* adam_v    = nullptr;
    double* stats    = nullptr; // standardisation sums
    uint32_t* status = nullptr;
    float* X         = nullptr; // pair set
    float* T         = nullptr;
    int32_t* idx     = nullptr;
    int32_t* cnt     = nullptr;
    int32_t* order   = nullptr; // shuffled pair indices of an epoch
    int32_t* h_order = nullptr; // pinned staging of the above
    int64_t cap      = 0;
    int64_t adam_t   = 0;
    int32_t pair_iters = 20;    // iterations of the plain solve that produced the pairs
    float mu[GPE_MLP_FEATURES], sd[GPE_MLP_FEATURES], ymu = 0.f, ysd = 1.f;
    void* base       = nullptr;
};

namespace gpe {

const MlpDev* mlp_device(const gpe_mlp* m) { return m->dev; }
MlpData mlp_data(gpe_mlp* m) { return MlpData{m->X, m->T, m->idx, m->cnt, m->cap}; }
int32_t mlp_pair_iters(const gpe_mlp* m) { return m->pair_iters; }
void mlp_set_pair_iters(gpe_mlp* m, int32_t iters) { m->pair_iters = iters; }

namespace {

constexpr int GB_N    = 80; // rows of the weight-gradient B operand: A1^T (64), X^T (12), ones, zero pad
constexpr int GB_ONES = 76;
constexpr uint32_t TRAIN_TMEM_COLS = 256;

struct __align__(128) MlpTrainSmem {
    uint16_t x[MLP_TILE * MLP_FP];
    uint16_t a1[MLP_TILE * MLP_H];
    uint16_t dz2[MLP_TILE * MLP_H];
    uint16_t ag[128 * MLP_TILE];  // rows 0-63: dZ2^T, rows 64-127: dZ1^T; K = the tile's pairs
    uint16_t bg[GB_N * MLP_TILE]; // rows 0-63: A1^T, 64-75: X^T, 76: ones (0 for padding rows), 77-79: 0
    uint16_t w1[MLP_H * MLP_FP];
    uint16_t w2[MLP_H * MLP_H];
    uint16_t w2t[MLP_H * MLP_H];
    float b1[MLP_H], b2[MLP_H], w3[MLP_H], mu[MLP_FP], isd[MLP_FP];
    float dw3[MLP_H];
    float db3, loss, b3, ymu, iysd;
    uint64_t bar;
    uint32_t tmem;
};

__device__ __forceinline__ uint16_t bf16_bits(float v)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    return *reinterpret_cast<const uint16_t*>(&h);
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { v += __shfl_xor_sync(0xffffffffu, v, o); }
    return v;
}

__global__ void __launch_bounds__(MLP_TILE, 1)
    k_mlp_train(const MlpDev* __restrict__ m, const float* __restrict__ X, const float* __restrict__ T,
                const int32_t* __restrict__ order, int32_t n, float inv_n, float* __restrict__ grad,
                uint32_t* __restrict__ status)
{
    extern __shared__ uint8_t smem_raw[];
    MlpTrainSmem& S = *reinterpret_cast<MlpTrainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                        ~static_cast<uintptr_t>(127));
    const uint32_t r     = threadIdx.x;
    const int32_t ntiles = (n + MLP_TILE - 1) / MLP_TILE;
    if ((int32_t)blockIdx.x >= ntiles) { return; } // uniform over the CTA, before any barrier

    // ---- stage the network, clear the accumulators ----
    {
        const uint4* s1 = reinterpret_cast<const uint4*>(m->w1);
        const uint4* s2 = reinterpret_cast<const uint4*>(m->w2);
        const uint4* s3 = reinterpret_cast<const uint4*>(m->w2t);
        for (int q = r; q < MLP_H * MLP_FP / 8; q += MLP_TILE) { reinterpret_cast<uint4*>(S.w1)[q] = s1[q]; }
        for (int q = r; q < MLP_H * MLP_H / 8; q += MLP_TILE) {
            reinterpret_cast<uint4*>(S.w2)[q]  = s2[q];
            reinterpret_cast<uint4*>(S.w2t)[q] = s3[q];
        }
        const uint4 z4 = make_uint4(0, 0, 0, 0);
        for (int q = r; q < GB_N * MLP_TILE / 8; q += MLP_TILE) { reinterpret_cast<uint4*>(S.bg)[q] = z4; }
        if (r < MLP_H) {
            S.b1[r]  = m->b1[r];
            S.b2[r]  = m->b2[r];
            S.w3[r]  = m->w3[r];
            S.dw3[r] = 0.f;
        }
        if (r < MLP_FP) {
            S.mu[r]  = m->mu[r];
            S.isd[r] = m->isd[r];
        }
        if (r == 0) {
            S.db3  = 0.f;
            S.loss = 0.f;
            S.b3   = m->b3;
            S.ymu  = m->ymu;
            S.iysd = m->ysd > 0.f ? 1.f / m->ysd : 0.f;
            tc::mbar_init(&S.bar, 1);
        }
        if (r < 32) { tc::tmem_alloc(&S.tmem, TRAIN_TMEM_COLS); }
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    }
    const uint32_t tm   = S.tmem;
    constexpr uint32_t ID64 = tc::idesc_bf16(128, 64);
    constexpr uint32_t ID80 = tc::idesc_bf16(128, GB_N);
    uint32_t phase      = 0;
    bool ok             = true;
    bool first          = true;
    float my_loss = 0.f, my_db3 = 0.f;
    const uint16_t one_bits = bf16_bits(1.f);

    for (int32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int32_t q    = tile * MLP_TILE + (int32_t)r;
        const bool valid   = q < n;
        const int32_t s    = valid ? (order ? __ldg(&order[q]) : q) : 0;
        // ---- standardised features: layer-1 A row and B rows 64-75 of the gradient product ----
        float xn[MLP_FP];
#pragma unroll
        for (int f = 0; f < MLP_FP; ++f) {
            xn[f] = (valid && f < MLP_F) ? (__ldg(&X[(size_t)s * MLP_F + (f < MLP_F ? f : 0)]) - S.mu[f]) * S.isd[f]
                                         : 0.f;
        }
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            uint4 u;
            u.x = tc::pack_bf16(xn[8 * c + 0], xn[8 * c + 1]);
            u.y = tc::pack_bf16(xn[8 * c + 2], xn[8 * c + 3]);
            u.z = tc::pack_bf16(xn[8 * c + 4], xn[8 * c + 5]);
            u.w = tc::pack_bf16(xn[8 * c + 6], xn[8 * c + 7]);
            *reinterpret_cast<uint4*>(&S.x[kmajor(r, 8 * c, MLP_FP)]) = u;
        }
#pragma unroll
        for (int f = 0; f < MLP_F; ++f) { S.bg[kmajor(64 + f, r, MLP_TILE)] = bf16_bits(xn[f]); }
        S.bg[kmajor(GB_ONES, r, MLP_TILE)] = valid ? one_bits : (uint16_t)0;
        const float tn = valid ? (__ldg(&T[s]) - S.ymu) * S.iysd : 0.f;
        tc::fence_async_smem();
        __syncthreads();
        if (r == 0) {
            tc::fence_after();
            tc::mma(tm, tc::sdesc(tc::saddr(S.x), 128, MLP_FP * 16), tc::sdesc(tc::saddr(S.w1), 128, MLP_FP * 16),
                    ID64, 0u);
            tc::commit(&S.bar);
        }
        ok = tc::mbar_wait(&S.bar, phase) && ok;
        phase ^= 1u;
        tc::fence_after();
        // ---- hidden layer 1 ----
        uint32_t mask1[2] = {0u, 0u};
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float z[16];
            tc::ld16(tc::lane_addr(tm, 16u * g), z);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float a[8];
#pragma unroll
                for (int qq = 0; qq < 8; ++qq) {
                    const int j  = 16 * g + 8 * c + qq;
                    const float v = z[8 * c + qq] + S.b1[j];
                    a[qq]         = fmaxf(v, 0.f);
                    if (v > 0.f) { mask1[j >> 5] |= 1u << (j & 31); }
                    S.bg[kmajor(j, r, MLP_TILE)] = bf16_bits(a[qq]);
                }
                uint4 u;
                u.x = tc::pack_bf16(a[0], a[1]);
                u.y = tc::pack_bf16(a[2], a[3]);
                u.z = tc::pack_bf16(a[4], a[5]);
                u.w = tc::pack_bf16(a[6], a[7]);
                *reinterpret_cast<uint4*>(&S.a1[kmajor(r, 16 * g + 8 * c, MLP_H)]) = u;
            }
        }
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        if (r == 0) {
            tc::fence_after();
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                tc::mma(tm + 64u, tc::sdesc(tc::saddr(S.a1) + 256u * k, 128, MLP_H * 16),
                        tc::sdesc(tc::saddr(S.w2) + 256u * k, 128, MLP_H * 16), ID64, k > 0 ? 1u : 0u);
            }
            tc::commit(&S.bar);
        }
        ok = tc::mbar_wait(&S.bar, phase) && ok;
        phase ^= 1u;
        tc::fence_after();
        // ---- output, loss, dZ2 ----
        float y = S.b3;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float z[16];
            tc::ld16(tc::lane_addr(tm, 64u + 16u * g), z);
#pragma unroll
            for (int qq = 0; qq < 16; ++qq) { y = fmaf(fmaxf(z[qq] + S.b2[16 * g + qq], 0.f), S.w3[16 * g + qq], y); }
        }
        const float e  = valid ? y - tn : 0.f;
        const float dy = 2.f * e * inv_n;
        my_loss        = fmaf(e, e, my_loss);
        my_db3 += dy;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float z[16];
            tc::ld16(tc::lane_addr(tm, 64u + 16u * g), z);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float d[8];
#pragma unroll
                for (int qq = 0; qq < 8; ++qq) {
                    const int j   = 16 * g + 8 * c + qq;
                    const float v = z[8 * c + qq] + S.b2[j];
                    d[qq]         = v > 0.f ? dy * S.w3[j] : 0.f;
                    const float p = warp_sum(dy * fmaxf(v, 0.f));
                    if ((r & 31) == 0) { atomicAdd(&S.dw3[j], p); }
                    S.ag[kmajor(j, r, MLP_TILE)] = bf16_bits(d[qq]);
                }
                uint4 u;
                u.x = tc::pack_bf16(d[0], d[1]);
                u.y = tc::pack_bf16(d[2], d[3]);
                u.z = tc::pack_bf16(d[4], d[5]);
                u.w = tc::pack_bf16(d[6], d[7]);
                *reinterpret_cast<uint4*>(&S.dz2[kmajor(r, 16 * g + 8 * c, MLP_H)]) = u;
            }
        }
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        if (r == 0) {
            tc::fence_after();
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                tc::mma(tm, tc::sdesc(tc::saddr(S.dz2) + 256u * k, 128, MLP_H * 16),
                        tc::sdesc(tc::saddr(S.w2t) + 256u * k, 128, MLP_H * 16), ID64, k > 0 ? 1u : 0u);
            }
            tc::commit(&S.bar);
        }
        ok = tc::mbar_wait(&S.bar, phase) && ok;
        phase ^= 1u;
        tc::fence_after();
        // ---- dZ1 ----
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float z[16];
            tc::ld16(tc::lane_addr(tm, 16u * g), z);
#pragma unroll
            for (int qq = 0; qq < 16; ++qq) {
                const int j   = 16 * g + qq;
                const float d = ((mask1[j >> 5] >> (j & 31)) & 1u) ? z[qq] : 0.f;
                S.ag[kmajor(64 + j, r, MLP_TILE)] = bf16_bits(d);
            }
        }
        tc::fence_before();
        tc::fence_async_smem();
        __syncthreads();
        if (r == 0) {
            tc::fence_after();
#pragma unroll
            for (uint32_t k = 0; k < MLP_TILE / 16; ++k) {
                tc::mma(tm + 128u, tc::sdesc(tc::saddr(S.ag) + 256u * k, 128, MLP_TILE * 16),
                        tc::sdesc(tc::saddr(S.bg) + 256u * k, 128, MLP_TILE * 16), ID80,
                        (first && k == 0) ? 0u : 1u);
            }
            tc::commit(&S.bar);
        }
        ok = tc::mbar_wait(&S.bar, phase) && ok; // the next tile overwrites the operands
        phase ^= 1u;
        tc::fence_after();
        first = false;
    }

    // ---- the CTA's sums into the global gradient ----
    my_loss = warp_sum(my_loss);
    my_db3  = warp_sum(my_db3);
    if ((r & 31) == 0) {
        atomicAdd(&S.loss, my_loss);
        atomicAdd(&S.db3, my_db3);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
#pragma unroll
    for (int g = 0; g < GB_N / 16; ++g) {
        float z[16];
        tc::ld16(tc::lane_addr(tm, 128u + 16u * g), z);
#pragma unroll
        for (int qq = 0; qq < 16; ++qq) {
            const int c = 16 * g + qq;
            if (r < 64) {
                if (c < 64) { atomicAdd(&grad[MLP_OFF_W2 + r * MLP_H + c], z[qq]); }
                if (c == GB_ONES) { atomicAdd(&grad[MLP_OFF_B2 + r], z[qq]); }
            } else {
                const int i = (int)r - 64;
                if (c >= 64 && c < 64 + MLP_F) { atomicAdd(&grad[MLP_OFF_W1 + i * MLP_F + (c - 64)], z[qq]); }
                if (c == GB_ONES) { atomicAdd(&grad[MLP_OFF_B1 + i], z[qq]); }
            }
        }
    }
    if (r < MLP_H) { atomicAdd(&grad[MLP_OFF_W3 + r], S.dw3[r]); }
    if (r == 0) {
        atomicAdd(&grad[MLP_OFF_B3], S.db3);
        atomicAdd(&grad[MLP_NW], S.loss);
    }
    if (!ok) { atomicOr(status, GPE_STATUS_TIMEOUT); }
    tc::fence_before();
    __syncthreads();
    if (r < 32) {
        tc::fence_after();
        tc::tmem_dealloc(tm, TRAIN_TMEM_COLS);
    }
}

// Writes parameter p of the FP32 vector into the kernels' image (BF16 layouts and FP32 vectors).
__device__ __forceinline__ void put_param(MlpDev* m, int p, float w)
{
    if (p < MLP_OFF_B1) {
        const int i = p / MLP_F, f = p % MLP_F;
        m->w1[kmajor(i, f, MLP_FP)] = bf16_bits(w);
    } else if (p < MLP_OFF_W2) {
        m->b1[p - MLP_OFF_B1] = w;
    } else if (p < MLP_OFF_B2) {
        const int j = (p - MLP_OFF_W2) / MLP_H, i = (p - MLP_OFF_W2) % MLP_H;
        m->w2[kmajor(j, i, MLP_H)]  = bf16_bits(w);
        m->w2t[kmajor(i, j, MLP_H)] = bf16_bits(w);
    } else if (p < MLP_OFF_W3) {
        m->b2[p - MLP_OFF_B2] = w;
    } else if (p < MLP_OFF_B3) {
        m->w3[p - MLP_OFF_W3] = w;
    } else {
        m->b3 = w;
    }
}

__global__ void k_mlp_pack(MlpDev* __restrict__ m, const float* __restrict__ master)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < MLP_NW) { put_param(m, p, master[p]); }
}

// AdamW (Loshchilov & Hutter 2019): decoupled weight decay on W1, W2 and w3; bc1, bc2 = 1 - beta^t.
__global__ void k_mlp_adamw(MlpDev* __restrict__ m, float* __restrict__ master, float* __restrict__ grad,
                            float* __restrict__ am, float* __restrict__ av, float lr, float wd, float b1, float b2,
                            float eps, float bc1, float bc2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        grad[MLP_NW + 1] += grad[MLP_NW];
        grad[MLP_NW] = 0.f;
    }
    if (p >= MLP_NW) { return; }
    const float g = grad[p];
    grad[p]       = 0.f;
    const float mm = b1 * am[p] + (1.f - b1) * g;
    const float vv = b2 * av[p] + (1.f - b2) * g * g;
    am[p]          = mm;
    av[p]          = vv;
    const bool decay = (p < MLP_OFF_B1) || (p >= MLP_OFF_W2 && p < MLP_OFF_B2) || (p >= MLP_OFF_W3 && p < MLP_OFF_B3);
    float w          = master[p];
    w -= lr * ((mm / bc1) / (sqrtf(vv / bc2) + eps) + (decay ? wd * w : 0.f));
    master[p] = w;
    put_param(m, p, w);
}

// Sums of x, x^2 per feature and of t, t^2 over pairs [0, n) (FP64).
__global__ void k_mlp_stats(const float* __restrict__ X, const float* __restrict__ T, int32_t n,
                            double* __restrict__ acc)
{
    double s[2 * MLP_F + 2];
#pragma unroll
    for (int q = 0; q < 2 * MLP_F + 2; ++q) { s[q] = 0.0; }
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int f = 0; f < MLP_F; ++f) {
            const double v = X[(size_t)i * MLP_F + f];
            s[f] += v;
            s[MLP_F + f] += v * v;
        }
        const double t = T[i];
        s[2 * MLP_F] += t;
        s[2 * MLP_F + 1] += t * t;
    }
#pragma unroll
    for (int q = 0; q < 2 * MLP_F + 2; ++q) {
        double v = s[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) { v += __shfl_xor_sync(0xffffffffu, v, o); }
        if ((threadIdx.x & 31) == 0) { atomicAdd(&acc[q], v); }
    }
}

__global__ void __launch_bounds__(MLP_TILE)
    k_mlp_infer(const MlpDev* __restrict__ m, const float* __restrict__ X, float* __restrict__ out, int32_t n,
                uint32_t* __restrict__ status)
{
    __shared__ MlpFwdSmem S;
    const int32_t ntiles = (n + MLP_TILE - 1) / MLP_TILE;
    if ((int32_t)blockIdx.x >= ntiles) { return; }
    mlp_fwd_setup(S, m);
    const float ymu = m->ymu, ysd = m->ysd;
    uint32_t phase  = 0;
    bool ok         = true;
    for (int32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int32_t q  = tile * MLP_TILE + (int32_t)threadIdx.x;
        const bool valid = q < n;
        float f[MLP_F];
#pragma unroll
        for (int k = 0; k < MLP_F; ++k) { f[k] = valid ? __ldg(&X[(size_t)q * MLP_F + k]) : 0.f; }
        const float y = mlp_fwd_tile(S, f, phase, ok);
        if (valid) { out[q] = fmaf(y, ysd, ymu); }
    }
    if (!ok) { atomicOr(status, GPE_STATUS_TIMEOUT); }
    mlp_fwd_teardown(S);
}

// ----- host helpers -------------------------------------------------------------------------------------
uint64_t splitmix64(uint64_t& s)
{
    // SplitMix64 (Steele, Lea & Flood 2014)
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

int32_t upload_norm(gpe_mlp* m, cudaStream_t st)
{
    float mu[MLP_FP] = {0}, isd[MLP_FP] = {0};
    for (int f = 0; f < MLP_F; ++f) {
        mu[f]  = m->mu[f];
        isd[f] = m->sd[f] > 0.f ? 1.f / m->sd[f] : 0.f;
    }
    const float y[2] = {m->ymu, m->ysd};
    GPE_TRY_CUDA(cudaMemcpyAsync(m->dev->mu, mu, sizeof(mu), cudaMemcpyHostToDevice, st));
    GPE_TRY_CUDA(cudaMemcpyAsync(m->dev->isd, isd, sizeof(isd), cudaMemcpyHostToDevice, st));
    GPE_TRY_CUDA(cudaMemcpyAsync(&m->dev->ymu, y, sizeof(y), cudaMemcpyHostToDevice, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    return GPE_OK;
}

int32_t read_status(gpe_mlp* m, cudaStream_t st)
{
    uint32_t v = 0;
    GPE_TRY_CUDA(cudaMemcpyAsync(&v, m->status, sizeof(v), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    if (v) {
        GPE_TRY_CUDA(cudaMemsetAsync(m->status, 0, sizeof(uint32_t), st));
        if (v & GPE_STATUS_TIMEOUT) {
            gpe::set_error(GPE_ERR_TIMEOUT, "a tensor-core wait of the network kernels gave up");
            return GPE_ERR_TIMEOUT;
        }
    }
    return GPE_OK;
}

int32_t pair_count(const gpe_mlp* m, cudaStream_t st, int64_t* n)
{
    int32_t c[2] = {0, 0};
    GPE_TRY_CUDA(cudaMemcpyAsync(c, m->cnt, sizeof(c), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    *n = std::min<int64_t>(c[1], m->cap);
    return GPE_OK;
}

int train_grid(int32_t n) { return std::max(1, std::min((n + MLP_TILE - 1) / MLP_TILE, gpe::sm_count())); }

size_t train_smem() { return sizeof(MlpTrainSmem) + 128; }

} // namespace
} // namespace gpe

using namespace gpe;

extern "C" {

int32_t gpe_mlp_create(int64_t max_pairs, uint64_t seed, gpe_mlp** out)
{
    gpe::clear_error();
    if (!out || max_pairs < 0 || max_pairs > (int64_t)INT32_MAX / 2) { return GPE_ERR_BAD_ARG; }
    *out    = nullptr;
    int dev = 0;
    int32_t rc = gpe::current_device(&dev);
    if (rc) { return rc; }
    gpe_mlp* m = new gpe_mlp();
    m->device  = dev;
    m->cap     = max_pairs;
    const size_t P = (size_t)std::max<int64_t>(max_pairs, 1);
    Carver c;
    const size_t o_dev  = c.take<MlpDev>(1);
    const size_t o_mas  = c.take<float>(MLP_NW);
    const size_t o_grad = c.take<float>(MLP_NW + 8);
    const size_t o_am   = c.take<float>(MLP_NW);
    const size_t o_av   = c.take<float>(MLP_NW);
    const size_t o_st   = c.take<double>(64);
    const size_t o_stat = c.take<uint32_t>(4);
    const size_t o_cnt  = c.take<int32_t>(4);
    const size_t o_X    = c.take<float>(P * MLP_F);
    const size_t o_T    = c.take<float>(P);
    const size_t o_idx  = c.take<int32_t>(P);
    const size_t o_ord  = c.take<int32_t>(P);
    cudaError_t e       = cudaMalloc(&m->base, c.off);
    if (e == cudaSuccess) { e = cudaMemset(m->base, 0, c.off); }
    if (e == cudaSuccess) { e = cudaMallocHost(&m->h_order, sizeof(int32_t) * P); }
    if (e == cudaSuccess) {
        e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem());
    }
    if (e != cudaSuccess) {
        gpe::set_cuda_error(e, "gpe_mlp_create");
        if (m->base) { cudaFree(m->base); }
        if (m->h_order) { cudaFreeHost(m->h_order); }
        delete m;
        return GPE_ERR_CUDA;
    }
    uint8_t* b  = static_cast<uint8_t*>(m->base);
    m->dev      = reinterpret_cast<MlpDev*>(b + o_dev);
    m->master   = reinterpret_cast<float*>(b + o_mas);
    m->grad     = reinterpret_cast<float*>(b + o_grad);
    m->adam_m   = reinterpret_cast<float*>(b + o_am);
    m->adam_v   = reinterpret_cast<float*>(b + o_av);
    m->stats    = reinterpret_cast<double*>(b + o_st);
    m->status   = reinterpret_cast<uint32_t*>(b + o_stat);
    m->cnt      = reinterpret_cast<int32_t*>(b + o_cnt);
    m->X        = reinterpret_cast<float*>(b + o_X);
    m->T        = reinterpret_cast<float*>(b + o_T);
    m->idx      = reinterpret_cast<int32_t*>(b + o_idx);
    m->order    = reinterpret_cast<int32_t*>(b + o_ord);
    // uniform He initialisation (He et al. 2015): U(-sqrt(6/fan_in), sqrt(6/fan_in)); the output layer
    // starts small so that an untrained network stays close to the previous-step warm start
    std::vector<float> w(MLP_NW, 0.f);
    uint64_t s = seed ^ 0x6A09E667F3BCC909ull;
    const double a1 = std::sqrt(6.0 / MLP_F), a2 = std::sqrt(6.0 / MLP_H), a3 = 0.1 * std::sqrt(6.0 / MLP_H);
    for (int p = MLP_OFF_W1; p < MLP_OFF_B1; ++p) { w[p] = (float)((2.0 * uniform01(s) - 1.0) * a1); }
    for (int p = MLP_OFF_W2; p < MLP_OFF_B2; ++p) { w[p] = (float)((2.0 * uniform01(s) - 1.0) * a2); }
    for (int p = MLP_OFF_W3; p < MLP_OFF_B3; ++p) { w[p] = (float)((2.0 * uniform01(s) - 1.0) * a3); }
    for (int f = 0; f < MLP_F; ++f) {
        m->mu[f] = 0.f;
        m->sd[f] = 1.f;
    }
    m->ymu = 0.f;
    m->ysd = 1.f;
    *out   = m;
    float blob[GPE_MLP_BLOB_FLOATS];
    std::memcpy(blob, w.data(), sizeof(float) * MLP_NW);
    for (int f = 0; f < MLP_F; ++f) {
        blob[MLP_NW + f]         = 0.f;
        blob[MLP_NW + MLP_F + f] = 1.f;
    }
    blob[MLP_NW + 2 * MLP_F]     = 0.f;
    blob[MLP_NW + 2 * MLP_F + 1] = 1.f;
    rc = gpe_mlp_set_blob(m, blob, GPE_MLP_BLOB_FLOATS);
    if (rc) {
        gpe_mlp_destroy(m);
        *out = nullptr;
    }
    return rc;
}

int32_t gpe_mlp_destroy(gpe_mlp* m)
{
    if (!m) { return GPE_ERR_BAD_ARG; }
    if (m->base) { cudaFree(m->base); }
    if (m->h_order) { cudaFreeHost(m->h_order); }
    delete m;
    return GPE_OK;
}

int32_t gpe_mlp_get_blob(const gpe_mlp* m, float* blob, int64_t n)
{
    gpe::clear_error();
    if (!m || !blob || n != GPE_MLP_BLOB_FLOATS) { return GPE_ERR_BAD_ARG; }
    GPE_TRY_CUDA(cudaMemcpy(blob, m->master, sizeof(float) * MLP_NW, cudaMemcpyDeviceToHost));
    for (int f = 0; f < MLP_F; ++f) {
        blob[MLP_NW + f]         = m->mu[f];
        blob[MLP_NW + MLP_F + f] = m->sd[f];
    }
    blob[MLP_NW + 2 * MLP_F]     = m->ymu;
    blob[MLP_NW + 2 * MLP_F + 1] = m->ysd;
    return GPE_OK;
}

int32_t gpe_mlp_set_blob(gpe_mlp* m, const float* blob, int64_t n)
{
    gpe::clear_error();
    if (!m || !blob || n != GPE_MLP_BLOB_FLOATS) { return GPE_ERR_BAD_ARG; }
    for (int64_t q = 0; q < n; ++q) {
        if (!std::isfinite(blob[q])) {
            gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mlp_set_blob: entry %lld is not finite", (long long)q);
            return GPE_ERR_BAD_ARG;
        }
    }
    for (int f = 0; f < MLP_F; ++f) {
        m->mu[f] = blob[MLP_NW + f];
        m->sd[f] = blob[MLP_NW + MLP_F + f];
    }
    m->ymu = blob[MLP_NW + 2 * MLP_F];
    m->ysd = blob[MLP_NW + 2 * MLP_F + 1];
    GPE_TRY_CUDA(cudaMemcpy(m->master, blob, sizeof(float) * MLP_NW, cudaMemcpyHostToDevice));
    GPE_TRY_CUDA(cudaMemset(m->adam_m, 0, sizeof(float) * MLP_NW));
    GPE_TRY_CUDA(cudaMemset(m->adam_v, 0, sizeof(float) * MLP_NW));
    m->adam_t = 0;
    k_mlp_pack<<<(MLP_NW + 255) / 256, 256>>>(m->dev, m->master);
    GPE_CHECK_LAUNCH("k_mlp_pack");
    int32_t rc = upload_norm(m, nullptr);
    if (rc) { return rc; }
    GPE_TRY_CUDA(cudaDeviceSynchronize());
    return GPE_OK;
}

int32_t gpe_mlp_num_pairs(const gpe_mlp* m, int64_t* n)
{
    if (!m || !n) { return GPE_ERR_BAD_ARG; }
    return pair_count(m, nullptr, n);
}

int32_t gpe_mlp_get_pairs(const gpe_mlp* m, float* features, float* targets, int32_t* index, int64_t n,
                          int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!m || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    int64_t have    = 0;
    int32_t rc      = pair_count(m, st, &have);
    if (rc) { return rc; }
    if (n != have) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mlp_get_pairs: n must equal the pair count (%lld)", (long long)have);
        return GPE_ERR_BAD_ARG;
    }
    const cudaMemcpyKind k = mem == GPE_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (n > 0) {
        if (features) { GPE_TRY_CUDA(cudaMemcpyAsync(features, m->X, sizeof(float) * MLP_F * (size_t)n, k, st)); }
        if (targets) { GPE_TRY_CUDA(cudaMemcpyAsync(targets, m->T, sizeof(float) * (size_t)n, k, st)); }
        if (index) { GPE_TRY_CUDA(cudaMemcpyAsync(index, m->idx, sizeof(int32_t) * (size_t)n, k, st)); }
    }
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    return GPE_OK;
}

int32_t gpe_mlp_set_pairs(gpe_mlp* m, const float* features, const float* targets, int64_t n, int32_t mem,
                          void* stream)
{
    gpe::clear_error();
    if (!m || n < 0 || (n > 0 && (!features || !targets)) || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) {
        return GPE_ERR_BAD_ARG;
    }
    if (n > m->cap) {
        gpe::set_error(GPE_ERR_CAPACITY, "gpe_mlp_set_pairs: %lld pairs exceed the capacity %lld", (long long)n,
                       (long long)m->cap);
        return GPE_ERR_CAPACITY;
    }
    cudaStream_t st        = as_stream(stream);
    const cudaMemcpyKind k = mem == GPE_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (n > 0) {
        GPE_TRY_CUDA(cudaMemcpyAsync(m->X, features, sizeof(float) * MLP_F * (size_t)n, k, st));
        GPE_TRY_CUDA(cudaMemcpyAsync(m->T, targets, sizeof(float) * (size_t)n, k, st));
        GPE_TRY_CUDA(cudaMemsetAsync(m->idx, 0xff, sizeof(int32_t) * (size_t)n, st));
    }
    const int32_t c[2] = {(int32_t)n, (int32_t)n};
    GPE_TRY_CUDA(cudaMemcpyAsync(m->cnt, c, sizeof(c), cudaMemcpyHostToDevice, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    return GPE_OK;
}

int32_t gpe_mlp_train(gpe_mlp* m, const gpe_mlp_train_params* tp, float* train_loss, float* val_loss, void* stream)
{
    gpe::clear_error();
    if (!m || !tp || tp->epochs < 0 || tp->batch <= 0 || !(tp->lr >= 0.f) || !(tp->val_fraction >= 0.f) ||
        !(tp->val_fraction < 1.f) || !(tp->beta1 >= 0.f && tp->beta1 < 1.f) || !(tp->beta2 >= 0.f && tp->beta2 < 1.f) ||
        tp->lr_schedule < 0 || tp->lr_schedule > 1) {
        return GPE_ERR_BAD_ARG;
    }
    cudaStream_t st = as_stream(stream);
    int64_t n       = 0;
    int32_t rc      = pair_count(m, st, &n);
    if (rc) { return rc; }
    const int64_t n_val   = (int64_t)std::floor((double)n * tp->val_fraction);
    const int64_t n_train = n - n_val;
    if (n_train <= 0) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_mlp_train: no training pairs");
        return GPE_ERR_NOT_READY;
    }
    // standardisation from the training pairs
    GPE_TRY_CUDA(cudaMemsetAsync(m->stats, 0, sizeof(double) * 64, st));
    k_mlp_stats<<<std::min<int64_t>((n_train + 255) / 256, 4 * gpe::sm_count()), 256, 0, st>>>(m->X, m->T,
                                                                                           (int32_t)n_train, m->stats);
    GPE_CHECK_LAUNCH("k_mlp_stats");
    double acc[2 * MLP_F + 2];
    GPE_TRY_CUDA(cudaMemcpyAsync(acc, m->stats, sizeof(acc), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    const double nn = (double)n_train;
    for (int f = 0; f < MLP_F; ++f) {
        const double mu = acc[f] / nn;
        const double va = std::max(acc[MLP_F + f] / nn - mu * mu, 0.0);
        const double sd = std::sqrt(va);
        m->mu[f]        = (float)mu;
        m->sd[f]        = sd > 1e-12 * std::max(1.0, std::fabs(mu)) ? (float)sd : 0.f;
    }
    {
        const double mu = acc[2 * MLP_F] / nn;
        const double sd = std::sqrt(std::max(acc[2 * MLP_F + 1] / nn - mu * mu, 0.0));
        m->ymu          = (float)mu;
        m->ysd          = sd > 0.0 ? (float)sd : 1.f;
    }
    rc = upload_norm(m, st);
    if (rc) { return rc; }
    GPE_TRY_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * (MLP_NW + 8), st));
    // epochs
    uint64_t rs      = tp->seed ^ 0xBB67AE8584CAA73Bull;
    const int32_t B  = tp->batch;
    float last_epoch = 0.f;
    const double steps_total = (double)tp->epochs * (double)((n_train + B - 1) / B);
    int64_t step             = 0;
    for (int32_t ep = 0; ep < tp->epochs; ++ep) {
        GPE_TRY_CUDA(cudaStreamSynchronize(st)); // the pinned order buffer is rewritten below
        for (int64_t q = 0; q < n_train; ++q) { m->h_order[q] = (int32_t)q; }
        for (int64_t q = n_train - 1; q > 0; --q) { // Fisher-Yates
            const int64_t j = (int64_t)(splitmix64(rs) % (uint64_t)(q + 1));
            std::swap(m->h_order[q], m->h_order[j]);
        }
        GPE_TRY_CUDA(cudaMemcpyAsync(m->order, m->h_order, sizeof(int32_t) * (size_t)n_train, cudaMemcpyHostToDevice, st));
        GPE_TRY_CUDA(cudaMemsetAsync(m->grad + MLP_NW + 1, 0, sizeof(float), st));
        for (int64_t b0 = 0; b0 < n_train; b0 += B) {
            const int32_t nb = (int32_t)std::min<int64_t>(B, n_train - b0);
            k_mlp_train<<<train_grid(nb), MLP_TILE, train_smem(), st>>>(m->dev, m->X, m->T, m->order + b0, nb,
                                                                       1.f / (float)nb, m->grad, m->status);
            GPE_CHECK_LAUNCH("k_mlp_train");
            ++m->adam_t;
            const float bc1 = 1.f - (float)std::pow((double)tp->beta1, (double)m->adam_t);
            const float bc2 = 1.f - (float)std::pow((double)tp->beta2, (double)m->adam_t);
            const float lr = tp->lr_schedule == 1
                                 ? (float)(0.5 * (double)tp->lr *
                                           (1.0 + std::cos(3.141592653589793 * (double)step / steps_total)))
                                 : tp->lr;
            ++step;
            k_mlp_adamw<<<(MLP_NW + 255) / 256, 256, 0, st>>>(m->dev, m->master, m->grad, m->adam_m, m->adam_v, lr,
                                                               tp->weight_decay, tp->beta1, tp->beta2, tp->adam_eps,
                                                               bc1, bc2);
            GPE_CHECK_LAUNCH("k_mlp_adamw");
            if (m->adam_t == 1) {
                rc = read_status(m, st); // a first step that timed out stops the run at once
                if (rc) { return rc; }
            }
        }
        float el = 0.f;
        GPE_TRY_CUDA(cudaMemcpyAsync(&el, m->grad + MLP_NW + 1, sizeof(float), cudaMemcpyDeviceToHost, st));
        GPE_TRY_CUDA(cudaStreamSynchronize(st));
        last_epoch = el / (float)n_train;
        rc         = read_status(m, st);
        if (rc) { return rc; }
    }
    if (train_loss) { *train_loss = last_epoch; }
    if (val_loss) {
        float vl = 0.f;
        if (n_val > 0) {
            GPE_TRY_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * (MLP_NW + 8), st));
            k_mlp_train<<<train_grid((int32_t)n_val), MLP_TILE, train_smem(), st>>>(
                m->dev, m->X + (size_t)n_train * MLP_F, m->T + n_train, nullptr, (int32_t)n_val, 1.f / (float)n_val,
                m->grad, m->status);
            GPE_CHECK_LAUNCH("k_mlp_train");
            GPE_TRY_CUDA(cudaMemcpyAsync(&vl, m->grad + MLP_NW, sizeof(float), cudaMemcpyDeviceToHost, st));
            GPE_TRY_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * (MLP_NW + 8), st));
            GPE_TRY_CUDA(cudaStreamSynchronize(st));
            vl /= (float)n_val;
        }
        *val_loss = vl;
    }
    return read_status(m, st);
}

int32_t gpe_mlp_infer(const gpe_mlp* m, const float* features, float* out, int64_t n, int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!m || n < 0 || (n > 0 && (!features || !out)) || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE) ||
        n > (int64_t)INT32_MAX / MLP_F) {
        return GPE_ERR_BAD_ARG;
    }
    if (n == 0) { return GPE_OK; }
    cudaStream_t st = as_stream(stream);
    const float* dX = features;
    float* dY       = out;
    void* tmp       = nullptr;
    if (mem == GPE_MEM_HOST) {
        GPE_TRY_CUDA(cudaMalloc(&tmp, sizeof(float) * (size_t)n * (MLP_F + 1)));
        dX = static_cast<float*>(tmp);
        dY = static_cast<float*>(tmp) + (size_t)n * MLP_F;
        cudaError_t e = cudaMemcpyAsync(const_cast<float*>(dX), features, sizeof(float) * (size_t)n * MLP_F,
                                        cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            cudaFree(tmp);
            gpe::set_cuda_error(e, "gpe_mlp_infer");
            return GPE_ERR_CUDA;
        }
    }
    const int32_t ntiles = (int32_t)((n + MLP_TILE - 1) / MLP_TILE);
    k_mlp_infer<<<std::min(ntiles, 6 * gpe::sm_count()), MLP_TILE, 0, st>>>(m->dev, dX, dY, (int32_t)n, m->status);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && mem == GPE_MEM_HOST) {
        e = cudaMemcpyAsync(out, dY, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) { e = cudaStreamSynchronize(st); }
    if (tmp) { cudaFree(tmp); }
    if (e != cudaSuccess) {
        gpe::set_cuda_error(e, "gpe_mlp_infer");
        return GPE_ERR_CUDA;
    }
    return read_status(const_cast<gpe_mlp*>(m), st);
}

int32_t gpe_mlp_gradient(gpe_mlp* m, const float* features, const float* targets, int64_t n, float* grad,
                         float* loss, int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!m || n <= 0 || !features || !targets || !grad || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE) ||
        n > (int64_t)INT32_MAX / MLP_F) {
        return GPE_ERR_BAD_ARG;
    }
    cudaStream_t st = as_stream(stream);
    void* tmp       = nullptr;
    GPE_TRY_CUDA(cudaMalloc(&tmp, sizeof(float) * ((size_t)n * (MLP_F + 1) + MLP_NW + 8)));
    float* dX = static_cast<float*>(tmp);
    float* dT = dX + (size_t)n * MLP_F;
    float* dG = dT + n;
    const cudaMemcpyKind k = mem == GPE_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    cudaError_t e          = cudaMemcpyAsync(dX, features, sizeof(float) * (size_t)n * MLP_F, k, st);
    if (e == cudaSuccess) { e = cudaMemcpyAsync(dT, targets, sizeof(float) * (size_t)n, k, st); }
    if (e == cudaSuccess) { e = cudaMemsetAsync(dG, 0, sizeof(float) * (MLP_NW + 8), st); }
    if (e == cudaSuccess) {
        k_mlp_train<<<train_grid((int32_t)n), MLP_TILE, train_smem(), st>>>(m->dev, dX, dT, nullptr, (int32_t)n,
                                                                           1.f / (float)n, dG, m->status);
        e = cudaGetLastError();
    }
    const cudaMemcpyKind ko = mem == GPE_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (e == cudaSuccess) { e = cudaMemcpyAsync(grad, dG, sizeof(float) * MLP_NW, ko, st); }
    float l = 0.f;
    if (e == cudaSuccess) { e = cudaMemcpyAsync(&l, dG + MLP_NW, sizeof(float), cudaMemcpyDeviceToHost, st); }
    if (e == cudaSuccess) { e = cudaStreamSynchronize(st); }
    cudaFree(tmp);
    if (e != cudaSuccess) {
        gpe::set_cuda_error(e, "gpe_mlp_gradient");
        return GPE_ERR_CUDA;
    }
    if (loss) { *loss = l / (float)n; }
    return read_status(m, st);
}

} // extern "C"
