// mlp.cuh — the warm-start network on the fifth-generation tensor cores (device code shared by the PBF
// warm-start pass and the training kernels).
//
// Network: 12 -> 64 -> 64 -> 1 with ReLU, BF16 operands, FP32 accumulation. One CTA of 128 threads runs a
// tile of 128 samples: thread r owns sample r, which is row r of every A operand and TMEM lane r of every
// accumulator (M = 128, cta_group::1). Operands live in shared memory in the canonical K-major layout
// without swizzle: 8x8 core matrices of 16-byte rows, the core matrices of one 8-row group consecutive
// along K (128 B apart, the descriptor's leading byte offset) and the 8-row groups K*16 B apart (the
// stride byte offset). One elected thread issues tcgen05.mma; tcgen05.commit arrives on an mbarrier that
// every thread waits on with a time limit; tcgen05.ld brings each thread its accumulator row.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gpe {

constexpr int MLP_F  = 12;  // features
constexpr int MLP_FP = 16;  // features padded to one MMA K step
constexpr int MLP_H  = 64;  // hidden width
constexpr int MLP_TILE = 128;
// parameter vector (row-major [out][in]): W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_F;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H;
constexpr int MLP_NW     = MLP_OFF_B3 + 1;
static_assert(MLP_NW == GPE_MLP_NUM_WEIGHTS, "parameter count");
constexpr uint64_t MLP_WAIT_NS = 50ull * 1000ull * 1000ull; // a tensor-core wait gives up after 50 ms

// Element index of (row, k) in a K-major tile whose rows hold K BF16 elements (see the layout above).
__host__ __device__ constexpr uint32_t kmajor(uint32_t row, uint32_t k, uint32_t K)
{
    return (row >> 3) * (K * 8u) + (k >> 3) * 64u + (row & 7u) * 8u + (k & 7u);
}

// The network as the kernels read it: BF16 weight images already in the K-major layout, so a CTA stages
// them with 16-byte copies, and the FP32 vectors.
struct __align__(128) MlpDev {
    uint16_t w1[MLP_H * MLP_FP];  // B of layer 1: N = 64 outputs, K = 16 (features 12..15 zero)
    uint16_t w2[MLP_H * MLP_H];   // B of layer 2: N = 64 outputs, K = 64 inputs
    uint16_t w2t[MLP_H * MLP_H];  // W2 transposed: B of dA1 = dZ2 W2 (N = inputs, K = outputs)
    float b1[MLP_H], b2[MLP_H], w3[MLP_H];
    float mu[MLP_FP], isd[MLP_FP]; // feature standardisation (isd = 1/std, 0 for a constant feature)
    float b3, ymu, ysd, pad;       // output bias, target mean and std
};

namespace tc {

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading byte offset (next core matrix along K), stride
// byte offset (next 8-row group), descriptor version 1 (bits 46-47), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
                 "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}

// Arrives once on the mbarrier when every tcgen05.mma issued so far by this thread has completed.
__device__ __forceinline__ void commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the completion of the barrier phase of the given parity; false after MLP_WAIT_NS without it.
// try_wait suspends the thread until the phase completes or a hardware time limit passes; the loop around it
// checks the global timer between tries.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(ok)
                 : "r"(saddr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    if (mbar_try(bar, parity)) { return true; }
    const uint64_t t0 = globaltimer();
    while (!mbar_try(bar, parity)) {
        if (globaltimer() - t0 > MLP_WAIT_NS) { return false; }
    }
    return true;
}

// generic-proxy shared-memory writes -> visible to the tensor cores (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// One full warp: allocates ncols TMEM columns (a power of two >= 32) and writes the address to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31); the load and its
// wait are one statement so that no use of the registers can be scheduled before the data has arrived.
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15}, [%16];\n\ttcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) { v[q] = __uint_as_float(r[q]); }
}

// TMEM address of this thread's lane at column col (lanes are the upper 16 bits)
__device__ __forceinline__ uint32_t lane_addr(uint32_t base, uint32_t col)
{
    return base + ((uint32_t)((threadIdx.x >> 5) * 32u) << 16) + col;
}

// Bulk copy (the TMA engine, untiled) of `bytes` from global to this CTA's shared memory; completion is
// signalled on the mbarrier as transaction bytes. Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b); // a -> low half (lower address)
    return *reinterpret_cast<const uint32_t*>(&h);
}

} // namespace tc

// ----- inference: the forward pass over one tile --------------------------------------------------------
struct __align__(128) MlpFwdSmem {
    uint16_t a1[2][MLP_TILE * MLP_FP]; // layer-1 A: standardised features (two buffers for streamed tiles)
    uint16_t a2[MLP_TILE * MLP_H];     // layer-2 A: hidden layer 1
    uint16_t w1[MLP_H * MLP_FP];
    uint16_t w2[MLP_H * MLP_H];
    float b1[MLP_H], b2[MLP_H], w3[MLP_H], mu[MLP_FP], isd[MLP_FP];
    float b3;
    uint64_t bar;      // tensor-core completion
    uint64_t ldbar[2]; // bulk-copy completion of a1[0], a1[1]
    uint32_t tmem;
};
// Bytes of one streamed layer-1 tile (128 rows x 16 BF16 in the K-major layout)
constexpr uint32_t MLP_A1_TILE_BYTES = MLP_TILE * MLP_FP * 2;
constexpr uint32_t MLP_FWD_TMEM_COLS = 64;

// All 128 threads: stage the weights, set up the barrier, allocate TMEM.
__device__ __forceinline__ void mlp_fwd_setup(MlpFwdSmem& S, const MlpDev* __restrict__ m)
{
    const int t = threadIdx.x;
    const uint4* w1s = reinterpret_cast<const uint4*>(m->w1);
    const uint4* w2s = reinterpret_cast<const uint4*>(m->w2);
    uint4* w1d       = reinterpret_cast<uint4*>(S.w1);
    uint4* w2d       = reinterpret_cast<uint4*>(S.w2);
    for (int q = t; q < MLP_H * MLP_FP / 8; q += MLP_TILE) { w1d[q] = w1s[q]; }
    for (int q = t; q < MLP_H * MLP_H / 8; q += MLP_TILE) { w2d[q] = w2s[q]; }
    if (t < MLP_H) {
        S.b1[t] = m->b1[t];
        S.b2[t] = m->b2[t];
        S.w3[t] = m->w3[t];
    }
    if (t < MLP_FP) {
        S.mu[t]  = m->mu[t];
        S.isd[t] = m->isd[t];
    }
    if (t == 0) {
        S.b3 = m->b3;
        tc::mbar_init(&S.bar, 1);
        tc::mbar_init(&S.ldbar[0], 1);
        tc::mbar_init(&S.ldbar[1], 1);
    }
    if (t < 32) { tc::tmem_alloc(&S.tmem, MLP_FWD_TMEM_COLS); }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
}

__device__ __forceinline__ void mlp_fwd_teardown(MlpFwdSmem& S)
{
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after();
        tc::tmem_dealloc(S.tmem, MLP_FWD_TMEM_COLS);
    }
}

// The standardised features of one row as its two 16-byte chunks of the layer-1 A tile (k = 0..7, 8..15).
__device__ __forceinline__ void mlp_pack_row(const float (&f)[MLP_F], const float* mu, const float* isd, uint4& c0,
                                             uint4& c1)
{
    float z[MLP_FP];
#pragma unroll
    for (int q = 0; q < MLP_FP; ++q) { z[q] = q < MLP_F ? (f[q < MLP_F ? q : 0] - mu[q]) * isd[q] : 0.f; }
    c0.x = tc::pack_bf16(z[0], z[1]);
    c0.y = tc::pack_bf16(z[2], z[3]);
    c0.z = tc::pack_bf16(z[4], z[5]);
    c0.w = tc::pack_bf16(z[6], z[7]);
    c1.x = tc::pack_bf16(z[8], z[9]);
    c1.y = tc::pack_bf16(z[10], z[11]);
    c1.z = tc::pack_bf16(z[12], z[13]);
    c1.w = tc::pack_bf16(z[14], z[15]);
}

__device__ __forceinline__ float mlp_fwd_core(MlpFwdSmem& S, int buf, uint32_t& phase, bool& ok);

// Every thread of the CTA: the standardised network output for this thread's features f (any values for
// rows without a sample). `phase` is the barrier parity, flipped per wait; `ok` turns false on a timeout.
__device__ __forceinline__ float mlp_fwd_tile(MlpFwdSmem& S, const float (&f)[MLP_F], uint32_t& phase, bool& ok)
{
    const uint32_t r = threadIdx.x;
    uint4 c0, c1;
    mlp_pack_row(f, S.mu, S.isd, c0, c1);
    *reinterpret_cast<uint4*>(&S.a1[0][kmajor(r, 0, MLP_FP)]) = c0;
    *reinterpret_cast<uint4*>(&S.a1[0][kmajor(r, 8, MLP_FP)]) = c1;
    tc::fence_async_smem();
    __syncthreads();
    return mlp_fwd_core(S, 0, phase, ok);
}

// The two layers from a layer-1 tile already in S.a1[buf] (written and fenced, or landed by a bulk copy whose
// barrier every thread has passed).
__device__ __forceinline__ float mlp_fwd_core(MlpFwdSmem& S, int buf, uint32_t& phase, bool& ok)
{
    const uint32_t r = threadIdx.x;
    constexpr uint32_t ID = tc::idesc_bf16(128, 64);
    if (r == 0) {
        tc::fence_after();
        tc::mma(S.tmem, tc::sdesc(tc::saddr(S.a1[buf]), 128, MLP_FP * 16),
                tc::sdesc(tc::saddr(S.w1), 128, MLP_FP * 16), ID, 0u);
        tc::commit(&S.bar);
    }
    ok = tc::mbar_wait(&S.bar, phase) && ok;
    phase ^= 1u;
    tc::fence_after();
    // hidden layer 1 -> layer-2 A row (64 BF16 = eight chunks)
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        float z[16];
        tc::ld16(tc::lane_addr(S.tmem, 16u * g), z);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            float a[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { a[q] = fmaxf(z[8 * c + q] + S.b1[16 * g + 8 * c + q], 0.f); }
            uint4 u;
            u.x = tc::pack_bf16(a[0], a[1]);
            u.y = tc::pack_bf16(a[2], a[3]);
            u.z = tc::pack_bf16(a[4], a[5]);
            u.w = tc::pack_bf16(a[6], a[7]);
            *reinterpret_cast<uint4*>(&S.a2[kmajor(r, 16 * g + 8 * c, MLP_H)]) = u;
        }
    }
    tc::fence_before();
    tc::fence_async_smem();
    __syncthreads();
    if (r == 0) {
        tc::fence_after();
#pragma unroll
        for (uint32_t s = 0; s < 4; ++s) {
            tc::mma(S.tmem, tc::sdesc(tc::saddr(S.a2) + 256u * s, 128, MLP_H * 16),
                    tc::sdesc(tc::saddr(S.w2) + 256u * s, 128, MLP_H * 16), ID, s > 0 ? 1u : 0u);
        }
        tc::commit(&S.bar);
    }
    ok = tc::mbar_wait(&S.bar, phase) && ok;
    phase ^= 1u;
    tc::fence_after();
    float y = S.b3;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        float z[16];
        tc::ld16(tc::lane_addr(S.tmem, 16u * g), z);
#pragma unroll
        for (int q = 0; q < 16; ++q) { y = fmaf(fmaxf(z[q] + S.b2[16 * g + q], 0.f), S.w3[16 * g + q], y); }
    }
    tc::fence_before(); // the next tile's MMA overwrites these columns after a barrier
    return y;
}

} // namespace gpe
