// sort.cu — the device-wide pieces of the cell counting sort: exclusive scan of the cell histogram and the
// scatter of (cell, rank) pairs into cell buckets.
//
// The reference sorts each 16x16-cell chunk inside one block: a shared-memory histogram by atomicAdd
// (PBF.cu:786-797), a 256-wide scan incPrefSum256 (PBF.cu:835-860) and a shared-memory scatter
// (PBF.cu:806-833). Chunks here are not bounded by shared memory (a scene holds up to millions of
// particles and cells), so the histogram and the scan run device-wide: the histogram is fused into the
// predict kernel (pbf.cu), the scan below is a reduce / down-sweep over tiles of 2048 cells (with a
// scan-of-block-sums launch in between for more than 2048 tiles), and the stable placement is finished by
// pbf.cu's gather kernel.
#include "gpe_internal.h"

namespace gpe {

namespace {

constexpr int SCAN_T    = 256;
constexpr int SCAN_I    = 8;
constexpr int SCAN_TILE = SCAN_T * SCAN_I;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) { v += t; }
    }
    return v;
}

// exclusive scan of one value per thread across a 256-thread block; returns the block total in *total
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t s_warp[SCAN_T / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(v);
    if (lane == 31) { s_warp[warp] = inc; }
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < SCAN_T / 32 ? s_warp[lane] : 0u;
        w          = warp_incl_scan(w);
        if (lane < SCAN_T / 32) { s_warp[lane] = w; }
    }
    __syncthreads();
    const uint32_t before = warp ? s_warp[warp - 1] : 0u;
    *total                = s_warp[SCAN_T / 32 - 1];
    __syncthreads();
    return before + inc - v;
}

// VEC: M is a multiple of 4 and count is 16-byte aligned (four cells per load)
template <bool VEC>
__global__ void __launch_bounds__(SCAN_T) k_scan_reduce(const uint32_t* __restrict__ count, uint32_t M,
                                                        uint32_t* __restrict__ bsum)
{
    const uint32_t base = blockIdx.x * SCAN_TILE;
    uint32_t s          = 0;
    if constexpr (VEC) {
#pragma unroll
        for (int t = 0; t < SCAN_I / 4; ++t) {
            const uint32_t idx = base + 4u * (t * SCAN_T + threadIdx.x);
            if (idx < M) {
                const uint4 c = *reinterpret_cast<const uint4*>(count + idx);
                s += (c.x + c.y) + (c.z + c.w);
            }
        }
    } else {
#pragma unroll
        for (int t = 0; t < SCAN_I; ++t) {
            const uint32_t idx = base + t * SCAN_T + threadIdx.x;
            if (idx < M) { s += count[idx]; }
        }
    }
    uint32_t total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) { bsum[blockIdx.x] = total; }
}

// one block: in-place exclusive scan of the block sums
__global__ void __launch_bounds__(SCAN_T) k_scan_bsum(uint32_t* __restrict__ bsum, uint32_t nb)
{
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += SCAN_T) {
        const uint32_t idx = base + threadIdx.x;
        const uint32_t v   = idx < nb ? bsum[idx] : 0u;
        uint32_t total;
        const uint32_t ex = block_excl_scan(v, &total);
        if (idx < nb) { bsum[idx] = carry + ex; }
        carry += total;
    }
}

// SUMS: bsum holds the tiles' totals (not scanned) and each block adds up those before it itself, which
// saves the single-block scan launch while the tiles are few (FUSED_MAX_TILES); else bsum is already the
// exclusive scan of the totals.
constexpr uint32_t FUSED_MAX_TILES = 2048;

// VEC: M is a multiple of 4 and the arrays are 16-byte aligned (zero8: 4-byte), so each thread moves four
// cells per access; the per-thread runs of SCAN_I cells are then read from shared memory as 16-byte words
// (2-way bank conflicts instead of 8-way).
template <bool SUMS, bool VEC>
__global__ void __launch_bounds__(SCAN_T) k_scan_down(uint32_t* __restrict__ count, uint32_t M,
                                                      const uint32_t* __restrict__ bsum,
                                                      uint32_t* __restrict__ start, uint8_t* __restrict__ zero8)
{
    __shared__ __align__(16) uint32_t s_tile[SCAN_TILE];
    const uint32_t base = blockIdx.x * SCAN_TILE;
    uint32_t prefix;
    if (SUMS) {
        uint32_t part = 0;
        for (uint32_t b = threadIdx.x; b < blockIdx.x; b += SCAN_T) { part += bsum[b]; }
        block_excl_scan(part, &prefix);
    } else {
        prefix = bsum[blockIdx.x];
    }
    // coalesced load, and zero the histogram for the next sort
    if constexpr (VEC) {
#pragma unroll
        for (int t = 0; t < SCAN_I / 4; ++t) {
            const uint32_t li  = 4u * (t * SCAN_T + threadIdx.x);
            const uint32_t idx = base + li;
            uint4 c            = make_uint4(0u, 0u, 0u, 0u);
            if (idx < M) {
                c                                        = *reinterpret_cast<const uint4*>(count + idx);
                *reinterpret_cast<uint4*>(count + idx)   = make_uint4(0u, 0u, 0u, 0u);
                if (zero8) { *reinterpret_cast<uint32_t*>(zero8 + idx) = 0u; }
            }
            *reinterpret_cast<uint4*>(s_tile + li) = c;
        }
    } else {
#pragma unroll
        for (int t = 0; t < SCAN_I; ++t) {
            const uint32_t li  = t * SCAN_T + threadIdx.x;
            const uint32_t idx = base + li;
            uint32_t c         = 0;
            if (idx < M) {
                c          = count[idx];
                count[idx] = 0u;
                if (zero8) { zero8[idx] = 0u; }
            }
            s_tile[li] = c;
        }
    }
    __syncthreads();
    // each thread owns SCAN_I consecutive cells
    uint32_t v[SCAN_I];
#pragma unroll
    for (int q = 0; q < SCAN_I / 4; ++q) {
        const uint4 w    = *reinterpret_cast<const uint4*>(s_tile + threadIdx.x * SCAN_I + 4 * q);
        v[4 * q + 0]     = w.x;
        v[4 * q + 1]     = w.y;
        v[4 * q + 2]     = w.z;
        v[4 * q + 3]     = w.w;
    }
    uint32_t s = 0;
#pragma unroll
    for (int t = 0; t < SCAN_I; ++t) {
        const uint32_t c = v[t];
        v[t]             = s;
        s += c;
    }
    uint32_t total;
    const uint32_t ex  = block_excl_scan(s, &total);
    const uint32_t off = prefix + ex;
#pragma unroll
    for (int q = 0; q < SCAN_I / 4; ++q) {
        *reinterpret_cast<uint4*>(s_tile + threadIdx.x * SCAN_I + 4 * q) =
            make_uint4(off + v[4 * q], off + v[4 * q + 1], off + v[4 * q + 2], off + v[4 * q + 3]);
    }
    __syncthreads();
    if constexpr (VEC) {
#pragma unroll
        for (int t = 0; t < SCAN_I / 4; ++t) {
            const uint32_t li  = 4u * (t * SCAN_T + threadIdx.x);
            const uint32_t idx = base + li;
            if (idx < M) { *reinterpret_cast<uint4*>(start + idx) = *reinterpret_cast<const uint4*>(s_tile + li); }
        }
    } else {
#pragma unroll
        for (int t = 0; t < SCAN_I; ++t) {
            const uint32_t li  = t * SCAN_T + threadIdx.x;
            const uint32_t idx = base + li;
            if (idx < M) { start[idx] = s_tile[li]; }
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) { start[M] = prefix + total; }
}

// The keys and ranks come from the same histogram as the starts; the bounds checks only keep an
// inconsistent pair (a caller's bug) from writing outside the arrays.
__global__ void k_scatter(const uint2* __restrict__ keyrank, int64_t n_host, const int32_t* __restrict__ n_dev,
                          const uint32_t* __restrict__ start, uint32_t* __restrict__ bucket, uint32_t ncells)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = n_dev ? (int64_t)__ldg(n_dev) : n_host;
    if (i >= n) { return; }
    const uint2 kr = keyrank[i];
    if (kr.x >= ncells) { return; }
    const uint32_t dst = __ldg(&start[kr.x]) + kr.y;
    if ((int64_t)dst < n) { bucket[dst] = (uint32_t)i; }
}

} // namespace

size_t scan_blocks(uint32_t n_keys) { return (n_keys + SCAN_TILE - 1) / SCAN_TILE; }

int32_t launch_exclusive_scan(uint32_t* count, uint32_t n_keys, uint32_t* bsum, uint32_t* start,
                              cudaStream_t st, uint8_t* zero_bytes)
{
    const uint32_t nb = (uint32_t)scan_blocks(n_keys);
    if (nb == 0) { return GPE_ERR_BAD_ARG; }
    const bool vec = n_keys % 4 == 0 && reinterpret_cast<uintptr_t>(count) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(start) % 16 == 0 && reinterpret_cast<uintptr_t>(zero_bytes) % 4 == 0;
    (vec ? k_scan_reduce<true> : k_scan_reduce<false>)<<<nb, SCAN_T, 0, st>>>(count, n_keys, bsum);
    GPE_CHECK_LAUNCH("k_scan_reduce");
    const bool sums = nb <= FUSED_MAX_TILES;
    if (!sums) {
        k_scan_bsum<<<1, SCAN_T, 0, st>>>(bsum, nb);
        GPE_CHECK_LAUNCH("k_scan_bsum");
    }
    auto down = sums ? (vec ? k_scan_down<true, true> : k_scan_down<true, false>)
                     : (vec ? k_scan_down<false, true> : k_scan_down<false, false>);
    down<<<nb, SCAN_T, 0, st>>>(count, n_keys, bsum, start, zero_bytes);
    GPE_CHECK_LAUNCH("k_scan_down");
    return GPE_OK;
}

int32_t scan_launches(uint32_t n_keys) { return scan_blocks(n_keys) <= FUSED_MAX_TILES ? 2 : 3; }

int32_t launch_scatter(const uint2* keyrank, int64_t n, const uint32_t* start, uint32_t* bucket, uint32_t ncells,
                       cudaStream_t st, const int32_t* n_dev)
{
    if (n <= 0) { return GPE_OK; }
    const int T = 256;
    k_scatter<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(keyrank, n, n_dev, start, bucket, ncells);
    GPE_CHECK_LAUNCH("k_scatter");
    return GPE_OK;
}

} // namespace gpe
