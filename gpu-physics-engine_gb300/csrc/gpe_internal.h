// gpe_internal.h — shared host/device helpers of the engine (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/gpe.h"

namespace gpe {

// ----- error plumbing (thread-local, like the reference's last_error in cuda-render.cu:20-27) -----
void set_error(int32_t status, const char* fmt, ...);
void set_cuda_error(cudaError_t e, const char* what);
void clear_error();

#define GPE_TRY_CUDA(expr)                                                                                 \
    do {                                                                                                   \
        cudaError_t e_ = (expr);                                                                           \
        if (e_ != cudaSuccess) {                                                                           \
            ::gpe::set_cuda_error(e_, #expr);                                                              \
            return GPE_ERR_CUDA;                                                                           \
        }                                                                                                  \
    } while (0)

#define GPE_CHECK_LAUNCH(name)                                                                             \
    do {                                                                                                   \
        cudaError_t e_ = cudaGetLastError();                                                               \
        if (e_ != cudaSuccess) {                                                                           \
            ::gpe::set_cuda_error(e_, name);                                                               \
            return GPE_ERR_CUDA;                                                                           \
        }                                                                                                  \
    } while (0)

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) & ~(a - 1); }

// Bump allocator over one device allocation (the reference carves each arena out of one cudaMalloc at
// 128 B alignment, cuda-engine.cpp:14-29; 256 B here so every array can be a TMA or vector base).
struct Carver {
    size_t off = 0;
    template <class T>
    size_t take(size_t count)
    {
        const size_t o = off;
        off            = align_up(off + sizeof(T) * (count ? count : 1), 256);
        return o;
    }
};

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int32_t current_device(int* dev);
int32_t sm_count();

// ----- counting sort of 32-bit keys (shared by PBF and the MPM spatial sort) -----
// Workspace sizes for a sort of up to n_max items into n_keys buckets.
size_t scan_blocks(uint32_t n_keys);
// count[n_keys] -> start[n_keys+1] exclusive scan; zeroes count (and zero_bytes[n_keys] when given). bsum
// needs scan_blocks(n_keys) entries.
int32_t launch_exclusive_scan(uint32_t* count, uint32_t n_keys, uint32_t* bsum, uint32_t* start,
                              cudaStream_t st, uint8_t* zero_bytes = nullptr);
// kernel launches of launch_exclusive_scan for n_keys buckets (2, or 3 beyond 2048 tiles)
int32_t scan_launches(uint32_t n_keys);
// bucket[start[key] + rank] = i for every (key, rank) pair. n sizes the launch; with n_dev the kernel takes
// the live count from the device (which must not exceed n).
int32_t launch_scatter(const uint2* keyrank, int64_t n, const uint32_t* start, uint32_t* bucket, uint32_t ncells,
                       cudaStream_t st, const int32_t* n_dev = nullptr);


// ----- warm-start network (mlp.cu) as the PBF engine sees it -----
struct MlpDev;
// Pair set of a network: features [cap][12] and targets [cap]; idx = the particle's sorted index when the
// pair was taken; cnt[0] = pairs written (appended with atomics), cnt[1] = pairs whose target is written.
struct MlpData {
    float* X;
    float* T;
    int32_t* idx;
    int32_t* cnt;
    int64_t cap;
};
const MlpDev* mlp_device(const gpe_mlp* m);
MlpData mlp_data(gpe_mlp* m);
// iterations per step of the plain solve whose pairs the network learned (20 unless collected otherwise)
int32_t mlp_pair_iters(const gpe_mlp* m);
void mlp_set_pair_iters(gpe_mlp* m, int32_t iters);

#if defined(__CUDACC__)
// Packed FP32 pairs (sm_100 and later): two IEEE round-to-nearest operations in one instruction, with the
// same results as the scalar forms component by component.
__device__ __forceinline__ float2 sub2(const float2 a, const float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "sub.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 fma2(const float2 a, const float2 b, const float2 c)
{
    float2 d;
    asm("{\n\t.reg .b64 a, b, c, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tmov.b64 c, {%6, %7};\n\t"
        "fma.rn.f32x2 d, a, b, c;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

__device__ __forceinline__ float2 add2(const float2 a, const float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "add.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mul2(const float2 a, const float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "mul.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
#endif

} // namespace gpe
