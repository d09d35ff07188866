// emit.cuh — hose-pipe particle source shared by the PBF and MPM emitters (device code).
//
// The lattice layout and the jitter follow the reference's emitterKernel (PBF.cu:984-1011) and
// MPMEmitterKernel (MPM.cu:398-421): particle i sits in column i % width and row i / width behind the nozzle,
// across = (col - (width-1)/2) * spacing, along = -(row + 1/2) * spacing in the frame of the flow direction,
// and is jittered by a Gaussian pair from curand's Philox generator initialised with (seed, i, 0).
#pragma once

#include <curand_kernel.h>

#include <algorithm>
#include <climits>
#include <cmath>

#include "gpe_internal.h"

namespace gpe {

struct HoseK {
    float ox, oy;   // nozzle centre
    float tx, ty;   // unit flow direction
    float nx, ny;   // unit normal (-t.y, t.x)
    float vx, vy;   // particle velocity
    float spacing, jitter;
    int32_t width, count;
    unsigned long long seed;
};

// Host: the hose's geometry; returns the requested count (width x rows), or -1 when width, rows or their
// product is not finite or exceeds INT32_MAX (the emitters then refuse the call with GPE_ERR_CAPACITY).
inline int32_t make_hose(const gpe_hose& h, float dt, uint64_t seed, HoseK* k)
{
    const float speed = std::sqrt(h.velocity[0] * h.velocity[0] + h.velocity[1] * h.velocity[1]);
    // width and rows as the reference rounds them (lround of the float quotients), range-checked in double
    const double wq = std::nearbyint((double)(h.nozzle_width / h.spacing));
    const double rq = std::nearbyint((double)(speed * dt * (float)h.steps_per_call / h.spacing));
    if (!(wq < 2147483647.0) || !(rq < 2147483647.0)) { return -1; } // also refuses NaN
    const int64_t w = std::max<int64_t>(1, (int64_t)std::lround(h.nozzle_width / h.spacing));
    const int64_t r = std::max<int64_t>(1, (int64_t)std::lround(speed * dt * (float)h.steps_per_call / h.spacing));
    if (w * r > (int64_t)INT32_MAX) { return -1; }
    const float inv   = speed > 1e-6f ? 1.f / speed : 0.f;
    k->ox             = h.origin[0];
    k->oy             = h.origin[1];
    k->tx             = h.velocity[0] * inv;
    k->ty             = h.velocity[1] * inv;
    k->nx             = -k->ty;
    k->ny             = k->tx;
    k->vx             = h.velocity[0];
    k->vy             = h.velocity[1];
    k->spacing        = h.spacing;
    k->jitter         = h.jitter;
    k->width          = (int32_t)w;
    k->count          = (int32_t)(w * r);
    k->seed           = (unsigned long long)seed;
    return k->count;
}

#ifdef __CUDACC__
__device__ __forceinline__ float2 hose_position(const HoseK& h, int32_t i)
{
    const int32_t col  = i % h.width;
    const int32_t row  = i / h.width;
    const float across = ((float)col - 0.5f * (float)(h.width - 1)) * h.spacing;
    const float along  = -((float)row + 0.5f) * h.spacing;
    float2 p = make_float2(h.ox + h.nx * across + h.tx * along, h.oy + h.ny * across + h.ty * along);
    if (h.jitter > 0.f) {
        curandStatePhilox4_32_10_t rng;
        curand_init(h.seed, (unsigned long long)i, 0ull, &rng);
        const float2 j2 = curand_normal2(&rng);
        p.x += j2.x * h.jitter;
        p.y += j2.y * h.jitter;
    }
    return p;
}

// Appends one slot per calling lane that passes `take`, with one atomic per warp; returns the slot or -1.
__device__ __forceinline__ int32_t append_slot(int32_t* count, bool take)
{
    const uint32_t active = __activemask();
    const uint32_t want   = __ballot_sync(active, take);
    const int32_t lane    = threadIdx.x & 31;
    const int32_t leader  = __ffs(want) - 1;
    int32_t base          = 0;
    if (want && lane == leader) { base = atomicAdd(count, __popc(want)); }
    if (!want) { return -1; }
    base = __shfl_sync(active, base, leader);
    return take ? base + __popc(want & ((1u << lane) - 1u)) : -1;
}
#endif

} // namespace gpe
