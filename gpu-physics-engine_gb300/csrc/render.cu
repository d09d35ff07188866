// render.cu — headless particle splat rasteriser: the reference's render path without D3D12
// (backgroundKernel and drawKernel, libs/render/source/cuda-render.cu:214-310, launched by launchFill
// :189-213), drawing a published view into a pitched RGBA8 device image.
//
// The reference blends every splat into the image with an unsynchronised read-modify-write per pixel
// (drawKernel, :296-307), so overlapping splats of concurrent threads can overwrite each other and the
// image depends on scheduling. Every splat has the same colour and alpha, so the sequential result depends
// only on how many splats cover a pixel: blending k times is f^k(background) with f the reference's
// alpha() (:244-258). Here a first pass counts the coverage of each pixel with atomics and a second pass
// shades each pixel by applying f that many times, so the image is the sequential one, bit for bit and
// independent of scheduling.
#include <cuda_runtime.h>

#include "gpe_internal.h"

namespace gpe {
namespace {

constexpr int SPLAT_R = 2; // the 5 x 5 footprint without its corners (:293-307)
constexpr uint8_t SPLAT_RGB[3] = {140u, 210u, 255u};
constexpr uint8_t SPLAT_A      = 100u;

// alpha(over, under) of the reference for one channel, in its operation order without contraction
__device__ __forceinline__ uint8_t blend(uint8_t over, uint8_t under, float a, float ia)
{
    const float s = __fadd_rn(__fadd_rn(__fmul_rn((float)over, a), __fmul_rn((float)under, ia)), 0.5f);
    return (uint8_t)s;
}

__global__ void k_splat_count(const gpe_view* __restrict__ vp, gpe_view vv, int32_t* __restrict__ cover,
                              int32_t width, int32_t height, float scale)
{
    const gpe_view view = vp ? *vp : vv;
    const int32_t chunk = blockIdx.y;
    if (chunk >= view.chunks_x * view.chunks_y) { return; }
    const int32_t n = min(view.counts[chunk], view.chunk_capacity);
    for (int32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
        const float2 p   = reinterpret_cast<const float2*>(view.pos)[(size_t)chunk * view.chunk_capacity + a];
        const int32_t px = (int32_t)(p.x * scale); // truncation, as (int32_t)(p.x * kSimScale) at :284
        const int32_t py = (int32_t)(p.y * scale);
        if (px < 0 || py < 0 || px >= width || py >= height) { continue; }
        for (int32_t i = -SPLAT_R; i <= SPLAT_R; ++i) {
            const int32_t y = py + i;
            if (y < 0 || y >= height) { continue; }
            for (int32_t j = -SPLAT_R; j <= SPLAT_R; ++j) {
                const int32_t x = px + j;
                if (x < 0 || x >= width || (abs(i) == SPLAT_R && abs(j) == SPLAT_R)) { continue; }
                atomicAdd(&cover[(size_t)y * width + x], 1);
            }
        }
    }
}

// Background (chunk grid lines or the vertical gradient, :224-242), then the splat blend applied as many
// times as the pixel is covered; f reaches its fixed point long before large counts, so the loop stops there.
__global__ void k_shade(uint8_t* __restrict__ rgba, int64_t pitch, const int32_t* __restrict__ cover, int32_t width,
                        int32_t height, int32_t line_every)
{
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= width || y >= height) { return; }
    uint8_t r, g, b;
    if (x % line_every == 0 || y % line_every == 0) {
        r = g = b = 0u;
    } else {
        const float t = __fmul_rn(100.f, __fdiv_rn((float)y, (float)height));
        r             = (uint8_t)(255u - (uint8_t)t);
        g             = (uint8_t)(160u - (uint8_t)t);
        b             = 80u;
    }
    const float a  = __fmul_rn((float)SPLAT_A, 1.f / 255.f);
    const float ia = __fsub_rn(1.f, a);
    const int32_t k = cover[(size_t)y * width + x];
    for (int32_t s = 0; s < k; ++s) {
        const uint8_t r2 = blend(SPLAT_RGB[0], r, a, ia);
        const uint8_t g2 = blend(SPLAT_RGB[1], g, a, ia);
        const uint8_t b2 = blend(SPLAT_RGB[2], b, a, ia);
        if (r2 == r && g2 == g && b2 == b) { break; } // fixed point: further splats change nothing
        r = r2;
        g = g2;
        b = b2;
    }
    uchar4* row = reinterpret_cast<uchar4*>(rgba + (size_t)y * (size_t)pitch);
    row[x]      = make_uchar4(r, g, b, 255u);
}

} // namespace
} // namespace gpe

using namespace gpe;

extern "C" int32_t gpe_render_frame(const gpe_raster* r, const gpe_view* view, int32_t view_mem, void* stream)
{
    gpe::clear_error();
    if (!r || !view || !r->rgba || !r->coverage || r->width <= 0 || r->height <= 0 ||
        r->pitch < 4 * (int64_t)r->width || !(r->scale > 0.f) || !(r->chunk_dim > 0.f) ||
        (view_mem != GPE_MEM_HOST && view_mem != GPE_MEM_DEVICE)) {
        return GPE_ERR_BAD_ARG;
    }
    const int32_t line_every = (int32_t)(r->chunk_dim * r->scale); // (int32_t)(kChunkDim * kSimScale), :228
    if (line_every <= 0) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st     = as_stream(stream);
    const gpe_view* vp  = view_mem == GPE_MEM_DEVICE ? view : nullptr;
    gpe_view vv{};
    int32_t chunks = 0;
    if (view_mem == GPE_MEM_HOST) {
        vv = *view;
        if (!vv.pos || !vv.counts || vv.chunks_x <= 0 || vv.chunks_y <= 0 || vv.chunk_capacity <= 0) {
            return GPE_ERR_BAD_ARG;
        }
        chunks = vv.chunks_x * vv.chunks_y;
    } else {
        gpe_view hv{};
        GPE_TRY_CUDA(cudaMemcpyAsync(&hv, view, sizeof(hv), cudaMemcpyDeviceToHost, st));
        GPE_TRY_CUDA(cudaStreamSynchronize(st));
        chunks = hv.chunks_x * hv.chunks_y;
    }
    GPE_TRY_CUDA(cudaMemsetAsync(r->coverage, 0, sizeof(int32_t) * (size_t)r->width * (size_t)r->height, st));
    if (chunks > 0) {
        k_splat_count<<<dim3(4, (unsigned)chunks), 256, 0, st>>>(vp, vv, r->coverage, r->width, r->height, r->scale);
        GPE_CHECK_LAUNCH("k_splat_count");
    }
    const dim3 blk(32, 8);
    k_shade<<<dim3((unsigned)((r->width + 31) / 32), (unsigned)((r->height + 7) / 8)), blk, 0, st>>>(
        r->rgba, r->pitch, r->coverage, r->width, r->height, line_every);
    GPE_CHECK_LAUNCH("k_shade");
    return GPE_OK;
}
