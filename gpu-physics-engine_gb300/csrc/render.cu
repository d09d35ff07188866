// render.cu — headless particle splat rasteriser: the reference's render path without D3D12
// (backgroundKernel and drawKernel, libs/render/source/cuda-render.cu:214-310, launched by launchFill
// :189-213), drawing a published view into a pitched RGBA8 device image.
//
// The reference blends every splat into the image with an unsynchronised read-modify-write per pixel
// (drawKernel, :296-307), so overlapping splats of concurrent threads can overwrite each other and the
// image depends on scheduling. Every splat has the same colour and alpha, so the sequential result depends
// only on how many splats cover a pixel: blending k times is f^k(background) with f the reference's
// alpha() (:244-258). Here a first pass counts, with one atomic per particle, the splats centred on each
// pixel; a second pass sums those counts over the footprint around each pixel (integer sums, exact) and
// shades the pixel by applying f that many times, so the image is the sequential one, bit for bit and
// independent of scheduling.
#include <cuda_runtime.h>

#include <algorithm>

#include "gpe_internal.h"

namespace gpe {
namespace {

constexpr int SPLAT_R = 2; // the 5 x 5 footprint without its corners (:293-307)
constexpr uint8_t SPLAT_R8 = 140u, SPLAT_G8 = 210u, SPLAT_B8 = 255u;
constexpr uint8_t SPLAT_A      = 100u;

// alpha(over, under) of the reference for one channel, in its operation order without contraction
__device__ __forceinline__ uint8_t blend(uint8_t over, uint8_t under, float a, float ia)
{
    const float s = __fadd_rn(__fadd_rn(__fmul_rn((float)over, a), __fmul_rn((float)under, ia)), 0.5f);
    return (uint8_t)s;
}

// Applications of f after which every channel sits at its fixed point, from any start byte: at most 11 for
// the splat colour (140, 210, 255) at alpha 100 (every start 0..255 iterated on the host); the table keeps
// 16 entries and f^k = f^15 for k >= 15.
constexpr int32_t BLEND_K = 16;
// The gradient background of a row is (255 - t, 160 - t, 80) with t = (uint8)(100 y / height) in 0..100;
// row BLEND_BLACK of the table starts from the grid lines' black.
constexpr int32_t BLEND_ROWS = 102, BLEND_BLACK = 101;

// f^k of every background, k = 0..15: the same for every frame and image size. Rebuilt by every frame's
// splat pass (identical bytes), so a frame never reads it before it exists.
__device__ uchar4 g_blend[BLEND_ROWS][BLEND_K];

__device__ __forceinline__ void build_blend_row(int32_t row)
{
    const float a  = __fmul_rn((float)SPLAT_A, 1.f / 255.f);
    const float ia = __fsub_rn(1.f, a);
    const uint8_t t = (uint8_t)min(row, 100);
    uchar4 c = row == BLEND_BLACK ? make_uchar4(0u, 0u, 0u, 255u)
                                  : make_uchar4((uint8_t)(255u - t), (uint8_t)(160u - t), 80u, 255u);
    g_blend[row][0] = c;
    for (int32_t k = 1; k < BLEND_K; ++k) {
        c.x             = blend(SPLAT_R8, c.x, a, ia);
        c.y             = blend(SPLAT_G8, c.y, a, ia);
        c.z             = blend(SPLAT_B8, c.z, a, ia);
        g_blend[row][k] = c;
    }
}

// One atomic per particle: the number of particles whose splat is centred on each pixel. Particles whose
// centre pixel lies outside the image draw nothing (the reference's early continue, :286-287). Block (0, 0)
// also writes the blend table.
__global__ void k_splat_point(const gpe_view* __restrict__ vp, gpe_view vv, int32_t* __restrict__ centres,
                              int32_t width, int32_t height, float scale)
{
    if (blockIdx.x == 0 && blockIdx.y == 0) {
        for (int32_t row = threadIdx.x; row < BLEND_ROWS; row += blockDim.x) { build_blend_row(row); }
    }
    const gpe_view view = vp ? *vp : vv;
    const int32_t chunks = view.chunks_x * view.chunks_y;
    for (int32_t chunk = blockIdx.y; chunk < chunks; chunk += gridDim.y) {
        const int32_t n                = min(view.counts[chunk], view.chunk_capacity);
        const float2* __restrict__ pos = reinterpret_cast<const float2*>(view.pos) + (size_t)chunk * view.chunk_capacity;
        for (int32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
            const float2 p   = pos[a];
            const int32_t px = (int32_t)(p.x * scale); // truncation, as (int32_t)(p.x * kSimScale) at :284
            const int32_t py = (int32_t)(p.y * scale);
            if (px < 0 || py < 0 || px >= width || py >= height) { continue; }
            atomicAdd(&centres[(size_t)py * width + px], 1);
        }
    }
}

constexpr int32_t SH_TW = 32, SH_ROWS = 8, SH_THREADS = 256; // a 32 x 8 block shades a 32 x 64 tile, 8 rows a thread
constexpr int32_t SH_TH = SH_ROWS * SH_THREADS / SH_TW;
constexpr int32_t SH_HW = SH_TW + 2 * SPLAT_R, SH_HH = SH_TH + 2 * SPLAT_R;

// The coverage of a pixel is the sum of the centre counts over the footprint around it: rows +-2 over
// columns +-1, rows -1..1 over columns +-2 (the 21 pixels of the 5 x 5 square without its corners). The
// centre counts of the tile and a 2-pixel halo are staged in shared memory, each thread keeps the 3- and
// 5-wide row sums of its 8 + 4 rows in registers. A pixel covered k times gets f^k(background) with f the
// reference's blend: the table row of its background (the chunk grid lines' black, or the row's gradient
// value, :224-242) at min(k, 15).
__global__ void __launch_bounds__(SH_THREADS)
    k_shade(uint8_t* __restrict__ rgba, int64_t pitch, const int32_t* __restrict__ centres, int32_t width,
            int32_t height, int32_t line_every)
{
    __shared__ int32_t t[SH_HH][SH_HW];
    __shared__ int32_t rowsel[SH_TH]; // table row of each tile row's background, grid columns aside
    const int32_t x0 = blockIdx.x * SH_TW, y0 = blockIdx.y * SH_TH;
    const int32_t tid = threadIdx.y * SH_TW + threadIdx.x;
    for (int32_t i = tid; i < SH_HH * SH_HW; i += SH_THREADS) {
        const int32_t ty = i / SH_HW, tx = i - ty * SH_HW;
        const int32_t gx = x0 + tx - SPLAT_R, gy = y0 + ty - SPLAT_R;
        t[ty][tx]        = (gx >= 0 && gy >= 0 && gx < width && gy < height) ? centres[(size_t)gy * width + gx] : 0;
    }
    if (tid < SH_TH) {
        const int32_t y = y0 + tid;
        rowsel[tid]     = y % line_every == 0 ? BLEND_BLACK
                                              : (int32_t)(uint8_t)__fmul_rn(100.f, __fdiv_rn((float)y, (float)height));
    }
    __syncthreads();
    const int32_t tx = threadIdx.x, ty0 = threadIdx.y * SH_ROWS;
    int32_t h3[SH_ROWS + 2 * SPLAT_R], h5[SH_ROWS + 2 * SPLAT_R];
#pragma unroll
    for (int32_t r = 0; r < SH_ROWS + 2 * SPLAT_R; ++r) {
        const int32_t* row = t[ty0 + r] + tx;
        h3[r]              = row[1] + row[2] + row[3];
        h5[r]              = h3[r] + row[0] + row[4];
    }
    const int32_t x = x0 + tx;
    if (x >= width) { return; }
    const bool xline = x % line_every == 0;
    uint8_t* out     = rgba + (size_t)(y0 + ty0) * (size_t)pitch + 4 * (size_t)x;
#pragma unroll
    for (int32_t j = 0; j < SH_ROWS; ++j) {
        if (y0 + ty0 + j >= height) { break; }
        const int32_t k  = min(h3[j] + h5[j + 1] + h5[j + 2] + h5[j + 3] + h3[j + 4], BLEND_K - 1);
        const int32_t sr = xline ? BLEND_BLACK : rowsel[ty0 + j];
        *reinterpret_cast<uchar4*>(out + (size_t)j * (size_t)pitch) = g_blend[sr][k];
    }
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
    // grid rows walk the chunks: one row a chunk for a host view; a device view is read only by the kernel
    // (its chunk count may change between replays of a captured frame), so a fixed 64 rows stride over them
    int32_t rows = 64;
    if (view_mem == GPE_MEM_HOST) {
        vv = *view;
        if (!vv.pos || !vv.counts || vv.chunks_x <= 0 || vv.chunks_y <= 0 || vv.chunk_capacity <= 0) {
            return GPE_ERR_BAD_ARG;
        }
        rows = (int32_t)std::min<int64_t>((int64_t)vv.chunks_x * vv.chunks_y, 65535);
    }
    GPE_TRY_CUDA(cudaMemsetAsync(r->coverage, 0, sizeof(int32_t) * (size_t)r->width * (size_t)r->height, st));
    {
        // about 32 blocks of 256 per SM: one particle a thread for a million particles
        const int32_t cols = max(1, (int32_t)std::min<int64_t>((32 * sm_count() + rows - 1) / rows, 65535));
        k_splat_point<<<dim3((unsigned)cols, (unsigned)rows), 256, 0, st>>>(vp, vv, r->coverage, r->width, r->height,
                                                                           r->scale);
        GPE_CHECK_LAUNCH("k_splat_point");
    }
    const dim3 blk(SH_TW, SH_THREADS / SH_TW);
    k_shade<<<dim3((unsigned)((r->width + SH_TW - 1) / SH_TW), (unsigned)((r->height + SH_TH - 1) / SH_TH)), blk, 0, st>>>(
        r->rgba, r->pitch, r->coverage, r->width, r->height, line_every);
    GPE_CHECK_LAUNCH("k_shade");
    return GPE_OK;
}
