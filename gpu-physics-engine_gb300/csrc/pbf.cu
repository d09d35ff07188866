// pbf.cu — Position-Based Fluids step on GB300 (sm_103a).
//
// One step (the reference's substep, PBF.cu:921-956) is:
//   predict + key + histogram   k_predict_hist   (prepNextSubstepKernel PBF.cu:786-797, made device-wide)
//   scan / scatter              sort.cu          (incPrefSum256 PBF.cu:835-860)
//   stable placement + gather   k_place          (PBF.cu:801-833; stable here, the reference's intra-cell
//                                                  order follows shared-memory atomic order)
//   iters x (lambda, delta p)   k_lambda, k_delta_p (PBF.cu:215-308, 365-499)
//   velocity + XSPH (+omega)    k_xsph           (PBF.cu:500-638 fused: v_j = (x*_j - x_j)/dt on the fly)
//   vorticity confinement       k_vorticity      (Macklin & Mueller 2013; absent in the reference)
//
// Layout: structure-of-arrays in HBM, particles of all scenes in one array sorted by global cell key
// (scene-major, then row-major cells), so a row of neighbour cells is one contiguous index range. Within a
// step each particle is held as its start position x and its displacement d = x* - x (one float4): the
// neighbour offset x*_i - x*_j = (x_i - x_j) + (d_i - d_j) and the velocity d / dt then keep FP32 precision
// relative to themselves, whatever the magnitude of the scene coordinates. The
// reference's per-chunk shared-memory pools, 1-cell halo copies and migration queues exist because a block
// of its design must hold a whole chunk; with a device-wide sort every scene is one domain, neighbours
// across what were chunk borders are read in place from L2, and a particle that crosses a border simply
// lands in another cell range at the next sort.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "emit.cuh"
#include "gpe_internal.h"
#include "mlp.cuh"

namespace gpe {

struct DomDev {
    float ox, oy;             // sort-grid origin (the scene's lower corner)
    float lox, loy, hix, hiy; // wall clamp box (handleOOB, PBF.cu:487-490)
    int32_t ncx, ncy;         // cells
    uint32_t coff;            // first global cell of the scene
    uint32_t pad[3];
};

struct PbfK {
    float h, h2, c6, cs, inv_w_dq, inv_cell;
    float rho0, inv_rho0, mass, inv_mass;
    float dt, inv_dt, g2x, g2y;
    float eps, scorr_k, dp_scale, c_min, xsph_c, vort_eps, v_max, v_min2, vort_dt;
    int32_t R;
    uint32_t flags;
    float margin;             // wall margin (positions stay below the box's upper edge by this much)
    int32_t n;                // particle count when n_dev is null
    const int32_t* n_dev;     // device-resident particle count (emitters append on the device)
    DomDev d0; // the scene when there is only one
    // candidate masks (cell h only): per particle the candidates within h + skin, per cell a mark that a
    // particle of the 3 x 3 cells around it moved too far for them
    const uint32_t* keys;     // sort cell of each slot
    uint4* nmask;
    uint8_t* mflag;
    float skin2;              // (h + skin)^2
    float move2;              // (skin / (2 iters))^2, shrunk by 1%
    // set for the XSPH pass of a step that also computes the next step's predicted cell keys and their
    // histogram (from the positions and velocities it writes); null otherwise
    uint2* hist_kr;
    uint32_t* hist_cnt;
    uint32_t ncells;          // sort cells of all scenes (the placement's bounds checks)
};


namespace {

constexpr int T_PART = 256; // threads per block for the per-particle kernels
constexpr int T_MAX  = 512; // the largest block the neighbour kernels are launched with (a tuning choice)

// particle count of a launch: the device counter when there is one (the reference keeps num_atoms on the
// device too, cuda-engine.h:133), else the value passed by the host
__device__ __forceinline__ int32_t count_of(const PbfK& k) { return k.n_dev ? __ldg(k.n_dev) : k.n; }

__device__ __forceinline__ int32_t cell_coord(float pos, float org, float inv, int32_t nc)
{
    // (pos - org) and the product are each rounded exactly once, as in the oracle; no contraction
    const float t = __fsub_rn(pos, org);
    const float u = __fmul_rn(t, inv);
    if (!(u >= 0.f)) { return 0; }
    if (u >= (float)nc) { return nc - 1; }
    return (int32_t)u;
}

template <bool MULTI>
__device__ __forceinline__ DomDev load_dom(const PbfK& k, const DomDev* __restrict__ doms,
                                           const int32_t* __restrict__ dom, int32_t i)
{
    if constexpr (MULTI) {
        return doms[__ldg(&dom[i])];
    } else {
        return k.d0;
    }
}

// A neighbour's value. Separate launches read through the read-only cache. Inside the persistent kernels
// (CG) the arrays are rewritten from phase to phase, which the read-only path does not allow, so the value
// is read with an ordinary L1-cached load (ld.global.ca): every phase reads only values written before its
// grid barrier, where each block's first thread takes the other blocks' writes with a gpu-scope acquire
// and a fence, and the block's barrier orders its other threads after that, so under the PTX memory model
// those loads observe the new values and L1 cannot serve lines cached before the barrier. (Reading them from
// L2 with ld.global.cg instead was slower: a 16,384-particle persistent step 0.195 against 0.157 ms.)
template <bool CG, class T>
__device__ __forceinline__ T ldn(const T* p)
{
    if constexpr (CG) {
        return __ldca(p);
    } else {
        return __ldg(p);
    }
}

// A particle of the step: start position x (.x, .y) and displacement d = x* - x (.z, .w).
__device__ __forceinline__ float2 xy_of(const float4 a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ float2 d_of(const float4 a) { return make_float2(a.z, a.w); }
// The offset x*_i - x*_j from the start positions and displacements. For neighbours x_i - x_j is exact (the
// two lie within a factor two of each other, Sterbenz), so the offset's only rounding is relative to itself,
// not to the coordinates; x* itself (x + d, rounded) is needed only to find a particle's cell.
__device__ __forceinline__ float2 offset(const float2 pi, const float2 di, const float4 b)
{
    return add2(sub2(pi, xy_of(b)), sub2(di, d_of(b)));
}

// a neighbour's (x, d) record and one more value of it (lambda, omega or the multiplier memory)
struct Nbr {
    float4 q;
    float a;
};

// Visits every particle index in the cells within R of the base cell of (px, py) (the reference scans the
// 3x3 cells around clamp(floorf(x)/kCellDim), PBF.cu:252-263). Each row of cells is one contiguous range.
template <class F>
__device__ __forceinline__ void for_neighbours(const DomDev& d, const PbfK& k, const uint32_t* __restrict__ start,
                                               float px, float py, F&& f)
{
    const int32_t bx = cell_coord(px, d.ox, k.inv_cell, d.ncx);
    const int32_t by = cell_coord(py, d.oy, k.inv_cell, d.ncy);
    const int32_t x0 = max(bx - k.R, 0);
    const int32_t x1 = min(bx + k.R, d.ncx - 1);
    const int32_t y0 = max(by - k.R, 0);
    const int32_t y1 = min(by + k.R, d.ncy - 1);
    for (int32_t y = y0; y <= y1; ++y) {
        const uint32_t row = d.coff + (uint32_t)y * (uint32_t)d.ncx;
        const uint32_t b   = __ldg(&start[row + x0]);
        const uint32_t e   = __ldg(&start[row + x1 + 1]);
        for (uint32_t j = b; j < e; ++j) { f(j); }
    }
}

// for_neighbours from a given base cell
template <class F>
__device__ __forceinline__ void for_neighbours_at(const DomDev& d, const PbfK& k, const uint32_t* __restrict__ start,
                                                  int32_t bx, int32_t by, F&& f)
{
    const int32_t x0 = max(bx - k.R, 0);
    const int32_t x1 = min(bx + k.R, d.ncx - 1);
    const int32_t y0 = max(by - k.R, 0);
    const int32_t y1 = min(by + k.R, d.ncy - 1);
    for (int32_t y = y0; y <= y1; ++y) {
        const uint32_t row = d.coff + (uint32_t)y * (uint32_t)d.ncx;
        const uint32_t b   = __ldg(&start[row + x0]);
        const uint32_t e   = __ldg(&start[row + x1 + 1]);
        for (uint32_t j = b; j < e; ++j) { f(j); }
    }
}

// ----- candidate masks -----------------------------------------------------------------------------------
// With sort cells of edge h a particle scans three rows of three cells, each row one contiguous range of
// slots. The first plain lambda pass of a step records which candidates of each row lie within h + skin
// (word r, bit t: the candidate at slot start[row r, first cell] + t), and the later passes of the step
// visit only those. Every pair within h is still visited, in the scan order, as long as
//   - the particle's base cell is still its sort cell (so its rows are the recorded ones), and
//   - no particle of the 3 x 3 cells around it has moved by skin / 2 or more since the masks were made:
//     a delta p pass that moves a particle by skin / (2 iters) or more marks the 9 cells around that
//     particle's sort cell for the rest of the step, and a particle whose own cell is marked scans in full.
// The terms of pairs beyond h are exact zeros in every sum (the sums start at +0, and adding a masked
// +-0 leaves any value bit for bit), so masked and full scans give the same result.
enum { MASK_OFF = 0, MASK_BUILD = 1, MASK_USE = 2 };
constexpr uint32_t MASK_BAD = 0x80000000u; // in word 0: this particle's masks are not usable

// The full scan of particle i whose base cell is (bx, by) (cell h, R = 1), recording its masks. f(j)
// returns whether candidate j lies within h + skin. The particle's own slot is not recorded: no pass takes
// a term from the self pair inside its loop (the density's self term is added after it); its bit is cleared
// after the scan, and self_in tells whether the scan met that slot.
template <class F>
__device__ __forceinline__ uint4 scan_build(const DomDev& d, const uint32_t* __restrict__ start, int32_t bx,
                                            int32_t by, int32_t i, bool& self_in, F&& f)
{
    const int32_t x0 = max(bx - 1, 0);
    const int32_t x1 = min(bx + 1, d.ncx - 1);
    uint32_t w[3]    = {0u, 0u, 0u};
    bool bad         = false;
    self_in          = false;
#pragma unroll
    for (int32_t r = 0; r < 3; ++r) {
        const int32_t y = by - 1 + r;
        if (y < 0 || y >= d.ncy) { continue; }
        const uint32_t row = d.coff + (uint32_t)y * (uint32_t)d.ncx;
        const uint32_t b   = __ldg(&start[row + x0]);
        const uint32_t e   = __ldg(&start[row + x1 + 1]);
        bad                = bad || (e - b > 31u);
        // one bit per slot, shifted along with the slot (a row of more than 31 slots is marked bad above,
        // and its bits are never read)
        uint32_t wr = 0u, bit = 1u;
        for (uint32_t j = b; j < e; ++j, bit <<= 1) { wr |= f(j) ? bit : 0u; }
        const uint32_t t = (uint32_t)i - b;
        if (t < e - b) { // the particle's own slot is in this row
            self_in = true;
            wr &= t < 31u ? ~(1u << t) : 0xffffffffu;
        }
        w[r] = wr;
    }
    return make_uint4((w[0] & ~MASK_BAD) | (bad ? MASK_BAD : 0u), w[1], w[2], 0u);
}

// Visits the candidates of the masks m around base cell (bx, by), in scan order. The three rows run as one
// loop (the next row with candidates takes over when a row's bits run out), so a warp iterates as often as
// its lane with the most candidates, not the sum over rows of each row's maximum.
template <class L, class A>
__device__ __forceinline__ void scan_masked(const DomDev& d, const uint32_t* __restrict__ start, int32_t bx,
                                            int32_t by, const uint4 m, L&& ld, A&& ap)
{
    // a row outside the scene has no bits, and its start is not read
    const uint32_t row0 = d.coff + (uint32_t)max(bx - 1, 0);
    const uint32_t ncx  = (uint32_t)d.ncx;
    uint32_t w1 = m.y, w2 = m.z;
    uint32_t bits = m.x & ~MASK_BAD;
    uint32_t base = bits ? __ldg(&start[row0 + (uint32_t)(by - 1) * ncx]) : 0u;
    uint32_t b1   = w1 ? __ldg(&start[row0 + (uint32_t)by * ncx]) : 0u;
    const uint32_t b2 = w2 ? __ldg(&start[row0 + (uint32_t)(by + 1) * ncx]) : 0u;
    if (bits == 0u) {
        bits = w1 ? w1 : w2;
        base = w1 ? b1 : b2;
        w1   = w1 ? w2 : 0u;
        b1   = b2;
        w2   = 0u;
    }
    while (bits) {
        const uint32_t t = (uint32_t)__ffs(bits) - 1u;
        bits &= bits - 1u;
        ap(base + t, ld(base + t));
        if (bits == 0u) {
            bits = w1 ? w1 : w2;
            base = w1 ? b1 : b2;
            w1   = w1 ? w2 : 0u;
            b1   = b2;
            w2   = 0u;
        }
    }
}

// The neighbour scan of particle i at (px, py) in mask mode MASK: ap(j, ld(j)) for every candidate j in
// scan order. ap returns whether j lies within h + skin (used by MASK_BUILD only). Returns true when the
// candidates came from the masks, which skip the particle's own slot: masks are used only while the
// particle is in its sort cell, so the full scan would have met that slot.
template <int MASK, bool CG, class L, class A, class AM>
__device__ __forceinline__ bool scan_ld2(const DomDev& d, const PbfK& k, const uint32_t* __restrict__ start,
                                         float px, float py, int32_t i, L&& ld, A&& ap, AM&& apm)
{
    auto f = [&](uint32_t j) -> bool { return ap(j, ld(j)); };
    if constexpr (MASK == MASK_OFF) {
        for_neighbours(d, k, start, px, py, f);
    } else {
        const int32_t bx   = cell_coord(px, d.ox, k.inv_cell, d.ncx);
        const int32_t by   = cell_coord(py, d.oy, k.inv_cell, d.ncy);
        const uint32_t key = d.coff + (uint32_t)by * (uint32_t)d.ncx + (uint32_t)bx;
        if constexpr (MASK == MASK_BUILD) {
            bool self_in;
            uint4 m = scan_build(d, start, bx, by, i, self_in, f);
            if (key != __ldg(&k.keys[i])) { m.x |= MASK_BAD; } // built around another cell than the sort cell
            k.nmask[i] = m;
        } else {
            const uint4 m = ldn<CG>(&k.nmask[i]);
            if (!(m.x & MASK_BAD) && key == __ldg(&k.keys[i]) && ldn<CG>(&k.mflag[key]) == 0) {
                scan_masked(d, start, bx, by, m, ld, apm);
                return true;
            } else {
                for_neighbours_at(d, k, start, bx, by, f);
            }
        }
    }
    return false;
}

// scan_ld2 with apm = ap. apm applies the candidates of masked scans, which never include the particle
// itself, so it may leave out the self-pair test.
template <int MASK, bool CG, class L, class A>
__device__ __forceinline__ bool scan_ld(const DomDev& d, const PbfK& k, const uint32_t* __restrict__ start,
                                        float px, float py, int32_t i, L&& ld, A&& ap)
{
    return scan_ld2<MASK, CG>(d, k, start, px, py, i, ld, ap, ap);
}

// scan_ld with one functor f(j) that loads and applies
template <int MASK, bool CG, class F>
__device__ __forceinline__ bool scan(const DomDev& d, const PbfK& k, const uint32_t* __restrict__ start, float px,
                                     float py, int32_t i, F&& f)
{
    return scan_ld<MASK, CG>(d, k, start, px, py, i, [](uint32_t j) { return j; },
                             [&](uint32_t j, uint32_t) -> bool { return f(j); });
}

// A delta p pass moved particle i (sort cell key) by at least skin / (2 iters): the particles of the 3 x 3
// cells around its sort cell scan in full for the rest of the step.
// Arguments by value: the call keeps them in registers (a reference would put the scene's DomDev on the stack).
__device__ __noinline__ void mark_mover(uint8_t* __restrict__ mflag, uint32_t coff, int32_t ncx, int32_t ncy,
                                        uint32_t key)
{
    const uint32_t local = key - coff;
    const int32_t cy     = (int32_t)(local / (uint32_t)ncx);
    const int32_t cx     = (int32_t)(local - (uint32_t)cy * (uint32_t)ncx);
    for (int32_t y = max(cy - 1, 0); y <= min(cy + 1, ncy - 1); ++y) {
        for (int32_t x = max(cx - 1, 0); x <= min(cx + 1, ncx - 1); ++x) {
            mflag[coff + (uint32_t)y * (uint32_t)ncx + (uint32_t)x] = 1u;
        }
    }
}


// integer mixer of the reference (hash, cuda-internal.cuh:19-27)
__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// pairDirection, PBF.cu:309-321
__device__ __forceinline__ void pair_direction(uint32_t a, uint32_t b, float& nx, float& ny)
{
    const uint32_t lo = min(a, b), hi = max(a, b);
    const float ang   = (float)(mix32(lo * 0x9E3779B9u ^ hi) & 0xFFFFu) * (6.2831853f / 65536.f);
    float s, c;
    __sincosf(ang, &s, &c);
    const float sign = (a < b) ? 1.f : -1.f;
    nx               = sign * c;
    ny               = sign * s;
}

// ----- predict + cell key + histogram rank (PBF.cu:786-797) ---------------------------------------------
// x* = x + dt v + dt^2 g, each operation rounded once as in the oracle (the placement recomputes it)
__device__ __forceinline__ float2 predict(const PbfK& k, float2 p, float2 w)
{
    return make_float2(__fadd_rn(__fmaf_rn(k.dt, w.x, p.x), k.g2x), __fadd_rn(__fmaf_rn(k.dt, w.y, p.y), k.g2y));
}

// Lanes of a warp that share a cell take consecutive ranks in lane order from one atomicAdd. All lanes of
// the warp call it; `valid` marks those that carry particle i.
// The rank of particle i among the particles of its cell key: lanes with the same key add their number to
// the cell's count with one atomic (the leader's), and each takes its place after the lanes before it. All
// lanes of the warp call it; valid marks those that carry a particle.
__device__ __forceinline__ void hist_rank(uint32_t key, bool valid, uint2* __restrict__ keyrank,
                                          uint32_t* __restrict__ count, int32_t i)
{
    const int32_t lane   = threadIdx.x & 31;
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const int32_t leader = __ffs(peers) - 1;
    uint32_t base        = 0;
    if (valid && lane == leader) { base = atomicAdd(&count[key], (uint32_t)__popc(peers)); }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (valid) {
        const uint32_t rank = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        keyrank[i]          = make_uint2(key, rank);
    }
}

// the sort cell key of predicted position ps in scene d
__device__ __forceinline__ uint32_t cell_key(const PbfK& k, const DomDev& d, float2 ps)
{
    const int32_t cx = cell_coord(ps.x, d.ox, k.inv_cell, d.ncx);
    const int32_t cy = cell_coord(ps.y, d.oy, k.inv_cell, d.ncy);
    return d.coff + (uint32_t)cy * (uint32_t)d.ncx + (uint32_t)cx;
}

template <bool MULTI>
__device__ __forceinline__ void predict_hist_one(const PbfK& k, const DomDev* __restrict__ doms,
                                                 const int32_t* __restrict__ dom, const float2* __restrict__ x,
                                                 const float2* __restrict__ v, uint2* __restrict__ keyrank,
                                                 uint32_t* __restrict__ count, int32_t i, bool valid)
{
    uint32_t key = 0xffffffffu;
    if (valid) { key = cell_key(k, load_dom<MULTI>(k, doms, dom, i), predict(k, x[i], v[i])); }
    hist_rank(key, valid, keyrank, count, i);
}

template <bool MULTI>
__global__ void __launch_bounds__(T_PART)
    k_predict_hist(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
                   const float2* __restrict__ x, const float2* __restrict__ v, uint2* __restrict__ keyrank,
                   uint32_t* __restrict__ count)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    predict_hist_one<MULTI>(k, doms, dom, x, v, keyrank, count, i, i < count_of(k));
}

// ----- stable placement + gather (PBF.cu:801-833) -------------------------------------------------------
// The atomic ranks are unique but depend on warp scheduling; the stable slot of particle i is the number of
// entries of its cell's bucket with a smaller pre-sort index.
// CG: start and bucket were written earlier in the same (persistent) kernel, so they are read with ldn<true>
// Output: the step's (x, d) records (xd_out, the engine), or x and x* as two float2 arrays (x_out, xs_out, the
// allocation-free sort). d = x* - x is computed from the FP32 x* that decided the cell key, so x + d gives that
// x* back (exactly while x and x* lie within a factor two of each other).
template <bool CG = false>
__device__ __forceinline__ void place_one(const PbfK& k, const uint2* __restrict__ keyrank,
                                          const uint32_t* __restrict__ start, const uint32_t* __restrict__ bucket,
                                          const float2* x_in, const float2* __restrict__ v_in,
                                          float4* __restrict__ xd_out, float2* __restrict__ x_out,
                                          float2* __restrict__ xs_out, uint32_t* __restrict__ perm,
                                          uint32_t* __restrict__ key_out,
                                          const uint32_t* __restrict__ id_in, uint32_t* __restrict__ id_out,
                                          const float* __restrict__ acc_in, float* __restrict__ prev_out,
                                          float* __restrict__ lam_out, int32_t i)
{
    const uint2 kr = keyrank[i];
    // the keys, the starts and the buckets come from one histogram; the bounds checks only keep an
    // inconsistent set (a caller's bug) from reading or writing outside the arrays
    const uint32_t n = (uint32_t)count_of(k);
    if (kr.x >= k.ncells) { return; }
    const uint32_t s = ldn<CG>(&start[kr.x]);
    const uint32_t e = min(ldn<CG>(&start[kr.x + 1]), n);
    uint32_t rank    = 0;
    for (uint32_t t = s; t < e; ++t) { rank += (ldn<CG>(&bucket[t]) < (uint32_t)i) ? 1u : 0u; }
    const uint32_t dst = s + rank;
    if (dst >= n) { return; }
    const float2 p     = x_in[i];
    const float2 ps    = predict(k, p, v_in[i]);
    if (xd_out) {
        xd_out[dst] = make_float4(p.x, p.y, __fsub_rn(ps.x, p.x), __fsub_rn(ps.y, p.y));
    } else {
        x_out[dst]  = p;
        xs_out[dst] = ps;
    }
    perm[dst]          = (uint32_t)i;
    key_out[dst]       = kr.x;
    if (id_in) { id_out[dst] = id_in[i]; }
    if (acc_in) {
        // the previous step's summed multiplier follows the particle into the new order
        const float a = acc_in[i];
        prev_out[dst] = a;
        if (lam_out) { lam_out[dst] = a; }
    }
}

__global__ void __launch_bounds__(T_PART)
    k_place(const PbfK k, const uint2* __restrict__ keyrank, const uint32_t* __restrict__ start,
            const uint32_t* __restrict__ bucket, const float2* __restrict__ x_in,
            const float2* __restrict__ v_in, float4* __restrict__ xd_out, float2* __restrict__ x_out,
            float2* __restrict__ xs_out, uint32_t* __restrict__ perm, uint32_t* __restrict__ key_out,
            const uint32_t* __restrict__ id_in, uint32_t* __restrict__ id_out, const float* __restrict__ acc_in,
            float* __restrict__ prev_out, float* __restrict__ lam_out)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count_of(k)) { return; }
    place_one(k, keyrank, start, bucket, x_in, v_in, xd_out, x_out, xs_out, perm, key_out, id_in, id_out, acc_in,
              prev_out, lam_out, i);
}

// ----- lambda (PBF.cu:243-294) --------------------------------------------------------------------------
// ACC_NONE: the reference's lambda, recomputed from scratch in every iteration.
// ACC_SUM:  the same, also added to the step's summed multiplier (training-pair collection).
// ACC_PROJ: a later iteration of a GPE_WARM_PREV step. The summed multiplier L (acc) is updated by the
//           projected increment L <- min(L - C_raw / (|grad C|^2 + eps), 0) with C_raw = rho/rho0 - 1
//           unclamped, and the pass moves the particles by the change of L; a sum that overshot is relaxed
//           again and L never turns into a pull (accumulated-multiplier clamping).
enum { ACC_NONE = 0, ACC_SUM = 1, ACC_PROJ = 2 };
template <bool MULTI, bool SELFG, int ACC, bool CG = false, int MASK = MASK_OFF>
__device__ __forceinline__ void lambda_one(const PbfK& k, const DomDev* __restrict__ doms,
                                           const int32_t* __restrict__ dom, const uint32_t* __restrict__ start,
                                           const float4* __restrict__ xd, float* __restrict__ lam,
                                           const uint32_t* __restrict__ pair_id, float* __restrict__ acc, int32_t i)
{
    const DomDev d       = load_dom<MULTI>(k, doms, dom, i);
    const uint32_t pbase = MULTI ? __ldg(&start[d.coff]) : 0u;
    const float4 p4      = ldn<CG>(&xd[i]);
    const float2 px = xy_of(p4), pd = d_of(p4);
    const float2 p       = add2(px, pd); // x*, for the cell lookup
    // The reference accumulates per pair sv = -cs m (h-r)^2 r/|r|, |sv|^2 / m and m W6 (PBF.cu:264-286).
    // Constants are hoisted: sx, sy = sum (h-r)^2 r/|r|, s4 = sum (h-r)^4 (= |sv|^2 / (cs m)^2 since r/|r| is a
    // unit vector), s6 = sum (h^2 - r^2)^3. The self pair (r = 0) is added after the loop: it contributes
    // h^6 to the density and, in the reference, a gradient of length cs m h^2 along pairDirection(i, i).
    float2 sg = make_float2(0.f, 0.f); // (sx, sy)
    float s4 = 0.f, s6 = 0.f;
    bool self_seen = false; // the atom's own slot can fall outside the scanned cells after large moves
    // Branch-free body: every lane of a warp runs the same instructions for every candidate and the terms of
    // pairs beyond h (and of the self pair) are masked to zero; a data-dependent accept branch here would
    // make each warp execute both paths on almost every iteration.
    // ME: the candidate may be the particle itself (full scans); masked scans never visit it
    auto body = [&](uint32_t j, const float4 q, auto me) -> bool {
        const float2 r  = offset(px, pd, q);
        const float r2  = fmaf(r.x, r.x, r.y * r.y);
        const bool self = decltype(me)::value && j == (uint32_t)i;
        self_seen       = self_seen || self;
        const bool in   = (r2 <= k.h2) && !self;
        const bool dir  = in && (r2 > 1e-12f);
        const float qq  = in ? k.h2 - r2 : 0.f;
        s6              = fmaf(qq * qq, qq, s6);
        const float inv = rsqrtf(dir ? r2 : 1.f);
        const float dif = dir ? k.h - r2 * inv : 0.f;
        const float d2  = dif * dif;
        const float w   = d2 * inv;
        sg              = fma2(make_float2(w, w), r, sg);
        s4              = fmaf(d2, d2, s4);
        if (SELFG && in && !dir && r.x == 0.f && r.y == 0.f) {
            // a distinct atom at the same position: the reference's pseudo-random pair direction
            float nx, ny;
            if (pair_id) {
                pair_direction(__ldg(&pair_id[i]), __ldg(&pair_id[j]), nx, ny);
            } else {
                pair_direction((uint32_t)i - pbase, j - pbase, nx, ny);
            }
            sg.x = fmaf(k.h2, nx, sg.x);
            sg.y = fmaf(k.h2, ny, sg.y);
            s4 = fmaf(k.h2, k.h2, s4);
        }
        return r2 < k.skin2;
    };
    auto ld   = [&](uint32_t j) { return ldn<CG>(&xd[j]); };
    auto full = [&](uint32_t j, const float4 q) -> bool { return body(j, q, std::true_type{}); };
    auto near = [&](uint32_t j, const float4 q) -> bool { return body(j, q, std::false_type{}); };
    if constexpr (MASK == MASK_BUILD) {
        // Record the masks with a distance-only scan of the 3 x 3 cells, then apply the lambda terms to the
        // recorded candidates alone (their loads hit L1): the same terms in the same order as the full
        // scan, whose other candidates (beyond h, or the particle itself) add exact zeros.
        const int32_t bx   = cell_coord(p.x, d.ox, k.inv_cell, d.ncx);
        const int32_t by   = cell_coord(p.y, d.oy, k.inv_cell, d.ncy);
        const uint32_t key = d.coff + (uint32_t)by * (uint32_t)d.ncx + (uint32_t)bx;
        bool seen          = false;
        uint4 m            = scan_build(d, start, bx, by, i, seen, [&](uint32_t j) -> bool {
            const float2 r = offset(px, pd, ld(j));
            return fmaf(r.x, r.x, r.y * r.y) < k.skin2;
        });
        const bool fits = !(m.x & MASK_BAD); // no row held more candidates than a mask word
        if (key != __ldg(&k.keys[i])) { m.x |= MASK_BAD; } // built around another cell than the sort cell
        k.nmask[i] = m;
        if (fits) {
            scan_masked(d, start, bx, by, m, ld, near);
            self_seen = seen;
        } else {
            for_neighbours_at(d, k, start, bx, by, [&](uint32_t j) { full(j, ld(j)); });
        }
    } else {
        const bool self_masked = scan_ld2<MASK, CG>(d, k, start, p.x, p.y, i, ld, full, near);
        self_seen              = self_seen || self_masked;
    }
    if (self_seen) {
        s6 = fmaf(k.h2 * k.h2, k.h2, s6);
        if (SELFG) {
            float nx, ny;
            const uint32_t a = pair_id ? __ldg(&pair_id[i]) : (uint32_t)i - pbase;
            pair_direction(a, a, nx, ny);
            sg.x = fmaf(k.h2, nx, sg.x);
            sg.y = fmaf(k.h2, ny, sg.y);
            s4 = fmaf(k.h2, k.h2, s4);
        }
    }
    const float csm  = k.cs * k.mass;
    const float rho  = k.mass * k.c6 * s6;
    const float gx = csm * sg.x, gy = csm * sg.y;
    const float gsq  = k.inv_mass * (csm * csm) * s4;
    const float C    = fmaxf(rho * k.inv_rho0 - 1.f, k.c_min);
    const float self = k.inv_mass * (gx * gx + gy * gy);
    const float grad = k.inv_rho0 * k.inv_rho0 * (self + gsq);
    if (ACC == ACC_PROJ) {
        const float lraw = -(rho * k.inv_rho0 - 1.f) / (grad + k.eps);
        const float a    = acc[i];
        const float an   = fminf(a + lraw, 0.f);
        lam[i]           = an - a;
        acc[i]           = an;
    } else {
        const float l = -C / (grad + k.eps);
        lam[i]        = l;
        if (ACC == ACC_SUM) { acc[i] += l; }
    }
}

// the mask-recording pass in 40 registers (3 blocks of 512 per SM), the masked passes in 32
template <bool MULTI, bool SELFG, int ACC, int MASK>
__global__ void __launch_bounds__(T_MAX, (MASK == MASK_BUILD && !SELFG) ? 3 : (MASK == MASK_USE ? 4 : 1))
    k_lambda(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
             const uint32_t* __restrict__ start, const float4* __restrict__ xd, float* __restrict__ lam,
             const uint32_t* __restrict__ pair_id, float* __restrict__ acc)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count_of(k)) {
        lambda_one<MULTI, SELFG, ACC, false, MASK>(k, doms, dom, start, xd, lam, pair_id, acc, i);
    }
}

// ----- delta p with artificial pressure and over-relaxation, then walls (PBF.cu:398-447, 471-499) -------
// ACCINIT: this pass applies the warm start; its multiplier starts the step's running sum.
template <bool MULTI, bool SCORR, bool ACCINIT, bool CG = false, int MASK = MASK_OFF>
__device__ __forceinline__ void delta_p_one(const PbfK& k, const DomDev* __restrict__ doms,
                                            const int32_t* __restrict__ dom, const uint32_t* __restrict__ start,
                                            const float4* __restrict__ xd, const float* __restrict__ lam,
                                            float4* __restrict__ xd_out, float* __restrict__ acc, int32_t i)
{
    const DomDev d  = load_dom<MULTI>(k, doms, dom, i);
    const float4 p4 = ldn<CG>(&xd[i]);
    const float2 px = xy_of(p4), pd = d_of(p4);
    const float2 p  = add2(px, pd); // x*, for the cell lookup
    const float li  = ldn<CG>(&lam[i]);
    if (ACCINIT) { acc[i] = li; }
    const float mli = li * k.mass;
    // dp = omega/(m rho0) sum (m lambda_i + m lambda_j - s_corr) * (-cs (h-r)^2 r/|r|) (PBF.cu:415-437); pairs
    // closer than 1e-6 (the self pair included) have a zero direction there and are skipped here.
    const float c6w = k.c6 * k.inv_w_dq;
    float2 sg = make_float2(0.f, 0.f); // (sx, sy)
    scan_ld<MASK, CG>(d, k, start, p.x, p.y, i,
                      [&](uint32_t j) { return Nbr{ldn<CG>(&xd[j]), ldn<CG>(&lam[j])}; },
                      [&](uint32_t, const Nbr ql) -> bool {
        const float lj  = ql.a;
        const float2 r  = offset(px, pd, ql.q);
        const float r2  = fmaf(r.x, r.x, r.y * r.y);
        const bool ok   = (r2 <= k.h2) && (r2 > 1e-12f); // masked, branch-free (see k_lambda)
        const float inv = rsqrtf(ok ? r2 : 1.f);
        float l         = fmaf(lj, k.mass, mli);
        if (SCORR) {
            const float qq    = k.h2 - r2;
            const float ratio = c6w * (qq * qq * qq);
            const float r2q   = ratio * ratio;
            l                 = fmaf(-k.scorr_k, r2q * r2q, l);
        }
        const float diff = k.h - r2 * inv;
        const float w    = ok ? diff * diff * inv * l : 0.f;
        sg               = fma2(make_float2(w, w), r, sg);
        return false;
    });
    const float s = -k.cs * k.dp_scale;
    // the correction moves the displacement; the position x + d is clamped to the walls (clamp<float>(v, lb,
    // ub), PBF.cu:496-497) by setting d = wall - x, exact next to the wall, so that x + d lands on it
    float dx = fmaf(s, sg.x, pd.x), dy = fmaf(s, sg.y, pd.y);
    const float ox = px.x + dx, oy = px.y + dy;
    dy = (oy > d.hiy) ? __fsub_rn(d.hiy, px.y) : ((oy < d.loy) ? __fsub_rn(d.loy, px.y) : dy);
    dx = (ox > d.hix) ? __fsub_rn(d.hix, px.x) : ((ox < d.lox) ? __fsub_rn(d.lox, px.x) : dx);
    xd_out[i] = make_float4(px.x, px.y, dx, dy);
    if constexpr (MASK == MASK_USE) {
        const float mx = dx - pd.x, my = dy - pd.y;
        if (!(fmaf(mx, mx, my * my) < k.move2)) { mark_mover(k.mflag, d.coff, d.ncx, d.ncy, __ldg(&k.keys[i])); }
    }
}

template <bool MULTI, bool SCORR, bool ACCINIT, int MASK>
__global__ void __launch_bounds__(T_MAX)
    k_delta_p(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
              const uint32_t* __restrict__ start, const float4* __restrict__ xd, const float* __restrict__ lam,
              float4* __restrict__ xd_out, float* __restrict__ acc)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count_of(k)) {
        delta_p_one<MULTI, SCORR, ACCINIT, false, MASK>(k, doms, dom, start, xd, lam, xd_out, acc, i);
    }
}

// ----- warm start: features of the first lambda pass ------------------------------------------------------
// The lambda sums of k_lambda plus the neighbour count and the poly6-weighted sum of the neighbours'
// lambda_prev; returns the cold first-iteration lambda and fills the network's 12 features (the order is
// the one documented with gpe_pbf_set_warm_start).
template <bool MULTI, bool SELFG, int MASK = MASK_OFF>
__device__ __forceinline__ float warm_features(const PbfK& k, const DomDev& d, const uint32_t* __restrict__ start,
                                               const float4* __restrict__ xd, const float* __restrict__ prev,
                                               const uint32_t* __restrict__ pair_id, int32_t i, uint32_t pbase,
                                               float (&f)[MLP_F])
{
    const float4 p4 = xd[i];
    const float2 px = xy_of(p4), pd = d_of(p4);
    const float2 p  = add2(px, pd); // x*
    float2 sg = make_float2(0.f, 0.f); // (sx, sy)
    float s4 = 0.f, s6 = 0.f, swl = 0.f;
    int32_t nn     = 0;
    bool self_seen = false;
    // ME: the candidate may be the particle itself (full scans); masked scans never visit it
    auto body = [&](uint32_t j, const Nbr ql, auto me) -> bool {
        const float4 q  = ql.q;
        const float lp  = ql.a;
        const float2 r  = offset(px, pd, q);
        const float r2  = fmaf(r.x, r.x, r.y * r.y);
        const bool self = decltype(me)::value && j == (uint32_t)i;
        self_seen       = self_seen || self;
        const bool in   = (r2 <= k.h2) && !self;
        const bool dir  = in && (r2 > 1e-12f);
        const float qq  = in ? k.h2 - r2 : 0.f;
        s6              = fmaf(qq * qq, qq, s6); // as in k_lambda, so the cold lambda is bit-identical
        swl             = fmaf(qq * qq * qq, lp, swl);
        nn += in ? 1 : 0;
        const float inv = rsqrtf(dir ? r2 : 1.f);
        const float dif = dir ? k.h - r2 * inv : 0.f;
        const float d2  = dif * dif;
        const float w   = d2 * inv;
        sg              = fma2(make_float2(w, w), r, sg);
        s4              = fmaf(d2, d2, s4);
        if (SELFG && in && !dir && r.x == 0.f && r.y == 0.f) {
            float nx, ny;
            if (pair_id) {
                pair_direction(__ldg(&pair_id[i]), __ldg(&pair_id[j]), nx, ny);
            } else {
                pair_direction((uint32_t)i - pbase, j - pbase, nx, ny);
            }
            sg.x = fmaf(k.h2, nx, sg.x);
            sg.y = fmaf(k.h2, ny, sg.y);
            s4 = fmaf(k.h2, k.h2, s4);
        }
        return r2 < k.skin2;
    };
    auto ld   = [&](uint32_t j) { return Nbr{__ldg(&xd[j]), __ldg(&prev[j])}; };
    auto full = [&](uint32_t j, const Nbr q) -> bool { return body(j, q, std::true_type{}); };
    auto near = [&](uint32_t j, const Nbr q) -> bool { return body(j, q, std::false_type{}); };
    if constexpr (MASK == MASK_BUILD) {
        // as in k_lambda: a distance-only scan records the masks, then the feature terms run over the
        // recorded candidates alone (the full scan's other candidates add exact zeros)
        const int32_t bx   = cell_coord(p.x, d.ox, k.inv_cell, d.ncx);
        const int32_t by   = cell_coord(p.y, d.oy, k.inv_cell, d.ncy);
        const uint32_t key = d.coff + (uint32_t)by * (uint32_t)d.ncx + (uint32_t)bx;
        bool seen          = false;
        uint4 m            = scan_build(d, start, bx, by, i, seen, [&](uint32_t j) -> bool {
            const float2 r = offset(px, pd, __ldg(&xd[j]));
            return fmaf(r.x, r.x, r.y * r.y) < k.skin2;
        });
        const bool fits = !(m.x & MASK_BAD);
        if (key != __ldg(&k.keys[i])) { m.x |= MASK_BAD; } // built around another cell than the sort cell
        k.nmask[i] = m;
        if (fits) {
            scan_masked(d, start, bx, by, m, ld, near);
            self_seen = seen;
        } else {
            for_neighbours_at(d, k, start, bx, by, [&](uint32_t j) { full(j, ld(j)); });
        }
    } else {
        scan_ld<MASK, false>(d, k, start, p.x, p.y, i, ld, full);
    }
    const float lpi = prev[i];
    if (self_seen) {
        s6  = fmaf(k.h2 * k.h2, k.h2, s6);
        swl = fmaf(k.h2 * k.h2 * k.h2, lpi, swl);
        if (SELFG) {
            float nx, ny;
            const uint32_t a = pair_id ? __ldg(&pair_id[i]) : (uint32_t)i - pbase;
            pair_direction(a, a, nx, ny);
            sg.x = fmaf(k.h2, nx, sg.x);
            sg.y = fmaf(k.h2, ny, sg.y);
            s4 = fmaf(k.h2, k.h2, s4);
        }
    }
    const float csm  = k.cs * k.mass;
    const float rho  = k.mass * k.c6 * s6;
    const float gx = csm * sg.x, gy = csm * sg.y;
    const float gsq  = k.inv_mass * (csm * csm) * s4;
    const float C    = fmaxf(rho * k.inv_rho0 - 1.f, k.c_min);
    const float self = k.inv_mass * (gx * gx + gy * gy);
    const float grad = k.inv_rho0 * k.inv_rho0 * (self + gsq);
    const float lam  = -C / (grad + k.eps);
    const float ddx = pd.x, ddy = pd.y; // x* - x
    const float inv_h = 1.f / k.h;
    const float wall  = fminf(fminf(p.x - d.lox, d.hix - p.x), fminf(p.y - d.loy, d.hiy - p.y)) * inv_h;
    f[0]  = (float)nn;
    f[1]  = lpi;
    f[2]  = rho * k.inv_rho0 - 1.f;
    f[3]  = C;
    f[4]  = sqrtf(ddx * ddx + ddy * ddy) * inv_h;
    f[5]  = -gx * k.inv_rho0; // dC_i/dx_i = -(cs m / rho0) sum (h-r)^2 r/|r|
    f[6]  = -gy * k.inv_rho0;
    f[7]  = sqrtf(f[5] * f[5] + f[6] * f[6]);
    f[8]  = grad;
    f[9]  = lam;
    f[10] = fminf(fmaxf(wall, 0.f), 4.f);
    f[11] = s6 > 0.f ? swl / s6 : 0.f;
    return lam;
}

// First lambda pass of a GPE_WARM_MLP step, part 1: the features at full occupancy (one thread per
// particle), standardised and rounded to BF16, written as the network's layer-1 A operand: tile t of 128
// particles is 4 KB at feat + t * 2048 in the tensor cores' K-major layout, so part 2 moves it to shared
// memory with one bulk copy. (Computing the features inside the tensor-core kernel caps the neighbour loop
// at the 7 CTAs of 4 warps that fit an SM beside their TMEM and operand tiles: 126 us against about 50 us
// here at 1M particles.) With MASK_BUILD the pass records the step's candidate masks with a distance-only
// scan and computes the features over the recorded candidates alone, as k_lambda does.
template <bool MULTI, bool SELFG, int MASK>
__global__ void __launch_bounds__(T_PART)
    k_lambda_feat(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
                  const uint32_t* __restrict__ start, const float4* __restrict__ xd, const float* __restrict__ prev,
                  const uint32_t* __restrict__ pair_id, const MlpDev* __restrict__ mlp, uint16_t* __restrict__ feat)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count_of(k)) { return; }
    const DomDev d       = load_dom<MULTI>(k, doms, dom, i);
    const uint32_t pbase = MULTI ? __ldg(&start[d.coff]) : 0u;
    float f[MLP_F];
    (void)warm_features<MULTI, SELFG, MASK>(k, d, start, xd, prev, pair_id, i, pbase, f);
    float mu[MLP_FP], isd[MLP_FP];
#pragma unroll
    for (int q = 0; q < MLP_FP; ++q) {
        mu[q]  = __ldg(&mlp->mu[q]);
        isd[q] = __ldg(&mlp->isd[q]);
    }
    uint4 c0, c1;
    mlp_pack_row(f, mu, isd, c0, c1);
    uint16_t* tile                                              = feat + (size_t)(i >> 7) * (MLP_TILE * MLP_FP);
    *reinterpret_cast<uint4*>(&tile[kmajor(i & 127, 0, MLP_FP)]) = c0;
    *reinterpret_cast<uint4*>(&tile[kmajor(i & 127, 8, MLP_FP)]) = c1;
}

// Part 2: the network on the tensor cores, persistent over tiles; each tile's operand arrives by a bulk
// copy issued one tile ahead into the other buffer. lambda = min(lambda_prev + r, 0).
__global__ void __launch_bounds__(MLP_TILE)
    k_mlp_apply(const PbfK k, const uint16_t* __restrict__ feat, const float* __restrict__ prev, float* __restrict__ lam,
                const MlpDev* __restrict__ mlp, uint32_t* __restrict__ status)
{
    __shared__ MlpFwdSmem S;
    const int32_t n      = count_of(k);
    const int32_t ntiles = (n + MLP_TILE - 1) / MLP_TILE;
    if ((int32_t)blockIdx.x >= ntiles) { return; } // uniform over the CTA, before any barrier
    mlp_fwd_setup(S, mlp);
    const float ymu = mlp->ymu, ysd = mlp->ysd;
    uint32_t phase = 0, ldph[2] = {0u, 0u};
    bool ok        = true;
    if (threadIdx.x == 0) {
        tc::bulk_g2s(S.a1[0], feat + (size_t)blockIdx.x * (MLP_TILE * MLP_FP), MLP_A1_TILE_BYTES, &S.ldbar[0]);
    }
    int b = 0;
    for (int32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, b ^= 1) {
        const int32_t next = tile + (int32_t)gridDim.x;
        if (threadIdx.x == 0 && next < ntiles) {
            // the other buffer was read by the previous tile's MMA, which has completed
            tc::bulk_g2s(S.a1[b ^ 1], feat + (size_t)next * (MLP_TILE * MLP_FP), MLP_A1_TILE_BYTES, &S.ldbar[b ^ 1]);
        }
        ok = tc::mbar_wait(&S.ldbar[b], ldph[b]) && ok;
        ldph[b] ^= 1u;
        __syncthreads(); // every thread has read the previous tile's accumulators before the MMA overwrites them
        const float y   = mlp_fwd_core(S, b, phase, ok);
        const int32_t i = tile * MLP_TILE + (int32_t)threadIdx.x;
        if (i < n) { lam[i] = fminf(__ldg(&prev[i]) + fmaf(y, ysd, ymu), 0.f); } // a summed multiplier only pushes
    }
    if (!ok) { atomicOr(status, GPE_STATUS_TIMEOUT); }
    mlp_fwd_teardown(S);
}

// Training-pair collection: the first lambda pass of a plain (cold) step, which also appends the features
// of the particles that a seeded hash selects (probability 1/stride; none when stride is 0); the step's
// summed multiplier over its params.iters iterations becomes their target.
struct CollectK {
    float* X;
    float* T;
    int32_t* idx;
    int32_t* cnt;
    int32_t cap;
    uint32_t salt;
    uint32_t stride;
};

template <bool MULTI, bool SELFG>
__global__ void __launch_bounds__(T_PART)
    k_lambda_collect(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
                     const uint32_t* __restrict__ start, const float4* __restrict__ xd,
                     const float* __restrict__ prev, float* __restrict__ lam, const uint32_t* __restrict__ pair_id,
                     const CollectK col)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count_of(k)) { return; }
    const DomDev d       = load_dom<MULTI>(k, doms, dom, i);
    const uint32_t pbase = MULTI ? __ldg(&start[d.coff]) : 0u;
    float f[MLP_F];
    lam[i] = warm_features<MULTI, SELFG>(k, d, start, xd, prev, pair_id, i, pbase, f);
    if (col.stride != 0u && mix32((uint32_t)i * 0x9E3779B9u ^ col.salt) % col.stride == 0u) {
        const int32_t slot = atomicAdd(&col.cnt[0], 1);
        if (slot < col.cap) {
#pragma unroll
            for (int q = 0; q < MLP_F; ++q) { col.X[(size_t)slot * MLP_F + q] = f[q]; }
            col.idx[slot] = i;
        }
    }
}

// Targets of the pairs taken this step: the step's summed multiplier minus lambda_prev.
__global__ void k_collect_targets(const int32_t* __restrict__ cnt, const float* __restrict__ X, float* __restrict__ T,
                                  const int32_t* __restrict__ idx, const float* __restrict__ acc, int32_t cap)
{
    const int32_t slot = cnt[1] + (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
    const int32_t end  = min(cnt[0], cap);
    if (slot >= end) { return; }
    T[slot] = acc[idx[slot]] - X[(size_t)slot * MLP_F + 1];
}

__global__ void k_collect_advance(int32_t* __restrict__ cnt, int32_t cap)
{
    const int32_t c = min(cnt[0], cap);
    cnt[0]          = c;
    cnt[1]          = c;
}

// velocityClamp, PBF.cu:629-638
__device__ __forceinline__ void velocity_clamp(const PbfK& k, float& vx, float& vy)
{
    const float v2  = fmaf(vx, vx, vy * vy);
    // v2 == 0 can only pass the first test when v_min == 0 (never in the reference); avoid 0 * inf there
    const float inv = (v2 < k.v_min2 || v2 == 0.f) ? 0.f : rsqrtf(v2);
    const float nx = vx * inv, ny = vy * inv;
    const float a   = v2 * inv;
    const float sp  = fminf(a, k.v_max);
    vx              = nx * sp;
    vy              = ny * sp;
}

// ----- velocity + XSPH (+ vorticity omega) (PBF.cu:538, 585-627) ---------------------------------------
template <bool MULTI, bool VORT, bool CG = false, int MASK = MASK_OFF>
__device__ __forceinline__ void xsph_one(const PbfK& k, const DomDev* __restrict__ doms,
                                         const int32_t* __restrict__ dom, const uint32_t* __restrict__ start,
                                         const float4* __restrict__ xd, float2* __restrict__ x_out,
                                         float2* __restrict__ v_out, float* __restrict__ omega,
                                         uint32_t* __restrict__ status, int32_t i, uint32_t* next_key = nullptr)
{
    const DomDev d  = load_dom<MULTI>(k, doms, dom, i);
    const float4 p4 = ldn<CG>(&xd[i]);
    const float2 px = xy_of(p4), pd = d_of(p4);
    const float2 p  = add2(px, pd); // x*: the step's end position
    // v = (x* - x) / dt = d / dt (PBF.cu:538): no cancellation of two large coordinates
    const float vax = pd.x * k.inv_dt, vay = pd.y * k.inv_dt;
    // dv = c sum (v_j - v_i) W6 (PBF.cu:602-615) with the poly6 coefficient hoisted; the self pair adds 0.
    // omega = sum (v_j - v_i) x grad_j W with grad_j W = +cs (h-r)^2 r/|r| (cs hoisted as well).
    float2 dvs = make_float2(0.f, 0.f); // (dvx, dvy)
    float w    = 0.f;
    // ME: the candidate may be the particle itself (full scans); masked scans never visit it
    auto xbody = [&](uint32_t j, const float4 q, auto me) -> bool {
        const float2 r  = offset(px, pd, q);
        const float rx = r.x, ry = r.y;
        // explicit fused forms: the result must not depend on how the compiler contracts this body in the
        // kernel it is inlined into (separate launches and the persistent solve are compared bit for bit)
        const float r2  = fmaf(rx, rx, ry * ry);
        // masked, branch-free (see k_lambda); the self pair adds nothing in exact arithmetic (v_i - v_i) and is
        // left out (masked scans skip the particle's own slot)
        const bool in   = (r2 <= k.h2) && !(decltype(me)::value && j == (uint32_t)i);
        const float2 dv = fma2(d_of(q), make_float2(k.inv_dt, k.inv_dt), make_float2(-vax, -vay));
        const float dx = dv.x, dy = dv.y;
        const float qq  = in ? k.h2 - r2 : 0.f;
        const float p6  = qq * qq * qq;
        dvs             = fma2(dv, make_float2(p6, p6), dvs);
        if (VORT) {
            const bool dir   = in && (r2 > 1e-12f);
            const float inv  = rsqrtf(dir ? r2 : 1.f);
            const float diff = k.h - r2 * inv;
            const float gm   = dir ? diff * diff * inv : 0.f;
            w                = fmaf(gm, fmaf(dx, ry, -(dy * rx)), w);
        }
        return false;
    };
    scan_ld2<MASK, CG>(d, k, start, p.x, p.y, i, [&](uint32_t j) { return ldn<CG>(&xd[j]); },
                       [&](uint32_t j, const float4 q) -> bool { return xbody(j, q, std::true_type{}); },
                       [&](uint32_t j, const float4 q) -> bool { return xbody(j, q, std::false_type{}); });
    w *= k.cs;
    const float cx = k.xsph_c * k.c6;
    float vx       = fmaf(dvs.x, cx, vax);
    float vy       = fmaf(dvs.y, cx, vay);
    if (!VORT && (k.flags & GPE_PBF_VEL_CLAMP)) { velocity_clamp(k, vx, vy); }
    if (!(isfinite(vx) && isfinite(vy) && isfinite(p.x) && isfinite(p.y))) {
        atomicOr(status, GPE_STATUS_NONFINITE);
    }
    v_out[i] = make_float2(vx, vy);
    x_out[i] = p; // the step's end position, in this step's sorted order
    if (VORT) { omega[i] = w; }
    // the next step's predicted cell, from the values just written (as k_predict_hist would read them)
    if (next_key) { *next_key = cell_key(k, d, predict(k, p, make_float2(vx, vy))); }
}

template <bool MULTI, bool VORT, int MASK>
__global__ void __launch_bounds__(T_MAX)
    k_xsph(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
           const uint32_t* __restrict__ start, const float4* __restrict__ xd, float2* __restrict__ x_out,
           float2* __restrict__ v_out, float* __restrict__ omega, uint32_t* __restrict__ status)
{
    const int32_t i  = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < count_of(k);
    if (!k.hist_cnt) { // uniform
        if (valid) { xsph_one<MULTI, VORT, false, MASK>(k, doms, dom, start, xd, x_out, v_out, omega, status, i); }
        return;
    }
    // XSPH of a step followed by another step without anything in between: the next step's cell keys and
    // histogram come from here, and its sort starts with the scan (bit for bit what k_predict_hist computes
    // from the same positions and velocities; only the order of the atomic ranks within a cell differs, which
    // the stable placement does not depend on)
    uint32_t key = 0xffffffffu;
    if (valid) { xsph_one<MULTI, VORT, false, MASK>(k, doms, dom, start, xd, x_out, v_out, omega, status, i, &key); }
    hist_rank(key, valid, k.hist_kr, k.hist_cnt, i);
}

// ----- vorticity confinement (Macklin & Mueller 2013 eq. 16) --------------------------------------------
template <bool MULTI, bool CG = false, int MASK = MASK_OFF>
__device__ __forceinline__ void vorticity_one(const PbfK& k, const DomDev* __restrict__ doms,
                                              const int32_t* __restrict__ dom, const uint32_t* __restrict__ start,
                                              const float4* __restrict__ xd, const float* __restrict__ omega,
                                              float2* __restrict__ v, int32_t i)
{
    const DomDev d  = load_dom<MULTI>(k, doms, dom, i);
    const float4 p4 = xd[i];
    const float2 px = xy_of(p4), pd = d_of(p4);
    const float2 p  = add2(px, pd); // x*, for the cell lookup
    const float wi = omega[i];
    const float aw = fabsf(wi);
    float2 eg = make_float2(0.f, 0.f); // (ex, ey)
    scan_ld<MASK, CG>(d, k, start, p.x, p.y, i,
                      [&](uint32_t j) { return Nbr{ldn<CG>(&xd[j]), ldn<CG>(&omega[j])}; },
                      [&](uint32_t, const Nbr qw) -> bool {
        const float wj   = qw.a;
        const float2 r   = offset(px, pd, qw.q);
        const float rx = r.x, ry = r.y;
        const float r2   = fmaf(rx, rx, ry * ry); // explicit fused forms, as in xsph_one
        const bool ok    = (r2 <= k.h2) && (r2 > 1e-12f); // masked, branch-free (see k_lambda)
        const float inv  = rsqrtf(ok ? r2 : 1.f);
        const float diff = k.h - r2 * inv;
        const float dwg  = ok ? (fabsf(wj) - aw) * (diff * diff * inv) : 0.f; // grad_i W = -cs (...)
        eg               = fma2(make_float2(dwg, dwg), r, eg);
        return false;
    });
    // only the direction of eta = grad|omega| is used, so the positive factor cs drops out; the sign stays
    const float ex = -eg.x;
    const float ey = -eg.y;
    float2 vv      = v[i];
    const float e2 = fmaf(ex, ex, ey * ey);
    if (e2 > 1e-40f) {
        const float il = rsqrtf(e2);
        vv.x           = fmaf(k.vort_dt, ey * il * wi, vv.x);
        vv.y           = fmaf(k.vort_dt, -ex * il * wi, vv.y);
    }
    if (k.flags & GPE_PBF_VEL_CLAMP) { velocity_clamp(k, vv.x, vv.y); }
    v[i] = vv;
}

template <bool MULTI, int MASK>
__global__ void __launch_bounds__(T_MAX)
    k_vorticity(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
                const uint32_t* __restrict__ start, const float4* __restrict__ xd,
                const float* __restrict__ omega, float2* __restrict__ v)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count_of(k)) { vorticity_one<MULTI, false, MASK>(k, doms, dom, start, xd, omega, v, i); }
}

// ----- the persistent solve: every Jacobi pass (and XSPH) of a step in one launch -----------------------
// For many small scenes (or one small one) a step is a chain of short passes whose launch gaps cost as much
// as the work; here the passes run back to back in one cooperative launch, separated by a grid barrier in
// global memory. The blocks take the blocks of particles of each pass from a ticket counter (for_blocks)
// and read the values written in earlier passes through L1 after each barrier (ldn<true>).
// The arrival counter, the generation word and the ticket counter sit in separate 128-byte lines, so that
// the blocks polling the generation do not contend with the arrivals or the tickets.
struct GridSync {
    unsigned int count;
    unsigned int pad0[31];
    unsigned int gen;
    unsigned int pad1[31];
    unsigned int ticket; // hands out blocks of particles (for_blocks)
    unsigned int pad2[31];
};

// f(i) for every particle i < n of a solve phase. While the phase has no more blocks of particles than the
// grid has blocks, block b takes block of particles b. Otherwise the blocks of particles are handed out in
// order from a ticket counter, so that a block that finishes early takes another (with a fixed grid-stride
// share instead, every barrier waited for the block that drew the most expensive particles: 256 batched
// scenes 4.15 against 1.63 ms per step, 1M particles 0.400 against 0.365 ms). Thread 0 fetches the next
// ticket while the block works on the current block of particles. Every block ends the phase on exactly
// one ticket past the last block of particles, so a phase takes (blocks of particles + gridDim.x) tickets,
// and tbase, the same in every block, finds the next phase's first. A thread may now take a particle that
// another block wrote in the previous phase, so the passes read even the particle's own values with
// ldn<true>.
template <class F>
__device__ __forceinline__ void for_blocks(GridSync* g, uint32_t& tbase, int32_t n, F&& f)
{
    __shared__ uint32_t s_t[2];
    const uint32_t nb = (uint32_t)((n + (int32_t)blockDim.x - 1) / (int32_t)blockDim.x);
    if (nb <= gridDim.x) {
        const int32_t i = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
        if (i < n) { f(i); }
        return;
    }
    if (threadIdx.x == 0) { s_t[0] = atomicAdd(&g->ticket, 1u) - tbase; }
    __syncthreads();
    uint32_t c = s_t[0];
    int b      = 0;
    while (c < nb) {
        uint32_t nx = 0u;
        if (threadIdx.x == 0) { nx = atomicAdd(&g->ticket, 1u); }
        const int32_t i = (int32_t)(c * blockDim.x + threadIdx.x);
        if (i < n) { f(i); }
        if (threadIdx.x == 0) { s_t[b ^ 1] = nx - tbase; }
        __syncthreads();
        b ^= 1;
        c = s_t[b];
    }
    tbase += nb + gridDim.x;
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// A barrier wait of the persistent solve gives up after 2 s. A barrier normally completes within a few
// microseconds; the limit is far above that so that a context the GPU merely time-slices with other
// processes (which can stall it for tens of milliseconds) is not reported as hung. The self-test of the
// bounded wait uses 100 ms.
constexpr uint64_t GRID_WAIT_NS     = 2000ull * 1000ull * 1000ull;
constexpr uint64_t GRID_SELFTEST_NS = 100ull * 1000ull * 1000ull;

// All threads of every block. False when this block gave up waiting (GPE_STATUS_TIMEOUT is set); the
// caller then returns, and the other blocks time out at their next barrier in turn.
__device__ __forceinline__ bool grid_barrier(GridSync* g, unsigned int& gen, uint32_t* status,
                                             uint64_t limit_ns = GRID_WAIT_NS)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned int target = gen + 1u;
        __threadfence(); // this block's writes are visible device-wide before it arrives
        if (atomicAdd(&g->count, 1u) == gridDim.x - 1u) {
            atomicExch(&g->count, 0u);
            __threadfence();
            atomicExch(&g->gen, target);
        } else {
            const uint64_t t0 = tc::globaltimer();
            while (ld_acquire(&g->gen) != target) {
                if (tc::globaltimer() - t0 > limit_ns) {
                    ok = 0;
                    atomicOr(status, GPE_STATUS_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    gen += 1u;
    return s_ok != 0;
}

// XSPH: the velocity pass runs here too; with vorticity confinement it runs as its usual launch after the
// kernel instead (the omega-carrying pass inlined here differs from its own kernel in the last bit).
// The Jacobi passes (and XSPH) of a step inside a persistent kernel; gen is the kernel's barrier count.
// False when a barrier wait gave up (the caller returns).
// one block at a barrier whose counter says another block has already arrived: the generation never
// advances, so the wait runs out (gpe_selftest_barrier_timeout)
__global__ void k_barrier_selftest(GridSync* g, uint32_t* status)
{
    unsigned int gen = 0u;
    grid_barrier(g, gen, status, GRID_SELFTEST_NS);
}

template <bool MULTI, bool SELFG, bool SCORR, bool XSPH, bool MASKS>
__device__ __forceinline__ bool solve_phases(const PbfK& k, const DomDev* __restrict__ doms,
                                             const int32_t* __restrict__ dom, const uint32_t* __restrict__ start,
                                             float4* __restrict__ xd_a, float4* __restrict__ xd_b,
                                             float2* x_out, float* __restrict__ lam,
                                             const uint32_t* __restrict__ pair_id, float2* __restrict__ v,
                                             float* __restrict__ omega, int32_t iters, GridSync* __restrict__ gs,
                                             unsigned int& gen, uint32_t* __restrict__ status)
{
    const int32_t n      = count_of(k);
    uint32_t tbase       = 0u;
    float4* cur          = xd_a;
    float4* nxt          = xd_b;
    constexpr int MU = MASKS ? MASK_USE : MASK_OFF;
    for (int32_t it = 0; it < iters; ++it) {
        if (MASKS && it == 0) {
            for_blocks(gs, tbase, n, [&](int32_t i) {
                lambda_one<MULTI, SELFG, ACC_NONE, true, MASK_BUILD>(k, doms, dom, start, cur, lam, pair_id, nullptr, i);
            });
        } else {
            for_blocks(gs, tbase, n, [&](int32_t i) {
                lambda_one<MULTI, SELFG, ACC_NONE, true, MU>(k, doms, dom, start, cur, lam, pair_id, nullptr, i);
            });
        }
        if (!grid_barrier(gs, gen, status)) { return false; }
        for_blocks(gs, tbase, n, [&](int32_t i) {
            delta_p_one<MULTI, SCORR, false, true, MU>(k, doms, dom, start, cur, lam, nxt, nullptr, i);
        });
        if (!grid_barrier(gs, gen, status)) { return false; }
        float4* t = cur;
        cur       = nxt;
        nxt       = t;
    }
    if (XSPH) {
        for_blocks(gs, tbase, n, [&](int32_t i) {
            xsph_one<MULTI, false, true, MU>(k, doms, dom, start, cur, x_out, v, omega, status, i);
        });
    }
    return true;
}

template <bool MULTI, bool SELFG, bool SCORR, bool XSPH, bool MASKS>
__global__ void __launch_bounds__(T_MAX, 3)
    k_solve_persistent(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
                       const uint32_t* __restrict__ start, float4* __restrict__ xd_a, float4* __restrict__ xd_b,
                       float2* __restrict__ x_out, float* __restrict__ lam, const uint32_t* __restrict__ pair_id,
                       float2* __restrict__ v, float* __restrict__ omega, int32_t iters, GridSync* __restrict__ gs,
                       uint32_t* __restrict__ status)
{
    unsigned int gen = 0u; // the barrier word is zeroed before every launch
    solve_phases<MULTI, SELFG, SCORR, XSPH, MASKS>(k, doms, dom, start, xd_a, xd_b, x_out, lam, pair_id, v, omega,
                                                   iters, gs, gen, status);
}

// ----- the whole step in one persistent launch ------------------------------------------------------------
// Predict + cell histogram, the scan of the histogram, the bucket scatter and the stable placement (the
// same algorithm as the separate sort launches, so keys and order are the same bit for bit), then the
// solve phases, all separated by grid barriers: a step is one cooperative launch (plus the barrier word's
// reset). The scan works on tiles of STEP_TILE cells; each block adds up the tile totals before its tile
// itself, as the separate scan does while the tiles are few.
constexpr int STEP_TILE = 2048;

// exclusive scan of one value per thread across the block (any multiple of 32 threads up to 1024); the
// block total in *total
__device__ __forceinline__ uint32_t block_excl_scan_any(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) { inc += t; }
    }
    if (lane == 31) { s_warp[warp] = inc; }
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) { w += t; }
        }
        if (lane < nw) { s_warp[lane] = w; }
    }
    __syncthreads();
    const uint32_t before = warp ? s_warp[warp - 1] : 0u;
    *total                = s_warp[nw - 1];
    __syncthreads();
    return before + inc - v;
}

struct SortBufs {
    float2* x;               // current positions (unsorted order); the step's end positions (sorted) replace them
    const float2* v;         // velocities (unsorted order)
    uint2* keyrank;
    uint32_t* count;         // histogram, zero on entry and on exit
    uint32_t* bsum;          // tile totals
    uint32_t* start;         // cell starts (ncells + 1)
    uint32_t* bucket;
    float4* xd_sorted;       // placed (x, d) records (the solve's first input)
    uint32_t* perm;
    uint32_t* keys;
    const uint32_t* id_in;   // ids to carry (or null)
    uint32_t* id_out;
    uint8_t* mflag;          // candidate-mask cell marks to clear (or null)
    uint32_t ncells;
};

template <bool MULTI, bool SELFG, bool SCORR, bool XSPH, bool MASKS>
__global__ void __launch_bounds__(T_MAX, 3)
    k_step_persistent(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
                      const SortBufs sb, float4* __restrict__ xd_b, float* __restrict__ lam,
                      const uint32_t* __restrict__ pair_id, float2* __restrict__ v_out, float* __restrict__ omega,
                      int32_t iters, GridSync* __restrict__ gs, uint32_t* __restrict__ status)
{
    __shared__ uint32_t s_tile[STEP_TILE];
    const int32_t n      = count_of(k);
    const int32_t stride = (int32_t)(gridDim.x * blockDim.x);
    const int32_t i0     = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
    unsigned int gen     = 0u; // the barrier word is zeroed before every launch
    const uint32_t M     = sb.ncells;
    const uint32_t tiles = (M + STEP_TILE - 1) / STEP_TILE;
    // predict, cell key and histogram (whole blocks iterate together: the warp ranks need full warps)
    for (int32_t base = (int32_t)(blockIdx.x * blockDim.x); base < n; base += stride) {
        const int32_t i = base + (int32_t)threadIdx.x;
        predict_hist_one<MULTI>(k, doms, dom, sb.x, sb.v, sb.keyrank, sb.count, i, i < n);
    }
    if (MASKS) {
        for (uint32_t c = (uint32_t)i0; c < M; c += (uint32_t)stride) { sb.mflag[c] = 0u; }
    }
    if (!grid_barrier(gs, gen, status)) { return; }
    // tile totals
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        uint32_t s = 0u;
        for (uint32_t c = t * STEP_TILE + threadIdx.x; c < min((t + 1) * STEP_TILE, M); c += blockDim.x) {
            s += __ldcg(&sb.count[c]);
        }
        uint32_t total;
        block_excl_scan_any(s, &total);
        if (threadIdx.x == 0) { sb.bsum[t] = total; }
    }
    if (!grid_barrier(gs, gen, status)) { return; }
    // exclusive scan: cell starts, and the histogram is zeroed for the next sort
    const uint32_t per = STEP_TILE / blockDim.x; // cells per thread, consecutive
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        uint32_t part = 0u;
        for (uint32_t b = threadIdx.x; b < t; b += blockDim.x) { part += __ldcg(&sb.bsum[b]); }
        uint32_t prefix;
        block_excl_scan_any(part, &prefix);
        const uint32_t base = t * STEP_TILE;
        for (uint32_t li = threadIdx.x; li < STEP_TILE; li += blockDim.x) {
            const uint32_t c = base + li;
            uint32_t cnt     = 0u;
            if (c < M) {
                cnt         = __ldcg(&sb.count[c]);
                sb.count[c] = 0u;
            }
            s_tile[li] = cnt;
        }
        __syncthreads();
        uint32_t s = 0u;
        for (uint32_t q = 0; q < per; ++q) {
            const uint32_t c = s_tile[threadIdx.x * per + q];
            s_tile[threadIdx.x * per + q] = s;
            s += c;
        }
        uint32_t total;
        const uint32_t ex = block_excl_scan_any(s, &total);
        for (uint32_t q = 0; q < per; ++q) { s_tile[threadIdx.x * per + q] += prefix + ex; }
        __syncthreads();
        for (uint32_t li = threadIdx.x; li < STEP_TILE; li += blockDim.x) {
            if (base + li < M) { sb.start[base + li] = s_tile[li]; }
        }
        if (t == tiles - 1u && threadIdx.x == 0) { sb.start[M] = prefix + total; }
        __syncthreads();
    }
    if (!grid_barrier(gs, gen, status)) { return; }
    // bucket scatter
    for (int32_t i = i0; i < n; i += stride) {
        const uint2 kr                        = __ldcg(&sb.keyrank[i]);
        sb.bucket[__ldcg(&sb.start[kr.x]) + kr.y] = (uint32_t)i;
    }
    if (!grid_barrier(gs, gen, status)) { return; }
    // stable placement and gather
    for (int32_t i = i0; i < n; i += stride) {
        place_one<true>(k, sb.keyrank, sb.start, sb.bucket, sb.x, sb.v, sb.xd_sorted, nullptr, nullptr, sb.perm,
                        sb.keys, sb.id_in, sb.id_out, nullptr, nullptr, nullptr, i);
    }
    // (every block has read its unsorted positions before this barrier; XSPH overwrites them later)
    if (!grid_barrier(gs, gen, status)) { return; }
    solve_phases<MULTI, SELFG, SCORR, XSPH, MASKS>(k, doms, dom, sb.start, sb.xd_sorted, xd_b, sb.x, lam, pair_id,
                                                   v_out, omega, iters, gs, gen, status);
}

// ----- density for the density-error metric --------------------------------------------------------------
template <bool MULTI>
__global__ void __launch_bounds__(T_PART)
    k_density(const PbfK k, const DomDev* __restrict__ doms, const int32_t* __restrict__ dom,
              const uint32_t* __restrict__ start, const float2* __restrict__ xs, float* __restrict__ rho_out,
              float* __restrict__ red)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float e         = 0.f;
    if (i < count_of(k)) {
        const DomDev d = load_dom<MULTI>(k, doms, dom, i);
        const float2 p = xs[i];
        float s6       = 0.f;
        for_neighbours(d, k, start, p.x, p.y, [&](uint32_t j) {
            const float2 q = __ldg(&xs[j]);
            const float rx = p.x - q.x, ry = p.y - q.y;
            const float r2 = fmaf(rx, rx, ry * ry);
            const float qq = (r2 <= k.h2) ? k.h2 - r2 : 0.f;
            s6             = fmaf(qq * qq, qq, s6);
        });
        const float rho = k.mass * k.c6 * s6;
        rho_out[i] = rho;
        e          = fmaxf(rho * k.inv_rho0 - 1.f, 0.f);
    }
    // block max and sum, then one atomic each (e >= 0 so its bits order like unsigned ints)
    float mx = e, sm = e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    __shared__ float s_mx[T_PART / 32], s_sm[T_PART / 32];
    if ((threadIdx.x & 31) == 0) {
        s_mx[threadIdx.x >> 5] = mx;
        s_sm[threadIdx.x >> 5] = sm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bm = 0.f, bs = 0.f;
        for (int w = 0; w < T_PART / 32; ++w) {
            bm = fmaxf(bm, s_mx[w]);
            bs += s_sm[w];
        }
        atomicMax(reinterpret_cast<unsigned int*>(&red[0]), __float_as_uint(bm));
        atomicAdd(reinterpret_cast<double*>(&red[2]), (double)bs);
    }
}

__global__ void k_check_domains(const int32_t* __restrict__ dom, int32_t n, int32_t nd, uint32_t* status)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) { return; }
    const int32_t d = dom[i];
    if (d < 0 || d >= nd || (i + 1 < n && dom[i + 1] < d)) { atomicOr(status, GPE_STATUS_CAPACITY); }
}

__global__ void k_set_count(int32_t* __restrict__ c, int32_t n) { *c = n; }

// ----- hose emitter (emitterKernel, PBF.cu:968-1032): appends at the device count -------------------------
__global__ void k_pbf_emit(const PbfK k, const HoseK h, float2* __restrict__ x, float2* __restrict__ v,
                           int32_t* __restrict__ count, int32_t cap, uint32_t* __restrict__ ids,
                           uint32_t* __restrict__ status)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= h.count) { return; }
    float2 p = hose_position(h, i);
    // atoms outside the scene are dropped (PBF.cu:1014-1016); the rest are kept inside the walls
    const DomDev& d = k.d0;
    const bool in   = p.x >= d.lox && p.y >= d.loy && p.x < d.hix + k.margin && p.y < d.hiy + k.margin;
    p.x             = fminf(p.x, d.hix);
    p.y             = fminf(p.y, d.hiy);
    float vx = h.vx, vy = h.vy;
    if (k.flags & GPE_PBF_VEL_CLAMP) {
        // velocityClamp, as emitterKernel applies to the stream velocity (PBF.cu:990-991)
        const float v2  = fmaf(vx, vx, vy * vy);
        const float inv = (v2 < k.v_min2 || v2 == 0.f) ? 0.f : rsqrtf(v2);
        const float sp  = fminf(v2 * inv, k.v_max);
        vx *= inv * sp;
        vy *= inv * sp;
    }
    const int32_t slot = append_slot(count, in);
    if (slot < 0) { return; }
    if (slot >= cap) {
        atomicOr(status, GPE_STATUS_CAPACITY);
        atomicMin(count, cap);
        return;
    }
    x[slot] = p;
    v[slot] = make_float2(vx, vy);
    if (ids) { ids[slot] = (uint32_t)slot; }
}

// ----- publish to a chunk-major view (PBFOutputKernel, PBF.cu:861-896) ------------------------------------
// The target is `vv`, or the struct at `vp` in device memory when vp is set (read when the kernel runs).
__global__ void k_view_zero(const gpe_view* __restrict__ vp)
{
    const gpe_view view = *vp;
    const int32_t nc    = view.chunks_x * view.chunks_y;
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        view.counts[c] = 0;
    }
}

// One block publishes PUB_PER_BLOCK consecutive particles. The chunk counters of a view sit side by side in
// one cache line, so one returning atomic per particle (or per warp) queues at one L2 slice. Here the lanes
// of a warp bound for the same chunk form a group (match_any); the group's first lane ranks the group in a
// shared-memory table of the block's chunks (open addressing over PUB_SLOTS slots), the block takes one
// global atomic per chunk it touches, and each particle is written at that base plus its rank. Particles
// past chunk_capacity give their slots back, so a full chunk ends at chunk_capacity as with one atomic per
// particle; slot order within a chunk depends on scheduling either way. A group that finds the table full
// (more than PUB_SLOTS chunks in one block) takes its own global atomic.
constexpr int32_t PUB_PER_THREAD = 4, PUB_PER_BLOCK = PUB_PER_THREAD * T_PART, PUB_SLOTS = 64;

__global__ void __launch_bounds__(T_PART)
    k_pbf_publish(const PbfK k, const gpe_view vv, const gpe_view* __restrict__ vp, const float2* __restrict__ x,
                  const float2* __restrict__ v, uint32_t* __restrict__ status)
{
    __shared__ int32_t key[PUB_SLOTS], cnt[PUB_SLOTS], base[PUB_SLOTS];
    const gpe_view view = vp ? *vp : vv;
    const int32_t n     = count_of(k);
    const int32_t i0    = blockIdx.x * PUB_PER_BLOCK + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    for (int32_t t = threadIdx.x; t < PUB_SLOTS; t += blockDim.x) {
        key[t] = -1;
        cnt[t] = 0;
    }
    __syncthreads();
    const float inv = 1.f / view.chunk_dim;
    int32_t c[PUB_PER_THREAD], slot[PUB_PER_THREAD], rank[PUB_PER_THREAD];
    float2 p[PUB_PER_THREAD];
#pragma unroll
    for (int32_t j = 0; j < PUB_PER_THREAD; ++j) {
        const int32_t i = i0 + j * T_PART;
        c[j]            = -1;
        if (i < n) {
            p[j]             = x[i];
            const int32_t cx = min(max((int32_t)floorf((p[j].x - k.d0.ox) * inv), 0), view.chunks_x - 1);
            const int32_t cy = min(max((int32_t)floorf((p[j].y - k.d0.oy) * inv), 0), view.chunks_y - 1);
            c[j]             = cx + cy * view.chunks_x;
        }
        const uint32_t group = __match_any_sync(0xffffffffu, c[j]);
        const int32_t leader = __ffs(group) - 1;
        const int32_t size   = __popc(group);
        int32_t h = -1, r = 0;
        if ((int32_t)lane == leader && c[j] >= 0) {
            int32_t probe = 0;
            for (h = (int32_t)(((uint32_t)c[j] * 2654435761u) >> 26); probe < PUB_SLOTS;
                 ++probe, h = (h + 1) & (PUB_SLOTS - 1)) {
                const int32_t old = atomicCAS(&key[h], -1, c[j]);
                if (old == -1 || old == c[j]) { break; }
            }
            if (probe < PUB_SLOTS) {
                r = atomicAdd(&cnt[h], size);
            } else { // table full: the group's own global slots
                h                  = -1;
                r                  = atomicAdd(&view.counts[c[j]], size);
                const int32_t over = min(r + size - view.chunk_capacity, size);
                if (over > 0) {
                    atomicOr(status, GPE_STATUS_CAPACITY);
                    atomicSub(&view.counts[c[j]], over);
                }
            }
        }
        slot[j] = __shfl_sync(0xffffffffu, h, leader);
        rank[j] = __shfl_sync(0xffffffffu, r, leader) + __popc(group & ((1u << lane) - 1u));
    }
    __syncthreads();
    for (int32_t t = threadIdx.x; t < PUB_SLOTS; t += blockDim.x) {
        if (key[t] < 0) { continue; }
        const int32_t b    = atomicAdd(&view.counts[key[t]], cnt[t]);
        const int32_t over = min(b + cnt[t] - view.chunk_capacity, cnt[t]);
        if (over > 0) {
            atomicOr(status, GPE_STATUS_CAPACITY);
            atomicSub(&view.counts[key[t]], over);
        }
        base[t] = b;
    }
    __syncthreads();
#pragma unroll
    for (int32_t j = 0; j < PUB_PER_THREAD; ++j) {
        if (c[j] < 0) { continue; }
        const int32_t sl = slot[j] >= 0 ? base[slot[j]] + rank[j] : rank[j];
        if (sl >= view.chunk_capacity) { continue; }
        const size_t o                         = (size_t)c[j] * (size_t)view.chunk_capacity + (size_t)sl;
        reinterpret_cast<float2*>(view.pos)[o] = p[j];
        reinterpret_cast<float2*>(view.vel)[o] = v[i0 + j * T_PART];
    }
}

// ----- chunk-major state, the reference's PBFArena layout (gpe_pbf_publish_chunks) ---------------------
// After a step the reference's arena holds, per chunk of the scene, its atoms sorted by the cell of their
// next prediction (prepNextSubstepKernel, PBF.cu:786-833): x and x* in chunk-local coordinates, the
// displacement, and per cell the packed range (end << 16) | start (PBF.cu:814-817). An atom belongs to the
// chunk of its prediction (migration, PBF.cu:639-737); within a cell the order follows atomics, as there.
// The cell histogram is accumulated in the caller's offsets array, which the scan then overwrites.
__device__ __forceinline__ int32_t chunk_cell_key(const PbfK& k, const gpe_chunk_state& c, float2 xs, int32_t* chunk,
                                                  float2* org)
{
    const float inv  = 1.f / c.chunk_dim;
    const int32_t cx = min(max((int32_t)floorf((xs.x - k.d0.ox) * inv), 0), c.chunks_x - 1);
    const int32_t cy = min(max((int32_t)floorf((xs.y - k.d0.oy) * inv), 0), c.chunks_y - 1);
    *org             = make_float2(k.d0.ox + (float)cx * c.chunk_dim, k.d0.oy + (float)cy * c.chunk_dim);
    const float cell = c.chunk_dim / (float)c.chunk_cells;
    const int32_t gx = min(max((int32_t)floorf((xs.x - org->x) / cell), 0), c.chunk_cells - 1);
    const int32_t gy = min(max((int32_t)floorf((xs.y - org->y) / cell), 0), c.chunk_cells - 1);
    *chunk           = cx + cy * c.chunks_x;
    return *chunk * c.chunk_cells * c.chunk_cells + gx + gy * c.chunk_cells;
}

__global__ void __launch_bounds__(T_PART)
    k_chunk_hist(const PbfK k, const gpe_chunk_state c, const float2* __restrict__ x, const float2* __restrict__ v,
                 uint2* __restrict__ keyrank)
{
    const int32_t i  = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < count_of(k);
    int32_t key      = -1;
    if (valid) {
        int32_t ch;
        float2 org;
        key = chunk_cell_key(k, c, predict(k, x[i], v[i]), &ch, &org);
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const int32_t leader = __ffs(peers) - 1;
    const int32_t lane   = threadIdx.x & 31;
    uint32_t base        = 0;
    if (valid && lane == leader) { base = atomicAdd(&c.offsets[key], (uint32_t)__popc(peers)); }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (valid) { keyrank[i] = make_uint2((uint32_t)key, base + (uint32_t)__popc(peers & ((1u << lane) - 1u))); }
}

// one block of 1024 threads per chunk: the cell counts become packed (end << 16) | start, capped at the
// chunk capacity
__global__ void __launch_bounds__(1024) k_chunk_scan(const gpe_chunk_state c, uint32_t* __restrict__ status)
{
    const int32_t cells = c.chunk_cells * c.chunk_cells;
    __shared__ uint32_t s_warp[32];
    uint32_t* off    = c.offsets + (size_t)blockIdx.x * (size_t)cells;
    const uint32_t v = (int32_t)threadIdx.x < cells ? off[threadIdx.x] : 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) { inc += t; }
    }
    if (lane == 31) { s_warp[warp] = inc; }
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) { w += t; }
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t end   = inc + (warp ? s_warp[warp - 1] : 0u);
    const uint32_t start = end - v;
    const uint32_t cap   = (uint32_t)c.chunk_capacity;
    if ((int32_t)threadIdx.x < cells) { off[threadIdx.x] = (min(end, cap) << 16) | min(start, cap); }
    if ((int32_t)threadIdx.x == cells - 1) {
        c.counts[blockIdx.x] = (int32_t)min(end, cap);
        if (end > cap) { atomicOr(status, GPE_STATUS_CAPACITY); }
    }
}

__global__ void __launch_bounds__(T_PART)
    k_chunk_place(const PbfK k, const gpe_chunk_state c, const float2* __restrict__ x, const float2* __restrict__ v,
                  const float* __restrict__ lam, const uint2* __restrict__ keyrank)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count_of(k)) { return; }
    const float2 p  = x[i];
    const float2 w  = v[i];
    const float2 xs = predict(k, p, w);
    int32_t ch;
    float2 org;
    (void)chunk_cell_key(k, c, xs, &ch, &org);
    const uint2 kr     = keyrank[i];
    const uint32_t o   = c.offsets[kr.x];
    const uint32_t sl  = (o & 0xFFFFu) + kr.y;
    if (sl >= (o >> 16)) { return; } // past the chunk's capacity (reported by the scan)
    const size_t q                        = (size_t)ch * (size_t)c.chunk_capacity + sl;
    reinterpret_cast<float2*>(c.pos)[q]   = make_float2(p.x - org.x, p.y - org.y);
    reinterpret_cast<float2*>(c.pred)[q]  = make_float2(xs.x - org.x, xs.y - org.y);
    reinterpret_cast<float2*>(c.vel)[q]   = w;
    if (c.lambda) { c.lambda[q] = lam[i]; }
}

__global__ void k_iota(uint32_t* __restrict__ a, int32_t n)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { a[i] = (uint32_t)i; }
}

} // namespace

} // namespace gpe

// =====================================================================================================
// Engine object
// =====================================================================================================

using namespace gpe;

struct PbfGraph {
    cudaGraphExec_t exec = nullptr;
    int id_end;
    bool hist_end; // the last step's XSPH left the next step's keys and histogram
};

struct gpe_pbf {
    int device = 0;
    gpe_pbf_params prm{};
    PbfK k{};
    int32_t nd = 0;
    std::vector<gpe_domain> doms;
    std::vector<DomDev> domdev;
    int64_t cap = 0, n = 0;
    uint32_t ncells = 0;
    uint64_t cells_cap = 0; // cell arrays are sized for this many cells

    void* base        = nullptr;
    DomDev* d_doms    = nullptr;
    float2* pos       = nullptr; // positions between steps (after a step: that step's sorted order)
    float4* xd[2]     = {};      // within a step: sorted (x, d) records, the current and the next
    float2* vel       = nullptr;
    float* lam        = nullptr;
    float* omega      = nullptr;
    float* rho        = nullptr;
    uint2* keyrank    = nullptr;
    uint32_t* bucket  = nullptr;
    uint32_t* count   = nullptr;
    uint32_t* start   = nullptr;
    uint32_t* bsum    = nullptr;
    uint32_t* perm    = nullptr;
    uint32_t* keys    = nullptr;
    int32_t* dom      = nullptr;
    uint32_t* ids[2]  = {};
    uint32_t* status  = nullptr;
    float* red        = nullptr;
    int32_t* d_count  = nullptr; // device-resident particle count
    bool dynamic      = false;   // GPE_PBF_DYNAMIC_COUNT: launches cover the capacity
    float* acc        = nullptr; // summed multiplier of the current step (sorted order of the step)
    float* prev       = nullptr; // the previous step's sum, carried into the current sorted order
    int32_t warm      = GPE_WARM_NONE;
    const gpe_mlp* mlp = nullptr;
    bool collecting   = false;   // gpe_mlp_collect: cold solve with summed multipliers and pair capture
    CollectK col{};
    bool pending_accinit = false; // stage API: the next DELTA_P starts the running sum
    bool mem_valid    = false;    // the multiplier memory holds a previous step's sums (else it is 0)
    int32_t lam_grid  = 0;        // persistent grid of k_mlp_apply
    int32_t block     = 256;      // threads per block of the neighbour kernels (tuning)
    bool persistent   = false;    // plain steps run their passes in one persistent launch (tuning)
    bool step_kernel  = false;    // ... and the predict + sort phases in that same launch (tuning)
    int32_t coop_grid = 0;        // blocks of the persistent launch (all resident)
    const void* coop_fn = nullptr; // the kernel coop_grid was sized for
    GridSync* gsync   = nullptr;  // its barrier word
    uint16_t* feat    = nullptr;  // network operand tiles (GPE_WARM_MLP), allocated on demand
    float skin        = 0.075f;   // candidate-mask skin in units of h (tuning; 0: full scans only)
    uint4* nmask      = nullptr;  // candidate masks of the current step
    uint8_t* mflag    = nullptr;  // per cell: a particle of its 3 x 3 cells moved too far for the masks
    bool masks_valid  = false;    // the masks were made in this step
    bool hist_ready   = false;    // the last step's XSPH left the next step's cell keys and histogram
    bool count_dirty  = false;    // ... and was dropped: the histogram array must be cleared before a sort
    int32_t dp_since_build = 0;   // delta p passes since they were made
    int32_t mask_passes = 1;      // delta p passes the move threshold k.move2 allows for

    // within a step (after PREDICT_SORT): XS = the current (x, d) records, XO = the other buffer; -1 between steps
    int XS = -1, XO = -1;
    int id_cur        = 0;
    bool have_state   = false;
    bool have_sort    = false;
    int32_t launches  = 0;
    std::map<std::tuple<int, int, int>, PbfGraph> graphs;

    void drop_graphs()
    {
        for (auto& g : graphs) {
            if (g.second.exec) { cudaGraphExecDestroy(g.second.exec); }
        }
        graphs.clear();
    }
};

namespace {

bool multi(const gpe_pbf* s) { return s->nd > 1; }
// steps that keep the summed multiplier: warm-started steps and training-pair collection
bool accumulating(const gpe_pbf* s) { return s->warm != GPE_WARM_NONE || s->collecting; }

int32_t validate_params(const gpe_pbf_params* p)
{
    if (!p) { return GPE_ERR_BAD_ARG; }
    if (!(p->h > 0.f) || !(p->rho0 > 0.f) || !(p->mass > 0.f) || !(p->dt > 0.f) || p->iters < 0 ||
        p->iters > 1000 || !(p->eps >= 0.f) || p->cell < 0.f) {
        gpe::set_error(GPE_ERR_BAD_ARG, "invalid PBF parameters (h, rho0, mass, dt must be > 0, iters in [0,1000])");
        return GPE_ERR_BAD_ARG;
    }
    const float cell = p->cell > 0.f ? p->cell : p->h;
    if (cell < 0.2f * p->h) {
        gpe::set_error(GPE_ERR_BAD_ARG, "cell size below h/5 is not supported");
        return GPE_ERR_BAD_ARG;
    }
    return GPE_OK;
}

// kernel constants; the float products follow the reference's constexpr evaluation order
PbfK make_k(const gpe_pbf_params& p)
{
    PbfK k{};
    const float cell = p.cell > 0.f ? p.cell : p.h;
    k.h              = p.h;
    k.h2             = p.h * p.h;
    const double hd  = p.h;
    k.c6             = p.poly6_coeff > 0.f ? p.poly6_coeff : (float)(4.0 / (M_PI * std::pow(hd, 8)));
    k.cs             = p.spiky_coeff > 0.f ? p.spiky_coeff : (float)(30.0 / (M_PI * std::pow(hd, 5)));
    const float d    = k.h2 - p.scorr_dq * p.scorr_dq;
    k.inv_w_dq       = 1.f / (k.c6 * d * d * d);
    k.inv_cell       = 1.0f / cell;
    k.rho0           = p.rho0;
    k.inv_rho0       = 1.f / p.rho0;
    k.mass           = p.mass;
    k.inv_mass       = 1.f / p.mass;
    k.dt             = p.dt;
    k.inv_dt         = 1.f / p.dt;
    const float dt2  = p.dt * p.dt;
    k.g2x            = dt2 * p.gravity[0];
    k.g2y            = dt2 * p.gravity[1];
    k.eps            = p.eps;
    k.scorr_k        = p.scorr_k;
    k.dp_scale       = p.omega * k.inv_mass * k.inv_rho0;
    k.c_min          = p.c_min;
    k.xsph_c         = p.xsph_c;
    k.vort_eps       = p.vort_eps;
    k.vort_dt        = p.dt * p.vort_eps;
    k.v_max          = p.v_max;
    k.v_min2         = p.v_min * p.v_min;
    int32_t R        = (int32_t)std::ceil(p.h / cell - 1e-4f);
    k.R              = R < 1 ? 1 : R;
    k.flags          = p.flags;
    k.margin         = p.wall_margin;
    return k;
}

// the engine's buffers and mask thresholds in the kernel constants
void bind_k(gpe_pbf* s)
{
    s->k.n_dev       = s->d_count;
    s->k.ncells      = s->ncells;
    s->k.keys        = s->keys;
    s->k.nmask       = s->nmask;
    s->k.mflag       = s->mflag;
    const float skin = s->skin * s->prm.h;
    s->k.skin2       = (s->prm.h + skin) * (s->prm.h + skin);
    // each of the step's delta p passes may move a particle by less than this, so all of them together
    // by less than skin / 2 (with 5% to spare for rounding)
    s->mask_passes   = std::max(s->prm.iters, 1);
    const float mv   = 0.95f * skin / (2.f * (float)s->mask_passes);
    s->k.move2       = mv * mv;
}

// masks in this engine's configuration: cell h (3 x 3 scan), a skin, at least one iteration
bool masks_on(const gpe_pbf* s) { return s->skin > 0.f && s->k.R == 1 && s->prm.iters > 0; }

// Cells along one edge of a scene; -1 when extent / cell is not finite or reaches 2^30 (the cast to int32
// would be undefined there). Scene extents are checked to be > 0 before this is called.
constexpr double MAX_CELLS_ALONG = (double)(1u << 30);
int32_t cells_along(float extent, float cell)
{
    const double c = std::ceil((double)(extent / cell));
    if (!(c < MAX_CELLS_ALONG)) { return -1; } // also false for NaN
    return c < 1.0 ? 1 : (int32_t)c;
}

void build_domains(gpe_pbf* s)
{
    const float cell = s->prm.cell > 0.f ? s->prm.cell : s->prm.h;
    s->domdev.resize((size_t)s->nd);
    uint64_t off = 0;
    for (int32_t d = 0; d < s->nd; ++d) {
        DomDev& o = s->domdev[(size_t)d];
        o         = DomDev{};
        o.ox      = s->doms[(size_t)d].origin[0];
        o.oy      = s->doms[(size_t)d].origin[1];
        o.lox     = s->doms[(size_t)d].origin[0];
        o.loy     = s->doms[(size_t)d].origin[1];
        o.hix     = (s->doms[(size_t)d].origin[0] + s->doms[(size_t)d].extent[0]) - s->prm.wall_margin;
        o.hiy     = (s->doms[(size_t)d].origin[1] + s->doms[(size_t)d].extent[1]) - s->prm.wall_margin;
        o.ncx     = cells_along(s->doms[(size_t)d].extent[0], cell);
        o.ncy     = cells_along(s->doms[(size_t)d].extent[1], cell);
        o.coff    = (uint32_t)off;
        off += (uint64_t)o.ncx * (uint64_t)o.ncy;
    }
    s->ncells  = (uint32_t)off;
    s->k       = make_k(s->prm);
    s->k.d0    = s->domdev[0];
    bind_k(s);
}

// Launch size: with a device-resident count that emitters can grow inside a captured graph, every launch
// covers the capacity and the kernels read the live count; otherwise the host count.
int64_t lsize(const gpe_pbf* s) { return s->dynamic ? s->cap : s->n; }

// Refreshes the host copy of the particle count from the device (only needed with a dynamic count).
int32_t sync_count(gpe_pbf* s, cudaStream_t st)
{
    if (!s->dynamic) { return GPE_OK; }
    int32_t c = 0;
    GPE_TRY_CUDA(cudaMemcpyAsync(&c, s->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    s->n = c;
    return GPE_OK;
}

// Total sort cells of the scenes; CELLS_INVALID when a scene's extent / cell is not finite or too large.
constexpr uint64_t CELLS_INVALID = ~(uint64_t)0;
uint64_t count_cells(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd)
{
    const float cell = p->cell > 0.f ? p->cell : p->h;
    uint64_t off     = 0;
    for (int32_t d = 0; d < nd; ++d) {
        const int32_t cx = cells_along(doms[d].extent[0], cell);
        const int32_t cy = cells_along(doms[d].extent[1], cell);
        if (cx < 0 || cy < 0) { return CELLS_INVALID; }
        off += (uint64_t)cx * (uint64_t)cy;
    }
    return off;
}

unsigned blocks_for(int64_t n) { return (unsigned)((n + T_PART - 1) / T_PART); }
// blocks of a neighbour-kernel launch at the tuned block size
unsigned nblk(const gpe_pbf* s) { return (unsigned)((lsize(s) + s->block - 1) / s->block); }

// ----- stage launchers ----------------------------------------------------------------------------------

// A call other than a step may change what the next step sorts (positions, velocities, count, parameters,
// cells): a histogram left by the last step's XSPH is dropped, and the next sort clears the histogram
// array before building its own (clear_hist).
void drop_hist(gpe_pbf* s)
{
    if (s->hist_ready) {
        s->hist_ready  = false;
        s->count_dirty = true;
    }
}

int32_t clear_hist(gpe_pbf* s, cudaStream_t st)
{
    if (s->count_dirty) {
        GPE_TRY_CUDA(cudaMemsetAsync(s->count, 0, sizeof(uint32_t) * (size_t)s->cells_cap, st));
        s->count_dirty = false;
    }
    return GPE_OK;
}

int32_t stage_predict_sort(gpe_pbf* s, cudaStream_t st)
{
    s->masks_valid  = false;
    const int32_t n = (int32_t)lsize(s);
    s->XS           = 0;
    s->XO           = 1;
    s->k.n = (int32_t)s->n;
    // the previous step's XSPH may already have computed the keys and the histogram (hist_ready)
    const bool fused = s->hist_ready;
    s->hist_ready    = false;
    const int32_t rch = clear_hist(s, st);
    if (rch) { return rch; }
    if (n > 0 && !fused) {
        if (multi(s)) {
            k_predict_hist<true><<<blocks_for(n), T_PART, 0, st>>>(s->k, s->d_doms, s->dom, s->pos, s->vel,
                                                                   s->keyrank, s->count);
        } else {
            k_predict_hist<false><<<blocks_for(n), T_PART, 0, st>>>(s->k, s->d_doms, s->dom, s->pos, s->vel,
                                                                    s->keyrank, s->count);
        }
        GPE_CHECK_LAUNCH("k_predict_hist");
    }
    // the scan also clears the candidate masks' cell marks for this step
    int32_t rc = launch_exclusive_scan(s->count, s->ncells, s->bsum, s->start, st, masks_on(s) ? s->mflag : nullptr);
    if (rc) { return rc; }
    rc = launch_scatter(s->keyrank, n, s->start, s->bucket, (uint32_t)s->ncells, st, s->d_count);
    if (rc) { return rc; }
    if (n > 0) {
        const bool ids = (s->prm.flags & (GPE_PBF_TRACK_IDS | GPE_PBF_PAIR_IDS)) != 0;
        k_place<<<blocks_for(n), T_PART, 0, st>>>(s->k, s->keyrank, s->start, s->bucket, s->pos, s->vel,
                                                  s->xd[s->XS], nullptr, nullptr, s->perm, s->keys,
                                                  ids ? s->ids[s->id_cur] : nullptr,
                                                  ids ? s->ids[s->id_cur ^ 1] : nullptr,
                                                  accumulating(s) ? s->acc : nullptr, s->prev,
                                                  (s->warm == GPE_WARM_PREV && !s->collecting) ? s->lam : nullptr);
        GPE_CHECK_LAUNCH("k_place");
        if (ids) { s->id_cur ^= 1; }
    }
    s->have_sort = true;
    s->launches += (fused ? 2 : 3) + scan_launches(s->ncells); // [predict + histogram,] scan, scatter, place
    return GPE_OK;
}

// Template dispatch tables: [multi scene][flag][accumulation mode]
using LamFn = cudaError_t (*)(unsigned, unsigned, cudaStream_t, const PbfK&, const DomDev*, const int32_t*, const uint32_t*,
                       const float4*, float*, const uint32_t*, float*, int);
template <bool M, bool S, int A>
cudaError_t lam_launch(unsigned g, unsigned blk, cudaStream_t st, const PbfK& k, const DomDev* doms, const int32_t* dom,
                const uint32_t* start, const float4* xs, float* lam, const uint32_t* pid, float* acc, int mask)
{
    if constexpr (A == ACC_PROJ) { // the projected-increment ablation keeps full scans
        k_lambda<M, S, A, MASK_OFF><<<g, blk, 0, st>>>(k, doms, dom, start, xs, lam, pid, acc);
        return cudaGetLastError();
    } else if (mask == MASK_BUILD) {
        k_lambda<M, S, A, MASK_BUILD><<<g, blk, 0, st>>>(k, doms, dom, start, xs, lam, pid, acc);
        return cudaGetLastError();
    } else if (mask == MASK_USE) {
        k_lambda<M, S, A, MASK_USE><<<g, blk, 0, st>>>(k, doms, dom, start, xs, lam, pid, acc);
        return cudaGetLastError();
    } else {
        k_lambda<M, S, A, MASK_OFF><<<g, blk, 0, st>>>(k, doms, dom, start, xs, lam, pid, acc);
        return cudaGetLastError();
    }
}
#define GPE_LAM3(M, S) {lam_launch<M, S, ACC_NONE>, lam_launch<M, S, ACC_SUM>, lam_launch<M, S, ACC_PROJ>}
const LamFn kLam[2][2][3] = {{GPE_LAM3(false, false), GPE_LAM3(false, true)},
                             {GPE_LAM3(true, false), GPE_LAM3(true, true)}};
#undef GPE_LAM3

using DpFn = cudaError_t (*)(unsigned, unsigned, cudaStream_t, const PbfK&, const DomDev*, const int32_t*, const uint32_t*,
                      const float4*, const float*, float4*, float*, int);
template <bool M, bool S, bool A>
cudaError_t dp_launch(unsigned g, unsigned blk, cudaStream_t st, const PbfK& k, const DomDev* doms, const int32_t* dom,
               const uint32_t* start, const float4* xs, const float* lam, float4* out, float* acc, int mask)
{
    if (mask == MASK_USE) {
        k_delta_p<M, S, A, MASK_USE><<<g, blk, 0, st>>>(k, doms, dom, start, xs, lam, out, acc);
        return cudaGetLastError();
    } else {
        k_delta_p<M, S, A, MASK_OFF><<<g, blk, 0, st>>>(k, doms, dom, start, xs, lam, out, acc);
        return cudaGetLastError();
    }
}
const DpFn kDp[2][2][2] = {{{dp_launch<false, false, false>, dp_launch<false, false, true>},
                            {dp_launch<false, true, false>, dp_launch<false, true, true>}},
                           {{dp_launch<true, false, false>, dp_launch<true, false, true>},
                            {dp_launch<true, true, false>, dp_launch<true, true, true>}}};

using FeatFn = void (*)(unsigned, unsigned, cudaStream_t, const PbfK&, const DomDev*, const int32_t*, const uint32_t*,
                        const float4*, const float*, const uint32_t*, const MlpDev*, uint16_t*, int);
template <bool M, bool S>
void feat_launch(unsigned g, unsigned blk, cudaStream_t st, const PbfK& k, const DomDev* doms, const int32_t* dom,
                 const uint32_t* start, const float4* xd, const float* prev, const uint32_t* pid, const MlpDev* mlp,
                 uint16_t* feat, int mask)
{
    if (mask == MASK_BUILD) {
        k_lambda_feat<M, S, MASK_BUILD><<<g, blk, 0, st>>>(k, doms, dom, start, xd, prev, pid, mlp, feat);
    } else {
        k_lambda_feat<M, S, MASK_OFF><<<g, blk, 0, st>>>(k, doms, dom, start, xd, prev, pid, mlp, feat);
    }
}
const FeatFn kFeat[2][2] = {{feat_launch<false, false>, feat_launch<false, true>},
                            {feat_launch<true, false>, feat_launch<true, true>}};

using ColFn = void (*)(unsigned, unsigned, cudaStream_t, const PbfK&, const DomDev*, const int32_t*, const uint32_t*,
                       const float4*, const float*, float*, const uint32_t*, const CollectK&);
template <bool M, bool S>
void col_launch(unsigned g, unsigned blk, cudaStream_t st, const PbfK& k, const DomDev* doms, const int32_t* dom,
                const uint32_t* start, const float4* xd, const float* prev, float* lam, const uint32_t* pid,
                const CollectK& col)
{
    k_lambda_collect<M, S><<<g, blk, 0, st>>>(k, doms, dom, start, xd, prev, lam, pid, col);
}
const ColFn kCol[2][2] = {{col_launch<false, false>, col_launch<false, true>},
                          {col_launch<true, false>, col_launch<true, true>}};

using XsFn = cudaError_t (*)(unsigned, unsigned, cudaStream_t, const PbfK&, const DomDev*, const int32_t*, const uint32_t*,
                      const float4*, float2*, float2*, float*, uint32_t*, int);
template <bool M, bool V>
cudaError_t xs_launch(unsigned g, unsigned blk, cudaStream_t st, const PbfK& k, const DomDev* doms, const int32_t* dom,
               const uint32_t* start, const float4* xd, float2* x_out, float2* v, float* om, uint32_t* status,
               int mask)
{
    if (mask == MASK_USE) {
        k_xsph<M, V, MASK_USE><<<g, blk, 0, st>>>(k, doms, dom, start, xd, x_out, v, om, status);
        return cudaGetLastError();
    } else {
        k_xsph<M, V, MASK_OFF><<<g, blk, 0, st>>>(k, doms, dom, start, xd, x_out, v, om, status);
        return cudaGetLastError();
    }
}
const XsFn kXs[2][2] = {{xs_launch<false, false>, xs_launch<false, true>},
                        {xs_launch<true, false>, xs_launch<true, true>}};

// accumulation mode of the lambda passes after the first in the engine's current mode
int acc_mode(const gpe_pbf* s)
{
    // a network step keeps its own Lambda as the memory; only the step that starts the memory (a plain
    // step with the training solve's iterations) and collection sum their iterations
    if (s->collecting || (s->warm == GPE_WARM_MLP && !s->mem_valid)) { return ACC_SUM; }
    return s->warm == GPE_WARM_PREV ? ACC_PROJ : ACC_NONE;
}

int32_t stage_lambda(gpe_pbf* s, cudaStream_t st, int acc)
{
    if (lsize(s) == 0) { return GPE_OK; }
    const int sg        = (s->prm.flags & GPE_PBF_SELF_GRAD) ? 1 : 0;
    const uint32_t* pid = (s->prm.flags & GPE_PBF_PAIR_IDS) ? s->ids[s->id_cur] : nullptr;
    int mask = MASK_OFF;
    if (masks_on(s) && acc != ACC_PROJ) {
        // the cell marks were cleared by this step's sort (marks left by a stage sequence without one only
        // make scans full, never skip a candidate)
        mask = s->masks_valid ? MASK_USE : MASK_BUILD;
    }
    GPE_TRY_CUDA(kLam[multi(s) ? 1 : 0][sg][acc](nblk(s), (unsigned)s->block, st, s->k, s->d_doms, s->dom, s->start,
                                                 s->xd[s->XS], s->lam, pid, s->acc, mask));
    if (mask == MASK_BUILD) {
        s->masks_valid    = true;
        s->dp_since_build = 0;
    }
    s->launches += 1;
    return GPE_OK;
}

// First lambda pass of an accumulating step: the network (GPE_WARM_MLP), the cold pass with pair capture
// (collection) or nothing (GPE_WARM_PREV: the sort already placed lambda_prev into lambda).
int32_t stage_lambda_warm(gpe_pbf* s, cudaStream_t st)
{
    if (lsize(s) == 0 || (s->warm == GPE_WARM_PREV && !s->collecting)) { return GPE_OK; }
    // a network step needs the memory of a previous step; the first step after a reset runs the plain pass
    // (no pairs taken) and starts the memory
    const int mi        = multi(s) ? 1 : 0;
    const int sg        = (s->prm.flags & GPE_PBF_SELF_GRAD) ? 1 : 0;
    const uint32_t* pid = (s->prm.flags & GPE_PBF_PAIR_IDS) ? s->ids[s->id_cur] : nullptr;
    if (s->warm == GPE_WARM_MLP && s->mem_valid && !s->collecting) {
        const gpe::MlpDev* md = gpe::mlp_device(s->mlp);
        // the feature pass scans every neighbour on the sorted positions: it makes the step's masks
        const int mask = masks_on(s) ? MASK_BUILD : MASK_OFF;
        kFeat[mi][sg](nblk(s), (unsigned)s->block, st, s->k, s->d_doms, s->dom, s->start, s->xd[s->XS], s->prev, pid,
                      md, s->feat, mask);
        GPE_CHECK_LAUNCH("k_lambda_feat");
        if (mask == MASK_BUILD) {
            s->masks_valid    = true;
            s->dp_since_build = 0;
        }
        const int64_t tiles = (lsize(s) + MLP_TILE - 1) / MLP_TILE;
        const unsigned g    = (unsigned)std::min<int64_t>(tiles, s->lam_grid);
        k_mlp_apply<<<g, MLP_TILE, 0, st>>>(s->k, s->feat, s->prev, s->lam, md, s->status);
        GPE_CHECK_LAUNCH("k_mlp_apply");
        s->launches += 1;
    } else {
        kCol[mi][sg](nblk(s), (unsigned)s->block, st, s->k, s->d_doms, s->dom, s->start, s->xd[s->XS], s->prev,
                     s->lam, pid, s->col);
        GPE_CHECK_LAUNCH("k_lambda_collect");
    }
    s->launches += 1;
    return GPE_OK;
}

int32_t stage_delta_p(gpe_pbf* s, cudaStream_t st, bool accinit)
{
    if (lsize(s) > 0) {
        const int sc = s->prm.scorr_k != 0.f ? 1 : 0;
        // the move threshold covers mask_passes passes after the masks were made (a step with more
        // iterations, such as the one that starts the network's memory, scans in full after those)
        if (s->masks_valid && s->dp_since_build >= s->mask_passes) { s->masks_valid = false; }
        const int mask = s->masks_valid ? MASK_USE : MASK_OFF;
        s->dp_since_build += 1;
        GPE_TRY_CUDA(kDp[multi(s) ? 1 : 0][sc][accinit ? 1 : 0](nblk(s), (unsigned)s->block, st, s->k, s->d_doms,
                                                                s->dom, s->start, s->xd[s->XS], s->lam,
                                                                s->xd[s->XO], s->acc, mask));
        s->launches += 1;
    }
    std::swap(s->XS, s->XO);
    return GPE_OK;
}

// next_hist: the step is followed by another with nothing in between (and no vorticity pass after XSPH):
// XSPH also computes the next step's cell keys and histogram, and the next sort skips k_predict_hist.
int32_t stage_xsph(gpe_pbf* s, cudaStream_t st, bool next_hist = false)
{
    if (lsize(s) == 0) { return GPE_OK; }
    const int vort = s->prm.vort_eps != 0.f ? 1 : 0;
    PbfK kk        = s->k;
    next_hist      = next_hist && vort == 0;
    if (next_hist) {
        kk.hist_kr  = s->keyrank;
        kk.hist_cnt = s->count; // zeroed by this step's scan
    }
    GPE_TRY_CUDA(kXs[multi(s) ? 1 : 0][vort](nblk(s), (unsigned)s->block, st, kk, s->d_doms, s->dom, s->start,
                                             s->xd[s->XS], s->pos, s->vel, s->omega, s->status,
                                             s->masks_valid ? MASK_USE : MASK_OFF));
    s->launches += 1;
    s->hist_ready = next_hist;
    return GPE_OK;
}


int32_t stage_vorticity(gpe_pbf* s, cudaStream_t st)
{
    if (lsize(s) == 0 || s->prm.vort_eps == 0.f) { return GPE_OK; }
    const unsigned g = nblk(s);
    const bool mu = s->masks_valid;
    if (multi(s)) {
        if (mu) {
            k_vorticity<true, MASK_USE><<<g, (unsigned)s->block, 0, st>>>(s->k, s->d_doms, s->dom, s->start,
                                                                         s->xd[s->XS], s->omega, s->vel);
        } else {
            k_vorticity<true, MASK_OFF><<<g, (unsigned)s->block, 0, st>>>(s->k, s->d_doms, s->dom, s->start,
                                                                         s->xd[s->XS], s->omega, s->vel);
        }
    } else {
        if (mu) {
            k_vorticity<false, MASK_USE><<<g, (unsigned)s->block, 0, st>>>(s->k, s->d_doms, s->dom, s->start,
                                                                          s->xd[s->XS], s->omega, s->vel);
        } else {
            k_vorticity<false, MASK_OFF><<<g, (unsigned)s->block, 0, st>>>(s->k, s->d_doms, s->dom, s->start,
                                                                          s->xd[s->XS], s->omega, s->vel);
        }
    }
    GPE_CHECK_LAUNCH("k_vorticity");
    s->launches += 1;
    return GPE_OK;
}

int32_t stage_finish(gpe_pbf* s)
{
    // XSPH wrote the step's end positions (sorted) into pos
    s->masks_valid = false;
    s->XS = s->XO = -1;
    return GPE_OK;
}

// The Jacobi passes and XSPH of a plain step in one cooperative launch (k_solve_persistent).
template <bool M, bool S, bool C, bool V, bool K>
const void* solve_fn()
{
    return reinterpret_cast<const void*>(k_solve_persistent<M, S, C, V, K>);
}
template <bool K>
const void* solve_kernel_k(bool m, bool sg, bool sc, bool v)
{
    const void* tab[16] = {
        solve_fn<false, false, false, false, K>(), solve_fn<false, false, false, true, K>(),
        solve_fn<false, false, true, false, K>(),  solve_fn<false, false, true, true, K>(),
        solve_fn<false, true, false, false, K>(),  solve_fn<false, true, false, true, K>(),
        solve_fn<false, true, true, false, K>(),   solve_fn<false, true, true, true, K>(),
        solve_fn<true, false, false, false, K>(),  solve_fn<true, false, false, true, K>(),
        solve_fn<true, false, true, false, K>(),   solve_fn<true, false, true, true, K>(),
        solve_fn<true, true, false, false, K>(),   solve_fn<true, true, false, true, K>(),
        solve_fn<true, true, true, false, K>(),    solve_fn<true, true, true, true, K>()};
    return tab[(m ? 8 : 0) + (sg ? 4 : 0) + (sc ? 2 : 0) + (v ? 1 : 0)];
}
const void* solve_kernel(const gpe_pbf* s)
{
    const bool m = multi(s), sg = (s->prm.flags & GPE_PBF_SELF_GRAD) != 0, sc = s->prm.scorr_k != 0.f,
               v = s->prm.vort_eps == 0.f; // XSPH inside the kernel
    return masks_on(s) ? solve_kernel_k<true>(m, sg, sc, v) : solve_kernel_k<false>(m, sg, sc, v);
}

// Blocks of a persistent launch: one per block of particles, at most as many as are resident at once (a
// small scene's barriers then wait on few blocks)
unsigned coop_blocks(const gpe_pbf* s)
{
    const int64_t need = (lsize(s) + s->block - 1) / s->block;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, s->coop_grid));
}

int32_t stage_solve_persistent(gpe_pbf* s, cudaStream_t st)
{
    if (lsize(s) > 0) {
        const void* fn = solve_kernel(s);
        if (s->coop_grid <= 0 || s->coop_fn != fn) {
            s->coop_fn = fn;
            int per_sm = 0;
            GPE_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, s->block, 0));
            s->coop_grid = std::max(1, per_sm) * gpe::sm_count();
        }
        const uint32_t* pid = (s->prm.flags & GPE_PBF_PAIR_IDS) ? s->ids[s->id_cur] : nullptr;
        PbfK k              = s->k;
        float4* xa          = s->xd[s->XS];
        float4* xb          = s->xd[s->XO];
        float2* xo          = s->pos;
        int32_t iters       = s->prm.iters;
        void* args[]        = {&k,  &s->d_doms, &s->dom, &s->start, &xa,   &xb,        &xo,
                               &s->lam, &pid, &s->vel, &s->omega, &iters, &s->gsync, &s->status};
        GPE_TRY_CUDA(cudaMemsetAsync(s->gsync, 0, sizeof(GridSync), st));
        if (masks_on(s)) { GPE_TRY_CUDA(cudaMemsetAsync(s->mflag, 0, (size_t)s->ncells, st)); }
        GPE_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(coop_blocks(s)), dim3((unsigned)s->block), args, 0, st));
        s->launches += 1;
    }
    if (s->prm.iters & 1) { std::swap(s->XS, s->XO); } // the kernel's final x* is in the other buffer
    return GPE_OK;
}

// The whole step in one cooperative launch (k_step_persistent): the host side of stage_predict_sort (buffer
// roles, id buffers) and of stage_solve_persistent.
template <bool M, bool S, bool C, bool V, bool K>
const void* step_fn()
{
    return reinterpret_cast<const void*>(k_step_persistent<M, S, C, V, K>);
}
template <bool K>
const void* step_kernel_k(bool m, bool sg, bool sc, bool v)
{
    const void* tab[16] = {
        step_fn<false, false, false, false, K>(), step_fn<false, false, false, true, K>(),
        step_fn<false, false, true, false, K>(),  step_fn<false, false, true, true, K>(),
        step_fn<false, true, false, false, K>(),  step_fn<false, true, false, true, K>(),
        step_fn<false, true, true, false, K>(),   step_fn<false, true, true, true, K>(),
        step_fn<true, false, false, false, K>(),  step_fn<true, false, false, true, K>(),
        step_fn<true, false, true, false, K>(),   step_fn<true, false, true, true, K>(),
        step_fn<true, true, false, false, K>(),   step_fn<true, true, false, true, K>(),
        step_fn<true, true, true, false, K>(),    step_fn<true, true, true, true, K>()};
    return tab[(m ? 8 : 0) + (sg ? 4 : 0) + (sc ? 2 : 0) + (v ? 1 : 0)];
}

int32_t stage_step_persistent(gpe_pbf* s, cudaStream_t st)
{
    drop_hist(s); // its sort phases build their own histogram
    const int32_t rch = clear_hist(s, st);
    if (rch) { return rch; }
    s->masks_valid = false;
    s->XS  = 0;
    s->XO  = 1;
    s->k.n = (int32_t)s->n;
    const bool ids = (s->prm.flags & (GPE_PBF_TRACK_IDS | GPE_PBF_PAIR_IDS)) != 0;
    if (lsize(s) > 0) {
        const bool m = multi(s), sg = (s->prm.flags & GPE_PBF_SELF_GRAD) != 0, sc = s->prm.scorr_k != 0.f,
                   v = s->prm.vort_eps == 0.f; // XSPH inside the kernel
        const void* fn = masks_on(s) ? step_kernel_k<true>(m, sg, sc, v) : step_kernel_k<false>(m, sg, sc, v);
        if (s->coop_grid <= 0 || s->coop_fn != fn) {
            s->coop_fn = fn;
            int per_sm = 0;
            GPE_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, s->block, 0));
            s->coop_grid = std::max(1, per_sm) * gpe::sm_count();
        }
        SortBufs sb{};
        sb.x         = s->pos;
        sb.v         = s->vel;
        sb.keyrank   = s->keyrank;
        sb.count     = s->count;
        sb.bsum      = s->bsum;
        sb.start     = s->start;
        sb.bucket    = s->bucket;
        sb.xd_sorted = s->xd[s->XS];
        sb.perm      = s->perm;
        sb.keys      = s->keys;
        sb.id_in     = ids ? s->ids[s->id_cur] : nullptr;
        sb.id_out    = ids ? s->ids[s->id_cur ^ 1] : nullptr;
        sb.mflag     = masks_on(s) ? s->mflag : nullptr;
        sb.ncells    = (uint32_t)s->ncells;
        const uint32_t* pid = (s->prm.flags & GPE_PBF_PAIR_IDS) ? sb.id_out : nullptr;
        PbfK k              = s->k;
        float4* xb          = s->xd[s->XO];
        int32_t iters       = s->prm.iters;
        void* args[]        = {&k, &s->d_doms, &s->dom, &sb, &xb, &s->lam, &pid, &s->vel, &s->omega, &iters,
                               &s->gsync, &s->status};
        GPE_TRY_CUDA(cudaMemsetAsync(s->gsync, 0, sizeof(GridSync), st));
        GPE_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(coop_blocks(s)), dim3((unsigned)s->block), args, 0, st));
        s->launches += 1;
    } else {
        // no particle: the cell starts are all zero (as the separate scan leaves them)
        int32_t rc = launch_exclusive_scan(s->count, s->ncells, s->bsum, s->start, st);
        if (rc) { return rc; }
        s->launches += scan_launches(s->ncells);
    }
    if (ids) { s->id_cur ^= 1; }
    s->have_sort = true;
    if (s->prm.iters & 1) { std::swap(s->XS, s->XO); } // the kernel's final x* is in the other buffer
    return GPE_OK;
}

// next_hist: another step follows directly (see stage_xsph)
int32_t run_step(gpe_pbf* s, cudaStream_t st, bool next_hist = false)
{
    const bool acc = accumulating(s);
    if (s->step_kernel && s->persistent && !acc) {
        int32_t rc = stage_step_persistent(s, st);
        if (rc == GPE_OK && s->prm.vort_eps != 0.f) {
            rc = stage_xsph(s, st);
            if (rc == GPE_OK) { rc = stage_vorticity(s, st); }
        }
        if (rc == GPE_OK) { rc = stage_finish(s); }
        return rc;
    }
    int32_t rc     = stage_predict_sort(s, st);
    if (rc == GPE_OK && s->persistent && !acc) {
        rc = stage_solve_persistent(s, st);
        if (rc == GPE_OK && s->prm.vort_eps != 0.f) {
            rc = stage_xsph(s, st);
            if (rc == GPE_OK) { rc = stage_vorticity(s, st); }
        }
        if (rc == GPE_OK) { rc = stage_finish(s); }
        return rc;
    }
    for (int32_t it = 0; it < s->prm.iters && rc == GPE_OK; ++it) {
        if (it == 0 && acc) {
            rc = stage_lambda_warm(s, st);
            if (rc == GPE_OK) { rc = stage_delta_p(s, st, true); }
        } else {
            rc = stage_lambda(s, st, acc_mode(s));
            if (rc == GPE_OK) { rc = stage_delta_p(s, st, false); }
        }
    }
    if (rc == GPE_OK) { rc = stage_xsph(s, st, next_hist && !s->collecting); }
    if (rc == GPE_OK) { rc = stage_vorticity(s, st); }
    if (rc == GPE_OK && s->collecting && s->col.stride != 0u && lsize(s) > 0) {
        k_collect_targets<<<blocks_for(lsize(s)), T_PART, 0, st>>>(s->col.cnt, s->col.X, s->col.T, s->col.idx,
                                                                s->acc, s->col.cap);
        GPE_CHECK_LAUNCH("k_collect_targets");
        k_collect_advance<<<1, 1, 0, st>>>(s->col.cnt, s->col.cap);
        GPE_CHECK_LAUNCH("k_collect_advance");
    }
    if (rc == GPE_OK) { rc = stage_finish(s); }
    if (rc == GPE_OK && acc && s->prm.iters > 0) { s->mem_valid = true; }
    return rc;
}

int32_t alloc_buffers(gpe_pbf* s)
{
    const size_t N = (size_t)s->cap;
    const size_t M = (size_t)s->cells_cap; // room for the finest sort grid the tuning may select
    Carver c;
    const size_t o_doms = c.take<DomDev>((size_t)s->nd);
    const size_t o_pos   = c.take<float2>(N);
    const size_t o_xd0   = c.take<float4>(N);
    const size_t o_xd1   = c.take<float4>(N);
    const size_t o_vel   = c.take<float2>(N);
    const size_t o_lam   = c.take<float>(N);
    const size_t o_om    = c.take<float>(N);
    const size_t o_rho   = c.take<float>(N);
    const size_t o_kr    = c.take<uint2>(N);
    const size_t o_bk    = c.take<uint32_t>(N);
    const size_t o_cnt   = c.take<uint32_t>(M);
    const size_t o_st    = c.take<uint32_t>(M + 1);
    const size_t o_bs    = c.take<uint32_t>(scan_blocks((uint32_t)M) + 1);
    const size_t o_perm  = c.take<uint32_t>(N);
    const size_t o_keys  = c.take<uint32_t>(N);
    const size_t o_dom   = c.take<int32_t>(N);
    const size_t o_id0   = c.take<uint32_t>(N);
    const size_t o_id1   = c.take<uint32_t>(N);
    const size_t o_stat  = c.take<uint32_t>(4);
    const size_t o_red   = c.take<float>(8);
    const size_t o_cnt1  = c.take<int32_t>(1);
    const size_t o_acc   = c.take<float>(N);
    const size_t o_prev  = c.take<float>(N);
    const size_t o_gs    = c.take<GridSync>(1);
    const size_t o_nm    = c.take<uint4>(N);
    const size_t o_mf    = c.take<uint8_t>(M);
    GPE_TRY_CUDA(cudaMalloc(&s->base, c.off));
    GPE_TRY_CUDA(cudaMemset(s->base, 0, c.off));
    uint8_t* b = static_cast<uint8_t*>(s->base);
    s->d_doms  = reinterpret_cast<DomDev*>(b + o_doms);
    s->pos     = reinterpret_cast<float2*>(b + o_pos);
    s->xd[0]   = reinterpret_cast<float4*>(b + o_xd0);
    s->xd[1]   = reinterpret_cast<float4*>(b + o_xd1);
    s->vel     = reinterpret_cast<float2*>(b + o_vel);
    s->lam     = reinterpret_cast<float*>(b + o_lam);
    s->omega   = reinterpret_cast<float*>(b + o_om);
    s->rho     = reinterpret_cast<float*>(b + o_rho);
    s->keyrank = reinterpret_cast<uint2*>(b + o_kr);
    s->bucket  = reinterpret_cast<uint32_t*>(b + o_bk);
    s->count   = reinterpret_cast<uint32_t*>(b + o_cnt);
    s->start   = reinterpret_cast<uint32_t*>(b + o_st);
    s->bsum    = reinterpret_cast<uint32_t*>(b + o_bs);
    s->perm    = reinterpret_cast<uint32_t*>(b + o_perm);
    s->keys    = reinterpret_cast<uint32_t*>(b + o_keys);
    s->dom     = reinterpret_cast<int32_t*>(b + o_dom);
    s->ids[0]  = reinterpret_cast<uint32_t*>(b + o_id0);
    s->ids[1]  = reinterpret_cast<uint32_t*>(b + o_id1);
    s->status  = reinterpret_cast<uint32_t*>(b + o_stat);
    s->red     = reinterpret_cast<float*>(b + o_red);
    s->d_count = reinterpret_cast<int32_t*>(b + o_cnt1);
    s->acc     = reinterpret_cast<float*>(b + o_acc);
    s->prev    = reinterpret_cast<float*>(b + o_prev);
    s->gsync   = reinterpret_cast<GridSync*>(b + o_gs);
    s->nmask   = reinterpret_cast<uint4*>(b + o_nm);
    s->mflag   = b + o_mf;
    bind_k(s);
    GPE_TRY_CUDA(cudaMemcpy(s->d_doms, s->domdev.data(), sizeof(DomDev) * (size_t)s->nd, cudaMemcpyHostToDevice));
    return GPE_OK;
}

cudaMemcpyKind kind_in(int32_t mem) { return mem == GPE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }
cudaMemcpyKind kind_out(int32_t mem) { return mem == GPE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost; }

} // namespace

// =====================================================================================================
// C ABI
// =====================================================================================================

extern "C" {

int32_t gpe_pbf_create(const gpe_pbf_params* params, const gpe_domain* domains, int32_t n_domains, int64_t capacity,
                       gpe_pbf** out)
{
    gpe::clear_error();
    if (!out || !domains || n_domains <= 0 || capacity < 0 || capacity > (int64_t)INT32_MAX / 2) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_create: bad arguments");
        return GPE_ERR_BAD_ARG;
    }
    *out       = nullptr;
    int32_t rc = validate_params(params);
    if (rc) { return rc; }
    for (int32_t d = 0; d < n_domains; ++d) {
        if (!(domains[d].extent[0] > 0.f) || !(domains[d].extent[1] > 0.f)) {
            gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_create: scene %d has a non-positive extent", d);
            return GPE_ERR_BAD_ARG;
        }
    }
    const uint64_t cells = count_cells(params, domains, n_domains);
    if (cells == CELLS_INVALID) {
        gpe::set_error(GPE_ERR_CAPACITY, "gpe_pbf_create: a scene extent is not finite or spans 2^30 cells or more");
        return GPE_ERR_CAPACITY;
    }
    if (cells == 0 || cells > (uint64_t)1 << 30) {
        gpe::set_error(GPE_ERR_CAPACITY, "gpe_pbf_create: %llu cells exceed the 2^30 limit",
                       (unsigned long long)cells);
        return GPE_ERR_CAPACITY;
    }
    int dev = 0;
    rc      = gpe::current_device(&dev);
    if (rc) { return rc; }
    gpe_pbf* s = new gpe_pbf();
    s->device  = dev;
    s->prm     = *params;
    s->nd      = n_domains;
    s->doms.assign(domains, domains + n_domains);
    s->dynamic = (params->flags & GPE_PBF_DYNAMIC_COUNT) != 0;
    s->cap = capacity;
    build_domains(s);
    {
        // the cell arrays also hold the h/2 grid, so that the tuning can select it later
        gpe_pbf_params half = *params;
        half.cell           = 0.5f * params->h;
        const uint64_t ch   = count_cells(&half, domains, n_domains);
        s->cells_cap        = std::max<uint64_t>(cells, ch <= ((uint64_t)1 << 30) ? ch : 0);
    }
    rc = alloc_buffers(s);
    if (rc) {
        if (s->base) { cudaFree(s->base); }
        delete s;
        return rc;
    }
    *out = s;
    return GPE_OK;
}

int32_t gpe_pbf_destroy(gpe_pbf* s)
{
    if (!s) { return GPE_ERR_BAD_ARG; }
    s->drop_graphs();
    if (s->base) { cudaFree(s->base); }
    if (s->feat) { cudaFree(s->feat); }
    delete s;
    return GPE_OK;
}

int32_t gpe_pbf_set_params(gpe_pbf* s, const gpe_pbf_params* params)
{
    gpe::clear_error();
    if (!s) { return GPE_ERR_BAD_ARG; }
    int32_t rc = validate_params(params);
    if (rc) { return rc; }
    const float c_old = s->prm.cell > 0.f ? s->prm.cell : s->prm.h;
    const float c_new = params->cell > 0.f ? params->cell : params->h;
    if (c_old != c_new) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_set_params: the sort-cell size is fixed at creation");
        return GPE_ERR_BAD_ARG;
    }
    drop_hist(s);
    s->prm     = *params;
    s->dynamic = (params->flags & GPE_PBF_DYNAMIC_COUNT) != 0;
    build_domains(s);
    GPE_TRY_CUDA(cudaMemcpy(s->d_doms, s->domdev.data(), sizeof(DomDev) * (size_t)s->nd, cudaMemcpyHostToDevice));
    s->drop_graphs();
    return GPE_OK;
}

int32_t gpe_pbf_get_params(const gpe_pbf* s, gpe_pbf_params* params)
{
    if (!s || !params) { return GPE_ERR_BAD_ARG; }
    *params = s->prm;
    return GPE_OK;
}

int32_t gpe_pbf_set_state(gpe_pbf* s, const float* pos, const float* vel, const int32_t* domain_id, int64_t n,
                          int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!s || n < 0 || (n > 0 && !pos) || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE && mem != GPE_MEM_PINNED)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_set_state: bad arguments");
        return GPE_ERR_BAD_ARG;
    }
    if (n > s->cap) {
        gpe::set_error(GPE_ERR_CAPACITY, "gpe_pbf_set_state: %lld particles exceed capacity %lld", (long long)n,
                       (long long)s->cap);
        return GPE_ERR_CAPACITY;
    }
    if (s->nd > 1 && n > 0 && !domain_id) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_set_state: domain_id is required with several scenes");
        return GPE_ERR_BAD_ARG;
    }
    if (s->nd > 1 && mem != GPE_MEM_DEVICE) { // host or pinned: checked here
        for (int64_t i = 0; i < n; ++i) {
            if (domain_id[i] < 0 || domain_id[i] >= s->nd || (i > 0 && domain_id[i] < domain_id[i - 1])) {
                gpe::set_error(GPE_ERR_BAD_ARG,
                               "gpe_pbf_set_state: domain_id must be in [0, n_domains) and non-decreasing");
                return GPE_ERR_BAD_ARG;
            }
        }
    }
    cudaStream_t st = as_stream(stream);
    drop_hist(s);
    s->XS = s->XO   = -1;
    s->id_cur     = 0;
    if (n > 0) {
        GPE_TRY_CUDA(cudaMemcpyAsync(s->pos, pos, sizeof(float2) * (size_t)n, kind_in(mem), st));
        if (vel) {
            GPE_TRY_CUDA(cudaMemcpyAsync(s->vel, vel, sizeof(float2) * (size_t)n, kind_in(mem), st));
        } else {
            GPE_TRY_CUDA(cudaMemsetAsync(s->vel, 0, sizeof(float2) * (size_t)n, st));
        }
        if (s->nd > 1) {
            GPE_TRY_CUDA(cudaMemcpyAsync(s->dom, domain_id, sizeof(int32_t) * (size_t)n, kind_in(mem), st));
            if (mem == GPE_MEM_DEVICE) {
                k_check_domains<<<blocks_for(n), T_PART, 0, st>>>(s->dom, (int32_t)n, s->nd, s->status);
                GPE_CHECK_LAUNCH("k_check_domains");
                uint32_t stt = 0;
                GPE_TRY_CUDA(cudaMemcpyAsync(&stt, s->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
                GPE_TRY_CUDA(cudaStreamSynchronize(st));
                if (stt & GPE_STATUS_CAPACITY) {
                    GPE_TRY_CUDA(cudaMemsetAsync(s->status, 0, sizeof(uint32_t), st));
                    gpe::set_error(GPE_ERR_BAD_ARG,
                                   "gpe_pbf_set_state: domain_id must be in [0, n_domains) and non-decreasing");
                    return GPE_ERR_BAD_ARG;
                }
            }
        }
        k_iota<<<blocks_for(n), T_PART, 0, st>>>(s->ids[0], (int32_t)n);
        GPE_CHECK_LAUNCH("k_iota");
    }
    k_set_count<<<1, 1, 0, st>>>(s->d_count, (int32_t)n);
    GPE_CHECK_LAUNCH("k_set_count");
    // a new particle set has no previous multipliers
    GPE_TRY_CUDA(cudaMemsetAsync(s->acc, 0, sizeof(float) * (size_t)s->cap, st));
    if (s->n != n && !s->dynamic) { s->drop_graphs(); }
    s->n          = n;
    s->have_state = true;
    s->have_sort  = false;
    s->mem_valid  = false;
    return GPE_OK;
}

int32_t gpe_pbf_get_state(gpe_pbf* s, float* pos, float* vel, int32_t* domain_id, int64_t n, int32_t mem,
                          void* stream)
{
    gpe::clear_error();
    if (!s) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    int32_t rc      = sync_count(s, st);
    if (rc) { return rc; }
    if (n != s->n || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE && mem != GPE_MEM_PINNED)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_get_state: n must equal the particle count");
        return GPE_ERR_BAD_ARG;
    }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    if (n > 0) {
        if (pos) { GPE_TRY_CUDA(cudaMemcpyAsync(pos, s->pos, sizeof(float2) * (size_t)n, kind_out(mem), st)); }
        if (vel) { GPE_TRY_CUDA(cudaMemcpyAsync(vel, s->vel, sizeof(float2) * (size_t)n, kind_out(mem), st)); }
        if (domain_id) {
            if (s->nd > 1) {
                GPE_TRY_CUDA(cudaMemcpyAsync(domain_id, s->dom, sizeof(int32_t) * (size_t)n, kind_out(mem), st));
            } else if (mem != GPE_MEM_DEVICE) {
                GPE_TRY_CUDA(cudaStreamSynchronize(st));
                std::memset(domain_id, 0, sizeof(int32_t) * (size_t)n);
            } else {
                GPE_TRY_CUDA(cudaMemsetAsync(domain_id, 0, sizeof(int32_t) * (size_t)n, st));
            }
        }
    }
    if (mem == GPE_MEM_HOST) { GPE_TRY_CUDA(cudaStreamSynchronize(st)); }
    return GPE_OK;
}

int32_t gpe_pbf_count(const gpe_pbf* s, int64_t* n)
{
    if (!s || !n) { return GPE_ERR_BAD_ARG; }
    // with a device-resident count the host copy is refreshed first (a cached value, hence the cast)
    const int32_t rc = sync_count(const_cast<gpe_pbf*>(s), nullptr);
    if (rc) { return rc; }
    *n = s->n;
    return GPE_OK;
}

int32_t gpe_pbf_num_cells(const gpe_pbf* s, int64_t* n_cells)
{
    if (!s || !n_cells) { return GPE_ERR_BAD_ARG; }
    *n_cells = (int64_t)s->ncells;
    return GPE_OK;
}

int32_t gpe_pbf_step(gpe_pbf* s, int32_t n_steps, void* stream)
{
    gpe::clear_error();
    if (!s || n_steps < 0) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_step: no state set");
        return GPE_ERR_NOT_READY;
    }
    if (n_steps == 0) { return GPE_OK; }
    cudaStream_t st = as_stream(stream);
    if (s->warm == GPE_WARM_MLP && !s->mem_valid) {
        // The step that starts the multiplier memory is a plain step with the iteration count of the solve
        // the network was trained on, so that the memory holds what the network expects as lambda_prev (a
        // memory started by a short solve would be carried forward at that solve's level). It differs from
        // the later steps and runs outside the graph.
        const int32_t iters = s->prm.iters;
        s->prm.iters        = gpe::mlp_pair_iters(s->mlp);
        s->launches         = 0;
        const int32_t rc    = run_step(s, st, true);
        s->prm.iters        = iters;
        if (rc) { return rc; }
        if (--n_steps == 0) { return GPE_OK; }
    }
    // the step sequence is captured once per (steps, whether the first sort's histogram is already there,
    // starting buffer roles) and replayed as one graph; every step but none in between leaves the next
    // step's keys and histogram (stage_xsph)
    const auto key = std::make_tuple(n_steps, (s->hist_ready ? 1 : 0) + (s->count_dirty ? 2 : 0), s->id_cur);
    auto it        = s->graphs.find(key);
    if (it == s->graphs.end()) {
        cudaStream_t cap_st = st;
        bool own            = false;
        if (cap_st == nullptr) {
            GPE_TRY_CUDA(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
            own = true;
        }
        const int id0    = s->id_cur;
        const bool hist0 = s->hist_ready, dirty0 = s->count_dirty;
        GPE_TRY_CUDA(cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
        s->launches = 0;
        int32_t rc  = GPE_OK;
        for (int32_t k = 0; k < n_steps && rc == GPE_OK; ++k) { rc = run_step(s, cap_st, true); }
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cap_st, &graph);
        PbfGraph pg;
        pg.id_end     = s->id_cur;
        pg.hist_end   = s->hist_ready;
        s->id_cur     = id0;
        s->hist_ready = hist0;
        s->count_dirty = dirty0;
        if (rc == GPE_OK && ce != cudaSuccess) {
            gpe::set_cuda_error(ce, "cudaStreamEndCapture");
            rc = GPE_ERR_CUDA;
        }
        if (rc == GPE_OK) {
            const cudaError_t ie = cudaGraphInstantiate(&pg.exec, graph, 0);
            if (ie != cudaSuccess) {
                gpe::set_cuda_error(ie, "cudaGraphInstantiate");
                rc = GPE_ERR_CUDA;
            }
        }
        if (graph) { cudaGraphDestroy(graph); }
        if (own) { cudaStreamDestroy(cap_st); }
        if (rc) { return rc; }
        s->launches /= n_steps;
        it = s->graphs.emplace(key, pg).first;
    }
    GPE_TRY_CUDA(cudaGraphLaunch(it->second.exec, st));
    s->id_cur      = it->second.id_end;
    s->hist_ready  = it->second.hist_end;
    s->count_dirty = false; // the graph's first sort cleared it
    s->have_sort  = true;
    return GPE_OK;
}

int32_t gpe_pbf_stage(gpe_pbf* s, int32_t stage, void* stream)
{
    gpe::clear_error();
    if (!s) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    cudaStream_t st = as_stream(stream);
    const bool in_step = s->XS >= 0;
    if (stage != GPE_PBF_STAGE_DENSITY) { drop_hist(s); } // the density pass reads positions and cell starts
    switch (stage) {
        case GPE_PBF_STAGE_PREDICT_SORT:
            if (in_step) { break; }
            return stage_predict_sort(s, st);
        case GPE_PBF_STAGE_LAMBDA:
            if (!in_step) { break; }
            return stage_lambda(s, st, acc_mode(s));
        case GPE_PBF_STAGE_WARM_LAMBDA:
            if (!in_step || !accumulating(s)) { break; }
            s->pending_accinit = true;
            return stage_lambda_warm(s, st);
        case GPE_PBF_STAGE_DELTA_P: {
            if (!in_step) { break; }
            const bool ai      = s->pending_accinit;
            s->pending_accinit = false;
            return stage_delta_p(s, st, ai);
        }
        case GPE_PBF_STAGE_XSPH:
            if (!in_step) { break; }
            return stage_xsph(s, st);
        case GPE_PBF_STAGE_VORTICITY:
            if (!in_step) { break; }
            return stage_vorticity(s, st);
        case GPE_PBF_STAGE_FINISH:
            if (!in_step) { break; }
            return stage_finish(s);
        case GPE_PBF_STAGE_DENSITY: {
            if (!s->have_sort || in_step) { break; }
            GPE_TRY_CUDA(cudaMemsetAsync(s->red, 0, sizeof(float) * 8, st));
            if (s->n > 0) {
                s->k.n = (int32_t)s->n;
                if (multi(s)) {
                    k_density<true><<<blocks_for(lsize(s)), T_PART, 0, st>>>(s->k, s->d_doms, s->dom, s->start,
                                                                         s->pos, s->rho, s->red);
                } else {
                    k_density<false><<<blocks_for(lsize(s)), T_PART, 0, st>>>(s->k, s->d_doms, s->dom, s->start,
                                                                          s->pos, s->rho, s->red);
                }
                GPE_CHECK_LAUNCH("k_density");
            }
            return GPE_OK;
        }
        default:
            gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_stage: unknown stage %d", stage);
            return GPE_ERR_BAD_ARG;
    }
    gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_stage: stage %d is out of order", stage);
    return GPE_ERR_NOT_READY;
}

int32_t gpe_pbf_density_error(gpe_pbf* s, float* max_err, float* mean_err, void* stream)
{
    if (!s || !max_err || !mean_err) { return GPE_ERR_BAD_ARG; }
    const int32_t rcn = sync_count(s, as_stream(stream));
    if (rcn) { return rcn; }
    int32_t rc = gpe_pbf_stage(s, GPE_PBF_STAGE_DENSITY, stream);
    if (rc) { return rc; }
    float red[8];
    cudaStream_t st = as_stream(stream);
    GPE_TRY_CUDA(cudaMemcpyAsync(red, s->red, sizeof(red), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    double sum;
    std::memcpy(&sum, &red[2], sizeof(double));
    *max_err  = red[0];
    *mean_err = s->n > 0 ? (float)(sum / (double)s->n) : 0.f;
    return GPE_OK;
}

// x* = x + d of every record, rounded once (field GPE_PBF_FIELD_PRED)
__global__ void k_xd_pred(const float4* __restrict__ xd, float2* __restrict__ out, int32_t n)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 a = xd[i];
        out[i]         = make_float2(__fadd_rn(a.x, a.z), __fadd_rn(a.y, a.w));
    }
}
// a written x*: d = x* - x
__global__ void k_xd_set_pred(float4* __restrict__ xd, const float2* __restrict__ xs, int32_t n)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 a = xd[i];
        const float2 q = xs[i];
        xd[i]          = make_float4(a.x, a.y, __fsub_rn(q.x, a.x), __fsub_rn(q.y, a.y));
    }
}

// Within a step, x (POS) and d (DISP) are the halves of the (x, d) records and x* (PRED) is computed from
// them; field_ptr reports those as their record array with a byte offset and a 16-byte stride.
struct FieldLoc {
    void* p;
    size_t esize;
    int64_t count;
    size_t stride; // 0: contiguous
    int kind;      // 0: plain memory, 1: x* computed from the records
};

static int32_t field_ptr(gpe_pbf* s, int32_t field, FieldLoc* f)
{
    const bool in_step = s->XS >= 0;
    f->count           = s->n;
    f->stride          = 0;
    f->kind            = 0;
    void** p           = &f->p;
    size_t* esize      = &f->esize;
    switch (field) {
        case GPE_PBF_FIELD_POS:
            if (in_step) {
                *p        = s->xd[s->XS];
                f->stride = sizeof(float4);
            } else {
                *p = s->pos;
            }
            *esize = 8;
            break;
        case GPE_PBF_FIELD_DISP:
            if (!in_step) { return GPE_ERR_NOT_READY; }
            *p        = reinterpret_cast<uint8_t*>(s->xd[s->XS]) + sizeof(float2);
            f->stride = sizeof(float4);
            *esize    = 8;
            break;
        case GPE_PBF_FIELD_VEL: *p = s->vel; *esize = 8; break;
        case GPE_PBF_FIELD_PRED:
            if (!in_step) { return GPE_ERR_NOT_READY; }
            *p      = s->xd[s->XS];
            *esize  = 8;
            f->kind = 1;
            break;
        case GPE_PBF_FIELD_LAMBDA: *p = s->lam; *esize = 4; break;
        case GPE_PBF_FIELD_KEY: *p = s->keys; *esize = 4; break;
        case GPE_PBF_FIELD_PERM: *p = s->perm; *esize = 4; break;
        case GPE_PBF_FIELD_CELL_START: *p = s->start; *esize = 4; f->count = (int64_t)s->ncells + 1; break;
        case GPE_PBF_FIELD_DOMAIN: *p = s->dom; *esize = 4; break;
        case GPE_PBF_FIELD_DENSITY: *p = s->rho; *esize = 4; break;
        case GPE_PBF_FIELD_ID: *p = s->ids[s->id_cur]; *esize = 4; break;
        case GPE_PBF_FIELD_OMEGA: *p = s->omega; *esize = 4; break;
        case GPE_PBF_FIELD_LAMBDA_PREV: *p = s->prev; *esize = 4; break;
        case GPE_PBF_FIELD_LAMBDA_SUM: *p = s->acc; *esize = 4; break;
        default: return GPE_ERR_BAD_ARG;
    }
    return GPE_OK;
}

int32_t gpe_pbf_get_field(gpe_pbf* s, int32_t field, void* dst, int64_t n_elems, int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!s || !dst || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) { return GPE_ERR_BAD_ARG; }
    const int32_t rcn = sync_count(s, as_stream(stream));
    if (rcn) { return rcn; }
    FieldLoc f{};
    int32_t rc = field_ptr(s, field, &f);
    if (rc) {
        gpe::set_error(rc, "gpe_pbf_get_field: field %d unavailable", field);
        return rc;
    }
    if (n_elems != f.count) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_get_field: field %d has %lld elements", field, (long long)f.count);
        return GPE_ERR_BAD_ARG;
    }
    cudaStream_t st = as_stream(stream);
    const size_t n  = (size_t)f.count;
    if (n > 0) {
        if (f.kind == 1) {
            // x* = x + d into the sort's (key, rank) scratch, which is free within a step, then out
            drop_hist(s); // the next step's keys may be waiting there
            float2* tmp = reinterpret_cast<float2*>(s->keyrank);
            k_xd_pred<<<blocks_for((int64_t)n), T_PART, 0, st>>>(static_cast<const float4*>(f.p), tmp, (int32_t)n);
            GPE_CHECK_LAUNCH("k_xd_pred");
            GPE_TRY_CUDA(cudaMemcpyAsync(dst, tmp, sizeof(float2) * n, kind_out(mem), st));
        } else if (f.stride) {
            GPE_TRY_CUDA(cudaMemcpy2DAsync(dst, f.esize, f.p, f.stride, f.esize, n, kind_out(mem), st));
        } else {
            GPE_TRY_CUDA(cudaMemcpyAsync(dst, f.p, f.esize * n, kind_out(mem), st));
        }
    }
    if (mem == GPE_MEM_HOST) { GPE_TRY_CUDA(cudaStreamSynchronize(st)); }
    return GPE_OK;
}

int32_t gpe_pbf_set_field(gpe_pbf* s, int32_t field, const void* src, int64_t n_elems, int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!s || !src || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) { return GPE_ERR_BAD_ARG; }
    if (field == GPE_PBF_FIELD_KEY || field == GPE_PBF_FIELD_PERM || field == GPE_PBF_FIELD_CELL_START ||
        field == GPE_PBF_FIELD_DOMAIN) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_set_field: field %d is derived and read-only", field);
        return GPE_ERR_BAD_ARG;
    }
    s->masks_valid = false; // a written position (or anything else) may move a particle past its masks
    drop_hist(s);
    FieldLoc f{};
    int32_t rc = field_ptr(s, field, &f);
    if (rc) { return rc; }
    if (n_elems != f.count) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    const size_t n  = (size_t)f.count;
    if (n > 0) {
        if (f.kind == 1) {
            // a new x* keeps x and sets d = x* - x
            float2* tmp = reinterpret_cast<float2*>(s->keyrank);
            GPE_TRY_CUDA(cudaMemcpyAsync(tmp, src, sizeof(float2) * n, kind_in(mem), st));
            k_xd_set_pred<<<blocks_for((int64_t)n), T_PART, 0, st>>>(static_cast<float4*>(f.p), tmp, (int32_t)n);
            GPE_CHECK_LAUNCH("k_xd_set_pred");
        } else if (f.stride) {
            GPE_TRY_CUDA(cudaMemcpy2DAsync(f.p, f.stride, src, f.esize, f.esize, n, kind_in(mem), st));
        } else {
            GPE_TRY_CUDA(cudaMemcpyAsync(f.p, src, f.esize * n, kind_in(mem), st));
        }
    }
    if (mem == GPE_MEM_HOST) { GPE_TRY_CUDA(cudaStreamSynchronize(st)); }
    if (field == GPE_PBF_FIELD_LAMBDA_SUM) { s->mem_valid = true; } // the caller supplied the memory
    return GPE_OK;
}

int32_t gpe_pbf_status(gpe_pbf* s, uint32_t* status, void* stream)
{
    if (!s || !status) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    GPE_TRY_CUDA(cudaMemcpyAsync(status, s->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaMemsetAsync(s->status, 0, sizeof(uint32_t), st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    return GPE_OK;
}

int32_t gpe_pbf_launches_per_step(const gpe_pbf* s, int32_t* launches)
{
    if (!s || !launches) { return GPE_ERR_BAD_ARG; }
    const bool warm      = s->prm.iters > 0;
    const bool vort      = s->prm.vort_eps != 0.f;
    const int32_t sorted = 3 + gpe::scan_launches(s->ncells); // predict + histogram, scan, scatter, place
    if (s->persistent && !accumulating(s)) {
        // the passes (and XSPH without vorticity) in one cooperative launch, with the sort in that launch too
        // for the whole-step kernel; with vorticity XSPH and the confinement keep their launches
        *launches = (s->step_kernel ? 0 : sorted) + 1 + (vort ? 2 : 0);
        return GPE_OK;
    }
    // GPE_WARM_PREV: lambda_prev is placed by the sort; GPE_WARM_MLP: features, then the network. Without
    // vorticity the previous step's XSPH computes the keys and histogram of consecutive steps (one launch
    // fewer).
    const int32_t first = (warm && s->warm == GPE_WARM_PREV) ? -1 : ((warm && s->warm == GPE_WARM_MLP) ? 1 : 0);
    *launches = sorted - (vort ? 0 : 1) + 2 * s->prm.iters + 1 + (vort ? 1 : 0) + first;
    return GPE_OK;
}

int32_t gpe_selftest_barrier_timeout(uint32_t* status)
{
    gpe::clear_error();
    if (!status) { return GPE_ERR_BAD_ARG; }
    void* buf = nullptr;
    GPE_TRY_CUDA(cudaMalloc(&buf, sizeof(GridSync) + sizeof(uint32_t)));
    GridSync* g    = static_cast<GridSync*>(buf);
    uint32_t* word = reinterpret_cast<uint32_t*>(g + 1);
    GridSync init{};
    init.count = 1u; // "another block has arrived": this one is not the last, so it waits for the generation
    cudaError_t e = cudaMemcpy(g, &init, sizeof(GridSync), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) { e = cudaMemset(word, 0, sizeof(uint32_t)); }
    if (e == cudaSuccess) {
        k_barrier_selftest<<<1, 32>>>(g, word);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) { e = cudaDeviceSynchronize(); }
    if (e == cudaSuccess) { e = cudaMemcpy(status, word, sizeof(uint32_t), cudaMemcpyDeviceToHost); }
    cudaFree(buf);
    if (e != cudaSuccess) {
        gpe::set_cuda_error(e, "gpe_selftest_barrier_timeout");
        return GPE_ERR_CUDA;
    }
    return GPE_OK;
}

} // extern "C"


extern "C" int32_t gpe_pbf_emit(gpe_pbf* s, const gpe_hose* hose, uint64_t seed, int32_t* requested, void* stream)
{
    gpe::clear_error();
    if (!s || !hose || !(hose->spacing > 0.f) || hose->steps_per_call < 0) { return GPE_ERR_BAD_ARG; }
    if (!s->dynamic || s->nd != 1) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_emit: needs GPE_PBF_DYNAMIC_COUNT and a single scene");
        return GPE_ERR_NOT_READY;
    }
    if (s->XS >= 0) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_emit: a step is in progress (stage API)");
        return GPE_ERR_NOT_READY;
    }
    drop_hist(s); // the new particles are not in the histogram the last step may have left
    HoseK h{};
    const int32_t cnt = make_hose(*hose, s->prm.dt, seed, &h);
    if (requested) { *requested = cnt; }
    if (cnt < 0 || (int64_t)cnt > s->cap) {
        gpe::set_error(GPE_ERR_CAPACITY, "emit: the hose asks for %s particles, more than the engine's capacity "
                       "of %lld", cnt < 0 ? "2^31 or more" : std::to_string(cnt).c_str(), (long long)s->cap);
        return GPE_ERR_CAPACITY;
    }
    cudaStream_t st = as_stream(stream);
    if (cnt > 0) {
        const bool ids = (s->prm.flags & (GPE_PBF_TRACK_IDS | GPE_PBF_PAIR_IDS)) != 0;
        k_pbf_emit<<<blocks_for(cnt), T_PART, 0, st>>>(s->k, h, s->pos, s->vel, s->d_count, (int32_t)s->cap,
                                                       ids ? s->ids[s->id_cur] : nullptr, s->status);
        GPE_CHECK_LAUNCH("k_pbf_emit");
    }
    s->have_state = true;
    return GPE_OK;
}

extern "C" int32_t gpe_pbf_publish(gpe_pbf* s, const gpe_view* view, int32_t view_mem, void* stream)
{
    gpe::clear_error();
    if (!s || !view || (view_mem != GPE_MEM_HOST && view_mem != GPE_MEM_DEVICE)) { return GPE_ERR_BAD_ARG; }
    if (view_mem == GPE_MEM_HOST && (!view->pos || !view->vel || !view->counts || view->chunks_x <= 0 ||
                                     view->chunks_y <= 0 || !(view->chunk_dim > 0.f) || view->chunk_capacity <= 0)) {
        return GPE_ERR_BAD_ARG;
    }
    if (s->XS >= 0) { return GPE_ERR_NOT_READY; }
    cudaStream_t st = as_stream(stream);
    const gpe_view* vp = nullptr;
    gpe_view vv{};
    if (view_mem == GPE_MEM_HOST) {
        vv = *view;
        GPE_TRY_CUDA(cudaMemsetAsync(vv.counts, 0, sizeof(int32_t) * (size_t)vv.chunks_x * vv.chunks_y, st));
    } else {
        vp = view;
        k_view_zero<<<(unsigned)sm_count(), T_PART, 0, st>>>(vp);
        GPE_CHECK_LAUNCH("k_view_zero");
    }
    if (lsize(s) > 0) {
        k_pbf_publish<<<(unsigned)((lsize(s) + PUB_PER_BLOCK - 1) / PUB_PER_BLOCK), T_PART, 0, st>>>(
            s->k, vv, vp, s->pos, s->vel, s->status);
        GPE_CHECK_LAUNCH("k_pbf_publish");
    }
    return GPE_OK;
}

extern "C" int32_t gpe_pbf_publish_chunks(gpe_pbf* s, const gpe_chunk_state* state, void* stream)
{
    gpe::clear_error();
    if (!s || !state) { return GPE_ERR_BAD_ARG; }
    if (s->nd != 1 || s->XS >= 0) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_publish_chunks: needs one scene, between steps");
        return GPE_ERR_NOT_READY;
    }
    const gpe_chunk_state c = *state;
    if (!c.pos || !c.pred || !c.vel || !c.counts || !c.offsets || c.chunks_x < 1 || c.chunks_y < 1 ||
        c.chunk_cells < 1 || c.chunk_cells > 32 || !(c.chunk_dim > 0.f) || c.chunk_capacity < 1 ||
        c.chunk_capacity > 0xFFFF) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_publish_chunks: bad chunk state (null array, more than 32 x 32 "
                                        "cells or 65535 slots per chunk)");
        return GPE_ERR_BAD_ARG;
    }
    cudaStream_t st     = as_stream(stream);
    const size_t chunks = (size_t)c.chunks_x * (size_t)c.chunks_y;
    drop_hist(s); // the chunk sort uses the (key, rank) array, where the next step's keys may be waiting
    GPE_TRY_CUDA(cudaMemsetAsync(c.offsets, 0, sizeof(uint32_t) * chunks * (size_t)(c.chunk_cells * c.chunk_cells), st));
    const int64_t n = lsize(s);
    if (n > 0) {
        k_chunk_hist<<<blocks_for(n), T_PART, 0, st>>>(s->k, c, s->pos, s->vel, s->keyrank);
        GPE_CHECK_LAUNCH("k_chunk_hist");
    }
    k_chunk_scan<<<(unsigned)chunks, 1024, 0, st>>>(c, s->status);
    GPE_CHECK_LAUNCH("k_chunk_scan");
    if (n > 0) {
        k_chunk_place<<<blocks_for(n), T_PART, 0, st>>>(s->k, c, s->pos, s->vel, s->lam, s->keyrank);
        GPE_CHECK_LAUNCH("k_chunk_place");
    }
    return GPE_OK;
}

extern "C" int32_t gpe_pbf_enqueue(gpe_pbf* s, int32_t n_steps, void* stream)
{
    gpe::clear_error();
    if (!s || n_steps < 0) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    if (s->XS >= 0) { return GPE_ERR_NOT_READY; }
    if (s->warm == GPE_WARM_MLP && !s->mem_valid) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_enqueue: run one gpe_pbf_step first to start the multiplier memory");
        return GPE_ERR_NOT_READY;
    }
    cudaStream_t st   = as_stream(stream);
    // the recorded sequence may be replayed after anything (a step of this engine may have left a histogram
    // in the array): it clears the histogram array, starts from the full sort and leaves no histogram behind
    // (its last step's XSPH computes none)
    drop_hist(s);
    s->count_dirty = true;
    int32_t rc    = GPE_OK;
    const int id0 = s->id_cur;
    for (int32_t k = 0; k < n_steps && rc == GPE_OK; ++k) { rc = run_step(s, st, k + 1 < n_steps); }
    if (rc) { return rc; }
    // return the id buffer role to where it started, so the recorded sequence can be replayed (positions stay
    // in one buffer: every step writes its end positions where it read its start positions)
    const size_t n = (size_t)lsize(s);
    if (s->id_cur != id0 && n > 0) {
        GPE_TRY_CUDA(cudaMemcpyAsync(s->ids[id0], s->ids[s->id_cur], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice,
                                     st));
    }
    s->id_cur    = id0;
    s->have_sort = true;
    return GPE_OK;
}

// =====================================================================================================
// Tuning (cell size, block size, persistent solve) and the autotuner
// =====================================================================================================

namespace {

int32_t apply_tuning(gpe_pbf* s, const gpe_pbf_tuning& t)
{
    if (!(t.cell >= 0.f) || (t.block != 128 && t.block != 256 && t.block != 512) ||
        (t.persistent < 0 || t.persistent > 2) || !(t.skin >= 0.f && t.skin <= 1.f)) {
        gpe::set_error(GPE_ERR_BAD_ARG,
                       "gpe_pbf_set_tuning: block must be 128, 256 or 512, persistent 0, 1 or 2, skin in [0, 1]");
        return GPE_ERR_BAD_ARG;
    }
    drop_hist(s);
    const float c_old = s->prm.cell > 0.f ? s->prm.cell : s->prm.h;
    const float c_new = t.cell > 0.f ? t.cell : s->prm.h;
    if (c_new != c_old) {
        if (c_new < 0.2f * s->prm.h) {
            gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_set_tuning: cell size below h/5");
            return GPE_ERR_BAD_ARG;
        }
        gpe_pbf_params np = s->prm;
        np.cell           = c_new;
        const uint64_t nc = count_cells(&np, s->doms.data(), s->nd);
        if (nc > s->cells_cap) {
            gpe::set_error(GPE_ERR_CAPACITY, "gpe_pbf_set_tuning: %llu cells exceed the %llu the engine holds",
                           (unsigned long long)nc, (unsigned long long)s->cells_cap);
            return GPE_ERR_CAPACITY;
        }
        s->prm.cell = c_new;
        build_domains(s);
        GPE_TRY_CUDA(cudaMemcpy(s->d_doms, s->domdev.data(), sizeof(DomDev) * (size_t)s->nd, cudaMemcpyHostToDevice));
        s->have_sort = false;
    }
    if (t.block != s->block) { s->coop_grid = 0; }
    s->block      = t.block;
    s->persistent  = t.persistent != 0;
    s->step_kernel = t.persistent == 2;
    s->skin        = t.skin;
    bind_k(s);
    s->drop_graphs();
    return GPE_OK;
}

struct TuneKey {
    int32_t nd, log_n, log_aspect, iters;
    uint32_t flags;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(nd, log_n, log_aspect, iters, flags) < std::tie(o.nd, o.log_n, o.log_aspect, o.iters, o.flags);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, gpe_pbf_tuning> g_tune_cache;

} // namespace

extern "C" int32_t gpe_pbf_get_tuning(const gpe_pbf* s, gpe_pbf_tuning* t)
{
    if (!s || !t) { return GPE_ERR_BAD_ARG; }
    t->cell       = s->prm.cell > 0.f ? s->prm.cell : s->prm.h;
    t->block      = s->block;
    t->persistent = s->step_kernel ? 2 : (s->persistent ? 1 : 0);
    t->skin       = s->skin;
    return GPE_OK;
}

extern "C" int32_t gpe_pbf_set_tuning(gpe_pbf* s, const gpe_pbf_tuning* t)
{
    gpe::clear_error();
    if (!s || !t) { return GPE_ERR_BAD_ARG; }
    if (s->XS >= 0) { return GPE_ERR_NOT_READY; }
    return apply_tuning(s, *t);
}

extern "C" int32_t gpe_pbf_autotune(gpe_pbf* s, int32_t trial_steps, gpe_pbf_tuning* best, float* ms_per_step,
                                    void* stream)
{
    gpe::clear_error();
    if (!s || trial_steps < 1) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state || s->XS >= 0 || s->warm != GPE_WARM_NONE || s->dynamic) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_pbf_autotune: needs a state, GPE_WARM_NONE and a host particle count");
        return GPE_ERR_NOT_READY;
    }
    cudaStream_t st = as_stream(stream);
    // the cache key: scenes, particle count and mean aspect to the nearest power of two, iterations, flags
    double aspect = 0.0;
    for (const gpe_domain& d : s->doms) { aspect += std::log2((double)d.extent[0] / (double)d.extent[1]); }
    const TuneKey key{s->nd, (int32_t)std::lround(std::log2((double)std::max<int64_t>(s->n, 1))),
                      (int32_t)std::lround(aspect / (double)s->nd), s->prm.iters,
                      s->prm.flags & (GPE_PBF_SELF_GRAD | GPE_PBF_PAIR_IDS)};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            const int32_t rc = apply_tuning(s, it->second);
            if (rc == GPE_OK && best) { *best = it->second; }
            if (ms_per_step) { *ms_per_step = -1.f; } // not timed: taken from the cache
            return rc;
        }
    }
    // save the state (positions, velocities, scenes, ids), restored before every trial and at the end
    const int64_t n   = s->n;
    const bool ids    = (s->prm.flags & (GPE_PBF_TRACK_IDS | GPE_PBF_PAIR_IDS)) != 0;
    void* save        = nullptr;
    const size_t nb   = (size_t)std::max<int64_t>(n, 1);
    GPE_TRY_CUDA(cudaMalloc(&save, nb * (2 * sizeof(float2) + 2 * sizeof(int32_t))));
    float2* sx        = static_cast<float2*>(save);
    float2* sv        = sx + nb;
    int32_t* sd       = reinterpret_cast<int32_t*>(sv + nb);
    uint32_t* sid     = reinterpret_cast<uint32_t*>(sd + nb);
    auto restore      = [&]() -> int32_t {
        int32_t rc = gpe_pbf_set_state(s, reinterpret_cast<float*>(sx), reinterpret_cast<float*>(sv),
                                       s->nd > 1 ? sd : nullptr, n, GPE_MEM_DEVICE, stream);
        if (rc == GPE_OK && ids && n > 0) {
            GPE_TRY_CUDA(cudaMemcpyAsync(s->ids[s->id_cur], sid, sizeof(uint32_t) * (size_t)n,
                                         cudaMemcpyDeviceToDevice, st));
        }
        return rc;
    };
    int32_t rc = gpe_pbf_get_state(s, reinterpret_cast<float*>(sx), reinterpret_cast<float*>(sv),
                                   s->nd > 1 ? sd : nullptr, n, GPE_MEM_DEVICE, stream);
    if (rc == GPE_OK && ids && n > 0) {
        const cudaError_t e = cudaMemcpyAsync(sid, s->ids[s->id_cur], sizeof(uint32_t) * (size_t)n,
                                              cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            gpe::set_cuda_error(e, "gpe_pbf_autotune");
            rc = GPE_ERR_CUDA;
        }
    }
    gpe_pbf_tuning start{};
    gpe_pbf_get_tuning(s, &start);
    gpe_pbf_tuning win = start;
    float win_ms       = -1.f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == GPE_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) {
        rc = GPE_ERR_CUDA;
    }
    // one trial: the candidate's time per step over trial_steps steps from the saved state, or -1 when it
    // cannot run (e.g. the h/2 grid does not fit) or its state went bad
    auto trial = [&](const gpe_pbf_tuning& cand) -> float {
        if (apply_tuning(s, cand) != GPE_OK) { return -1.f; }
        rc = restore();
        if (rc) { return -1.f; }
        // two untimed steps capture the candidate's graph
        if (gpe_pbf_step(s, 2, stream) != GPE_OK || cudaStreamSynchronize(st) != cudaSuccess) {
            cudaGetLastError();
            return -1.f;
        }
        cudaEventRecord(e0, st);
        const int32_t src = gpe_pbf_step(s, trial_steps, stream);
        cudaEventRecord(e1, st);
        if (src != GPE_OK || cudaEventSynchronize(e1) != cudaSuccess) {
            cudaGetLastError();
            return -1.f;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        uint32_t stt = 0;
        gpe_pbf_status(s, &stt, stream);
        return stt != 0 ? -1.f : ms / (float)trial_steps;
    };
    // cell h with candidate masks (skin 0.1, 0.075 or 0.05 h) and without, and h/2 (no masks: its scan has
    // five rows)
    const float cells[5] = {s->prm.h, s->prm.h, s->prm.h, s->prm.h, 0.5f * s->prm.h};
    const float skins[5] = {0.1f, 0.075f, 0.05f, 0.f, 0.f};
    const int32_t blocks[3] = {128, 256, 512};
    std::vector<std::pair<float, gpe_pbf_tuning>> timed;
    for (int ci = 0; ci < 5 && rc == GPE_OK; ++ci) {
        for (int bi = 0; bi < 3 && rc == GPE_OK; ++bi) {
            for (int pi = 0; pi < 3 && rc == GPE_OK; ++pi) {
                const gpe_pbf_tuning cand{cells[ci], blocks[bi], pi, skins[ci]};
                const float ms = trial(cand);
                if (ms >= 0.f) { timed.emplace_back(ms, cand); }
            }
        }
    }
    // The leading candidates are often within 1-2% of each other, about as much as one trial's timing
    // varies: the three fastest run three more trials each, taking turns, and the one with the smallest
    // median of its four times wins.
    std::stable_sort(timed.begin(), timed.end(),
                     [](const auto& a, const auto& b) { return a.first < b.first; });
    const size_t finalists = std::min<size_t>(timed.size(), 3);
    std::vector<std::vector<float>> times(finalists);
    for (size_t f = 0; f < finalists; ++f) { times[f].push_back(timed[f].first); }
    for (int round = 0; round < 3 && rc == GPE_OK && finalists > 1; ++round) {
        for (size_t f = 0; f < finalists && rc == GPE_OK; ++f) {
            const float ms = trial(timed[f].second);
            if (ms >= 0.f) { times[f].push_back(ms); }
        }
    }
    for (size_t f = 0; f < finalists; ++f) {
        std::vector<float>& t = times[f];
        std::sort(t.begin(), t.end());
        const float med = t.size() % 2 ? t[t.size() / 2] : 0.5f * (t[t.size() / 2 - 1] + t[t.size() / 2]);
        if (win_ms < 0.f || med < win_ms) {
            win_ms = med;
            win    = timed[f].second;
        }
    }
    if (e0) { cudaEventDestroy(e0); }
    if (e1) { cudaEventDestroy(e1); }
    int32_t rc2 = apply_tuning(s, win_ms >= 0.f ? win : start);
    if (rc2 == GPE_OK) { rc2 = restore(); }
    cudaStreamSynchronize(st);
    cudaFree(save);
    if (rc) { return rc; }
    if (rc2) { return rc2; }
    if (win_ms >= 0.f) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = win;
    }
    if (best) { *best = win_ms >= 0.f ? win : start; }
    if (ms_per_step) { *ms_per_step = win_ms; }
    return GPE_OK;
}

// =====================================================================================================
// Warm start and training-pair collection
// =====================================================================================================

extern "C" int32_t gpe_pbf_set_warm_start(gpe_pbf* s, int32_t mode, const gpe_mlp* mlp)
{
    gpe::clear_error();
    if (!s || mode < GPE_WARM_NONE || mode > GPE_WARM_MLP || (mode == GPE_WARM_MLP && !mlp)) {
        return GPE_ERR_BAD_ARG;
    }
    if (s->XS >= 0) { return GPE_ERR_NOT_READY; }
    drop_hist(s);
    if (mode == GPE_WARM_MLP) {
        // the network kernel's tiles live in shared memory: prefer the largest carveout so that 6 CTAs fit
        GPE_TRY_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(k_mlp_apply),
                                          cudaFuncAttributePreferredSharedMemoryCarveout,
                                          (int)cudaSharedmemCarveoutMaxShared));
        // persistent grid: one wave of resident CTAs, as many per SM as shared memory (about 36 KB a CTA plus
        // the driver's 1 KB: 6), registers and TMEM (512 columns / 64: 8) allow, so that no CTA waits for
        // TMEM and none queues behind CTAs that work through all their tiles first (8 CTAs per SM, 1.33
        // waves: 94 against 90 us for features and network at 1M particles)
        cudaFuncAttributes fa{};
        GPE_TRY_CUDA(cudaFuncGetAttributes(&fa, k_mlp_apply));
        int dev = 0, smem_sm = 0, regs_sm = 0;
        GPE_TRY_CUDA(cudaGetDevice(&dev));
        GPE_TRY_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        GPE_TRY_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
        const int by_smem = smem_sm / (int)(fa.sharedSizeBytes + 1024);
        const int by_regs = regs_sm / std::max(1, fa.numRegs * MLP_TILE);
        const int per_sm  = std::max(1, std::min({by_smem, by_regs, (int)(512 / MLP_FWD_TMEM_COLS)}));
        s->lam_grid       = per_sm * gpe::sm_count();
        if (!s->feat) {
            // layer-1 operand tiles of the network, 32 B per particle, whole tiles
            const size_t tiles = (size_t)((s->cap + MLP_TILE - 1) / MLP_TILE);
            GPE_TRY_CUDA(cudaMalloc(&s->feat, (tiles > 0 ? tiles : 1) * MLP_A1_TILE_BYTES));
        }
    }
    s->warm = mode;
    s->mlp  = mode == GPE_WARM_MLP ? mlp : nullptr;
    s->mem_valid = false;
    GPE_TRY_CUDA(cudaMemset(s->acc, 0, sizeof(float) * (size_t)s->cap));
    GPE_TRY_CUDA(cudaDeviceSynchronize());
    s->drop_graphs();
    return GPE_OK;
}

extern "C" int32_t gpe_mlp_collect(gpe_mlp* m, gpe_pbf* s, int32_t n_steps, int32_t stride, uint64_t seed,
                                   void* stream)
{
    gpe::clear_error();
    if (!m || !s || n_steps < 0 || stride < 1) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    if (s->warm != GPE_WARM_NONE || s->XS >= 0) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_mlp_collect: the engine must be in GPE_WARM_NONE between steps");
        return GPE_ERR_NOT_READY;
    }
    cudaStream_t st       = as_stream(stream);
    const gpe::MlpData md = gpe::mlp_data(m);
    GPE_TRY_CUDA(cudaMemsetAsync(s->acc, 0, sizeof(float) * (size_t)s->cap, st));
    drop_hist(s);
    uint64_t rs   = seed;
    int32_t rc    = GPE_OK;
    s->collecting = true;
    for (int32_t k = 0; k < n_steps && rc == GPE_OK; ++k) {
        // SplitMix64 (Steele, Lea & Flood 2014) step for the per-step selection salt
        uint64_t z = (rs += 0x9E3779B97F4A7C15ull);
        z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        // the first step has no previous multipliers to learn from: it only starts the sums
        s->col = CollectK{md.X, md.T, md.idx, md.cnt, (int32_t)md.cap, (uint32_t)z, k == 0 ? 0u : (uint32_t)stride};
        rc     = run_step(s, st);
    }
    s->collecting = false;
    s->col        = CollectK{};
    gpe::mlp_set_pair_iters(m, s->prm.iters);
    if (rc) { return rc; }
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    s->have_sort = true;
    return GPE_OK;
}

// =====================================================================================================
// Allocation-free predict + sort (gpe_pbf_predict_sort_noalloc)
//
// For callers that cannot call cudaMalloc (a host whose device memory belongs to another framework, a
// real-time loop that must not allocate after start-up). The scratch of the sort — unsorted predictions,
// (key, rank) pairs, cell buckets, the cell histogram and the scan's block sums — lives in one fixed
// static device array sized for GPE_NOALLOC_MAX_PARTICLES particles and GPE_NOALLOC_MAX_CELLS cells. Every
// GPU that loads this library holds the array until the process exits. All calls share it and each call
// overwrites it; the histogram is cleared at the start of every call. Calls that overlap on the GPU race.
// =====================================================================================================

namespace {

constexpr size_t NA_MAX_N     = (size_t)GPE_NOALLOC_MAX_PARTICLES;
constexpr size_t NA_MAX_CELLS = (size_t)GPE_NOALLOC_MAX_CELLS;
constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t NA_OFF_KR    = 0;                                                  // uint2[n]
constexpr size_t NA_OFF_BK    = na_align(NA_OFF_KR + sizeof(uint2) * NA_MAX_N);     // uint32[n]
constexpr size_t NA_OFF_CNT   = na_align(NA_OFF_BK + sizeof(uint32_t) * NA_MAX_N);  // uint32[cells]
constexpr size_t NA_OFF_BS    = na_align(NA_OFF_CNT + sizeof(uint32_t) * NA_MAX_CELLS);
constexpr size_t NA_BYTES     = na_align(NA_OFF_BS + sizeof(uint32_t) * (NA_MAX_CELLS / 2048 + 1));

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
uint8_t* g_na_ptr[NA_MAX_DEVICES] = {};

} // namespace

static __device__ __align__(256) uint8_t gpe_noalloc_scratch[NA_BYTES];

namespace {

// Device address of the scratch array on the current device. In host code the symbol itself is only a
// host-side stand-in, so the address is looked up once per device (with that device current) and cached.
int32_t noalloc_scratch(uint8_t** out)
{
    int dev = 0;
    GPE_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NA_MAX_DEVICES) {
        gpe::set_error(GPE_ERR_DEVICE, "gpe_pbf_predict_sort_noalloc: device %d out of range", dev);
        return GPE_ERR_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void* p             = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, gpe_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            gpe::set_cuda_error(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress");
            return GPE_ERR_CUDA;
        }
        g_na_ptr[dev] = static_cast<uint8_t*>(p);
    }
    *out = g_na_ptr[dev];
    return GPE_OK;
}

} // namespace

extern "C" int32_t gpe_pbf_predict_sort_noalloc(const gpe_pbf_params* params, const gpe_domain* domain,
                                                const float* pos, const float* vel, int64_t n, float* pos_sorted,
                                                float* pred_sorted, uint32_t* key_sorted, uint32_t* perm,
                                                uint32_t* cell_start, int64_t n_cells, void* stream)
{
    gpe::clear_error();
    if (!domain || !cell_start || n < 0 ||
        (n > 0 && (!pos || !vel || !pos_sorted || !pred_sorted || !key_sorted || !perm))) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_predict_sort_noalloc: null pointer or negative size");
        return GPE_ERR_BAD_ARG;
    }
    int32_t rc = validate_params(params);
    if (rc) { return rc; }
    if (!(domain->extent[0] > 0.f) || !(domain->extent[1] > 0.f)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_predict_sort_noalloc: non-positive scene extent");
        return GPE_ERR_BAD_ARG;
    }
    const uint64_t cells = count_cells(params, domain, 1);
    if (cells == CELLS_INVALID) {
        gpe::set_error(GPE_ERR_CAPACITY,
                       "gpe_pbf_predict_sort_noalloc: the scene extent is not finite or spans 2^30 cells or more");
        return GPE_ERR_CAPACITY;
    }
    if ((int64_t)cells != n_cells) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_pbf_predict_sort_noalloc: the scene has %llu cells, not %lld",
                       (unsigned long long)cells, (long long)n_cells);
        return GPE_ERR_BAD_ARG;
    }
    if ((size_t)n > NA_MAX_N || (size_t)cells > NA_MAX_CELLS) {
        gpe::set_error(GPE_ERR_CAPACITY,
                       "gpe_pbf_predict_sort_noalloc: %lld particles / %llu cells exceed the static scratch "
                       "limits of %d particles / %d cells",
                       (long long)n, (unsigned long long)cells, GPE_NOALLOC_MAX_PARTICLES, GPE_NOALLOC_MAX_CELLS);
        return GPE_ERR_CAPACITY;
    }
    // The kernels access pos, vel, pos_sorted and pred_sorted as float2 and the index arrays as 32-bit words:
    // a misaligned caller pointer (a view offset by one float, say) would fault the whole context, so it is
    // refused here, before any device work.
    const auto misaligned = [](const void* ptr, uintptr_t a) { return (reinterpret_cast<uintptr_t>(ptr) & (a - 1)) != 0; };
    if (misaligned(cell_start, 4) ||
        (n > 0 && (misaligned(pos, 8) || misaligned(vel, 8) || misaligned(pos_sorted, 8) ||
                   misaligned(pred_sorted, 8) || misaligned(key_sorted, 4) || misaligned(perm, 4)))) {
        gpe::set_error(GPE_ERR_BAD_ARG,
                       "gpe_pbf_predict_sort_noalloc: pos, vel, pos_sorted and pred_sorted must be 8-byte aligned, "
                       "key_sorted, perm and cell_start 4-byte aligned");
        return GPE_ERR_BAD_ARG;
    }
    uint8_t* scratch = nullptr;
    rc               = noalloc_scratch(&scratch);
    if (rc) { return rc; }
    uint2* keyrank   = reinterpret_cast<uint2*>(scratch + NA_OFF_KR);
    uint32_t* bucket = reinterpret_cast<uint32_t*>(scratch + NA_OFF_BK);
    uint32_t* count  = reinterpret_cast<uint32_t*>(scratch + NA_OFF_CNT);
    uint32_t* bsum   = reinterpret_cast<uint32_t*>(scratch + NA_OFF_BS);

    // kernel constants for the one scene, as build_domains derives them for an engine
    const float cell = params->cell > 0.f ? params->cell : params->h;
    PbfK k           = make_k(*params);
    DomDev d{};
    d.ox   = domain->origin[0];
    d.oy   = domain->origin[1];
    d.lox  = domain->origin[0];
    d.loy  = domain->origin[1];
    d.hix  = (domain->origin[0] + domain->extent[0]) - params->wall_margin;
    d.hiy  = (domain->origin[1] + domain->extent[1]) - params->wall_margin;
    d.ncx  = cells_along(domain->extent[0], cell);
    d.ncy  = cells_along(domain->extent[1], cell);
    d.coff = 0;
    k.d0   = d;
    k.n    = (int32_t)n;
    k.ncells = (uint32_t)cells;

    cudaStream_t st = as_stream(stream);
    // the histogram must start at zero whatever an earlier (possibly failed) call left behind
    GPE_TRY_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t) * cells, st));
    if (n > 0) {
        k_predict_hist<false><<<blocks_for(n), T_PART, 0, st>>>(k, nullptr, nullptr,
                                                                reinterpret_cast<const float2*>(pos),
                                                                reinterpret_cast<const float2*>(vel), keyrank,
                                                                count);
        GPE_CHECK_LAUNCH("k_predict_hist (noalloc)");
    }
    rc = launch_exclusive_scan(count, (uint32_t)cells, bsum, cell_start, st);
    if (rc) { return rc; }
    if (n > 0) {
        rc = launch_scatter(keyrank, n, cell_start, bucket, (uint32_t)cells, st);
        if (rc) { return rc; }
        k_place<<<blocks_for(n), T_PART, 0, st>>>(k, keyrank, cell_start, bucket,
                                                  reinterpret_cast<const float2*>(pos),
                                                  reinterpret_cast<const float2*>(vel), nullptr,
                                                  reinterpret_cast<float2*>(pos_sorted),
                                                  reinterpret_cast<float2*>(pred_sorted), perm, key_sorted, nullptr,
                                                  nullptr, nullptr, nullptr, nullptr);
        GPE_CHECK_LAUNCH("k_place (noalloc)");
    }
    return GPE_OK;
}
