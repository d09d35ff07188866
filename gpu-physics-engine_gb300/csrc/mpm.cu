// mpm.cu — MLS-MPM step on GB300 (sm_103a).
//
// The reference runs, per substep, resetGrid -> P2GKernel -> gridKernel -> G2PKernel (MPM.cu:353-371) with
// 27 scalar global atomics per particle (MPM.cu:124-126) and a separate streaming pass over the grid.
// Here one step is three launches:
//   k_p2g            P2G, two consecutive particles per thread: lanes that share a stencil base node
//                    (particles are kept sorted by base node) sum their contributions per node with a
//                    segmented shuffle reduction, and the run's first lane adds each of its 9 node sums to
//                    the grid with one vector global atomic (red.global.add.v4.f32, resolved in L2).
//   k_grid_vel       the grid update (v = p/m + g dt, walls, MPM.cu:150-175) once per node into an array of
//                    node velocities (8 bytes a node), zeroing the grid read two steps earlier in the same
//                    pass (three grids rotate).
//   k_g2p            G2P: each particle gathers its 9 node velocities from that array (L1/L2 hits: sorted
//                    neighbours share nodes).
// (Measured alternatives, each slower: a G2P that staged its block's node box in shared memory and updated
// each node there, 0.198 against 0.186 ms per step at 4M particles; a G2P fused with the next step's P2G,
// 0.159 against 0.153 ms, its 64 registers holding both passes' state.)
// Stage kernels (k_clear, k_p2g, k_grid, k_g2p on an updated grid) reproduce the reference's four kernels
// one to one for stage-level parity tests.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <type_traits>
#include <vector>

#include "emit.cuh"
#include "gpe_internal.h"

namespace gpe {

// One scene's node grid: nodes [goff, goff + nx * ny) of the node array, row-major; its particles are
// clamped to [lo, hi] (handleOOB, MPM.cu:267-301).
struct MpmScene {
    int32_t nx, ny;
    uint32_t goff;
    float lo_x, lo_y, hi_x, hi_y;
};

struct MpmK {
    float dx, inv_dx, goff, dt;
    float gdt_x, gdt_y;
    float mass, vol0;
    int32_t bc_type, bc_width;
    MpmScene s0;            // the scene when there is one
    const MpmScene* scenes; // device table when there are several (particles carry their scene)
    int32_t n_scenes;
    int64_t nn;             // nodes of all scenes
    int32_t material;
    uint32_t flags;
    float k_bulk, gamma, p_min, p_max, J_min, J_max;
    float mu0, la0, theta_c, theta_s, hardening;
    float sh0, sh1, sh2, sh3; // sand friction-angle hardening, degrees
    float sand_cf;            // (d la + 2 mu) / (2 mu), d = 2
    float apic_s; // 4 / dx^2
    int32_t n;            // particle count when n_dev is null
    const int32_t* n_dev; // device-resident count (the reference's num_points[0], MPM.cu:64)
};

namespace {

constexpr int T_MPM     = 256;

// single-material modes are the material ids; MODE_MIXED reads an id per particle
enum MatMode { MODE_FLUID = 0, MODE_COROT = 1, MODE_SNOW = 2, MODE_NEOHOOKEAN = 3, MODE_SAND = 4, MODE_MIXED = 8 };

// materials whose particles carry F / J between steps (corotated and Neo-Hookean need no J: their volume
// is det F; the fluid keeps F only when asked to, as the reference does)
__device__ __forceinline__ bool keeps_f(int m, bool track_f) { return m != MODE_FLUID || track_f; }
__device__ __forceinline__ bool keeps_j(int m) { return m == MODE_FLUID || m == MODE_SNOW || m == MODE_SAND; }

__device__ __forceinline__ int32_t count_of(const MpmK& k) { return k.n_dev ? __ldg(k.n_dev) : k.n; }

// the scene of particle i (ids are checked when set; clamped here as well, so that no id reads past the table).
// MS: the engine holds several scenes (kernels for one scene compile without the lookup).
template <bool MS = true>
__device__ __forceinline__ MpmScene scene_of(const MpmK& k, const int32_t* __restrict__ sid, int32_t i)
{
    if (!MS || k.n_scenes <= 1) { return k.s0; }
    return k.scenes[min(max(__ldg(&sid[i]), 0), k.n_scenes - 1)];
}

// the scene that owns node idx (the last whose first node is not past idx)
__device__ __forceinline__ MpmScene scene_of_node(const MpmK& k, int64_t idx)
{
    if (k.n_scenes <= 1) { return k.s0; }
    int32_t lo = 0, hi = k.n_scenes - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if ((int64_t)k.scenes[mid].goff <= idx) {
            lo = mid;
        } else {
            hi = mid - 1;
        }
    }
    return k.scenes[lo];
}

struct Stencil {
    int32_t bx, by;
    float fx, fy;
    float wx[3], wy[3];
};

// quadratic B-spline weights, MPM.cu:92-110 (gridCoord MPM.cu:84)
__device__ __forceinline__ Stencil stencil(const MpmK& k, const MpmScene& sc, float2 p, uint32_t* status)
{
    Stencil s;
    const float gx = p.x * k.inv_dx + k.goff;
    const float gy = p.y * k.inv_dx + k.goff;
    int32_t bx     = (int32_t)floorf(gx - 0.5f);
    int32_t by     = (int32_t)floorf(gy - 0.5f);
    if (bx < 0 || by < 0 || bx > sc.nx - 3 || by > sc.ny - 3) {
        // outside the halo: clamp the stencil to the grid and report it (the reference relies on its 2-node
        // halo instead, MPM.cu:84 / cuda-engine.h:192-194)
        atomicOr(status, GPE_STATUS_CAPACITY);
        bx = min(max(bx, 0), sc.nx - 3);
        by = min(max(by, 0), sc.ny - 3);
    }
    s.bx     = bx;
    s.by     = by;
    s.fx     = gx - (float)bx;
    s.fy     = gy - (float)by;
    s.wx[0]  = 0.5f * (1.5f - s.fx) * (1.5f - s.fx);
    s.wx[1]  = 0.75f - (s.fx - 1.0f) * (s.fx - 1.0f);
    s.wx[2]  = 0.5f * (s.fx - 0.5f) * (s.fx - 0.5f);
    s.wy[0]  = 0.5f * (1.5f - s.fy) * (1.5f - s.fy);
    s.wy[1]  = 0.75f - (s.fy - 1.0f) * (s.fy - 1.0f);
    s.wy[2]  = 0.5f * (s.fy - 0.5f) * (s.fy - 0.5f);
    return s;
}

__device__ __forceinline__ int mat_of(const MpmK& k, int mode, const int32_t* __restrict__ mat, int32_t i)
{
    return mode == MODE_MIXED ? __ldg(&mat[i]) : mode;
}

// rotation of the polar decomposition F = R S of a 2x2 matrix (row-major xx, xy, yx, yy)
__device__ __forceinline__ float4 polar_rotation(float4 F)
{
    const float c = F.x + F.w, s = F.z - F.y;
    const float n2 = c * c + s * s;
    if (n2 < 1e-30f) { return make_float4(1.f, 0.f, 0.f, 1.f); }
    const float in = rsqrtf(n2);
    return make_float4(c * in, -s * in, s * in, c * in);
}

// 2x2 SVD through the polar decomposition: F = U diag(s) V^T with U, V rotations
__device__ __forceinline__ void svd2(float4 F, float4& U, float2& s, float4& V)
{
    const float4 R = polar_rotation(F);
    const float a  = R.x * F.x + R.z * F.z;
    const float b  = R.x * F.y + R.z * F.w;
    const float d  = R.y * F.y + R.w * F.w;
    float c = 1.f, sn = 0.f;
    if (fabsf(b) > 1e-30f) { sincosf(0.5f * atan2f(2.f * b, a - d), &sn, &c); }
    V   = make_float4(c, -sn, sn, c);
    s.x = c * c * a + 2.f * c * sn * b + sn * sn * d;
    s.y = sn * sn * a - 2.f * c * sn * b + c * c * d;
    U   = make_float4(R.x * V.x + R.y * V.z, R.x * V.y + R.y * V.w, R.z * V.x + R.w * V.z, R.z * V.y + R.w * V.w);
}

// Affine momentum Q = m C + coeff * Kirchhoff stress. Fluid: P2GKernel MPM.cu:68-80; elastic: fixed
// corotated tau = 2 mu (F - R) F^T + la (J - 1) J I (Stomakhin et al. 2012), snow hardening exp(xi(1-Jp));
// Neo-Hookean; sand (Klar et al. 2016).
__device__ __forceinline__ float4 affine(const MpmK& k, int m, float4 Cp, float4 F, float J)
{
    if (m == MODE_FLUID) {
        const float inv_j    = 1.f / J;
        const float p_hat    = k.k_bulk * ((k.gamma == 1.f ? inv_j : powf(inv_j, k.gamma)) - 1.f);
        const float pressure = fminf(fmaxf(p_hat, k.p_min), k.p_max);
        const float V_p      = k.vol0 * J;
        const float coeff    = -k.dt * V_p * 4 * k.inv_dx * k.inv_dx;
        return make_float4(k.mass * Cp.x + coeff * -pressure, k.mass * Cp.y + coeff * 0.f,
                           k.mass * Cp.z + coeff * 0.f, k.mass * Cp.w + coeff * -pressure);
    }
    float t0, t1, t2, t3; // Kirchhoff stress
    if (m == MODE_NEOHOOKEAN) {
        // tau = mu (F F^T - I) + la ln(J) I
        const float lj = k.la0 * logf(fmaxf(F.x * F.w - F.y * F.z, 1e-6f));
        t0             = k.mu0 * (F.x * F.x + F.y * F.y - 1.f) + lj;
        t1             = k.mu0 * (F.x * F.z + F.y * F.w);
        t2             = t1;
        t3             = k.mu0 * (F.z * F.z + F.w * F.w - 1.f) + lj;
    } else if (m == MODE_SAND) {
        // St. Venant-Kirchhoff on the Hencky strain: tau = U (2 mu eps + la tr(eps) I) U^T, eps = ln(sigma)
        float4 U, V;
        float2 sg;
        svd2(F, U, sg, V);
        const float e0 = logf(fmaxf(sg.x, 1e-6f)), e1 = logf(fmaxf(sg.y, 1e-6f));
        const float lt = k.la0 * (e0 + e1);
        const float a0 = 2.f * k.mu0 * e0 + lt, a1 = 2.f * k.mu0 * e1 + lt;
        t0             = U.x * U.x * a0 + U.y * U.y * a1;
        t1             = U.x * U.z * a0 + U.y * U.w * a1;
        t2             = t1;
        t3             = U.z * U.z * a0 + U.w * U.w * a1;
    } else {
        float mu = k.mu0, la = k.la0;
        if (m == MODE_SNOW) {
            const float hf = __expf(k.hardening * (1.f - J));
            mu *= hf;
            la *= hf;
        }
        const float4 R  = polar_rotation(F);
        const float Je  = F.x * F.w - F.y * F.z;
        const float a0 = F.x - R.x, a1 = F.y - R.y, a2 = F.z - R.z, a3 = F.w - R.w;
        const float vol = la * (Je - 1.f) * Je;
        t0              = 2.f * mu * (a0 * F.x + a1 * F.y) + vol;
        t1              = 2.f * mu * (a0 * F.z + a1 * F.w);
        t2              = 2.f * mu * (a2 * F.x + a3 * F.y);
        t3              = 2.f * mu * (a2 * F.z + a3 * F.w) + vol;
    }
    const float coeff = -k.dt * k.vol0 * 4.f * k.inv_dx * k.inv_dx;
    return make_float4(k.mass * Cp.x + coeff * t0, k.mass * Cp.y + coeff * t1, k.mass * Cp.z + coeff * t2,
                       k.mass * Cp.w + coeff * t3);
}

// node velocity as the reference's gridKernel leaves it (MPM.cu:150-175), from the raw accumulated node
__device__ __forceinline__ float2 node_velocity(const MpmK& k, const MpmScene& sc, float4 g, int32_t x, int32_t y)
{
    if (!(g.z > 0.f)) { return make_float2(0.f, 0.f); }
    const float inv_m = 1.f / g.z;
    float vx          = g.x * inv_m + k.gdt_x;
    float vy          = g.y * inv_m + k.gdt_y;
    const bool wl = x <= k.bc_width, wr = x >= sc.nx - 1 - k.bc_width;
    const bool wb = y <= k.bc_width, wt = y >= sc.ny - 1 - k.bc_width;
    if (k.bc_type == GPE_MPM_BC_STICKY) {
        if (wl || wr || wb || wt) { vx = vy = 0.f; }
    } else {
        if (wl && vx < 0.f) {
            vx = 0.f;
        } else if (wr && vx > 0.f) {
            vx = 0.f;
        }
        if (wb && vy < 0.f) {
            vy = 0.f;
        } else if (wt && vy > 0.f) {
            vy = 0.f;
        }
    }
    return make_float2(vx, vy);
}

struct PState {
    float2 x, v;
    float4 C, F;
    float J;
};

// G2P body (gridToParticle MPM.cu:227-265, handleOOB MPM.cu:267-301).
// G2P of one particle whose stencil is s; nv(x, y) gives the velocity of scene-local node (x, y)
template <class NodeVel>
__device__ __forceinline__ void g2p_finish(const MpmK& k, const MpmScene& sc, int m, bool track_f, const Stencil& s,
                                           NodeVel nv, PState& ps, uint32_t* status)
{
    // the 2D terms as packed FP32 pairs: vel, (B.x, B.z) and (B.y, B.w)
    float2 vel = make_float2(0.f, 0.f), bxz = make_float2(0.f, 0.f), byw = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float w       = s.wx[i] * s.wy[j];
            const float dpx     = ((float)i - s.fx) * k.dx;
            const float dpy     = ((float)j - s.fy) * k.dx;
            const float2 vi     = nv(s.bx + i, s.by + j);
            const float2 ww     = make_float2(w, w);
            vel                 = fma2(ww, vi, vel);
            const float2 wv     = mul2(ww, vi);
            bxz                 = fma2(wv, make_float2(dpx, dpx), bxz);
            byw                 = fma2(wv, make_float2(dpy, dpy), byw);
        }
    }
    const float4 B = make_float4(bxz.x, byw.x, bxz.y, byw.y);
    float2 pos = make_float2(ps.x.x + vel.x * k.dt, ps.x.y + vel.y * k.dt);
    ps.C       = make_float4(k.apic_s * B.x, k.apic_s * B.y, k.apic_s * B.z, k.apic_s * B.w);
    // handleOOB
    if (!isfinite(pos.x) || !isfinite(vel.x)) {
        pos.x = 0.5f * (sc.lo_x + sc.hi_x);
        vel.x = 0.f;
        atomicOr(status, GPE_STATUS_NONFINITE);
    }
    if (!isfinite(pos.y) || !isfinite(vel.y)) {
        pos.y = 0.5f * (sc.lo_y + sc.hi_y);
        vel.y = 0.f;
        atomicOr(status, GPE_STATUS_NONFINITE);
    }
    if (pos.x < sc.lo_x) {
        pos.x = sc.lo_x;
        vel.x = fmaxf(vel.x, 0.f);
    }
    if (pos.x > sc.hi_x) {
        pos.x = sc.hi_x;
        vel.x = fminf(vel.x, 0.f);
    }
    if (pos.y < sc.lo_y) {
        pos.y = sc.lo_y;
        vel.y = fmaxf(vel.y, 0.f);
    }
    if (pos.y > sc.hi_y) {
        pos.y = sc.hi_y;
        vel.y = fminf(vel.y, 0.f);
    }
    ps.x = pos;
    ps.v = vel;
    // F <- (I + dt C) F; J <- J det(I + dt C), clamped (MPM.cu:258-265)
    const float4 A = make_float4(1 + ps.C.x * k.dt, ps.C.y * k.dt, ps.C.z * k.dt, 1 + ps.C.w * k.dt);
    if (keeps_f(m, track_f)) {
        const float4 F = ps.F;
        ps.F           = make_float4(A.x * F.x + A.y * F.z, A.x * F.y + A.y * F.w, A.z * F.x + A.w * F.z,
                                     A.z * F.y + A.w * F.w);
    }
    if (m == MODE_FLUID) {
        float J = ps.J * (A.x * A.w - A.y * A.z);
        ps.J    = fminf(fmaxf(J, k.J_min), k.J_max);
    } else if (m == MODE_SNOW) {
        float4 U, V;
        float2 sg;
        svd2(ps.F, U, sg, V);
        const float lo = 1.f - k.theta_c, hi = 1.f + k.theta_s;
        const float c0 = fminf(fmaxf(sg.x, lo), hi), c1 = fminf(fmaxf(sg.y, lo), hi);
        ps.J *= (sg.x * sg.y) / (c0 * c1);
        ps.F = make_float4(U.x * c0 * V.x + U.y * c1 * V.y, U.x * c0 * V.z + U.y * c1 * V.w,
                           U.z * c0 * V.x + U.w * c1 * V.y, U.z * c0 * V.z + U.w * c1 * V.w);
    } else if (m == MODE_SAND) {
        // Drucker-Prager return mapping of the Hencky strain (Klar et al. 2016, d = 2): expansion projects to
        // the cone's tip (F = U V^T), a state outside the cone onto its surface; J holds 1 + q
        float4 U, V;
        float2 sg;
        svd2(ps.F, U, sg, V);
        const float e0 = logf(fmaxf(sg.x, 1e-6f)), e1 = logf(fmaxf(sg.y, 1e-6f));
        const float tr = e0 + e1;
        const float d0 = e0 - 0.5f * tr, d1 = e1 - 0.5f * tr;
        const float dn = sqrtf(d0 * d0 + d1 * d1);
        const float q  = ps.J - 1.f;
        const float phi = k.sh0 + (k.sh1 * q - k.sh3) * expf(-k.sh2 * q);
        const float sp  = sinf(phi * 0.017453292519943295f);
        const float alpha = 1.632993161855452f * sp / (3.f - sp); // sqrt(2/3) * 2 sin(phi) / (3 - sin(phi))
        float c0 = 1.f, c1 = 1.f, dq = 0.f;
        bool proj = true;
        if (tr >= 0.f) {
            dq = sqrtf(e0 * e0 + e1 * e1);
        } else {
            const float dg = dn + k.sand_cf * tr * alpha;
            if (dg <= 0.f) {
                proj = false;
            } else {
                const float f = dg / dn;
                c0            = expf(e0 - f * d0);
                c1            = expf(e1 - f * d1);
                dq            = dg;
            }
        }
        if (proj) {
            ps.J += dq;
            ps.F = make_float4(U.x * c0 * V.x + U.y * c1 * V.y, U.x * c0 * V.z + U.y * c1 * V.w,
                               U.z * c0 * V.x + U.w * c1 * V.y, U.z * c0 * V.z + U.w * c1 * V.w);
        }
    }
}

// The node term of one particle (stencil s, velocity v, affine matrix Q) for node (i, j) of its stencil,
// added to (c, cm): w (m v + Q dp) and w m (particleToGrid, MPM.cu:116-126); momentum as packed FP32 pairs
__device__ __forceinline__ void p2g_term(const MpmK& k, const Stencil& s, float2 v, float4 Q, int i, int j,
                                         float2& c, float& cm)
{
    const float w   = s.wx[i] * s.wy[j];
    const float dpx = ((float)i - s.fx) * k.dx;
    const float dpy = ((float)j - s.fy) * k.dx;
    const float2 a  = fma2(make_float2(Q.y, Q.w), make_float2(dpy, dpy),
                           mul2(make_float2(Q.x, Q.z), make_float2(dpx, dpx)));
    c               = add2(c, mul2(make_float2(w, w), fma2(v, make_float2(k.mass, k.mass), a)));
    cm += w * k.mass;
}

// particle i's scene, stencil, velocity and affine matrix for P2G
template <int MODE, bool MS>
__device__ __forceinline__ void p2g_load(const MpmK& k, const float2* __restrict__ x, const float2* __restrict__ v,
                                         const float4* __restrict__ C, const float4* __restrict__ F,
                                         const float* __restrict__ J, const int32_t* __restrict__ mat,
                                         const int32_t* __restrict__ sid, int32_t i, MpmScene& sc, Stencil& s,
                                         float2& vv, float4& Q, uint32_t* status)
{
    sc              = scene_of<MS>(k, sid, i);
    const int m     = mat_of(k, MODE, mat, i);
    const float4 Fp = (m == MODE_FLUID) ? make_float4(1.f, 0.f, 0.f, 1.f) : F[i];
    const float Jp  = keeps_j(m) ? J[i] : 1.f;
    Q               = affine(k, m, C[i], Fp, Jp);
    vv              = v[i];
    s               = stencil(k, sc, x[i], status);
}

// ----- kernels -------------------------------------------------------------------------------------------

__global__ void k_clear(float4* __restrict__ grid, int64_t nn)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += stride) {
        grid[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// P2G, two consecutive particles per thread (particles 2t and 2t + 1). Particles are kept sorted by stencil
// base node, so consecutive lanes mostly share their base node and with it all 9 target nodes. When a
// thread's two particles share one, their terms are summed in registers; then, for each node, the lanes of a
// run (consecutive lanes with the same base node, 64 particles a warp) sum their contributions with a
// segmented shuffle reduction (2 to 5 rounds, as the warp's longest run needs), and the run's first lane adds
// the node sum to the grid with one vector global atomic (red.global.add.v4.f32, resolved in L2). A first
// particle whose base node differs from its partner's (a run boundary inside the thread) adds its 9 terms
// with atomics of its own. One particle per thread measured slower: 0.185 against 0.153 ms per 4M-particle
// step, its shuffle rounds covering half as many particles; staging node sums in a shared-memory tile of the
// block's nodes (float atomics on shared memory, a block barrier, a flush) slower again.
// status[2] counts the warps that need the 5-round reduction (a run of more than 16 lanes).
template <int MODE, bool MS>
__global__ void __launch_bounds__(T_MPM)
    k_p2g(const MpmK k, const float2* __restrict__ x, const float2* __restrict__ v, const float4* __restrict__ C,
          const float4* __restrict__ F, const float* __restrict__ J, const int32_t* __restrict__ mat,
          const int32_t* __restrict__ sid, float4* __restrict__ grid, uint32_t* status)
{
    const int32_t t  = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t n  = count_of(k);
    const int32_t i0 = 2 * t, i1 = 2 * t + 1;
    const bool ok0 = i0 < n, ok1 = i1 < n;
    MpmScene sc0 = k.s0, sc1 = k.s0;
    Stencil s0{}, s1{};
    float2 v0 = make_float2(0.f, 0.f), v1 = v0;
    float4 Q0 = make_float4(0.f, 0.f, 0.f, 0.f), Q1 = Q0;
    if (ok0) { p2g_load<MODE, MS>(k, x, v, C, F, J, mat, sid, i0, sc0, s0, v0, Q0, status); }
    if (ok1) { p2g_load<MODE, MS>(k, x, v, C, F, J, mat, sid, i1, sc1, s1, v1, Q1, status); }
    const uint32_t key0 = ok0 ? sc0.goff + (uint32_t)s0.by * (uint32_t)sc0.nx + (uint32_t)s0.bx : 0xffffffffu;
    const uint32_t key1 = ok1 ? sc1.goff + (uint32_t)s1.by * (uint32_t)sc1.nx + (uint32_t)s1.bx : 0xffffffffu;
    const bool join = ok1 && key0 == key1; // the first particle joins the thread's run
    const bool solo = ok0 && !join;        // the first particle goes to the grid on its own
    // runs of lanes with the same base node (that of the second particle)
    const uint32_t lane    = threadIdx.x & 31u;
    const uint32_t prev    = __shfl_up_sync(0xffffffffu, key1, 1);
    const bool head        = lane == 0u || prev != key1;
    const uint32_t heads   = __ballot_sync(0xffffffffu, head);
    const uint32_t later   = lane == 31u ? 0u : (heads & (0xffffffffu << (lane + 1u)));
    const uint32_t run_end = later ? (uint32_t)(__ffs(later) - 1) : 32u; // first lane of the next run
    const uint32_t longest = __reduce_max_sync(0xffffffffu, head ? run_end - lane : 0u);
    float4* const base1    = grid + (size_t)sc1.goff + (size_t)s1.by * (size_t)sc1.nx + (size_t)s1.bx;
    auto scatter = [&](auto rounds) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int i = q % 3, j = q / 3;
            float2 c = make_float2(0.f, 0.f);
            float cm = 0.f;
            if (join) { p2g_term(k, s0, v0, Q0, i, j, c, cm); }
            if (ok1) { p2g_term(k, s1, v1, Q1, i, j, c, cm); }
#pragma unroll
            for (uint32_t d = 1u; d < (1u << decltype(rounds)::value); d <<= 1) {
                const float ox = __shfl_down_sync(0xffffffffu, c.x, d);
                const float oy = __shfl_down_sync(0xffffffffu, c.y, d);
                const float om = __shfl_down_sync(0xffffffffu, cm, d);
                if (lane + d < run_end) {
                    c = add2(c, make_float2(ox, oy));
                    cm += om;
                }
            }
            if (head && ok1) { atomicAdd(base1 + (size_t)j * (size_t)sc1.nx + i, make_float4(c.x, c.y, cm, 0.f)); }
        }
    };
    // warp-uniform branches on the longest run
    if (longest <= 4u) {
        scatter(std::integral_constant<int, 2>{});
    } else if (longest <= 8u) {
        scatter(std::integral_constant<int, 3>{});
    } else if (longest <= 16u) {
        scatter(std::integral_constant<int, 4>{});
    } else {
        if (lane == 0u) { atomicAdd(status + 2, 1u); }
        scatter(std::integral_constant<int, 5>{});
    }
    if (solo) {
        float4* const base0 = grid + (size_t)sc0.goff + (size_t)s0.by * (size_t)sc0.nx + (size_t)s0.bx;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int i = q % 3, j = q / 3;
            float2 c = make_float2(0.f, 0.f);
            float cm = 0.f;
            p2g_term(k, s0, v0, Q0, i, j, c, cm);
            atomicAdd(base0 + (size_t)j * (size_t)sc0.nx + i, make_float4(c.x, c.y, cm, 0.f));
        }
    }
}

// gridKernel, MPM.cu:131-177 (in place)
__global__ void k_grid(const MpmK k, float4* __restrict__ grid)
{
    const int64_t nn     = k.nn;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn; idx += stride) {
        float4 g        = grid[idx];
        const MpmScene sc    = scene_of_node(k, idx);
        const int64_t local  = idx - (int64_t)sc.goff;
        const float2 vv      = node_velocity(k, sc, g, (int32_t)(local % sc.nx), (int32_t)(local / sc.nx));
        g.x             = vv.x;
        g.y             = vv.y;
        grid[idx]       = g;
    }
}

// The grid update once per node (gridKernel, MPM.cu:131-177) into node velocities, and the zeroing of the
// grid read two steps earlier (zero may be null).
template <bool MS>
__global__ void k_grid_vel(const MpmK k, const float4* __restrict__ grid, float2* __restrict__ vel,
                           float4* __restrict__ zero, int64_t nn)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn; idx += stride) {
        const float4 g      = grid[idx];
        const MpmScene sc   = MS ? scene_of_node(k, idx) : k.s0;
        const int64_t local = idx - (int64_t)sc.goff;
        vel[idx]            = node_velocity(k, sc, g, (int32_t)(local % sc.nx), (int32_t)(local / sc.nx));
        if (zero) { zero[idx] = make_float4(0.f, 0.f, 0.f, 0.f); }
    }
}

// G2P from node velocities: node q's velocity is vel[q * VS] (VS = 1: the node-velocity array; VS = 2: the
// .xy of a float4 grid that k_grid updated in place). Writes the whole particle state.
// 6 blocks per SM (40 registers; the scene-lookup variants spill a little there)
template <int MODE, int VS, bool MS>
__global__ void __launch_bounds__(T_MPM, 6)
    k_g2p(const MpmK k, const float2* __restrict__ vel, float2* __restrict__ x, float2* __restrict__ v,
          float4* __restrict__ C, float4* __restrict__ F, float* __restrict__ J, const int32_t* __restrict__ mat,
          const int32_t* __restrict__ sid, uint32_t* status)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count_of(k)) { return; }
    const int m        = mat_of(k, MODE, mat, i);
    const bool track_f = (k.flags & GPE_MPM_FLAG_FLUID_F) != 0;
    const MpmScene sc  = scene_of<MS>(k, sid, i);
    PState ps;
    ps.x             = x[i];
    ps.F             = keeps_f(m, track_f) ? F[i] : make_float4(1.f, 0.f, 0.f, 1.f);
    ps.J             = keeps_j(m) ? J[i] : 1.f;
    const Stencil s  = stencil(k, sc, ps.x, status);
    const float2* nv = vel + (size_t)VS * (size_t)sc.goff;
    g2p_finish(k, sc, m, track_f, s,
               [&](int32_t nxi, int32_t nyj) {
                   return __ldg(&nv[(size_t)VS * ((size_t)nyj * (size_t)sc.nx + (size_t)nxi)]);
               },
               ps, status);
    x[i] = ps.x;
    v[i] = ps.v;
    C[i] = ps.C;
    if (keeps_f(m, track_f)) { F[i] = ps.F; }
    if (keeps_j(m)) { J[i] = ps.J; }
}

// ----- spatial sort of the particles (keeps P2G runs long and G2P gathers local) ---------------------------
__global__ void __launch_bounds__(T_MPM)
    k_mpm_key(const MpmK k, const float2* __restrict__ x, const int32_t* __restrict__ sid, uint2* __restrict__ keyrank,
              uint32_t* __restrict__ count, uint32_t* status)
{
    const int32_t i    = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid   = i < count_of(k);
    const int32_t lane = threadIdx.x & 31;
    uint32_t key       = 0xffffffffu;
    if (valid) {
        const MpmScene sc = scene_of(k, sid, i);
        const Stencil s   = stencil(k, sc, x[i], status);
        key               = sc.goff + (uint32_t)s.by * (uint32_t)sc.nx + (uint32_t)s.bx;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const int32_t leader = __ffs(peers) - 1;
    uint32_t base        = 0;
    if (valid && lane == leader) { base = atomicAdd(&count[key], (uint32_t)__popc(peers)); }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (valid) { keyrank[i] = make_uint2(key, base + (uint32_t)__popc(peers & ((1u << lane) - 1u))); }
}

// Moves particle i to slot start[key] + rank, with the rank its warp took from the key's counter in
// k_mpm_key. Within a base node the particles keep whatever order those atomics gave: P2G adds each node's
// terms in an order that float atomics leave open anyway, so the sort needs no stable placement (no bucket
// scatter and no search of the bucket for the particle's rank; the re-sort of 4M particles 0.145 ms with
// them). The keys, ranks and starts come from one histogram; the bounds checks only keep an inconsistent
// set from writing outside the arrays.
__global__ void __launch_bounds__(T_MPM)
    k_mpm_place(const int32_t* __restrict__ n_dev, uint32_t nn, const uint2* __restrict__ keyrank,
                const uint32_t* __restrict__ start, const float2* __restrict__ x0, const float2* __restrict__ v0,
                const float4* __restrict__ C0, const float4* __restrict__ F0, const float* __restrict__ J0,
                const int32_t* __restrict__ m0, const uint32_t* __restrict__ id0, float2* __restrict__ x1,
                float2* __restrict__ v1, float4* __restrict__ C1, float4* __restrict__ F1, float* __restrict__ J1,
                int32_t* __restrict__ m1, uint32_t* __restrict__ id1, const int32_t* __restrict__ sid0,
                int32_t* __restrict__ sid1)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t n = __ldg(n_dev);
    if (i >= n) { return; }
    const uint2 kr = keyrank[i];
    if (kr.x >= nn) { return; }
    const uint32_t d = __ldg(&start[kr.x]) + kr.y;
    if (d >= (uint32_t)n) { return; }
    x1[d]  = x0[i];
    v1[d]  = v0[i];
    C1[d]  = C0[i];
    F1[d]  = F0[i];
    J1[d]  = J0[i];
    m1[d]  = m0[i];
    id1[d] = id0[i];
    if (sid0) { sid1[d] = sid0[i]; }
}

// scene ids in the caller's order (ids_in[original index]) into storage order; ids out of range are reported
// (GPE_STATUS_CAPACITY) and stored as 0
__global__ void k_mpm_scene_ids(int32_t n, int32_t n_scenes, const uint32_t* __restrict__ id,
                                const int32_t* __restrict__ ids_in, int32_t* __restrict__ sid, uint32_t* status)
{
    const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) { return; }
    const uint32_t o = id[j];
    int32_t q        = (o < (uint32_t)n) ? ids_in[o] : -1;
    if (q < 0 || q >= n_scenes) {
        atomicOr(status, GPE_STATUS_CAPACITY);
        q = 0;
    }
    sid[j] = q;
}

// get_state helper: put particle i back at its original index id[i]
__global__ void k_mpm_unsort(int32_t n, const uint32_t* __restrict__ id, const float2* __restrict__ x0,
                             const float2* __restrict__ v0, const float4* __restrict__ C0,
                             const float4* __restrict__ F0, const float* __restrict__ J0, float2* __restrict__ x1,
                             float2* __restrict__ v1, float4* __restrict__ C1, float4* __restrict__ F1,
                             float* __restrict__ J1)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) { return; }
    const uint32_t d = id[i];
    x1[d]            = x0[i];
    v1[d]            = v0[i];
    C1[d]            = C0[i];
    F1[d]            = F0[i];
    J1[d]            = J0[i];
}

__global__ void k_mpm_init(int32_t n, uint32_t* __restrict__ id, float2* __restrict__ v, float4* __restrict__ C,
                           float4* __restrict__ F, float* __restrict__ J, int32_t* __restrict__ mat, int set_v,
                           int set_C, int set_F, int set_J, int set_m, int32_t material)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) { return; }
    id[i] = (uint32_t)i;
    if (set_v) { v[i] = make_float2(0.f, 0.f); }
    if (set_C) { C[i] = make_float4(0.f, 0.f, 0.f, 0.f); }
    if (set_F) { F[i] = make_float4(1.f, 0.f, 0.f, 1.f); }
    if (set_J) { J[i] = 1.f; }
    if (set_m) { mat[i] = material; }
}

__global__ void k_mpm_set_count(int32_t* __restrict__ c, int32_t n)
{
    c[0] = n;
    c[1] = n;
}

// hose emitter (MPMEmitterKernel, MPM.cu:380-438): appends at the device count with C = 0, F = I, J = 1
__global__ void k_mpm_emit(const HoseK h, float2* __restrict__ x, float2* __restrict__ v, float4* __restrict__ C,
                           float4* __restrict__ F, float* __restrict__ J, int32_t* __restrict__ mat,
                           uint32_t* __restrict__ id, int32_t material, int32_t* __restrict__ count, int32_t cap,
                           uint32_t* __restrict__ status)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= h.count) { return; }
    const float2 p     = hose_position(h, i);
    const int32_t slot = append_slot(count, true);
    if (slot < 0) { return; }
    if (slot >= cap) {
        atomicOr(status, GPE_STATUS_CAPACITY);
        atomicMin(count, cap);
        return;
    }
    x[slot]   = p;
    v[slot]   = make_float2(h.vx, h.vy);
    C[slot]   = make_float4(0.f, 0.f, 0.f, 0.f);
    F[slot]   = make_float4(1.f, 0.f, 0.f, 1.f);
    J[slot]   = 1.f;
    mat[slot] = material;
    id[slot]  = (uint32_t)slot;
}

// publish (MPMOutputKernel, MPM.cu:302-322): consecutive blocks of chunk_capacity particles, bounded by the view
__global__ void k_mpm_publish(const gpe_view vv, const gpe_view* __restrict__ vp, const float2* __restrict__ x,
                              const float2* __restrict__ v, int32_t* __restrict__ count)
{
    const gpe_view view  = vp ? *vp : vv; // vp: the struct lives in device memory and is read at run time
    const int32_t n      = count[0];
    if (blockIdx.x == 0 && threadIdx.x == 0) { count[1] = n; } // num_points[1] = num_points[0], MPM.cu:317
    const int32_t chunks = view.chunks_x * view.chunks_y;
    const int64_t limit  = (int64_t)chunks * view.chunk_capacity;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += stride) {
        if (i < chunks) {
            const int64_t left = (int64_t)n - i * view.chunk_capacity;
            view.counts[i]     = (int32_t)(left < 0 ? 0 : (left > view.chunk_capacity ? view.chunk_capacity : left));
        }
        if (i < n) {
            reinterpret_cast<float2*>(view.pos)[i] = x[i];
            reinterpret_cast<float2*>(view.vel)[i] = v[i];
        }
    }
}

} // namespace
} // namespace gpe

using namespace gpe;

struct MpmGraph {
    cudaGraphExec_t exec = nullptr;
    int ga_end;
    int cur_end;
    int32_t launches = 0; // kernel launches per step of the captured sequence (rounded up)
};

struct gpe_mpm {
    int device = 0;
    gpe_mpm_params prm{};
    MpmK k{};
    int64_t cap = 0, n = 0;
    int64_t nn  = 0; // nodes
    void* base  = nullptr;
    float2* x[2]    = {};
    float2* v[2]    = {};
    float4* C[2]    = {};
    float4* F[2]    = {};
    float* J[2]     = {};
    int32_t* mat[2] = {};
    uint32_t* id[2] = {};
    int32_t* sid[2] = {};          // scene of each particle (several scenes only)
    std::vector<MpmScene> scenes;  // several scenes: their grids, in the order of the node array
    MpmScene* d_scenes = nullptr;
    float4* grid[3] = {};
    float2* vel_n   = nullptr; // node velocities of the current step (k_grid_vel)
    uint2* keyrank  = nullptr;
    uint32_t* count  = nullptr;
    uint32_t* start  = nullptr;
    uint32_t* bsum   = nullptr;
    uint32_t* status = nullptr;
    int32_t* d_count = nullptr; // device-resident particle count
    bool dynamic     = false;   // GPE_MPM_FLAG_DYNAMIC_COUNT: launches cover the capacity
    int cur = 0;        // which particle buffer set is current
    int ga  = 0;        // grid holding the current step's nodes; ga+1, ga+2 (mod 3) are zero between steps
    bool grids_dirty = false;
    bool have_state  = false;
    int64_t steps_since_sort = 0;
    int32_t launches = 0;
    std::map<std::tuple<int, int, int, int>, MpmGraph> graphs;

    void drop_graphs()
    {
        for (auto& g : graphs) {
            if (g.second.exec) { cudaGraphExecDestroy(g.second.exec); }
        }
        graphs.clear();
    }
};

namespace {

int32_t mpm_validate(const gpe_mpm_params* p)
{
    if (!p || !(p->dx > 0.f) || p->nx < 3 || p->ny < 3 || !(p->dt > 0.f) || !(p->mass > 0.f) || p->bc_width < 0 ||
        p->material < 0 || p->material > GPE_MPM_MAT_SAND || (int64_t)p->nx * p->ny > ((int64_t)1 << 30)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "invalid MPM parameters");
        return GPE_ERR_BAD_ARG;
    }
    return GPE_OK;
}

MpmK mpm_make_k(const gpe_mpm_params& p)
{
    MpmK k{};
    k.dx        = p.dx;
    k.inv_dx    = 1.f / p.dx;
    k.goff      = p.grid_offset;
    k.dt        = p.dt;
    k.s0        = MpmScene{p.nx, p.ny, 0u, p.clamp_lo[0], p.clamp_lo[1], p.clamp_hi[0], p.clamp_hi[1]};
    k.n_scenes  = 1;
    k.nn        = (int64_t)p.nx * p.ny;
    k.gdt_x     = p.gravity[0] * p.dt;
    k.gdt_y     = p.gravity[1] * p.dt;
    k.mass      = p.mass;
    k.vol0      = p.vol0;
    k.bc_type   = p.bc_type;
    k.bc_width  = p.bc_width;
    k.material  = p.material;
    k.flags     = p.flags;
    k.k_bulk    = p.k_bulk;
    k.gamma     = p.gamma;
    k.p_min     = p.p_min;
    k.p_max     = p.p_max;
    k.J_min     = p.J_min;
    k.J_max     = p.J_max;
    k.mu0       = p.E / (2.f * (1.f + p.nu));
    k.la0       = p.E * p.nu / ((1.f + p.nu) * (1.f - 2.f * p.nu));
    k.theta_c   = p.theta_c;
    k.theta_s   = p.theta_s;
    k.hardening = p.hardening;
    const bool dflt = p.sand_h[0] == 0.f && p.sand_h[1] == 0.f && p.sand_h[2] == 0.f && p.sand_h[3] == 0.f;
    k.sh0       = dflt ? 35.f : p.sand_h[0]; // Klar et al. 2016
    k.sh1       = dflt ? 9.f : p.sand_h[1];
    k.sh2       = dflt ? 0.2f : p.sand_h[2];
    k.sh3       = dflt ? 10.f : p.sand_h[3];
    k.sand_cf   = (2.f * k.la0 + 2.f * k.mu0) / (2.f * k.mu0);
    k.apic_s    = 4.f * k.inv_dx * k.inv_dx;
    return k;
}

int mode_of(const gpe_mpm* s)
{
    return (s->prm.flags & GPE_MPM_FLAG_PER_PARTICLE_MATERIAL) ? MODE_MIXED : s->prm.material;
}

unsigned mblocks(int64_t n) { return (unsigned)((n + T_MPM - 1) / T_MPM); }

// launch size: the capacity when emitters grow the device-resident count inside replayed graphs
int64_t lsz(const gpe_mpm* s) { return s->dynamic ? s->cap : s->n; }

int32_t mpm_sync_count(gpe_mpm* s, cudaStream_t st)
{
    if (!s->dynamic) { return GPE_OK; }
    int32_t c = 0;
    GPE_TRY_CUDA(cudaMemcpyAsync(&c, s->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    s->n   = c;
    s->k.n = c;
    return GPE_OK;
}

unsigned grid_blocks(int64_t nn)
{
    const int64_t want = (nn + T_MPM - 1) / T_MPM;
    const int64_t cap  = (int64_t)gpe::sm_count() * 8;
    return (unsigned)(want < cap ? (want > 0 ? want : 1) : cap);
}

template <int MODE>
int32_t launch_p2g_t(gpe_mpm* s, float4* grid, cudaStream_t st)
{
    const int c = s->cur;
    if (s->scenes.size() > 1) {
        k_p2g<MODE, true><<<mblocks((lsz(s) + 1) / 2), T_MPM, 0, st>>>(s->k, s->x[c], s->v[c], s->C[c], s->F[c], s->J[c],
                                                            s->mat[c], s->sid[c], grid, s->status);
    } else {
        k_p2g<MODE, false><<<mblocks((lsz(s) + 1) / 2), T_MPM, 0, st>>>(s->k, s->x[c], s->v[c], s->C[c], s->F[c], s->J[c],
                                                             s->mat[c], nullptr, grid, s->status);
    }
    GPE_CHECK_LAUNCH("k_p2g");
    return GPE_OK;
}

int32_t launch_p2g(gpe_mpm* s, float4* grid, cudaStream_t st)
{
    if (lsz(s) == 0) { return GPE_OK; }
    s->launches += 1;
    switch (mode_of(s)) {
        case MODE_FLUID: return launch_p2g_t<MODE_FLUID>(s, grid, st);
        case MODE_COROT: return launch_p2g_t<MODE_COROT>(s, grid, st);
        case MODE_SNOW: return launch_p2g_t<MODE_SNOW>(s, grid, st);
        case MODE_NEOHOOKEAN: return launch_p2g_t<MODE_NEOHOOKEAN>(s, grid, st);
        case MODE_SAND: return launch_p2g_t<MODE_SAND>(s, grid, st);
        default: return launch_p2g_t<MODE_MIXED>(s, grid, st);
    }
}

// G2P from node velocities vel (stride VS float2 per node, see k_g2p)
template <int MODE, int VS>
int32_t launch_g2p_t(gpe_mpm* s, const float2* vel, cudaStream_t st)
{
    const int c = s->cur;
    if (s->scenes.size() > 1) {
        k_g2p<MODE, VS, true><<<mblocks(lsz(s)), T_MPM, 0, st>>>(s->k, vel, s->x[c], s->v[c], s->C[c], s->F[c],
                                                                s->J[c], s->mat[c], s->sid[c], s->status);
    } else {
        k_g2p<MODE, VS, false><<<mblocks(lsz(s)), T_MPM, 0, st>>>(s->k, vel, s->x[c], s->v[c], s->C[c], s->F[c],
                                                                 s->J[c], s->mat[c], nullptr, s->status);
    }
    GPE_CHECK_LAUNCH("k_g2p");
    return GPE_OK;
}

template <int VS>
int32_t launch_g2p(gpe_mpm* s, const float2* vel, cudaStream_t st)
{
    if (lsz(s) == 0) { return GPE_OK; }
    s->launches += 1;
    switch (mode_of(s)) {
        case MODE_FLUID: return launch_g2p_t<MODE_FLUID, VS>(s, vel, st);
        case MODE_COROT: return launch_g2p_t<MODE_COROT, VS>(s, vel, st);
        case MODE_SNOW: return launch_g2p_t<MODE_SNOW, VS>(s, vel, st);
        case MODE_NEOHOOKEAN: return launch_g2p_t<MODE_NEOHOOKEAN, VS>(s, vel, st);
        case MODE_SAND: return launch_g2p_t<MODE_SAND, VS>(s, vel, st);
        default: return launch_g2p_t<MODE_MIXED, VS>(s, vel, st);
    }
}

// node velocities of grid into s->vel_n, zeroing grid `zero` (or nothing) in the same pass
int32_t launch_grid_vel(gpe_mpm* s, const float4* grid, float4* zero, cudaStream_t st)
{
    if (s->scenes.size() > 1) {
        k_grid_vel<true><<<grid_blocks(s->nn), T_MPM, 0, st>>>(s->k, grid, s->vel_n, zero, s->nn);
    } else {
        k_grid_vel<false><<<grid_blocks(s->nn), T_MPM, 0, st>>>(s->k, grid, s->vel_n, zero, s->nn);
    }
    GPE_CHECK_LAUNCH("k_grid_vel");
    s->launches += 1;
    return GPE_OK;
}

int32_t mpm_sort(gpe_mpm* s, cudaStream_t st)
{
    if (lsz(s) <= 1) { return GPE_OK; }
    const int c = s->cur, o = c ^ 1;
    k_mpm_key<<<mblocks(lsz(s)), T_MPM, 0, st>>>(s->k, s->x[c], s->sid[c], s->keyrank, s->count, s->status);
    GPE_CHECK_LAUNCH("k_mpm_key");
    int32_t rc = launch_exclusive_scan(s->count, (uint32_t)s->nn, s->bsum, s->start, st);
    if (rc) { return rc; }
    k_mpm_place<<<mblocks(lsz(s)), T_MPM, 0, st>>>(s->d_count, (uint32_t)s->nn, s->keyrank, s->start, s->x[c],
                                                  s->v[c], s->C[c], s->F[c], s->J[c], s->mat[c], s->id[c], s->x[o],
                                                  s->v[o], s->C[o], s->F[o], s->J[o], s->mat[o], s->id[o],
                                                  s->sid[c], s->sid[o]);
    GPE_CHECK_LAUNCH("k_mpm_place");
    s->cur ^= 1;
    s->launches += 2 + scan_launches((uint32_t)s->nn); // key, scan, placement
    return GPE_OK;
}

// n_steps steps: [sort], P2G, (n-1) x (node velocities, G2P, P2G), node velocities, G2P. Grids ga+1 and ga+2
// are zero on entry and exit.
int32_t mpm_run(gpe_mpm* s, int32_t n_steps, bool do_sort, cudaStream_t st)
{
    int32_t rc = GPE_OK;
    if (do_sort) { rc = mpm_sort(s, st); }
    if (rc) { return rc; }
    int a = (s->ga + 1) % 3;
    rc    = launch_p2g(s, s->grid[a], st);
    for (int32_t t = 1; t < n_steps && rc == GPE_OK; ++t) {
        const int b = (a + 1) % 3, z = (a + 2) % 3;
        if (lsz(s) > 0) {
            // node velocities of this step (zeroing the grid read two steps ago), its G2P, and the P2G of the
            // next step into the zero grid b
            rc = launch_grid_vel(s, s->grid[a], s->grid[z], st);
            if (rc == GPE_OK) { rc = launch_g2p<1>(s, s->vel_n, st); }
            if (rc == GPE_OK) { rc = launch_p2g(s, s->grid[b], st); }
        } else {
            k_clear<<<grid_blocks(s->nn), T_MPM, 0, st>>>(s->grid[z], s->nn);
            GPE_CHECK_LAUNCH("k_clear");
        }
        a = b;
    }
    if (rc) { return rc; }
    // last G2P; zero the grid that was used before this one so two zero grids follow `a`
    rc = launch_grid_vel(s, s->grid[a], s->grid[(a + 2) % 3], st);
    if (rc == GPE_OK) { rc = launch_g2p<1>(s, s->vel_n, st); }
    s->ga = a;
    return rc;
}

// the engine's buffers and scene table in the kernel constants
void bind_scenes(gpe_mpm* s)
{
    s->k.n_dev = s->d_count;
    if (s->scenes.size() > 1) {
        s->k.scenes   = s->d_scenes;
        s->k.n_scenes = (int32_t)s->scenes.size();
        s->k.s0       = s->scenes[0];
        s->k.nn       = s->nn;
    }
}

int32_t mpm_alloc(gpe_mpm* s)
{
    const size_t N = (size_t)s->cap;
    const size_t M = (size_t)s->nn;
    Carver c;
    size_t ox[2], ov[2], oC[2], oF[2], oJ[2], om[2], oid[2], og[3];
    for (int b = 0; b < 2; ++b) {
        ox[b]  = c.take<float2>(N);
        ov[b]  = c.take<float2>(N);
        oC[b]  = c.take<float4>(N);
        oF[b]  = c.take<float4>(N);
        oJ[b]  = c.take<float>(N);
        om[b]  = c.take<int32_t>(N);
        oid[b] = c.take<uint32_t>(N);
    }
    for (int b = 0; b < 3; ++b) { og[b] = c.take<float4>(M); }
    const size_t ovn = c.take<float2>(M);
    const size_t okr = c.take<uint2>(N);
    const size_t ocn = c.take<uint32_t>(M);
    const size_t ost = c.take<uint32_t>(M + 1);
    const size_t obs = c.take<uint32_t>(scan_blocks((uint32_t)M) + 1);
    const size_t oss = c.take<uint32_t>(4);
    const size_t ocnt = c.take<int32_t>(2);
    const bool several = s->scenes.size() > 1;
    size_t osid[2] = {0, 0}, osc = 0;
    if (several) {
        osid[0] = c.take<int32_t>(N);
        osid[1] = c.take<int32_t>(N);
        osc     = c.take<MpmScene>(s->scenes.size());
    }
    GPE_TRY_CUDA(cudaMalloc(&s->base, c.off));
    GPE_TRY_CUDA(cudaMemset(s->base, 0, c.off));
    uint8_t* b = static_cast<uint8_t*>(s->base);
    for (int q = 0; q < 2; ++q) {
        s->x[q]   = reinterpret_cast<float2*>(b + ox[q]);
        s->v[q]   = reinterpret_cast<float2*>(b + ov[q]);
        s->C[q]   = reinterpret_cast<float4*>(b + oC[q]);
        s->F[q]   = reinterpret_cast<float4*>(b + oF[q]);
        s->J[q]   = reinterpret_cast<float*>(b + oJ[q]);
        s->mat[q] = reinterpret_cast<int32_t*>(b + om[q]);
        s->id[q]  = reinterpret_cast<uint32_t*>(b + oid[q]);
    }
    for (int q = 0; q < 3; ++q) { s->grid[q] = reinterpret_cast<float4*>(b + og[q]); }
    s->vel_n   = reinterpret_cast<float2*>(b + ovn);
    s->keyrank = reinterpret_cast<uint2*>(b + okr);
    s->count   = reinterpret_cast<uint32_t*>(b + ocn);
    s->start   = reinterpret_cast<uint32_t*>(b + ost);
    s->bsum    = reinterpret_cast<uint32_t*>(b + obs);
    s->status  = reinterpret_cast<uint32_t*>(b + oss);
    s->d_count = reinterpret_cast<int32_t*>(b + ocnt);
    if (several) {
        s->sid[0]   = reinterpret_cast<int32_t*>(b + osid[0]);
        s->sid[1]   = reinterpret_cast<int32_t*>(b + osid[1]);
        s->d_scenes = reinterpret_cast<MpmScene*>(b + osc);
        GPE_TRY_CUDA(cudaMemcpy(s->d_scenes, s->scenes.data(), sizeof(MpmScene) * s->scenes.size(),
                                cudaMemcpyHostToDevice));
    }
    bind_scenes(s);
    return GPE_OK;
}

cudaMemcpyKind mk_in(int32_t mem) { return mem == GPE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }
cudaMemcpyKind mk_out(int32_t mem) { return mem == GPE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost; }

} // namespace

extern "C" {

int32_t gpe_mpm_create(const gpe_mpm_params* params, int64_t capacity, gpe_mpm** out)
{
    return gpe_mpm_create_scenes(params, nullptr, 0, capacity, out);
}

int32_t gpe_mpm_create_scenes(const gpe_mpm_params* params, const gpe_mpm_scene* scenes, int32_t n_scenes,
                              int64_t capacity, gpe_mpm** out)
{
    gpe::clear_error();
    if (!out || capacity < 0 || capacity > (int64_t)INT32_MAX / 2 || n_scenes < 0 || (n_scenes > 0 && !scenes)) {
        return GPE_ERR_BAD_ARG;
    }
    *out = nullptr;
    // several scenes: their grids one after the other; the first scene's size stands in for params' grid
    std::vector<MpmScene> table;
    gpe_mpm_params prm = params ? *params : gpe_mpm_params{};
    int64_t nodes      = 0;
    for (int32_t q = 0; q < n_scenes; ++q) {
        const gpe_mpm_scene& sc = scenes[q];
        if (sc.nx < 3 || sc.ny < 3) {
            gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_create_scenes: scene %d needs at least 3 x 3 nodes", q);
            return GPE_ERR_BAD_ARG;
        }
        table.push_back(MpmScene{sc.nx, sc.ny, (uint32_t)nodes, sc.clamp_lo[0], sc.clamp_lo[1], sc.clamp_hi[0],
                                 sc.clamp_hi[1]});
        nodes += (int64_t)sc.nx * sc.ny;
        if (nodes > ((int64_t)1 << 30)) {
            gpe::set_error(GPE_ERR_CAPACITY, "gpe_mpm_create_scenes: more than 2^30 nodes");
            return GPE_ERR_CAPACITY;
        }
    }
    if (n_scenes > 0) {
        prm.nx           = scenes[0].nx;
        prm.ny           = scenes[0].ny;
        prm.clamp_lo[0]  = scenes[0].clamp_lo[0];
        prm.clamp_lo[1]  = scenes[0].clamp_lo[1];
        prm.clamp_hi[0]  = scenes[0].clamp_hi[0];
        prm.clamp_hi[1]  = scenes[0].clamp_hi[1];
    }
    int32_t rc = mpm_validate(params ? &prm : nullptr);
    if (rc) { return rc; }
    int dev = 0;
    rc      = gpe::current_device(&dev);
    if (rc) { return rc; }
    gpe_mpm* s = new gpe_mpm();
    s->device  = dev;
    s->prm     = prm;
    s->k       = mpm_make_k(prm);
    s->dynamic = (prm.flags & GPE_MPM_FLAG_DYNAMIC_COUNT) != 0;
    s->cap     = capacity;
    s->nn      = n_scenes > 0 ? nodes : (int64_t)prm.nx * prm.ny;
    if (n_scenes > 1) { s->scenes = std::move(table); }
    rc         = mpm_alloc(s);
    if (rc) {
        if (s->base) { cudaFree(s->base); }
        delete s;
        return rc;
    }
    *out = s;
    return GPE_OK;
}

int32_t gpe_mpm_destroy(gpe_mpm* s)
{
    if (!s) { return GPE_ERR_BAD_ARG; }
    s->drop_graphs();
    if (s->base) { cudaFree(s->base); }
    delete s;
    return GPE_OK;
}

int32_t gpe_mpm_set_params(gpe_mpm* s, const gpe_mpm_params* params)
{
    gpe::clear_error();
    if (!s) { return GPE_ERR_BAD_ARG; }
    int32_t rc = mpm_validate(params);
    if (rc) { return rc; }
    if (s->scenes.size() <= 1 && (params->nx != s->prm.nx || params->ny != s->prm.ny)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_set_params: the node grid is fixed at creation");
        return GPE_ERR_BAD_ARG;
    }
    s->prm        = *params;
    const int32_t n = s->k.n;
    s->k          = mpm_make_k(*params);
    s->k.n        = n;
    bind_scenes(s);
    s->dynamic    = (params->flags & GPE_MPM_FLAG_DYNAMIC_COUNT) != 0;
    s->drop_graphs();
    return GPE_OK;
}

int32_t gpe_mpm_set_state(gpe_mpm* s, const float* pos, const float* vel, const float* C, const float* F,
                          const float* J, const int32_t* material, int64_t n, int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!s || n < 0 || (n > 0 && !pos) || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_set_state: bad arguments");
        return GPE_ERR_BAD_ARG;
    }
    if (n > s->cap) {
        gpe::set_error(GPE_ERR_CAPACITY, "gpe_mpm_set_state: %lld particles exceed capacity %lld", (long long)n,
                       (long long)s->cap);
        return GPE_ERR_CAPACITY;
    }
    if (mem == GPE_MEM_HOST && material) {
        for (int64_t i = 0; i < n; ++i) {
            if (material[i] < 0 || material[i] > GPE_MPM_MAT_SAND) {
                gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_set_state: material ids must be in [0, 4]");
                return GPE_ERR_BAD_ARG;
            }
        }
    }
    cudaStream_t st = as_stream(stream);
    s->cur          = 0;
    if (n > 0) {
        GPE_TRY_CUDA(cudaMemcpyAsync(s->x[0], pos, sizeof(float2) * (size_t)n, mk_in(mem), st));
        if (vel) { GPE_TRY_CUDA(cudaMemcpyAsync(s->v[0], vel, sizeof(float2) * (size_t)n, mk_in(mem), st)); }
        if (C) { GPE_TRY_CUDA(cudaMemcpyAsync(s->C[0], C, sizeof(float4) * (size_t)n, mk_in(mem), st)); }
        if (F) { GPE_TRY_CUDA(cudaMemcpyAsync(s->F[0], F, sizeof(float4) * (size_t)n, mk_in(mem), st)); }
        if (J) { GPE_TRY_CUDA(cudaMemcpyAsync(s->J[0], J, sizeof(float) * (size_t)n, mk_in(mem), st)); }
        if (material) {
            GPE_TRY_CUDA(cudaMemcpyAsync(s->mat[0], material, sizeof(int32_t) * (size_t)n, mk_in(mem), st));
        }
        k_mpm_init<<<mblocks(n), T_MPM, 0, st>>>((int32_t)n, s->id[0], s->v[0], s->C[0], s->F[0], s->J[0], s->mat[0],
                                                  !vel, !C, !F, !J, !material, s->prm.material);
        GPE_CHECK_LAUNCH("k_mpm_init");
        // several scenes: every particle in scene 0 until gpe_mpm_set_scene_ids says otherwise
        if (s->sid[0]) { GPE_TRY_CUDA(cudaMemsetAsync(s->sid[0], 0, sizeof(int32_t) * (size_t)n, st)); }
    }
    k_mpm_set_count<<<1, 1, 0, st>>>(s->d_count, (int32_t)n);
    GPE_CHECK_LAUNCH("k_mpm_set_count");
    if (s->n != n && !s->dynamic) { s->drop_graphs(); }
    s->n                = n;
    s->k.n              = (int32_t)n;
    s->have_state       = true;
    s->grids_dirty      = true;
    // a new state is in the caller's order: the next step sorts it by stencil base node first
    s->steps_since_sort = s->prm.sort_interval;
    if (mem == GPE_MEM_HOST) { GPE_TRY_CUDA(cudaStreamSynchronize(st)); }
    return GPE_OK;
}

int32_t gpe_mpm_get_state(gpe_mpm* s, float* pos, float* vel, float* C, float* F, float* J, int64_t n, int32_t mem,
                          void* stream)
{
    gpe::clear_error();
    if (!s) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    const int32_t rc = mpm_sync_count(s, st);
    if (rc) { return rc; }
    if (n != s->n || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_get_state: n must equal the particle count");
        return GPE_ERR_BAD_ARG;
    }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    if (n > 0) {
        // particles are returned at their original indices
        const int c = s->cur, o = c ^ 1;
        k_mpm_unsort<<<mblocks(n), T_MPM, 0, st>>>((int32_t)n, s->id[c], s->x[c], s->v[c], s->C[c], s->F[c], s->J[c],
                                                   s->x[o], s->v[o], s->C[o], s->F[o], s->J[o]);
        GPE_CHECK_LAUNCH("k_mpm_unsort");
        if (pos) { GPE_TRY_CUDA(cudaMemcpyAsync(pos, s->x[o], sizeof(float2) * (size_t)n, mk_out(mem), st)); }
        if (vel) { GPE_TRY_CUDA(cudaMemcpyAsync(vel, s->v[o], sizeof(float2) * (size_t)n, mk_out(mem), st)); }
        if (C) { GPE_TRY_CUDA(cudaMemcpyAsync(C, s->C[o], sizeof(float4) * (size_t)n, mk_out(mem), st)); }
        if (F) { GPE_TRY_CUDA(cudaMemcpyAsync(F, s->F[o], sizeof(float4) * (size_t)n, mk_out(mem), st)); }
        if (J) { GPE_TRY_CUDA(cudaMemcpyAsync(J, s->J[o], sizeof(float) * (size_t)n, mk_out(mem), st)); }
    }
    if (mem == GPE_MEM_HOST) { GPE_TRY_CUDA(cudaStreamSynchronize(st)); }
    return GPE_OK;
}

int32_t gpe_mpm_set_scene_ids(gpe_mpm* s, const int32_t* scene_id, int64_t n, int32_t mem, void* stream)
{
    gpe::clear_error();
    if (!s || (n > 0 && !scene_id) || (mem != GPE_MEM_HOST && mem != GPE_MEM_DEVICE)) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    int32_t rc      = mpm_sync_count(s, st);
    if (rc) { return rc; }
    if (!s->have_state || n != s->n) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_set_scene_ids: n must equal the particle count");
        return GPE_ERR_BAD_ARG;
    }
    const int32_t ns = s->scenes.empty() ? 1 : (int32_t)s->scenes.size();
    if (mem == GPE_MEM_HOST) {
        for (int64_t i = 0; i < n; ++i) {
            if (scene_id[i] < 0 || scene_id[i] >= ns) {
                gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_set_scene_ids: ids must be in [0, %d)", ns);
                return GPE_ERR_BAD_ARG;
            }
        }
    }
    if (ns == 1 || n == 0) { return GPE_OK; } // one scene: every particle is in it
    // the caller's ids go through the other storage set, then into storage order
    const int c = s->cur, o = c ^ 1;
    GPE_TRY_CUDA(cudaMemcpyAsync(s->sid[o], scene_id, sizeof(int32_t) * (size_t)n, mk_in(mem), st));
    uint32_t* flag = s->status + 1; // a word of its own, so the engine's status bits stay as they are
    GPE_TRY_CUDA(cudaMemsetAsync(flag, 0, sizeof(uint32_t), st));
    k_mpm_scene_ids<<<mblocks(n), T_MPM, 0, st>>>((int32_t)n, ns, s->id[c], s->sid[o], s->sid[c], flag);
    GPE_CHECK_LAUNCH("k_mpm_scene_ids");
    uint32_t bad = 0;
    GPE_TRY_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    if (bad) {
        gpe::set_error(GPE_ERR_BAD_ARG, "gpe_mpm_set_scene_ids: ids must be in [0, %d)", ns);
        return GPE_ERR_BAD_ARG;
    }
    s->steps_since_sort = s->prm.sort_interval; // the particles' keys changed: sort again first
    return GPE_OK;
}

int32_t gpe_mpm_count(const gpe_mpm* s, int64_t* n)
{
    if (!s || !n) { return GPE_ERR_BAD_ARG; }
    // with a device-resident count the host copy is refreshed first (a cached value, hence the cast)
    const int32_t rc = mpm_sync_count(const_cast<gpe_mpm*>(s), nullptr);
    if (rc) { return rc; }
    *n = s->n;
    return GPE_OK;
}

int32_t gpe_mpm_step(gpe_mpm* s, int32_t n_steps, void* stream)
{
    gpe::clear_error();
    if (!s || n_steps < 0) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    if (n_steps == 0) { return GPE_OK; }
    cudaStream_t st = as_stream(stream);
    if (s->grids_dirty) {
        for (int q = 0; q < 3; ++q) { GPE_TRY_CUDA(cudaMemsetAsync(s->grid[q], 0, sizeof(float4) * (size_t)s->nn, st)); }
        s->grids_dirty = false;
    }
    const bool do_sort = s->prm.sort_interval > 0 && s->steps_since_sort >= s->prm.sort_interval;
    const auto key     = std::make_tuple(n_steps, s->ga, s->cur, (int)do_sort);
    auto it            = s->graphs.find(key);
    if (it == s->graphs.end()) {
        cudaStream_t cap_st = st;
        bool own            = false;
        if (cap_st == nullptr) {
            GPE_TRY_CUDA(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
            own = true;
        }
        const int ga0 = s->ga, cur0 = s->cur;
        GPE_TRY_CUDA(cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
        s->launches = 0;
        int32_t rc  = mpm_run(s, n_steps, do_sort, cap_st);
        cudaGraph_t graph    = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cap_st, &graph);
        MpmGraph g;
        g.launches = (s->launches + n_steps - 1) / n_steps;
        g.ga_end  = s->ga;
        g.cur_end = s->cur;
        s->ga     = ga0;
        s->cur    = cur0;
        if (rc == GPE_OK && ce != cudaSuccess) {
            gpe::set_cuda_error(ce, "cudaStreamEndCapture");
            rc = GPE_ERR_CUDA;
        }
        if (rc == GPE_OK) {
            const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
            if (ie != cudaSuccess) {
                gpe::set_cuda_error(ie, "cudaGraphInstantiate");
                rc = GPE_ERR_CUDA;
            }
        }
        if (graph) { cudaGraphDestroy(graph); }
        if (own) { cudaStreamDestroy(cap_st); }
        if (rc) { return rc; }
        it = s->graphs.emplace(key, g).first;
    }
    GPE_TRY_CUDA(cudaGraphLaunch(it->second.exec, st));
    s->ga       = it->second.ga_end;
    s->cur      = it->second.cur_end;
    s->launches = it->second.launches;
    s->steps_since_sort = do_sort ? n_steps : s->steps_since_sort + n_steps;
    return GPE_OK;
}

int32_t gpe_mpm_stage(gpe_mpm* s, int32_t stage, void* stream)
{
    gpe::clear_error();
    if (!s) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    cudaStream_t st = as_stream(stream);
    float4* g       = s->grid[s->ga];
    s->grids_dirty  = true;
    switch (stage) {
        case GPE_MPM_STAGE_CLEAR:
            k_clear<<<grid_blocks(s->nn), T_MPM, 0, st>>>(g, s->nn);
            GPE_CHECK_LAUNCH("k_clear");
            return GPE_OK;
        case GPE_MPM_STAGE_P2G: return launch_p2g(s, g, st);
        case GPE_MPM_STAGE_GRID:
            k_grid<<<grid_blocks(s->nn), T_MPM, 0, st>>>(s->k, g);
            GPE_CHECK_LAUNCH("k_grid");
            return GPE_OK;
        case GPE_MPM_STAGE_G2P: return launch_g2p<2>(s, reinterpret_cast<const float2*>(g), st);
        case GPE_MPM_STAGE_SORT: return mpm_sort(s, st);
        default: return GPE_ERR_BAD_ARG;
    }
}

int32_t gpe_mpm_get_grid(gpe_mpm* s, float* dst, int64_t n_nodes, int32_t mem, void* stream)
{
    if (!s || !dst || n_nodes != s->nn) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    GPE_TRY_CUDA(cudaMemcpyAsync(dst, s->grid[s->ga], sizeof(float4) * (size_t)s->nn, mk_out(mem), st));
    if (mem == GPE_MEM_HOST) { GPE_TRY_CUDA(cudaStreamSynchronize(st)); }
    return GPE_OK;
}

int32_t gpe_mpm_p2g_wide_warps(gpe_mpm* s, uint32_t* count, void* stream)
{
    if (!s || !count) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    GPE_TRY_CUDA(cudaMemcpyAsync(count, s->status + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaMemsetAsync(s->status + 2, 0, sizeof(uint32_t), st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    return GPE_OK;
}

int32_t gpe_mpm_status(gpe_mpm* s, uint32_t* status, void* stream)
{
    if (!s || !status) { return GPE_ERR_BAD_ARG; }
    cudaStream_t st = as_stream(stream);
    GPE_TRY_CUDA(cudaMemcpyAsync(status, s->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GPE_TRY_CUDA(cudaMemsetAsync(s->status, 0, sizeof(uint32_t), st));
    GPE_TRY_CUDA(cudaStreamSynchronize(st));
    return GPE_OK;
}

int32_t gpe_mpm_launches_per_step(const gpe_mpm* s, int32_t* launches)
{
    if (!s || !launches) { return GPE_ERR_BAD_ARG; }
    *launches = s->launches; // of the last gpe_mpm_step, per step
    return GPE_OK;
}

int32_t gpe_mpm_emit(gpe_mpm* s, const gpe_hose* hose, uint64_t seed, int32_t* requested, void* stream)
{
    gpe::clear_error();
    if (!s || !hose || !(hose->spacing > 0.f) || hose->steps_per_call < 0) { return GPE_ERR_BAD_ARG; }
    if (!s->dynamic) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_mpm_emit: needs GPE_MPM_FLAG_DYNAMIC_COUNT");
        return GPE_ERR_NOT_READY;
    }
    if (s->scenes.size() > 1) {
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_mpm_emit: an engine of one scene only");
        return GPE_ERR_NOT_READY;
    }
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
        const int c = s->cur;
        k_mpm_emit<<<mblocks(cnt), T_MPM, 0, st>>>(h, s->x[c], s->v[c], s->C[c], s->F[c], s->J[c], s->mat[c], s->id[c],
                                                    s->prm.material, s->d_count, (int32_t)s->cap, s->status);
        GPE_CHECK_LAUNCH("k_mpm_emit");
    }
    s->have_state = true;
    return GPE_OK;
}

int32_t gpe_mpm_publish(gpe_mpm* s, const gpe_view* view, int32_t view_mem, void* stream)
{
    gpe::clear_error();
    if (!s || !view || (view_mem != GPE_MEM_HOST && view_mem != GPE_MEM_DEVICE)) { return GPE_ERR_BAD_ARG; }
    if (view_mem == GPE_MEM_HOST && (!view->pos || !view->vel || !view->counts || view->chunks_x <= 0 ||
                                     view->chunks_y <= 0 || view->chunk_capacity <= 0)) {
        return GPE_ERR_BAD_ARG;
    }
    if (s->prm.sort_interval > 0) {
        // publish order is the storage order; re-sorting would shuffle it between ticks
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_mpm_publish: needs sort_interval == 0");
        return GPE_ERR_NOT_READY;
    }
    if (s->scenes.size() > 1) { // positions are scene-local: a chunk view covers one scene
        gpe::set_error(GPE_ERR_NOT_READY, "gpe_mpm_publish: an engine of one scene only");
        return GPE_ERR_NOT_READY;
    }
    cudaStream_t st = as_stream(stream);
    gpe_view vv{};
    const gpe_view* vp = nullptr;
    unsigned blocks    = (unsigned)gpe::sm_count() * 8;
    if (view_mem == GPE_MEM_HOST) {
        vv     = *view;
        blocks = grid_blocks((int64_t)vv.chunks_x * vv.chunks_y * vv.chunk_capacity);
    } else {
        vp = view;
    }
    k_mpm_publish<<<blocks, T_MPM, 0, st>>>(vv, vp, s->x[s->cur], s->v[s->cur], s->d_count);
    GPE_CHECK_LAUNCH("k_mpm_publish");
    return GPE_OK;
}

int32_t gpe_mpm_buffers(gpe_mpm* s, float** pos, float** vel, float** C, float** F, float** J, int32_t** count)
{
    if (!s) { return GPE_ERR_BAD_ARG; }
    const int c = s->cur;
    if (pos) { *pos = reinterpret_cast<float*>(s->x[c]); }
    if (vel) { *vel = reinterpret_cast<float*>(s->v[c]); }
    if (C) { *C = reinterpret_cast<float*>(s->C[c]); }
    if (F) { *F = reinterpret_cast<float*>(s->F[c]); }
    if (J) { *J = s->J[c]; }
    if (count) { *count = s->d_count; }
    return GPE_OK;
}

int32_t gpe_mpm_enqueue(gpe_mpm* s, int32_t n_steps, void* stream)
{
    gpe::clear_error();
    if (!s || n_steps < 0) { return GPE_ERR_BAD_ARG; }
    if (!s->have_state) { return GPE_ERR_NOT_READY; }
    cudaStream_t st = as_stream(stream);
    if (n_steps == 0) { return GPE_OK; }
    // the recorded sequence starts from cleared grids and grid 0, whatever the previous sequence left
    for (int q = 0; q < 3; ++q) { GPE_TRY_CUDA(cudaMemsetAsync(s->grid[q], 0, sizeof(float4) * (size_t)s->nn, st)); }
    s->ga          = 2; // mpm_run scatters the first step into grid (ga + 1) % 3 == 0
    s->grids_dirty = false;
    const int32_t rc = mpm_run(s, n_steps, false, st);
    s->ga            = 2;
    s->grids_dirty   = true; // the next engine-owned step clears the grids again
    return rc;
}

} // extern "C"
