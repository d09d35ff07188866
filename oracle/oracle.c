/*
 * oracle.c — CPU restatement of the reference's PBF and MLS-MPM solver steps (test infrastructure only; the
 * engine never links or calls this file). Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC.
 *
 * PBF follows libs/cuda-engine/source/PBF.cu:
 *   predict + cell key + counting sort  PBF.cu:786-833 (prepNextSubstepKernel), sort made stable here
 *   lambda                              PBF.cu:243-294 (lambdaKernel), pairDirection PBF.cu:309-321,
 *                                       poly6 PBF.cu:322-326, spiky PBF.cu:327-336
 *   delta p + s_corr + omega            PBF.cu:395-438 (posCorrectionKernel), walls PBF.cu:471-499
 *   velocity + XSPH + velocity clamp    PBF.cu:500-553, 554-628, 629-638
 * with the constants of libs/common/include/common/constants.h:34-55 passed in as gpe_pbf_params. The world
 * is one global uniform grid per scene: the reference's 16x16-cell chunks with 1-cell halos cover the same
 * neighbour set (PBF-internal.cuh:178-212), so chunking is not restated. Vorticity confinement is absent
 * from the reference and follows Macklin & Mueller 2013, eq. 15-16.
 *
 * MLS-MPM follows libs/cuda-engine/source/MPM.cu:
 *   P2G with the J-based EOS            MPM.cu:62-129 (P2GKernel, particleToGrid), gridCoord MPM.cu:84
 *   grid update                         MPM.cu:131-177 (gridKernel)
 *   G2P, F and J update, handleOOB      MPM.cu:196-301 (gridToParticle, handleOOB); matMul2D/det2D
 *                                       cuda-internal.cuh:44-56
 * The fixed-corotated and snow models (absent in the reference) follow Stomakhin et al. 2012/2013 and the
 * MLS-MPM formulation of Hu et al. 2018; the Neo-Hookean model is the compressible form of Bonet & Wood
 * (tau = mu (F F^T - I) + la ln J I); sand follows the Drucker-Prager elastoplasticity of Klar et al. 2016
 * (Hencky-strain St. Venant-Kirchhoff stress, return mapping onto the friction cone, friction-angle
 * hardening with the accumulated plastic strain q, kept as J = 1 + q).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int32_t orc_num_threads(void)
{
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}

/* ===================================================================================================== */
/* PBF                                                                                                    */
/* ===================================================================================================== */

typedef struct {
    int64_t coff;           /* first global cell of the scene */
    int32_t ncx, ncy;       /* cells                          */
    float ox, oy;           /* origin                          */
    float lox, loy, hix, hiy; /* wall clamp box                */
} dinfo;

static float cell_size(const gpe_pbf_params* p) { return p->cell > 0.f ? p->cell : p->h; }

static int32_t scan_radius(const gpe_pbf_params* p)
{
    const int32_t r = (int32_t)ceilf(p->h / cell_size(p) - 1e-4f);
    return r < 1 ? 1 : r;
}

static int32_t cells_along(float extent, float cell)
{
    const int32_t c = (int32_t)ceilf(extent / cell);
    return c < 1 ? 1 : c;
}

static void build_dinfo(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, dinfo* out)
{
    const float c = cell_size(p);
    int64_t off = 0;
    for (int32_t d = 0; d < nd; ++d) {
        out[d].coff = off;
        out[d].ncx  = cells_along(doms[d].extent[0], c);
        out[d].ncy  = cells_along(doms[d].extent[1], c);
        out[d].ox   = doms[d].origin[0];
        out[d].oy   = doms[d].origin[1];
        out[d].lox  = doms[d].origin[0];
        out[d].loy  = doms[d].origin[1];
        out[d].hix  = (doms[d].origin[0] + doms[d].extent[0]) - p->wall_margin;
        out[d].hiy  = (doms[d].origin[1] + doms[d].extent[1]) - p->wall_margin;
        off += (int64_t)out[d].ncx * out[d].ncy;
    }
}

int64_t orc_pbf_num_cells(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd)
{
    const float c = cell_size(p);
    int64_t off = 0;
    for (int32_t d = 0; d < nd; ++d) {
        off += (int64_t)cells_along(doms[d].extent[0], c) * cells_along(doms[d].extent[1], c);
    }
    return off;
}

/* Cell coordinate of a position, FP32 with the device's operation order: (pos - origin) rounded, then
 * times 1/cell rounded, truncated and clamped to the grid (PBF.cu:792-793 clamps floorf(x)/kCellDim). */
static int32_t cell_coord(float pos, float org, float inv_cell, int32_t nc)
{
    const volatile float t = pos - org;
    const volatile float u = t * inv_cell;
    if (!(u >= 0.f)) { return 0; }
    if (u >= (float)nc) { return nc - 1; }
    return (int32_t)u;
}

static int32_t dom_of(const int32_t* dom, int64_t i) { return dom ? dom[i] : 0; }

/* Integer mixer of the reference (hash, cuda-internal.cuh:19-27); the same constants are required for the
 * pair directions to agree. */
static uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

/* pairDirection, PBF.cu:309-321: a pseudo-random unit vector for a coincident pair (a, b) */
static void pair_direction(int64_t a, int64_t b, double* dx, double* dy)
{
    const uint32_t lo  = (uint32_t)(a < b ? a : b);
    const uint32_t hi  = (uint32_t)(a < b ? b : a);
    const float ang    = (float)(mix32(lo * 0x9E3779B9u ^ hi) & 0xFFFFu) * (6.2831853f / 65536.f);
    const double sign  = (a < b) ? 1.0 : -1.0;
    *dx                = sign * cos((double)ang);
    *dy                = sign * sin((double)ang);
}

typedef struct {
    double h, h2, c6, cs, inv_w_dq;
    float inv_cell;
    int32_t R;
} kconst;

static kconst make_kconst(const gpe_pbf_params* p)
{
    kconst k;
    const double h = p->h;
    k.h            = h;
    k.h2           = (double)(p->h * p->h);
    k.c6           = p->poly6_coeff > 0.f ? (double)p->poly6_coeff : 4.0 / (M_PI * pow(h, 8));
    k.cs           = p->spiky_coeff > 0.f ? (double)p->spiky_coeff : 30.0 / (M_PI * pow(h, 5));
    const double d = k.h2 - (double)p->scorr_dq * (double)p->scorr_dq;
    k.inv_w_dq     = 1.0 / (k.c6 * d * d * d);
    k.inv_cell     = 1.0f / cell_size(p);
    k.R            = scan_radius(p);
    return k;
}

/* Neighbour ranges of a particle: rows of cells around its base cell (the reference scans the 3x3 cells
 * around clamp(floorf(x)/kCellDim), PBF.cu:252-263; a row of cells is one contiguous range after the
 * row-major sort). Returns the number of rows written. */
static int32_t scan_rows(const dinfo* di, const kconst* k, const uint32_t* cs, float px, float py, int64_t* beg,
                         int64_t* end)
{
    const int32_t bx = cell_coord(px, di->ox, k->inv_cell, di->ncx);
    const int32_t by = cell_coord(py, di->oy, k->inv_cell, di->ncy);
    const int32_t x0 = bx - k->R < 0 ? 0 : bx - k->R;
    const int32_t x1 = bx + k->R > di->ncx - 1 ? di->ncx - 1 : bx + k->R;
    int32_t nr       = 0;
    for (int32_t y = by - k->R; y <= by + k->R; ++y) {
        if (y < 0 || y >= di->ncy) { continue; }
        const int64_t row = di->coff + (int64_t)y * di->ncx;
        beg[nr]           = cs[row + x0];
        end[nr]           = cs[row + x1 + 1];
        ++nr;
    }
    return nr;
}

void orc_pbf_predict_sort(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n,
                          const float* x, const float* v, const int32_t* dom, uint32_t* key, uint32_t* perm,
                          uint32_t* cell_start, float* x_sorted, float* xs_sorted, int32_t* dom_sorted)
{
    dinfo* di = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    const int64_t ncells = orc_pbf_num_cells(p, doms, nd);
    const kconst k       = make_kconst(p);
    const float dt       = p->dt;
    const float dt2      = dt * dt;
    const float g2x      = dt2 * p->gravity[0];
    const float g2y      = dt2 * p->gravity[1];

    float* xs       = (float*)malloc(sizeof(float) * 2 * (size_t)(n > 0 ? n : 1));
    uint32_t* kk    = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    uint32_t* count = (uint32_t*)calloc((size_t)ncells + 1, sizeof(uint32_t));

    /* predict (PBF.cu:790-791) and key (PBF.cu:792-794) */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const dinfo* d  = &di[dom_of(dom, i)];
        const float px  = fmaf(dt, v[2 * i], x[2 * i]) + g2x;
        const float py  = fmaf(dt, v[2 * i + 1], x[2 * i + 1]) + g2y;
        xs[2 * i]       = px;
        xs[2 * i + 1]   = py;
        const int32_t cx = cell_coord(px, d->ox, k.inv_cell, d->ncx);
        const int32_t cy = cell_coord(py, d->oy, k.inv_cell, d->ncy);
        kk[i]            = (uint32_t)(d->coff + (int64_t)cy * d->ncx + cx);
    }
    /* stable counting sort */
    for (int64_t i = 0; i < n; ++i) { count[kk[i]]++; }
    uint32_t run = 0;
    for (int64_t c = 0; c < ncells; ++c) {
        const uint32_t t = count[c];
        cell_start[c]    = run;
        count[c]         = run;
        run += t;
    }
    cell_start[ncells] = run;
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t dst = count[kk[i]]++;
        perm[dst]          = (uint32_t)i;
    }
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n; ++s) {
        const uint32_t i      = perm[s];
        key[s]                = kk[i];
        x_sorted[2 * s]       = x[2 * i];
        x_sorted[2 * s + 1]   = x[2 * i + 1];
        xs_sorted[2 * s]      = xs[2 * i];
        xs_sorted[2 * s + 1]  = xs[2 * i + 1];
        if (dom_sorted) { dom_sorted[s] = dom_of(dom, i); }
    }
    free(count);
    free(kk);
    free(xs);
    free(di);
}

/* ----- lambda: PBF.cu:243-294 ----- */
static double lambda_one(const gpe_pbf_params* p, const kconst* k, const dinfo* d, const uint32_t* cs, int64_t i,
                         int64_t pbase, const double* xs, const uint32_t* pair_id, double* rho_out,
                         double* lraw_out)
{
    const double px = xs[2 * i], py = xs[2 * i + 1];
    int64_t beg[16], end[16];
    const int32_t nr = scan_rows(d, k, cs, (float)px, (float)py, beg, end);
    const double m   = p->mass;
    double gx = 0, gy = 0, gsq = 0, rho = 0;
    for (int32_t r = 0; r < nr; ++r) {
        for (int64_t j = beg[r]; j < end[r]; ++j) {
            const double rx = px - xs[2 * j], ry = py - xs[2 * j + 1];
            const double r2 = rx * rx + ry * ry;
            if (r2 > k->h2) { continue; }
            double dist = 0.0, nx = 0.0, ny = 0.0;
            if (r2 > 1e-12) {
                dist = sqrt(r2);
                nx   = rx / dist;
                ny   = ry / dist;
            }
            if (px == xs[2 * j] && py == xs[2 * j + 1]) {
                if (p->flags & GPE_PBF_SELF_GRAD) {
                    if (pair_id) {
                        pair_direction(pair_id[i], pair_id[j], &nx, &ny);
                    } else {
                        pair_direction(i - pbase, j - pbase, &nx, &ny);
                    }
                } else {
                    nx = ny = 0.0;
                }
            }
            const double diff = k->h - dist;
            const double sc   = -k->cs * diff * diff;
            const double svx  = sc * nx * m, svy = sc * ny * m;
            gx += svx;
            gy += svy;
            gsq += (svx * svx + svy * svy) / m;
            const double q = k->h2 - r2;
            rho += m * k->c6 * q * q * q;
        }
    }
    double C = rho / p->rho0 - 1.0;
    if (C < p->c_min) { C = p->c_min; }
    const double self = (gx * gx + gy * gy) / m;
    const double grad = (self + gsq) / ((double)p->rho0 * p->rho0);
    if (rho_out) { *rho_out = rho; }
    if (lraw_out) { *lraw_out = -(rho / p->rho0 - 1.0) / (grad + p->eps); } /* unclamped C */
    return -C / (grad + p->eps);
}

static int64_t* dom_pbase(const dinfo* di, int32_t nd, const uint32_t* cs)
{
    int64_t* pb = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nd > 0 ? nd : 1));
    for (int32_t d = 0; d < nd; ++d) { pb[d] = cs[di[d].coff]; }
    return pb;
}

static double* to_double(const float* a, int64_t n)
{
    double* o = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) { o[i] = a[i]; }
    return o;
}

static void lambda_pass(const gpe_pbf_params* p, const dinfo* di, const int64_t* pb, int64_t n, const double* xs,
                        const int32_t* dom, const uint32_t* cs, const uint32_t* pair_id, double* lambda, double* rho)
{
    const kconst k = make_kconst(p);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t d = dom_of(dom, i);
        double r;
        lambda[i] = lambda_one(p, &k, &di[d], cs, i, pb[d], xs, pair_id, &r, NULL);
        if (rho) { rho[i] = r; }
    }
}

/* A later iteration of a warm-started step (the device's k_lambda with ACC): the summed multiplier moves by
 * the unclamped lambda and is projected to <= 0; delta receives the change, which the delta-p pass applies. */
static void lambda_proj_pass(const gpe_pbf_params* p, const dinfo* di, const int64_t* pb, int64_t n, const double* xs,
                             const int32_t* dom, const uint32_t* cs, const uint32_t* pair_id, double* sum,
                             double* delta)
{
    const kconst k = make_kconst(p);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t d = dom_of(dom, i);
        double lraw;
        (void)lambda_one(p, &k, &di[d], cs, i, pb[d], xs, pair_id, NULL, &lraw);
        double an = sum[i] + lraw;
        if (an > 0.0) { an = 0.0; }
        delta[i] = an - sum[i];
        sum[i]   = an;
    }
}

/* ----- delta p: PBF.cu:398-447 and handleOOB PBF.cu:471-499 ----- */
static void delta_p_pass(const gpe_pbf_params* p, const dinfo* di, int64_t n, const double* xs, const int32_t* dom,
                         const uint32_t* cs, const double* lambda, double* out)
{
    const kconst k = make_kconst(p);
    const double m = p->mass;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const dinfo* d  = &di[dom_of(dom, i)];
        const double px = xs[2 * i], py = xs[2 * i + 1];
        const double li = lambda[i];
        int64_t beg[16], end[16];
        const int32_t nr = scan_rows(d, &k, cs, (float)px, (float)py, beg, end);
        double dx = 0, dy = 0;
        for (int32_t r = 0; r < nr; ++r) {
            for (int64_t j = beg[r]; j < end[r]; ++j) {
                const double rx = px - xs[2 * j], ry = py - xs[2 * j + 1];
                const double r2 = rx * rx + ry * ry;
                if (r2 > k.h2) { continue; }
                double dist = 0.0, nx = 0.0, ny = 0.0;
                if (r2 > 1e-12) {
                    dist = sqrt(r2);
                    nx   = rx / dist;
                    ny   = ry / dist;
                }
                const double q  = k.h2 - r2;
                double scorr    = 0.0;
                if (p->scorr_k != 0.f) {
                    const double ratio = k.c6 * q * q * q * k.inv_w_dq;
                    const double r2q   = ratio * ratio;
                    scorr              = p->scorr_k * r2q * r2q;
                }
                const double l    = li * m + lambda[j] * m - scorr;
                const double diff = k.h - dist;
                const double sc   = -k.cs * diff * diff;
                dx += sc * nx * l;
                dy += sc * ny * l;
            }
        }
        const double s = (double)p->omega / (m * p->rho0);
        double nxp     = px + dx * s;
        double nyp     = py + dy * s;
        /* clamp<float>(v, lb, ub): above ub -> ub, below lb -> lb */
        if (nyp > d->hiy) { nyp = d->hiy; } else if (nyp < d->loy) { nyp = d->loy; }
        if (nxp > d->hix) { nxp = d->hix; } else if (nxp < d->lox) { nxp = d->lox; }
        out[2 * i]     = nxp;
        out[2 * i + 1] = nyp;
    }
}

/* velocityClamp, PBF.cu:629-638 */
static void vel_clamp(const gpe_pbf_params* p, double* vx, double* vy)
{
    const double v2 = *vx * *vx + *vy * *vy;
    /* v2 == 0 only matters when v_min == 0 (the reference always has v_min > 0): the clamp is then 0/0 */
    if (v2 < (double)p->v_min * p->v_min || v2 == 0.0) {
        *vx = *vy = 0.0;
        return;
    }
    const double a = sqrt(v2);
    const double s = a < p->v_max ? a : p->v_max;
    *vx            = *vx / a * s;
    *vy            = *vy / a * s;
}

/* ----- velocity + XSPH: PBF.cu:538, 585-627; vorticity (Macklin & Mueller eq. 15) ----- */
static void xsph_pass(const gpe_pbf_params* p, const dinfo* di, int64_t n, const double* x, const double* xs,
                      const int32_t* dom, const uint32_t* cs, double* vout, double* omega)
{
    const kconst k     = make_kconst(p);
    const double idt   = 1.0 / p->dt;
    const int vort     = p->vort_eps != 0.f;
    const int do_clamp = (p->flags & GPE_PBF_VEL_CLAMP) && !vort;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const dinfo* d   = &di[dom_of(dom, i)];
        const double px  = xs[2 * i], py = xs[2 * i + 1];
        const double vax = (px - x[2 * i]) * idt, vay = (py - x[2 * i + 1]) * idt;
        int64_t beg[16], end[16];
        const int32_t nr = scan_rows(d, &k, cs, (float)px, (float)py, beg, end);
        double dvx = 0, dvy = 0, w = 0;
        for (int32_t r = 0; r < nr; ++r) {
            for (int64_t j = beg[r]; j < end[r]; ++j) {
                const double rx = px - xs[2 * j], ry = py - xs[2 * j + 1];
                const double r2 = rx * rx + ry * ry;
                if (r2 > k.h2) { continue; }
                const double vbx = (xs[2 * j] - x[2 * j]) * idt, vby = (xs[2 * j + 1] - x[2 * j + 1]) * idt;
                const double q   = k.h2 - r2;
                const double p6  = k.c6 * q * q * q;
                dvx += (vbx - vax) * p6;
                dvy += (vby - vay) * p6;
                if (vort && r2 > 1e-12) {
                    const double dist = sqrt(r2);
                    const double diff = k.h - dist;
                    const double gm   = k.cs * diff * diff / dist; /* grad_j W_ij = +cs (h-r)^2 r_ij/|r_ij| */
                    const double gxj = gm * rx, gyj = gm * ry;
                    w += (vbx - vax) * gyj - (vby - vay) * gxj;
                }
            }
        }
        double vx = vax + p->xsph_c * dvx;
        double vy = vay + p->xsph_c * dvy;
        if (do_clamp) { vel_clamp(p, &vx, &vy); }
        vout[2 * i]     = vx;
        vout[2 * i + 1] = vy;
        if (omega) { omega[i] = w; }
    }
}

/* vorticity confinement, Macklin & Mueller 2013 eq. 16: eta = grad |omega|, N = eta/|eta|,
 * f = eps (N x omega), v += dt f */
static void vorticity_pass(const gpe_pbf_params* p, const dinfo* di, int64_t n, const double* xs,
                           const int32_t* dom, const uint32_t* cs, const double* omega, double* v)
{
    const kconst k     = make_kconst(p);
    const int do_clamp = (p->flags & GPE_PBF_VEL_CLAMP) != 0;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const dinfo* d  = &di[dom_of(dom, i)];
        const double px = xs[2 * i], py = xs[2 * i + 1];
        const double wi = fabs(omega[i]);
        int64_t beg[16], end[16];
        const int32_t nr = scan_rows(d, &k, cs, (float)px, (float)py, beg, end);
        double ex = 0, ey = 0;
        for (int32_t r = 0; r < nr; ++r) {
            for (int64_t j = beg[r]; j < end[r]; ++j) {
                const double rx = px - xs[2 * j], ry = py - xs[2 * j + 1];
                const double r2 = rx * rx + ry * ry;
                if (r2 > k.h2 || r2 <= 1e-12) { continue; }
                const double dist = sqrt(r2);
                const double diff = k.h - dist;
                const double gm   = -k.cs * diff * diff / dist; /* grad_i W_ij */
                const double dw   = fabs(omega[j]) - wi;
                ex += dw * gm * rx;
                ey += dw * gm * ry;
            }
        }
        const double el = sqrt(ex * ex + ey * ey);
        double vx = v[2 * i], vy = v[2 * i + 1];
        if (el > 1e-20) {
            const double Nx = ex / el, Ny = ey / el;
            vx += p->dt * p->vort_eps * (Ny * omega[i]);
            vy += p->dt * p->vort_eps * (-Nx * omega[i]);
        }
        if (do_clamp) { vel_clamp(p, &vx, &vy); }
        v[2 * i]     = vx;
        v[2 * i + 1] = vy;
    }
}

static void density_pass(const gpe_pbf_params* p, const dinfo* di, int64_t n, const double* xs, const int32_t* dom,
                         const uint32_t* cs, double* rho)
{
    const kconst k = make_kconst(p);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const dinfo* d  = &di[dom_of(dom, i)];
        const double px = xs[2 * i], py = xs[2 * i + 1];
        int64_t beg[16], end[16];
        const int32_t nr = scan_rows(d, &k, cs, (float)px, (float)py, beg, end);
        double s         = 0.0;
        for (int32_t r = 0; r < nr; ++r) {
            for (int64_t j = beg[r]; j < end[r]; ++j) {
                const double rx = px - xs[2 * j], ry = py - xs[2 * j + 1];
                const double r2 = rx * rx + ry * ry;
                if (r2 > k.h2) { continue; }
                const double q = k.h2 - r2;
                s += p->mass * k.c6 * q * q * q;
            }
        }
        rho[i] = s;
    }
}

/* ----- public stage wrappers (FP32 in/out) ----- */
void orc_pbf_lambda(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                    const int32_t* dom, const uint32_t* cell_start, const uint32_t* pair_id, float* lambda,
                    float* rho)
{
    dinfo* di   = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    int64_t* pb = dom_pbase(di, nd, cell_start);
    double* xd  = to_double(xs, 2 * n);
    double* l   = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double* r   = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    lambda_pass(p, di, pb, n, xd, dom, cell_start, pair_id, l, r);
    for (int64_t i = 0; i < n; ++i) {
        lambda[i] = (float)l[i];
        if (rho) { rho[i] = (float)r[i]; }
    }
    free(r);
    free(l);
    free(xd);
    free(pb);
    free(di);
}

void orc_pbf_delta_p(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                     const int32_t* dom, const uint32_t* cell_start, const float* lambda, float* xs_out)
{
    dinfo* di  = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    double* xd = to_double(xs, 2 * n);
    double* ld = to_double(lambda, n);
    double* o  = (double*)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    delta_p_pass(p, di, n, xd, dom, cell_start, ld, o);
    for (int64_t i = 0; i < 2 * n; ++i) { xs_out[i] = (float)o[i]; }
    free(o);
    free(ld);
    free(xd);
    free(di);
}

void orc_pbf_xsph(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* x,
                  const float* xs, const int32_t* dom, const uint32_t* cell_start, float* v_out, float* omega)
{
    dinfo* di   = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    double* xd  = to_double(x, 2 * n);
    double* xsd = to_double(xs, 2 * n);
    double* vo  = (double*)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    double* w   = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    xsph_pass(p, di, n, xd, xsd, dom, cell_start, vo, w);
    for (int64_t i = 0; i < n; ++i) {
        v_out[2 * i]     = (float)vo[2 * i];
        v_out[2 * i + 1] = (float)vo[2 * i + 1];
        if (omega) { omega[i] = (float)w[i]; }
    }
    free(w);
    free(vo);
    free(xsd);
    free(xd);
    free(di);
}

void orc_pbf_vorticity(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n,
                       const float* xs, const int32_t* dom, const uint32_t* cell_start, const float* omega,
                       float* v_inout)
{
    dinfo* di   = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    double* xsd = to_double(xs, 2 * n);
    double* wd  = to_double(omega, n);
    double* vd  = to_double(v_inout, 2 * n);
    vorticity_pass(p, di, n, xsd, dom, cell_start, wd, vd);
    for (int64_t i = 0; i < 2 * n; ++i) { v_inout[i] = (float)vd[i]; }
    free(vd);
    free(wd);
    free(xsd);
    free(di);
}

void orc_pbf_density(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                     const int32_t* dom, const uint32_t* cell_start, float* rho)
{
    dinfo* di   = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    double* xsd = to_double(xs, 2 * n);
    double* r   = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    density_pass(p, di, n, xsd, dom, cell_start, r);
    for (int64_t i = 0; i < n; ++i) { rho[i] = (float)r[i]; }
    free(r);
    free(xsd);
    free(di);
}

void orc_pbf_density_error(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n,
                           const float* x, const int32_t* dom, const uint32_t* cell_start, double* max_err,
                           double* mean_err)
{
    dinfo* di  = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    double* xd = to_double(x, 2 * n);
    double* r  = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    density_pass(p, di, n, xd, dom, cell_start, r);
    double mx = 0.0, sum = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double e = r[i] / p->rho0 - 1.0;
        if (e < 0.0) { e = 0.0; }
        if (e > mx) { mx = e; }
        sum += e;
    }
    *max_err  = mx;
    *mean_err = n > 0 ? sum / (double)n : 0.0;
    free(r);
    free(xd);
    free(di);
}

void orc_pbf_step(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, float* x, float* v,
                  int32_t* dom, uint32_t* pair_id, int32_t n_steps, float* lambda_out, uint32_t* cell_start_out)
{
    dinfo* di            = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    const int64_t ncells = orc_pbf_num_cells(p, doms, nd);
    const size_t nn      = (size_t)(n > 0 ? n : 1);
    uint32_t* key        = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* perm       = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* cs         = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)ncells + 1));
    float* xsort         = (float*)malloc(sizeof(float) * 2 * nn);
    float* xssort        = (float*)malloc(sizeof(float) * 2 * nn);
    int32_t* dsort       = (int32_t*)malloc(sizeof(int32_t) * nn);
    double* xd           = (double*)malloc(sizeof(double) * 2 * nn);
    double* xsa          = (double*)malloc(sizeof(double) * 2 * nn);
    double* xsb          = (double*)malloc(sizeof(double) * 2 * nn);
    double* lam          = (double*)malloc(sizeof(double) * nn);
    double* vd           = (double*)malloc(sizeof(double) * 2 * nn);
    double* w            = (double*)malloc(sizeof(double) * nn);
    uint32_t* pid_sorted = pair_id ? (uint32_t*)malloc(sizeof(uint32_t) * nn) : NULL;
    for (int32_t s = 0; s < n_steps; ++s) {
        orc_pbf_predict_sort(p, doms, nd, n, x, v, dom, key, perm, cs, xsort, xssort, dsort);
        if (pair_id) {
            for (int64_t i = 0; i < n; ++i) { pid_sorted[i] = pair_id[perm[i]]; }
            memcpy(pair_id, pid_sorted, sizeof(uint32_t) * nn);
        }
        int64_t* pb = dom_pbase(di, nd, cs);
        for (int64_t i = 0; i < 2 * n; ++i) {
            xd[i]  = xsort[i];
            xsa[i] = xssort[i];
        }
        for (int32_t it = 0; it < p->iters; ++it) {
            lambda_pass(p, di, pb, n, xsa, dsort, cs, pid_sorted, lam, NULL);
            delta_p_pass(p, di, n, xsa, dsort, cs, lam, xsb);
            double* t = xsa;
            xsa       = xsb;
            xsb       = t;
        }
        xsph_pass(p, di, n, xd, xsa, dsort, cs, vd, w);
        if (p->vort_eps != 0.f) { vorticity_pass(p, di, n, xsa, dsort, cs, w, vd); }
        for (int64_t i = 0; i < 2 * n; ++i) {
            x[i] = (float)xsa[i];
            v[i] = (float)vd[i];
        }
        if (dom) {
            for (int64_t i = 0; i < n; ++i) { dom[i] = dsort[i]; }
        }
        free(pb);
    }
    if (lambda_out) {
        for (int64_t i = 0; i < n; ++i) { lambda_out[i] = (float)lam[i]; }
    }
    if (cell_start_out) { memcpy(cell_start_out, cs, sizeof(uint32_t) * ((size_t)ncells + 1)); }
    free(pid_sorted);
    free(w);
    free(vd);
    free(lam);
    free(xsb);
    free(xsa);
    free(xd);
    free(dsort);
    free(xssort);
    free(xsort);
    free(cs);
    free(perm);
    free(key);
    free(di);
}

/* ===================================================================================================== */
/* PBF warm start: features, the network (with the device's BF16 operand roundings), warm-started steps     */
/* ===================================================================================================== */

/* FP32 value of v rounded to the nearest BF16, ties to even (the operand rounding of the tensor-core path) */
static double bf16r(double v)
{
    float f = (float)v;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) { return f; }
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    memcpy(&f, &u, 4);
    return f;
}

#define NF GPE_MLP_FEATURES
#define NH GPE_MLP_HIDDEN
enum { W1 = 0, B1 = W1 + NH * NF, W2 = B1 + NH, B2 = W2 + NH * NH, W3 = B2 + NH, B3 = W3 + NH, NW = B3 + 1 };

/* The 12 features of particle i (the device's warm_features) and the cold first-iteration lambda. */
static double features_one(const gpe_pbf_params* p, const kconst* k, const dinfo* d, const uint32_t* cs, int64_t i,
                           int64_t pbase, const double* xs, const double* x, const double* prev,
                           const uint32_t* pair_id, double f[NF])
{
    const double px = xs[2 * i], py = xs[2 * i + 1];
    int64_t beg[16], end[16];
    const int32_t nr = scan_rows(d, k, cs, (float)px, (float)py, beg, end);
    const double m   = p->mass;
    double gx = 0, gy = 0, gsq = 0, rho = 0, sw = 0, swl = 0;
    int64_t nn = 0;
    for (int32_t r = 0; r < nr; ++r) {
        for (int64_t j = beg[r]; j < end[r]; ++j) {
            const double rx = px - xs[2 * j], ry = py - xs[2 * j + 1];
            const double r2 = rx * rx + ry * ry;
            if (r2 > k->h2) { continue; }
            if (j != i) { ++nn; }
            double dist = 0.0, nx = 0.0, ny = 0.0;
            if (r2 > 1e-12) {
                dist = sqrt(r2);
                nx   = rx / dist;
                ny   = ry / dist;
            }
            if (px == xs[2 * j] && py == xs[2 * j + 1]) {
                if (p->flags & GPE_PBF_SELF_GRAD) {
                    if (pair_id) {
                        pair_direction(pair_id[i], pair_id[j], &nx, &ny);
                    } else {
                        pair_direction(i - pbase, j - pbase, &nx, &ny);
                    }
                } else {
                    nx = ny = 0.0;
                }
            }
            const double diff = k->h - dist;
            const double sc   = -k->cs * diff * diff;
            const double svx  = sc * nx * m, svy = sc * ny * m;
            gx += svx;
            gy += svy;
            gsq += (svx * svx + svy * svy) / m;
            const double q  = k->h2 - r2;
            const double w6 = q * q * q;
            rho += m * k->c6 * w6;
            sw += w6;
            swl += w6 * prev[j];
        }
    }
    double C = rho / p->rho0 - 1.0;
    if (C < p->c_min) { C = p->c_min; }
    const double self = (gx * gx + gy * gy) / m;
    const double grad = (self + gsq) / ((double)p->rho0 * p->rho0);
    const double lam  = -C / (grad + p->eps);
    const double dx = px - x[2 * i], dy = py - x[2 * i + 1];
    double wall = px - d->lox;
    if (d->hix - px < wall) { wall = d->hix - px; }
    if (py - d->loy < wall) { wall = py - d->loy; }
    if (d->hiy - py < wall) { wall = d->hiy - py; }
    wall /= (double)p->h;
    f[0]  = (double)nn;
    f[1]  = prev[i];
    f[2]  = rho / p->rho0 - 1.0;
    f[3]  = C;
    f[4]  = sqrt(dx * dx + dy * dy) / (double)p->h;
    f[5]  = gx / p->rho0;
    f[6]  = gy / p->rho0;
    f[7]  = sqrt(f[5] * f[5] + f[6] * f[6]);
    f[8]  = grad;
    f[9]  = lam;
    f[10] = wall < 0.0 ? 0.0 : (wall > 4.0 ? 4.0 : wall);
    f[11] = sw > 0.0 ? swl / sw : 0.0;
    return lam;
}

static void features_pass(const gpe_pbf_params* p, const dinfo* di, const int64_t* pb, int64_t n, const double* xs,
                          const double* x, const double* prev, const int32_t* dom, const uint32_t* cs,
                          const uint32_t* pair_id, double* feat, double* lam)
{
    const kconst k = make_kconst(p);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t d = dom_of(dom, i);
        double f[NF];
        const double l = features_one(p, &k, &di[d], cs, i, pb[d], xs, x, prev, pair_id, f);
        if (feat) { memcpy(&feat[i * NF], f, sizeof(f)); }
        if (lam) { lam[i] = l; }
    }
}

void orc_pbf_features(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                      const float* x, const float* prev, const int32_t* dom, const uint32_t* cell_start,
                      const uint32_t* pair_id, float* features)
{
    dinfo* di     = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    int64_t* pb   = dom_pbase(di, nd, cell_start);
    double* xsd   = to_double(xs, 2 * n);
    double* xd    = to_double(x, 2 * n);
    double* pd    = to_double(prev, n);
    double* f     = (double*)malloc(sizeof(double) * NF * (size_t)(n > 0 ? n : 1));
    features_pass(p, di, pb, n, xsd, xd, pd, dom, cell_start, pair_id, f, NULL);
    for (int64_t q = 0; q < NF * n; ++q) { features[q] = (float)f[q]; }
    free(f);
    free(pd);
    free(xd);
    free(xsd);
    free(pb);
    free(di);
}

/* Network restated from its parameter blob (layout in gpe.h); operands rounded to BF16 where the device
 * feeds the tensor cores, everything else in FP64. */
typedef struct {
    double w1[NH][NF], b1[NH], w2[NH][NH], b2[NH], w3[NH], b3;
    double mu[NF], isd[NF], ymu, ysd;
    int rnd; /* 1: BF16 operand roundings of the device; 0: plain FP64 (for finite-difference checks) */
} mlpnet;

static double opr(const mlpnet* m, double v) { return m->rnd ? bf16r(v) : v; }

static void mlp_load(const float* blob, mlpnet* m, int rnd)
{
    m->rnd = rnd;
    for (int i = 0; i < NH; ++i) {
        for (int f = 0; f < NF; ++f) { m->w1[i][f] = opr(m, blob[W1 + i * NF + f]); }
        m->b1[i] = blob[B1 + i];
        for (int q = 0; q < NH; ++q) { m->w2[i][q] = opr(m, blob[W2 + i * NH + q]); }
        m->b2[i] = blob[B2 + i];
        m->w3[i] = blob[W3 + i];
    }
    m->b3 = blob[B3];
    for (int f = 0; f < NF; ++f) {
        m->mu[f]        = blob[NW + f];
        const float sd  = blob[NW + NF + f];
        m->isd[f]       = sd > 0.f ? (double)(1.0f / sd) : 0.0;
    }
    m->ymu = blob[NW + 2 * NF];
    m->ysd = blob[NW + 2 * NF + 1];
}

/* forward for one standardised-and-rounded input; returns y (standardised) and the layer values */
static double mlp_fwd(const mlpnet* m, const double* xin, double xb[NF], double z1[NH], double a1b[NH],
                      double z2[NH])
{
    for (int f = 0; f < NF; ++f) { xb[f] = opr(m, (xin[f] - m->mu[f]) * m->isd[f]); }
    for (int i = 0; i < NH; ++i) {
        double s = 0.0;
        for (int f = 0; f < NF; ++f) { s += m->w1[i][f] * xb[f]; }
        z1[i]  = s + m->b1[i];
        a1b[i] = opr(m, z1[i] > 0.0 ? z1[i] : 0.0);
    }
    double y = m->b3;
    for (int j = 0; j < NH; ++j) {
        double s = 0.0;
        for (int i = 0; i < NH; ++i) { s += m->w2[j][i] * a1b[i]; }
        z2[j] = s + m->b2[j];
        y += (z2[j] > 0.0 ? z2[j] : 0.0) * m->w3[j];
    }
    return y;
}

void orc_mlp_forward(const float* blob, int64_t n, const float* X, float* out, int32_t bf16)
{
    mlpnet* m = (mlpnet*)malloc(sizeof(mlpnet));
    mlp_load(blob, m, bf16);
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n; ++s) {
        double xin[NF], xb[NF], z1[NH], a1b[NH], z2[NH];
        for (int f = 0; f < NF; ++f) { xin[f] = X[s * NF + f]; }
        const double y = mlp_fwd(m, xin, xb, z1, a1b, z2);
        out[s]         = (float)(y * m->ysd + m->ymu);
    }
    free(m);
}

void orc_mlp_gradient(const float* blob, int64_t n, const float* X, const float* T, double* grad, double* loss,
                      int32_t bf16)
{
    mlpnet* m = (mlpnet*)malloc(sizeof(mlpnet));
    mlp_load(blob, m, bf16);
    memset(grad, 0, sizeof(double) * NW);
    const double iysd = m->ysd > 0.0 ? (double)(1.0f / (float)m->ysd) : 0.0;
    double L          = 0.0;
    for (int64_t s = 0; s < n; ++s) {
        double xin[NF], xb[NF], z1[NH], a1b[NH], z2[NH], dz2b[NH], dz1b[NH];
        for (int f = 0; f < NF; ++f) { xin[f] = X[s * NF + f]; }
        const double y  = mlp_fwd(m, xin, xb, z1, a1b, z2);
        const double tn = ((double)T[s] - m->ymu) * iysd;
        const double e  = y - tn;
        const double dy = 2.0 * e / (double)n;
        L += e * e;
        for (int j = 0; j < NH; ++j) {
            const double a2 = z2[j] > 0.0 ? z2[j] : 0.0;
            grad[W3 + j] += dy * a2;
            dz2b[j] = opr(m, z2[j] > 0.0 ? dy * m->w3[j] : 0.0);
            grad[B2 + j] += dz2b[j];
            for (int i = 0; i < NH; ++i) { grad[W2 + j * NH + i] += dz2b[j] * a1b[i]; }
        }
        grad[B3] += dy;
        for (int i = 0; i < NH; ++i) {
            double da = 0.0;
            for (int j = 0; j < NH; ++j) { da += dz2b[j] * m->w2[j][i]; }
            dz1b[i] = opr(m, z1[i] > 0.0 ? da : 0.0);
            grad[B1 + i] += dz1b[i];
            for (int f = 0; f < NF; ++f) { grad[W1 + i * NF + f] += dz1b[i] * xb[f]; }
        }
    }
    *loss = n > 0 ? L / (double)n : 0.0;
    free(m);
}

/* Warm-started steps (mode GPE_WARM_PREV / GPE_WARM_MLP) or cold steps that keep the summed multipliers
 * (GPE_WARM_NONE). acc holds the previous step's sums in the current order and receives this step's sums
 * in the new sorted order. blob is the network for GPE_WARM_MLP. */
void orc_pbf_step_warm(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, float* x, float* v,
                       int32_t* dom, uint32_t* pair_id, float* acc, int32_t mode, const float* blob,
                       int32_t n_steps)
{
    dinfo* di            = (dinfo*)malloc(sizeof(dinfo) * (size_t)nd);
    build_dinfo(p, doms, nd, di);
    const int64_t ncells = orc_pbf_num_cells(p, doms, nd);
    const size_t nn      = (size_t)(n > 0 ? n : 1);
    uint32_t* key        = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* perm       = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* cs         = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)ncells + 1));
    float* xsort         = (float*)malloc(sizeof(float) * 2 * nn);
    float* xssort        = (float*)malloc(sizeof(float) * 2 * nn);
    int32_t* dsort       = (int32_t*)malloc(sizeof(int32_t) * nn);
    double* xd           = (double*)malloc(sizeof(double) * 2 * nn);
    double* xsa          = (double*)malloc(sizeof(double) * 2 * nn);
    double* xsb          = (double*)malloc(sizeof(double) * 2 * nn);
    double* lam          = (double*)malloc(sizeof(double) * nn);
    double* sum          = (double*)malloc(sizeof(double) * nn);
    double* prev         = (double*)malloc(sizeof(double) * nn);
    double* feat         = (double*)malloc(sizeof(double) * NF * nn);
    double* vd           = (double*)malloc(sizeof(double) * 2 * nn);
    double* w            = (double*)malloc(sizeof(double) * nn);
    uint32_t* pid_sorted = pair_id ? (uint32_t*)malloc(sizeof(uint32_t) * nn) : NULL;
    mlpnet* net          = NULL;
    if (mode == GPE_WARM_MLP) {
        net = (mlpnet*)malloc(sizeof(mlpnet));
        mlp_load(blob, net, 1);
    }
    for (int32_t s = 0; s < n_steps; ++s) {
        orc_pbf_predict_sort(p, doms, nd, n, x, v, dom, key, perm, cs, xsort, xssort, dsort);
        if (pair_id) {
            for (int64_t i = 0; i < n; ++i) { pid_sorted[i] = pair_id[perm[i]]; }
            memcpy(pair_id, pid_sorted, sizeof(uint32_t) * nn);
        }
        for (int64_t i = 0; i < n; ++i) { prev[i] = acc[perm[i]]; }
        int64_t* pb = dom_pbase(di, nd, cs);
        for (int64_t i = 0; i < 2 * n; ++i) {
            xd[i]  = xsort[i];
            xsa[i] = xssort[i];
        }
        for (int32_t it = 0; it < p->iters; ++it) {
            if (it == 0) {
                if (mode == GPE_WARM_MLP) {
                    features_pass(p, di, pb, n, xsa, xd, prev, dsort, cs, pid_sorted, feat, NULL);
#pragma omp parallel for schedule(static)
                    for (int64_t i = 0; i < n; ++i) {
                        double xb[NF], z1[NH], a1b[NH], z2[NH];
                        const double y = mlp_fwd(net, &feat[i * NF], xb, z1, a1b, z2);
                        const double l = prev[i] + (y * net->ysd + net->ymu);
                        lam[i]         = l < 0.0 ? l : 0.0;
                    }
                } else if (mode == GPE_WARM_PREV) {
                    memcpy(lam, prev, sizeof(double) * nn);
                } else {
                    lambda_pass(p, di, pb, n, xsa, dsort, cs, pid_sorted, lam, NULL);
                }
                memcpy(sum, lam, sizeof(double) * nn);
            } else if (mode == GPE_WARM_PREV) {
                lambda_proj_pass(p, di, pb, n, xsa, dsort, cs, pid_sorted, sum, lam);
            } else {
                lambda_pass(p, di, pb, n, xsa, dsort, cs, pid_sorted, lam, NULL);
                if (mode == GPE_WARM_NONE) {
                    for (int64_t i = 0; i < n; ++i) { sum[i] += lam[i]; }
                }
            }
            delta_p_pass(p, di, n, xsa, dsort, cs, lam, xsb);
            double* t = xsa;
            xsa       = xsb;
            xsb       = t;
        }
        xsph_pass(p, di, n, xd, xsa, dsort, cs, vd, w);
        if (p->vort_eps != 0.f) { vorticity_pass(p, di, n, xsa, dsort, cs, w, vd); }
        for (int64_t i = 0; i < 2 * n; ++i) {
            x[i] = (float)xsa[i];
            v[i] = (float)vd[i];
        }
        for (int64_t i = 0; i < n; ++i) { acc[i] = p->iters > 0 ? (float)sum[i] : 0.f; }
        if (dom) {
            for (int64_t i = 0; i < n; ++i) { dom[i] = dsort[i]; }
        }
        free(pb);
    }
    free(net);
    free(pid_sorted);
    free(w);
    free(vd);
    free(feat);
    free(prev);
    free(sum);
    free(lam);
    free(xsb);
    free(xsa);
    free(xd);
    free(dsort);
    free(xssort);
    free(xsort);
    free(cs);
    free(perm);
    free(key);
    free(di);
}

/* ===================================================================================================== */
/* Splat rasteriser: backgroundKernel, alpha and drawKernel of libs/render/source/cuda-render.cu:214-310,     */
/* run sequentially (chunk by chunk, atom by atom) into a tightly packed RGBA8 image                        */
/* ===================================================================================================== */

static uint8_t blend_ch(uint8_t over, uint8_t under, float a, float ia)
{
    return (uint8_t)((float)over * a + (float)under * ia + 0.5f); /* alpha(), cuda-render.cu:244-258 */
}

void orc_render_frame(int32_t width, int32_t height, float scale, float chunk_dim, int32_t chunks, int32_t capacity,
                      const float* pos, const int32_t* counts, uint8_t* rgba)
{
    const int32_t every = (int32_t)(chunk_dim * scale);
    for (int32_t y = 0; y < height; ++y) {
        for (int32_t x = 0; x < width; ++x) {
            uint8_t* px = &rgba[((size_t)y * width + x) * 4];
            if (x % every == 0 || y % every == 0) {
                px[0] = px[1] = px[2] = 0;
            } else {
                const float t = 100.f * ((float)y / (float)height);
                px[0]         = (uint8_t)(255u - (uint8_t)t);
                px[1]         = (uint8_t)(160u - (uint8_t)t);
                px[2]         = 80;
            }
            px[3] = 255;
        }
    }
    const float c  = 1.f / 255.f;
    const float a  = (float)100 * c;
    const float ia = 1.f - a;
    for (int32_t ch = 0; ch < chunks; ++ch) {
        const int32_t n = counts[ch] < capacity ? counts[ch] : capacity;
        for (int32_t k = 0; k < n; ++k) {
            const float* p   = &pos[((size_t)ch * capacity + k) * 2];
            const int32_t px = (int32_t)(p[0] * scale);
            const int32_t py = (int32_t)(p[1] * scale);
            if (px < 0 || py < 0 || px >= width || py >= height) { continue; }
            for (int32_t i = -2; i <= 2; ++i) {
                if (py + i < 0 || py + i >= height) { continue; }
                for (int32_t j = -2; j <= 2; ++j) {
                    if (px + j < 0 || px + j >= width || ((i == 2 || i == -2) && (j == 2 || j == -2))) { continue; }
                    uint8_t* q = &rgba[((size_t)(py + i) * width + (px + j)) * 4];
                    q[0]       = blend_ch(140, q[0], a, ia);
                    q[1]       = blend_ch(210, q[1], a, ia);
                    q[2]       = blend_ch(255, q[2], a, ia);
                    q[3]       = 255;
                }
            }
        }
    }
}

/* ===================================================================================================== */
/* MLS-MPM                                                                                                */
/* ===================================================================================================== */

static int mpm_material(const gpe_mpm_params* p, const int32_t* mat, int64_t i)
{
    if (mat && (p->flags & GPE_MPM_FLAG_PER_PARTICLE_MATERIAL)) { return mat[i]; }
    return p->material;
}

/* quadratic B-spline weights, MPM.cu:92-110 */
static void bspline(double g, int32_t* base, double* f, double w[3])
{
    const double b = floor(g - 0.5);
    *base          = (int32_t)b;
    *f             = g - b;
    const double fx = *f;
    w[0]            = 0.5 * (1.5 - fx) * (1.5 - fx);
    w[1]            = 0.75 - (fx - 1.0) * (fx - 1.0);
    w[2]            = 0.5 * (fx - 0.5) * (fx - 0.5);
}

/* polar decomposition of a 2x2 matrix (row-major a b / c d): F = R S with R a rotation */
static void polar2(const double F[4], double R[4])
{
    double cx = F[0] + F[3], sx = F[2] - F[1];
    const double nrm = sqrt(cx * cx + sx * sx);
    if (nrm < 1e-30) {
        R[0] = 1; R[1] = 0; R[2] = 0; R[3] = 1;
        return;
    }
    cx /= nrm;
    sx /= nrm;
    R[0] = cx; R[1] = -sx; R[2] = sx; R[3] = cx;
}

/* 2x2 SVD F = U diag(s) V^T with U, V rotations (s may carry the sign of det F in s[1]) */
static void svd2(const double F[4], double U[4], double s[2], double V[4])
{
    double R[4];
    polar2(F, R);
    /* S = R^T F, symmetric */
    const double a = R[0] * F[0] + R[2] * F[2];
    const double b = R[0] * F[1] + R[2] * F[3];
    const double d = R[1] * F[1] + R[3] * F[3];
    double c = 1.0, sn = 0.0;
    if (fabs(b) > 1e-30) {
        const double th = 0.5 * atan2(2.0 * b, a - d);
        c               = cos(th);
        sn              = sin(th);
    }
    V[0] = c; V[1] = -sn; V[2] = sn; V[3] = c;
    /* eigenvalues of S in the V basis */
    s[0] = c * c * a + 2.0 * c * sn * b + sn * sn * d;
    s[1] = sn * sn * a - 2.0 * c * sn * b + c * c * d;
    /* U = R V */
    U[0] = R[0] * V[0] + R[1] * V[2];
    U[1] = R[0] * V[1] + R[1] * V[3];
    U[2] = R[2] * V[0] + R[3] * V[2];
    U[3] = R[2] * V[1] + R[3] * V[3];
}

/* affine momentum matrix Q = m C + coeff * stress (MPM.cu:68-80 for the fluid) */
static void mpm_affine(const gpe_mpm_params* p, int mat, const float* C, const float* F, double J, double Q[4])
{
    const double inv_dx = 1.0 / p->dx;
    const double m      = p->mass;
    double tau[4]       = {0, 0, 0, 0};
    double coeff;
    if (mat == GPE_MPM_MAT_FLUID) {
        double pr = (double)p->k_bulk * (pow(1.0 / J, (double)p->gamma) - 1.0);
        if (pr < p->p_min) { pr = p->p_min; }
        if (pr > p->p_max) { pr = p->p_max; }
        tau[0] = -pr;
        tau[3] = -pr;
        const double Vp = (double)p->vol0 * J;
        coeff           = -(double)p->dt * Vp * 4.0 * inv_dx * inv_dx;
    } else if (mat == GPE_MPM_MAT_NEOHOOKEAN) {
        const double Fd[4] = {F[0], F[1], F[2], F[3]};
        const double mu    = (double)p->E / (2.0 * (1.0 + p->nu));
        const double la    = (double)p->E * p->nu / ((1.0 + p->nu) * (1.0 - 2.0 * p->nu));
        double Je          = Fd[0] * Fd[3] - Fd[1] * Fd[2];
        if (Je < 1e-6) { Je = 1e-6; }
        const double lj = la * log(Je);
        tau[0] = mu * (Fd[0] * Fd[0] + Fd[1] * Fd[1] - 1.0) + lj;
        tau[1] = mu * (Fd[0] * Fd[2] + Fd[1] * Fd[3]);
        tau[2] = tau[1];
        tau[3] = mu * (Fd[2] * Fd[2] + Fd[3] * Fd[3] - 1.0) + lj;
        coeff  = -(double)p->dt * p->vol0 * 4.0 * inv_dx * inv_dx;
    } else if (mat == GPE_MPM_MAT_SAND) {
        const double Fd[4] = {F[0], F[1], F[2], F[3]};
        const double mu    = (double)p->E / (2.0 * (1.0 + p->nu));
        const double la    = (double)p->E * p->nu / ((1.0 + p->nu) * (1.0 - 2.0 * p->nu));
        double U[4], sg[2], V[4];
        svd2(Fd, U, sg, V);
        const double e0 = log(sg[0] > 1e-6 ? sg[0] : 1e-6), e1 = log(sg[1] > 1e-6 ? sg[1] : 1e-6);
        const double a0 = 2.0 * mu * e0 + la * (e0 + e1), a1 = 2.0 * mu * e1 + la * (e0 + e1);
        /* tau = U diag(a) U^T */
        tau[0] = U[0] * U[0] * a0 + U[1] * U[1] * a1;
        tau[1] = U[0] * U[2] * a0 + U[1] * U[3] * a1;
        tau[2] = tau[1];
        tau[3] = U[2] * U[2] * a0 + U[3] * U[3] * a1;
        coeff  = -(double)p->dt * p->vol0 * 4.0 * inv_dx * inv_dx;
    } else {
        const double Fd[4] = {F[0], F[1], F[2], F[3]};
        double mu = (double)p->E / (2.0 * (1.0 + p->nu));
        double la = (double)p->E * p->nu / ((1.0 + p->nu) * (1.0 - 2.0 * p->nu));
        if (mat == GPE_MPM_MAT_SNOW) {
            const double hf = exp((double)p->hardening * (1.0 - J)); /* J holds the plastic J_p */
            mu *= hf;
            la *= hf;
        }
        double R[4];
        polar2(Fd, R);
        const double Je = Fd[0] * Fd[3] - Fd[1] * Fd[2];
        /* tau = 2 mu (F - R) F^T + la (Je - 1) Je I */
        const double A[4] = {Fd[0] - R[0], Fd[1] - R[1], Fd[2] - R[2], Fd[3] - R[3]};
        tau[0] = 2.0 * mu * (A[0] * Fd[0] + A[1] * Fd[1]) + la * (Je - 1.0) * Je;
        tau[1] = 2.0 * mu * (A[0] * Fd[2] + A[1] * Fd[3]);
        tau[2] = 2.0 * mu * (A[2] * Fd[0] + A[3] * Fd[1]);
        tau[3] = 2.0 * mu * (A[2] * Fd[2] + A[3] * Fd[3]) + la * (Je - 1.0) * Je;
        coeff  = -(double)p->dt * p->vol0 * 4.0 * inv_dx * inv_dx;
    }
    for (int k = 0; k < 4; ++k) { Q[k] = m * C[k] + coeff * tau[k]; }
}

void orc_mpm_p2g(const gpe_mpm_params* p, int64_t n, const float* x, const float* v, const float* C,
                 const float* F, const float* J, const int32_t* mat, double* grid)
{
    const size_t nn = (size_t)p->nx * (size_t)p->ny;
    memset(grid, 0, sizeof(double) * 3 * nn);
    const double inv_dx = 1.0 / p->dx;
    const double m      = p->mass;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const int mt = mpm_material(p, mat, i);
        double Q[4];
        mpm_affine(p, mt, &C[4 * i], &F[4 * i], (double)J[i], Q);
        int32_t bx, by;
        double fx, fy, wx[3], wy[3];
        bspline((double)x[2 * i] * inv_dx + p->grid_offset, &bx, &fx, wx);
        bspline((double)x[2 * i + 1] * inv_dx + p->grid_offset, &by, &fy, wy);
        if (bx < 0) { bx = 0; }
        if (by < 0) { by = 0; }
        if (bx > p->nx - 3) { bx = p->nx - 3; }
        if (by > p->ny - 3) { by = p->ny - 3; }
        for (int a = 0; a < 3; ++a) {
            for (int b = 0; b < 3; ++b) {
                const double w   = wx[a] * wy[b];
                const double dpx = ((double)a - fx) * p->dx, dpy = ((double)b - fy) * p->dx;
                const double afx = dpx * Q[0] + dpy * Q[1];
                const double afy = dpx * Q[2] + dpy * Q[3];
                const size_t node = (size_t)(by + b) * (size_t)p->nx + (size_t)(bx + a);
                const double gx = w * (v[2 * i] * m + afx), gy = w * (v[2 * i + 1] * m + afy), gm = w * m;
#pragma omp atomic
                grid[3 * node] += gx;
#pragma omp atomic
                grid[3 * node + 1] += gy;
#pragma omp atomic
                grid[3 * node + 2] += gm;
            }
        }
    }
}

void orc_mpm_grid_update(const gpe_mpm_params* p, double* grid)
{
    const int32_t bw = p->bc_width;
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < (int64_t)p->nx * p->ny; ++idx) {
        double* g = &grid[3 * idx];
        if (g[2] > 0.0) {
            const int32_t xx = (int32_t)(idx % p->nx);
            const int32_t yy = (int32_t)(idx / p->nx);
            double vx        = g[0] / g[2] + (double)p->gravity[0] * p->dt;
            double vy        = g[1] / g[2] + (double)p->gravity[1] * p->dt;
            const int wl = xx <= bw, wr = xx >= p->nx - 1 - bw, wb = yy <= bw, wt = yy >= p->ny - 1 - bw;
            if (p->bc_type == GPE_MPM_BC_STICKY) {
                if (wl || wr || wb || wt) { vx = vy = 0.0; }
            } else {
                if (wl && vx < 0.0) { vx = 0.0; } else if (wr && vx > 0.0) { vx = 0.0; }
                if (wb && vy < 0.0) { vy = 0.0; } else if (wt && vy > 0.0) { vy = 0.0; }
            }
            g[0] = vx;
            g[1] = vy;
        } else {
            g[0] = 0.0;
            g[1] = 0.0;
        }
    }
}

/* Drucker-Prager return mapping of the Hencky strain (Klar et al. 2016, d = 2). F is projected in place
 * and *J (= 1 + q) grows by the plastic strain increment; returns whether F changed. */
static int sand_project(const gpe_mpm_params* p, double F[4], double* J, double sc[2])
{
    const int dflt = p->sand_h[0] == 0.f && p->sand_h[1] == 0.f && p->sand_h[2] == 0.f && p->sand_h[3] == 0.f;
    const double h0 = dflt ? 35.0 : p->sand_h[0], h1 = dflt ? 9.0 : p->sand_h[1];
    const double h2 = dflt ? 0.2 : p->sand_h[2], h3 = dflt ? 10.0 : p->sand_h[3];
    const double mu = (double)p->E / (2.0 * (1.0 + p->nu));
    const double la = (double)p->E * p->nu / ((1.0 + p->nu) * (1.0 - 2.0 * p->nu));
    double U[4], sg[2], V[4];
    svd2(F, U, sg, V);
    const double e0 = log(sg[0] > 1e-6 ? sg[0] : 1e-6), e1 = log(sg[1] > 1e-6 ? sg[1] : 1e-6);
    const double tr = e0 + e1;
    const double d0 = e0 - 0.5 * tr, d1 = e1 - 0.5 * tr;
    const double dn = sqrt(d0 * d0 + d1 * d1);
    const double q = *J - 1.0;
    const double phi = h0 + (h1 * q - h3) * exp(-h2 * q); /* degrees */
    const double sp = sin(phi * M_PI / 180.0);
    const double alpha = sqrt(2.0 / 3.0) * 2.0 * sp / (3.0 - sp);
    double dq;
    if (tr >= 0.0) { /* expansion: the cone's tip */
        sc[0] = sc[1] = 1.0;
        dq = sqrt(e0 * e0 + e1 * e1);
    } else {
        const double dg = dn + (2.0 * la + 2.0 * mu) / (2.0 * mu) * tr * alpha;
        if (dg <= 0.0) { return 0; } /* inside the cone: elastic */
        sc[0] = exp(e0 - dg / dn * d0);
        sc[1] = exp(e1 - dg / dn * d1);
        dq    = dg;
    }
    *J += dq;
    F[0] = U[0] * sc[0] * V[0] + U[1] * sc[1] * V[1];
    F[1] = U[0] * sc[0] * V[2] + U[1] * sc[1] * V[3];
    F[2] = U[2] * sc[0] * V[0] + U[3] * sc[1] * V[1];
    F[3] = U[2] * sc[0] * V[2] + U[3] * sc[1] * V[3];
    return 1;
}

void orc_mpm_g2p(const gpe_mpm_params* p, int64_t n, const double* grid, float* x, float* v, float* C,
                 float* F, float* J, const int32_t* mat)
{
    const double inv_dx = 1.0 / p->dx;
    const double dt     = p->dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const int mt = mpm_material(p, mat, i);
        int32_t bx, by;
        double fx, fy, wx[3], wy[3];
        bspline((double)x[2 * i] * inv_dx + p->grid_offset, &bx, &fx, wx);
        bspline((double)x[2 * i + 1] * inv_dx + p->grid_offset, &by, &fy, wy);
        if (bx < 0) { bx = 0; }
        if (by < 0) { by = 0; }
        if (bx > p->nx - 3) { bx = p->nx - 3; }
        if (by > p->ny - 3) { by = p->ny - 3; }
        double vx = 0, vy = 0, B[4] = {0, 0, 0, 0};
        for (int a = 0; a < 3; ++a) {
            for (int b = 0; b < 3; ++b) {
                const double w    = wx[a] * wy[b];
                const double dpx  = ((double)a - fx) * p->dx, dpy = ((double)b - fy) * p->dx;
                const size_t node = (size_t)(by + b) * (size_t)p->nx + (size_t)(bx + a);
                const double gvx = grid[3 * node], gvy = grid[3 * node + 1];
                vx += w * gvx;
                vy += w * gvy;
                B[0] += w * gvx * dpx;
                B[1] += w * gvx * dpy;
                B[2] += w * gvy * dpx;
                B[3] += w * gvy * dpy;
            }
        }
        const double s = 4.0 * inv_dx * inv_dx;
        double px      = x[2 * i] + vx * dt;
        double py      = x[2 * i + 1] + vy * dt;
        double Cn[4]   = {s * B[0], s * B[1], s * B[2], s * B[3]};
        /* handleOOB, MPM.cu:267-301 */
        if (!isfinite(px) || !isfinite(vx)) { px = 0.5 * ((double)p->clamp_lo[0] + p->clamp_hi[0]); vx = 0.0; }
        if (!isfinite(py) || !isfinite(vy)) { py = 0.5 * ((double)p->clamp_lo[1] + p->clamp_hi[1]); vy = 0.0; }
        if (px < p->clamp_lo[0]) { px = p->clamp_lo[0]; if (vx < 0.0) { vx = 0.0; } }
        if (px > p->clamp_hi[0]) { px = p->clamp_hi[0]; if (vx > 0.0) { vx = 0.0; } }
        if (py < p->clamp_lo[1]) { py = p->clamp_lo[1]; if (vy < 0.0) { vy = 0.0; } }
        if (py > p->clamp_hi[1]) { py = p->clamp_hi[1]; if (vy > 0.0) { vy = 0.0; } }
        /* F <- (I + dt C) F, J <- J det(I + dt C) (MPM.cu:258-265) */
        const double A[4]  = {1.0 + Cn[0] * dt, Cn[1] * dt, Cn[2] * dt, 1.0 + Cn[3] * dt};
        const double Fo[4] = {F[4 * i], F[4 * i + 1], F[4 * i + 2], F[4 * i + 3]};
        double Fn[4]       = {A[0] * Fo[0] + A[1] * Fo[2], A[0] * Fo[1] + A[1] * Fo[3],
                              A[2] * Fo[0] + A[3] * Fo[2], A[2] * Fo[1] + A[3] * Fo[3]};
        double Jn          = J[i];
        if (mt == GPE_MPM_MAT_FLUID) {
            Jn *= A[0] * A[3] - A[1] * A[2];
            if (Jn < p->J_min) { Jn = p->J_min; }
            if (Jn > p->J_max) { Jn = p->J_max; }
        } else if (mt == GPE_MPM_MAT_SNOW) {
            double U[4], sg[2], V[4];
            svd2(Fn, U, sg, V);
            double sc[2];
            for (int k = 0; k < 2; ++k) {
                sc[k] = sg[k];
                if (sc[k] < 1.0 - p->theta_c) { sc[k] = 1.0 - p->theta_c; }
                if (sc[k] > 1.0 + p->theta_s) { sc[k] = 1.0 + p->theta_s; }
            }
            Jn *= (sg[0] * sg[1]) / (sc[0] * sc[1]);
            /* F = U diag(sc) V^T */
            Fn[0] = U[0] * sc[0] * V[0] + U[1] * sc[1] * V[1];
            Fn[1] = U[0] * sc[0] * V[2] + U[1] * sc[1] * V[3];
            Fn[2] = U[2] * sc[0] * V[0] + U[3] * sc[1] * V[1];
            Fn[3] = U[2] * sc[0] * V[2] + U[3] * sc[1] * V[3];
        } else if (mt == GPE_MPM_MAT_SAND) {
            double sc[2];
            (void)sand_project(p, Fn, &Jn, sc); /* Fn recomposed from the projected singular values sc */
        }
        x[2 * i]     = (float)px;
        x[2 * i + 1] = (float)py;
        v[2 * i]     = (float)vx;
        v[2 * i + 1] = (float)vy;
        for (int k = 0; k < 4; ++k) {
            C[4 * i + k] = (float)Cn[k];
            F[4 * i + k] = (float)Fn[k];
        }
        J[i] = (float)Jn;
    }
}

void orc_mpm_step(const gpe_mpm_params* p, int64_t n, float* x, float* v, float* C, float* F, float* J,
                  const int32_t* mat, int32_t n_steps)
{
    double* grid = (double*)malloc(sizeof(double) * 3 * (size_t)p->nx * (size_t)p->ny);
    for (int32_t s = 0; s < n_steps; ++s) {
        orc_mpm_p2g(p, n, x, v, C, F, J, mat, grid);
        orc_mpm_grid_update(p, grid);
        orc_mpm_g2p(p, n, grid, x, v, C, F, J, mat);
    }
    free(grid);
}
