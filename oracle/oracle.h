/*
 * oracle.h — CPU restatement of the reference solver steps. TEST INFRASTRUCTURE ONLY: this library is
 * the checker for the CUDA engine and the timed CPU baseline; the engine never links or calls it.
 *
 * Arithmetic is FP64 except where the reference's FP32 rounding decides an integer result (the predicted
 * position that feeds the cell key, the cell key itself and the base cell of a neighbour scan), which is
 * restated in FP32 with the same operation order as the device so that keys and sorted order are
 * bit-exact. Parity of this restatement with the reference build is checked by the GPU tests that run the
 * reference's own kernels (tests/test_reference_parity.py) and by the committed fixtures in tests/golden.
 */
#ifndef GPE_ORACLE_H
#define GPE_ORACLE_H

#include <stdint.h>

#include "../include/gpe.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------- PBF ---------- */
int64_t orc_pbf_num_cells(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd);
/* Predict x* = fma(dt, v, x) + dt^2 g in FP32, compute the cell key and stable-sort by key.
 * Outputs are in sorted order: key, perm (pre-sort index), x, x*, dom; cell_start has n_cells+1 entries. */
void orc_pbf_predict_sort(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n,
                          const float* x, const float* v, const int32_t* dom, uint32_t* key, uint32_t* perm,
                          uint32_t* cell_start, float* x_sorted, float* xs_sorted, int32_t* dom_sorted);
/* Stage restatements on sorted inputs (FP64 arithmetic, FP32 in/out). */
/* pair_id (sorted order, may be NULL) seeds the coincident-pair direction instead of the sorted index */
void orc_pbf_lambda(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                    const int32_t* dom, const uint32_t* cell_start, const uint32_t* pair_id, float* lambda,
                    float* rho);
void orc_pbf_delta_p(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                     const int32_t* dom, const uint32_t* cell_start, const float* lambda, float* xs_out);
void orc_pbf_xsph(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* x,
                  const float* xs, const int32_t* dom, const uint32_t* cell_start, float* v_out, float* omega);
void orc_pbf_vorticity(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n,
                       const float* xs, const int32_t* dom, const uint32_t* cell_start, const float* omega,
                       float* v_inout);
void orc_pbf_density(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                     const int32_t* dom, const uint32_t* cell_start, float* rho);
/* Whole steps. x, v, dom (and pair_id, may be NULL) are the state in the current order and are replaced by
 * the state in the new sorted order after each step (x <- final x*). Between iterations x* is kept in FP64.
 * lambda (may be NULL) receives the last iteration's lambda. */
void orc_pbf_step(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, float* x, float* v,
                  int32_t* dom, uint32_t* pair_id, int32_t n_steps, float* lambda, uint32_t* cell_start_out);
/* max_i max(rho_i/rho0-1,0) and mean of the same over particles, from orc_pbf_density on x. */
void orc_pbf_density_error(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n,
                           const float* x, const int32_t* dom, const uint32_t* cell_start, double* max_err,
                           double* mean_err);

/* ---------- PBF warm start ---------- */
/* The 12 warm-start features (gpe.h) of every sorted particle: xs = sorted x*, x = sorted x, prev = the
 * previous step's summed multipliers in sorted order. features: n x 12. */
void orc_pbf_features(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, const float* xs,
                      const float* x, const float* prev, const int32_t* dom, const uint32_t* cell_start,
                      const uint32_t* pair_id, float* features);
/* The network from its blob (GPE_MLP_BLOB_FLOATS): out = de-standardised prediction of n raw feature rows.
 * bf16 = 1 rounds the tensor-core operands (standardised features, W1, W2, hidden layer 1, and in the
 * gradient dZ2 and dZ1) to BF16 as the device does; 0 computes in plain FP64. */
void orc_mlp_forward(const float* blob, int64_t n, const float* X, float* out, int32_t bf16);
/* Gradient (GPE_MLP_NUM_WEIGHTS) of mean((y - t_std)^2) over n pairs; loss receives that mean. */
void orc_mlp_gradient(const float* blob, int64_t n, const float* X, const float* T, double* grad, double* loss,
                      int32_t bf16);
/* Steps that keep a per-particle multiplier memory (acc: in the current order in, in the new order out):
 *   GPE_WARM_NONE  the plain step (a pair-collecting step); acc <- the sum of its iterations' lambdas
 *   GPE_WARM_PREV  first delta-p pass with lambda_prev, later iterations update the sum by the unclamped
 *                  lambda projected to <= 0 and apply the change; acc <- that sum
 *   GPE_WARM_MLP   first delta-p pass with L = min(lambda_prev + r, 0), r from the network blob, later
 *                  iterations plain; acc <- L
 * Other arguments as orc_pbf_step. */
void orc_pbf_step_warm(const gpe_pbf_params* p, const gpe_domain* doms, int32_t nd, int64_t n, float* x, float* v,
                       int32_t* dom, uint32_t* pair_id, float* acc, int32_t mode, const float* blob,
                       int32_t n_steps);

/* ---------- splat rasteriser ---------- */
/* The reference's background and splat blend, sequentially (chunk by chunk, atom by atom): pos holds
 * chunks * capacity float2 (chunk-major, as a published view), counts the atoms per chunk; rgba receives
 * width * height * 4 bytes. */
void orc_render_frame(int32_t width, int32_t height, float scale, float chunk_dim, int32_t chunks, int32_t capacity,
                      const float* pos, const int32_t* counts, uint8_t* rgba);

/* ---------- MLS-MPM ---------- */
/* grid: nx*ny*3 doubles (momentum x, momentum y, mass) */
void orc_mpm_p2g(const gpe_mpm_params* p, int64_t n, const float* x, const float* v, const float* C,
                 const float* F, const float* J, const int32_t* mat, double* grid);
/* in place: momentum -> velocity, gravity, walls */
void orc_mpm_grid_update(const gpe_mpm_params* p, double* grid);
/* grid: velocities (after orc_mpm_grid_update). Updates the particle state in place. */
void orc_mpm_g2p(const gpe_mpm_params* p, int64_t n, const double* grid, float* x, float* v, float* C,
                 float* F, float* J, const int32_t* mat);
void orc_mpm_step(const gpe_mpm_params* p, int64_t n, float* x, float* v, float* C, float* F, float* J,
                  const int32_t* mat, int32_t n_steps);

int32_t orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
