/*
 * gpe.h — C ABI of the GB300 particle engine (PBF and MLS-MPM solver steps).
 *
 * Every entry point takes plain pointers and sizes and returns an int32 status (GPE_OK == 0, negative on
 * failure), following the error convention of the reference's only C ABI,
 * libs/render/include/render/cuda-interface.h:30-42 (0 ok, -1 CUDA error kept in last_error, -2 device
 * mismatch, -3 not initialised, -4 bad argument, -5 already initialised), extended with -6 capacity
 * overflow, -7 non-finite state and -8 device wait timeout.
 *
 * The handle-based entry points replace the reference's C++ engine interface
 * (libs/cuda-engine/include/cuda-engine/cuda-engine.h): gpe_pbf_create/destroy stand in for the PBFArena
 * constructor/destructor (cuda-engine.cpp:102-143), gpe_pbf_step for one launch of the tick graph built by
 * instantiatePBFGraph (cuda-engine.h:164-167, PBF.cu:901-961), gpe_mpm_* likewise for MPMArena
 * (cuda-engine.h:190-216) and instantiateMPMGraph (cuda-engine.h:227-230, MPM.cu:326-374).
 *
 * Streams are passed as void* holding a cudaStream_t (NULL = legacy default stream). All work of one handle
 * must be issued from one host thread on one stream, as in the reference (cuda-engine.h:171).
 */
#ifndef GPE_H
#define GPE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----- status codes ------------------------------------------------------------------------------------ */
#define GPE_OK 0
#define GPE_ERR_CUDA (-1)      /* a CUDA runtime call failed; gpe_last_cuda_error() has the cudaError_t   */
#define GPE_ERR_DEVICE (-2)    /* no usable device, or the handle belongs to another device               */
#define GPE_ERR_NOT_READY (-3) /* handle not initialised / state not set / extension missing            */
#define GPE_ERR_BAD_ARG (-4)   /* null pointer, negative size, inconsistent parameters                   */
#define GPE_ERR_ALREADY (-5)   /* already initialised                                                    */
#define GPE_ERR_CAPACITY (-6)  /* particle, cell or scratch capacity exceeded                            */
#define GPE_ERR_NONFINITE (-7) /* the device status word recorded a non-finite value                     */
#define GPE_ERR_TIMEOUT (-8)   /* a bounded device wait gave up                                          */

/* memory kinds for state transfer */
#define GPE_MEM_HOST 0
#define GPE_MEM_DEVICE 1
/* page-locked host memory (cudaHostAlloc / cudaHostRegister), for gpe_pbf_set_state and gpe_pbf_get_state
 * only: the copy is enqueued on the stream and the call returns without waiting, so copies of one engine
 * can overlap another engine's work; the caller synchronizes the stream before reusing (set) or reading
 * (get) the buffer. */
#define GPE_MEM_PINNED 2

/* device status word bits (gpe_*_status) */
#define GPE_STATUS_NONFINITE 0x1u
#define GPE_STATUS_CAPACITY 0x2u
#define GPE_STATUS_CELL_OVERFLOW 0x4u
#define GPE_STATUS_TIMEOUT 0x8u

const char* gpe_error_name(int32_t status);
int32_t gpe_last_cuda_error(void);        /* cudaError_t of the last failing CUDA call on this thread */
const char* gpe_last_error_message(void); /* human readable detail of the last failure on this thread */
int32_t gpe_version(void);                /* major*10000 + minor*100 + patch                           */

/* ======================================================================================================
 * Position-Based Fluids
 * ====================================================================================================== */

/* PBF flags */
#define GPE_PBF_SELF_GRAD 0x1u    /* include the self pair's pseudo-random spiky gradient in the lambda
                                     denominator exactly as the reference does (PBF.cu:264-285 loops over
                                     the atom itself; coincident pairs take pairDirection, PBF.cu:309-321) */
#define GPE_PBF_VEL_CLAMP 0x2u    /* clamp |v| to [v_min, v_max] after XSPH (velocityClamp, PBF.cu:629-638) */
#define GPE_PBF_TRACK_IDS 0x4u    /* carry a particle id through every sort (for external bookkeeping)      */
#define GPE_PBF_DYNAMIC_COUNT 0x10u /* keep the particle count on the device: launches cover the capacity and
                                       read the live count, so emitters (gpe_pbf_emit) can add particles
                                       between steps of a replayed graph, as the reference's hosePipe does
                                       through its migration queues (PBF.cu:1021-1030); one scene only       */
#define GPE_PBF_PAIR_IDS 0x8u     /* seed pairDirection with the tracked particle ids instead of the sorted
                                     index within the scene (the reference seeds it with the atom's slot in
                                     its chunk, PBF.cu:277); implies GPE_PBF_TRACK_IDS                       */

typedef struct gpe_pbf_params {
    float h;            /* smoothing radius (reference kH, constants.h:35)                          */
    float cell;         /* sort-cell edge; 0 selects h (reference kCellDim == kH, constants.h:46)  */
    float rho0;         /* rest density (kRho0, constants.h:36)                                     */
    float mass;         /* particle mass (kMass, constants.h:27)                                    */
    float dt;           /* step length; 1 makes velocities per-step displacements as in the
                           reference (cuda-engine.h:131)                                              */
    float gravity[2];   /* acceleration; x* = x + dt v + dt^2 g (PBF.cu:790-791 adds kGravityStep) */
    int32_t iters;      /* Jacobi iterations per step (kIters, PBF.cu:12)                            */
    float eps;          /* constraint relaxation (kEpsilon, PBF.cu:14)                               */
    float scorr_k;      /* artificial pressure scale (kSCorrK, PBF.cu:15); 0 disables                */
    float scorr_dq;     /* artificial pressure reference distance (kDq, constants.h:40)              */
    float omega;        /* over-relaxation of the Jacobi update (kOmega, PBF.cu:20)                  */
    float c_min;        /* lower clamp of the density constraint (kMinC, PBF.cu:21)                   */
    float xsph_c;       /* XSPH coefficient applied to sum (v_j - v_i) W_ij (kC, PBF.cu:16)          */
    float vort_eps;     /* vorticity-confinement strength; 0 disables (absent in the reference)     */
    float v_max;        /* velocity clamp (kMaxSpeed, PBF.cu:23), used with GPE_PBF_VEL_CLAMP        */
    float v_min;        /* below this speed v is zeroed (kMinSpeed, PBF.cu:22)                       */
    float wall_margin;  /* positions are clamped to [lo, hi - wall_margin] (PBF.cu:487-490 uses 1e-3) */
    float poly6_coeff;  /* 0 selects 4/(pi h^8); the reference uses 1/(64*3.14159f), constants.h:38  */
    float spiky_coeff;  /* 0 selects 30/(pi h^5); the reference uses 30/(32*3.14159f), constants.h:39 */
    uint32_t flags;     /* GPE_PBF_* */
} gpe_pbf_params;

/* One independent scene (domain). A scene is an axis-aligned box with walls on all four sides and its own
 * uniform sort grid; scenes never exchange particles. One scene reproduces the reference's whole world
 * (kSceneDimX x kSceneDimY chunks, constants.h:11-12); many scenes form the batched launch. */
typedef struct gpe_domain {
    float origin[2]; /* lower corner */
    float extent[2]; /* box size     */
} gpe_domain;

typedef struct gpe_pbf gpe_pbf;

/* Stages of one PBF step, in order. gpe_pbf_step runs PREDICT_SORT, iters x (LAMBDA, DELTA_P), XSPH,
 * [VORTICITY if vort_eps != 0], FINISH. */
#define GPE_PBF_STAGE_PREDICT_SORT 0 /* prepNextSubstepKernel PBF.cu:738-834 (predict, cell key, sort)       */
#define GPE_PBF_STAGE_LAMBDA 1       /* lambdaKernel PBF.cu:215-308                                           */
#define GPE_PBF_STAGE_DELTA_P 2      /* posCorrectionKernel PBF.cu:365-470 + handleOOB PBF.cu:471-499         */
#define GPE_PBF_STAGE_XSPH 3         /* velocityKernel PBF.cu:500-553 + XSPHKernel PBF.cu:554-638 (fused)     */
#define GPE_PBF_STAGE_VORTICITY 4    /* vorticity confinement (Macklin & Mueller 2013 eq. 15-16)              */
#define GPE_PBF_STAGE_FINISH 5       /* x <- x*, publish the step                                             */
#define GPE_PBF_STAGE_DENSITY 6      /* recompute rho for the density-error metric (not part of a step)       */
#define GPE_PBF_STAGE_WARM_LAMBDA 7  /* first lambda of a warm-started step (gpe_pbf_set_warm_start); the next
                                        DELTA_P starts the step's multiplier sum from it                        */

/* Fields that can be read or written for inspection (element types in brackets). All are in the current
 * sorted order; n_elems counts elements of the field's type. */
#define GPE_PBF_FIELD_POS 0        /* x  [float2]                                          */
#define GPE_PBF_FIELD_VEL 1        /* v  [float2]                                          */
#define GPE_PBF_FIELD_PRED 2       /* x* [float2]                                          */
#define GPE_PBF_FIELD_LAMBDA 3     /* lambda [float]                                       */
#define GPE_PBF_FIELD_KEY 4        /* global cell key of each sorted particle [uint32]     */
#define GPE_PBF_FIELD_PERM 5       /* pre-sort index of each sorted particle [uint32]      */
#define GPE_PBF_FIELD_CELL_START 6 /* exclusive scan of cell counts, n_cells+1 [uint32]    */
#define GPE_PBF_FIELD_DOMAIN 7     /* scene of each particle [int32]                       */
#define GPE_PBF_FIELD_DENSITY 8    /* rho from the last DENSITY stage [float]              */
#define GPE_PBF_FIELD_ID 9         /* particle id (GPE_PBF_TRACK_IDS) [uint32]             */
#define GPE_PBF_FIELD_OMEGA 10     /* vorticity from the last XSPH stage [float]           */
#define GPE_PBF_FIELD_LAMBDA_PREV 11 /* previous step's summed multiplier, sorted [float]   */
#define GPE_PBF_FIELD_LAMBDA_SUM 12  /* this step's summed multiplier so far [float]        */
#define GPE_PBF_FIELD_DISP 13      /* d = x* - x within a step [float2]: a step holds each particle as its start
                                      position x (POS) and its displacement d, so that neighbour offsets and
                                      velocities d / dt keep FP32 precision at any coordinate magnitude; PRED
                                      is x + d rounded once                                                      */

int32_t gpe_pbf_create(const gpe_pbf_params* params, const gpe_domain* domains, int32_t n_domains,
                       int64_t capacity, gpe_pbf** out);
int32_t gpe_pbf_destroy(gpe_pbf* pbf);
int32_t gpe_pbf_set_params(gpe_pbf* pbf, const gpe_pbf_params* params);
int32_t gpe_pbf_get_params(const gpe_pbf* pbf, gpe_pbf_params* params);
/* Replace the particle state. pos/vel hold n float2 (interleaved x,y); domain_id holds n scene indices and
 * may be NULL when there is one scene. mem selects host or device pointers. */
int32_t gpe_pbf_set_state(gpe_pbf* pbf, const float* pos, const float* vel, const int32_t* domain_id,
                          int64_t n, int32_t mem, void* stream);
int32_t gpe_pbf_get_state(gpe_pbf* pbf, float* pos, float* vel, int32_t* domain_id, int64_t n, int32_t mem,
                          void* stream);
int32_t gpe_pbf_count(const gpe_pbf* pbf, int64_t* n);
int32_t gpe_pbf_num_cells(const gpe_pbf* pbf, int64_t* n_cells);
int32_t gpe_pbf_step(gpe_pbf* pbf, int32_t n_steps, void* stream);
int32_t gpe_pbf_stage(gpe_pbf* pbf, int32_t stage, void* stream);
int32_t gpe_pbf_get_field(gpe_pbf* pbf, int32_t field, void* dst, int64_t n_elems, int32_t mem, void* stream);
int32_t gpe_pbf_set_field(gpe_pbf* pbf, int32_t field, const void* src, int64_t n_elems, int32_t mem,
                          void* stream);
/* max_i max(rho_i/rho0 - 1, 0) and its mean over particles, with rho recomputed by a separate pass. */
int32_t gpe_pbf_density_error(gpe_pbf* pbf, float* max_err, float* mean_err, void* stream);
/* Reads and clears the device status word (GPE_STATUS_*); synchronises the stream. */
int32_t gpe_pbf_status(gpe_pbf* pbf, uint32_t* status, void* stream);
/* Number of kernel launches the last gpe_pbf_step issued per step. */
int32_t gpe_pbf_launches_per_step(const gpe_pbf* pbf, int32_t* launches);
/* Self-test of the bounded device waits (no counterpart in the reference): one block arrives at the
 * persistent kernels' grid barrier set up to expect one more arrival than it will get, so its wait gives up
 * after a 100 ms limit, records GPE_STATUS_TIMEOUT and the kernel returns; *status receives the device
 * status word. The device stays usable afterwards. (Inside the persistent solve the same wait gives up after
 * 2 s, far above a barrier's microseconds, so that a context that the GPU time-slices with other processes
 * is not reported as hung.) */
int32_t gpe_selftest_barrier_timeout(uint32_t* status);

/* A "hose pipe" source (hosePipe, PBF.cu:1033-1065 and MPM.cu:439-473): rows of particles on a square lattice
 * behind a nozzle, moving with `velocity`, optionally jittered by a Gaussian of standard deviation `jitter`
 * drawn with curand's Philox generator seeded by (seed, particle index) as the reference does. Emits
 * width x rows particles with width = max(1, round(nozzle_width / spacing)) and
 * rows = max(1, round(|velocity| * dt * steps_per_call / spacing)). */
typedef struct gpe_hose {
    float origin[2];        /* nozzle centre                                                     */
    float velocity[2];      /* particle velocity in the engine's units                           */
    float nozzle_width;     /* width of the stream                                               */
    float spacing;          /* lattice spacing of the emitted particles                          */
    float jitter;           /* standard deviation of the position jitter; 0 = none               */
    int32_t steps_per_call; /* solver steps between calls (the reference's tick = 20 substeps)  */
} gpe_hose;

/* Output target for publishing a step's particles to a renderer (the reference's View, cuda-engine.h:51-57):
 * chunk-major arrays of chunks_x * chunks_y chunks with chunk_capacity slots each; counts receives the
 * number of particles written per chunk. All pointers are device pointers. */
typedef struct gpe_view {
    float* pos;             /* float2[chunks * chunk_capacity], positions in scene coordinates   */
    float* vel;             /* float2[chunks * chunk_capacity]                                   */
    int32_t* counts;        /* int32[chunks]                                                     */
    int32_t chunks_x, chunks_y;
    float chunk_dim;        /* chunk edge (kChunkDim, constants.h:48)                            */
    int32_t chunk_capacity; /* slots per chunk (kMaxAtoms, constants.h:50)                       */
} gpe_view;

/* Appends the hose's particles (needs GPE_PBF_DYNAMIC_COUNT). Particles outside the scene are dropped, as
 * in emitterKernel (PBF.cu:1014-1016); beyond the capacity they are dropped and GPE_STATUS_CAPACITY is set.
 * *requested receives width x rows (the reference's return value). */
int32_t gpe_pbf_emit(gpe_pbf* pbf, const gpe_hose* hose, uint64_t seed, int32_t* requested, void* stream);
/* Writes every particle into the chunk of its position (PBFOutputKernel, PBF.cu:861-896). view_mem says
 * where the gpe_view struct itself lives: GPE_MEM_HOST (read now) or GPE_MEM_DEVICE (read by the kernels
 * when they run, so a captured graph follows later updates of the struct, as the reference's __constant__
 * c_output does, PBF.cu:29 and TickStaging::outputTargetUpload, PBF.cu:50-55). */
int32_t gpe_pbf_publish(gpe_pbf* pbf, const gpe_view* view, int32_t view_mem, void* stream);
/* The engine's state in the reference's chunk-major arena layout (PBFArena, cuda-engine.h:124-161, as
 * prepNextSubstepKernel leaves it, PBF.cu:786-833): every particle in the chunk of its next prediction
 * x* = x + dt v + dt^2 g, chunk-local x (pos, the arena's pos[0]) and x* (pred, pos[1]), v (vel; the per-step
 * displacement when dt = 1), the last Jacobi multiplier (lambda, may be NULL), particles per chunk (counts,
 * num_atoms) and per cell of a chunk's chunk_cells x chunk_cells grid the packed slot range
 * (end << 16) | start of the particles whose prediction lies in it (offsets, chunk-major, row-major cells).
 * Within a cell the order follows atomics, as in the reference; particles beyond a chunk's capacity are left
 * out and GPE_STATUS_CAPACITY is set. */
typedef struct gpe_chunk_state {
    float* pos;         /* float2[chunks * chunk_capacity]  */
    float* pred;        /* float2[chunks * chunk_capacity]  */
    float* vel;         /* float2[chunks * chunk_capacity]  */
    float* lambda;      /* float[chunks * chunk_capacity]   */
    int32_t* counts;    /* int32[chunks]                    */
    uint32_t* offsets;  /* uint32[chunks * chunk_cells^2]   */
    int32_t chunks_x, chunks_y;
    int32_t chunk_cells;    /* cells along a chunk edge, at most 32 (kGridDim, constants.h:45) */
    float chunk_dim;        /* chunk edge (kChunkDim, constants.h:48)                          */
    int32_t chunk_capacity; /* slots per chunk, at most 65535 (kMaxAtoms, constants.h:50)      */
} gpe_chunk_state;
/* Writes the state between steps (one scene). The struct is read when the call is made; its arrays are device
 * memory (the reference's arena members), written when the work runs, so the call can be recorded into a
 * graph. */
int32_t gpe_pbf_publish_chunks(gpe_pbf* pbf, const gpe_chunk_state* state, void* stream);
/* Issues n_steps steps on the stream without an engine-owned graph, so that they can be recorded into the
 * caller's own stream capture (the reference's instantiatePBFGraph builds one graph per tick, PBF.cu:901-961).
 * Buffer roles are returned to their starting state at the end, so a captured sequence can be replayed. */
int32_t gpe_pbf_enqueue(gpe_pbf* pbf, int32_t n_steps, void* stream);

/* ======================================================================================================
 * Learned warm start of the PBF constraint solve
 * ======================================================================================================
 * The Jacobi solve computes in every iteration a multiplier lambda_i = -C_i / (|grad C|^2 + eps) per particle
 * (lambdaKernel, PBF.cu:243-294) and moves the particles by it (posCorrectionKernel, PBF.cu:395-438). Summed
 * over a plain solve of many iterations it is Lambda_i, the multiplier the converged solve applies. A
 * warm-started step uses a prediction of Lambda_i in its first delta-p pass instead of the cold
 * first-iteration lambda; its other iters - 1 passes are the plain iteration, which stays the fallback and
 * decides the result. Each particle keeps a multiplier memory carried through the sorts, lambda_prev.
 *
 *   GPE_WARM_MLP   Lambda = min(lambda_prev + r, 0), r from a 12 -> 64 -> 64 -> 1 ReLU network run on the
 *                  tensor cores (BF16 operands, FP32 accumulation) inside the first lambda pass; the later
 *                  passes are the reference's iteration; the memory keeps Lambda plus their lambdas, the
 *                  step's total multiplier, as in the training pairs. The first step after a reset has no
 *                  memory and runs the plain first pass instead (gpe_pbf_enqueue wants one step before).
 *   GPE_WARM_PREV  Lambda = lambda_prev, no network: the non-learned warm start. The later passes move the
 *                  summed multiplier by the unclamped lambda, projected to <= 0, and the memory keeps that
 *                  sum. Carrying a position-based multiplier across steps counts the last step's correction
 *                  twice (it is already in the velocity); this mode is kept as the ablation it is, not as a
 *                  stable solver.
 *
 * Network features, per particle, from the sorted predicted positions x* of the step:
 *    0 neighbours within h (self excluded)           6 dC/dy
 *    1 lambda_prev                                    7 |grad C|
 *    2 rho* / rho0 - 1                                  8 the lambda denominator without eps
 *    3 C = max(rho* / rho0 - 1, c_min)                  9 the cold first-iteration lambda
 *    4 |x* - x| / h                                  10 distance to the nearest wall / h, at most 4
 *    5 dC/dx                                         11 poly6-weighted mean of the neighbours' lambda_prev
 * Training pairs are (features, Lambda - lambda_prev) from the plain solver run with many iterations, whose
 * own Lambda is lambda_prev of its next step; the network is trained on the GPU (forward and backward
 * products on the tensor cores, AdamW) on standardised features and targets. */
typedef struct gpe_mlp gpe_mlp;
#define GPE_MLP_FEATURES 12
#define GPE_MLP_HIDDEN 64
/* parameter vector, row-major [out][in]: W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3 */
#define GPE_MLP_NUM_WEIGHTS 5057
/* blob: parameters, feature mean[12], feature std[12], target mean, target std */
#define GPE_MLP_BLOB_FLOATS 5083

typedef struct gpe_mlp_train_params {
    int32_t epochs;
    int32_t batch;       /* pairs per optimiser step                                                    */
    float lr;            /* AdamW (Loshchilov & Hutter 2019) step size                                 */
    float weight_decay;  /* decoupled decay of W1, W2, w3                                              */
    float beta1, beta2, adam_eps;
    float val_fraction;  /* the last pairs of the set are held out for the validation loss             */
    uint64_t seed;       /* shuffling of the training pairs                                            */
    int32_t lr_schedule; /* 0: constant lr; 1: cosine decay from lr to 0 over the call's optimiser steps
                            (Loshchilov & Hutter 2017), which settles the final weights                 */
} gpe_mlp_train_params;

#define GPE_WARM_NONE 0
#define GPE_WARM_PREV 1
#define GPE_WARM_MLP 2

/* A network with seeded uniform He initialisation, room for max_pairs training pairs, identity
 * standardisation. */
int32_t gpe_mlp_create(int64_t max_pairs, uint64_t seed, gpe_mlp** out);
int32_t gpe_mlp_destroy(gpe_mlp* mlp);
/* Save / load: n must be GPE_MLP_BLOB_FLOATS. */
int32_t gpe_mlp_get_blob(const gpe_mlp* mlp, float* blob, int64_t n);
int32_t gpe_mlp_set_blob(gpe_mlp* mlp, const float* blob, int64_t n);
/* Runs n_steps plain steps of pbf (params.iters iterations each) that also sum their multipliers, and
 * appends, from every step after the first, a pair for each particle that a seeded hash selects with
 * probability 1/stride. pbf must be in GPE_WARM_NONE. Pairs beyond max_pairs are dropped. */
int32_t gpe_mlp_collect(gpe_mlp* mlp, gpe_pbf* pbf, int32_t n_steps, int32_t stride, uint64_t seed, void* stream);
int32_t gpe_mlp_num_pairs(const gpe_mlp* mlp, int64_t* n);
/* features [n][12], targets [n], index [n] (the particle's sorted index when the pair was taken); any
 * output may be NULL. n must equal the pair count. */
int32_t gpe_mlp_get_pairs(const gpe_mlp* mlp, float* features, float* targets, int32_t* index, int64_t n,
                          int32_t mem, void* stream);
int32_t gpe_mlp_set_pairs(gpe_mlp* mlp, const float* features, const float* targets, int64_t n, int32_t mem,
                          void* stream);
/* Sets the standardisation from the training part of the pair set, then trains. train_loss / val_loss
 * (may be NULL) receive the mean squared error of the standardised target over the last epoch and over
 * the held-out pairs. */
int32_t gpe_mlp_train(gpe_mlp* mlp, const gpe_mlp_train_params* params, float* train_loss, float* val_loss,
                      void* stream);
/* r for n raw feature vectors (features [n][12] -> out [n], de-standardised). */
int32_t gpe_mlp_infer(const gpe_mlp* mlp, const float* features, float* out, int64_t n, int32_t mem,
                      void* stream);
/* Gradient of the mean over the n pairs of (y - t)^2, y the network output and t the standardised target,
 * with respect to the parameter vector (grad [GPE_MLP_NUM_WEIGHTS]); *loss receives that mean. Device
 * memory of the network is unchanged. */
int32_t gpe_mlp_gradient(gpe_mlp* mlp, const float* features, const float* targets, int64_t n, float* grad,
                         float* loss, int32_t mem, void* stream);
/* Selects the warm start of pbf's later steps; mlp is required for GPE_WARM_MLP and must outlive its use.
 * Resets lambda_prev to 0. */
int32_t gpe_pbf_set_warm_start(gpe_pbf* pbf, int32_t mode, const gpe_mlp* mlp);

/* ======================================================================================================
 * Headless particle splat rasteriser
 * ======================================================================================================
 * The reference's render path without D3D12 (backgroundKernel and drawKernel launched by launchFill,
 * libs/render/source/cuda-render.cu:189-310) into a pitched RGBA8 device image: the background (black chunk
 * grid lines every chunk_dim * scale pixels, else a vertical gradient), then every particle of a published
 * view as a 5 x 5 splat without corners blended with the reference's alpha() (:244-258), at pixel
 * ((int)(x * scale), (int)(y * scale)). The reference's unsynchronised blend makes overlapping splats race;
 * here each pixel gets the sequential result (the blend applied once per covering splat), independent of
 * scheduling. */
typedef struct gpe_raster {
    uint8_t* rgba;     /* device image, `pitch` bytes per row                                            */
    int64_t pitch;     /* >= 4 * width                                                                   */
    int32_t width, height;
    float scale;       /* pixels per scene unit (kSimScale, constants.h:59)                              */
    float chunk_dim;   /* chunk edge in scene units (kChunkDim, constants.h:48)                          */
    int32_t* coverage; /* device scratch of width * height int32 (splats centred on each pixel)        */
} gpe_raster;
/* view_mem: where the gpe_view struct lives (its arrays are device memory either way). */
int32_t gpe_render_frame(const gpe_raster* raster, const gpe_view* view, int32_t view_mem, void* stream);

/* ======================================================================================================
 * Tuning of the PBF step and the autotuner
 * ======================================================================================================
 * A tuning changes how a step runs, not what it computes: for a given cell size every choice gives the same
 * result bit for bit. */
typedef struct gpe_pbf_tuning {
    float cell;         /* sort-cell edge; 0 selects h. h/2 scans 5 x 5 cells of a quarter of the area,
                           testing fewer candidates per particle, over more and shorter cell rows          */
    int32_t block;      /* threads per block of the neighbour kernels: 128, 256 or 512                 */
    int32_t persistent; /* 1: the Jacobi passes and XSPH of a plain step run in one cooperative launch
                           with grid barriers between them (for many small scenes, whose steps are
                           otherwise launch-bound; vorticity keeps its own launches); 2: the predict +
                           cell sort runs inside that launch too (the sort strategy: its histogram,
                           scan, scatter and stable placement as phases between grid barriers instead of
                           five launches), so a plain step is one launch; 0: one launch per pass
                           (on a GB300, 0 measured fastest for 16k and 1M particles and 256 scenes, by
                           15-30%; the autotuner times all three)                                       */
    float skin;         /* candidate masks, in units of h, in [0, 1] (cell h only; default 0.075): the
                           first lambda pass of a step records per particle which candidates of its
                           3 x 3 cells lie within h + skin * h, and the later passes of the step visit
                           only those while no particle nearby has moved by skin * h / 2 (else that
                           particle's neighbourhood scans in full). Same result bit for bit; 0 turns
                           the masks off                                                                */
} gpe_pbf_tuning;

int32_t gpe_pbf_get_tuning(const gpe_pbf* pbf, gpe_pbf_tuning* tuning);
/* A new cell size rebuilds the scenes' sort grids (the engine holds cell arrays for h/2 and for the cell
 * size it was created with). */
int32_t gpe_pbf_set_tuning(gpe_pbf* pbf, const gpe_pbf_tuning* tuning);
/* Times trial_steps steps of every candidate (cell h with mask skin 0.1, 0.075 or 0.05 or without masks,
 * or h/2; block 128, 256 or 512; persistent 0, 1 or 2) on the current state, which is restored after every
 * trial and at the end; the three fastest run three more trials each, taking turns, and the one with the
 * smallest median time is applied;
 * *best and *ms_per_step receive it and that median (-1 when the choice came from the cache). Choices are
 * cached for the process per (scenes, particle count and mean scene aspect to the nearest power of two,
 * iterations, pair-direction flags). Needs GPE_WARM_NONE and a host particle count. */
int32_t gpe_pbf_autotune(gpe_pbf* pbf, int32_t trial_steps, gpe_pbf_tuning* best, float* ms_per_step,
                         void* stream);

/* Allocation-free predict + cell sort for one scene. It has no counterpart in the reference (whose arenas
 * are all allocated up front, cuda-engine.cpp:102-139); it exists for callers that cannot call cudaMalloc,
 * such as a host whose device memory is owned by another framework, or a real-time loop that must not
 * allocate once it is running. It runs the same kernels as GPE_PBF_STAGE_PREDICT_SORT on caller buffers
 * and keeps its scratch in a fixed static device array (7.0 MiB, sized for the limits below, held by every
 * GPU that loads the library until the process exits), so it never allocates.
 *   in : pos, vel  n float2 (device pointers), one scene `domain`, `params`
 *   out: pos_sorted, pred_sorted n float2; key_sorted, perm n uint32; cell_start n_cells + 1 uint32
 *        (n_cells from the scene extent and the sort-cell size, as gpe_pbf_num_cells reports).
 * Limits: n <= GPE_NOALLOC_MAX_PARTICLES and n_cells <= GPE_NOALLOC_MAX_CELLS, else GPE_ERR_CAPACITY.
 * The first call on a device looks up the scratch array's device address (cudaGetSymbolAddress) and should
 * come before any stream capture. Under lazy module loading the array itself is created when the library's
 * device code is first used on the device, which can be this first call; make it early, before device memory
 * runs short. pos, vel, pos_sorted and pred_sorted must be 8-byte aligned and key_sorted, perm and cell_start
 * 4-byte aligned, else GPE_ERR_BAD_ARG before any device work. All calls share the one array: calls that overlap on the GPU (on
 * different streams, or from several host threads) race, so serialise them. */
#define GPE_NOALLOC_MAX_PARTICLES (1 << 18)
#define GPE_NOALLOC_MAX_CELLS (1 << 20)
int32_t gpe_pbf_predict_sort_noalloc(const gpe_pbf_params* params, const gpe_domain* domain, const float* pos,
                                     const float* vel, int64_t n, float* pos_sorted, float* pred_sorted,
                                     uint32_t* key_sorted, uint32_t* perm, uint32_t* cell_start, int64_t n_cells,
                                     void* stream);

/* ======================================================================================================
 * MLS-MPM
 * ====================================================================================================== */

#define GPE_MPM_MAT_FLUID 0      /* J-based equation of state (reference P2GKernel, MPM.cu:68-80)          */
#define GPE_MPM_MAT_COROTATED 1  /* fixed-corotated elasticity (Stomakhin et al. 2012)                     */
#define GPE_MPM_MAT_SNOW 2       /* fixed-corotated with plasticity clamp and hardening (Stomakhin 2013)  */
#define GPE_MPM_MAT_NEOHOOKEAN 3 /* compressible Neo-Hookean: tau = mu (F F^T - I) + la ln(J) I (J = det F,
                                    floored at 1e-6)                                                        */
#define GPE_MPM_MAT_SAND 4       /* Drucker-Prager elastoplastic sand (Klar et al. 2016): St. Venant-Kirchhoff
                                    stress on the Hencky strain, return mapping of the log singular values
                                    onto the friction cone, friction-angle hardening; the particle's J holds
                                    1 + q, q the accumulated plastic strain (J = 1: q = 0)                   */

#define GPE_MPM_BC_SLIP 0        /* zero the velocity component into the wall (MPM.cu:159-168)             */
#define GPE_MPM_BC_STICKY 1      /* zero the whole node velocity inside the wall band                      */

#define GPE_MPM_FLAG_PER_PARTICLE_MATERIAL 0x1u /* read a material id per particle instead of params.material */
#define GPE_MPM_FLAG_DYNAMIC_COUNT 0x4u /* keep the particle count on the device (the reference's num_points,
                                           cuda-engine.h:206-208) so gpe_mpm_emit can add particles between
                                           steps of a replayed graph; launches cover the capacity        */
#define GPE_MPM_FLAG_FLUID_F 0x2u /* keep updating F for fluid particles, as the reference does although nothing
                                     reads it (MPM.cu:258-263, cuda-engine.h:203); off saves 32 B/particle */

typedef struct gpe_mpm_params {
    float dx;          /* node spacing (kDx, constants.h:80)                                    */
    float grid_offset; /* node coordinate of world x = 0, in nodes (kGridHalo, MPM.cu:84)        */
    int32_t nx, ny;    /* node grid (kGridDimX/Y, constants.h:76-77)                              */
    float dt;          /* step (dt, constants.h:88)                                              */
    float gravity[2];  /* added as g dt to node velocity (MPM.cu:154 adds kGravity*dt on y)       */
    float mass;        /* particle mass (kMass)                                                  */
    float vol0;        /* rest volume (kRestVol, constants.h:81)                                 */
    int32_t bc_type;   /* GPE_MPM_BC_*                                                           */
    int32_t bc_width;  /* wall band in nodes (kGridHalo == 2 in the reference)                   */
    float clamp_lo[2]; /* particle position clamp in G2P (handleOOB, MPM.cu:267-301)             */
    float clamp_hi[2];
    int32_t material;  /* GPE_MPM_MAT_* when no per-particle material is given                   */
    float k_bulk;      /* EOS stiffness (kStiffness, constants.h:84)                              */
    float gamma;       /* EOS exponent (kGamma, constants.h:85)                                   */
    float p_min, p_max;/* pressure clamp (kMinPress/kMaxPress, constants.h:86-87)                */
    float J_min, J_max;/* J clamp after the update (MPM.cu:265 uses 0.1, 10)                     */
    float E, nu;       /* Young's modulus and Poisson ratio (corotated / snow)                   */
    float theta_c, theta_s, hardening; /* snow plasticity (Stomakhin 2013)                       */
    int32_t sort_interval; /* re-sort particles by cell every this many steps; 0 = never. Within a
                              cell the storage order is that of the sort's atomics (get_state
                              returns the caller's order all the same)                       */
    uint32_t flags;    /* GPE_MPM_FLAG_*                                                         */
    float sand_h[4];   /* sand friction angle in degrees, phi = h0 + (h1 q - h3) exp(-h2 q) (Klar et al.
                          2016); all zero selects their (35, 9, 0.2, 10)                          */
} gpe_mpm_params;

typedef struct gpe_mpm gpe_mpm;

#define GPE_MPM_STAGE_CLEAR 0 /* resetGridKernel MPM.cu:46-51            */
#define GPE_MPM_STAGE_P2G 1   /* P2GKernel MPM.cu:53-129                  */
#define GPE_MPM_STAGE_GRID 2  /* gridKernel MPM.cu:131-177                */
#define GPE_MPM_STAGE_G2P 3   /* G2PKernel MPM.cu:178-301                 */
#define GPE_MPM_STAGE_SORT 4  /* spatial re-sort of the particles         */

int32_t gpe_mpm_create(const gpe_mpm_params* params, int64_t capacity, gpe_mpm** out);

/* Several independent scenes in one engine (a batch; the reference runs one scene per arena). Scene q has its
 * own node grid of nx x ny nodes (the node array holds the scenes' grids one after the other, in the order
 * given) and its own particle clamp; the scenes share every other parameter (dx, dt, mass, materials, walls of
 * bc_width nodes along each grid's edges). Particle positions are in their scene's coordinates, and each step
 * is one set of launches over all scenes. params->nx, ny and the clamps are taken from scenes[0] and otherwise
 * unused. Emitters and publish need an engine of one scene. */
typedef struct gpe_mpm_scene {
    int32_t nx, ny;
    float clamp_lo[2], clamp_hi[2];
} gpe_mpm_scene;
int32_t gpe_mpm_create_scenes(const gpe_mpm_params* params, const gpe_mpm_scene* scenes, int32_t n_scenes,
                              int64_t capacity, gpe_mpm** out);
/* The scene of each particle, in the order gpe_mpm_set_state received them (which puts every particle in
 * scene 0): n = the particle count, ids in [0, n_scenes); GPE_ERR_BAD_ARG (and no change) otherwise. */
int32_t gpe_mpm_set_scene_ids(gpe_mpm* mpm, const int32_t* scene_id, int64_t n, int32_t mem, void* stream);
int32_t gpe_mpm_destroy(gpe_mpm* mpm);
int32_t gpe_mpm_set_params(gpe_mpm* mpm, const gpe_mpm_params* params);
/* pos, vel: n float2; C, F: n float4 row-major (xx, xy, yx, yy); J: n float (for snow it is the plastic
 * J_p); material: n int32 or NULL. Any of vel/C/F/J may be NULL (zero velocity and C, identity F, J = 1). */
int32_t gpe_mpm_set_state(gpe_mpm* mpm, const float* pos, const float* vel, const float* C, const float* F,
                          const float* J, const int32_t* material, int64_t n, int32_t mem, void* stream);
int32_t gpe_mpm_get_state(gpe_mpm* mpm, float* pos, float* vel, float* C, float* F, float* J, int64_t n,
                          int32_t mem, void* stream);
int32_t gpe_mpm_count(const gpe_mpm* mpm, int64_t* n);
/* One step = clear + P2G + grid update + G2P; consecutive steps run fused (G2P of one step with P2G of the
 * next in one launch). */
int32_t gpe_mpm_step(gpe_mpm* mpm, int32_t n_steps, void* stream);
int32_t gpe_mpm_stage(gpe_mpm* mpm, int32_t stage, void* stream);
/* Node grid of the current step: nx*ny float4 (momentum or velocity x, y; mass; unused). */
int32_t gpe_mpm_get_grid(gpe_mpm* mpm, float* dst, int64_t n_nodes, int32_t mem, void* stream);
int32_t gpe_mpm_status(gpe_mpm* mpm, uint32_t* status, void* stream);
/* Diagnostic without a counterpart in the reference (whose P2G, MPM.cu:116-126, issues one global atomic per
 * node and particle): reads and clears the number of warps whose P2G summed their particles' node
 * contributions with the 5-round segmented reduction since the last call. A P2G warp holds 64 consecutive
 * particles, two per lane; it needs 5 rounds when more than 16 consecutive lanes share the stencil base node
 * of their second particle (about 33 or more particles on one base node: scenes at about 30 particles per
 * cell). */
int32_t gpe_mpm_p2g_wide_warps(gpe_mpm* mpm, uint32_t* count, void* stream);
int32_t gpe_mpm_launches_per_step(const gpe_mpm* mpm, int32_t* launches);
/* Appends the hose's particles at the live count (MPMEmitterKernel, MPM.cu:380-438): C = 0, F = I, J = 1
 * and the engine's material; needs GPE_MPM_FLAG_DYNAMIC_COUNT. *requested receives width x rows. */
int32_t gpe_mpm_emit(gpe_mpm* mpm, const gpe_hose* hose, uint64_t seed, int32_t* requested, void* stream);
/* Copies the particles into the view in blocks of chunk_capacity consecutive particles (MPMOutputKernel,
 * MPM.cu:302-322); writes stop at the view's capacity, which the reference's kernel can overrun. view_mem as
 * for gpe_pbf_publish. */
int32_t gpe_mpm_publish(gpe_mpm* mpm, const gpe_view* view, int32_t view_mem, void* stream);
/* Issues n_steps steps on the stream without an engine-owned graph (see gpe_pbf_enqueue); the sequence
 * starts by clearing the node grids so that a captured sequence can be replayed. No spatial re-sort runs. */
int32_t gpe_mpm_enqueue(gpe_mpm* mpm, int32_t n_steps, void* stream);
/* Device pointers of the particle arrays in storage order (valid while sort_interval == 0, since a re-sort
 * moves the particles to the other buffer set) and of the device count: count[0] is the live count,
 * count[1] the count at the last publish (the reference's num_points, cuda-engine.h:206-208). Any pointer
 * argument may be NULL. */
int32_t gpe_mpm_buffers(gpe_mpm* mpm, float** pos, float** vel, float** C, float** F, float** J, int32_t** count);

#ifdef __cplusplus
}
#endif

#endif /* GPE_H */
