// cuda-engine.cu — the reference's engine interface (cuda-engine.h) on top of the GB300 engine's C ABI.
//
// Reference behaviour mirrored here: the arenas' allocation and lifetime (cuda-engine.cpp:14-175), the
// triple-buffered output (cuda-engine.cpp:72-98), the staged output-target upload into device memory
// (PBF.cu:37-62, MPM.cu:19-44), one graph per tick of kNumSteps PBF substeps / kSubsteps MPM substeps that
// ends by publishing into the current target (PBF.cu:901-961, MPM.cu:326-374) and the hose-pipe emitters
// (PBF.cu:1033-1065, MPM.cu:439-473). The PBF dials that the reference keeps private to PBF.cu (PBF.cu:12-23)
// are restated below with the same values; GPE_PBF_ITERS / GPE_PBF_SUBSTEPS override the first two.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "cuda-engine/cuda-engine.h"
#include "gpe.h"

#ifndef GPE_PBF_ITERS
#define GPE_PBF_ITERS 2
#endif
#ifndef GPE_PBF_SUBSTEPS
#define GPE_PBF_SUBSTEPS 20
#endif

namespace {

constexpr int32_t kIters     = GPE_PBF_ITERS;
constexpr int32_t kNumSteps  = GPE_PBF_SUBSTEPS;
constexpr float kEpsilon     = 0.005f;
constexpr float kSCorrK      = 0.005f;
constexpr float kC           = 0.035f;
constexpr float kPBF_dt      = kDt / (float)kNumSteps;
constexpr float kPBFGravity  = 1000.f;
constexpr float kGravityStep = kPBFGravity * kPBF_dt * kPBF_dt;
constexpr float kOmega       = 1.25f;
constexpr float kMinC        = -0.002f;
constexpr float kMinSpeed    = 0.00005f;
constexpr float kMaxSpeed    = 1.f;

// device-resident output targets, read by the recorded publish when the tick runs (the reference's
// __constant__ View c_output, PBF.cu:29 / MPM.cu:13) and the seam offsets (c_torus, PBF.cu:33)
__device__ gpe_view g_pbf_view;
__device__ gpe_view g_mpm_view;
__device__ int2 g_torus;

void must(int32_t rc, const char* what)
{
    if (rc != GPE_OK) {
        std::fprintf(stderr, "%s: %s %s\n", what, gpe_error_name(rc), gpe_last_error_message());
        std::abort();
    }
}

gpe_view chunk_view(const View& v)
{
    gpe_view g{};
    g.pos            = reinterpret_cast<float*>(v.pos);
    g.vel            = reinterpret_cast<float*>(v.vel);
    g.counts         = v.num_atoms;
    g.chunks_x       = kSceneDimX;
    g.chunks_y       = kSceneDimY;
    g.chunk_dim      = kChunkDim;
    g.chunk_capacity = kMaxAtoms;
    return g;
}

gpe_pbf_params pbf_params()
{
    gpe_pbf_params p{};
    p.h           = kH;
    p.cell        = (float)kCellDim;
    p.rho0        = kRho0;
    p.mass        = kMass;
    p.dt          = 1.f; // velocities are per-substep displacements (cuda-engine.h:131)
    p.gravity[0]  = 0.f;
    p.gravity[1]  = kGravityStep;
    p.iters       = kIters;
    p.eps         = kEpsilon;
    p.scorr_k     = kSCorrK;
    p.scorr_dq    = kDq;
    p.omega       = kOmega;
    p.c_min       = kMinC;
    p.xsph_c      = kC;
    p.vort_eps    = 0.f;
    p.v_max       = kMaxSpeed;
    p.v_min       = kMinSpeed;
    p.wall_margin = 1e-3f;
    p.poly6_coeff = kCoeffPoly6;
    p.spiky_coeff = kCoeffSpiky;
    p.flags       = GPE_PBF_SELF_GRAD | GPE_PBF_VEL_CLAMP | GPE_PBF_DYNAMIC_COUNT;
    return p;
}

gpe_mpm_params mpm_params()
{
    gpe_mpm_params p{};
    p.dx          = kDx;
    p.grid_offset = (float)kGridHalo;
    p.nx          = (int32_t)kGridDimX;
    p.ny          = (int32_t)kGridDimY;
    p.dt          = dt;
    p.gravity[0]  = 0.f;
    p.gravity[1]  = kGravity;
    p.mass        = kMass;
    p.vol0        = kRestVol;
    p.bc_type     = GPE_MPM_BC_SLIP;
    p.bc_width    = (int32_t)kGridHalo;
    p.clamp_lo[0] = 0.f;
    p.clamp_lo[1] = 0.f;
    p.clamp_hi[0] = (float)kSimWidth;
    p.clamp_hi[1] = (float)kSimHeight;
    p.material    = GPE_MPM_MAT_FLUID;
    p.k_bulk      = kStiffness;
    p.gamma       = kGamma;
    p.p_min       = kMinPress;
    p.p_max       = kMaxPress;
    p.J_min       = 0.1f;
    p.J_max       = 10.f;
    p.sort_interval = 0;
    p.flags       = GPE_MPM_FLAG_FLUID_F | GPE_MPM_FLAG_DYNAMIC_COUNT;
    return p;
}

size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }

void make_tick_env(GraphEnv& g)
{
    CUDACHECK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    CUDACHECK(cudaEventCreateWithFlags(&g.tick_done, cudaEventDisableTiming));
    CUDACHECK(cudaEventCreate(&g.t0));
    CUDACHECK(cudaEventCreate(&g.t1));
}

} // namespace

// ===== GraphEnv ==========================================================

GraphEnv::~GraphEnv()
{
    if (exec) { cudaGraphExecDestroy(exec); }
    if (graph) { cudaGraphDestroy(graph); }
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    if (t1) { cudaEventDestroy(t1); }
    if (t0) { cudaEventDestroy(t0); }
    if (tick_done) { cudaEventDestroy(tick_done); }
}

// ===== Output ============================================================

OutputArena::OutputArena()
{
    const size_t f2    = align128((size_t)kNumChunks * kMaxAtoms * sizeof(float2));
    const size_t ints  = align128((size_t)kNumChunks * sizeof(int32_t));
    CUDACHECK(cudaMalloc((void**)&base, 2 * f2 + ints));
    CUDACHECK(cudaMemset(base, 0, 2 * f2 + ints));
    pos       = reinterpret_cast<float2*>(base);
    vel       = reinterpret_cast<float2*>(base + f2);
    num_atoms = reinterpret_cast<int32_t*>(base + 2 * f2);
}

OutputArena::~OutputArena()
{
    if (base) { cudaFree(base); }
}

void OutputBuffer::roll()
{
    read_slot.store(write_slot, std::memory_order_release);
    write_slot = (write_slot + 1) % 3;
}

View OutputBuffer::readTarget()
{
    const int32_t s = read_slot.load(std::memory_order_acquire);
    return View{buffer[s].pos, buffer[s].vel, buffer[s].num_atoms, s};
}

View OutputBuffer::writeTarget()
{
    const int32_t s = write_slot;
    return View{buffer[s].pos, buffer[s].vel, buffer[s].num_atoms, s};
}

// ===== TickStaging =======================================================

struct TickStaging::Staged
{
    View target;
    int2 torus;
    gpe_view device_view; // what outputTargetUpload copies to the device
};

TickStaging::~TickStaging()
{
    if (staged) { cudaFreeHost(staged); }
}

void TickStaging::init(View initial_target, int2 initial_seams, cudaStream_t stream)
{
    CUDACHECK(cudaMallocHost((void**)&staged, sizeof(Staged)));
    staged->target = initial_target;
    staged->torus  = initial_seams;
    outputTargetUpload(stream);
    torusUpload(stream);
}

View& TickStaging::target() { return staged->target; }
int2& TickStaging::torus() { return staged->torus; }

void TickStaging::outputTargetUpload(cudaStream_t stream)
{
    staged->device_view = chunk_view(staged->target);
    CUDACHECK(cudaMemcpyToSymbolAsync(g_pbf_view, &staged->device_view, sizeof(gpe_view), 0, cudaMemcpyHostToDevice,
                                      stream));
}

// Seams other than (0, 0) would rotate the chunk storage of a streaming world (PBF-internal.cuh:307-347);
// the engine's scene is one walled domain stored by position, so a moved seam is refused instead of being
// silently ignored.
void require_no_seam(const int2& t)
{
    if (t.x != 0 || t.y != 0) {
        std::fprintf(stderr, "torusUpload: seams (%d, %d) are not supported: the engine simulates one walled scene "
                             "(seams must stay at (0, 0))\n", t.x, t.y);
        std::abort();
    }
}

void TickStaging::torusUpload(cudaStream_t stream)
{
    require_no_seam(staged->torus);
    CUDACHECK(cudaMemcpyToSymbolAsync(g_torus, &staged->torus, sizeof(int2), 0, cudaMemcpyHostToDevice, stream));
}

struct MPMTickStaging::Staged
{
    View target;
    int2 torus;
    gpe_view device_view;
};

MPMTickStaging::~MPMTickStaging()
{
    if (staged) { cudaFreeHost(staged); }
}

void MPMTickStaging::init(View initial_target, int2 initial_seams, cudaStream_t stream)
{
    CUDACHECK(cudaMallocHost((void**)&staged, sizeof(Staged)));
    staged->target = initial_target;
    staged->torus  = initial_seams;
    outputTargetUpload(stream);
    torusUpload(stream);
}

View& MPMTickStaging::target() { return staged->target; }
int2& MPMTickStaging::torus() { return staged->torus; }

void MPMTickStaging::outputTargetUpload(cudaStream_t stream)
{
    staged->device_view = chunk_view(staged->target);
    CUDACHECK(cudaMemcpyToSymbolAsync(g_mpm_view, &staged->device_view, sizeof(gpe_view), 0, cudaMemcpyHostToDevice,
                                      stream));
}

void MPMTickStaging::torusUpload(cudaStream_t stream)
{
    require_no_seam(staged->torus);
    CUDACHECK(cudaMemcpyToSymbolAsync(g_torus, &staged->torus, sizeof(int2), 0, cudaMemcpyHostToDevice, stream));
}

// ===== PBF ===============================================================

PBFArena::PBFArena()
{
    // the reference's arena (cuda-engine.cpp:102-139): the chunk-major state is written at the end of every
    // tick; the migration queues and halos are allocated for code that touches them (the engine has neither)
    const size_t offs   = align128((size_t)kNumChunks * kCellsPerChunk * sizeof(uint32_t));
    const size_t inner2 = align128((size_t)kNumChunks * kMaxAtoms * sizeof(float2));
    const size_t inner1 = align128((size_t)kNumChunks * kMaxAtoms * sizeof(float));
    const size_t counts = align128((size_t)kNumChunks * sizeof(int32_t));
    const size_t ext    = (size_t)(kSceneDimX + 2) * (kSceneDimY + 2);
    const size_t mig2   = align128(ext * kMaxMigrants * sizeof(float2));
    const size_t migc   = align128(ext * sizeof(int32_t));
    const size_t hoffs  = align128((size_t)kNumChunks * kHaloCells * sizeof(uint32_t));
    const size_t halo2  = align128((size_t)kNumChunks * kHaloAtoms * sizeof(float2));
    const size_t halo1  = align128((size_t)kNumChunks * kHaloAtoms * sizeof(float));
    const size_t total  = offs + 3 * inner2 + inner1 + counts + 2 * mig2 + migc + hoffs + 3 * halo2 + halo1;
    CUDACHECK(cudaMalloc((void**)&base, total));
    CUDACHECK(cudaMemset(base, 0, total));
    uint8_t* p   = base;
    auto take    = [&p](size_t b) { uint8_t* r = p; p += b; return r; };
    offsets      = reinterpret_cast<uint32_t*>(take(offs));
    pos[0]       = reinterpret_cast<float2*>(take(inner2));
    pos[1]       = reinterpret_cast<float2*>(take(inner2));
    vel          = reinterpret_cast<float2*>(take(inner2));
    lambda       = reinterpret_cast<float*>(take(inner1));
    num_atoms    = reinterpret_cast<int32_t*>(take(counts));
    mig_pos      = reinterpret_cast<float2*>(take(mig2));
    mig_vel      = reinterpret_cast<float2*>(take(mig2));
    mig_count    = reinterpret_cast<int32_t*>(take(migc));
    halo_offsets = reinterpret_cast<uint32_t*>(take(hoffs));
    halo_pos[0]  = reinterpret_cast<float2*>(take(halo2));
    halo_pos[1]  = reinterpret_cast<float2*>(take(halo2));
    halo_vel     = reinterpret_cast<float2*>(take(halo2));
    halo_lambda  = reinterpret_cast<float*>(take(halo1));

    const gpe_pbf_params prm = pbf_params();
    gpe_domain scene{};
    scene.extent[0] = (float)kSceneDimX * kChunkDim;
    scene.extent[1] = (float)kSceneDimY * kChunkDim;
    must(gpe_pbf_create(&prm, &scene, 1, (int64_t)kNumChunks * kMaxAtoms, &engine_), "gpe_pbf_create");
    must(gpe_pbf_set_state(engine_, nullptr, nullptr, nullptr, 0, GPE_MEM_HOST, nullptr), "gpe_pbf_set_state");
}

PBFArena::~PBFArena()
{
    if (engine_) { gpe_pbf_destroy(engine_); }
    if (base) { cudaFree(base); }
}

void instantiatePBFGraph(GraphEnv& g, PBFArena& pbf)
{
    make_tick_env(g);
    gpe_view* target = nullptr;
    CUDACHECK(cudaGetSymbolAddress((void**)&target, g_pbf_view));
    // the arena's chunk-major members mirror the engine's state at the end of every tick, as the reference's
    // arena holds it after its last substep's prepNextSubstepKernel (PBF.cu:786-833)
    gpe_chunk_state arena{};
    arena.pos            = reinterpret_cast<float*>(pbf.pos[0]);
    arena.pred           = reinterpret_cast<float*>(pbf.pos[1]);
    arena.vel            = reinterpret_cast<float*>(pbf.vel);
    arena.lambda         = pbf.lambda;
    arena.counts         = pbf.num_atoms;
    arena.offsets        = pbf.offsets;
    arena.chunks_x       = kSceneDimX;
    arena.chunks_y       = kSceneDimY;
    arena.chunk_cells    = kGridDim;
    arena.chunk_dim      = kChunkDim;
    arena.chunk_capacity = kMaxAtoms;
    CUDACHECK(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
    must(gpe_pbf_enqueue(pbf.engine(), kNumSteps, g.stream), "gpe_pbf_enqueue");
    must(gpe_pbf_publish(pbf.engine(), target, GPE_MEM_DEVICE, g.stream), "gpe_pbf_publish");
    must(gpe_pbf_publish_chunks(pbf.engine(), &arena, g.stream), "gpe_pbf_publish_chunks");
    CUDACHECK(cudaStreamEndCapture(g.stream, &g.graph));
    CUDACHECK(cudaGraphInstantiate(&g.exec, g.graph, 0));
}

int32_t hosePipe(const cudaStream_t stream, const PBFArena& pbf, const float2 origin, const float2 velocity,
                 const float nozzle_width, const float spacing, const float vel_jitter, const uint64_t tick)
{
    gpe_hose h{};
    h.origin[0]      = origin.x;
    h.origin[1]      = origin.y;
    h.velocity[0]    = velocity.x; // per-substep displacement, as the reference's emitter takes it
    h.velocity[1]    = velocity.y;
    h.nozzle_width   = nozzle_width;
    h.spacing        = spacing;
    h.jitter         = vel_jitter;
    h.steps_per_call = kNumSteps;
    int32_t count    = 0;
    must(gpe_pbf_emit(pbf.engine(), &h, tick, &count, stream), "gpe_pbf_emit");
    return count;
}

// ===== MPM ===============================================================

MPMArena::MPMArena()
{
    const gpe_mpm_params prm = mpm_params();
    must(gpe_mpm_create(&prm, kNumAtoms, &engine_), "gpe_mpm_create");
    must(gpe_mpm_set_state(engine_, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, GPE_MEM_HOST, nullptr),
         "gpe_mpm_set_state");
    float *p = nullptr, *v = nullptr, *c = nullptr, *f = nullptr, *j = nullptr;
    must(gpe_mpm_buffers(engine_, &p, &v, &c, &f, &j, &num_points), "gpe_mpm_buffers");
    pos     = reinterpret_cast<float2*>(p);
    vel     = reinterpret_cast<float2*>(v);
    C       = reinterpret_cast<float4*>(c);
    F       = reinterpret_cast<float4*>(f);
    J       = j;
    grid[0] = nullptr; // the engine's node grids are internal (three of them, rotated within a tick)
    grid[1] = nullptr;
}

MPMArena::~MPMArena()
{
    if (engine_) { gpe_mpm_destroy(engine_); }
}

int32_t hosePipe(const cudaStream_t stream, MPMArena& mpm, const float2 origin, const float2 velocity,
                 const float nozzle_width, const float spacing, const float vel_jitter, const uint64_t tick)
{
    gpe_hose h{};
    h.origin[0]      = origin.x;
    h.origin[1]      = origin.y;
    h.velocity[0]    = velocity.x / kDt; // the reference's MPM emitter turns the per-tick velocity into units/s
    h.velocity[1]    = velocity.y / kDt;
    h.nozzle_width   = nozzle_width;
    h.spacing        = spacing;
    h.jitter         = vel_jitter;
    h.steps_per_call = kSubsteps;
    int32_t count    = 0;
    must(gpe_mpm_emit(mpm.engine(), &h, tick, &count, stream), "gpe_mpm_emit");
    return count;
}

void instantiateMPMGraph(GraphEnv& g, MPMArena& mpm)
{
    make_tick_env(g);
    gpe_view* target = nullptr;
    CUDACHECK(cudaGetSymbolAddress((void**)&target, g_mpm_view));
    CUDACHECK(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
    must(gpe_mpm_enqueue(mpm.engine(), kSubsteps, g.stream), "gpe_mpm_enqueue");
    must(gpe_mpm_publish(mpm.engine(), target, GPE_MEM_DEVICE, g.stream), "gpe_mpm_publish");
    CUDACHECK(cudaStreamEndCapture(g.stream, &g.graph));
    CUDACHECK(cudaGraphInstantiate(&g.exec, g.graph, 0));
}
