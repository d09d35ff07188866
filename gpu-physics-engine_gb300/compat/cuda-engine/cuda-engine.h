// cuda-engine.h — the reference's engine interface (libs/cuda-engine/include/cuda-engine/cuda-engine.h),
// implemented headless on the GB300 engine (include/gpe.h). Code written against the reference — its
// drivers main/PBF-master.cpp and main/MPM-master.cpp minus the window thread — compiles against this header
// unchanged and links libgpe_compat.so + libgpe.so.
//
// Types, members and function signatures are the reference's, because drivers use them directly
// (pbf.halo_offsets, g.stream, g.exec, ...). What differs is behind them:
//   * PBFArena / MPMArena own a gpe_pbf / gpe_mpm engine. The live particle state is the engine's
//     (scene-wide sorted arrays for PBF, flat arrays for MPM). PBFArena's chunk-major members offsets,
//     pos[0], pos[1], vel, lambda and num_atoms are written at the end of every tick with the state in the
//     reference's layout (gpe_pbf_publish_chunks): each atom in the chunk of its next prediction, chunk-local
//     coordinates, cells packed as (end << 16) | start. The migration queues and halos are allocated with the
//     reference's sizes for code that touches them; the engine has neither (one scene-wide sort replaces
//     them). MPMArena's pos/vel/C/F/J/num_points point at the engine's own arrays; num_points[0] is the live
//     count and num_points[1] the count at the last publish, set by the publish as MPMOutputKernel does
//     (MPM.cu:317).
//   * instantiate*Graph records one tick — kNumSteps PBF substeps (kSubsteps MPM substeps) and the publish
//     into the current output target — into g.graph, and instantiates g.exec, as the reference does.
//   * hosePipe appends particles on the device (gpe_*_emit) instead of going through migration queues.
//   * TickStaging uploads the output target into a device-resident view that the recorded publish reads at
//     run time, like the reference's __constant__ c_output. The torus seams must stay (0, 0), as the
//     reference's drivers keep them (main/PBF-master.cpp:48-50): torusUpload aborts with a message for any
//     other value, since the engine's scene is one walled domain and has no chunk storage to rotate.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstdio>

#include <cuda_runtime_api.h>
#include <vector_types.h>

#include "common/umbrella.h"

struct gpe_pbf;
struct gpe_mpm;

// ===== General Structs ===============================================

struct GraphEnv
{
    cudaStream_t stream   = nullptr;
    cudaGraph_t graph     = nullptr;
    cudaGraphExec_t exec  = nullptr;
    cudaEvent_t tick_done = nullptr; // cudaEventDisableTiming
    cudaEvent_t t0 = nullptr, t1 = nullptr;

    GraphEnv() = default;
    ~GraphEnv();
    GraphEnv(const GraphEnv&)            = delete;
    GraphEnv& operator=(const GraphEnv&) = delete;
};

// ===== Tick Output Objects ===========================================

// One tick's output for the renderer: chunk-major, kMaxAtoms slots per chunk, scene coordinates.
struct OutputArena
{
    float2* pos        = nullptr;
    float2* vel        = nullptr;
    int32_t* num_atoms = nullptr;

    OutputArena();
    ~OutputArena();
    OutputArena(const OutputArena&)            = delete;
    OutputArena& operator=(const OutputArena&) = delete;

  private:
    uint8_t* base = nullptr;
};

struct View
{
    float2* pos        = nullptr;
    float2* vel        = nullptr;
    int32_t* num_atoms = nullptr;
    int32_t slot       = -1;
};

// Triple buffer: the renderer reads slot i % 3 while the engine writes (i + 1) % 3.
class OutputBuffer
{
  public:
    void roll();
    View readTarget();
    View writeTarget();

    OutputBuffer()
        : read_slot(0),
          write_slot(1) {};
    OutputBuffer(const OutputBuffer&)            = delete;
    OutputBuffer& operator=(const OutputBuffer&) = delete;

  private:
    std::atomic<int32_t> read_slot;
    int32_t write_slot;
    OutputArena buffer[3]{};
};

struct TickStaging
{
    TickStaging() = default;
    ~TickStaging();

    void init(View initial_target, int2 initial_seams, cudaStream_t stream);
    View& target();
    int2& torus();
    void outputTargetUpload(cudaStream_t stream);
    void torusUpload(cudaStream_t stream);

    TickStaging(const TickStaging&)            = delete;
    TickStaging& operator=(const TickStaging&) = delete;

  private:
    struct Staged;
    Staged* staged = nullptr; // one pinned allocation
};

// ===== PBF ==========================================================

struct PBFArena
{
    uint32_t* offsets = nullptr;
    float2* pos[2]{};
    float2* vel        = nullptr;
    float* lambda      = nullptr;
    int32_t* num_atoms = nullptr;

    float2* mig_pos    = nullptr;
    float2* mig_vel    = nullptr;
    int32_t* mig_count = nullptr;

    uint32_t* halo_offsets = nullptr;
    float2* halo_pos[2]{};
    float2* halo_vel   = nullptr;
    float* halo_lambda = nullptr;

    PBFArena();
    ~PBFArena();
    PBFArena(const PBFArena&)            = delete;
    PBFArena& operator=(const PBFArena&) = delete;

    // the engine behind the arena (an addition to the reference's interface)
    gpe_pbf* engine() const { return engine_; }

  private:
    uint8_t* base    = nullptr;
    gpe_pbf* engine_ = nullptr;
};

void instantiatePBFGraph(GraphEnv& g, PBFArena& pbf);
int32_t hosePipe(const cudaStream_t stream, const PBFArena& pbf, const float2 origin, const float2 velocity,
                 const float nozzle_width, const float spacing, const float vel_jitter, const uint64_t tick);

// ===== MPM ==========================================================

struct MPMNodeHandles
{
    cudaGraphNode_t clear;
    cudaGraphNode_t output;
};

struct MPMArena
{
    float4* grid[2];
    float2* pos = nullptr;
    float2* vel = nullptr;
    float4* C   = nullptr;
    float4* F   = nullptr;
    float* J    = nullptr;
    int32_t* num_points = nullptr; // [0] the live count, [1] the count at the last publish

    MPMArena();
    ~MPMArena();
    MPMArena(const MPMArena&)            = delete;
    MPMArena& operator=(const MPMArena&) = delete;

    gpe_mpm* engine() const { return engine_; }

  private:
    gpe_mpm* engine_ = nullptr;
};

int32_t hosePipe(const cudaStream_t stream, MPMArena& mpm, const float2 origin, const float2 velocity,
                 const float nozzle_width, const float spacing, const float vel_jitter, const uint64_t tick);
void instantiateMPMGraph(GraphEnv& g_env, MPMArena& mpm);

struct MPMTickStaging
{
    MPMTickStaging() = default;
    ~MPMTickStaging();

    void init(View initial_target, int2 initial_seams, cudaStream_t stream);
    View& target();
    int2& torus();
    void outputTargetUpload(cudaStream_t stream);
    void torusUpload(cudaStream_t stream);

    MPMTickStaging(const MPMTickStaging&)            = delete;
    MPMTickStaging& operator=(const MPMTickStaging&) = delete;

  private:
    struct Staged;
    Staged* staged = nullptr;
};
