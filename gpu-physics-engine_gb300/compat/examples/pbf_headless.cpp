// pbf_headless — the reference's PBF driver loop (main/PBF-master.cpp:33-122) without the window thread,
// written against cuda-engine.h: emit with the hose pipe until TARGET_COUNT atoms, launch one tick graph per
// iteration, roll the triple-buffered output and report the tick times. Ends by checking that the last
// published output holds every atom of the engine, inside the scene. Exit status 0 on success.
//   usage: pbf_headless [ticks]
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "common/umbrella.h"
#include "cuda-engine/cuda-engine.h"
#include "gpe.h"

constexpr float2 origin        = {(float)kSceneDimX * float(kChunkDim) / 3.f, kChunkDim * 2.f};
constexpr float2 velocity      = {1.f, -0.3f};
constexpr float nozzle_width   = 8.f;
constexpr float spacing        = 1.05f * 1.f;
constexpr float jitter         = spacing * 0.05f;
constexpr int32_t TARGET_COUNT = 40000;

int main(int argc, char** argv)
{
    const int ticks = argc > 1 ? std::atoi(argv[1]) : 300;
    PBFArena pbf;
    OutputBuffer buff;
    GraphEnv g{};
    instantiatePBFGraph(g, pbf);
    TickStaging stg;
    stg.init(buff.writeTarget(), int2{0, 0}, g.stream);

    int32_t atoms = 0;
    float total_ms = 0.f, longest = 0.f;
    for (int tick = 0; tick < ticks; ++tick) {
        if (tick > 0) {
            CUDACHECK(cudaEventSynchronize(g.tick_done));
            buff.roll();
            stg.target() = buff.writeTarget();
            stg.outputTargetUpload(g.stream);
            float ms = 0.f;
            CUDACHECK(cudaEventElapsedTime(&ms, g.t0, g.t1));
            total_ms += ms;
            longest = ms > longest ? ms : longest;
        }
        CUDACHECK(cudaMemsetAsync(pbf.halo_offsets, 0, (size_t)kNumChunks * kHaloCells * sizeof(uint32_t), g.stream));
        if (atoms < TARGET_COUNT) {
            atoms += hosePipe(g.stream, pbf, origin, velocity, nozzle_width, spacing, jitter, (uint64_t)tick);
        }
        CUDACHECK(cudaEventRecord(g.t0, g.stream));
        CUDACHECK(cudaGraphLaunch(g.exec, g.stream));
        CUDACHECK(cudaEventRecord(g.t1, g.stream));
        CUDACHECK(cudaEventRecord(g.tick_done, g.stream));
    }
    CUDACHECK(cudaStreamSynchronize(g.stream));

    // the last tick published into the current write target
    const View out = buff.writeTarget();
    std::vector<int32_t> counts(kNumChunks);
    std::vector<float2> pos((size_t)kNumChunks * kMaxAtoms);
    CUDACHECK(cudaMemcpy(counts.data(), out.num_atoms, sizeof(int32_t) * counts.size(), cudaMemcpyDeviceToHost));
    CUDACHECK(cudaMemcpy(pos.data(), out.pos, sizeof(float2) * pos.size(), cudaMemcpyDeviceToHost));
    int64_t engine_n = 0;
    gpe_pbf_count(pbf.engine(), &engine_n);
    int64_t published = 0, outside = 0;
    for (int c = 0; c < kNumChunks; ++c) {
        published += counts[(size_t)c];
        const float cx = (float)(c % kSceneDimX) * kChunkDim, cy = (float)(c / kSceneDimX) * kChunkDim;
        for (int a = 0; a < counts[(size_t)c]; ++a) {
            const float2 p = pos[(size_t)c * kMaxAtoms + a];
            const bool ok  = std::isfinite(p.x) && std::isfinite(p.y) && p.x >= cx - 1e-3f &&
                            p.x <= cx + kChunkDim + 1e-3f && p.y >= cy - 1e-3f && p.y <= cy + kChunkDim + 1e-3f;
            outside += ok ? 0 : 1;
        }
    }
    uint32_t status = 0;
    gpe_pbf_status(pbf.engine(), &status, nullptr);
    std::printf("{\"ticks\": %d, \"requested\": %d, \"engine_atoms\": %lld, \"published\": %lld, \"misplaced\": %lld, "
                "\"status\": %u, \"avg_tick_ms\": %.4f, \"longest_tick_ms\": %.4f}\n",
                ticks, atoms, (long long)engine_n, (long long)published, (long long)outside, status,
                ticks > 1 ? total_ms / (float)(ticks - 1) : 0.f, longest);
    const bool ok = engine_n > 0 && published == engine_n && outside == 0 && engine_n <= atoms && status == 0;
    return ok ? 0 : 1;
}
