// mpm_headless — the reference's MLS-MPM driver loop (main/MPM-master.cpp:33-116) without the window thread,
// written against cuda-engine.h. Ends by checking that the last published output holds every particle, with
// finite positions inside the simulation box. Exit status 0 on success.
//   usage: mpm_headless [ticks]
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "common/umbrella.h"
#include "cuda-engine/cuda-engine.h"
#include "gpe.h"

constexpr float2 origin        = {30.f, 30.f};
constexpr float2 velocity      = {12.f, 0.f};
constexpr float nozzle_width   = 30.f;
constexpr float spacing        = 1.05f * 1.2f;
constexpr float jitter         = spacing * 0.2f;
constexpr int32_t TARGET_COUNT = 100000;

int main(int argc, char** argv)
{
    const int ticks = argc > 1 ? std::atoi(argv[1]) : 300;
    MPMArena mpm;
    OutputBuffer buff;
    GraphEnv g{};
    instantiateMPMGraph(g, mpm);
    MPMTickStaging stg;
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
        if (atoms < TARGET_COUNT) {
            atoms += hosePipe(g.stream, mpm, origin, velocity, nozzle_width, spacing, jitter, (uint64_t)tick);
        }
        CUDACHECK(cudaEventRecord(g.t0, g.stream));
        CUDACHECK(cudaGraphLaunch(g.exec, g.stream));
        CUDACHECK(cudaEventRecord(g.t1, g.stream));
        CUDACHECK(cudaEventRecord(g.tick_done, g.stream));
    }
    CUDACHECK(cudaStreamSynchronize(g.stream));

    const View out = buff.writeTarget();
    std::vector<int32_t> counts(kNumChunks);
    CUDACHECK(cudaMemcpy(counts.data(), out.num_atoms, sizeof(int32_t) * counts.size(), cudaMemcpyDeviceToHost));
    int64_t published = 0;
    for (int c = 0; c < kNumChunks; ++c) { published += counts[(size_t)c]; }
    std::vector<float2> pos((size_t)published);
    CUDACHECK(cudaMemcpy(pos.data(), out.pos, sizeof(float2) * pos.size(), cudaMemcpyDeviceToHost));
    int64_t outside = 0;
    for (const float2& p : pos) {
        const bool ok = std::isfinite(p.x) && std::isfinite(p.y) && p.x >= 0.f && p.y >= 0.f &&
                        p.x <= (float)kSimWidth && p.y <= (float)kSimHeight;
        outside += ok ? 0 : 1;
    }
    int64_t engine_n = 0;
    gpe_mpm_count(mpm.engine(), &engine_n);
    const int64_t capacity = (int64_t)kNumChunks * kMaxAtoms;
    std::printf("{\"ticks\": %d, \"requested\": %d, \"engine_particles\": %lld, \"published\": %lld, "
                "\"misplaced\": %lld, \"avg_tick_ms\": %.4f, \"longest_tick_ms\": %.4f}\n",
                ticks, atoms, (long long)engine_n, (long long)published, (long long)outside,
                ticks > 1 ? total_ms / (float)(ticks - 1) : 0.f, longest);
    const bool ok = engine_n == atoms && published == (engine_n < capacity ? engine_n : capacity) && outside == 0;
    return ok ? 0 : 1;
}
