// pbf_headless — the reference's PBF driver loop (main/PBF-master.cpp:33-122) without the window thread,
// written against cuda-engine.h: emit with the hose pipe until TARGET_COUNT atoms, launch one tick graph per
// iteration, roll the triple-buffered output and report the tick times. Ends by checking that the last
// published output holds every atom of the engine, inside the scene, and that the arena's own chunk-major
// members hold them too, each in the chunk and cell of its prediction. Exit status 0 on success.
//   usage: pbf_headless [ticks]
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
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
    // the arena's own members after the last tick: every atom in the chunk and cell of its prediction pos[1]
    // (chunk-local), per cell the packed range (end << 16) | start, and x* - x the displacement vel + gravity
    std::vector<int32_t> na(kNumChunks);
    std::vector<uint32_t> offs((size_t)kNumChunks * kCellsPerChunk);
    std::vector<float2> p0((size_t)kNumChunks * kMaxAtoms), p1(p0.size()), v0(p0.size());
    CUDACHECK(cudaMemcpy(na.data(), pbf.num_atoms, sizeof(int32_t) * na.size(), cudaMemcpyDeviceToHost));
    CUDACHECK(cudaMemcpy(offs.data(), pbf.offsets, sizeof(uint32_t) * offs.size(), cudaMemcpyDeviceToHost));
    CUDACHECK(cudaMemcpy(p0.data(), pbf.pos[0], sizeof(float2) * p0.size(), cudaMemcpyDeviceToHost));
    CUDACHECK(cudaMemcpy(p1.data(), pbf.pos[1], sizeof(float2) * p1.size(), cudaMemcpyDeviceToHost));
    CUDACHECK(cudaMemcpy(v0.data(), pbf.vel, sizeof(float2) * v0.size(), cudaMemcpyDeviceToHost));
    int64_t arena_atoms = 0, arena_bad = 0;
    for (int c = 0; c < kNumChunks; ++c) {
        arena_atoms += na[(size_t)c];
        uint32_t expect = 0;
        for (int cell = 0; cell < kCellsPerChunk; ++cell) {
            const uint32_t o = offs[(size_t)c * kCellsPerChunk + cell], st = o & 0xFFFFu, en = o >> 16;
            arena_bad += (st != expect || en < st) ? 1 : 0;
            expect = en;
            for (uint32_t a = st; a < en && a < (uint32_t)kMaxAtoms; ++a) {
                const size_t q = (size_t)c * kMaxAtoms + a;
                const int gx   = std::min(std::max((int)std::floor(p1[q].x) / kCellDim, 0), kGridDim - 1);
                const int gy   = std::min(std::max((int)std::floor(p1[q].y) / kCellDim, 0), kGridDim - 1);
                const float dx = p1[q].x - p0[q].x - v0[q].x, dy = p1[q].y - p0[q].y - v0[q].y;
                arena_bad += (gx + gy * kGridDim != cell || std::fabs(dx) > 1e-3f || std::fabs(dy) > 1e-2f) ? 1 : 0;
            }
        }
        arena_bad += expect != (uint32_t)na[(size_t)c] ? 1 : 0;
    }
    uint32_t status = 0;
    gpe_pbf_status(pbf.engine(), &status, nullptr);
    std::printf("{\"ticks\": %d, \"requested\": %d, \"engine_atoms\": %lld, \"published\": %lld, \"misplaced\": %lld, "
                "\"arena_atoms\": %lld, \"arena_inconsistent\": %lld, "
                "\"status\": %u, \"avg_tick_ms\": %.4f, \"longest_tick_ms\": %.4f}\n",
                ticks, atoms, (long long)engine_n, (long long)published, (long long)outside, (long long)arena_atoms,
                (long long)arena_bad, status, ticks > 1 ? total_ms / (float)(ticks - 1) : 0.f, longest);
    const bool ok = engine_n > 0 && published == engine_n && outside == 0 && engine_n <= atoms && status == 0 &&
                    arena_atoms == engine_n && arena_bad == 0;
    return ok ? 0 : 1;
}
