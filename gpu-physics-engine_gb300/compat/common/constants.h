// common/constants.h of the headless engine: the configuration constants that code written against the
// reference's interface compiles with (the reference's libs/common/include/common/constants.h). The names
// are fixed by that interface and the values are the reference's, except that the scene size in chunks
// (GPE_REF_SCENE_X/Y), the migration queue depth (GPE_REF_MAX_MIGRANTS) and the MPM particle capacity
// (GPE_REF_MPM_ATOMS) can be set with -D. The compat layer (cuda-engine.h) sizes its arenas and its output
// views from them, and the parity tests compile the reference's own kernels against the same file.
#pragma once
#include <chrono>
#include <stddef.h>
#include <stdint.h>

#ifndef GPE_REF_SCENE_X
#define GPE_REF_SCENE_X 12
#endif
#ifndef GPE_REF_SCENE_Y
#define GPE_REF_SCENE_Y 6
#endif
#ifndef GPE_REF_MAX_MIGRANTS
#define GPE_REF_MAX_MIGRANTS 320
#endif
#ifndef GPE_REF_MPM_ATOMS
#define GPE_REF_MPM_ATOMS (400 * 1000)
#endif

// scene and launch shape
constexpr int32_t kSceneDimX = GPE_REF_SCENE_X;
constexpr int32_t kSceneDimY = GPE_REF_SCENE_Y;
constexpr size_t kCudaBlockX = 32;
constexpr size_t kCudaBlockY = 8;
constexpr size_t kCudaGridX  = 6;
constexpr size_t kCudaGridY  = 6;

// time and shared physics
constexpr auto kTickPeriod = std::chrono::milliseconds(32);
constexpr float kDt        = std::chrono::duration<float>(kTickPeriod).count();
constexpr float kGravity   = 700.f;
constexpr float kMass      = 1.f;
constexpr float kInvMass   = 1.f / kMass;
constexpr float kPi        = 3.14159f;

// PBF kernels and chunk structure
constexpr float kH          = 2.f;
constexpr float kRho0       = 1.015f;
constexpr float kInvRho0    = 1.f / kRho0;
constexpr float kCoeffPoly6 = 1.f / (64.f * kPi);
constexpr float kCoeffSpiky = 30.f / (32.f * kPi);
constexpr float kDq         = 0.2f * kH;
constexpr float kInvPoly6Dq =
    1.f / (kCoeffPoly6 * (kH * kH - kDq * kDq) * (kH * kH - kDq * kDq) * (kH * kH - kDq * kDq));
constexpr int32_t kGridDim       = 16;
constexpr int32_t kCellDim       = 2;
constexpr int32_t kCellSlots     = 8;
constexpr float kChunkDim        = 32.f;
constexpr int32_t kNumChunks     = kSceneDimX * kSceneDimY;
constexpr int32_t kMaxAtoms      = 128 * 12;
constexpr int32_t kMaxMigrants   = GPE_REF_MAX_MIGRANTS;
constexpr int32_t kCellsPerChunk = kGridDim * kGridDim;
constexpr int32_t kHaloCells     = 4 * kGridDim + 4;
constexpr int32_t kHaloAtoms     = kHaloCells * kCellSlots;

// Renderer (the splat rasteriser's image: kSimScale pixels per scene unit)
constexpr float kSimScale    = 5.f;
constexpr size_t kDispWidth  = (size_t)((float)kSceneDimX * kChunkDim * kSimScale);
constexpr size_t kDispHeight = (size_t)((float)kSceneDimY * kChunkDim * kSimScale);

// MLS-MPM
constexpr int32_t kSubsteps   = 20;
constexpr size_t kSimWidth    = (size_t)(kSceneDimX * (int32_t)kChunkDim);
constexpr size_t kSimHeight   = (size_t)(kSceneDimY * (int32_t)kChunkDim);
constexpr size_t kGridHalo    = 2;
constexpr size_t kGridCellDim = 2;
constexpr size_t kGridDimX    = (kSimWidth / kGridCellDim) + kGridHalo * 2;
constexpr size_t kGridDimY    = (kSimHeight / kGridCellDim) + kGridHalo * 2;
constexpr float kDx           = (float)kGridCellDim;
constexpr float inv_dx        = 1.f / kDx;
constexpr float kRestVol      = 1.2f;
constexpr int32_t kNumAtoms   = GPE_REF_MPM_ATOMS;
constexpr float kStiffness    = 8.2e4f;
constexpr float kGamma        = 3.2f;
constexpr float kMinPress     = -0.f * kStiffness;
constexpr float kMaxPress     = 10.f * kStiffness;
constexpr float dt            = kDt / kSubsteps;
