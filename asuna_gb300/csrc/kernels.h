// kernels.h — launch interface of the wavefront kernels.
#pragma once
#include <cuda_runtime.h>

#include "dev_types.h"

namespace asuna {

struct KParams {
  SceneDev S;
  WaveDev W;
  uint32_t depth;  // bounce being processed (1-based)
  int32_t cur;     // extend queue holding this bounce's rays (0/1)
  int32_t records; // write per-path parity records
  int32_t counters;
  uint32_t refillLanes;  // traversal: idle lanes of a warp that trigger a queue fetch
  int32_t speculate;     // traversal: postponed leaves walk on speculatively
  int32_t occupancy;     // traversal: resident blocks per SM of the kernel variant (8, 10 or 12)
  int32_t stackLimit;    // traversal: stack entries a ray may use, in [1, kStackDepth] (the host clamps it)
  int32_t blockThreads;  // traversal: threads per block (64, 128, 256; 0 = 128)
  int32_t sharedStack;   // traversal: stack entries in shared memory (16, 24, 32; 0 = 24)
};

constexpr int kTraceThreads = 128;
constexpr int kTraceMinBlocks = 8;   // resident blocks per SM the traversal kernels are compiled for
constexpr int kStackDepth = 64;      // traversal stack entries per ray
constexpr int kSharedStack = 24;     // of which in shared memory (the rest in local memory)
constexpr int kRefillLanes = 8;      // default idle lanes of a warp that trigger a queue fetch
constexpr int kShadeMinBlocks = 3;   // resident 256-thread blocks per SM the shading kernel is compiled for

void launchRaygen(const KParams& P, int grid, cudaStream_t s);
void launchShade(const KParams& P, int grid, cudaStream_t s);
// kernels launchShade issues for a scene's class mask (classify included)
int shadeLaunches(uint32_t classMask);
void launchAccumulate(const KParams& P, uint32_t maxPix, uint32_t nranges, cudaStream_t s);
// counting-sorts extend queue P.cur into queue P.cur ^ 1 (count, scan,
// scatter); mode 1: octant + 4^3 origin cells, 2: octant + 8^3 (Morton)
void launchSortQueue(const KParams& P, int mode, int grid, cudaStream_t s);
void launchRecords(const KParams& P, asuna_path_record* out, int grid, cudaStream_t s);
void launchExtend(const KParams& P, int grid, cudaStream_t s);
void launchConnect(const KParams& P, int grid, cudaStream_t s);
// resident blocks per SM of the traversal variant (occupancy class 8/10/12 =
// 32/40/48 resident warps, block size, shared-memory stack entries)
int traceBlocksPerSm(int occupancy = kTraceMinBlocks, int blockThreads = kTraceThreads,
                     int sharedStack = kSharedStack);
int shadeBlocksPerSm();

// Standalone ray queries (tests): rays are (o.xyz, tmin), (d.xyz, tmax).
void launchTraceQuery(const SceneDev& S, const float4* o, const float4* d, uint32_t n, int anyHit, float4* hit,
                      uint32_t* inst, cudaStream_t s);

}  // namespace asuna
