// handles.h — the opaque handles of the C ABI (context, scene, film), shared
// by the translation units that launch the render path.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "dev_types.h"

struct WaveAlloc {
  void* base = nullptr;
  uint64_t capacity = 0;
  asuna::WaveDev view{};
};

// One captured wavefront sequence, replayed while its key (scene, buffers,
// grids, batch structure) stays the same.
struct GraphEntry {
  std::vector<uint64_t> key;
  cudaGraphExec_t exec = nullptr;
  std::vector<std::pair<int, size_t>> timed;  // (kernel kind, first event index)
  uint64_t lastUse = 0;
};

struct asuna_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int numSMs = 0;
  int traceGrid = 0, shadeGrid = 0, raygenGrid = 0;
  int traceGridShadow = 0;  // the occlusion pass's traversal grid
  int traceBlocksCap = 0;   // asuna_ctx_set_launch's traversal blocks per SM (0 = all that fit)
  asuna::DevCounters* cnt = nullptr;
  asuna::DevCounters* hostCnt = nullptr;
  WaveAlloc wave;
  uint64_t pathBudget = 4ull << 30;
  int counters = 0;
  std::vector<cudaEvent_t> events;
  // device-resident shot and batch records at stable addresses (graph replay)
  asuna::ShotDev* dShots = nullptr;
  size_t shotsCap = 0;
  asuna::RangeDev* dRanges = nullptr;
  size_t rangesCap = 0;
  int graphs = 1;
  // traversal settings of the extend [0] and connect [1] passes
  uint32_t refill[2] = {8, 8};
  int32_t speculate[2] = {1, 1};
  int32_t occupancy = 8;  // traversal kernel variant: resident 128-thread blocks per SM (8, 10, 12)
  int32_t occupancyShadow = 8;  // the same for the occlusion pass
  int32_t traceThreads = 128;  // traversal kernel variant: threads per block
  int32_t sharedStack = 24;    // traversal kernel variant: stack entries in shared memory
  int32_t raySort = 3;    // extend-queue sort mode before secondary passes (0 off)
  int32_t stackLimit = 0; // traversal stack entries a ray may use (0 = the compiled capacity)
  int32_t bvhBuild = 0;   // bottom-level BVHs: 0 built on the device, 1 on host threads
  // traversals cut short on the device: the cumulative device count is
  // copied to hostErr after every render (errEvent marks the copy); the
  // host reports each increase over errSeen as ASUNA_ERR_TRAVERSAL
  unsigned long long* hostErr = nullptr;
  cudaEvent_t errEvent = nullptr;
  bool errPending = false;
  unsigned long long errSeen = 0;
  uint64_t useClock = 0;
  std::vector<GraphEntry> gcache;
};

struct asuna_scene {
  int device = 0;
  std::vector<void*> allocs;
  asuna::SceneDev view{};
  asuna_scene_stats stats{};
};

struct asuna_film {
  int device = 0;
  uint32_t width = 0, height = 0;
  float4* rad = nullptr;
  float4* w = nullptr;
  float4* ch = nullptr;
};

