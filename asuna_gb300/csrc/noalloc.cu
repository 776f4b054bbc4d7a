// noalloc.cu — a render entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc at render time: code running while a
// memory pool or budget is locked by its owner, hosts that give the library a
// fixed device footprint up front, or render threads that must never reach
// the driver's allocator.  For them asuna_render_noalloc runs the same
// wavefront kernels as asuna_render, with all of its scratch (path-state
// queues, counters, the shot and batch records) in one file-scope device
// array of fixed size instead of per-context allocations.  The caller passes
// the inputs and outputs (a scene and a film created beforehand) and a
// stream.
//
// The array holds kNoAllocMaxPaths path slots (ASUNA_NOALLOC_MAX_PATHS =
// 262,144, 244 bytes each, about 61 MiB in all); every GPU that loads this
// library keeps it until the process exits.  A frame of more pixels than
// that is rejected with ASUNA_ERR_INVALID.
//
// The device address of the array is looked up once per device, the first
// time the entry point runs on it (cudaGetSymbolAddress with that device
// current); make that first call before any stream capture.  Every call
// shares the one array and it keeps the previous call's contents: the
// kernels reset the counters they rely on at the start of each wavefront.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads without ordering) race on the array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.h"
#include "handles.h"
#include "kernels.h"

using namespace asuna;

namespace {

constexpr uint64_t kNoAllocMaxPaths = ASUNA_NOALLOC_MAX_PATHS;
constexpr uint64_t kNoAllocMaxRanges = 64;

constexpr uint64_t pad256(uint64_t b) { return (b + 255) / 256 * 256; }
// scratch layout: per-path arrays (12 x 16 B; 4 B each for the hit
// instances and every shading-class list), counters, shot, ranges
constexpr uint64_t kPerPath16 = pad256(kNoAllocMaxPaths * 16);
constexpr uint64_t kPerPath4 = pad256(kNoAllocMaxPaths * 4);
constexpr uint64_t kOffCounters = 12 * kPerPath16 + (1 + kNumShadeClasses) * kPerPath4;
constexpr uint64_t kOffShot = kOffCounters + pad256(sizeof(DevCounters));
constexpr uint64_t kOffRanges = kOffShot + pad256(sizeof(ShotDev));
constexpr uint64_t kScratchBytes = kOffRanges + pad256(kNoAllocMaxRanges * sizeof(RangeDev));

__device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex gSetupMutex;
void* gScratchAddr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once.
int scratchAddress(int device, unsigned char** out) {
  std::lock_guard<std::mutex> lock(gSetupMutex);
  if (!gScratchAddr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess || !p)
      return fail(ASUNA_ERR_CUDA, "asuna_render_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    gScratchAddr[device] = p;
  }
  *out = static_cast<unsigned char*>(gScratchAddr[device]);
  return ASUNA_OK;
}

int renderNoAlloc(const asuna_scene* s, const asuna_shot* shot, asuna_film* film, cudaStream_t stream) {
  if (!s || !shot || !film) return fail(ASUNA_ERR_INVALID, "asuna_render_noalloc: null argument");
  if (s->device != film->device) return fail(ASUNA_ERR_INVALID, "asuna_render_noalloc: scene and film on different devices");
  if (s->device < 0 || s->device >= kMaxDevices) return fail(ASUNA_ERR_INVALID, "asuna_render_noalloc: device ordinal");
  if (shot->width != film->width || shot->height != film->height)
    return fail(ASUNA_ERR_INVALID, "asuna_render_noalloc: shot %ux%u does not match film %ux%u", shot->width,
                shot->height, film->width, film->height);
  const uint64_t npix = uint64_t(shot->width) * shot->height;
  if (npix == 0 || npix > kNoAllocMaxPaths)
    return fail(ASUNA_ERR_INVALID,
                "asuna_render_noalloc: a frame of %llu pixels exceeds the scratch maximum of %llu paths "
                "(use asuna_render)",
                (unsigned long long)npix, (unsigned long long)kNoAllocMaxPaths);
  if (shot->state.max_path_depth < 1 || shot->state.max_path_depth > 32)
    return fail(ASUNA_ERR_INVALID, "asuna_render_noalloc: max_path_depth %d outside [1, 32]",
                shot->state.max_path_depth);
  if (shot->state.n_multi_channel > ASUNA_MAX_CHANNELS)
    return fail(ASUNA_ERR_INVALID, "asuna_render_noalloc: %u channels exceed %d", shot->state.n_multi_channel,
                ASUNA_MAX_CHANNELS);
  if (shot->camera.type != ASUNA_CAMERA_PERSPECTIVE && shot->camera.type != ASUNA_CAMERA_OPENCV)
    return fail(ASUNA_ERR_UNSUPPORTED, "asuna_render_noalloc: camera type %u", shot->camera.type);
  if (shot->frames == 0) return ASUNA_OK;
  const uint64_t framesPerBatch = kNoAllocMaxPaths / npix;

  int prev = 0;
  ASUNA_CUDA_TRY(cudaGetDevice(&prev));
  if (prev != s->device) ASUNA_CUDA_TRY(cudaSetDevice(s->device));
  struct Restore {
    int dev, prev;
    ~Restore() {
      if (dev != prev) cudaSetDevice(prev);
    }
  } restore{s->device, prev};
  unsigned char* base = nullptr;
  int rc = scratchAddress(s->device, &base);
  if (rc) return rc;
  int numSMs = 0;
  ASUNA_CUDA_TRY(cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, s->device));

  KParams P{};
  P.S = s->view;
  P.refillLanes = kRefillLanes;
  P.speculate = 1;
  P.occupancy = kTraceMinBlocks;
  WaveDev& W = P.W;
  float4* f16[12];
  for (int k = 0; k < 12; ++k) f16[k] = reinterpret_cast<float4*>(base + uint64_t(k) * kPerPath16);
  W.rayO[0] = f16[0];
  W.rayO[1] = f16[1];
  W.rayD[0] = f16[2];
  W.rayD[1] = f16[3];
  W.hit = f16[4];
  W.shO = f16[5];
  W.shD = f16[6];
  W.shC = f16[7];
  W.thp = f16[8];
  W.rad = f16[9];
  W.info = reinterpret_cast<uint4*>(f16[10]);
  W.rec = reinterpret_cast<uint4*>(f16[11]);
  W.hitInst = reinterpret_cast<uint32_t*>(base + 12 * kPerPath16);
  for (int k = 0; k < kNumShadeClasses; ++k)
    W.cls[k] = reinterpret_cast<uint32_t*>(base + 12 * kPerPath16 + uint64_t(1 + k) * kPerPath4);
  W.cnt = reinterpret_cast<DevCounters*>(base + kOffCounters);
  ShotDev* dShot = reinterpret_cast<ShotDev*>(base + kOffShot);
  RangeDev* dRanges = reinterpret_cast<RangeDev*>(base + kOffRanges);
  W.shots = dShot;

  ShotDev sd;
  std::memset(&sd, 0, sizeof(sd));
  sd.cam = shot->camera;
  sd.state = shot->state;
  sd.width = shot->width;
  sd.height = shot->height;
  sd.seed = shot->seed;
  sd.flags = shot->flags;
  sd.rrDepth = shot->rr_depth;
  sd.depthSlot = shot->depth_out_channel;
  sd.filmRad = film->rad;
  sd.filmW = film->w;
  sd.filmCh = film->ch;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(dShot, &sd, sizeof(sd), cudaMemcpyHostToDevice, stream));

  // batches of whole frames, up to kNoAllocMaxRanges of them staged per upload
  const int traceGrid = numSMs * traceBlocksPerSm(), shadeGrid = numSMs * 8, raygenGrid = numSMs * 16;
  const int maxDepth = shot->state.max_path_depth;
  uint32_t f = 0;
  while (f < shot->frames) {
    RangeDev staged[kNoAllocMaxRanges];
    uint32_t nr = 0;
    for (uint32_t g = f; g < shot->frames && nr < kNoAllocMaxRanges; ++nr) {
      uint32_t k = uint32_t(std::min<uint64_t>(framesPerBatch, shot->frames - g));
      RangeDev& r = staged[nr];
      std::memset(&r, 0, sizeof(r));
      r.pathBegin = 0;
      r.shot = 0;
      r.frameBegin = shot->frame0 + g;
      r.nframes = k;
      r.npix = uint32_t(npix);
      g += k;
    }
    ASUNA_CUDA_TRY(cudaMemcpyAsync(dRanges, staged, nr * sizeof(RangeDev), cudaMemcpyHostToDevice, stream));
    for (uint32_t b = 0; b < nr; ++b) {
      W.ranges = dRanges + b;
      W.numRanges = 1;
      W.numPaths = staged[b].nframes * uint32_t(npix);
      P.cur = 0;
      P.depth = 0;
      const int rg = int(std::min<uint64_t>((W.numPaths + 255) / 256, uint64_t(raygenGrid)));
      launchRaygen(P, std::max(rg, 1), stream);
      for (int depth = 1; depth <= wavefrontPasses(maxDepth, s->view); ++depth) {
        P.depth = uint32_t(depth);
        launchExtend(P, traceGrid, stream);
        launchShade(P, shadeGrid, stream);
        launchConnect(P, traceGrid, stream);
        P.cur ^= 1;
      }
      launchAccumulate(P, uint32_t(npix), 1, stream);
      f += staged[b].nframes;
    }
    // the next group's range records overwrite dRanges: order after this group
    if (f < shot->frames) ASUNA_CUDA_TRY(cudaStreamSynchronize(stream));
  }
  ASUNA_CUDA_TRY(cudaGetLastError());
  return ASUNA_OK;
}

}  // namespace

extern "C" int asuna_render_noalloc(const asuna_scene* scene, const asuna_shot* shot, asuna_film* film,
                                    void* stream) {
  clearError();
  return renderNoAlloc(scene, shot, film, static_cast<cudaStream_t>(stream));
}
