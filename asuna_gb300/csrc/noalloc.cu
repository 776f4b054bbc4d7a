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
// shares the one array and it keeps the previous call's contents: the call
// writes its shot and batch records and clears its error count in the array
// with small kernels queued ahead of the render (their values travel as
// kernel parameters), and the kernels reset the queue counters they rely on
// at the start of each wavefront.  Calls whose work overlaps on the GPU
// (different streams, or different host threads without ordering) race on
// the array.
//
// The call waits for its work on the stream to finish, then reads the
// array's count of traversals cut short: a nonzero count is returned as
// ASUNA_ERR_TRAVERSAL.  Because it waits, it does not run on a stream that
// is being captured (ASUNA_ERR_UNSUPPORTED, before any work is queued).
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

constexpr uint64_t pad256(uint64_t b) { return (b + 255) / 256 * 256; }
// scratch layout: per-path arrays (12 x 16 B, regions 8 and 9 together
// holding the 32-byte path records; 4 B each for the hit instances and
// every shading-class list), counters, shot, the current batch's range
// record
constexpr uint64_t kPerPath16 = pad256(kNoAllocMaxPaths * 16);
constexpr uint64_t kPerPath4 = pad256(kNoAllocMaxPaths * 4);
constexpr uint64_t kOffCounters = 12 * kPerPath16 + (1 + kNumShadeClasses) * kPerPath4;
constexpr uint64_t kOffShot = kOffCounters + pad256(sizeof(DevCounters));
constexpr uint64_t kOffRanges = kOffShot + pad256(sizeof(ShotDev));
constexpr uint64_t kScratchBytes = kOffRanges + pad256(sizeof(RangeDev));

__device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

// Start of a call: the shot record, and a zero error count.
__global__ void k_noallocBegin(ShotDev* dst, ShotDev shot, DevCounters* cnt) {
  if (threadIdx.x == 0) {
    *dst = shot;
    cnt->stackOverflow = 0;
  }
}

// Start of a batch: its range record (ordered after the previous batch's
// kernels by the stream).
__global__ void k_noallocRange(RangeDev* dst, RangeDev range) {
  if (threadIdx.x == 0) *dst = range;
}

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
  cudaGetLastError();  // a non-sticky error left by the caller's own CUDA calls is not this call's failure
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  ASUNA_CUDA_TRY(cudaStreamIsCapturing(stream, &capture));
  if (capture != cudaStreamCaptureStatusNone)
    return fail(ASUNA_ERR_UNSUPPORTED,
                "asuna_render_noalloc waits for its work to finish and cannot run on a stream being captured");
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
  P.stackLimit = kStackDepth;
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
  W.path = reinterpret_cast<PathDev*>(f16[8]);  // 32 B per path: the 16-byte regions 8 and 9
  W.rad = f16[10];
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
  k_noallocBegin<<<1, 32, 0, stream>>>(dShot, sd, W.cnt);

  // batches of whole frames, each with its range record written in order
  const int traceGrid = numSMs * traceBlocksPerSm(), shadeGrid = numSMs * 8, raygenGrid = numSMs * 16;
  const int maxDepth = shot->state.max_path_depth;
  W.ranges = dRanges;
  W.numRanges = 1;
  for (uint32_t f = 0; f < shot->frames;) {
    RangeDev r;
    std::memset(&r, 0, sizeof(r));
    r.pathBegin = 0;
    r.shot = 0;
    r.frameBegin = shot->frame0 + f;
    r.nframes = uint32_t(std::min<uint64_t>(framesPerBatch, shot->frames - f));
    r.npix = uint32_t(npix);
    k_noallocRange<<<1, 32, 0, stream>>>(dRanges, r);
    W.numPaths = r.nframes * uint32_t(npix);
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
    f += r.nframes;
  }
  ASUNA_CUDA_TRY(cudaGetLastError());
  // wait for the work, then read the count of traversals cut short
  unsigned long long cut = 0;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(&cut, &W.cnt->stackOverflow, sizeof(cut), cudaMemcpyDeviceToHost, stream));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(stream));
  if (cut)
    return fail(ASUNA_ERR_TRAVERSAL,
                "asuna_render_noalloc: traversal cut short (stack full or a loop bound reached) in %llu warps or "
                "rays: the image is wrong",
                cut);
  return ASUNA_OK;
}

}  // namespace

extern "C" int asuna_render_noalloc(const asuna_scene* scene, const asuna_shot* shot, asuna_film* film,
                                    void* stream) {
  clearError();
  return renderNoAlloc(scene, shot, film, static_cast<cudaStream_t>(stream));
}
