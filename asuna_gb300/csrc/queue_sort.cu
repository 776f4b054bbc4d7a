// queue_sort.cu — reorders an extend queue so that a warp's rays travel alike.
//
// Continuation rays leave the shading kernels in the order their warps
// finished, which for diffuse bounces means random directions side by side;
// the traversal then serialises the warp over lanes that walk different
// parts of the BVH.  Before a secondary extend pass the queue is counting-
// sorted by a 9-bit key: the direction octant (which fixes the near-child
// order of every node) and a 4 x 4 x 4 cell of the origin in the scene
// bounds (mode 1), or a 12-bit key: the octant and an 8 x 8 x 8 cell in
// Morton order, so neighbouring cells stay neighbours (mode 2), or the same
// two with the origin cell major (mode 3).  The sort
// writes into the idle ping-pong queue; the pass then runs
// on that queue.  Only the order changes: every ray carries its path index,
// and closest hits break exact ties by (instance, primitive), so results do
// not depend on it.
//
//   count    per-block shared histograms folded into the global one
//   scan     one block: exclusive prefix sum -> scatter cursors; the sorted
//            queue's length; the histogram cleared for the next pass
//   scatter  per chunk of rays: shared ranks, one global reservation per key
//            and chunk, then the moves (o, d: 32 B per ray)
#include <cuda_runtime.h>

#include "kernels.h"

namespace asuna {
namespace {

constexpr int kSortThreads = 256;
constexpr int kRaysPerThread = 8;
constexpr int kChunk = kSortThreads * kRaysPerThread;  // rays per scatter block pass

// cell of one origin coordinate in [0, n) (cellScale maps the bounds to 4
// cells; NaN and out-of-bounds origins land in the edge cells)
__device__ __forceinline__ uint32_t cellOf(float v, float lo, float sc, float n) {
  const float c = (v - lo) * sc * (n * 0.25f);
  return c >= 1.0f ? uint32_t(fminf(c, n - 1.0f)) : 0u;
}
__device__ __forceinline__ uint32_t spread3(uint32_t x) {  // 3 bits -> bits 0, 3, 6
  return (x & 1u) | ((x & 2u) << 2) | ((x & 4u) << 4);
}
template <int MODE>
__device__ __forceinline__ uint32_t sortKey(const SceneDev& S, float4 o, float4 d) {
  const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
  if (MODE == 1)
    return (oct << 6) | (cellOf(o.x, S.boundLo.x, S.cellScale.x, 4.0f) << 4) |
           (cellOf(o.y, S.boundLo.y, S.cellScale.y, 4.0f) << 2) | cellOf(o.z, S.boundLo.z, S.cellScale.z, 4.0f);
  if (MODE == 3)  // origin cell (8^3, Morton) major, octant minor
    return (((spread3(cellOf(o.x, S.boundLo.x, S.cellScale.x, 8.0f)) << 2) |
             (spread3(cellOf(o.y, S.boundLo.y, S.cellScale.y, 8.0f)) << 1) |
             spread3(cellOf(o.z, S.boundLo.z, S.cellScale.z, 8.0f)))
            << 3) |
           oct;
  return (oct << 9) | (spread3(cellOf(o.x, S.boundLo.x, S.cellScale.x, 8.0f)) << 2) |
         (spread3(cellOf(o.y, S.boundLo.y, S.cellScale.y, 8.0f)) << 1) |
         spread3(cellOf(o.z, S.boundLo.z, S.cellScale.z, 8.0f));
}
template <int MODE> __host__ __device__ constexpr int keysOf() { return MODE == 1 ? 512 : 4096; }

template <int MODE>
__global__ void __launch_bounds__(kSortThreads) k_sortCount(KParams P) {
  constexpr int K = keysOf<MODE>();
  __shared__ uint32_t h[K];
  const WaveDev& W = P.W;
  for (int k = threadIdx.x; k < K; k += blockDim.x) h[k] = 0u;
  __syncthreads();
  const uint32_t n = W.cnt->c[kCntExtend0 + P.cur];
  const float4* o = W.rayO[P.cur];
  const float4* d = W.rayD[P.cur];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&h[sortKey<MODE>(P.S, __ldg(&o[i]), __ldg(&d[i]))], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    if (h[k]) atomicAdd(&W.cnt->sortHist[k], h[k]);
}

// one block of 1024 threads, kSortKeys / 1024 consecutive keys each (the
// keys a mode does not use are empty)
constexpr int kScanThreads = 1024;
constexpr int kKeysPerThread = kSortKeys / kScanThreads;
static_assert(kSortKeys % kScanThreads == 0, "scan tiling");
__global__ void __launch_bounds__(kScanThreads) k_sortScan(KParams P) {
  __shared__ uint32_t v[kScanThreads];
  const WaveDev& W = P.W;
  const int t = threadIdx.x;
  uint32_t c[kKeysPerThread], run = 0;
#pragma unroll
  for (int j = 0; j < kKeysPerThread; ++j) {
    c[j] = W.cnt->sortHist[kKeysPerThread * t + j];
    run += c[j];
  }
  v[t] = run;
  __syncthreads();
  // Hillis-Steele inclusive scan of the per-thread sums
  for (int off = 1; off < kScanThreads; off <<= 1) {
    const uint32_t add = t >= off ? v[t - off] : 0u;
    __syncthreads();
    v[t] += add;
    __syncthreads();
  }
  uint32_t start = v[t] - run;
#pragma unroll
  for (int j = 0; j < kKeysPerThread; ++j) {
    W.cnt->sortCursor[kKeysPerThread * t + j] = start;
    W.cnt->sortHist[kKeysPerThread * t + j] = 0u;
    start += c[j];
  }
  if (t == kScanThreads - 1) W.cnt->c[kCntExtend0 + (P.cur ^ 1)] = v[t];
}

template <int MODE>
__global__ void __launch_bounds__(kSortThreads) k_sortScatter(KParams P) {
  constexpr int K = keysOf<MODE>();
  __shared__ uint32_t h[K];
  __shared__ uint32_t base[K];
  const WaveDev& W = P.W;
  const uint32_t n = W.cnt->c[kCntExtend0 + P.cur];
  const float4* so = W.rayO[P.cur];
  const float4* sd = W.rayD[P.cur];
  float4* to = W.rayO[P.cur ^ 1];
  float4* td = W.rayD[P.cur ^ 1];
  for (uint32_t c0 = blockIdx.x * uint32_t(kChunk); c0 < n; c0 += gridDim.x * uint32_t(kChunk)) {
    for (int k = threadIdx.x; k < K; k += blockDim.x) h[k] = 0u;
    __syncthreads();
    float4 o[kRaysPerThread], d[kRaysPerThread];
    uint32_t key[kRaysPerThread], rank[kRaysPerThread];
#pragma unroll
    for (int j = 0; j < kRaysPerThread; ++j) {
      const uint32_t i = c0 + uint32_t(j * kSortThreads) + threadIdx.x;
      key[j] = 0xffffffffu;
      if (i < n) {
        o[j] = __ldg(&so[i]);
        d[j] = __ldg(&sd[i]);
        key[j] = sortKey<MODE>(P.S, o[j], d[j]);
        rank[j] = atomicAdd(&h[key[j]], 1u);
      }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x)
      if (h[k]) base[k] = atomicAdd(&W.cnt->sortCursor[k], h[k]);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRaysPerThread; ++j)
      if (key[j] != 0xffffffffu) {
        const uint32_t slot = base[key[j]] + rank[j];
        to[slot] = o[j];
        td[slot] = d[j];
      }
    __syncthreads();
  }
}

}  // namespace

void launchSortQueue(const KParams& P, int mode, int grid, cudaStream_t s) {
  if (mode == 1) {
    k_sortCount<1><<<grid, kSortThreads, 0, s>>>(P);
    k_sortScan<<<1, kScanThreads, 0, s>>>(P);
    k_sortScatter<1><<<grid, kSortThreads, 0, s>>>(P);
  } else if (mode == 2) {
    k_sortCount<2><<<grid, kSortThreads, 0, s>>>(P);
    k_sortScan<<<1, kScanThreads, 0, s>>>(P);
    k_sortScatter<2><<<grid, kSortThreads, 0, s>>>(P);
  } else {
    k_sortCount<3><<<grid, kSortThreads, 0, s>>>(P);
    k_sortScan<<<1, kScanThreads, 0, s>>>(P);
    k_sortScatter<3><<<grid, kSortThreads, 0, s>>>(P);
  }
}

}  // namespace asuna
