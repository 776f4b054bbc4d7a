// bvh_device.cu — bottom-level acceleration structures built on the GPU.
//
// Replaces the driver's BLAS builds of PipelineRaytrace::createBottomLevelAS
// (src/pipeline/pipeline_raytrace.cpp:107-147) with the same binned
// surface-area-heuristic algorithm as the host builder (bvh_build.cpp): 32
// bins per axis over the centroid bounds, cost 1 + (A_L N_L + A_R N_R) / A,
// leaves of at most 4 triangles made where the SAH prefers them, index
// halving where all centroids coincide or past depth 40, child boxes widened
// by a relative 2^-20.  The output is the traversal's layout: 64-byte
// BvhNode (child boxes + refs), leaves as (first, count) ranges of 48-byte
// TriDev records in leaf order.  Every mesh is built at once.
//
// Two phases:
//  * large tasks (more than kSmallTask primitives) level by level: blocks
//    bin chunks of a task's primitives into shared memory and merge into the
//    task's global bins; one warp per task picks the split; blocks partition
//    their chunks into the other order buffer (one reservation per block);
//  * small tasks: one warp builds a task's whole subtree depth first with its
//    bins and task stack in shared memory, allocating nodes from 64-node
//    chunks so a subtree's nodes stay together.
// Float bounds are accumulated with integer atomics on order-preserving
// keys.  Every loop is bounded by its range; a warp whose task stack would
// overflow stops and reports it (the build fails, nothing is left running).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

#include "bvh_device.h"
#include "common.h"

namespace asuna {
namespace {

constexpr int kBins = 32;
constexpr int kBinWords = 13;  // lo xyz, hi xyz, centroid lo xyz, centroid hi xyz, count (keys)
constexpr int kTaskBinWords = 3 * kBins * kBinWords;
constexpr uint32_t kSmallTask = 2048;   // primitives: at most this many -> one warp builds the subtree
constexpr uint32_t kChunk = 4096;       // primitives per block in the large-task kernels
constexpr uint32_t kMedianDepth = 40;   // past this depth: halve by index (depth stays bounded)
constexpr int kMaxLeaf = 4;
constexpr int kWarpStack = 60;          // pending subtasks of one warp's depth-first build
constexpr uint32_t kNodeChunk = 64;
constexpr int kSmallWarps = 4;          // warps per block in the small-task kernel

// order-preserving float <-> uint keys (atomicMin/atomicMax on floats);
// empty bounds start at the keys of +FLT_MAX (minima) and -FLT_MAX (maxima)
constexpr uint32_t kKeyLoInit = 0xff7fffffu, kKeyHiInit = 0x00800000u;
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float funkey(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

struct BTask {
  uint32_t begin, end;  // positions in the order arrays
  int32_t node;         // root task: its node; else the parent whose slot it fills
  uint32_t flags;       // bit 0 side, bit 1 root, bit 2 buffer holding the range, depth << 8
  float blo[3], bhi[3];  // box of the primitives
  float clo[3], chi[3];  // box of their centroids
};
static_assert(sizeof(BTask) == 64, "BTask is 64 bytes");

__host__ __device__ inline uint32_t taskDepth(const BTask& t) { return t.flags >> 8; }
__host__ __device__ inline uint32_t taskBuf(const BTask& t) { return (t.flags >> 2) & 1u; }

// Split decided for a large task.
struct BSplit {
  int32_t kind;  // 0 leaf, 1 bins, 2 index halving
  int32_t axis, bin;
  uint32_t nL;
  int32_t node;  // the inner node the task became
  float lo, scale;  // bin mapping on the split axis
  BTask left, right;
};

struct BuildCtx {
  const float4* pbox;  // 2 per primitive: lo, hi
  const float4* cen;
  uint32_t* ord[2];
  uint32_t* ordFinal;
  BvhNode* nodes;
  uint32_t nodeCap;
  uint32_t* counters;  // [0] nodes used, [1] max depth, [2] error, [3] next-level large tasks, [4] small tasks
  BTask* nextLarge;
  uint32_t nextLargeCap;
  BTask* small;
  uint32_t smallCap;
};
enum { kCtrNodes = 0, kCtrDepth = 1, kCtrError = 2, kCtrNextLarge = 3, kCtrSmall = 4, kCtrSmallNext = 5, kCtrNum = 8 };
enum { kErrNodes = 1, kErrStack = 2, kErrTasks = 4 };

__device__ __forceinline__ float boxArea(float lx, float ly, float lz, float hx, float hy, float hz) {
  const float dx = hx - lx, dy = hy - ly, dz = hz - lz;
  if (dx < 0.0f || dy < 0.0f || dz < 0.0f) return 0.0f;
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__device__ __forceinline__ void widen(float& lo, float& hi) {
  const float e = fmaxf(fabsf(lo), fabsf(hi)) * 9.5367431640625e-07f + 1e-30f;
  lo -= e;
  hi += e;
}

// Writes child slot `side` of node `n`: the widened box and the reference.
__device__ __forceinline__ void setChild(BvhNode* n, int side, const float* blo, const float* bhi, int32_t ref) {
  float lo[3] = {blo[0], blo[1], blo[2]}, hi[3] = {bhi[0], bhi[1], bhi[2]};
  for (int k = 0; k < 3; ++k) widen(lo[k], hi[k]);
  nodeSetBox(*n, side, lo, hi);
  (side == 0 ? n->ref.x : n->ref.y) = ref;
}

__host__ __device__ __forceinline__ bool isMinWord(int w) { return w < 3 || (w >= 6 && w < 9); }
__host__ __device__ __forceinline__ uint32_t initWord(int w) {
  return w == kBinWords - 1 ? 0u : isMinWord(w) ? kKeyLoInit : kKeyHiInit;
}

__device__ __forceinline__ void clearBins(uint32_t* bins, int lane, int nlanes) {
  for (int i = lane; i < kTaskBinWords; i += nlanes) bins[i] = initWord(i % kBinWords);
}

// Bin of a centroid coordinate: the host builder's int((c - lo) * scale), clamped.
__device__ __forceinline__ int binOf(float c, float lo, float scale) {
  int k = int((c - lo) * scale);
  return min(max(k, 0), kBins - 1);
}

// Adds primitive p to the task's bins (axes with a non-empty centroid extent).
__device__ __forceinline__ void binPrim(uint32_t* bins, const BuildCtx& C, uint32_t p, const float* clo,
                                        const float* scale) {
  const float4 c = __ldg(&C.cen[p]);
  const float4 lo = __ldg(&C.pbox[2 * size_t(p)]), hi = __ldg(&C.pbox[2 * size_t(p) + 1]);
  const float cc[3] = {c.x, c.y, c.z};
  const uint32_t kl[3] = {fkey(lo.x), fkey(lo.y), fkey(lo.z)}, kh[3] = {fkey(hi.x), fkey(hi.y), fkey(hi.z)};
  const uint32_t kc[3] = {fkey(c.x), fkey(c.y), fkey(c.z)};
  for (int ax = 0; ax < 3; ++ax) {
    if (!(scale[ax] > 0.0f)) continue;
    uint32_t* b = bins + (ax * kBins + binOf(cc[ax], clo[ax], scale[ax])) * kBinWords;
    for (int k = 0; k < 3; ++k) {
      atomicMin(&b[k], kl[k]);
      atomicMax(&b[3 + k], kh[k]);
      atomicMin(&b[6 + k], kc[k]);
      atomicMax(&b[9 + k], kc[k]);
    }
    atomicAdd(&b[12], 1u);
  }
}

__device__ __forceinline__ void binScales(const BTask& t, float* scale) {
  for (int ax = 0; ax < 3; ++ax) {
    const float ext = t.chi[ax] - t.clo[ax];
    scale[ax] = ext > 0.0f ? float(kBins) / ext : 0.0f;
  }
}

// Warp-wide split decision over a task's bins (lane k holds bin k).  Returns
// kind 0 leaf / 1 bins / 2 index halving with the children's boxes and
// counts, as the host builder decides (first minimum over axes, then bins).
__device__ BSplit decideSplit(const uint32_t* bins, const BTask& t, int lane) {
  BSplit s;
  s.kind = 0;
  s.axis = -1;
  s.bin = -1;
  s.nL = 0;
  s.node = -1;
  s.lo = 0.0f;
  s.scale = 0.0f;
  const uint32_t n = t.end - t.begin;
  const uint32_t depth = taskDepth(t);
  float scale[3];
  binScales(t, scale);
  const bool anyExt = scale[0] > 0.0f || scale[1] > 0.0f || scale[2] > 0.0f;
  if (n <= 1) return s;
  if (!anyExt || depth >= kMedianDepth) {
    if (!anyExt && n <= uint32_t(kMaxLeaf)) return s;
    s.kind = 2;
    s.nL = n / 2;
    return s;
  }
  const float parentArea = fmaxf(boxArea(t.blo[0], t.blo[1], t.blo[2], t.bhi[0], t.bhi[1], t.bhi[2]), 1e-30f);
  float best = FLT_MAX;
  int bestAx = -1, bestBin = -1;
  // per axis: inclusive prefix (left) and suffix (right) of box and count
  for (int ax = 0; ax < 3; ++ax) {
    if (!(scale[ax] > 0.0f)) continue;
    const uint32_t* b = bins + (ax * kBins + lane) * kBinWords;
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
      lo[k] = funkey(b[k]);
      hi[k] = funkey(b[3 + k]);
    }
    uint32_t cnt = b[12];
    float plo[3] = {lo[0], lo[1], lo[2]}, phi[3] = {hi[0], hi[1], hi[2]};
    uint32_t pc = cnt;
    float slo[3] = {lo[0], lo[1], lo[2]}, shi[3] = {hi[0], hi[1], hi[2]};
    uint32_t sc = cnt;
    for (int off = 1; off < 32; off <<= 1) {
      float ul[3], uh[3], dl[3], dh[3];
      for (int k = 0; k < 3; ++k) {
        ul[k] = __shfl_up_sync(0xffffffffu, plo[k], off);
        uh[k] = __shfl_up_sync(0xffffffffu, phi[k], off);
        dl[k] = __shfl_down_sync(0xffffffffu, slo[k], off);
        dh[k] = __shfl_down_sync(0xffffffffu, shi[k], off);
      }
      const uint32_t uc = __shfl_up_sync(0xffffffffu, pc, off), dc = __shfl_down_sync(0xffffffffu, sc, off);
      if (lane >= off) {
        for (int k = 0; k < 3; ++k) {
          plo[k] = fminf(plo[k], ul[k]);
          phi[k] = fmaxf(phi[k], uh[k]);
        }
        pc += uc;
      }
      if (lane + off < 32) {
        for (int k = 0; k < 3; ++k) {
          slo[k] = fminf(slo[k], dl[k]);
          shi[k] = fmaxf(shi[k], dh[k]);
        }
        sc += dc;
      }
    }
    // right side of split `lane` = suffix of lane + 1
    float rlo[3], rhi[3];
    for (int k = 0; k < 3; ++k) {
      rlo[k] = __shfl_down_sync(0xffffffffu, slo[k], 1);
      rhi[k] = __shfl_down_sync(0xffffffffu, shi[k], 1);
    }
    const uint32_t rc = __shfl_down_sync(0xffffffffu, sc, 1);
    float cost = FLT_MAX;
    if (lane < kBins - 1 && pc > 0 && rc > 0)
      cost = 1.0f + (boxArea(plo[0], plo[1], plo[2], phi[0], phi[1], phi[2]) * float(pc) +
                     boxArea(rlo[0], rlo[1], rlo[2], rhi[0], rhi[1], rhi[2]) * float(rc)) /
                        parentArea;
    // first minimum over the lanes of this axis
    float c = cost;
    int at = lane;
    for (int off = 16; off; off >>= 1) {
      const float oc = __shfl_xor_sync(0xffffffffu, c, off);
      const int oa = __shfl_xor_sync(0xffffffffu, at, off);
      if (oc < c || (oc == c && oa < at)) {
        c = oc;
        at = oa;
      }
    }
    if (c < best) {
      best = c;
      bestAx = ax;
      bestBin = at;
    }
  }
  if (bestAx < 0) {
    if (n > uint32_t(kMaxLeaf)) {
      s.kind = 2;
      s.nL = n / 2;
    }
    return s;
  }
  if (n <= uint32_t(kMaxLeaf) && best >= float(n)) return s;
  // the chosen split's children: boxes, centroid boxes and counts from the bins
  s.kind = 1;
  s.axis = bestAx;
  s.bin = bestBin;
  s.lo = t.clo[bestAx];
  s.scale = scale[bestAx];
  const uint32_t* b = bins + (bestAx * kBins + lane) * kBinWords;
  const bool isLeft = lane <= bestBin;
  const uint32_t cnt = b[12];
  // reduce separately over the left (lane <= bestBin) and right lanes
  float lv[12], rv[12];
  for (int k = 0; k < 12; ++k) {
    const float id = isMinWord(k) ? FLT_MAX : -FLT_MAX;
    const float v = funkey(b[k]);
    lv[k] = isLeft ? v : id;
    rv[k] = isLeft ? id : v;
  }
  uint32_t lc = isLeft ? cnt : 0u, rcn = isLeft ? 0u : cnt;
  for (int off = 16; off; off >>= 1) {
    for (int k = 0; k < 12; ++k) {
      const float ol = __shfl_xor_sync(0xffffffffu, lv[k], off), orr = __shfl_xor_sync(0xffffffffu, rv[k], off);
      lv[k] = isMinWord(k) ? fminf(lv[k], ol) : fmaxf(lv[k], ol);
      rv[k] = isMinWord(k) ? fminf(rv[k], orr) : fmaxf(rv[k], orr);
    }
    lc += __shfl_xor_sync(0xffffffffu, lc, off);
    rcn += __shfl_xor_sync(0xffffffffu, rcn, off);
  }
  s.nL = lc;
  for (int k = 0; k < 3; ++k) {
    s.left.blo[k] = lv[k];
    s.left.bhi[k] = lv[3 + k];
    s.left.clo[k] = lv[6 + k];
    s.left.chi[k] = lv[9 + k];
    s.right.blo[k] = rv[k];
    s.right.bhi[k] = rv[3 + k];
    s.right.clo[k] = rv[6 + k];
    s.right.chi[k] = rv[9 + k];
  }
  (void)rcn;
  return s;
}

// Child tasks of a split task that became node `node`: ranges, buffer,
// depth, and (for index halving) boxes recomputed by the caller.
__device__ __forceinline__ void childTasks(const BTask& t, const BSplit& s, int32_t node, BTask& l, BTask& r) {
  const uint32_t depth = taskDepth(t) + 1;
  const uint32_t buf = taskBuf(t) ^ 1u;
  l = s.left;
  r = s.right;
  l.begin = t.begin;
  l.end = t.begin + s.nL;
  r.begin = t.begin + s.nL;
  r.end = t.end;
  l.node = r.node = node;
  l.flags = (depth << 8) | (buf << 2) | 0u;
  r.flags = (depth << 8) | (buf << 2) | 1u;
}

// Side of a primitive at position `pos` of task t under split s.
__device__ __forceinline__ bool goesLeft(const BuildCtx& C, const BTask& t, const BSplit& s, uint32_t pos,
                                         uint32_t p) {
  if (s.kind == 2) return pos < t.begin + s.nL;
  const float4 c = __ldg(&C.cen[p]);
  const float cc = s.axis == 0 ? c.x : (s.axis == 1 ? c.y : c.z);
  return binOf(cc, s.lo, s.scale) <= s.bin;
}

__device__ __forceinline__ void noteDepth(const BuildCtx& C, uint32_t d) { atomicMax(&C.counters[kCtrDepth], d); }

// Writes a leaf for task t (its parent's slot, or slot 0 of its root node)
// and moves its primitives into the final order.
__device__ __forceinline__ void emitLeaf(const BuildCtx& C, const BTask& t) {
  BvhNode* n = C.nodes + t.node;
  const int side = (t.flags & 2u) ? 0 : int(t.flags & 1u);
  setChild(n, side, t.blo, t.bhi, encodeLeaf(t.begin, t.end - t.begin));
  const uint32_t* src = C.ord[taskBuf(t)];
  for (uint32_t i = t.begin; i < t.end; ++i) C.ordFinal[i] = src[i];
}

// Node for a task that splits: the root keeps its node; others take one from
// `alloc` and fill their parent's slot with it.
template <class Alloc>
__device__ __forceinline__ int32_t innerNode(const BuildCtx& C, const BTask& t, bool writer, Alloc&& alloc) {
  if (t.flags & 2u) return t.node;
  const int32_t idx = alloc();
  if (idx < 0) return -1;
  if (writer) setChild(C.nodes + t.node, int(t.flags & 1u), t.blo, t.bhi, idx);
  return idx;
}

// ---------------------------------------------------------------------------
// primitive boxes and centroids; per-mesh root bounds (keys)
__global__ void k_primBounds(const VtxDev* __restrict__ vtx, const uint4* __restrict__ idx,
                             const uint32_t* __restrict__ triBase, const uint32_t* __restrict__ vtxBase, int nm,
                             uint32_t N, float4* pbox, float4* cen, uint32_t* ord0, uint32_t* meshKeys) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < N;
  int m = 0;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, c[3] = {0, 0, 0};
  if (valid) {
    int a = 0, b = nm;  // largest m with triBase[m] <= p
    while (b - a > 1) {
      const int mid = (a + b) / 2;
      if (__ldg(&triBase[mid]) <= p) a = mid; else b = mid;
    }
    m = a;
    const uint4 t = __ldg(&idx[p]);
    const uint32_t vb = __ldg(&vtxBase[m]);
    const float4 p0 = __ldg(&vtx[vb + t.x].pu), p1 = __ldg(&vtx[vb + t.y].pu), p2 = __ldg(&vtx[vb + t.z].pu);
    const float a0[3] = {p0.x, p0.y, p0.z}, a1[3] = {p1.x, p1.y, p1.z}, a2[3] = {p2.x, p2.y, p2.z};
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(a0[k], fminf(a1[k], a2[k]));
      hi[k] = fmaxf(a0[k], fmaxf(a1[k], a2[k]));
      c[k] = 0.5f * (lo[k] + hi[k]);
    }
    pbox[2 * size_t(p)] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    pbox[2 * size_t(p) + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    cen[p] = make_float4(c[0], c[1], c[2], 0.0f);
    ord0[p] = p;
  }
  // per-mesh bounds: one atomic per warp when the whole warp is in one mesh
  const unsigned lane = threadIdx.x & 31u;
  const int m0 = __shfl_sync(0xffffffffu, m, 0);
  const bool uniform = __all_sync(0xffffffffu, !valid || m == m0);
  uint32_t key[12];
  for (int k = 0; k < 3; ++k) {
    key[k] = valid ? fkey(lo[k]) : kKeyLoInit;
    key[3 + k] = valid ? fkey(hi[k]) : kKeyHiInit;
    key[6 + k] = valid ? fkey(c[k]) : kKeyLoInit;
    key[9 + k] = valid ? fkey(c[k]) : kKeyHiInit;
  }
  if (uniform) {
    for (int off = 16; off; off >>= 1)
      for (int k = 0; k < 12; ++k) {
        const uint32_t o = __shfl_xor_sync(0xffffffffu, key[k], off);
        key[k] = isMinWord(k) ? min(key[k], o) : max(key[k], o);
      }
    if (lane == 0 && valid) {
      uint32_t* dst = meshKeys + size_t(m0) * 12;
      for (int k = 0; k < 12; ++k) {
        if (isMinWord(k)) atomicMin(&dst[k], key[k]); else atomicMax(&dst[k], key[k]);
      }
    }
  } else if (valid) {
    uint32_t* dst = meshKeys + size_t(m) * 12;
    for (int k = 0; k < 12; ++k) {
      if (isMinWord(k)) atomicMin(&dst[k], key[k]); else atomicMax(&dst[k], key[k]);
    }
  }
}

// ---------------------------------------------------------------------------
// large tasks: one chunk (task, first, last) per block
struct Chunk {
  uint32_t task, first, last;
};

__global__ void __launch_bounds__(256) k_binLarge(BuildCtx C, const BTask* __restrict__ tasks,
                                                  const Chunk* __restrict__ chunks, uint32_t* gbins) {
  __shared__ uint32_t bins[kTaskBinWords];
  const Chunk ch = chunks[blockIdx.x];
  const BTask t = tasks[ch.task];
  clearBins(bins, threadIdx.x, blockDim.x);
  __syncthreads();
  float scale[3];
  binScales(t, scale);
  const uint32_t* ord = C.ord[taskBuf(t)];
  for (uint32_t i = ch.first + threadIdx.x; i < ch.last; i += blockDim.x) binPrim(bins, C, ord[i], t.clo, scale);
  __syncthreads();
  uint32_t* g = gbins + size_t(ch.task) * kTaskBinWords;
  for (int i = threadIdx.x; i < kTaskBinWords; i += blockDim.x) {
    const int w = i % kBinWords;
    const uint32_t v = bins[i];
    if (v == initWord(w)) continue;
    if (w == kBinWords - 1)
      atomicAdd(&g[i], v);
    else if (isMinWord(w))
      atomicMin(&g[i], v);
    else
      atomicMax(&g[i], v);
  }
}

__global__ void k_clearBins(uint32_t* gbins, uint32_t ntasks) {
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= size_t(ntasks) * kTaskBinWords) return;
  gbins[i] = initWord(int(i % kBinWords));
}

// One warp per large task: the split, the inner node, the partition cursors.
__global__ void k_splitLarge(BuildCtx C, const BTask* __restrict__ tasks, uint32_t ntasks,
                             const uint32_t* __restrict__ gbins, BSplit* splits, uint32_t* cursors) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) / 32u;
  const int lane = threadIdx.x & 31;
  if (w >= ntasks) return;
  const BTask t = tasks[w];
  BSplit s = decideSplit(gbins + size_t(w) * kTaskBinWords, t, lane);
  if (lane == 0) {
    noteDepth(C, taskDepth(t));
    // large tasks always hold more primitives than a leaf: kind 0 cannot occur
    if (s.kind == 0) {
      s.kind = 2;
      s.nL = (t.end - t.begin) / 2;
    }
    const int32_t node = innerNode(C, t, true, [&] {
      const uint32_t i = atomicAdd(&C.counters[kCtrNodes], 1u);
      if (i >= C.nodeCap) {
        atomicOr(&C.counters[kCtrError], uint32_t(kErrNodes));
        return -1;
      }
      return int32_t(i);
    });
    s.node = node;
    splits[w] = s;
    cursors[2 * w] = t.begin;
    cursors[2 * w + 1] = t.begin + s.nL;
  }
}

__global__ void __launch_bounds__(256) k_partitionLarge(BuildCtx C, const BTask* __restrict__ tasks,
                                                        const Chunk* __restrict__ chunks,
                                                        const BSplit* __restrict__ splits, uint32_t* cursors) {
  __shared__ uint32_t warpL[8], warpR[8], baseL, baseR;
  const Chunk ch = chunks[blockIdx.x];
  const BTask t = tasks[ch.task];
  const BSplit& s = splits[ch.task];
  const uint32_t* src = C.ord[taskBuf(t)];
  uint32_t* dst = C.ord[taskBuf(t) ^ 1u];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x / 32u;
  for (uint32_t base = ch.first; base < ch.last; base += blockDim.x) {
    const uint32_t pos = base + threadIdx.x;
    const bool valid = pos < ch.last;
    uint32_t p = 0;
    bool left = false;
    if (valid) {
      p = src[pos];
      left = goesLeft(C, t, s, pos, p);
    }
    const unsigned bl = __ballot_sync(0xffffffffu, valid && left), br = __ballot_sync(0xffffffffu, valid && !left);
    if (lane == 0) {
      warpL[warp] = __popc(bl);
      warpR[warp] = __popc(br);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t tl = 0, tr = 0;
      for (unsigned k = 0; k < blockDim.x / 32u; ++k) {
        const uint32_t a = warpL[k], b = warpR[k];
        warpL[k] = tl;
        warpR[k] = tr;
        tl += a;
        tr += b;
      }
      baseL = tl ? atomicAdd(&cursors[2 * ch.task], tl) : 0u;
      baseR = tr ? atomicAdd(&cursors[2 * ch.task + 1], tr) : 0u;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
    if (valid) {
      const uint32_t at = left ? baseL + warpL[warp] + __popc(bl & below) : baseR + warpR[warp] + __popc(br & below);
      if (at >= t.begin && at < t.end) dst[at] = p;
      else atomicOr(&C.counters[kCtrError], uint32_t(kErrTasks));
    }
    __syncthreads();
  }
}

// Child tasks of the large tasks: to the next level, or to the small list.
__global__ void k_childrenLarge(BuildCtx C, const BTask* __restrict__ tasks, uint32_t ntasks,
                                const BSplit* __restrict__ splits) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= ntasks) return;
  const BTask t = tasks[w];
  const BSplit s = splits[w];
  if (s.node < 0) return;
  BTask ch[2];
  childTasks(t, s, s.node, ch[0], ch[1]);
  for (int k = 0; k < 2; ++k) {
    BTask c = ch[k];
    if (s.kind == 2) {
      // halving: the children keep the parent's bounds (they are recomputed
      // below from the primitives when the child is binned; for the box in
      // the node slot the parent's box is conservative)
      for (int a = 0; a < 3; ++a) {
        c.blo[a] = t.blo[a];
        c.bhi[a] = t.bhi[a];
        c.clo[a] = t.clo[a];
        c.chi[a] = t.chi[a];
      }
    }
    const uint32_t n = c.end - c.begin;
    if (n > kSmallTask) {
      const uint32_t i = atomicAdd(&C.counters[kCtrNextLarge], 1u);
      if (i < C.nextLargeCap) C.nextLarge[i] = c;
      else atomicOr(&C.counters[kCtrError], uint32_t(kErrTasks));
    } else {
      const uint32_t i = atomicAdd(&C.counters[kCtrSmall], 1u);
      if (i < C.smallCap) C.small[i] = c;
      else atomicOr(&C.counters[kCtrError], uint32_t(kErrTasks));
    }
  }
}

// ---------------------------------------------------------------------------
// Small tasks: each warp builds whole subtrees, depth first.
__global__ void __launch_bounds__(kSmallWarps * 32) k_buildSmall(BuildCtx C, uint32_t ntasks) {
  __shared__ uint32_t sbins[kSmallWarps][kTaskBinWords];
  __shared__ BTask sstack[kSmallWarps][kWarpStack];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x / 32;
  uint32_t* bins = sbins[wib];
  BTask* stack = sstack[wib];
  uint32_t nodeNext = 0, nodeEnd = 0;  // this warp's current chunk of node indices
  auto alloc = [&]() -> int32_t {
    if (nodeNext == nodeEnd) {
      uint32_t b = 0;
      if (lane == 0) b = atomicAdd(&C.counters[kCtrNodes], kNodeChunk);
      b = __shfl_sync(0xffffffffu, b, 0);
      if (b + kNodeChunk > C.nodeCap) {
        if (lane == 0) atomicOr(&C.counters[kCtrError], uint32_t(kErrNodes));
        return -1;
      }
      nodeNext = b;
      nodeEnd = b + kNodeChunk;
    }
    return int32_t(nodeNext++);
  };
  for (;;) {
    uint32_t ti = 0;
    if (lane == 0) ti = atomicAdd(&C.counters[kCtrSmallNext], 1u);
    ti = __shfl_sync(0xffffffffu, ti, 0);
    if (ti >= ntasks) break;
    int sp = 0;
    if (lane == 0) stack[0] = C.small[ti];
    sp = 1;
    __syncwarp();
    while (sp > 0) {
      const BTask t = stack[sp - 1];
      __syncwarp();
      --sp;
      const uint32_t n = t.end - t.begin;
      if (lane == 0) noteDepth(C, taskDepth(t));
      float scale[3];
      binScales(t, scale);
      clearBins(bins, lane, 32);
      __syncwarp();
      const uint32_t* src = C.ord[taskBuf(t)];
      if (n > 1)
        for (uint32_t i = t.begin + lane; i < t.end; i += 32) binPrim(bins, C, src[i], t.clo, scale);
      __syncwarp();
      BSplit s = decideSplit(bins, t, lane);
      __syncwarp();
      if (s.kind == 0) {
        if (lane == 0) emitLeaf(C, t);
        continue;
      }
      const int32_t node = innerNode(C, t, lane == 0, alloc);
      if (node < 0) break;
      // partition into the other buffer, stable within each side
      uint32_t* dst = C.ord[taskBuf(t) ^ 1u];
      uint32_t nl = 0, nr = 0;
      const unsigned below = (1u << lane) - 1u;
      for (uint32_t base = t.begin; base < t.end; base += 32) {
        const uint32_t pos = base + lane;
        const bool valid = pos < t.end;
        uint32_t p = 0;
        bool left = false;
        if (valid) {
          p = src[pos];
          left = goesLeft(C, t, s, pos, p);
        }
        const unsigned bl = __ballot_sync(0xffffffffu, valid && left), br = __ballot_sync(0xffffffffu, valid && !left);
        if (valid) {
          const uint32_t at = left ? t.begin + nl + __popc(bl & below) : t.begin + s.nL + nr + __popc(br & below);
          if (at < t.end) dst[at] = p;
        }
        nl += __popc(bl);
        nr += __popc(br);
      }
      if (nl != s.nL) {
        if (lane == 0) atomicOr(&C.counters[kCtrError], uint32_t(kErrTasks));
        break;
      }
      BTask l, r;
      childTasks(t, s, node, l, r);
      __syncwarp();  // the partition's writes before any lane reads them
      if (s.kind == 2) {
        // index halving: recompute the halves' boxes from their primitives
        float v[2][12];
        for (int side = 0; side < 2; ++side) {
          const BTask& c = side ? r : l;
          float a[12];
          for (int k = 0; k < 3; ++k) {
            a[k] = FLT_MAX;
            a[3 + k] = -FLT_MAX;
            a[6 + k] = FLT_MAX;
            a[9 + k] = -FLT_MAX;
          }
          for (uint32_t i = c.begin + lane; i < c.end; i += 32) {
            const uint32_t p = dst[i];
            const float4 lo = __ldg(&C.pbox[2 * size_t(p)]), hi = __ldg(&C.pbox[2 * size_t(p) + 1]);
            const float4 cc = __ldg(&C.cen[p]);
            const float L[3] = {lo.x, lo.y, lo.z}, H[3] = {hi.x, hi.y, hi.z}, Cc[3] = {cc.x, cc.y, cc.z};
            for (int k = 0; k < 3; ++k) {
              a[k] = fminf(a[k], L[k]);
              a[3 + k] = fmaxf(a[3 + k], H[k]);
              a[6 + k] = fminf(a[6 + k], Cc[k]);
              a[9 + k] = fmaxf(a[9 + k], Cc[k]);
            }
          }
          for (int off = 16; off; off >>= 1)
            for (int k = 0; k < 12; ++k) {
              const float o = __shfl_xor_sync(0xffffffffu, a[k], off);
              a[k] = isMinWord(k) ? fminf(a[k], o) : fmaxf(a[k], o);
            }
          for (int k = 0; k < 12; ++k) v[side][k] = a[k];
        }
        for (int k = 0; k < 3; ++k) {
          l.blo[k] = v[0][k];
          l.bhi[k] = v[0][3 + k];
          l.clo[k] = v[0][6 + k];
          l.chi[k] = v[0][9 + k];
          r.blo[k] = v[1][k];
          r.bhi[k] = v[1][3 + k];
          r.clo[k] = v[1][6 + k];
          r.chi[k] = v[1][9 + k];
        }
      }
      if (sp + 2 > kWarpStack) {
        if (lane == 0) atomicOr(&C.counters[kCtrError], uint32_t(kErrStack));
        break;
      }
      __syncwarp();
      if (lane == 0) {
        stack[sp] = r;
        stack[sp + 1] = l;
      }
      sp += 2;
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// Leaf triangles in leaf order: TriDev = object-space vertices, primitive id.
__global__ void k_emitTris(const VtxDev* __restrict__ vtx, const uint4* __restrict__ idx,
                           const uint32_t* __restrict__ triBase, const uint32_t* __restrict__ vtxBase, int nm,
                           uint32_t N, const uint32_t* __restrict__ ordFinal, TriDev* tris) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int a = 0, b = nm;
  while (b - a > 1) {
    const int mid = (a + b) / 2;
    if (__ldg(&triBase[mid]) <= i) a = mid; else b = mid;
  }
  const uint32_t p = ordFinal[i];
  if (p < __ldg(&triBase[a]) || p >= __ldg(&triBase[a + 1])) return;  // (checked on the host afterwards)
  const uint4 t = __ldg(&idx[p]);
  const uint32_t vb = __ldg(&vtxBase[a]);
  const float4 p0 = __ldg(&vtx[vb + t.x].pu), p1 = __ldg(&vtx[vb + t.y].pu), p2 = __ldg(&vtx[vb + t.z].pu);
  TriDev d;
  d.v0 = make_float4(p0.x, p0.y, p0.z, __uint_as_float(p - __ldg(&triBase[a])));
  d.v1 = make_float4(p1.x, p1.y, p1.z, 0.0f);
  d.v2 = make_float4(p2.x, p2.y, p2.z, 0.0f);
  tris[i] = d;
}

// Every final position holds a primitive of its own mesh exactly once:
// counts primitives whose position is outside their mesh's range, and marks
// each primitive seen (a second sighting counts as an error too).
__global__ void k_checkOrder(const uint32_t* __restrict__ triBase, int nm, uint32_t N,
                             const uint32_t* __restrict__ ordFinal, uint32_t* seen, uint32_t* errors) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int a = 0, b = nm;
  while (b - a > 1) {
    const int mid = (a + b) / 2;
    if (__ldg(&triBase[mid]) <= i) a = mid; else b = mid;
  }
  const uint32_t p = ordFinal[i];
  if (p >= N || p < __ldg(&triBase[a]) || p >= __ldg(&triBase[a + 1])) {
    atomicAdd(errors, 1u);
    return;
  }
  if (atomicExch(&seen[p], 1u) != 0u) atomicAdd(errors, 1u);
}

template <class T>
int devAlloc(T** p, size_t n, std::vector<void*>& tmp) {
  *p = nullptr;
  ASUNA_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T)));
  tmp.push_back(*p);
  return ASUNA_OK;
}

}  // namespace

int buildBlasDevice(const VtxDev* vtx, const uint4* idx, const std::vector<uint32_t>& triBase,
                    const std::vector<uint32_t>& vtxBase, uint32_t extraNodes, cudaStream_t st, DeviceBlas& out) {
  const int nm = int(triBase.size()) - 1;
  const uint32_t N = triBase[nm];
  out = DeviceBlas{};
  out.roots.assign(nm, -1);
  std::vector<void*> tmp;
  struct Free {
    std::vector<void*>& v;
    ~Free() {
      for (void* p : v) cudaFree(p);
    }
  } freeTmp{tmp};
  // node capacity: inner nodes <= primitives, plus the roots, plus the
  // unused tails of the small-task builders' 64-node chunks
  const uint32_t smallMax = 2 * (N / kSmallTask + 1) + 2 * uint32_t(nm) + 64;
  const uint64_t cap64 = uint64_t(N) + nm + uint64_t(smallMax) * kNodeChunk + 1024;
  if (cap64 + extraNodes > (1ull << 31)) return fail(ASUNA_ERR_UNSUPPORTED, "BVH node count exceeds 2^31");
  const uint32_t nodeCap = uint32_t(cap64);
  ASUNA_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&out.nodes), size_t(nodeCap + extraNodes) * sizeof(BvhNode)));
  ASUNA_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&out.tris), std::max<size_t>(N, 1) * sizeof(TriDev)));
  out.nodeCapacity = nodeCap + extraNodes;
  if (N == 0) return ASUNA_OK;

  uint32_t *dTriBase, *dVtxBase, *meshKeys, *counters, *ordFinal, *ord0, *ord1;
  float4 *pbox, *cen;
  int rc;
  if ((rc = devAlloc(&dTriBase, nm + 1, tmp)) || (rc = devAlloc(&dVtxBase, nm, tmp)) ||
      (rc = devAlloc(&meshKeys, size_t(nm) * 12, tmp)) || (rc = devAlloc(&counters, kCtrNum, tmp)) ||
      (rc = devAlloc(&ordFinal, N, tmp)) || (rc = devAlloc(&ord0, N, tmp)) || (rc = devAlloc(&ord1, N, tmp)) ||
      (rc = devAlloc(&pbox, size_t(N) * 2, tmp)) || (rc = devAlloc(&cen, N, tmp)))
    return rc;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(dTriBase, triBase.data(), (nm + 1) * 4, cudaMemcpyHostToDevice, st));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(dVtxBase, vtxBase.data(), nm * 4, cudaMemcpyHostToDevice, st));
  {
    std::vector<uint32_t> init(size_t(nm) * 12);
    for (size_t i = 0; i < init.size(); ++i) init[i] = isMinWord(int(i % 12)) ? kKeyLoInit : kKeyHiInit;
    ASUNA_CUDA_TRY(cudaMemcpyAsync(meshKeys, init.data(), init.size() * 4, cudaMemcpyHostToDevice, st));
  }
  ASUNA_CUDA_TRY(cudaMemsetAsync(counters, 0, kCtrNum * 4, st));
  ASUNA_CUDA_TRY(cudaMemsetAsync(out.nodes, 0, size_t(nodeCap) * sizeof(BvhNode), st));
  k_primBounds<<<(N + 255) / 256, 256, 0, st>>>(vtx, idx, dTriBase, dVtxBase, nm, N, pbox, cen, ord0, meshKeys);
  ASUNA_CUDA_TRY(cudaGetLastError());
  std::vector<uint32_t> keys(size_t(nm) * 12);
  ASUNA_CUDA_TRY(cudaMemcpyAsync(keys.data(), meshKeys, keys.size() * 4, cudaMemcpyDeviceToHost, st));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(st));
  auto unkey = [](uint32_t k) {
    const uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
  };
  // roots: node r for the r-th non-empty mesh, both slots empty (a point at
  // 1e30 that no ray with tmax <= 1e10 reaches, as the host builder makes)
  std::vector<BTask> large, smallInit;
  std::vector<BvhNode> rootInit;
  for (int m = 0; m < nm; ++m) {
    const uint32_t n = triBase[m + 1] - triBase[m];
    if (!n) continue;
    const int32_t r = int32_t(rootInit.size());
    out.roots[m] = r;
    BvhNode e{};
    e.xy[0] = e.xy[1] = e.zs = make_float4(1e30f, 1e30f, 1e30f, 1e30f);
    e.ref = make_int4(kStackSentinel, kStackSentinel, 0, 0);
    rootInit.push_back(e);
    BTask t{};
    t.begin = triBase[m];
    t.end = triBase[m + 1];
    t.node = r;
    t.flags = (1u << 8) | 2u;
    for (int k = 0; k < 3; ++k) {
      t.blo[k] = unkey(keys[size_t(m) * 12 + k]);
      t.bhi[k] = unkey(keys[size_t(m) * 12 + 3 + k]);
      t.clo[k] = unkey(keys[size_t(m) * 12 + 6 + k]);
      t.chi[k] = unkey(keys[size_t(m) * 12 + 9 + k]);
    }
    (n > kSmallTask ? large : smallInit).push_back(t);
  }
  const uint32_t nroots = uint32_t(rootInit.size());
  ASUNA_CUDA_TRY(cudaMemcpyAsync(out.nodes, rootInit.data(), nroots * sizeof(BvhNode), cudaMemcpyHostToDevice, st));
  {
    const uint32_t c0 = nroots;
    ASUNA_CUDA_TRY(cudaMemcpyAsync(&counters[kCtrNodes], &c0, 4, cudaMemcpyHostToDevice, st));
  }
  // task lists
  BTask *dLarge, *dNext, *dSmall;
  const uint32_t largeCap = 2 * (N / kSmallTask + 1) + uint32_t(nm) + 16;
  if ((rc = devAlloc(&dLarge, largeCap, tmp)) || (rc = devAlloc(&dNext, largeCap, tmp)) ||
      (rc = devAlloc(&dSmall, smallMax, tmp)))
    return rc;
  if (smallInit.size() > smallMax) return fail(ASUNA_ERR_INVALID, "device BVH build: too many small meshes");
  if (!smallInit.empty())
    ASUNA_CUDA_TRY(cudaMemcpyAsync(dSmall, smallInit.data(), smallInit.size() * sizeof(BTask), cudaMemcpyHostToDevice,
                                   st));
  {
    const uint32_t c = uint32_t(smallInit.size());
    ASUNA_CUDA_TRY(cudaMemcpyAsync(&counters[kCtrSmall], &c, 4, cudaMemcpyHostToDevice, st));
  }
  BuildCtx C;
  C.pbox = pbox;
  C.cen = cen;
  C.ord[0] = ord0;
  C.ord[1] = ord1;
  C.ordFinal = ordFinal;
  C.nodes = out.nodes;
  C.nodeCap = nodeCap;
  C.counters = counters;
  C.nextLarge = dNext;
  C.nextLargeCap = largeCap;
  C.small = dSmall;
  C.smallCap = smallMax;
  // ---- large tasks, level by level ----
  uint32_t* gbins = nullptr;
  BSplit* splits = nullptr;
  uint32_t* cursors = nullptr;
  Chunk* dChunks = nullptr;
  size_t gbinsCap = 0, chunksCap = 0;
  int levels = 0;
  while (!large.empty()) {
    if (++levels > int(kMedianDepth) + 32) return fail(ASUNA_ERR_INVALID, "device BVH build: no progress");
    const uint32_t nt = uint32_t(large.size());
    std::vector<Chunk> chunks;
    for (uint32_t t = 0; t < nt; ++t)
      for (uint32_t f = large[t].begin; f < large[t].end; f += kChunk)
        chunks.push_back({t, f, std::min(large[t].end, f + kChunk)});
    if (nt > gbinsCap) {
      if (gbins) cudaFree(gbins);
      if (splits) cudaFree(splits);
      if (cursors) cudaFree(cursors);
      tmp.erase(std::remove_if(tmp.begin(), tmp.end(),
                               [&](void* p) { return p == gbins || p == splits || p == cursors; }),
                tmp.end());
      gbinsCap = std::max<size_t>(nt, 64);
      if ((rc = devAlloc(&gbins, gbinsCap * kTaskBinWords, tmp)) || (rc = devAlloc(&splits, gbinsCap, tmp)) ||
          (rc = devAlloc(&cursors, gbinsCap * 2, tmp)))
        return rc;
    }
    if (chunks.size() > chunksCap) {
      if (dChunks) cudaFree(dChunks);
      tmp.erase(std::remove(tmp.begin(), tmp.end(), static_cast<void*>(dChunks)), tmp.end());
      chunksCap = std::max<size_t>(chunks.size(), 256);
      if ((rc = devAlloc(&dChunks, chunksCap, tmp))) return rc;
    }
    ASUNA_CUDA_TRY(cudaMemcpyAsync(dLarge, large.data(), nt * sizeof(BTask), cudaMemcpyHostToDevice, st));
    ASUNA_CUDA_TRY(
        cudaMemcpyAsync(dChunks, chunks.data(), chunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice, st));
    const size_t nb = size_t(nt) * kTaskBinWords;
    k_clearBins<<<unsigned((nb + 255) / 256), 256, 0, st>>>(gbins, nt);
    k_binLarge<<<unsigned(chunks.size()), 256, 0, st>>>(C, dLarge, dChunks, gbins);
    k_splitLarge<<<(nt * 32 + 127) / 128, 128, 0, st>>>(C, dLarge, nt, gbins, splits, cursors);
    k_partitionLarge<<<unsigned(chunks.size()), 256, 0, st>>>(C, dLarge, dChunks, splits, cursors);
    const uint32_t zero = 0;
    ASUNA_CUDA_TRY(cudaMemcpyAsync(&counters[kCtrNextLarge], &zero, 4, cudaMemcpyHostToDevice, st));
    k_childrenLarge<<<(nt + 127) / 128, 128, 0, st>>>(C, dLarge, nt, splits);
    ASUNA_CUDA_TRY(cudaGetLastError());
    uint32_t ctr[kCtrNum];
    ASUNA_CUDA_TRY(cudaMemcpyAsync(ctr, counters, sizeof(ctr), cudaMemcpyDeviceToHost, st));
    ASUNA_CUDA_TRY(cudaStreamSynchronize(st));
    if (ctr[kCtrError]) return fail(ASUNA_ERR_INVALID, "device BVH build failed (error bits %u)", ctr[kCtrError]);
    const uint32_t nn = std::min(ctr[kCtrNextLarge], largeCap);
    large.resize(nn);
    if (nn)
      ASUNA_CUDA_TRY(cudaMemcpyAsync(large.data(), dNext, nn * sizeof(BTask), cudaMemcpyDeviceToHost, st));
    ASUNA_CUDA_TRY(cudaStreamSynchronize(st));
  }
  // ---- small tasks: one warp per subtree ----
  uint32_t ctr[kCtrNum];
  ASUNA_CUDA_TRY(cudaMemcpyAsync(ctr, counters, sizeof(ctr), cudaMemcpyDeviceToHost, st));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(st));
  const uint32_t nsmall = std::min(ctr[kCtrSmall], smallMax);
  if (nsmall) {
    int dev = 0, sms = 0;
    ASUNA_CUDA_TRY(cudaGetDevice(&dev));
    ASUNA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int per = 0;
    ASUNA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_buildSmall, kSmallWarps * 32, 0));
    const uint32_t grid = std::max(1u, std::min(uint32_t(sms * std::max(per, 1)), (nsmall + kSmallWarps - 1) / kSmallWarps));
    k_buildSmall<<<grid, kSmallWarps * 32, 0, st>>>(C, nsmall);
    ASUNA_CUDA_TRY(cudaGetLastError());
  }
  // ---- leaf triangles ----
  uint32_t* seen;
  if ((rc = devAlloc(&seen, N + 1, tmp))) return rc;
  ASUNA_CUDA_TRY(cudaMemsetAsync(seen, 0, size_t(N + 1) * 4, st));
  k_checkOrder<<<(N + 255) / 256, 256, 0, st>>>(dTriBase, nm, N, ordFinal, seen, seen + N);
  k_emitTris<<<(N + 255) / 256, 256, 0, st>>>(vtx, idx, dTriBase, dVtxBase, nm, N, ordFinal, out.tris);
  ASUNA_CUDA_TRY(cudaGetLastError());
  uint32_t orderErrors = 0;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(ctr, counters, sizeof(ctr), cudaMemcpyDeviceToHost, st));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(&orderErrors, seen + N, 4, cudaMemcpyDeviceToHost, st));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(st));
  if (ctr[kCtrError]) return fail(ASUNA_ERR_INVALID, "device BVH build failed (error bits %u)", ctr[kCtrError]);
  if (orderErrors) return fail(ASUNA_ERR_INVALID, "device BVH build: %u primitives misplaced", orderErrors);
  out.nodeCount = std::min(ctr[kCtrNodes], nodeCap);
  out.maxDepth = ctr[kCtrDepth];
  out.rootNodes.resize(nroots);
  if (nroots)
    ASUNA_CUDA_TRY(cudaMemcpy(out.rootNodes.data(), out.nodes, nroots * sizeof(BvhNode), cudaMemcpyDeviceToHost));
  // the capacity bound is loose (about one node per primitive): move the
  // nodes into an array of the size used, with the caller's extra room
  const size_t used = size_t(out.nodeCount) + extraNodes;
  if (used < size_t(out.nodeCapacity) * 9 / 10) {
    BvhNode* tight = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(&tight), used * sizeof(BvhNode)) == cudaSuccess) {
      ASUNA_CUDA_TRY(cudaMemcpyAsync(tight, out.nodes, size_t(out.nodeCount) * sizeof(BvhNode),
                                     cudaMemcpyDeviceToDevice, st));
      ASUNA_CUDA_TRY(cudaStreamSynchronize(st));
      cudaFree(out.nodes);
      out.nodes = tight;
      out.nodeCapacity = uint32_t(used);
    } else {
      cudaGetLastError();  // keep the loose array
    }
  }
  return ASUNA_OK;
}

}  // namespace asuna
