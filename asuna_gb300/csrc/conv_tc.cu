// conv_tc.cu — 3x3 convolution (stride 1, zero padding 1) on the
// fifth-generation tensor cores: tcgen05.mma with the accumulator in tensor
// memory, operands staged in shared memory by TMA.
//
// One CTA computes T (up to 4) 16 x 8 pixel tiles side by side in x (M = 128
// each, one TMEM accumulator per tile) for one slice of nt output channels
// (N = nt, a multiple of 16, at most 256 and small enough that three weight
// stages fit shared memory; cout is split into cout / nt slices, the slice
// index varying fastest across the grid so the CTAs that read one activation
// region run together and share it in L2).  The T tiles share every weight
// stage, so weights are fetched once per 128 T pixels.  The input channels
// are consumed in groups of 16 (K = 16 per MMA):
//   * activations: for each 8-channel chunk, one TMA tiled load of the
//     18 x (8T + 2) halo of the tiles from the NHWC tensor (zero fill outside
//     the image) lands as [row][col][8] bf16 (slots padded to 128 B); for tap
//     (dy, dx) and tile t the A operand is the view starting at pixel
//     (dy, dx + 8t) of that halo: 8-row core matrices are 8 consecutive
//     pixels of one image row, image rows are (8T + 2) * 16 B apart (stride
//     dimension), the second 8-channel chunk is one slot further (leading
//     dimension) — K-major, no swizzle;
//   * weights: pre-arranged as [slice][cin/16][tap][chunk][nt][8] so one
//     group's nine taps are one contiguous bulk copy, B = [chunk][nt][8] per
//     tap;
//   * 9 T MMAs per group accumulate into TMEM (fp32, lane = pixel of a tile,
//     column = tile t * nt + output channel); a 3-stage ring of shared-memory
//     buffers is refilled as tcgen05.commit reports each stage's MMAs done.
// The CTAs are persistent and warp-specialised: one elected thread of a
// fifth warp issues the copies and the MMAs of a stream of units (the ring
// runs ahead across unit boundaries, the MMAs alternate between two TMEM
// accumulator buffers); the four epilogue warps read their 32 TMEM lanes
// each (tcgen05.ld) of the finished buffer, apply bias, ReLU and the ReLU
// mask, store bf16 (or fp32) and hand the buffer back, while the next unit's
// MMAs run.  Every mbarrier wait is bounded: on expiry the CTA records an
// error, stops its work and still frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/asuna_denoise.h"
#include "common.h"

namespace asuna {
namespace tc {
namespace {

constexpr int kTileH = 16, kTileW = 8;                         // pixels per MMA tile (M = 128)
constexpr int kHaloH = kTileH + 2;
constexpr int kMaxTiles = 4;                                   // tiles per CTA, side by side in x
constexpr int kMaxStages = 8;  // copy-ring depth, chosen per layer in [2, 8]
constexpr int kHeader = 256;   // barriers, the TMEM address and the abort flag
// One TMA box of 8 channels covers the halo of T tiles: 18 x (8T + 2) pixels
// of 16 bytes; its shared-memory slot is padded to 128 bytes.
__host__ __device__ constexpr int haloW(int T) { return kTileW * T + 2; }
__host__ __device__ constexpr int boxBytes(int T) { return kHaloH * haloW(T) * 16; }
__host__ __device__ constexpr int chunkBytes(int T) { return (boxBytes(T) + 127) / 128 * 128; }
__host__ __device__ constexpr int actStage(int T) { return 2 * chunkBytes(T); }  // 16 channels
constexpr uint32_t kWaitLimit = 1u << 20;                      // try_wait rounds before giving up

__device__ int g_tcError;  // set when a wait expired; read and cleared by asuna_nn_tc_status

constexpr size_t kSmemLimit = 227 * 1024;
// Every MMA operand view stays inside its stage: the A view of tile T-1 at
// tap (2, 2) ends at ((2 * haloW + 2 + 8 (T-1)) + 15 haloW + 8) * 16 bytes =
// 17 haloW * 16 = boxBytes, the end of the halo box, and the second 8-channel
// chunk's at chunkBytes + boxBytes <= actStage.
__host__ __device__ constexpr int wStage(int nt) { return 9 * 2 * nt * 16; }  // one 16-channel group
// S ring stages of activations; weights either in the ring (a stage per
// group) or resident (all `groups` of the layer, loaded once per CTA)
size_t smemFor(int nt, int T, int S, bool resident, int groups) {
  return kHeader + size_t(S) * actStage(T) + size_t(resident ? groups : S) * wStage(nt);
}
uint32_t pow2Cols(int n) {
  uint32_t c = 32;
  while (c < uint32_t(n)) c <<= 1;
  return c;
}
// Output channels per CTA: the widest slice (fewest slices) that divides cout
// into multiples of 16 and whose one-tile stages fit shared memory.
int sliceWidth(int cout) {
  for (int s = 1; s <= cout / 16; ++s) {
    const int nt = cout / s;
    if (cout % s == 0 && nt % 16 == 0 && nt <= 256 && smemFor(nt, 1, 3, false, 0) <= kSmemLimit) return nt;
  }
  return 16;
}
// Pixel tiles per unit (T), resident CTAs per SM, ring depth and weight
// residency: the choice with the most tiles in flight per SM (T x CTAs),
// where a CTA needs two accumulator buffers of T x nt tensor-memory columns
// (512 per SM), its shared memory, and 192 threads of 72 registers (four
// CTAs fit); then resident weights (single-slice layers whose weights fit:
// read from L2 once per CTA instead of once per unit), then the deepest ring
// the CTAs' shared memory holds; ties go to smaller T (more CTAs, rings that
// run independently).  T stays within the image width.
struct TileShape {
  int T, perSm, stages;
  bool resident;
};
int shapePolicy() {
  static const int p = [] {
    const char* e = std::getenv("ASUNA_TC_SHAPE_POLICY");
    return e ? std::atoi(e) : 0;
  }();
  return p;
}
TileShape tileShape(int nt, int slices, int groups, int w, size_t smemSm, size_t reserve) {
  const int policy = shapePolicy();
  TileShape best{1, 1, 2, false};
  long long bestKey = -1;
  for (int T = 1; T <= kMaxTiles; ++T) {
    if (T > 1 && kTileW * (T - 1) >= w) break;
    const uint32_t cols = pow2Cols(2 * T * nt);
    if (cols > 512) break;
    for (int res = 0; res <= (slices == 1 ? 1 : 0); ++res) {
      if (smemFor(nt, T, 2, res, groups) > kSmemLimit) continue;
      // CTAs per SM at the shallowest ring, then the deepest ring they allow
      const int per = std::max(
          1, std::min({int(smemSm / (smemFor(nt, T, 2, res, groups) + reserve)), 4, int(512 / cols)}));
      const size_t budget = std::min(kSmemLimit, smemSm / size_t(per) - reserve);
      int S = 2;
      while (S < kMaxStages && smemFor(nt, T, S + 1, res, groups) <= budget) ++S;
      if (res && S < 3) continue;  // resident weights only beside a ring of 3 or more
      // policy 0: tiles in flight, then CTAs, residency, ring depth;
      // policy 1: tiles in flight, then residency, ring depth (fewer, deeper CTAs)
      const long long key = policy == 0 ? (((long long)(per * T) * 8 + per) * 2 + res) * 16 + S
                                        : (((long long)(per * T) * 2 + res) * 16 + S) * 8 + (8 - T);
      if (key > bestKey) {
        bestKey = key;
        best = {T, per, S, res != 0};
      }
    }
  }
  return best;
}

__device__ __forceinline__ uint32_t smem(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbarExpectTx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tmaLoad4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulkLoad(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// shared-memory matrix descriptor: start, leading (K) and stride (M/N)
// byte offsets, fixed bits 46-48 = 0b001, no swizzle
__device__ __forceinline__ uint64_t matDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}
// instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major
__device__ __forceinline__ uint32_t instrDesc(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void fenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
  const __nv_bfloat16* wt;    // [cout/nt][cin/16][9][2][nt][8]
  const float* bias;          // [cout] or null
  const __nv_bfloat16* mask;  // [P][cout] or null
  void* out;                  // [P][cout]
  int n, h, w, cin, cout;
  int nt, slices;             // output channels per CTA, cout / nt
  int tiles;                  // 16 x 8 pixel tiles per unit, side by side in x
  int tilesX, tilesY;         // units (16 x 8 tiles pixels) per image row / column
  int units;                  // tilesX * tilesY * n * slices
  int relu, outF32;
  uint32_t tmemCols;          // two accumulator buffers of tiles * nt columns
  uint32_t wStageBytes;       // 9 * 2 * nt * 16
  int stages;                 // copy-ring depth
  int resident;               // weights loaded once per CTA (one slice)
};

// a unit: slice (fastest), then tile column, tile row, image
struct Unit {
  int slice, img, x0, y0;
};
__device__ __forceinline__ Unit unitOf(const TcArgs& a, int u) {
  Unit r;
  r.slice = u % a.slices;
  u /= a.slices;
  const int tx = u % a.tilesX;
  u /= a.tilesX;
  const int ty = u % a.tilesY;
  r.img = u / a.tilesY;
  r.x0 = tx * kTileW * a.tiles;
  r.y0 = ty * kTileH;
  return r;
}

// an abort flag that is never set: for the drains, which wait out the
// copies and MMAs in flight even after an abort
__device__ const int kNeverAbort = 0;

// bounded wait for phase `parity` of the barrier, false when it expired;
// it also gives up once another role has recorded an abort
__device__ __forceinline__ bool mbarWaitOr(uint32_t bar, uint32_t parity, const volatile int* abortFlag) {
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255u) == 255u && *abortFlag) return false;
  }
  return false;
}
__device__ __forceinline__ void mbarArrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Persistent CTAs, warp-specialised: warps 0-3 are the epilogue (TMEM lane
// quarter = warp), warp 4's first lane issues the TMA copies, warp 5's first
// lane the MMAs.  Units (T tiles of one channel slice) are taken
// round-robin; the copy ring runs ahead across unit boundaries, the MMA
// thread never waits for its own MMAs, and the MMAs alternate between two
// accumulator buffers, so one unit's epilogue overlaps the next unit's
// MMAs.  Barriers: full / empty per ring stage (copies landed / MMAs done
// reading), accFull / accEmpty per accumulator buffer, drain (every MMA of
// the CTA done, before TMEM is freed).
constexpr int kEpiWarps = 4;
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr int kThreads = 32 * (kEpiWarps + 2);

__global__ void __launch_bounds__(kThreads, 1) k_conv_tc(const __grid_constant__ CUtensorMap act, TcArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  // [0, 128): barriers, the TMEM address and the abort flag; then the
  // activation stages and the weight stages
  uint64_t* full = reinterpret_cast<uint64_t*>(sm);
  uint64_t* empty = full + kMaxStages;
  uint64_t* accFull = empty + kMaxStages;
  uint64_t* accEmpty = accFull + 2;
  uint64_t* drain = accEmpty + 2;
  uint64_t* wFull = drain + 1;  // resident weights landed
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(wFull + 1);
  volatile int* abortFlag = reinterpret_cast<volatile int*>(tmemSlot + 1);
  static_assert((2 * kMaxStages + 6) * 8 + 8 <= kHeader, "barrier header");
  const int T = a.tiles, hw = haloW(T), S = a.stages;
  const uint32_t chunk = uint32_t(chunkBytes(T)), stageA = uint32_t(actStage(T));
  unsigned char* actBase = sm + kHeader;
  unsigned char* wBase = actBase + S * stageA;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbarInit(smem(&full[s]), 1);
      mbarInit(smem(&empty[s]), 1);
    }
    mbarInit(smem(wFull), 1);
    for (int b = 0; b < 2; ++b) {
      mbarInit(smem(&accFull[b]), 1);
      mbarInit(smem(&accEmpty[b]), kEpiWarps);
    }
    mbarInit(smem(drain), 1);
    // a CTA that finds an expired wait recorded skips its work: one failure
    // costs one timeout, not one per CTA
    *abortFlag = *reinterpret_cast<volatile int*>(&g_tcError) ? 1 : 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem(tmemSlot)),
                 "r"(a.tmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fenceBefore();
  __syncthreads();
  fenceAfter();
  const uint32_t tmem = *tmemSlot;
  const int groups = a.cin / 16;
  const int myUnits = blockIdx.x < a.units ? (a.units - 1 - int(blockIdx.x)) / int(gridDim.x) + 1 : 0;
  const int total = myUnits * groups;  // stream position q = (unit k of this CTA, channel group g)
  const uint32_t bufCols = uint32_t(T * a.nt);
  auto fail = [&]() {
    *abortFlag = 1;
    atomicExch(&g_tcError, 1);
  };

  if (warp == kProducerWarp) {
    if (lane == 0 && !*abortFlag) {
      if (a.resident && total > 0) {
        // the whole layer's weights (one slice), once
        mbarExpectTx(smem(wFull), uint32_t(groups) * a.wStageBytes);
        bulkLoad(smem(wBase), a.wt, uint32_t(groups) * a.wStageBytes, smem(wFull));
      }
      int q = 0;
      for (; q < total; ++q) {
        const int k = q / groups, g = q % groups, s = q % S;
        const uint32_t use = uint32_t(q / S);
        // the MMAs of this stage's previous use are done reading it
        if (use > 0 && !mbarWaitOr(smem(&empty[s]), (use - 1) & 1u, abortFlag)) break;
        const Unit U = unitOf(a, int(blockIdx.x) + k * int(gridDim.x));
        const __nv_bfloat16* wt = a.wt + size_t(U.slice) * size_t(groups) * (a.wStageBytes / 2);
        const uint32_t bar = smem(&full[s]);
        mbarExpectTx(bar, uint32_t(2 * boxBytes(T)) + (a.resident ? 0u : a.wStageBytes));
        const uint32_t dstA = smem(actBase + s * stageA);
        tmaLoad4d(dstA, &act, g * 16, U.x0 - 1, U.y0 - 1, U.img, bar);
        tmaLoad4d(dstA + chunk, &act, g * 16 + 8, U.x0 - 1, U.y0 - 1, U.img, bar);
        if (!a.resident)
          bulkLoad(smem(wBase + size_t(s) * a.wStageBytes), wt + size_t(g) * (a.wStageBytes / 2), a.wStageBytes,
                   bar);
      }
      if (q < total) fail();
      // the last copies of each stage have landed before the CTA may exit
      for (int r = q - 1; r >= 0 && r >= q - S; --r)
        mbarWaitOr(smem(&full[r % S]), uint32_t(r / S) & 1u, &kNeverAbort);
      if (a.resident && total > 0) mbarWaitOr(smem(wFull), 0u, &kNeverAbort);
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      if (!*abortFlag) {
        const uint32_t idesc = instrDesc(uint32_t(a.nt));
        const uint32_t bTap = uint32_t(2 * a.nt * 16);
        bool ok = !a.resident || total == 0 || mbarWaitOr(smem(wFull), 0u, abortFlag);
        if (!ok) fail();
        for (int q = 0; q < total && ok; ++q) {
          const int k = q / groups, g = q % groups, s = q % S;
          const uint32_t use = uint32_t(q / S), buf = uint32_t(k & 1);
          if (g == 0 && k >= 2) {
            // the epilogue has read this buffer's previous unit out
            if (!mbarWaitOr(smem(&accEmpty[buf]), uint32_t((k >> 1) - 1) & 1u, abortFlag)) {
              fail();
              break;
            }
            fenceAfter();
          }
          if (!mbarWaitOr(smem(&full[s]), use & 1u, abortFlag)) {
            fail();
            break;
          }
          fenceAfter();
          const uint32_t aBase = smem(actBase + s * stageA);
          const uint32_t bBase = smem(wBase + size_t(a.resident ? g : s) * a.wStageBytes);
          const uint32_t acc = tmem + buf * bufCols;
#pragma unroll 1
          for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3, dx = tap % 3;
            const uint64_t db = matDesc(bBase + uint32_t(tap) * bTap, uint32_t(a.nt * 16), 128u);
            // tile t: the view starting 8 t pixels further along the halo
            // rows; its accumulator is columns [t nt, (t + 1) nt) of the buffer
            for (int t2 = 0; t2 < T; ++t2) {
              const uint64_t da =
                  matDesc(aBase + uint32_t(dy * hw + dx + kTileW * t2) * 16u, chunk, uint32_t(hw * 16));
              mma(acc + uint32_t(t2 * a.nt), da, db, idesc, (g > 0 || tap > 0) ? 1u : 0u);
            }
          }
          commit(smem(&empty[s]));
          if (g == groups - 1) commit(smem(&accFull[buf]));
        }
      }
      // every MMA issued by this thread has finished before TMEM is freed
      commit(smem(drain));
      mbarWaitOr(smem(drain), 0u, &kNeverAbort);
    }
  } else {
    // epilogue: warp w owns TMEM lanes 32w..32w+31 = pixels 32w..32w+31 of each tile
    const int m = warp * 32 + lane;
    for (int k = 0; k < myUnits; ++k) {
      const uint32_t buf = uint32_t(k & 1);
      if (!mbarWaitOr(smem(&accFull[buf]), uint32_t(k >> 1) & 1u, abortFlag)) {
        if (lane == 0) fail();
        break;
      }
      fenceAfter();
      const Unit U = unitOf(a, int(blockIdx.x) + k * int(gridDim.x));
      const int n0 = U.slice * a.nt;
      const uint32_t laneBase = tmem + (uint32_t(warp * 32) << 16) + buf * bufCols;
      for (int t2 = 0; t2 < T; ++t2)
        for (int c0 = 0; c0 < a.nt; c0 += 16) {
          const int py = U.y0 + m / kTileW, px = U.x0 + kTileW * t2 + m % kTileW;
          const bool inside = py < a.h && px < a.w;
          // 16 consecutive channels of one pixel: 32 B (bf16) or 64 B (f32),
          // aligned as cout and n0 + c0 are multiples of 16
          const size_t e = ((size_t(U.img) * a.h + py) * a.w + px) * size_t(a.cout) + size_t(n0 + c0);
          float v[16];
          ld16(laneBase + uint32_t(t2 * a.nt + c0), v);
          if (!inside) continue;
          if (a.bias) {
            const float4* b4 = reinterpret_cast<const float4*>(a.bias + n0 + c0);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const float4 b = __ldg(&b4[i]);
              v[4 * i] += b.x;
              v[4 * i + 1] += b.y;
              v[4 * i + 2] += b.z;
              v[4 * i + 3] += b.w;
            }
          }
          if (a.relu) {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.0f);
          }
          if (a.mask) {
            const uint4* m4 = reinterpret_cast<const uint4*>(a.mask + e);
            const uint4 mm[2] = {m4[0], m4[1]};
            const __nv_bfloat16* mk = reinterpret_cast<const __nv_bfloat16*>(mm);
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (!(__bfloat162float(mk[i]) > 0.0f)) v[i] = 0.0f;
          }
          if (a.outF32) {
            float4* o4 = reinterpret_cast<float4*>(static_cast<float*>(a.out) + e);
#pragma unroll
            for (int i = 0; i < 4; ++i) o4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
          } else {
            uint4 pk[2];
            __nv_bfloat162* h2 = reinterpret_cast<__nv_bfloat162*>(pk);
#pragma unroll
            for (int i = 0; i < 8; ++i) h2[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
            uint4* o4 = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(a.out) + e);
            o4[0] = pk[0];
            o4[1] = pk[1];
          }
        }
      // this warp's lanes of the buffer are read: hand it back to the MMAs
      fenceBefore();
      __syncwarp();
      if (lane == 0) mbarArrive(smem(&accEmpty[buf]));
    }
  }
  fenceBefore();
  __syncthreads();
  if (warp == 0) {
    fenceAfter();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmemCols) : "memory");
  }
}

// [cout][9][cin] -> [cout/nt][cin/16][9][2][nt][8]
__global__ void k_weights_tc(const __nv_bfloat16* w, __nv_bfloat16* o, int cout, int cin, int nt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cout * 9 * cin) return;
  const int ci = i % cin, tap = (i / cin) % 9, co = i / (9 * cin);
  const int g = ci / 16, c = (ci / 8) & 1, e = ci & 7;
  const int slice = co / nt, cl = co % nt;
  o[(((((size_t(slice) * (cin / 16) + g) * 9 + tap) * 2 + c) * nt + cl) * 8) + e] = w[i];
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeFn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

}  // namespace
}  // namespace tc
}  // namespace asuna

using namespace asuna;
using namespace asuna::tc;

extern "C" {

int asuna_nn_weights_tc(void* stream, const void* w, void* wtc, int cout, int cin) {
  if (!w || !wtc || cin % 16 || cout % 16) return fail(ASUNA_ERR_INVALID, "asuna_nn_weights_tc: bad argument");
  const int n = cout * 9 * cin;
  k_weights_tc<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(w), static_cast<__nv_bfloat16*>(wtc), cout, cin, sliceWidth(cout));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ASUNA_OK : fail(ASUNA_ERR_CUDA, "asuna_nn_weights_tc: %s", cudaGetErrorString(e));
}

int asuna_nn_conv3x3_tc(void* stream, const void* in, int n, int h, int w, int cin, const void* weight_tc,
                        const float* bias, int cout, int relu, const void* mask, void* out, int out_f32) {
  if (!in || !weight_tc || !out || n <= 0 || h <= 0 || w <= 0)
    return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_tc: bad argument");
  if (cin % 16 || cout % 16)
    return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_tc: cin %% 16 and cout %% 16 required");
  // the copies and the epilogue's 16-byte loads and stores need 16-byte bases
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(weight_tc) | reinterpret_cast<uintptr_t>(bias) |
       reinterpret_cast<uintptr_t>(mask) | reinterpret_cast<uintptr_t>(out)) % 16)
    return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_tc: operands must be 16-byte aligned");
  EncodeTiledFn enc = encodeFn();
  if (!enc) return fail(ASUNA_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  int dev = 0, sms = 1, smemSm = 0, reserve = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smemSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  const int nt = sliceWidth(cout);
  const TileShape shape = tileShape(nt, cout / nt, cin / 16, w, size_t(smemSm), size_t(reserve));
  const int T = shape.T;
  // NHWC bf16 as a 4-D tensor (C, W, H, N); box = 8 channels x the T tiles' halo
  CUtensorMap map;
  const cuuint64_t dims[4] = {cuuint64_t(cin), cuuint64_t(w), cuuint64_t(h), cuuint64_t(n)};
  const cuuint64_t strides[3] = {cuuint64_t(cin) * 2, cuuint64_t(w) * cin * 2, cuuint64_t(h) * w * cin * 2};
  const cuuint32_t box[4] = {8, cuuint32_t(haloW(T)), kHaloH, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(in), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_tc: tensor map encoding failed (%d)", int(r));
  TcArgs a{};
  a.wt = static_cast<const __nv_bfloat16*>(weight_tc);
  a.bias = bias;
  a.mask = static_cast<const __nv_bfloat16*>(mask);
  a.out = out;
  a.n = n;
  a.h = h;
  a.w = w;
  a.cin = cin;
  a.cout = cout;
  a.tiles = T;
  a.tilesX = (w + kTileW * T - 1) / (kTileW * T);
  a.tilesY = (h + kTileH - 1) / kTileH;
  a.relu = relu;
  a.outF32 = out_f32;
  a.nt = nt;
  a.slices = cout / a.nt;
  a.tmemCols = pow2Cols(2 * T * nt);
  a.wStageBytes = uint32_t(wStage(a.nt));
  a.stages = shape.stages;
  a.resident = shape.resident ? 1 : 0;
  const size_t smemBytes = smemFor(a.nt, T, a.stages, shape.resident, cin / 16);
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemLimit));
    // the whole unified L1 as shared memory, so two CTAs of ~87 KB share an
    // SM (and the occupancy query below counts them)
    cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  });
  if (smemBytes > kSmemLimit) return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_tc: cout %d needs too much shared memory", cout);
  const long long units = (long long)a.tilesX * a.tilesY * n * a.slices;
  if (units > (1ll << 31) - 1) return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_tc: too many tiles");
  a.units = int(units);
  // persistent grid: the CTAs that fit on the device at once, or fewer
  // when there is less work
  const int perSm = shape.perSm;
  const long long grid = std::min<long long>(units, (long long)sms * perSm);
  k_conv_tc<<<unsigned(std::max<long long>(grid, 1)), kThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(map,
                                                                                                                 a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ASUNA_OK : fail(ASUNA_ERR_CUDA, "asuna_nn_conv3x3_tc: %s", cudaGetErrorString(e));
}

int asuna_nn_tc_status(int* expired) {
  if (!expired) return fail(ASUNA_ERR_INVALID, "null argument");
  int zero = 0;
  if (cudaMemcpyFromSymbol(expired, g_tcError, sizeof(int)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_tcError, &zero, sizeof(int)) != cudaSuccess)
    return fail(ASUNA_ERR_CUDA, "asuna_nn_tc_status: %s", cudaGetErrorString(cudaGetLastError()));
  return ASUNA_OK;
}

}  // extern "C"
