// dev_types.h — data layout of a scene, a film and the wavefront queues in HBM.
//
// Shared by the host C++ code and the CUDA kernels.  Everything the traversal
// and shading kernels read per ray is 16-byte aligned so each record is moved
// with 128-bit loads.
#pragma once
#include <cstdint>

#include <vector_types.h>

#include "../../include/asuna_rt.h"

namespace asuna {

// ---- acceleration structure -------------------------------------------------
// Binary BVH node, 64 B: the two child boxes, then the child references.
// ref >= 0: inner node index; ref < 0: leaf, decoded by leafFirst/leafCount
// (BLAS: first triangle, count <= 8; TLAS: instance).  The planes are laid
// out in (x, y) pairs and a z quad, so the traversal computes the six slab
// distances of a child with three packed two-lane operations against the
// ray's (o.x, o.y) / (o.z, o.z) pairs.
struct __align__(16) BvhNode {
  float4 xy[2];  // child c: lo.x, lo.y, hi.x, hi.y
  float4 zs;     // c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z
  int4 ref;      // c0, c1, unused, unused
};
static_assert(sizeof(BvhNode) == 64, "BvhNode is 64 bytes");

inline __host__ __device__ void nodeSetBox(BvhNode& n, int c, const float* lo, const float* hi) {
  n.xy[c].x = lo[0];
  n.xy[c].y = lo[1];
  n.xy[c].z = hi[0];
  n.xy[c].w = hi[1];
  float* z = &n.zs.x;
  z[2 * c] = lo[2];
  z[2 * c + 1] = hi[2];
}
inline __host__ __device__ void nodeGetBox(const BvhNode& n, int c, float* lo, float* hi) {
  const float* z = &n.zs.x;
  lo[0] = n.xy[c].x;
  lo[1] = n.xy[c].y;
  lo[2] = z[2 * c];
  hi[0] = n.xy[c].z;
  hi[1] = n.xy[c].w;
  hi[2] = z[2 * c + 1];
}

constexpr int kMaxLeafTris = 8;
constexpr int32_t kStackSentinel = INT32_MIN;  // "leave the BLAS" marker
inline __host__ __device__ int32_t encodeLeaf(uint32_t first, uint32_t count) {
  return ~int32_t(first * 8u + (count - 1u));
}
inline __host__ __device__ uint32_t leafFirst(int32_t ref) { return uint32_t(~ref) >> 3; }
inline __host__ __device__ uint32_t leafCount(int32_t ref) { return (uint32_t(~ref) & 7u) + 1u; }
constexpr uint32_t kMaxLeafFirst = (1u << 28) - 1u;

// Leaf triangle in BVH order, 48 B: object-space vertices; v0.w holds the
// mesh-local primitive id (float bits).
struct __align__(16) TriDev {
  float4 v0, v1, v2;
};

// Shading vertex, 32 B: (pos.xyz, uv.x), (normal.xyz, uv.y).
struct __align__(16) VtxDev {
  float4 pu;
  float4 nv;
};

// Instance record, 128 B.
struct __align__(16) InstDev {
  float4 w2o[3];  // world -> object rows (double inverse rounded once)
  float4 o2w[3];  // object -> world rows (as given)
  int32_t blasRoot;  // inner-node index of the mesh BLAS (-1: empty mesh)
  uint32_t vtxBase;  // first vertex of the mesh in the vertex arrays
  uint32_t idxBase;  // first triangle of the mesh in the index array
  int32_t matId;     // material (-1 for emitters)
  int32_t lightId;   // >= 0: emitter instance
  uint32_t matType;
  uint32_t pad[2];
};
static_assert(sizeof(InstDev) == 128, "InstDev is 128 bytes");

// Packed material, 96 B: (diffuse.xyz, type bits), (alpha.x, alpha.y, ior,
// fdrInt), (radiance.xyz, 0), (radiance_factor.xyz, 0); an emissive material
// holds its radiance in place of the diffuse albedo; conductors keep eta in
// radiance and k in radiance_factor, as the reference's loader does (other
// types pack their own fields into b, c, d: see the upload).  Texture ids
// (-1 = none): t0 = (diffuse, normal, roughness, metalness), t1 = (radiance,
// tangent, opacity, -).
struct __align__(16) MatDev {
  float4 a;
  float4 b;
  float4 c;
  float4 d;
  int4 t0;
  int4 t1;
};

// Packed light, 80 B: (position, type bits), (direction, radius),
// (radiance, 0), (u, area), (v, doubleSide bits).
struct __align__(16) LightDev {
  float4 pos;
  float4 dir;
  float4 rad;
  float4 u;
  float4 v;
};

// Device view of one uploaded scene.
struct SceneDev {
  const BvhNode* nodes;  // all BLAS nodes, then the TLAS nodes
  const TriDev* tris;
  const VtxDev* vtx;
  const uint4* idx;  // mesh-local vertex indices (x, y, z), w unused
  const InstDev* inst;
  const MatDev* mats;
  const LightDev* lights;
  const float4* env;    // W*H rgba
  const float2* marg;   // W*H (.x inverse CDF, .y pdf)
  const float2* cond;   // W*H
  const float4* texels;  // every material texture, one after another
  const int4* texInfo;   // per texture: (first texel, width, height, 0)
  float4 boundLo;        // world bounds of the instances (xyz) ...
  float4 cellScale;      // ... and 4 / extent per axis: the ray-sort origin cells
  int32_t tlasRoot;
  int32_t envW, envH;
  int32_t numInst;
  uint32_t classMask;  // shading classes some instance can reach (bit k = class k)
  uint32_t passThrough;  // 1: some material can pass rays through (opacity)
  asuna_sun_and_sky sky;  // in_use = 1: the sun & sky replaces the environment map
};
// Wavefront passes of a batch: one per bounce, plus the pass-through reserve.
inline int wavefrontPasses(int maxDepth, const SceneDev& S) {
  return maxDepth + (S.passThrough ? ASUNA_MAX_PASS_THROUGH : 0);
}
// Path info word y: lobe flags in the low 16 bits, pass-throughs so far above.
constexpr uint32_t kFlagsMask = 0xffffu;
constexpr int kPassShift = 16;

// ---- shots, films, batches ----------------------------------------------------
struct __align__(16) ShotDev {
  asuna_camera cam;       // 224 B
  asuna_rt_state state;   // 84 B
  uint32_t width, height;
  uint32_t seed, flags;
  uint32_t rrDepth;
  int32_t depthSlot;
  float4* filmRad;        // image 0
  float4* filmW;          // image 8
  float4* filmCh;         // images 1..7, contiguous (7 * W * H)
};

// A contiguous run of paths: frames [frameBegin, frameBegin + nframes) of
// one shot, all pixels, path index = pathBegin + (frame - frameBegin) * npix + pixel.
struct __align__(16) RangeDev {
  uint32_t pathBegin;
  uint32_t shot;
  uint32_t frameBegin;
  uint32_t nframes;
  uint32_t npix;
  uint32_t pad[3];
};

// Counters in device memory.
enum CounterSlot {
  kCntExtend0 = 0,  // rays in extend queue 0
  kCntExtend1 = 1,  // rays in extend queue 1
  kCntShadow = 2,   // rays in the shadow queue
  kCntFetchExtend = 3,
  kCntFetchShadow = 4,
  kCntCls0 = 5,  // rays per shading class (kNumShadeClasses slots)
  kCntNum32 = 24
};

// Shading classes: the hits of an extend pass are split by what shades them,
// so every shading kernel runs one material's code with full warps.
enum ShadeClass {
  kClsTerminal = 0,    // miss, light hit, emissive surface: the path ends
  kClsLambertian = 1,
  kClsRoughPlastic = 2,
  kClsDielectric = 3,
  kClsPlastic = 4,
  kClsMirror = 5,
  kClsConductor = 6,
  kClsRoughConductor = 7,
  kClsPhong = 8,
  kClsPbr = 9,  // brdf_pbr_metalness_roughness
  kClsDisney = 10,
  kClsKang18 = 11,
  kNumShadeClasses = 12
};
static_assert(kCntCls0 + kNumShadeClasses <= kCntNum32, "class counters exceed the counter page's slots");
// The class that shades a hit on a surface of material `type` (not a light).
#if defined(__CUDACC__)
__host__ __device__
#endif
inline int shadeClassOf(uint32_t type) {
  switch (type) {
    case ASUNA_MAT_ROUGH_PLASTIC: return kClsRoughPlastic;
    case ASUNA_MAT_DIELECTRIC: return kClsDielectric;
    case ASUNA_MAT_PLASTIC: return kClsPlastic;
    case ASUNA_MAT_MIRROR: return kClsMirror;
    case ASUNA_MAT_CONDUCTOR: return kClsConductor;
    case ASUNA_MAT_ROUGH_CONDUCTOR: return kClsRoughConductor;
    case ASUNA_MAT_PHONG: return kClsPhong;
    case ASUNA_MAT_PBR_METALNESS_ROUGHNESS: return kClsPbr;
    case ASUNA_MAT_DISNEY: return kClsDisney;
    case ASUNA_MAT_KANG18: return kClsKang18;
    case ASUNA_MAT_EMISSIVE: return kClsTerminal;
    default: return kClsLambertian;
  }
}
// Ray-queue sort: key = direction octant and an origin cell (at most 4,096
// keys).
constexpr int kSortKeys = 4096;
struct DevCounters {
  uint32_t c[kCntNum32];
  uint32_t sortHist[kSortKeys];    // rays per key (zeroed by the scan after use)
  uint32_t sortCursor[kSortKeys];  // next slot per key while scattering
  unsigned long long extendRays;
  unsigned long long shadowRays;
  unsigned long long nodes;   // closest-hit traversal
  unsigned long long tris;
  unsigned long long paths;
  unsigned long long shNodes;  // occlusion traversal
  unsigned long long shTris;
  // traversals cut short by a full stack or a loop bound (must stay 0);
  // last, so the render statistics can be cleared without it: the count
  // only grows, and the host reports each increase as a render error
  unsigned long long stackOverflow;
};

struct __align__(32) PathDev {
  float4 thp;
  uint4 info;
};
static_assert(sizeof(PathDev) == 32, "PathDev is 32 bytes");

// Wavefront buffers (structure of arrays, indexed by queue slot or path).
struct WaveDev {
  // extend queues (ping-pong): (o.xyz, tmax), (d.xyz, path index bits)
  float4* rayO[2];
  float4* rayD[2];
  // closest-hit results of the current extend queue: (t, u, v, prim bits), inst
  float4* hit;
  uint32_t* hitInst;
  // shadow queue: (o.xyz, tmax), (d.xyz, path bits), (contribution.xyz, 0)
  float4* shO;
  float4* shD;
  float4* shC;
  // path state.  The shading passes reach it by path index, scattered: the
  // throughput and the path's counters share one 32-byte record (one sector
  // per gather instead of two); the radiance stays an array of its own, as
  // the occlusion pass adds to it and the accumulation reads it in path
  // order; the parity records are only written when asked for.
  PathDev* path;  // thp = throughput.xyz, pdf of the last BSDF sample;
                  // info = seed, last BSDF lobe flags, range index, local index
  float4* rad;    // radiance.xyz, filter weight
  uint4* rec;     // parity records: signature, unoccluded bits, shadow bits, depth
  uint32_t* cls[kNumShadeClasses];  // extend-queue indices of each shading class
  DevCounters* cnt;
  const RangeDev* ranges;
  const ShotDev* shots;
  uint32_t numRanges;
  uint32_t numPaths;
};

}  // namespace asuna
