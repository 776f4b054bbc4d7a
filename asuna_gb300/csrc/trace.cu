// trace.cu — two-level BVH traversal kernels (closest hit and occlusion).
//
// Software replacement for the RT-core traversal behind traceRayEXT
// (src/shaders/raytrace.projective.rgen:108-109 closest hit with tmin 1e-5 and
// tmax 1e10; rgen:117-122 occlusion with tmin 0, tmax dist - 2*EPS,
// terminate-on-first-hit).  Facing culling is off, as the reference's
// instances set VK_GEOMETRY_INSTANCE_TRIANGLE_FACING_CULL_DISABLE_BIT_KHR
// (src/pipeline/pipeline_raytrace.cpp:132).
//
// Persistent warps refill their idle lanes from the queue (one atomic per
// refill and warp); each thread walks TLAS -> BLAS with a per-thread stack
// in shared memory (entry k of thread t at sstack[k * TB + t], bank-conflict
// free) that spills into thread-local memory past its shared part.  Node and
// triangle records are read with 128-bit read-only loads; the slab distances
// of a node are computed with packed two-lane (f32x2) arithmetic.  The ray is
// moved into object space and tested against triangles with the watertight
// algorithm of Woop, Benthin and Wald (JCGT 2013) using explicitly rounded
// operations, so the hits equal the CPU oracle's bit for bit; box tests use
// (lo - o) * (1/d) with the far distance widened by 2^-20, which keeps them
// conservative.
#include <cuda_runtime.h>

#include "kernels.h"

namespace asuna {
namespace {

struct WT {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

__device__ __forceinline__ float sel(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ WT wtPre(float3 d) {
  WT w;
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  float dz = sel(d, kz);
  if (dz < 0.0f) {
    int t = kx;
    kx = ky;
    ky = t;
  }
  w.kx = kx;
  w.ky = ky;
  w.kz = kz;
  w.Sx = __fdiv_rn(sel(d, kx), dz);
  w.Sy = __fdiv_rn(sel(d, ky), dz);
  w.Sz = __fdiv_rn(1.0f, dz);
  return w;
}

// Watertight test; same operations and order as the CPU oracle.
__device__ __forceinline__ bool wtTri(const WT& w, float3 o, float4 p0, float4 p1, float4 p2, float tmin, float tmax,
                                      float& t, float& b1, float& b2) {
  const float3 A = make_float3(__fsub_rn(p0.x, o.x), __fsub_rn(p0.y, o.y), __fsub_rn(p0.z, o.z));
  const float3 B = make_float3(__fsub_rn(p1.x, o.x), __fsub_rn(p1.y, o.y), __fsub_rn(p1.z, o.z));
  const float3 C = make_float3(__fsub_rn(p2.x, o.x), __fsub_rn(p2.y, o.y), __fsub_rn(p2.z, o.z));
  const float Akz = sel(A, w.kz), Bkz = sel(B, w.kz), Ckz = sel(C, w.kz);
  const float Ax = __fsub_rn(sel(A, w.kx), __fmul_rn(w.Sx, Akz)), Ay = __fsub_rn(sel(A, w.ky), __fmul_rn(w.Sy, Akz));
  const float Bx = __fsub_rn(sel(B, w.kx), __fmul_rn(w.Sx, Bkz)), By = __fsub_rn(sel(B, w.ky), __fmul_rn(w.Sy, Bkz));
  const float Cx = __fsub_rn(sel(C, w.kx), __fmul_rn(w.Sx, Ckz)), Cy = __fsub_rn(sel(C, w.ky), __fmul_rn(w.Sy, Ckz));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = __double2float_rn(__dsub_rn(__dmul_rn(double(Cx), double(By)), __dmul_rn(double(Cy), double(Bx))));
    V = __double2float_rn(__dsub_rn(__dmul_rn(double(Ax), double(Cy)), __dmul_rn(double(Ay), double(Cx))));
    W = __double2float_rn(__dsub_rn(__dmul_rn(double(Bx), double(Ay)), __dmul_rn(double(By), double(Ax))));
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = __fadd_rn(__fadd_rn(U, V), W);
  if (det == 0.0f) return false;
  const float Az = __fmul_rn(w.Sz, Akz), Bz = __fmul_rn(w.Sz, Bkz), Cz = __fmul_rn(w.Sz, Ckz);
  const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
  const float rcp = __fdiv_rn(1.0f, det);
  const float tt = __fmul_rn(T, rcp);
  if (!(tt >= tmin && tt <= tmax)) return false;
  t = tt;
  b1 = __fmul_rn(V, rcp);
  b2 = __fmul_rn(W, rcp);
  return true;
}

// Three-input min / max (one instruction each on sm_100 and later; exact,
// like fminf / fmaxf, for the finite values the slab test produces).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Inverse direction for the slab tests, from the hardware reciprocal
// (rcp.approx, within one ulp of 1/x for the normal values it is given):
// the box tests stay conservative, as the far distance is widened by 2^-20
// (16 ulp), far more than the reciprocal's error; hits come from the
// watertight triangle test alone, so they do not depend on it.
__device__ __forceinline__ float rcpApprox(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// (magnitudes clamped to [1e-30, 1e30], so the reciprocal stays a normal
// number that the flush-to-zero form returns unchanged)
__device__ __forceinline__ float3 safeInv(float3 d) {
  auto inv = [](float x) { return rcpApprox(copysignf(fminf(fmaxf(fabsf(x), 1e-30f), 1e30f), x)); };
  return make_float3(inv(d.x), inv(d.y), inv(d.z));
}

// Packed pairs of IEEE single-precision values in one 64-bit register pair:
// the f32x2 add / mul of sm_100 and later issue as one instruction and round
// each lane to nearest, like the scalar operations they replace, so the slab
// distances are bit-identical to (plane - o) * (1/d) computed one by one.
typedef unsigned long long F2;
__device__ __forceinline__ F2 pack2(float a, float b) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void unpack2(F2 p, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(p));
}
// (planes - o) * inv, lane by lane; returns the two distances
__device__ __forceinline__ void slab2(F2 planes, F2 o, F2 inv, float& t0, float& t1) {
  F2 d, t;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(planes), "l"(o));
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(d), "l"(inv));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(t0), "=f"(t1) : "l"(t));
}

__device__ __forceinline__ void xformRay(const float4* w, float3 o, float3 d, float3& oo, float3& dd) {
  float4 r0 = __ldg(&w[0]), r1 = __ldg(&w[1]), r2 = __ldg(&w[2]);
  auto po = [&](float4 r) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.x, o.x), __fmul_rn(r.y, o.y)), __fmul_rn(r.z, o.z)), r.w);
  };
  auto pd = [&](float4 r) { return __fadd_rn(__fadd_rn(__fmul_rn(r.x, d.x), __fmul_rn(r.y, d.y)), __fmul_rn(r.z, d.z)); };
  oo = make_float3(po(r0), po(r1), po(r2));
  dd = make_float3(pd(r0), pd(r1), pd(r2));
}

constexpr float kFarScale = 1.00000095367431640625f;  // 1 + 2^-20
constexpr int32_t kDone = INT32_MIN + 1;               // stack empty: traversal over
constexpr int32_t kNoLeaf = INT32_MIN + 2;             // no postponed leaf
constexpr uint32_t kTraceSpinCap = 1u << 20;           // inner steps of one warp pass
constexpr uint32_t kTraceRayCap = 1u << 16;            // leaves + transitions of one ray

__device__ __forceinline__ bool isLeafRef(int32_t r) { return r < 0 && r != kStackSentinel && r != kDone; }

struct HitOut {
  float u, v;  // (the distance is the traversal's `best`)
  uint32_t prim, inst;
};

// Traversal state of one ray (while-while traversal with postponed leaves,
// after Aila and Laine, "Understanding the efficiency of ray traversal on
// GPUs", HPG 2009).  innerStep() visits one inner node; a BLAS leaf met
// there is postponed and, when `speculate`, the lane goes on visiting inner
// nodes while other lanes of the warp still look for a leaf.  leafOrMove()
// then tests the triangles of one leaf, or makes one TLAS/BLAS transition.
//
// The state is kept small (the kernel is bound by the latency of its node
// fetches, so resident warps matter): the world-space ray is read again from
// its source at the few instance transitions instead of being held, the
// watertight test's axis permutation is packed into one word, the closest
// distance is `best`, and the stack cap comes from the launch.
template <int TB, int SHS>  // threads per block, stack entries in shared memory
struct Trav {
  F2 oxy, oz2;  // ray origin in the current space: (o.x, o.y), (o.z, o.z)
  F2 ixy, iz2;  // inverse direction in the current space, likewise
  float Sx, Sy, Sz;  // watertight shear of the current space's direction
  uint32_t kxyz;     // its axis permutation, kx | ky << 2 | kz << 4
  float tmin, best;
  uint32_t curInst;
  int sp;  // stack entries in use
  int32_t ref, leaf;
  bool found, inBlas;
  HitOut h;

  __device__ __forceinline__ void setShear(const WT& w) {
    Sx = w.Sx;
    Sy = w.Sy;
    Sz = w.Sz;
    kxyz = uint32_t(w.kx) | uint32_t(w.ky) << 2 | uint32_t(w.kz) << 4;
  }
  __device__ __forceinline__ WT shear() const {
    WT w;
    w.kx = int(kxyz & 3u);
    w.ky = int((kxyz >> 2) & 3u);
    w.kz = int(kxyz >> 4);
    w.Sx = Sx;
    w.Sy = Sy;
    w.Sz = Sz;
    return w;
  }

  __device__ __forceinline__ void init(const SceneDev& S, float3 ro, float3 rd, float t0, float t1) {
    setSpace(ro, safeInv(rd));
    tmin = t0;
    best = t1;
    curInst = 0;
    sp = 0;
    ref = S.tlasRoot;
    leaf = kNoLeaf;
    found = false;
    inBlas = false;
  }

  __device__ __forceinline__ void setSpace(float3 o, float3 inv) {
    oxy = pack2(o.x, o.y);
    oz2 = pack2(o.z, o.z);
    ixy = pack2(inv.x, inv.y);
    iz2 = pack2(inv.z, inv.z);
  }
  __device__ __forceinline__ float3 origin() const {
    float x, y, z, z2;
    unpack2(oxy, x, y);
    unpack2(oz2, z, z2);
    return make_float3(x, y, z);
  }

  // Stack: the first SHS entries in shared memory (stride TB: bank-conflict
  // free), deeper ones in thread-local memory.
  __device__ __forceinline__ void push(int32_t* sh, int32_t* loc, int32_t v, int lim, bool& ovf) {
    if (sp >= lim) {
      ovf = true;
      return;
    }
    if (sp < SHS)
      sh[sp * TB] = v;
    else
      loc[sp - SHS] = v;
    ++sp;
  }
  __device__ __forceinline__ int32_t popOrDone(const int32_t* sh, const int32_t* loc) {
    if (sp == 0) return kDone;
    --sp;
    return sp < SHS ? sh[sp * TB] : loc[sp - SHS];
  }

  template <bool COUNT>
  __device__ __forceinline__ void innerStep(const SceneDev& S, int32_t* sh, int32_t* loc, int lim, uint32_t& nNodes,
                                            bool& ovf) {
    const BvhNode* n = S.nodes + ref;
    // the 16-byte plane records as pairs: (lo.x, lo.y), (hi.x, hi.y) of
    // each child; (lo.z, hi.z) of child 0, of child 1
    const ulonglong2 c0 = __ldg(reinterpret_cast<const ulonglong2*>(&n->xy[0]));
    const ulonglong2 c1 = __ldg(reinterpret_cast<const ulonglong2*>(&n->xy[1]));
    const ulonglong2 zs = __ldg(reinterpret_cast<const ulonglong2*>(&n->zs));
    const int4 rr = __ldg(&n->ref);
    if (COUNT) ++nNodes;
    float tx0, tx1, ty0, ty1, tz0, tz1, ux0, ux1, uy0, uy1, uz0, uz1;
    slab2(c0.x, oxy, ixy, tx0, ty0);
    slab2(c0.y, oxy, ixy, tx1, ty1);
    slab2(zs.x, oz2, iz2, tz0, tz1);
    slab2(c1.x, oxy, ixy, ux0, uy0);
    slab2(c1.y, oxy, ixy, ux1, uy1);
    slab2(zs.y, oz2, iz2, uz0, uz1);
    const float a0 = fmax3(fminf(tx0, tx1), fminf(ty0, ty1), fmaxf(fminf(tz0, tz1), tmin));
    const float a1 = fmin3(fmaxf(tx0, tx1), fmaxf(ty0, ty1), fminf(fmaxf(tz0, tz1), best)) * kFarScale;
    const float b0 = fmax3(fminf(ux0, ux1), fminf(uy0, uy1), fmaxf(fminf(uz0, uz1), tmin));
    const float b1 = fmin3(fmaxf(ux0, ux1), fmaxf(uy0, uy1), fminf(fmaxf(uz0, uz1), best)) * kFarScale;
    const bool h0 = a0 <= a1, h1 = b0 <= b1;
    if (h0 && h1) {
      const bool swap = b0 < a0;
      push(sh, loc, swap ? rr.x : rr.y, lim, ovf);
      ref = swap ? rr.y : rr.x;
    } else if (h0 || h1) {
      ref = h0 ? rr.x : rr.y;
    } else {
      ref = popOrDone(sh, loc);
    }
    if (inBlas && leaf == kNoLeaf && isLeafRef(ref)) {
      leaf = ref;  // postpone: test it together with the other lanes' leaves
      ref = popOrDone(sh, loc);
    }
  }

  // Returns true when the traversal is over.  `src.world(i, o, d)` gives
  // ray i's world-space origin and direction again.
  template <bool ANY, bool COUNT, class Src>
  __device__ __forceinline__ bool leafOrMove(const SceneDev& S, const Src& src, uint32_t idx, int32_t* sh,
                                             int32_t* loc, int lim, uint32_t& nTris, bool& ovf) {
    int32_t L = kNoLeaf;
    if (leaf != kNoLeaf) {
      L = leaf;
      leaf = kNoLeaf;
    } else if (inBlas && isLeafRef(ref)) {
      L = ref;
      ref = popOrDone(sh, loc);
    }
    if (L != kNoLeaf) {
      const uint32_t first = leafFirst(L), cnt = leafCount(L);
      const WT wt = shear();
      const float3 o = origin();
      for (uint32_t k = 0; k < cnt; ++k) {
        const TriDev* tr = S.tris + first + k;
        const float4 p0 = __ldg(&tr->v0), p1 = __ldg(&tr->v1), p2 = __ldg(&tr->v2);
        if (COUNT) ++nTris;
        float t, b1, b2;
        if (wtTri(wt, o, p0, p1, p2, tmin, best, t, b1, b2)) {
          if (ANY) {
            found = true;
            return true;
          }
          const uint32_t prim = __float_as_uint(p0.w);
          // exact ties resolve to the lowest (instance, primitive), so the
          // result does not depend on traversal order
          if (!found || t < best || (curInst < h.inst || (curInst == h.inst && prim < h.prim))) {
            found = true;
            best = t;
            h.u = b1;
            h.v = b2;
            h.prim = prim;
            h.inst = curInst;
          }
        }
      }
      return false;
    }
    if (ref == kDone) return true;
    if (ref == kStackSentinel) {
      // leaving a BLAS: back to the world-space ray
      inBlas = false;
      float3 wo, wd;
      src.world(idx, wo, wd);
      setSpace(wo, safeInv(wd));
      ref = popOrDone(sh, loc);
      return false;
    }
    // TLAS leaf: enter the instance's BLAS in object space
    curInst = leafFirst(ref);
    const InstDev* in = S.inst + curInst;
    const int32_t root = __ldg(&in->blasRoot);
    if (root >= 0 && sp < lim) {
      float3 wo, wd, o, d;
      src.world(idx, wo, wd);
      xformRay(in->w2o, wo, wd, o, d);
      setSpace(o, safeInv(d));
      setShear(wtPre(d));
      inBlas = true;
      push(sh, loc, kStackSentinel, lim, ovf);
      ref = root;
      return false;
    }
    if (root >= 0) ovf = true;
    ref = popOrDone(sh, loc);
    return false;
  }
};

// Persistent warp over a ray source.  Lanes whose ray is finished take the
// next rays of the source (one fetch per refill, per warp) while the other
// lanes keep traversing.  Src supplies count, fetch(n) -> first index (called
// by one lane), commit(first, n) (called by every lane), load(i, tr) and
// finish(i, tr).
template <bool ANY, bool COUNT, bool SPEC, int TB, int SHS, class Src>
__device__ __forceinline__ void traceWarp(const SceneDev& S, Src& src, int32_t* sh, int32_t* loc, uint32_t refill,
                                          int lim, uint32_t& nNodes, uint32_t& nTris, bool& ovf) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lanesBelow = (1u << lane) - 1u;
  bool active = false, drained = false;
  uint32_t idx = 0, events = 0;
  Trav<TB, SHS> tr;
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (idle && !drained && (uint32_t(__popc(idle)) >= refill || idle == 0xffffffffu)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (int(lane) == leader) base = src.fetch(uint32_t(__popc(idle)));
      base = __shfl_sync(0xffffffffu, base, leader);
      src.commit(base, uint32_t(__popc(idle)));
      drained = base + uint32_t(__popc(idle)) >= src.count;
      if (!active) {
        const uint32_t r = base + uint32_t(__popc(idle & lanesBelow));
        if (r < src.count) {
          idx = r;
          active = true;
          events = 0;
          src.load(S, r, tr);
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) {
      if (drained) break;
      continue;
    }
    // inner nodes until every lane holds a leaf (or waits at a transition)
    // (lanes without a leaf make progress every iteration, so the loop ends;
    // with SPEC the others walk on speculatively meanwhile).  Both loops
    // carry a bound far above any real traversal: past it the warp stops
    // and reports the error instead of running on.
    uint32_t spin = 0;
    for (;;) {
      const bool stepping = active && tr.ref >= 0;
      const bool needy = stepping && tr.leaf == kNoLeaf;
      if (!__any_sync(0xffffffffu, needy)) break;
      if (++spin > kTraceSpinCap) break;
      if (SPEC ? stepping : needy) tr.template innerStep<COUNT>(S, sh, loc, lim, nNodes, ovf);
    }
    if (spin > kTraceSpinCap) {
      ovf = true;
      break;
    }
    if (active && (tr.template leafOrMove<ANY, COUNT>(S, src, idx, sh, loc, lim, nTris, ovf) ||
                   ++events > kTraceRayCap)) {
      if (events > kTraceRayCap) ovf = true;
      active = false;
      src.finish(idx, tr);
    }
  }
}

// Ray queue of a wavefront pass.
template <bool ANY>
struct QueueSrc {
  const WaveDev* W;
  const KParams* P;
  const float4 *rO, *rD;
  uint32_t* fetchCtr;
  uint32_t count;
  __device__ __forceinline__ uint32_t fetch(uint32_t n) { return atomicAdd(fetchCtr, n); }
  __device__ __forceinline__ void commit(uint32_t, uint32_t) {}
  template <class T>
  __device__ __forceinline__ void load(const SceneDev& S, uint32_t r, T& tr) {
    const float4 o4 = __ldg(&rO[r]);
    const float4 d4 = __ldg(&rD[r]);
    if (ANY)
      tr.init(S, make_float3(o4.x, o4.y, o4.z), make_float3(d4.x, d4.y, d4.z), 0.0f, o4.w);
    else
      tr.init(S, make_float3(o4.x, o4.y, o4.z), make_float3(d4.x, d4.y, d4.z), 0.00001f, 10000000000.0f);
  }
  __device__ __forceinline__ void world(uint32_t r, float3& o, float3& d) const {
    const float4 o4 = __ldg(&rO[r]);
    const float4 d4 = __ldg(&rD[r]);
    o = make_float3(o4.x, o4.y, o4.z);
    d = make_float3(d4.x, d4.y, d4.z);
  }
  template <class T>
  __device__ __forceinline__ void finish(uint32_t i, const T& tr) {
    if (ANY) {
      if (!tr.found) {
        const uint32_t p = __float_as_uint(__ldg(&rD[i].w));
        const float4 c = __ldg(&W->shC[i]);
        float4 r = W->rad[p];
        r.x = r.x + c.x;
        r.y = r.y + c.y;
        r.z = r.z + c.z;
        W->rad[p] = r;
        if (P->records) W->rec[p].y |= 1u << (P->depth - (W->path[p].info.y >> kPassShift) - 1u);
      }
    } else if (tr.found) {
      W->hit[i] = make_float4(tr.best, tr.h.u, tr.h.v, __uint_as_float(tr.h.prim));
      W->hitInst[i] = tr.h.inst;
    } else {
      W->hit[i] = make_float4(-1.0f, 0.0f, 0.0f, 0.0f);
      W->hitInst[i] = 0xffffffffu;
    }
  }
};

// TB: threads per block; MINB: resident blocks per SM the variant is
// compiled for (its register cap); SHS: stack entries in shared memory
template <bool ANY, bool COUNT, bool SPEC, int TB, int MINB, int SHS>
__global__ void __launch_bounds__(TB, MINB) k_trace(KParams P) {
  __shared__ int32_t sstack[SHS * TB];
  int32_t lstack[kStackDepth - SHS];
  int32_t* sh = sstack + threadIdx.x;
  const WaveDev& W = P.W;
  const int cur = P.cur;
  uint32_t* countPtr = ANY ? &W.cnt->c[kCntShadow] : &W.cnt->c[kCntExtend0 + cur];
  QueueSrc<ANY> src;
  src.W = &P.W;
  src.P = &P;
  src.fetchCtr = ANY ? &W.cnt->c[kCntFetchShadow] : &W.cnt->c[kCntFetchExtend];
  src.count = *countPtr;
  src.rO = ANY ? W.shO : W.rayO[cur];
  src.rD = ANY ? W.shD : W.rayD[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (ANY) {
      W.cnt->shadowRays += src.count;
      W.cnt->c[kCntFetchExtend] = 0;  // the next extend pass fetches from 0
    } else {
      W.cnt->extendRays += src.count;
      W.cnt->c[kCntExtend0 + (cur ^ 1)] = 0;  // shade appends into the other queue
      W.cnt->c[kCntShadow] = 0;
      for (int k = 0; k < kNumShadeClasses; ++k) W.cnt->c[kCntCls0 + k] = 0;  // classify appends
    }
  }
  uint32_t nNodes = 0, nTris = 0;
  bool ovf = false;
  // (the instrumented variant walks without speculation, so its node counts
  // are those of the ordered traversal)
  // (P.stackLimit is in [1, kStackDepth]: the host clamps it)
  traceWarp<ANY, COUNT, SPEC, TB, SHS>(P.S, src, sh, lstack, P.refillLanes, P.stackLimit, nNodes, nTris, ovf);
  if (ovf) atomicAdd(&W.cnt->stackOverflow, 1ull);
  if (COUNT) {
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long a = nNodes, b = nTris;
    for (int off = 16; off; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if (lane == 0) {
      atomicAdd(ANY ? &W.cnt->shNodes : &W.cnt->nodes, a);
      atomicAdd(ANY ? &W.cnt->shTris : &W.cnt->tris, b);
    }
  }
}

// Rays given as arrays (asuna_scene_trace): each warp walks its own
// contiguous slice of the rays with the same warp loop.
struct ArraySrc {
  const float4 *o, *d;
  float4* hit;
  uint32_t* inst;
  uint32_t cursor, count;
  int anyHit;
  __device__ __forceinline__ uint32_t fetch(uint32_t) { return cursor; }
  // every lane of the warp advances its copy of the cursor alike
  __device__ __forceinline__ void commit(uint32_t base, uint32_t n) { cursor = base + n; }
  template <class T>
  __device__ __forceinline__ void load(const SceneDev& S, uint32_t r, T& tr) {
    const float4 o4 = o[r], d4 = d[r];
    tr.init(S, make_float3(o4.x, o4.y, o4.z), make_float3(d4.x, d4.y, d4.z), o4.w, d4.w);
  }
  __device__ __forceinline__ void world(uint32_t r, float3& wo, float3& wd) const {
    const float4 o4 = o[r], d4 = d[r];
    wo = make_float3(o4.x, o4.y, o4.z);
    wd = make_float3(d4.x, d4.y, d4.z);
  }
  template <class T>
  __device__ __forceinline__ void finish(uint32_t i, const T& tr) {
    if (tr.found) {
      hit[i] = anyHit ? make_float4(1.0f, 0.0f, 0.0f, 0.0f)
                      : make_float4(tr.best, tr.h.u, tr.h.v, __uint_as_float(tr.h.prim));
      inst[i] = anyHit ? 0u : tr.h.inst;
    } else {
      hit[i] = make_float4(-1.0f, 0.0f, 0.0f, 0.0f);
      inst[i] = 0xffffffffu;
    }
  }
};

__global__ void __launch_bounds__(kTraceThreads) k_query(SceneDev S, const float4* o, const float4* d, uint32_t n,
                                                         int anyHit, float4* hit, uint32_t* inst) {
  __shared__ int32_t sstack[kSharedStack * kTraceThreads];
  int32_t lstack[kStackDepth - kSharedStack];
  int32_t* sh = sstack + threadIdx.x;
  const uint32_t warps = gridDim.x * (blockDim.x / 32u);
  const uint32_t w = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
  const uint32_t per = (n + warps - 1) / warps;
  const uint32_t lo = min(n, w * per), hi = min(n, lo + per);
  // indices are relative to the slice
  ArraySrc src{o + lo, d + lo, hit + lo, inst + lo, 0u, hi - lo, anyHit};
  uint32_t a = 0, b = 0;
  bool ovf = false;
  if (anyHit)
    traceWarp<true, false, true, kTraceThreads, kSharedStack>(S, src, sh, lstack, kRefillLanes, kStackDepth, a, b,
                                                              ovf);
  else
    traceWarp<false, false, true, kTraceThreads, kSharedStack>(S, src, sh, lstack, kRefillLanes, kStackDepth, a, b,
                                                               ovf);
}

}  // namespace

namespace {
// Kernel variants: threads per block (64, 128, 256) x resident warps per SM
// (32, 40, 48: the occupancy class 8, 10, 12 of 128-thread blocks) x stack
// entries in shared memory (16, 24, 32).
template <bool ANY, int TB, int OCC, int SHS>
void launchShape(const KParams& P, int grid, cudaStream_t s) {
  constexpr int MINB = OCC * 128 / TB;
  if (P.speculate)
    k_trace<ANY, false, true, TB, MINB, SHS><<<grid, TB, 0, s>>>(P);
  else
    k_trace<ANY, false, false, TB, MINB, SHS><<<grid, TB, 0, s>>>(P);
}
template <bool ANY, int TB, int OCC>
void launchOcc(const KParams& P, int grid, cudaStream_t s) {
  if (P.sharedStack >= 32)
    launchShape<ANY, TB, OCC, 32>(P, grid, s);
  else if (P.sharedStack > 0 && P.sharedStack <= 16)
    launchShape<ANY, TB, OCC, 16>(P, grid, s);
  else
    launchShape<ANY, TB, OCC, 24>(P, grid, s);
}
template <bool ANY, int TB>
void launchTb(const KParams& P, int grid, cudaStream_t s) {
  if (P.occupancy >= 12)
    launchOcc<ANY, TB, 12>(P, grid, s);
  else if (P.occupancy >= 10)
    launchOcc<ANY, TB, 10>(P, grid, s);
  else
    launchOcc<ANY, TB, kTraceMinBlocks>(P, grid, s);
}
template <bool ANY>
void launchTrace(const KParams& P, int grid, cudaStream_t s) {
  if (P.counters)
    k_trace<ANY, true, false, kTraceThreads, kTraceMinBlocks, kSharedStack><<<grid, kTraceThreads, 0, s>>>(P);
  else if (P.blockThreads == 64)
    launchTb<ANY, 64>(P, grid, s);
  else if (P.blockThreads == 256)
    launchTb<ANY, 256>(P, grid, s);
  else
    launchTb<ANY, 128>(P, grid, s);
}
template <int TB, int OCC, int SHS>
int blocksOf() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace<false, false, true, TB, OCC * 128 / TB, SHS>, TB, 0);
  return n;
}
template <int TB, int OCC>
int blocksOcc(int sharedStack) {
  return sharedStack >= 32 ? blocksOf<TB, OCC, 32>()
         : (sharedStack > 0 && sharedStack <= 16) ? blocksOf<TB, OCC, 16>() : blocksOf<TB, OCC, 24>();
}
template <int TB>
int blocksTb(int occupancy, int sharedStack) {
  return occupancy >= 12 ? blocksOcc<TB, 12>(sharedStack)
         : occupancy >= 10 ? blocksOcc<TB, 10>(sharedStack) : blocksOcc<TB, kTraceMinBlocks>(sharedStack);
}
}  // namespace

void launchExtend(const KParams& P, int grid, cudaStream_t s) { launchTrace<false>(P, grid, s); }
void launchConnect(const KParams& P, int grid, cudaStream_t s) { launchTrace<true>(P, grid, s); }
int traceBlocksPerSm(int occupancy, int blockThreads, int sharedStack) {
  const int n = blockThreads == 64    ? blocksTb<64>(occupancy, sharedStack)
                : blockThreads == 256 ? blocksTb<256>(occupancy, sharedStack)
                                      : blocksTb<128>(occupancy, sharedStack);
  return n > 0 ? n : 1;
}
void launchTraceQuery(const SceneDev& S, const float4* o, const float4* d, uint32_t n, int anyHit, float4* hit,
                      uint32_t* inst, cudaStream_t s) {
  int grid = int((n + kTraceThreads - 1) / kTraceThreads);
  if (grid > 4096) grid = 4096;
  if (grid < 1) grid = 1;
  k_query<<<grid, kTraceThreads, 0, s>>>(S, o, d, n, anyHit, hit, inst);
}

}  // namespace asuna
