// shade.cu — ray generation, shading and film accumulation kernels.
//
// One wavefront iteration per path depth: raygen fills extend queue 0 with
// camera rays; after each closest-hit pass, `shade` runs the miss shader or
// the closest-hit shader of the hit material (emitters use the Lambertian
// light branch), writes next-event shadow rays into the shadow queue and the
// continuation rays into the other extend queue (warp-aggregated ballot/popc
// compaction, one atomic per warp); `accumulate` folds the finished samples
// into the film in frame order.
//
// Restates (file:line of the reference):
//   raygen      raytrace.projective.rgen:26-100 (seed, jitter, cameras)
//   shade/miss  raytrace.default.rmiss:24-56
//   shade/hit   rchit_layouts.glsl:61-167, brdf_lambertian.rchit:12-151,
//               brdf_rough_plastic.rchit:191-269, bsdf_dielectric.rchit:74-139,
//               brdf_emissive.rchit:12-27, brdf_plastic.rchit:43-205,
//               brdf_mirror.rchit:12-106, brdf_conductor.rchit:14-164,
//               brdf_rough_conductor.rchit, brdf_phong.rchit:12-194,
//               brdf_pbr_metalness_roughness.rchit:12-219,
//               brdf_disney.rchit:31-477, brdf_kang18.rchit:11-249
//   accumulate  raytrace.projective.rgen:134-179
//
// Compiled with -fmad=false: the float arithmetic rounds operation by
// operation in the order of the reference's GLSL source.
#include <cuda_runtime.h>

#include "dev_math.cuh"
#include "kernels.h"

namespace asuna {
using namespace dm;

namespace {

__device__ __forceinline__ uint32_t laneId() { return threadIdx.x & 31u; }

// Block-aggregated appends to the shadow queue and the next extend queue:
// every thread of the block calls it once per round (the barriers are
// uniform); one shared-memory add per warp and queue, then one global add per
// queue and block, so the two hot queue counters see an eighth of the
// atomics of per-warp appends.  Returns the slots of the thread's entries.
__device__ __forceinline__ void blockAppend2(bool wantA, bool wantB, uint32_t* counterA, uint32_t* counterB,
                                             uint32_t* shCount, uint32_t* shBase, uint32_t& slotA,
                                             uint32_t& slotB) {
  if (threadIdx.x < 2) shCount[threadIdx.x] = 0u;
  __syncthreads();
  const unsigned ma = __ballot_sync(0xffffffffu, wantA), mb = __ballot_sync(0xffffffffu, wantB);
  uint32_t offA = 0, offB = 0;
  if (laneId() == 0) {
    if (ma) offA = atomicAdd(&shCount[0], uint32_t(__popc(ma)));
    if (mb) offB = atomicAdd(&shCount[1], uint32_t(__popc(mb)));
  }
  offA = __shfl_sync(0xffffffffu, offA, 0);
  offB = __shfl_sync(0xffffffffu, offB, 0);
  __syncthreads();
  if (threadIdx.x == 0 && shCount[0]) shBase[0] = atomicAdd(counterA, shCount[0]);
  if (threadIdx.x == 1 && shCount[1]) shBase[1] = atomicAdd(counterB, shCount[1]);
  __syncthreads();
  const unsigned below = (1u << laneId()) - 1u;
  slotA = wantA ? shBase[0] + offA + uint32_t(__popc(ma & below)) : 0u;
  slotB = wantB ? shBase[1] + offB + uint32_t(__popc(mb & below)) : 0u;
}

__device__ __forceinline__ uint32_t findRange(const RangeDev* r, uint32_t n, uint32_t p) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&r[mid].pathBegin) <= p)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t sigMix(uint32_t h, uint32_t v) {
  return h ^ (v + 0x9e3779b9u + (h << 6) + (h >> 2));
}

}  // namespace

// ---------------------------------------------------------------------------
// raygen: raytrace.projective.rgen:26-100
__global__ void __launch_bounds__(256) k_raygen(KParams P) {
  const WaveDev& W = P.W;
  const uint32_t stride = gridDim.x * blockDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    W.cnt->c[kCntExtend0] = W.numPaths;
    W.cnt->c[kCntExtend1] = 0;
    W.cnt->c[kCntShadow] = 0;
    W.cnt->c[kCntFetchExtend] = 0;
    W.cnt->c[kCntFetchShadow] = 0;
    W.cnt->paths += W.numPaths;
  }
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W.numPaths; p += stride) {
    const uint32_t ri = findRange(W.ranges, W.numRanges, p);
    const RangeDev R = W.ranges[ri];
    const ShotDev& sh = W.shots[R.shot];
    const uint32_t local = p - R.pathBegin;
    const uint32_t frame = R.frameBegin + local / R.npix;
    const uint32_t pix = local % R.npix;
    const uint32_t x = pix % sh.width, y = pix / sh.width;
    uint32_t seed = xxhash32(x, y, hashFrame(frame, sh.seed));
    const asuna_camera& cam = sh.cam;
    f3 origin = transformPoint(cam.camera_to_world, splat(0.0f));
    f2 jitter = (frame == 0) ? f2{0.5f, 0.5f} : rnd2(seed);
    f2 pixel{float(x) + jitter.x, float(y) + jitter.y};
    f3 ro = origin, rd = splat(0.0f);
    if (cam.type == ASUNA_CAMERA_PERSPECTIVE) {
      f3 pCamera = transformPoint(cam.raster_to_camera, f3{pixel.x, pixel.y, 0.0f});
      f3 r = makeNormal(pCamera);
      if (cam.aperture > 0.0f) {
        f2 uLens = rnd2(seed);
        f2 d = concentricSampleDisk(uLens);
        f2 pLens{cam.aperture * d.x, cam.aperture * d.y};
        float ft = cam.focal_distance / r.z;
        f3 pFocus = ft * r;
        f3 o{pLens.x, pLens.y, 0.0f};
        ro = transformPoint(cam.camera_to_world, o);
        r = pFocus - o;
      }
      rd = transformDirection(cam.camera_to_world, r);
    } else if (cam.type == ASUNA_CAMERA_OPENCV) {
      float px = (pixel.x - cam.fxfycxcy[2]) / cam.fxfycxcy[0];
      float py = (pixel.y - cam.fxfycxcy[3]) / cam.fxfycxcy[1];
      rd = transformDirection(cam.camera_to_world, f3{px, py, 1.0f});
    }
    // Gaussian filter weight of this sample, rgen:134-145
    const float alpha = -2.0f;
    const float expXY = mexp(alpha * 2.0f * 2.0f);
    float ox = jitter.x - 0.5f, oy = jitter.y - 0.5f;
    float fw = gmax(0.0f, mexp(alpha * ox * ox) - expXY) * gmax(0.0f, mexp(alpha * oy * oy) - expXY);
    W.rayO[0][p] = make_float4(ro.x, ro.y, ro.z, INF);
    W.rayD[0][p] = make_float4(rd.x, rd.y, rd.z, __uint_as_float(p));
    W.path[p].thp = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    W.rad[p] = make_float4(0.0f, 0.0f, 0.0f, fw);
    W.path[p].info = make_uint4(seed, EBsdfNull, ri, local);
    if (P.records) W.rec[p] = make_uint4(0u, 0u, 0u, 1u);
    if (frame == 0) {
      // AOV images are rewritten at frame 0 (rgen:155-162): clear to (0,0,0,1)
      const uint32_t npx = sh.width * sh.height;
      for (uint32_t c = 0; c < sh.state.n_multi_channel && c < ASUNA_MAX_CHANNELS; ++c)
        sh.filmCh[size_t(c) * npx + pix] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    }
  }
}

// ---------------------------------------------------------------------------
namespace {

struct HitSt {
  f3 pos, V, N, ffN, X, Y;
  float u, v;
};

// rchit_layouts.glsl:61-95 (getHitState + configureShadingFrame)
__device__ __forceinline__ HitSt hitState(const SceneDev& S, const InstDev& in, uint32_t prim, float bu, float bv,
                                          f3 rd, uint32_t useFaceNormal) {
  HitSt st;
  const uint4 id = __ldg(&S.idx[in.idxBase + prim]);
  const VtxDev* vb = S.vtx + in.vtxBase;
  const float4 p0 = __ldg(&vb[id.x].pu), n0 = __ldg(&vb[id.x].nv);
  const float4 p1 = __ldg(&vb[id.y].pu), n1 = __ldg(&vb[id.y].nv);
  const float4 p2 = __ldg(&vb[id.z].pu), n2 = __ldg(&vb[id.z].nv);
  float bx = 1.0f - bu - bv, by = bu, bz = bv;
  st.u = p0.w * bx + p1.w * by + p2.w * bz;
  st.v = n0.w * bx + n1.w * by + n2.w * bz;
  f3 po = ld3(p0) * bx + ld3(p1) * by + ld3(p2) * bz;
  const float4 o0 = in.o2w[0], o1 = in.o2w[1], o2 = in.o2w[2];
  st.pos = f3{o0.x * po.x + o0.y * po.y + o0.z * po.z + o0.w, o1.x * po.x + o1.y * po.y + o1.z * po.z + o1.w,
              o2.x * po.x + o2.y * po.y + o2.z * po.z + o2.w};
  const float4 w0 = in.w2o[0], w1 = in.w2o[1], w2 = in.w2o[2];
  f3 n = ld3(n0) * bx + ld3(n1) * by + ld3(n2) * bz;
  st.N = makeNormal(f3{n.x * w0.x + n.y * w1.x + n.z * w2.x, n.x * w0.y + n.y * w1.y + n.z * w2.y,
                       n.x * w0.z + n.y * w1.z + n.z * w2.z});
  if (useFaceNormal == 1) {
    f3 g = cross(ld3(p1) - ld3(p0), ld3(p2) - ld3(p0));
    st.N = makeNormal(f3{g.x * w0.x + g.y * w1.x + g.z * w2.x, g.x * w0.y + g.y * w1.y + g.z * w2.y,
                         g.x * w0.z + g.y * w1.z + g.z * w2.z});
  }
  st.V = makeNormal(-rd);
  basis(st.N, st.X, st.Y);
  st.ffN = dot(st.N, st.V) > 0.0f ? st.N : -st.N;
  return st;
}

// textureEval (rchit_layouts.glsl:169-171), .rgb
__device__ __forceinline__ f3 texRGB(const SceneDev& S, int id, float u, float v) {
  const int4 ti = __ldg(&S.texInfo[id]);
  return tex4rgb(S.texels + uint32_t(ti.x), ti.y, ti.z, u, v);
}
// a normal-map texel (2c - 1) times the instance's world-to-object matrix
// as a row vector: how the reference moves object-space normals to world
__device__ __forceinline__ f3 objectToWorldNormal(const InstDev& in, f3 n) {
  const float4 w0 = in.w2o[0], w1 = in.w2o[1], w2 = in.w2o[2];
  return f3{n.x * w0.x + n.y * w1.x + n.z * w2.x, n.x * w0.y + n.y * w1.y + n.z * w2.y,
            n.x * w0.z + n.y * w1.z + n.z * w2.z};
}

// The "Fetch textures" block at the top of each material's hit shader:
// brdf_lambertian.rchit:80-90 (diffuse, tangent-space normal), the same in
// brdf_plastic/mirror/conductor/phong; brdf_rough_plastic.rchit:196-208 and
// brdf_rough_conductor.rchit:152-164 add alpha (.rg); bsdf_dielectric.rchit:
// 79-86 normal only; brdf_pbr_metalness_roughness.rchit:136-149 and
// brdf_disney.rchit:380-391 add metalness and roughness (.r);
// brdf_kang18.rchit:140-175 specular (.rgb), alpha (.rg), object-space normal
// and tangent maps; brdf_emissive.rchit:20-23 radiance = factor * texel.
// A normal map is followed by configureShadingFrame, which with
// use_face_normal puts the geometric normal back: the map then has no effect.
template <int CLS>
__device__ __forceinline__ void applyTextures(const SceneDev& S, const InstDev& in, MatDev& m, HitSt& st,
                                              uint32_t useFaceNormal) {
  if (CLS == kClsTerminal) {
    if (m.t1.x >= 0) {
      const f3 r = ld3(m.d) * texRGB(S, m.t1.x, st.u, st.v);
      m.a = make_float4(r.x, r.y, r.z, m.a.w);
    }
    return;
  }
  if (CLS != kClsDielectric && m.t0.x >= 0) {
    const f3 c = texRGB(S, m.t0.x, st.u, st.v);
    m.a = make_float4(c.x, c.y, c.z, m.a.w);
  }
  if ((CLS == kClsRoughPlastic || CLS == kClsRoughConductor || CLS == kClsKang18) && m.t0.z >= 0) {
    const f3 c = texRGB(S, m.t0.z, st.u, st.v);
    m.b.x = c.x;
    m.b.y = c.y;
  }
  if (CLS == kClsPbr) {
    if (m.t0.w >= 0) m.c.y = texRGB(S, m.t0.w, st.u, st.v).x;
    if (m.t0.z >= 0) m.c.x = texRGB(S, m.t0.z, st.u, st.v).x;
  }
  if (CLS == kClsDisney) {
    if (m.t0.w >= 0) m.c.x = texRGB(S, m.t0.w, st.u, st.v).x;
    if (m.t0.z >= 0) m.c.y = texRGB(S, m.t0.z, st.u, st.v).x;
  }
  if (CLS == kClsKang18 && m.t0.w >= 0) {
    const f3 c = texRGB(S, m.t0.w, st.u, st.v);
    m.c = make_float4(c.x, c.y, c.z, m.c.w);
  }
  if (m.t0.y >= 0 && useFaceNormal != 1u) {
    const f3 c = texRGB(S, m.t0.y, st.u, st.v);
    const f3 n = f3{2.0f * c.x - 1.0f, 2.0f * c.y - 1.0f, 2.0f * c.z - 1.0f};
    st.N = makeNormal(CLS == kClsKang18 ? objectToWorldNormal(in, n) : toWorld(st.X, st.Y, st.N, n));
    basis(st.N, st.X, st.Y);
    st.ffN = dot(st.N, st.V) > 0.0f ? st.N : -st.N;
  }
  if (CLS == kClsKang18 && m.t1.y >= 0) {
    const f3 c = texRGB(S, m.t1.y, st.u, st.v);
    st.X = makeNormal(objectToWorldNormal(in, f3{2.0f * c.x - 1.0f, 2.0f * c.y - 1.0f, 2.0f * c.z - 1.0f}));
  }
}

struct PathIO {
  uint32_t seed;
  uint32_t bflags;
  float bpdf;
  f3 thp;
  f3 rad;
  bool stop;
  // next-event record of this bounce
  bool dskip;
  f3 drad, dro, drd;
  float ddist;
  // continuation
  f3 nro, nrd;
};

// rchit_layouts.glsl:118-167 (sampleLights, with sampleEnvironmentLight 98-116)
__device__ __forceinline__ f3 sampleLights(const SceneDev& S, const ShotDev& sh, PathIO& io, f3 rd, f3 pos, f3 nrm,
                                           bool& visible, LRec& lRec) {
  bool allowDoubleSide = false;
  f3 radiance = splat(0.0f);
  const bool sky = S.sky.in_use == 1;
  const bool hasEnv = sh.state.has_env_map == 1u || sky;
  const bool hasLight = sh.state.num_lights > 0;
  float envSel, anaSel;
  if (hasEnv && hasLight) {
    envSel = anaSel = 0.5f;
  } else if (hasEnv) {
    envSel = 1.0f;
    anaSel = 0.0f;
  } else if (hasLight) {
    envSel = 0.0f;
    anaSel = 1.0f;
  } else {
    envSel = anaSel = 0.0f;
  }
  float sel = rnd(io.seed);
  if (sel < envSel) {
    lRec.flags = EArea;
    lRec.dist = INF;
    lRec.n = -makeNormal(rd);
    f2 u = rnd2(io.seed);
    if (sky) {
      // sample_light.glsl:137-141
      lRec.d = uniformSampleSphere(u);
      lRec.pdf = INV_4PI;
      radiance = evalSunSky(S, lRec.d) / envSel;
    } else {
      radiance = sampleEnvmap(S, sh, u, lRec.d, lRec.pdf) / envSel;
    }
    allowDoubleSide = true;
  } else if (sel < envSel + anaSel) {
    const int n = sh.state.num_lights;
    int idx = min(1 + __float2int_rz(rnd(io.seed) * float(n)), n);
    const LightDev l = S.lights[idx];
    f2 u = rnd2(io.seed);
    radiance = sampleOneLight(u, l, pos, lRec) * float(n) / anaSel;
    allowDoubleSide = (__float_as_uint(l.v.w) == 1u);
  }
  io.dro = offsetPositionAlongNormal(pos, nrm);
  io.drd = lRec.d;
  io.ddist = lRec.dist;
  visible = (dot(lRec.d, nrm) > 0.0f && lRec.pdf > 0.0f);
  visible = visible && (dot(lRec.n, lRec.d) < 0.0f || allowDoubleSide);
  return radiance;
}

// Next-event estimation of a material hit.  The three material hit shaders
// brdf_phong.rchit:12-30 (flag EArea): normalised Phong lobe mixed with the
// Lambertian lobe by the luminances of the two reflectances.
__device__ __forceinline__ f3 phongEval(f3 L, f3 V, f3 N, f3 kd, f3 ks, float n) {
  const float NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL < 0.0f || NdotV < 0.0f) return splat(0.0f);
  const f3 H = normalize(L + V);
  const f3 diffuseLobe = kd * INV_PI;
  const f3 specularLobe = ks * mpow(gmax(dot(H, N), 0.0f), n) * (n + 2.0f) * INV_2PI;
  const float db = luminance(kd), sb = luminance(ks);
  const float dw = db / (db + sb), sw = 1.0f - dw;
  return (dw * diffuseLobe + sw * specularLobe) * NdotL;
}
// brdf_phong.rchit:32-37
__device__ __forceinline__ float phongLobePdf(f3 L, f3 V, f3 N, float n) {
  const f3 H = normalize(L + V);
  const float NdotH = gmax(dot(H, N), 0.0f), VdotH = gmax(dot(H, V), 0.0f);
  return (n + 1.0f) * INV_2PI * mpow(NdotH, n) * 0.25f / (VdotH + EPS);
}

// brdf_pbr_metalness_roughness.rchit:14-16, 57-86 (flags unused): GGX with
// Schlick Fresnel (f0 = mix(F0(eta), albedo, metalness)) plus the Lambertian
// base weighted by 1 - metalness
__device__ __forceinline__ f3 pbrEval(f3 L, f3 V, f3 N, f3 X, f3 Y, f3 albedo, float a, float metalness, float eta) {
  const float NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= 0.0f || NdotV <= 0.0f) return splat(0.0f);
  const f3 H = makeNormal(L + V);
  const float HdotN = dot(H, N), HdotX = dot(H, X), HdotY = dot(H, Y), HdotV = dot(H, V);
  const float F0 = sqr((eta - 1.0f) / (eta + 1.0f));
  const f3 f0 = splat(F0) * (1.0f - metalness) + albedo * metalness;
  const f3 Fs = f0 + (splat(1.0f) - f0) * mpow(gclamp(1.0f - HdotV, 0.0f, 1.0f), 5.0f);
  const float Ds = dAnisoGGX(HdotN, HdotX, HdotY, a, a);
  float Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), a, a);
  Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), a, a);
  const f3 diffuse = albedo * (1.0f - metalness) * INV_PI;
  const f3 specular = Fs * Ds * Gs;
  return (diffuse + specular) * NdotL;
}
// 88-105: fixed 0.2 / 0.8 mixture of the cosine and GGX pdfs (EArea only)
__device__ __forceinline__ float pbrPdf(f3 L, f3 V, f3 N, f3 X, f3 Y, float a) {
  const float NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= 0.0f || NdotV <= 0.0f) return 0.0f;
  const f3 H = makeNormal(L + V);
  const f3 wh = makeNormal(toLocal(X, Y, N, H)), wo = makeNormal(toLocal(X, Y, N, V)),
           wi = makeNormal(toLocal(X, Y, N, L));
  return 0.2f * cosineHemispherePdf(wi.z) + (1.0f - 0.2f) * importanceAnisoGGXPdf(wh, wo, a, a);
}

// brdf_kang18.rchit:57-111: anisotropic GGX with scalar Schlick Fresnel over
// a Lambertian base; lobe probability from the two luminances
__device__ __forceinline__ f3 kangEval(f3 L, f3 V, f3 N, f3 X, f3 Y, f3 kd, f3 ks, float ax, float ay, float eta) {
  const float NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= 0.0f || NdotV <= 0.0f) return splat(0.0f);
  const f3 H = makeNormal(L + V);
  const float HdotN = dot(H, N), HdotX = dot(H, X), HdotY = dot(H, Y), HdotV = dot(H, V);
  const float F0 = sqr((eta - 1.0f) / (eta + 1.0f));
  const float Fs = F0 + (1.0f - F0) * mpow(gclamp(1.0f - HdotV, 0.0f, 1.0f), 5.0f);
  const float Ds = dAnisoGGX(HdotN, HdotX, HdotY, ax, ay);
  float Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
  Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
  const f3 diffuse = kd * INV_PI;
  const f3 specular = ks * Fs * Ds * Gs;
  return (diffuse + specular) * NdotL;
}
__device__ __forceinline__ float kangDiffuseProb(f3 kd, f3 ks) {
  const float pd = 0.212671f * kd.x + 0.715160f * kd.y + 0.072169f * kd.z;
  const float ps = 0.212671f * ks.x + 0.715160f * ks.y + 0.072169f * ks.z;
  return pd / (pd + ps + EPS);
}
__device__ __forceinline__ float kangPdf(f3 L, f3 V, f3 N, f3 X, f3 Y, float ax, float ay, f3 kd, f3 ks) {
  const float NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= 0.0f || NdotV <= 0.0f) return 0.0f;
  const f3 H = makeNormal(L + V);
  const f3 wh = makeNormal(toLocal(X, Y, N, H)), wo = makeNormal(toLocal(X, Y, N, V)),
           wi = makeNormal(toLocal(X, Y, N, L));
  const float dp = kangDiffuseProb(kd, ks);
  return dp * cosineHemispherePdf(wi.z) + (1.0f - dp) * importanceAnisoGGXPdf(wh, wo, ax, ay);
}

// ---- brdf_disney.rchit (float restatement; expressions in source order) ----
namespace disney {
struct Mat {  // DisneyMaterial (31-48) without the unused fields
  f3 baseColor;
  float metallic, roughness, subsurface, specularTint, sheen, sheenTint, clearcoat, clearcoatRoughness, ax, ay;
};
__device__ __forceinline__ float mix1(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ f3 mix3(f3 x, f3 y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ float lum(f3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
// 54-59
__device__ __forceinline__ float GTR1(float NDotH, float a) {
  if (a >= 1.0f) return INV_PI;
  const float a2 = a * a;
  const float t = 1.0f + (a2 - 1.0f) * NDotH * NDotH;
  return (a2 - 1.0f) / (PI * mlog(a2) * t);
}
// 61-74 (r1 drives both angles; r2 unused, as written)
__device__ __forceinline__ f3 SampleGTR1(float rgh, float r1) {
  const float a = gmax(0.001f, rgh);
  const float a2 = a * a;
  const float phi = r1 * TWO_PI;
  const float cosTheta = sqrtf((1.0f - mpow(a2, 1.0f - r1)) / (1.0f - a2));
  const float sinTheta = gclamp(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
  return f3{sinTheta * mcos(phi), sinTheta * msin(phi), cosTheta};
}
// 95-114
__device__ __forceinline__ f3 SampleGGXVNDF(f3 V, float ax, float ay, float r1, float r2) {
  const f3 Vh = normalize(f3{ax * V.x, ay * V.y, V.z});
  const float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  const f3 T1 = lensq > 0.0f ? f3{-Vh.y, Vh.x, 0.0f} * (1.0f / sqrtf(lensq)) : f3{1.0f, 0.0f, 0.0f};
  const f3 T2 = cross(Vh, T1);
  const float r = sqrtf(r1);
  const float phi = 2.0f * PI * r2;
  const float t1 = r * mcos(phi);
  float t2 = r * msin(phi);
  const float sv = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - sv) * sqrtf(1.0f - t1 * t1) + sv * t2;
  const f3 Nh = t1 * T1 + t2 * T2 + sqrtf(gmax(0.0f, 1.0f - t1 * t1 - t2 * t2)) * Vh;
  return normalize(f3{ax * Nh.x, ay * Nh.y, gmax(0.0f, Nh.z)});
}
// 116-121
__device__ __forceinline__ float GTR2Aniso(float NDotH, float HDotX, float HDotY, float ax, float ay) {
  const float a = HDotX / ax, b = HDotY / ay;
  const float c = a * a + b * b + NDotH * NDotH;
  return 1.0f / (PI * ax * ay * c * c);
}
// 133-144
__device__ __forceinline__ float SmithG(float NDotV, float alphaG) {
  const float a = alphaG * alphaG, b = NDotV * NDotV;
  return (2.0f * NDotV) / (NDotV + sqrtf(a + b - a * b));
}
__device__ __forceinline__ float SmithGAniso(float NDotV, float VDotX, float VDotY, float ax, float ay) {
  const float a = VDotX * ax, b = VDotY * ay, c = NDotV;
  return (2.0f * NDotV) / (NDotV + sqrtf(a * a + b * b + c * c));
}
// 146-170
__device__ __forceinline__ float SchlickFresnel(float u) {
  const float m = gclamp(1.0f - u, 0.0f, 1.0f);
  const float m2 = m * m;
  return m2 * m2 * m;
}
__device__ __forceinline__ float DielectricFresnel(float cosThetaI, float eta) {
  const float sinThetaTSq = eta * eta * (1.0f - cosThetaI * cosThetaI);
  if (sinThetaTSq > 1.0f) return 1.0f;
  const float cosThetaT = sqrtf(gmax(1.0f - sinThetaTSq, 0.0f));
  const float rs = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
  const float rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  return 0.5f * (rs * rs + rp * rp);
}
__device__ __forceinline__ float Fresnel(float metallic, float eta, float LDotH, float VDotH) {
  return mix1(DielectricFresnel(fabsf(VDotH), eta), SchlickFresnel(LDotH), metallic);
}
// 172-195
__device__ __forceinline__ f3 EvalDiffuse(const Mat& mat, f3 Csheen, f3 V, f3 L, f3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return splat(0.0f);
  const float FL = SchlickFresnel(L.z), FV = SchlickFresnel(V.z), FH = SchlickFresnel(dot(L, H));
  const float Fd90 = 0.5f + 2.0f * dot(L, H) * dot(L, H) * mat.roughness;
  const float Fd = mix1(1.0f, Fd90, FL) * mix1(1.0f, Fd90, FV);
  const float Fss90 = dot(L, H) * dot(L, H) * mat.roughness;
  const float Fss = mix1(1.0f, Fss90, FL) * mix1(1.0f, Fss90, FV);
  const float ss = 1.25f * (Fss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
  const f3 Fsheen = FH * mat.sheen * Csheen;
  pdf = L.z * INV_PI;
  return (1.0f - mat.metallic) * (INV_PI * mix1(Fd, ss, mat.subsurface) * mat.baseColor + Fsheen);
}
// 197-211
__device__ __forceinline__ f3 EvalSpecReflection(const Mat& mat, float eta, f3 specCol, f3 V, f3 L, f3 H,
                                                 float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return splat(0.0f);
  const float FM = Fresnel(mat.metallic, eta, dot(L, H), dot(V, H));
  const f3 F = mix3(specCol, splat(1.0f), FM);
  const float D = GTR2Aniso(H.z, H.x, H.y, mat.ax, mat.ay);
  const float G1 = SmithGAniso(fabsf(V.z), V.x, V.y, mat.ax, mat.ay);
  const float G2 = G1 * SmithGAniso(fabsf(L.z), L.x, L.y, mat.ax, mat.ay);
  pdf = G1 * D / (4.0f * V.z);
  return F * D * G2 / (4.0f * L.z * V.z);
}
// 213-226
__device__ __forceinline__ f3 EvalClearcoat(const Mat& mat, f3 V, f3 L, f3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return splat(0.0f);
  const float FH = DielectricFresnel(dot(V, H), 1.0f / 1.5f);
  const float F = mix1(0.04f, 1.0f, FH);
  const float D = GTR1(H.z, mat.clearcoatRoughness);
  const float G = SmithG(L.z, 0.25f) * SmithG(V.z, 0.25f);
  const float jacobian = 1.0f / (4.0f * dot(V, H));
  pdf = D * H.z * jacobian;
  return splat(0.25f) * mat.clearcoat * F * D * G / (4.0f * L.z * V.z);
}
// 228-250
__device__ __forceinline__ void SpecColor(const Mat& mat, float eta, f3& specCol, f3& sheenCol) {
  const float l = lum(mat.baseColor);
  const f3 ctint = l > 0.0f ? mat.baseColor / l : splat(1.0f);
  const float F0 = (1.0f - eta) / (1.0f + eta);
  specCol = mix3(F0 * F0 * mix3(splat(1.0f), ctint, mat.specularTint), mat.baseColor, mat.metallic);
  sheenCol = mix3(splat(1.0f), ctint, mat.sheenTint);
}
__device__ __forceinline__ void LobeProbabilities(const Mat& mat, f3 specCol, float approxFresnel, float& diffuseWt,
                                                  float& specReflectWt, float& clearcoatWt) {
  diffuseWt = lum(mat.baseColor) * (1.0f - mat.metallic);
  specReflectWt = lum(mix3(specCol, splat(1.0f), approxFresnel));
  clearcoatWt = 0.25f * mat.clearcoat * (1.0f - mat.metallic);
  const float totalWt = diffuseWt + specReflectWt + clearcoatWt;
  diffuseWt = diffuseWt / totalWt;
  specReflectWt = specReflectWt / totalWt;
  clearcoatWt = clearcoatWt / totalWt;
}
// 252-300 (EArea at every call site)
__device__ __forceinline__ f3 eval(f3 L, f3 V, f3 N, f3 X, f3 Y, const Mat& mat, float eta, float& bsdfPdf) {
  f3 weight = splat(0.0f);
  bsdfPdf = 0.0f;
  V = toLocal(X, Y, N, V);
  L = toLocal(X, Y, N, L);
  if (L.z <= 0.0f || V.z <= 0.0f) return weight;
  f3 H = normalize(L + V);
  if (H.z < 0.0f) H = -H;
  f3 specCol, sheenCol;
  SpecColor(mat, eta, specCol, sheenCol);
  float diffuseWt, specReflectWt, clearcoatWt;
  LobeProbabilities(mat, specCol, Fresnel(mat.metallic, eta, dot(L, H), dot(V, H)), diffuseWt, specReflectWt,
                    clearcoatWt);
  float pdf = 0.0f;
  if (diffuseWt > 0.0f && L.z > 0.0f) {
    weight = weight + EvalDiffuse(mat, sheenCol, V, L, H, pdf);
    bsdfPdf = bsdfPdf + pdf * diffuseWt;
  }
  if (specReflectWt > 0.0f && L.z > 0.0f && V.z > 0.0f) {
    weight = weight + EvalSpecReflection(mat, eta, specCol, V, L, H, pdf);
    bsdfPdf = bsdfPdf + pdf * specReflectWt;
  }
  if (clearcoatWt > 0.0f && L.z > 0.0f && V.z > 0.0f) {
    weight = weight + EvalClearcoat(mat, V, L, H, pdf);
    bsdfPdf = bsdfPdf + pdf * clearcoatWt;
  }
  return weight * L.z;
}
// main 419-439: the material as the shader derives it
__device__ __forceinline__ Mat fromDev(const MatDev& m) {
  Mat d;
  const float rough = m.c.y;
  const float aspect = sqrtf(1.0f - m.b.x * 0.9f);
  d.ax = gmax(0.001f, rough * rough / aspect);
  d.ay = gmax(0.001f, rough * rough * aspect);
  d.baseColor = ld3(m.a);
  d.metallic = m.c.x;
  d.roughness = gmax(rough * rough, 0.001f);
  d.subsurface = m.c.z;
  d.specularTint = m.c.w;
  d.sheen = m.d.x;
  d.sheenTint = m.d.y;
  d.clearcoat = m.d.z;
  d.clearcoatRoughness = mix1(0.1f, 0.001f, m.d.w);
  return d;
}
}  // namespace disney

// (brdf_lambertian.rchit:110-134, brdf_rough_plastic.rchit:224-250,
// bsdf_dielectric.rchit:248-271) all start with sampleLights(pos, ffN) and
// differ only in the BSDF eval/pdf pair, so light sampling runs once here and
// the material selects the pair.
__device__ __forceinline__ void nextEvent(const SceneDev& S, const ShotDev& sh, PathIO& io, const HitSt& st,
                                          const MatDev& m, uint32_t type, f3 rd) {
  bool visible;
  LRec lRec{splat(0.0f), splat(0.0f), 0.0f, 0.0f, 0u};
  f3 Ld = splat(0.0f);
  const f3 r = sampleLights(S, sh, io, rd, st.pos, st.ffN, visible, lRec);
  if (visible) {
    f3 w = splat(0.0f);
    float bpdf = 0.0f;
    if (type == ASUNA_MAT_ROUGH_PLASTIC) {
      const float eta = m.b.z, fdrInt = m.b.w, invEta2 = 1.0f / (eta * eta);
      const float ax = gmax(EPS, m.b.x), ay = gmax(EPS, m.b.y);
      const f3 kd = ld3(m.a);
      const float ssw = luminance(kd);
      // The reference's call sites (brdf_rough_plastic.rchit:234-240) pass
      // (.., fdrInt, ax, ay, invEta2, ..) and (.., eta, ax, ay, ..) into
      // parameters declared (.., fdrInt, invEta2, ax, ay, ..) and
      // (.., ax, ay, eta, ..); kept as written.
      w = rpEval(lRec.d, st.V, st.ffN, st.X, st.Y, kd, splat(1.0f), eta, fdrInt, ax, ay, invEta2, EArea);
      bpdf = rpPdf(lRec.d, st.V, st.ffN, st.X, st.Y, eta, ax, ay, ssw, lRec.flags);
    } else if (type == ASUNA_MAT_PLASTIC) {
      // brdf_plastic.rchit:43-61 eval with EArea, 63-84 pdf with lRec.flags
      const float eta = m.b.z, fdrInt = m.b.w, invEta2 = 1.0f / (eta * eta);
      const f3 kd = ld3(m.a);
      const float dAvg = luminance(kd), sAvg = luminance(splat(1.0f));
      const float ssw = sAvg / (dAvg + sAvg);
      const f3 L = lRec.d, V = st.V, N = st.ffN;
      const float NdotL = dot(L, N), NdotV = dot(V, N);
      if (!(NdotL < 0.0f || NdotV < 0.0f)) {
        float c0;
        const float Fo = fresnelDielectricExt(NdotV, c0, eta);
        float c1;
        const float Fi = fresnelDielectricExt(NdotL, c1, eta);
        f3 diff = kd;
        diff = diff / (splat(1.0f) - diff * fdrInt);
        w = (1.0f - Fi) * (1.0f - Fo) * diff * invEta2 * INV_PI * NdotL;
        const float probSpecular = (Fo * ssw) / (Fo * ssw + (1.0f - Fo) * (1.0f - ssw));
        if (lRec.flags & EDelta) {
          if (fabsf(dot(reflect(-V, N), L) - 1.0f) < EPS) bpdf = probSpecular;
        } else if (lRec.flags & EArea) {
          bpdf = NdotL * (1.0f - probSpecular);  // no 1/pi, as in the reference
        }
      }
    } else if (type == ASUNA_MAT_CONDUCTOR) {
      // brdf_conductor.rchit:38-63: eval is zero for area samples; pdf 1 on the
      // mirror direction of a delta light (front side only)
      const float NdotL = dot(lRec.d, st.ffN), NdotV = dot(st.V, st.ffN);
      if (!(NdotL < 0.0f || NdotV < 0.0f) && (lRec.flags & EDelta) &&
          fabsf(dot(reflect(-st.V, st.ffN), lRec.d) - 1.0f) < EPS)
        bpdf = 1.0f;
    } else if (type == ASUNA_MAT_ROUGH_CONDUCTOR) {
      // brdf_rough_conductor.rchit:72-101 (Fresnel at N.L, as the reference)
      const float ax = gmax(EPS, m.b.x), ay = gmax(EPS, m.b.y);
      const f3 L = lRec.d, V = st.V, N = st.ffN, X = st.X, Y = st.Y;
      const float NdotL = dot(L, N), NdotV = dot(V, N);
      if (!(NdotL < 0.0f || NdotV < 0.0f)) {
        const f3 H = makeNormal(L + V);
        const f3 Fs = conductorReflectance3(ld3(m.c), ld3(m.d), NdotL);
        float Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
        Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
        const float Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
        w = ld3(m.a) * Fs * Gs * Ds * NdotL;
        if (lRec.flags & EArea) {
          const f3 wi = toLocal(X, Y, N, L), wo = toLocal(X, Y, N, V);
          bpdf = importanceAnisoGGXPdf(makeNormal(wi + wo), wo, ax, ay);
        }
      }
    } else if (type == ASUNA_MAT_MIRROR) {
      // brdf_mirror.rchit:12-26: eval is zero for area samples; pdf 1 on the
      // mirror direction of a delta light
      if ((lRec.flags & EDelta) && fabsf(dot(reflect(-st.V, st.ffN), lRec.d) - 1.0f) < EPS) bpdf = 1.0f;
    } else if (type == ASUNA_MAT_DIELECTRIC) {
      // eval() with EArea returns 0 (bsdf_dielectric.rchit:26-38); pdf 41-52
      const float ior = m.b.z;
      const float eta = dot(st.V, st.N) > 0.0f ? (1.0f / ior) : ior;
      if (lRec.flags & EDelta) {
        const f3 L = lRec.d, V = st.V, N = st.ffN;
        const float F = dielectricFresnel(fabsf(dot(V, N)), eta);
        if (dot(L, N) > 0.0f) {
          if (fabsf(dot(reflect(-V, N), L) - 1.0f) < EPS) bpdf = F;
        } else {
          if (fabsf(dot(refract(-V, N, eta), L) - 1.0f) < EPS) bpdf = 1.0f - F;
        }
      }
    } else if (type == ASUNA_MAT_PBR_METALNESS_ROUGHNESS) {
      // brdf_pbr_metalness_roughness.rchit:184-195
      const float a = gmax(sqr(m.c.x), 0.001f);
      w = pbrEval(lRec.d, st.V, st.ffN, st.X, st.Y, ld3(m.a), a, m.c.y, m.b.z);
      if (lRec.flags & EArea) bpdf = pbrPdf(lRec.d, st.V, st.ffN, st.X, st.Y, a);
    } else if (type == ASUNA_MAT_KANG18) {
      // brdf_kang18.rchit:198-221 (eval ignores the flags, pdf does not)
      const float ax = gmax(m.b.x, EPS), ay = gmax(m.b.y, EPS);
      const f3 kd = ld3(m.a), ks = ld3(m.c);
      w = kangEval(lRec.d, st.V, st.ffN, st.X, st.Y, kd, ks, ax, ay, m.b.z);
      if (lRec.flags & EArea) bpdf = kangPdf(lRec.d, st.V, st.ffN, st.X, st.Y, ax, ay, kd, ks);
    } else if (type == ASUNA_MAT_DISNEY) {
      // brdf_disney.rchit:450-466: eval (and its pdf) with EArea for every light
      const disney::Mat dm = disney::fromDev(m);
      const float eta = dot(st.V, st.N) > 0.0f ? (1.0f / m.b.z) : m.b.z;
      w = disney::eval(lRec.d, st.V, st.ffN, st.X, st.Y, dm, eta, bpdf);
    } else if (type == ASUNA_MAT_PHONG) {
      // brdf_phong.rchit:12-30 eval with EArea, 39-52 pdf with lRec.flags
      const f3 kd = ld3(m.a), ks = ld3(m.c);
      w = phongEval(lRec.d, st.V, st.ffN, kd, ks, m.c.w);
      if (lRec.flags & EArea) {
        const float db = luminance(kd), sb = luminance(ks);
        const float dw = db / (db + sb), sw = 1.0f - dw;
        bpdf = dw * cosineHemispherePdf(dot(st.ffN, lRec.d)) + sw * phongLobePdf(lRec.d, st.V, st.ffN, m.c.w);
      }
    } else {
      // Lambertian eval 12-21 (flag EArea), pdf 23-29 (lRec.flags)
      const float NdotL = dot(st.ffN, lRec.d), NdotV = dot(st.ffN, st.V);
      if (!(NdotL < 0.0f || NdotV < 0.0f)) w = ld3(m.a) * INV_PI * NdotL;
      bpdf = (lRec.flags & EArea) ? cosineHemispherePdf(dot(st.ffN, lRec.d)) : 0.0f;
    }
    const float mis = powerHeuristic(lRec.pdf, bpdf);
    Ld = Ld + mis * w * r * io.thp / (lRec.pdf + EPS);
  }
  io.drad = Ld;
  io.dskip = !visible;
}

// BSDF sampling of the continuation ray: brdf_lambertian.rchit:31-42,136-151
__device__ __forceinline__ void sampleLambertian(PathIO& io, const HitSt& st, f3 kd) {
  f2 u = rnd2(io.seed);
  f3 wi = cosineSampleHemisphere(u);
  float pdf = cosineHemispherePdf(wi.z);
  f3 d = toWorld(st.X, st.Y, st.ffN, wi);
  f3 w = kd * INV_PI * fabsf(wi.z);
  if (pdf <= 0.0f || length(w) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = EDiffuseReflection;
  io.bpdf = pdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = d;
  io.thp = io.thp * (w / pdf);
}

// brdf_rough_plastic.rchit:138-189,252-269
__device__ __forceinline__ void sampleRoughPlastic(PathIO& io, const HitSt& st, const MatDev& m) {
  const float eta = m.b.z;
  const float fdrInt = m.b.w;
  const float invEta2 = 1.0f / (eta * eta);
  const float ax = gmax(EPS, m.b.x);
  const float ay = gmax(EPS, m.b.y);
  const f3 kd = ld3(m.a);
  const float ssw = luminance(kd);
  const f3 ks = splat(1.0f);
  f2 u = rnd2(io.seed);
  const f3 V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  f3 weight = splat(0.0f);
  float bpdf = 0.0f;
  uint32_t bflags = EBsdfNull;
  f3 bd = splat(0.0f);
  const float NdotV = dot(V, N);
  if (NdotV > 0.0f) {
    float ct;
    float Fo = fresnelDielectricExt(NdotV, ct, eta);
    float substrateWeight = ssw * (1.0f - Fo);
    float specularWeight = Fo;
    float probSpecular = specularWeight / (specularWeight + substrateWeight);
    if (u.x < probSpecular) {
      u.x = u.x / probSpecular;
      f3 wo = toLocal(X, Y, N, V);
      f3 wi = importanceSampleAnisoGGX(u, wo, ax, ay);
      f3 L = toWorld(X, Y, N, wi);
      bd = L;
      f3 H = makeNormal(V + L);
      f3 wh = makeNormal(wi + wo);
      float NdotL = dot(N, L);
      float ct2;
      float Fs = fresnelDielectricExt(dot(H, V), ct2, eta);
      float Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
      Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
      float Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
      bflags = EGlossyReflection;
      bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay) * probSpecular;
      weight = ks * Fs * Gs * Ds * NdotL;
    } else {
      u.x = (u.x - probSpecular) / (1.0f + EPS - probSpecular);
      f3 wi = cosineSampleHemisphere(u);
      float ct2;
      float Fi = fresnelDielectricExt(wi.z, ct2, eta);
      f3 diff = kd;
      diff = diff / (splat(1.0f) - diff * fdrInt);
      bpdf = (1.0f - probSpecular) * cosineHemispherePdf(wi.z);
      bd = toWorld(X, Y, N, wi);
      bflags = EDiffuseReflection;
      weight = (1.0f - Fi) * (1.0f - Fo) * invEta2 * diff * INV_PI * fabsf(wi.z);
    }
  }
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / (bpdf + EPS));
}

// brdf_plastic.rchit:86-120,187-205
__device__ __forceinline__ void samplePlastic(PathIO& io, const HitSt& st, const MatDev& m) {
  const float eta = m.b.z, fdrInt = m.b.w, invEta2 = 1.0f / (eta * eta);
  const f3 kd = ld3(m.a);
  const float dAvg = luminance(kd), sAvg = luminance(splat(1.0f));
  const float ssw = sAvg / (dAvg + sAvg);
  f2 u = rnd2(io.seed);
  const f3 V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  f3 weight = splat(0.0f), bd = splat(0.0f);
  float bpdf = 0.0f;
  uint32_t bflags = EBsdfNull;
  const float NdotV = dot(V, N);
  if (NdotV > 0.0f) {
    float c0;
    const float Fo = fresnelDielectricExt(NdotV, c0, eta);
    const float probSpecular = (Fo * ssw) / (Fo * ssw + (1.0f - Fo) * (1.0f - ssw));
    if (u.x < probSpecular) {
      bd = makeNormal(reflect(-V, N));
      bflags = ESpecularReflection;
      bpdf = probSpecular;
      weight = splat(1.0f) * Fo;
    } else {
      u.x = (u.x - probSpecular) / (1.0f + EPS - probSpecular);
      const f3 wi = cosineSampleHemisphere(u);
      float c1;
      const float Fi = fresnelDielectricExt(wi.z, c1, eta);
      f3 diff = kd;
      diff = diff / (splat(1.0f) - diff * fdrInt);
      bpdf = (1.0f - probSpecular) * cosineHemispherePdf(wi.z);
      bd = toWorld(X, Y, N, wi);
      bflags = EDiffuseReflection;
      weight = (1.0f - Fi) * (1.0f - Fo) * invEta2 * diff * INV_PI * fabsf(wi.z);
    }
  }
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / (bpdf + EPS));
}

// brdf_phong.rchit:54-84,178-193: lobe chosen by the diffuse weight; the
// Phong lobe samples the half vector (cos^(1/(n+1))) and reflects V about it
__device__ __forceinline__ void samplePhong(PathIO& io, const HitSt& st, const MatDev& m) {
  const f3 kd = ld3(m.a), ks = ld3(m.c);
  const float n = m.c.w;
  f2 u = rnd2(io.seed);
  const f3 V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  const float db = luminance(kd), sb = luminance(ks);
  const float dw = db / (db + sb), sw = 1.0f - dw;
  f3 bd;
  float bpdf;
  uint32_t bflags;
  if (u.x < dw) {
    u.x = u.x / dw;
    const f3 wi = cosineSampleHemisphere(u);
    bpdf = cosineHemispherePdf(wi.z);
    bd = toWorld(X, Y, N, wi);
    bflags = EDiffuseReflection;
  } else {
    u.x = (u.x - dw) / sw;
    const float cosTheta = mpow(u.x, 1.0f / (n + 1.0f));
    const float phi = TWO_PI * u.y;
    const float sinTheta = sqrtf(gmax(0.0f, 1.0f - cosTheta * cosTheta));
    const f3 wh = f3{sinTheta * msin(phi), sinTheta * mcos(phi), cosTheta};
    const f3 H = toWorld(X, Y, N, wh);
    bd = reflect(-V, H);
    bpdf = phongLobePdf(bd, V, N, n);
    bflags = EGlossyReflection;
  }
  const f3 weight = phongEval(bd, V, N, kd, ks, n);
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / bpdf);
}

// brdf_pbr_metalness_roughness.rchit:107-129,203-219: the direction pair is
// drawn before the lobe choice; the pdf is the chosen lobe's alone and the
// weight carries a second |cos| (as the reference writes them)
__device__ __forceinline__ void samplePbr(PathIO& io, const HitSt& st, const MatDev& m) {
  const float a = gmax(sqr(m.c.x), 0.001f);
  f2 u = rnd2(io.seed);
  const f3 V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  const f3 wo = makeNormal(toLocal(X, Y, N, V));
  f3 wi;
  float bpdf;
  uint32_t bflags;
  if (rnd(io.seed) < 0.2f) {
    wi = cosineSampleHemisphere(u);
    bflags = EDiffuseReflection;
    bpdf = cosineHemispherePdf(wi.z);
  } else {
    wi = importanceSampleAnisoGGX(u, wo, a, a);
    const f3 wh = makeNormal(wi + wo);
    bpdf = importanceAnisoGGXPdf(wh, wo, a, a);
    bflags = EGlossyReflection;
  }
  const f3 bd = toWorld(X, Y, N, wi);
  const f3 weight = pbrEval(bd, V, N, X, Y, ld3(m.a), a, m.c.y, m.b.z) * fabsf(wi.z);
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / (bpdf + EPS));
}

// brdf_kang18.rchit:113-135,223-249: direction pair, then the lobe choice;
// the pdf is the chosen lobe's alone
__device__ __forceinline__ void sampleKang18(PathIO& io, const HitSt& st, const MatDev& m) {
  const float ax = gmax(m.b.x, EPS), ay = gmax(m.b.y, EPS);
  const f3 kd = ld3(m.a), ks = ld3(m.c);
  const f2 u = rnd2(io.seed);
  const f3 V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  const f3 wo = makeNormal(toLocal(X, Y, N, V));
  const float dp = kangDiffuseProb(kd, ks);
  f3 wi;
  float bpdf;
  uint32_t bflags;
  if (rnd(io.seed) < dp) {
    wi = cosineSampleHemisphere(u);
    bflags = EDiffuseReflection;
    bpdf = cosineHemispherePdf(wi.z);
  } else {
    wi = importanceSampleAnisoGGX(u, wo, ax, ay);
    const f3 wh = makeNormal(wi + wo);
    bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
    bflags = EGlossyReflection;
  }
  const f3 bd = toWorld(X, Y, N, wi);
  const f3 weight = kangEval(bd, V, N, X, Y, kd, ks, ax, ay, m.b.z);
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / (bpdf + EPS));
}

// brdf_disney.rchit:302-378,469-477: lobe CDF (diffuse, clearcoat, specular)
// from an approximate Fresnel at N; the weight is scaled by |dot(N, L)| with
// N in world and L in the local frame (as the reference writes it)
__device__ __forceinline__ void sampleDisney(PathIO& io, const HitSt& st, const MatDev& m) {
  using namespace disney;
  const Mat mat = fromDev(m);
  const float eta = dot(st.V, st.N) > 0.0f ? (1.0f / m.b.z) : m.b.z;
  const f2 u = rnd2(io.seed);
  float pdf = 0.0f;
  f3 f = splat(0.0f);
  float r1 = u.x;
  const float r2 = u.y;
  const f3 N = st.ffN, X = st.X, Y = st.Y;
  const f3 V = toLocal(X, Y, N, st.V);
  f3 L;
  f3 specCol, sheenCol;
  SpecColor(mat, eta, specCol, sheenCol);
  float diffuseWt, specReflectWt, clearcoatWt;
  LobeProbabilities(mat, specCol, Fresnel(mat.metallic, eta, V.z, V.z), diffuseWt, specReflectWt, clearcoatWt);
  const float cdf0 = diffuseWt;
  const float cdf1 = cdf0 + clearcoatWt;
  uint32_t bflags;
  if (r1 < cdf0) {
    r1 = r1 / cdf0;
    L = cosineSampleHemisphere(f2{r1, r2});
    const f3 H = normalize(L + V);
    f = EvalDiffuse(mat, sheenCol, V, L, H, pdf);
    pdf = pdf * diffuseWt;
    bflags = EDiffuseReflection;
  } else if (r1 < cdf1) {
    r1 = (r1 - cdf0) / (cdf1 - cdf0);
    f3 H = SampleGTR1(mat.clearcoatRoughness, r1);
    if (H.z < 0.0f) H = -H;
    L = normalize(reflect(-V, H));
    f = EvalClearcoat(mat, V, L, H, pdf);
    pdf = pdf * clearcoatWt;
    bflags = EGlossyReflection;
  } else {
    r1 = (r1 - cdf1) / (1.0f - cdf1);
    f3 H = SampleGGXVNDF(V, mat.ax, mat.ay, r1, r2);
    if (H.z < 0.0f) H = -H;
    L = normalize(reflect(-V, H));
    f = EvalSpecReflection(mat, eta, specCol, V, L, H, pdf);
    pdf = pdf * specReflectWt;
    bflags = EGlossyReflection;
  }
  const f3 bd = toWorld(X, Y, N, L);
  const f3 weight = f * fabsf(dot(N, L));
  if (pdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = pdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / pdf);
}

// brdf_conductor.rchit:65-80,141-163: the direction sample ignores its two
// random numbers but draws them
__device__ __forceinline__ void sampleConductor(PathIO& io, const HitSt& st, const MatDev& m) {
  rnd2(io.seed);
  const f3 V = st.V, N = st.ffN;
  if (!(dot(V, N) > 0.0f)) {
    io.stop = true;
    return;
  }
  const f3 bd = reflect(-V, N);
  const f3 weight = ld3(m.a) * conductorReflectance3(ld3(m.c), ld3(m.d), dot(N, bd));
  if (length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = ESpecularReflection;
  io.bpdf = 1.0f;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = bd;
  io.thp = io.thp * (weight / (1.0f + EPS));
}

// brdf_rough_conductor.rchit:103-131,187-206
__device__ __forceinline__ void sampleRoughConductor(PathIO& io, const HitSt& st, const MatDev& m) {
  const float ax = gmax(EPS, m.b.x), ay = gmax(EPS, m.b.y);
  f2 u = rnd2(io.seed);
  const f3 V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  const float NdotV = dot(V, N);
  if (NdotV <= 0.0f) {
    io.stop = true;
    return;
  }
  const f3 wo = toLocal(X, Y, N, V);
  const f3 wi = importanceSampleAnisoGGX(u, wo, ax, ay);
  const f3 L = toWorld(X, Y, N, wi);
  const f3 H = makeNormal(V + L);
  const f3 wh = makeNormal(wi + wo);
  const float NdotL = dot(N, L);
  const f3 Fs = conductorReflectance3(ld3(m.c), ld3(m.d), NdotL);
  float Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
  Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
  const float Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
  const float bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
  const f3 weight = ld3(m.a) * Fs * Gs * Ds * NdotL;
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = EGlossyReflection;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = L;
  io.thp = io.thp * (weight / (bpdf + EPS));
}

// brdf_mirror.rchit:28-37,88-106
__device__ __forceinline__ void sampleMirror(PathIO& io, const HitSt& st, const MatDev& m) {
  const f3 weight = ld3(m.a);
  if (length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = ESpecularReflection;
  io.bpdf = 1.0f;
  io.nro = offsetPositionAlongNormal(st.pos, st.ffN);
  io.nrd = reflect(-st.V, st.ffN);
  io.thp = io.thp * (weight / 1.0f);
}

// bsdf_dielectric.rchit:54-72,273-289
__device__ __forceinline__ void sampleDielectric(PathIO& io, const HitSt& st, const MatDev& m) {
  const float ior = m.b.z;
  const float eta = dot(st.V, st.N) > 0.0f ? (1.0f / ior) : ior;
  float u = rnd(io.seed);
  const f3 V = st.V, N = st.ffN;
  float F = dielectricFresnel(fabsf(dot(V, N)), eta);
  f3 bd, weight;
  float bpdf;
  uint32_t bflags;
  if (u < F) {
    bd = makeNormal(reflect(-V, N));
    bpdf = F;
    bflags = ESpecularReflection;
    weight = F * splat(1.0f);
  } else {
    bd = makeNormal(refract(-V, N, eta));
    bpdf = 1.0f - F;
    bflags = ESpecularTransmission;
    weight = (1.0f - F) * splat(1.0f) * eta * eta;
  }
  if (bpdf <= 0.0f || length(weight) == 0.0f) {
    io.stop = true;
    return;
  }
  io.bflags = bflags;
  io.bpdf = bpdf;
  io.nro = offsetPositionAlongNormal(st.pos, gsign(dot(bd, st.N)) * st.N);
  io.nrd = bd;
  io.thp = io.thp * (weight / (bpdf + EPS));
}

}  // namespace

// ---------------------------------------------------------------------------
// Splits the hits of the extend queue into the shading classes (material
// sort).  A block takes 256 hits at a time: lanes are grouped by class in
// each warp (one shared-memory add per class present), then one global
// append per class present in the block, so the few class counters see
// eight times fewer atomics than with per-warp appends.  Classes that no hit
// of a pass uses cost one empty launch.
__global__ void __launch_bounds__(256) k_classify(KParams P) {
  __shared__ uint32_t count[kNumShadeClasses], base[kNumShadeClasses];
  const WaveDev& W = P.W;
  const SceneDev& S = P.S;
  const uint32_t n = W.cnt->c[kCntExtend0 + P.cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // the connect kernel that follows fetches shadow rays from 0
    W.cnt->c[kCntFetchShadow] = 0;
  }
  const uint32_t stride = gridDim.x * blockDim.x;
  // (i0 is the same for every thread of the block: the barriers are uniform)
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    if (threadIdx.x < kNumShadeClasses) count[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t i = i0 + threadIdx.x;
    int cls = -1;
    if (i < n) {
      const uint32_t inst = W.hitInst[i];
      cls = kClsTerminal;
      if (inst != 0xffffffffu) {
        const InstDev& in = S.inst[inst];
        if (__ldg(&in.lightId) < 0) {
          cls = shadeClassOf(__ldg(&in.matType));
        }
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, cls);
    const int leader = __ffs(peers) - 1;
    uint32_t off = 0;
    if (int(laneId()) == leader && cls >= 0) off = atomicAdd(&count[cls], uint32_t(__popc(peers)));
    off = __shfl_sync(0xffffffffu, off, leader);
    __syncthreads();
    if (threadIdx.x < kNumShadeClasses && count[threadIdx.x])
      base[threadIdx.x] = atomicAdd(&W.cnt->c[kCntCls0 + threadIdx.x], count[threadIdx.x]);
    __syncthreads();
    // (count was last read before the barrier above and base is written
    // again only after two more: the next round may start at once)
    if (cls >= 0) W.cls[cls][base[cls] + off + uint32_t(__popc(peers & ((1u << laneId()) - 1u)))] = i;
  }
}

// Shades the rays of one class: the miss shader, the light / emissive hit
// shaders (class kClsTerminal), or one material's hit shader with its
// next-event estimation and BSDF sampling.
template <int CLS>
__global__ void __launch_bounds__(256, kShadeMinBlocks) k_shadeClass(KParams P) {
  __shared__ uint32_t appendCount[2], appendBase[2];
  const WaveDev& W = P.W;
  const SceneDev& S = P.S;
  const int cur = P.cur, nxt = cur ^ 1;
  const uint32_t n = W.cnt->c[kCntCls0 + CLS];
  const uint32_t* list = W.cls[CLS];
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    const bool valid = i0 + threadIdx.x < n;
    const uint32_t i = valid ? list[i0 + threadIdx.x] : 0u;
    bool wantNext = false, wantShadow = false;
    PathIO io;
    uint32_t p = 0;
    uint4 rc = make_uint4(0, 0, 0, 0);
    if (valid) {
      const float4 o4 = W.rayO[cur][i];
      const float4 d4 = W.rayD[cur][i];
      p = __float_as_uint(d4.w);
      const f3 ro = ld3(o4), rd = ld3(d4);
      const float4 h4 = W.hit[i];
      const uint32_t inst = W.hitInst[i];
      const float4 t4 = W.path[p].thp;
      const float4 r4 = W.rad[p];
      const uint4 inf = W.path[p].info;
      if (P.records) rc = W.rec[p];
      const RangeDev R = W.ranges[inf.z];
      const ShotDev& sh = W.shots[R.shot];
      const uint32_t frame = R.frameBegin + inf.w / R.npix;
      const uint32_t pix = inf.w % R.npix;
      // a path that passed through surfaces without a bounce is that many
      // passes behind the wavefront: its own depth is what the shaders see
      uint32_t passes = inf.y >> kPassShift;
      const uint32_t depth = P.depth - passes;
      bool passThrough = false;
      io.seed = inf.x;
      io.bflags = inf.y & kFlagsMask;
      io.bpdf = t4.w;
      io.thp = ld3(t4);
      io.rad = ld3(r4);
      io.stop = false;
      io.dskip = true;
      io.drad = splat(0.0f);
      if (CLS == kClsTerminal && inst == 0xffffffffu) {
        // raytrace.default.rmiss:24-56
        io.stop = true;
        const bool sky = S.sky.in_use == 1;
        f3 env = sky ? evalSunSky(S, rd) : (sh.state.has_env_map == 1u) ? evalEnvmap(S, sh, rd) : ld3(sh.state.bg_color);
        float mis = 1.0f;
        if (depth != 1u && isNonSpecular(io.bflags)) {
          float envPdf = sky ? INV_4PI : (sh.state.has_env_map == 1u) ? pdfEnvmap(S, sh, rd) : INV_4PI;
          mis = powerHeuristic(io.bpdf, envPdf);
        }
        io.rad = io.rad + io.thp * env * mis;
        rc.x = sigMix(rc.x, 0xffffffffu);
      } else {
        const InstDev& in = S.inst[inst];
        const uint32_t prim = __float_as_uint(h4.w);
        rc.x = sigMix(rc.x, (inst << 20) ^ prim);
        HitSt st = hitState(S, in, prim, h4.y, h4.z, rd, sh.state.use_face_normal);
        if (CLS == kClsTerminal && in.lightId >= 0) {
          // brdf_lambertian.rchit:44-68 (hitLight)
          const LightDev l = S.lights[in.lightId];
          f3 ldir = makeNormal(rd);
          f3 lnrm = makeNormal(cross(ld3(l.u), ld3(l.v)));
          float proj = dot(lnrm, ldir);
          io.stop = true;
          if (!(proj > 0.0f && __float_as_uint(l.v.w) == 0u)) {
            float mis = 1.0f;
            if (isNonSpecular(io.bflags) && depth != 1u) {
              float dist = length(st.pos - ro);
              float d2 = dist * dist;
              float lpdf = d2 / (l.u.w * fabsf(proj) + EPS);
              mis = powerHeuristic(io.bpdf, lpdf);
            }
            io.rad = io.rad + io.thp * ld3(l.rad) * mis;
          }
        } else {
          MatDev m = S.mats[in.matId];
          applyTextures<CLS>(S, in, m, st, sh.state.use_face_normal);
          if (CLS == kClsKang18) {
            // brdf_kang18.rchit:178-181: the tangent frame is rebuilt from N and X
            st.Y = makeNormal(cross(st.N, st.X));
            st.X = makeNormal(cross(st.Y, st.N));
            st.ffN = dot(st.N, st.V) > 0.0f ? st.N : -st.N;
          }
          if (CLS == kClsPbr || CLS == kClsDisney || CLS == kClsKang18) {
            // brdf_pbr_metalness_roughness.rchit:151-160, brdf_disney.rchit:
            // 408-417, brdf_kang18.rchit:150-187: with probability opacity
            // the ray goes on from the far side of the surface, same
            // direction, no bounce counted (depth--), no light sample
            float opacity = CLS == kClsPbr ? m.c.z : (CLS == kClsDisney ? m.b.y : m.c.w);
            if (m.t1.z >= 0) opacity = texRGB(S, m.t1.z, st.u, st.v).x;
            passThrough = rnd(io.seed) < opacity;
          }
          if (passThrough) {
            io.nro = offsetPositionAlongNormal(st.pos, -st.ffN);
            io.nrd = rd;
          } else if (CLS == kClsPbr && depth == 1u && frame == 0u && sh.state.n_multi_channel > 0u) {
            // 169-174: albedo and the face-forward normal only
            const asuna_rt_state& ps = sh.state;
            const size_t npx = size_t(sh.width) * sh.height;
            if (ps.diffuse_out_channel >= 0 && ps.diffuse_out_channel < ASUNA_MAX_CHANNELS)
              sh.filmCh[size_t(ps.diffuse_out_channel) * npx + pix] = make_float4(m.a.x, m.a.y, m.a.z, 1.0f);
            if (ps.normal_out_channel >= 0 && ps.normal_out_channel < ASUNA_MAX_CHANNELS)
              sh.filmCh[size_t(ps.normal_out_channel) * npx + pix] = make_float4(st.ffN.x, st.ffN.y, st.ffN.z, 1.0f);
          }
          if ((CLS == kClsLambertian || CLS == kClsPhong || CLS == kClsKang18) && !passThrough && depth == 1u &&
              frame == 0u && sh.state.n_multi_channel > 0u) {
            // brdf_lambertian.rchit:93-108; brdf_phong.rchit:135-150 and
            // brdf_kang18.rchit:194-211 write the face-forward normal and the
            // specular reflectance (kang18: the rebuilt tangent, (ax, ay, 0))
            const asuna_rt_state& ps = sh.state;
            float4* ch = sh.filmCh;
            const size_t npx = size_t(sh.width) * sh.height;
            auto put = [&](int slot, f3 v) {
              if (slot >= 0 && slot < ASUNA_MAX_CHANNELS) ch[size_t(slot) * npx + pix] = make_float4(v.x, v.y, v.z, 1.0f);
            };
            put(ps.diffuse_out_channel, ld3(m.a));
            put(ps.normal_out_channel, CLS == kClsLambertian ? st.N : st.ffN);
            put(ps.specular_out_channel, CLS == kClsLambertian ? splat(0.0f) : ld3(m.c));
            put(ps.tangent_out_channel, st.X);
            put(ps.roughness_out_channel, CLS == kClsKang18 ? f3{gmax(m.b.x, EPS), gmax(m.b.y, EPS), 0.0f}
                                                            : f3{1.0f, 1.0f, 0.0f});
            put(ps.position_out_channel, st.pos);
            put(ps.uv_out_channel, f3{st.u, st.v, 1.0f});
          }
          if (CLS == kClsTerminal) {
            // brdf_emissive.rchit:12-27: add the emitted radiance and stop
            io.stop = true;
            if (sh.state.ignore_emissive == 0u) io.rad = io.rad + ld3(m.a) * io.thp;
          } else if (!passThrough) {
            constexpr uint32_t type = CLS == kClsRoughPlastic ? ASUNA_MAT_ROUGH_PLASTIC
                                      : CLS == kClsDielectric ? ASUNA_MAT_DIELECTRIC
                                      : CLS == kClsPlastic    ? ASUNA_MAT_PLASTIC
                                      : CLS == kClsMirror     ? ASUNA_MAT_MIRROR
                                      : CLS == kClsConductor  ? ASUNA_MAT_CONDUCTOR
                                      : CLS == kClsRoughConductor ? ASUNA_MAT_ROUGH_CONDUCTOR
                                      : CLS == kClsPhong      ? ASUNA_MAT_PHONG
                                      : CLS == kClsPbr        ? ASUNA_MAT_PBR_METALNESS_ROUGHNESS
                                      : CLS == kClsDisney     ? ASUNA_MAT_DISNEY
                                      : CLS == kClsKang18     ? ASUNA_MAT_KANG18
                                                              : ASUNA_MAT_LAMBERTIAN;
            nextEvent(S, sh, io, st, m, type, rd);
            if (CLS == kClsRoughPlastic)
              sampleRoughPlastic(io, st, m);
            else if (CLS == kClsDielectric)
              sampleDielectric(io, st, m);
            else if (CLS == kClsPlastic)
              samplePlastic(io, st, m);
            else if (CLS == kClsMirror)
              sampleMirror(io, st, m);
            else if (CLS == kClsConductor)
              sampleConductor(io, st, m);
            else if (CLS == kClsRoughConductor)
              sampleRoughConductor(io, st, m);
            else if (CLS == kClsPhong)
              samplePhong(io, st, m);
            else if (CLS == kClsPbr)
              samplePbr(io, st, m);
            else if (CLS == kClsDisney)
              sampleDisney(io, st, m);
            else if (CLS == kClsKang18)
              sampleKang18(io, st, m);
            else
              sampleLambertian(io, st, ld3(m.a));
          }
          rc.x = sigMix(rc.x, io.stop ? 0xfffu : io.bflags);
        }
        if (depth == 1u && frame == 0u && sh.depthSlot >= 0 && sh.depthSlot < ASUNA_MAX_CHANNELS) {
          const size_t npx = size_t(sh.width) * sh.height;
          sh.filmCh[size_t(sh.depthSlot) * npx + pix] = make_float4(h4.x, h4.x, h4.x, 1.0f);
        }
      }
      wantShadow = !io.dskip;
      // rgen:101-133: a pass-through leaves depth unchanged, so the loop goes on
      bool alive = passThrough || (!io.stop && depth < uint32_t(sh.state.max_path_depth));
      if (passThrough) ++passes;
      if (CLS != kClsTerminal && alive && !passThrough && (sh.flags & ASUNA_SHOT_RR) && depth >= sh.rrDepth) {
        // Russian roulette (extension; off for the reference's streams)
        float q = gmin(0.95f, gmax(io.thp.x, gmax(io.thp.y, io.thp.z)));
        float u = rnd(io.seed);
        if (!(u < q))
          alive = false;
        else
          io.thp = io.thp / q;
      }
      wantNext = alive;
      if (P.records) {
        rc.w = depth;
        if (wantShadow) rc.z |= 1u << (depth - 1u);
      }
      // path state
      W.path[p].thp = make_float4(io.thp.x, io.thp.y, io.thp.z, io.bpdf);
      W.rad[p] = make_float4(io.rad.x, io.rad.y, io.rad.z, r4.w);
      W.path[p].info = make_uint4(io.seed, io.bflags | (passes << kPassShift), inf.z, inf.w);
      if (P.records) W.rec[p] = rc;
    }
    __syncwarp();
    if (CLS != kClsTerminal) {  // terminal paths append nothing
      // (i0 is the same for every thread of the block: the barriers inside
      // are reached by all of them, round by round)
      uint32_t sslot, nslot;
      blockAppend2(wantShadow, wantNext, &W.cnt->c[kCntShadow], &W.cnt->c[kCntExtend0 + nxt], appendCount,
                   appendBase, sslot, nslot);
      if (wantShadow) {
        float maxDist = io.ddist - 2.0f * EPS;
        W.shO[sslot] = make_float4(io.dro.x, io.dro.y, io.dro.z, maxDist);
        W.shD[sslot] = make_float4(io.drd.x, io.drd.y, io.drd.z, __uint_as_float(p));
        W.shC[sslot] = make_float4(io.drad.x, io.drad.y, io.drad.z, 0.0f);
      }
      if (wantNext) {
        W.rayO[nxt][nslot] = make_float4(io.nro.x, io.nro.y, io.nro.z, INF);
        W.rayD[nxt][nslot] = make_float4(io.nrd.x, io.nrd.y, io.nrd.z, __uint_as_float(p));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// accumulate: rgen:147-179, frames in order, one thread per pixel of a range
__global__ void __launch_bounds__(256) k_accumulate(KParams P) {
  const WaveDev& W = P.W;
  const RangeDev R = W.ranges[blockIdx.y];
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= R.npix) return;
  const ShotDev& sh = W.shots[R.shot];
  float4 old = sh.filmRad[pix];
  float ow = sh.filmW[pix].x;
  for (uint32_t f = 0; f < R.nframes; ++f) {
    const uint32_t p = R.pathBegin + f * R.npix + pix;
    const uint32_t frame = R.frameBegin + f;
    const float4 r4 = W.rad[p];
    const float fw = r4.w;
    float rcl[3] = {gclamp(r4.x, 0.0f, 10.0f), gclamp(r4.y, 0.0f, 10.0f), gclamp(r4.z, 0.0f, 10.0f)};
    float rws[3] = {fw * rcl[0], fw * rcl[1], fw * rcl[2]};
    if (frame == 0) {
      old = make_float4(rws[0] / fw, rws[1] / fw, rws[2] / fw, 1.0f);
      ow = fw;
    } else {
      float nw = ow + fw;
      old = make_float4((old.x * ow + rws[0]) / nw, (old.y * ow + rws[1]) / nw, (old.z * ow + rws[2]) / nw, 1.0f);
      ow = nw;
    }
  }
  sh.filmRad[pix] = old;
  sh.filmW[pix] = make_float4(ow, ow, ow, ow);
}

// ---------------------------------------------------------------------------
// parity records: copy per-path radiance / filter weight with the record
__global__ void __launch_bounds__(256) k_records(KParams P, asuna_path_record* out) {
  const WaveDev& W = P.W;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W.numPaths; p += gridDim.x * blockDim.x) {
    const float4 r4 = W.rad[p];
    const uint4 rc = W.rec[p];
    asuna_path_record o;
    o.radiance[0] = r4.x;
    o.radiance[1] = r4.y;
    o.radiance[2] = r4.z;
    o.filter_weight = r4.w;
    o.depth = rc.w;
    o.signature = rc.x;
    o.events = rc.y;
    o.shadows = rc.z;
    out[p] = o;
  }
}

// ---------------------------------------------------------------------------
void launchRaygen(const KParams& P, int grid, cudaStream_t s) { k_raygen<<<grid, 256, 0, s>>>(P); }
// classify, then one kernel per shading class the scene's materials can
// reach (each a persistent grid over its own list)
void launchShade(const KParams& P, int grid, cudaStream_t s) {
  k_classify<<<grid, 256, 0, s>>>(P);
  const uint32_t m = P.S.classMask | (1u << kClsTerminal);
  if (m & (1u << kClsTerminal)) k_shadeClass<kClsTerminal><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsLambertian)) k_shadeClass<kClsLambertian><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsRoughPlastic)) k_shadeClass<kClsRoughPlastic><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsDielectric)) k_shadeClass<kClsDielectric><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsPlastic)) k_shadeClass<kClsPlastic><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsMirror)) k_shadeClass<kClsMirror><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsConductor)) k_shadeClass<kClsConductor><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsRoughConductor)) k_shadeClass<kClsRoughConductor><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsPhong)) k_shadeClass<kClsPhong><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsPbr)) k_shadeClass<kClsPbr><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsDisney)) k_shadeClass<kClsDisney><<<grid, 256, 0, s>>>(P);
  if (m & (1u << kClsKang18)) k_shadeClass<kClsKang18><<<grid, 256, 0, s>>>(P);
}
int shadeLaunches(uint32_t classMask) { return 1 + __builtin_popcount(classMask | (1u << kClsTerminal)); }
int shadeBlocksPerSm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadeClass<kClsRoughPlastic>, 256, 0);
  return n > 0 ? n : 1;
}
void launchAccumulate(const KParams& P, uint32_t maxPix, uint32_t nranges, cudaStream_t s) {
  dim3 g((maxPix + 255) / 256, nranges);
  k_accumulate<<<g, 256, 0, s>>>(P);
}
void launchRecords(const KParams& P, asuna_path_record* out, int grid, cudaStream_t s) {
  k_records<<<grid, 256, 0, s>>>(P, out);
}

}  // namespace asuna
