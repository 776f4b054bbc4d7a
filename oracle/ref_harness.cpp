// ref_harness.cpp — runs the reference's own ray-tracing shader code on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Includes the shader source translated by
// oracle/gen_ref.py (into oracle/_ref/gen/, never committed) and supplies what
// the Vulkan ray-tracing pipeline gives those shaders: the descriptor-bound
// globals (push constant, camera UBO, instances, lights, env samplers, output
// images), the gl_* built-ins, and traceRayEXT.  traceRayEXT runs the CPU
// oracle's closest-hit / any-hit traversal, then invokes the miss shader or
// the closest-hit shader selected the way the reference's SBT does
// (instance SBT offset = material type, emitters use the Lambertian group;
// src/pipeline/pipeline_raytrace.cpp:134-140).
//
// Built into oracle/_ref/libasuna_ref.so by oracle/build_oracle.py when the
// reference tree is present; pins oracle/asuna_oracle.cpp.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <new>
#include <cstdint>
#include <thread>
#include <vector>

#include "asuna_oracle.h"
#include "glsl_shim.h"
// The reference's shared host/shader headers, compiled as C++ exactly as the
// reference's host code compiles them.
#include <shared/binding.h>
#include <shared/camera.h>
#include <shared/instance.h>
#include <shared/light.h>
#include <shared/material.h>
#include <shared/pushconstant.h>
#include <shared/sun_and_sky.h>
#include <shared/vertex.h>

static_assert(sizeof(GpuVertex) == sizeof(asuna_vertex), "GpuVertex layout");
static_assert(sizeof(GpuMaterial) == sizeof(asuna_material), "GpuMaterial layout");
static_assert(sizeof(GpuLight) == sizeof(asuna_light), "GpuLight layout");
static_assert(sizeof(GpuCamera) == sizeof(asuna_camera), "GpuCamera layout");
static_assert(sizeof(GpuPushConstantRaytrace) == sizeof(asuna_rt_state), "push constant layout");
static_assert(sizeof(GpuSunAndSky) == sizeof(asuna_sun_and_sky), "GpuSunAndSky layout");

namespace glslx {
// ---- globals the shaders reach through descriptors / built-ins ------------
struct InstancesBuf {
  GpuInstance* i;
};
struct LightsBuf {
  GpuLight* l;
};
struct Vertices {
  GpuVertex* v;
  explicit Vertices(uint64_t a) : v(reinterpret_cast<GpuVertex*>(a)) {}
};
struct Indices {
  ivec3* i;
  explicit Indices(uint64_t a) : i(reinterpret_cast<ivec3*>(a)) {}
};
struct Materials {
  GpuMaterial* m;
  explicit Materials(uint64_t a) : m(reinterpret_cast<GpuMaterial*>(a)) {}
};

static accelerationStructureEXT tlas;
static image2D images[NUM_OUTPUT_IMAGES];
static GpuCamera cameraInfo;
static GpuSunAndSky sunAndSky;
static sampler2D envmapSamplers[3];
static std::vector<sampler2D> textureSamplers(1);
static InstancesBuf instances;
static LightsBuf lights;
static thread_local GpuPushConstantRaytrace pc;
static thread_local uvec3 gl_LaunchIDEXT;
static thread_local int gl_InstanceID;
static thread_local int gl_PrimitiveID;
static thread_local vec3 gl_WorldRayDirectionEXT;
static thread_local mat4x3 gl_ObjectToWorldEXT;
static thread_local mat4x3 gl_WorldToObjectEXT;
static thread_local vec2 _bary;
static thread_local bool isShadowed;

void traceRayEXT(accelerationStructureEXT, uint flags, uint mask, uint sbtOffset, uint sbtStride, uint missIndex,
                 vec3 origin, float tmin, vec3 dir, float tmax, int payloadLoc);
}  // namespace glslx

namespace glslx {
#include "structs.glsl.h"
static thread_local RayPayload payload;
#include "raytrace.projective.rgen.h"
#include "raytrace.default.rmiss.h"
#include "raytrace.shadow.rmiss.h"
#include "raytrace.brdf_lambertian.rchit.h"
#include "raytrace.brdf_rough_plastic.rchit.h"
#include "raytrace.bsdf_dielectric.rchit.h"
#include "raytrace.brdf_emissive.rchit.h"
#include "raytrace.brdf_plastic.rchit.h"
#include "raytrace.brdf_mirror.rchit.h"
#include "raytrace.brdf_conductor.rchit.h"
#include "raytrace.brdf_rough_conductor.rchit.h"
#include "raytrace.brdf_phong.rchit.h"
#include "raytrace.brdf_pbr_metalness_roughness.rchit.h"
#include "raytrace.brdf_disney.rchit.h"
#include "raytrace.brdf_kang18.rchit.h"
}  // namespace glslx

namespace {
struct RefScene {
  const oracle_scene* os = nullptr;
  std::vector<GpuInstance> inst;
  std::vector<glslx::mat4x3> o2w, w2o;
  std::vector<int> lightId, matType;
  std::vector<GpuLight> lights;
  std::vector<GpuMaterial> mats;
  std::vector<float> env, marg, cond;
};
RefScene* gS = nullptr;

struct PathTls {
  uint32_t sig, events, shadows;
};
thread_local PathTls tls;
// rays this thread traced (closest hit, occlusion)
thread_local uint64_t tlsExtendRays = 0, tlsShadowRays = 0;

inline uint32_t sigMix(uint32_t h, uint32_t v) { return h ^ (v + 0x9e3779b9u + (h << 6) + (h >> 2)); }

glslx::mat4x3 toMat4x3(const float* rm) {
  glslx::mat4x3 m;
  for (int c = 0; c < 4; ++c) m.c[c] = glslx::vec3(rm[0 * 4 + c], rm[1 * 4 + c], rm[2 * 4 + c]);
  return m;
}
}  // namespace

namespace glslx {
void traceRayEXT(accelerationStructureEXT, uint, uint, uint, uint, uint, vec3 origin, float tmin, vec3 dir, float tmax,
                 int payloadLoc) {
  float o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
  const uint32_t bit = 1u << (payload.pRec.depth - 1);
  if (payloadLoc == 1) {
    // occlusion ray: terminate on first hit, no closest-hit shader
    ++tlsShadowRays;
    tls.shadows |= bit;
    if (!oracle_occluded(gS->os, o, d, tmin, tmax)) {
      stage_shadow::main();
      tls.events |= bit;
    }
    return;
  }
  float t, bu, bv;
  uint32_t inst, prim;
  ++tlsExtendRays;
  if (!oracle_trace(gS->os, o, d, tmin, tmax, &t, &inst, &prim, &bu, &bv)) {
    stage_miss::main();
    tls.sig = sigMix(tls.sig, 0xffffffffu);
    return;
  }
  gl_InstanceID = int(inst);
  gl_PrimitiveID = int(prim);
  _bary = vec2(bu, bv);
  gl_WorldRayDirectionEXT = dir;
  gl_ObjectToWorldEXT = gS->o2w[inst];
  gl_WorldToObjectEXT = gS->w2o[inst];
  tls.sig = sigMix(tls.sig, (inst << 20) ^ prim);
  if (gS->lightId[inst] >= 0) {
    stage_lambertian::main();
    return;
  }
  switch (gS->matType[inst]) {
    case MaterialTypeBrdfRoughPlastic:
      stage_rough_plastic::main();
      break;
    case MaterialTypeBsdfDielectric:
      stage_dielectric::main();
      break;
    case MaterialTypeBrdfEmissive:
      stage_emissive::main();
      break;
    case MaterialTypeBrdfPlastic:
      stage_plastic::main();
      break;
    case MaterialTypeBrdfMirror:
      stage_mirror::main();
      break;
    case MaterialTypeBrdfConductor:
      stage_conductor::main();
      break;
    case MaterialTypeBrdfRoughConductor:
      stage_rough_conductor::main();
      break;
    case MaterialTypeBrdfPhong:
      stage_phong::main();
      break;
    case MaterialTypeBrdfPbrMetalnessRoughness:
      stage_pbr::main();
      break;
    case MaterialTypeBrdfDisney:
      stage_disney::main();
      break;
    case MaterialTypeBrdfKang18:
      stage_kang18::main();
      break;
    default:
      stage_lambertian::main();
      break;
  }
  tls.sig = sigMix(tls.sig, payload.pRec.stop ? 0xfffu : payload.bRec.flags);
}
}  // namespace glslx

extern "C" {

uint32_t ref_xxhash32(uint32_t x, uint32_t y, uint32_t z) { return glslx::xxhash32Seed(glslx::uvec3(glslx::uvec2{x, y}, z)); }
float ref_rand(uint32_t* state) {
  glslx::uint s = *state;
  float r = glslx::rand(s);
  *state = s;
  return r;
}

// Renders a shot with the reference's shader code; film = 9 images of
// W*H*4 floats; records (optional) hold the clamped per-path radiance (the
// rgen writes the clamp back into the payload, rgen:147), depth, signature
// and shadow bits.  Only seed 0 (the reference's streams) is meaningful.
// Scene state of the shaders' descriptors, set up for one render.
static int refSetup(const asuna_scene_desc* d, const asuna_shot* shot, float* film, RefScene& S) {
  using namespace glslx;
  oracle_scene* os = nullptr;
  int rc = oracle_scene_create(d, &os);
  if (rc) return rc;
  S.os = os;
  const uint32_t W = shot->width, H = shot->height;
  S.lights.assign(reinterpret_cast<const GpuLight*>(d->lights), reinterpret_cast<const GpuLight*>(d->lights) + d->num_lights);
  S.mats.assign(reinterpret_cast<const GpuMaterial*>(d->materials),
                reinterpret_cast<const GpuMaterial*>(d->materials) + d->num_materials);
  for (uint32_t i = 0; i < d->num_instances; ++i) {
    const asuna_instance_desc& in = d->instances[i];
    const asuna_mesh_desc& m = d->meshes[in.mesh_id];
    GpuInstance gi{};
    gi.vertexAddress = reinterpret_cast<uint64_t>(m.vertices);
    gi.indexAddress = reinterpret_cast<uint64_t>(m.indices);
    gi.materialAddress = in.light_id < 0 ? reinterpret_cast<uint64_t>(&S.mats[in.material_id]) : 0;
    gi.lightId = in.light_id;
    S.inst.push_back(gi);
    float w2o[12];
    oracle_invert3x4(in.transform, w2o);
    S.o2w.push_back(toMat4x3(in.transform));
    S.w2o.push_back(toMat4x3(w2o));
    S.lightId.push_back(in.light_id);
    S.matType.push_back(in.light_id < 0 ? int(S.mats[in.material_id].type) : 0);
  }
  // env samplers: data, conditional (.x inverse CDF, .y pdf), marginal
  uint32_t ew = 1, eh = 1;
  if (d->envmap.rgba && d->envmap.width && d->envmap.height) {
    ew = d->envmap.width;
    eh = d->envmap.height;
    S.env.assign(d->envmap.rgba, d->envmap.rgba + size_t(ew) * eh * 4);
  } else {
    S.env.assign(4, 0.0f);
  }
  S.marg.assign(size_t(ew) * eh * 2, 0.0f);
  S.cond.assign(size_t(ew) * eh * 2, 0.0f);
  if (d->envmap.rgba && d->envmap.width) oracle_envmap_tables(ew, eh, S.env.data(), S.marg.data(), S.cond.data());
  gS = &S;
  textureSamplers.assign(std::max(1u, d->num_textures), sampler2D{});
  for (uint32_t i = 0; i < d->num_textures; ++i)
    textureSamplers[i] = sampler2D{int(d->textures[i].width), int(d->textures[i].height), 4, d->textures[i].rgba};
  envmapSamplers[0] = sampler2D{int(ew), int(eh), 4, S.env.data()};
  envmapSamplers[1] = sampler2D{int(ew), int(eh), 2, S.marg.data()};
  envmapSamplers[2] = sampler2D{int(ew), int(eh), 2, S.cond.data()};
  instances.i = S.inst.data();
  lights.l = S.lights.data();
  std::memcpy(&cameraInfo, &shot->camera, sizeof(GpuCamera));
  sunAndSky = GpuSunAndSky{};
  sunAndSky.in_use = 0;
  if (d->sun_and_sky) std::memcpy(&sunAndSky, d->sun_and_sky, sizeof(GpuSunAndSky));
  for (int k = 0; k < NUM_OUTPUT_IMAGES; ++k) images[k] = image2D{film + size_t(k) * W * H * 4, int(W), int(H)};
  return ASUNA_OK;
}

static void refTeardown(RefScene& S) {
  gS = nullptr;
  oracle_scene_destroy(const_cast<oracle_scene*>(S.os));
}

// Runs the rgen for frames [frame0, frame0 + frames) of the listed pixels
// (all pixels when `pixels` is NULL) on `nthreads` threads.
static void refRun(const asuna_shot* shot, const uint32_t* pixels, uint32_t npix, asuna_path_record* records,
                   int nthreads, uint64_t* extendRays, uint64_t* shadowRays) {
  using namespace glslx;
  const uint32_t W = shot->width;
  GpuPushConstantRaytrace base;
  std::memcpy(&base, &shot->state, sizeof(base));
  base.spp = 1;
  if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<uint32_t> next{0};
  std::atomic<uint64_t> ext{0}, sh{0};
  auto worker = [&] {
    tlsExtendRays = tlsShadowRays = 0;
    for (;;) {
      uint32_t k = next.fetch_add(1);
      if (k >= npix) break;
      const uint32_t i = pixels ? pixels[k] : k;
      for (uint32_t f = 0; f < shot->frames; ++f) {
        uint32_t frame = shot->frame0 + f;
        pc = base;
        pc.curFrame = int(frame);
        gl_LaunchIDEXT = uvec3(uvec2{i % W, i / W}, 0u);
        tls = PathTls{0, 0, 0};
        stage_rgen::main();
        if (records) {
          asuna_path_record& r = records[size_t(f) * npix + k];
          r.radiance[0] = payload.pRec.radiance.x;
          r.radiance[1] = payload.pRec.radiance.y;
          r.radiance[2] = payload.pRec.radiance.z;
          r.filter_weight = 0.0f;
          uint32_t dep = payload.pRec.depth;
          r.depth = dep > uint32_t(pc.maxPathDepth) ? uint32_t(pc.maxPathDepth) : dep;
          r.signature = tls.sig;
          r.events = tls.events;
          r.shadows = tls.shadows;
        }
      }
    }
    ext += tlsExtendRays;
    sh += tlsShadowRays;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
  worker();
  for (auto& t : th) t.join();
  if (extendRays) *extendRays = ext.load();
  if (shadowRays) *shadowRays = sh.load();
}

// Renders a shot with the reference's shader code; film = 9 images of
// W*H*4 floats; records (optional) hold the clamped per-path radiance (the
// rgen writes the clamp back into the payload, rgen:147), depth, signature
// and shadow bits.  Only seed 0 (the reference's streams) is meaningful.
int ref_render(const asuna_scene_desc* d, const asuna_shot* shot, float* film, asuna_path_record* records,
               int nthreads) {
  if (!d || !shot || !film) return ASUNA_ERR_INVALID;
  if (shot->seed != 0 || (shot->flags & ASUNA_SHOT_RR)) return ASUNA_ERR_UNSUPPORTED;
  RefScene S;
  int rc = refSetup(d, shot, film, S);
  if (rc) return rc;
  refRun(shot, nullptr, shot->width * shot->height, records, nthreads, nullptr, nullptr);
  refTeardown(S);
  return ASUNA_OK;
}

// The reference's shader code over pixel samples (throughput measurement).
// ref_sample_begin sets the shaders' scene state up once (the oracle's BVH
// build included) for shots of `shot`'s size writing into `film` (9 images
// of W*H*4 floats, kept by the caller); ref_sample_run renders frames
// [frame0, frame0 + frames) of the listed pixels and reports the rays traced
// and the seconds spent; ref_sample_end releases the state.  One session at
// a time (the shaders' descriptors are process-wide).  The reference has no
// Russian roulette: a shot asking for it is rejected.
void* ref_sample_begin(const asuna_scene_desc* d, const asuna_shot* shot, float* film) {
  if (!d || !shot || !film || gS) return nullptr;
  RefScene* S = new (std::nothrow) RefScene;
  if (!S) return nullptr;
  if (refSetup(d, shot, film, *S) != ASUNA_OK) {
    delete S;
    return nullptr;
  }
  return S;
}

int ref_sample_run(void* session, const asuna_shot* shot, const uint32_t* pixels, uint32_t npixels, int nthreads,
                   oracle_stats* stats) {
  if (!session || session != gS || !shot || !pixels || !stats) return ASUNA_ERR_INVALID;
  if (shot->seed != 0 || (shot->flags & ASUNA_SHOT_RR)) return ASUNA_ERR_UNSUPPORTED;
  const uint32_t npix = shot->width * shot->height;
  for (uint32_t k = 0; k < npixels; ++k)
    if (pixels[k] >= npix) return ASUNA_ERR_INVALID;
  std::memcpy(&glslx::cameraInfo, &shot->camera, sizeof(GpuCamera));
  if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
  const auto t0 = std::chrono::steady_clock::now();
  uint64_t ext = 0, sh = 0;
  refRun(shot, pixels, npixels, nullptr, nthreads, &ext, &sh);
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::memset(stats, 0, sizeof(*stats));
  stats->paths = uint64_t(npixels) * shot->frames;
  stats->extend_rays = ext;
  stats->shadow_rays = sh;
  stats->seconds = sec;
  stats->threads = nthreads;
  return ASUNA_OK;
}

void ref_sample_end(void* session) {
  if (!session || session != gS) return;
  RefScene* S = static_cast<RefScene*>(session);
  refTeardown(*S);
  delete S;
}

}  // extern "C"
