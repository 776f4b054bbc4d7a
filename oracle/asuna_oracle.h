/*
 * asuna_oracle.h — CPU oracle of the path-tracer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a scalar C++ restatement of the
 * reference's ray-tracing path (Asuna's GLSL shaders: raytrace.projective.rgen,
 * raytrace.default.rmiss, raytrace.shadow.rmiss, utils/{math,structs,
 * rchit_layouts,sample_light}.glsl, bxdf/{brdf_lambertian,brdf_rough_plastic,
 * bsdf_dielectric,brdf_emissive}.rchit) used as the checker of the CUDA path.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it;
 * the library never does.
 *
 * Parity status: pinned against the reference's own shader source compiled as
 * host C++ (see oracle/gen_ref.py) and against golden vectors generated from
 * it.  BVH traversal is this oracle's own (the reference's is closed RT-core
 * hardware), so hit selection at exact ties is not pinned by the reference.
 */
#ifndef ASUNA_ORACLE_H
#define ASUNA_ORACLE_H

#include "../include/asuna_rt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene oracle_scene;

typedef struct oracle_stats {
  uint64_t paths;
  uint64_t extend_rays;
  uint64_t shadow_rays;
  uint64_t nodes_visited;
  uint64_t tris_tested;
  double seconds;
  int threads;
} oracle_stats;

/* Builds the oracle's own BVHs (object-median split) and env tables. */
int oracle_scene_create(const asuna_scene_desc* desc, oracle_scene** out);
void oracle_scene_destroy(oracle_scene* s);

/*
 * Renders frames [shot->frame0, shot->frame0 + shot->frames) of one shot.
 * film: 9 images of width*height*4 floats (in/out; read when frame0 > 0).
 * records: one per (frame, pixel) in [frame][pixel-list] order, or NULL.
 * pixels/npixels: optional subset of linear pixel indices (NULL = all).
 * precision: 32 = float (parity), 64 = double (quality reference).
 */
int oracle_render(const oracle_scene* s, const asuna_shot* shot, float* film,
                  asuna_path_record* records, const uint32_t* pixels, uint32_t npixels,
                  int nthreads, int precision, oracle_stats* stats);

/* Per-path radiance only (no film), double precision accumulation of a
 * pixel subset: out[i*3+c] = mean clamped radiance weighted by the filter,
 * i.e. the converged pixel value estimate after `shot->frames` frames. */
int oracle_render_pixels_f64(const oracle_scene* s, const asuna_shot* shot, const uint32_t* pixels,
                             uint32_t npixels, int nthreads, double* out_rgb, double* out_var,
                             oracle_stats* stats);

/* Known-answer hooks. */
uint32_t oracle_xxhash32(uint32_t x, uint32_t y, uint32_t z);
uint32_t oracle_pcg(uint32_t* state);
float oracle_rand(uint32_t* state);
/* Closest hit in world space; returns 1 on hit. */
int oracle_trace(const oracle_scene* s, const float o[3], const float d[3], float tmin, float tmax,
                 float* t, uint32_t* inst, uint32_t* prim, float* bu, float* bv);
/* Any hit in [tmin, tmax]; returns 1 if occluded. */
int oracle_occluded(const oracle_scene* s, const float o[3], const float d[3], float tmin,
                    float tmax);
/* World-to-object 3x4 of an object-to-world 3x4 (double inverse, rounded once). */
void oracle_invert3x4(const float* m12, float* out12);
/* The float transcendentals of include/asuna_math.h: 0 sin, 1 cos, 2 exp,
 * 3 acos, 4 atan2(x, y), 5 log2, 6 exp2, 7 pow(x, y), 8 log, 9 tan. */
float oracle_math(int which, float x, float y);
/* Env tables (marginal/conditional .xy per texel). */
int oracle_envmap_tables(uint32_t w, uint32_t h, const float* rgba, float* marg_xy, float* cond_xy);
/* Post pass (tone mapping) of one RGBA image, as the library's asuna_tonemap. */
int oracle_tonemap(const float* rgba, uint32_t w, uint32_t h, const asuna_post_state* post, float* out);

/* Host preprocessing a scene description needs, restated here so that a run
 * timing only the reference's code builds its workload without the library.
 * computeDiffuseFresnel (src/loader/material.cpp:6-37). */
float oracle_diffuse_fresnel(float ior, int samples);
/* CameraPerspective::toGpuStruct (src/core/camera.cpp:28-62, 87-99; view =
 * scale(1,-1,-1) * lookAt, src/core/camera.h:26-28); fov horizontal, degrees. */
int oracle_camera_perspective(const float eye[3], const float lookat[3], const float up[3], float fov_deg,
                              float aperture, float focal_distance, uint32_t width, uint32_t height,
                              asuna_camera* out);

#ifdef __cplusplus
}
#endif

#endif
