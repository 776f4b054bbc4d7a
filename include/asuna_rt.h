/*
 * asuna_rt.h — C ABI of the GB300 path-tracer core.
 *
 * This is the drop-in boundary for Asuna's Vulkan ray-tracing path
 * (camera rays -> BVH traversal -> BSDF/NEE/MIS shading -> accumulation into
 * radiance/AOV images).  Every entry point takes plain pointers and sizes and
 * returns an int status (ASUNA_OK == 0); the text of the last failure on the
 * calling thread is returned by asuna_last_error().  No call ever exits the
 * process (the reference calls exit(1) on every error, src/loader/utils.h:11-16).
 *
 * Device ABI.  The structs below are byte-for-byte the reference's shared
 * host/shader structs (src/shared/), so a caller that already fills
 * GpuVertex / GpuMaterial / GpuLight / GpuCamera / GpuPushConstantRaytrace can
 * pass its arrays unchanged.  Matrices are 16 floats in column-major order,
 * the GLSL/nvmath convention of the reference (src/shared/camera.h:15-24).
 *
 * Replaced reference interfaces (file:line in the reference project):
 *   asuna_scene_create      Scene::submit (src/scene/scene.cpp:26-85) +
 *                           PipelineRaytrace::createBottomLevelAS/TopLevelAS
 *                           (src/pipeline/pipeline_raytrace.cpp:107-147)
 *   asuna_render            the offline frame loop of Tracer::runOffline
 *                           (src/tracer/tracer.cpp:204-258) around
 *                           PipelineRaytrace::run (pipeline_raytrace.cpp:36-74)
 *   asuna_film_read         Tracer::saveBufferToImage read-back
 *                           (src/tracer/tracer.cpp:313-395)
 *   asuna_json_load         Loader::loadSceneFromJson + Loader::parse
 *                           (src/loader/loader.cpp:67-144) with Scene::reset /
 *                           addLight / addInstance (src/scene/scene.cpp:87-316)
 *   asuna_tracer_run_offline Tracer::runOffline + callSavingImage
 *                           (src/tracer/tracer.cpp:177-291)
 */
#ifndef ASUNA_RT_H
#define ASUNA_RT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASUNA_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------ */
enum {
  ASUNA_OK = 0,
  ASUNA_ERR_INVALID = 1,     /* bad argument, size or handle               */
  ASUNA_ERR_CUDA = 2,        /* a CUDA runtime call failed                 */
  ASUNA_ERR_OOM = 3,         /* device or host allocation failed           */
  ASUNA_ERR_IO = 4,          /* file could not be read or written          */
  ASUNA_ERR_PARSE = 5,       /* JSON / OBJ / image syntax or schema error  */
  ASUNA_ERR_TIMEOUT = 6,     /* a bounded device wait gave up              */
  ASUNA_ERR_UNSUPPORTED = 7, /* feature outside the implemented plugin set */
  ASUNA_ERR_NO_DEVICE = 8,   /* no CUDA device / library built without it  */
  ASUNA_ERR_BUSY = 9,        /* server queue full: request rejected        */
  ASUNA_ERR_TRAVERSAL = 10   /* a BVH traversal was cut short (stack or
                                loop bound): the rendered image is wrong  */
};

/* ---- enums of the reference's plugin dispatch --------------------------- */
/* CameraType, src/shared/camera.h:7-11 */
enum { ASUNA_CAMERA_PERSPECTIVE = 0, ASUNA_CAMERA_OPENCV = 1, ASUNA_CAMERA_UNDEFINED = 2 };
/* LightType, src/shared/light.h:7-13 */
enum {
  ASUNA_LIGHT_DIRECTIONAL = 0,
  ASUNA_LIGHT_RECT = 1,
  ASUNA_LIGHT_TRIANGLE = 2,
  ASUNA_LIGHT_POINT = 3,
  ASUNA_LIGHT_UNDEFINED = 4
};
/* MaterialType, src/shared/material.h:7-21 (the eight marked (*) are
 * implemented; others are rejected with ASUNA_ERR_UNSUPPORTED) */
enum {
  ASUNA_MAT_LAMBERTIAN = 0, /* (*) brdf_lambertian   */
  ASUNA_MAT_KANG18 = 1, /* (*) brdf_kang18        */
  ASUNA_MAT_EMISSIVE = 2, /* (*) brdf_emissive      */
  ASUNA_MAT_PBR_METALNESS_ROUGHNESS = 3, /* (*) brdf_pbr_metalness_roughness */
  ASUNA_MAT_PLASTIC = 4, /* (*) brdf_plastic       */
  ASUNA_MAT_ROUGH_PLASTIC = 5, /* (*) brdf_rough_plastic */
  ASUNA_MAT_CONDUCTOR = 6, /* (*) brdf_conductor     */
  ASUNA_MAT_ROUGH_CONDUCTOR = 7, /* (*) brdf_rough_conductor */
  ASUNA_MAT_MIRROR = 8, /* (*) brdf_mirror        */
  ASUNA_MAT_DISNEY = 9, /* (*) brdf_disney        */
  ASUNA_MAT_DIELECTRIC = 10, /* (*) bsdf_dielectric    */
  ASUNA_MAT_PHONG = 11, /* (*) brdf_phong         */
  ASUNA_MAT_NUM = 12
};

/* Number of RGBA32F output images of the reference: image 0 = radiance,
 * 1..7 = multi-channel AOVs, 8 = filter-weight sum (src/shared/binding.h:70). */
#define ASUNA_NUM_OUTPUT_IMAGES 9
#define ASUNA_MAX_CHANNELS 7
/* Opacity pass-throughs (brdf_pbr_metalness_roughness / brdf_disney /
 * brdf_kang18: a ray that passes a surface without counting a bounce) a path
 * may take in one render beyond its max_path_depth bounces; a path that needs
 * more ends there.  Only scenes whose materials can pass rays run the extra
 * wavefront passes. */
#define ASUNA_MAX_PASS_THROUGH 24

/* AOV channel kinds; "multi_channel" strings of src/loader/loader.cpp:177-183.
 * ASUNA_CH_DEPTH (primary-hit distance) is an addition of this library. */
enum {
  ASUNA_CH_DIFFUSE = 0, /* "diffuse" (alias "albedo") */
  ASUNA_CH_NORMAL = 1,
  ASUNA_CH_SPECULAR = 2,
  ASUNA_CH_TANGENT = 3,
  ASUNA_CH_ROUGHNESS = 4,
  ASUNA_CH_POSITION = 5,
  ASUNA_CH_UV = 6,
  ASUNA_CH_DEPTH = 7
};

/* ---- device ABI structs (byte-identical to src/shared/) --------------- */

/* GpuVertex, src/shared/vertex.h:6-11 — 44 bytes, scalar layout. */
typedef struct asuna_vertex {
  float pos[3];
  float uv[2];
  float normal[3];
  float tangent[3];
} asuna_vertex;

/* GpuMaterial, src/shared/material.h:24-49 — 132 bytes, scalar layout.
 * For rough plastic, radiance[0] holds fdrInt (src/loader/material.cpp:230). */
typedef struct asuna_material {
  float diffuse[3];
  float rho_spec[3];
  float aniso_alpha[2];
  float ior;
  float roughness;
  float subsurface;
  float specular;
  float specular_tint;
  float anisotropic;
  float sheen;
  float sheen_tint;
  float clearcoat;
  float clearcoat_gloss;
  float radiance[3];
  float metalness;
  float radiance_factor[3];
  int32_t diffuse_texture_id;
  int32_t roughness_texture_id;
  int32_t metalness_texture_id;
  int32_t radiance_texture_id;
  int32_t normal_texture_id;
  int32_t tangent_texture_id;
  int32_t opacity_texture_id;
  uint32_t type;
} asuna_material;

/* GpuLight, src/shared/light.h:16-25 — 76 bytes, scalar layout. */
typedef struct asuna_light {
  int32_t type;
  float position[3];
  float direction[3];
  float radiance[3];
  float u[3];
  float v[3];
  float radius;
  float area;
  uint32_t double_side;
} asuna_light;

/* GpuCamera, src/shared/camera.h:15-24 — 224 bytes, std140 layout. */
typedef struct asuna_camera {
  float raster_to_camera[16];
  float camera_to_world[16];
  float env_transform[16];
  float fxfycxcy[4];
  uint32_t type;
  float aperture;
  float focal_distance;
  float padding;
} asuna_camera;

/* GpuPushConstantRaytrace, src/shared/pushconstant.h:10-34 — 84 bytes. */
typedef struct asuna_rt_state {
  int32_t spp;
  int32_t cur_frame;
  int32_t max_path_depth;
  int32_t num_lights;
  float bg_color[3];
  uint32_t use_face_normal;
  uint32_t ignore_emissive;
  uint32_t has_env_map;
  float env_map_resolution[2];
  float env_map_intensity;
  uint32_t n_multi_channel;
  int32_t diffuse_out_channel;
  int32_t specular_out_channel;
  int32_t roughness_out_channel;
  int32_t normal_out_channel;
  int32_t position_out_channel;
  int32_t tangent_out_channel;
  int32_t uv_out_channel;
} asuna_rt_state;

/* ---- scene description (the reference's device buffers, flattened) ------ */

/* One mesh = one BLAS of the reference (src/core/mesh.cpp:147-192):
 * opaque triangles, uint32 indices, GpuVertex attributes. */
typedef struct asuna_mesh_desc {
  uint32_t num_vertices;
  uint32_t num_triangles;
  const asuna_vertex* vertices; /* num_vertices entries            */
  const uint32_t* indices;      /* 3 * num_triangles entries       */
} asuna_mesh_desc;

/* One TLAS instance (src/core/instance.h:46-68, src/shared/instance.h:7-16).
 * transform: object->world, 3 rows x 4 columns, row-major (the 3x4 of
 * VkTransformMatrixKHR).  light_id >= 0 marks an emitter instance whose hits
 * run the light branch of the Lambertian hit shader; material_id is then unused. */
typedef struct asuna_instance_desc {
  float transform[12];
  uint32_t mesh_id;
  int32_t material_id;
  int32_t light_id;
  uint32_t reserved;
} asuna_instance_desc;

/* Equirectangular environment map (src/core/texture.cpp:144-226).  The
 * inverse-CDF tables are computed by the library from the texels. */
typedef struct asuna_envmap_desc {
  uint32_t width;
  uint32_t height;
  const float* rgba; /* width*height*4 floats, row-major, NULL = none */
} asuna_envmap_desc;

/* A material texture: width x height RGBA32F texels, row 0 first (v = 0),
 * sampled as the reference's texture(): bilinear, REPEAT, base level
 * (src/core/texture.cpp:99-129, rchit_layouts.glsl:169-171). */
typedef struct asuna_texture_desc {
  uint32_t width;
  uint32_t height;
  const float* rgba;
} asuna_texture_desc;

/* GpuSunAndSky, src/shared/sun_and_sky.h:6-27 — 96 bytes, scalar layout:
 * the analytic sun & sky environment (src/shaders/utils/sun_and_sky.glsl).
 * With in_use = 1 it replaces the environment map in the miss shading and
 * the environment light sample (raytrace.default.rmiss:30-31,
 * rchit_layouts.glsl:105-107); asuna_sun_and_sky_default gives the
 * reference's defaults (Scene::reset, src/scene/scene.cpp:112-129). */
typedef struct asuna_sun_and_sky {
  float rgb_unit_conversion[3];
  float multiplier;
  float haze;
  float redblueshift;
  float saturation;
  float horizon_height;
  float ground_color[3];
  float horizon_blur;
  float night_color[3];
  float sun_disk_intensity;
  float sun_direction[3];
  float sun_disk_scale;
  float sun_glow_intensity;
  int32_t y_is_up;
  int32_t physically_scaled_sun;
  int32_t in_use;
} asuna_sun_and_sky;

typedef struct asuna_scene_desc {
  uint32_t num_meshes;
  const asuna_mesh_desc* meshes;
  uint32_t num_instances;
  const asuna_instance_desc* instances;
  uint32_t num_materials;
  const asuna_material* materials;
  uint32_t num_lights; /* lights[0] is the reference's dummy light   */
  const asuna_light* lights;
  asuna_envmap_desc envmap;
  uint32_t num_textures; /* the materials' *_texture_id index this list; */
  const asuna_texture_desc* textures; /* textures[0] is the dummy texture */
  const asuna_sun_and_sky* sun_and_sky; /* NULL = not in use (the reference's default) */
} asuna_scene_desc;

/* ---- shots ----------------------------------------------------------------
 * One shot = one camera pose + pipeline state rendered for `frames` frames of
 * one sample each, exactly the offline loop of src/tracer/tracer.cpp:204-258:
 * frame f hashes (x, y, f) into the pixel seed and frame 0 samples the pixel
 * centre.  frame0 > 0 resumes an existing film.  `seed` is folded into the
 * hashed frame word (seed 0 = the reference's streams). */
enum {
  ASUNA_SHOT_RR = 1u << 0 /* Russian roulette after rr_depth (extension; off = reference) */
};

typedef struct asuna_shot {
  asuna_camera camera;
  asuna_rt_state state; /* state.spp and state.cur_frame are ignored */
  uint32_t width;
  uint32_t height;
  uint32_t frames;
  uint32_t frame0;
  uint32_t seed;
  uint32_t flags;
  uint32_t rr_depth;
  int32_t depth_out_channel; /* AOV slot (0..6) of the depth channel, -1 = none */
} asuna_shot;

/* Per-path record for parity checks (one per (frame, pixel)). */
typedef struct asuna_path_record {
  float radiance[3];   /* path radiance before the [0,10] clamp           */
  float filter_weight; /* Gaussian filter weight of the sample            */
  uint32_t depth;      /* last depth reached (1-based)                    */
  uint32_t signature;  /* hash of hit instance/primitive/lobe sequence    */
  uint32_t events;     /* bit d: shadow ray at depth d+1 was unoccluded   */
  uint32_t shadows;    /* bit d: a shadow ray was traced at depth d+1      */
} asuna_path_record;

/* Counters of one render call (device-side, exact). */
typedef struct asuna_render_stats {
  uint64_t paths;          /* camera rays = samples                         */
  uint64_t extend_rays;    /* closest-hit rays (camera + continuation)      */
  uint64_t shadow_rays;    /* occlusion rays                                */
  uint64_t nodes_visited;  /* closest-hit BVH nodes (traversal counters on)  */
  uint64_t tris_tested;    /* closest-hit triangle tests (counters on)      */
  uint64_t shadow_nodes_visited; /* occlusion BVH nodes (counters on)       */
  uint64_t shadow_tris_tested;   /* occlusion triangle tests (counters on)  */
  double ms_total;         /* device time of the call (CUDA events)         */
  double ms_extend;        /* device time of closest-hit traversal kernels  */
  double ms_connect;       /* device time of occlusion traversal kernels    */
  double ms_shade;         /* device time of shading kernels                */
  uint64_t extend_launches;
  uint64_t connect_launches;
  uint64_t kernel_launches; /* every kernel the call launched (all waves)   */
  double ms_sort;          /* device time of extend-queue sorting           */
} asuna_render_stats;

typedef struct asuna_scene_stats {
  uint64_t triangles;
  uint64_t instances;
  uint64_t blas_nodes;
  uint64_t tlas_nodes;
  uint64_t device_bytes;
  double build_ms;
} asuna_scene_stats;

typedef struct asuna_ctx asuna_ctx;
typedef struct asuna_scene asuna_scene;
typedef struct asuna_film asuna_film;
typedef struct asuna_json_scene asuna_json_scene;

/* ---- library ------------------------------------------------------------- */
int asuna_abi_version(void);
const char* asuna_last_error(void);

/* ---- context: one CUDA device + one stream ------------------------------- */
/* Replaces ContextAware::init (src/context/context.cpp:8-27); the context is
 * bound to one CUDA stream; calls on one context are serialised on it. */
int asuna_ctx_create(int device_ordinal, asuna_ctx** out);
int asuna_ctx_destroy(asuna_ctx* ctx);
int asuna_ctx_sync(asuna_ctx* ctx);
/* The cudaStream_t the context launches on (for interop), as void*. */
void* asuna_ctx_stream(asuna_ctx* ctx);
/* Traversal counters (nodes/triangles) for the next renders: 0 off, 1 on.
 * Counting adds global atomics; keep it off when timing. */
int asuna_ctx_set_counters(asuna_ctx* ctx, int enable);
/* Device memory budget for wavefront path state, in bytes (0 = default):
 * sets how many paths (frames x pixels) one wavefront carries. */
int asuna_ctx_set_path_budget(asuna_ctx* ctx, uint64_t bytes);
/* Capture each render's launch sequence as a CUDA graph and replay it while
 * the scene, buffers and batch structure repeat (1 = on, the default). */
int asuna_ctx_set_graphs(asuna_ctx* ctx, int enable);
/* Persistent-grid sizes in resident blocks per SM of the traversal and
 * shading kernels (0 = default, capped at the occupancy limit). */
int asuna_ctx_set_launch(asuna_ctx* ctx, int trace_blocks_per_sm, int shade_blocks_per_sm);
/* Traversal settings of the closest-hit (extend) and occlusion (shadow)
 * passes: idle lanes of a warp that trigger a refill from the ray queue
 * (1..32, 0 = default 8), speculative walking past a postponed leaf (1 on,
 * 0 off, -1 default on) and the kernel variant's resident blocks per SM
 * (8, 10 or 12 — fewer registers, more warps; 0 = default 8).  Results do
 * not depend on them. */
int asuna_ctx_set_traversal(asuna_ctx* ctx, int refill_extend, int refill_shadow, int speculate_extend,
                            int speculate_shadow, int blocks_per_sm);
/* Shape of the traversal kernel variant: threads per block (64, 128 or 256)
 * and traversal-stack entries kept in shared memory (16, 24 or 32; the rest
 * of the 64 in thread-local memory); 0 = 128 / 24.  Results do not depend
 * on them. */
int asuna_ctx_set_traversal_shape(asuna_ctx* ctx, int threads_per_block, int shared_stack_entries);
/* The traversal kernel variant's resident blocks per SM of the closest-hit
 * (extend) and occlusion (shadow) passes separately (8, 10 or 12; 0 = 8);
 * asuna_ctx_set_traversal sets both to its value.  Results do not depend on
 * them. */
int asuna_ctx_set_traversal_occupancy(asuna_ctx* ctx, int extend_blocks_per_sm, int shadow_blocks_per_sm);
/* Reorders the extend queue before every secondary pass by direction and
 * origin so warps carry rays that walk alike: 0 off, 1 octant x 4 x 4 x 4
 * origin cells, 2 octant x 8 x 8 x 8 cells in Morton order, 3 the same with
 * the origin cell major (the default).  Results do not depend on it. */
int asuna_ctx_set_ray_sort(asuna_ctx* ctx, int mode);
/* Caps the traversal stack at `entries` per ray (1..64; 0 = 64, the
 * compiled capacity, which every scene asuna_scene_create accepts fits).
 * A traversal that needs more entries is cut short and the render reports
 * ASUNA_ERR_TRAVERSAL; a lower cap serves to test that error path. */
int asuna_ctx_set_traversal_stack(asuna_ctx* ctx, int entries);
/* Where asuna_scene_create builds the bottom-level BVHs: 0 on the device
 * (the default), 1 on host threads.  Both run the same binned-SAH
 * algorithm; rendered results do not depend on the choice (leaf order and
 * node numbering may differ, hits do not). */
int asuna_ctx_set_bvh_build(asuna_ctx* ctx, int mode);

/* ---- scene: upload + acceleration-structure build ------------------------ */
/* Replaces Scene::submit + BLAS/TLAS build.  Host arrays are deep-copied; the
 * scene is immutable afterwards and may be shared by renders on any context
 * of the same device. */
int asuna_scene_create(asuna_ctx* ctx, const asuna_scene_desc* desc, asuna_scene** out);
/* The reference's sun & sky defaults (Scene::reset, scene.cpp:112-129; in_use 0). */
void asuna_sun_and_sky_default(asuna_sun_and_sky* out);
int asuna_scene_destroy(asuna_scene* scene);
int asuna_scene_get_stats(const asuna_scene* scene, asuna_scene_stats* out);
/* The checks asuna_scene_create runs before any upload (indices in range,
 * implemented material types and features, lights), on the host alone. */
int asuna_scene_validate(const asuna_scene_desc* desc);

/* ---- film: the 9 RGBA32F output images ---------------------------------- */
int asuna_film_create(asuna_ctx* ctx, uint32_t width, uint32_t height, asuna_film** out);
int asuna_film_destroy(asuna_film* film);
/* image: 0 radiance, 1..7 AOV channels, 8 filter-weight sum.  Copies
 * width*height*4 floats into host memory (pinned or pageable). */
int asuna_film_read(asuna_ctx* ctx, asuna_film* film, int image, float* host_rgba);
/* Device address of film image `image` (0..8; width x height RGBA32F,
 * valid while the film lives) for zero-copy use on the context's stream. */
int asuna_film_image(asuna_film* film, int image, float** device_rgba);
int asuna_film_clear(asuna_ctx* ctx, asuna_film* film);

/* ---- render --------------------------------------------------------------- */
/* Renders shot->frames frames into film (asynchronous on the context's
 * stream; stats, if non-NULL, forces a synchronisation and is filled).
 * A traversal cut short on the device (ASUNA_ERR_TRAVERSAL) is reported by
 * the call itself when it synchronises (stats or records requested), else
 * by the next call on the context that waits for the stream:
 * asuna_ctx_sync, asuna_film_read, or a render with stats. */
int asuna_render(asuna_ctx* ctx, const asuna_scene* scene, const asuna_shot* shot,
                 asuna_film* film, asuna_render_stats* stats);
/* Renders n shots (any resolutions / frame counts) in one wavefront. */
int asuna_render_batch(asuna_ctx* ctx, const asuna_scene* scene, const asuna_shot* shots,
                       asuna_film* const* films, uint32_t n, asuna_render_stats* stats);
/* Parity mode: renders one shot and writes one asuna_path_record per
 * (frame, pixel) into host memory, ordered [frame][y][x]. */
int asuna_render_paths(asuna_ctx* ctx, const asuna_scene* scene, const asuna_shot* shot,
                       asuna_film* film, asuna_path_record* host_records);

/* Traversal query (tests, tools): n rays of 8 floats (o.xyz, tmin, d.xyz,
 * tmax); hits receive (t, u, v, primitive bits) or t = -1 on a miss, inst the
 * instance index or 0xffffffff.  any_hit = 1 gives occlusion only. */
int asuna_scene_trace(asuna_ctx* ctx, const asuna_scene* scene, const float* rays, uint32_t n, int any_hit,
                      float* hits, uint32_t* inst);

/* ---- allocation-free render ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they render (an owner holds the memory pool or budget, a
 * fixed footprint was granted up front, or a render thread must stay out of
 * the allocator): renders shot->frames frames of one shot into `film` like
 * asuna_render, on `stream` (a cudaStream_t; NULL = default stream), with
 * all scratch in one fixed device array compiled into the library.  The
 * array holds ASUNA_NOALLOC_MAX_PATHS path slots (about 61 MiB, kept by
 * every GPU that loads the library until exit); a frame with more pixels is
 * rejected with ASUNA_ERR_INVALID.  The array's address is set up on a
 * device by the first call there: make that call before any stream capture.
 * Calls share the array; calls that overlap on the GPU race.  The call
 * waits for its work on `stream` to finish and returns ASUNA_ERR_TRAVERSAL
 * if a traversal was cut short; on a stream that is being captured it
 * queues nothing and returns ASUNA_ERR_UNSUPPORTED. */
#define ASUNA_NOALLOC_MAX_PATHS 262144
int asuna_render_noalloc(const asuna_scene* scene, const asuna_shot* shot, asuna_film* film, void* stream);

/* ---- host side: JSON scene description ---------------------------------- */
/* Parses an Asuna scene JSON file (Loader::parse, src/loader/loader.cpp:91-144)
 * and assembles the device-ABI arrays the way Scene does (dummy light 0,
 * dummy material 0, rect lights as two-triangle emitter instances, mesh
 * lights as one triangle light per facet). */
int asuna_json_load(const char* path, asuna_json_scene** out);
int asuna_json_load_string(const char* text, const char* base_dir, asuna_json_scene** out);
int asuna_json_free(asuna_json_scene* js);
/* View of the assembled arrays; valid until asuna_json_free. */
int asuna_json_scene_desc(const asuna_json_scene* js, asuna_scene_desc* out);
/* Number of shots (autofit adds one when the file has none). */
int asuna_json_num_shots(const asuna_json_scene* js, uint32_t* out);
int asuna_json_get_shot(const asuna_json_scene* js, uint32_t index, asuna_shot* out);
/* Channel kinds of the scene's multi_channel list (ASUNA_CH_*), count in *n. */
int asuna_json_channels(const asuna_json_scene* js, uint32_t* n, int32_t* kinds);
struct asuna_post_state;
/* The post-pass state of the scene file ("post_processing.tone_mapping"). */
int asuna_json_post_state(const asuna_json_scene* js, struct asuna_post_state* out);

/* ---- host side: camera helpers (src/core/camera.cpp:28-99) ---------------- */
/* Fills a perspective GpuCamera from look-at parameters; fov in degrees is
 * the horizontal field of view of the reference. */
int asuna_camera_perspective(const float eye[3], const float lookat[3], const float up[3],
                             float fov_deg, float aperture, float focal_distance,
                             uint32_t width, uint32_t height, asuna_camera* out);
int asuna_camera_opencv(const float eye[3], const float lookat[3], const float up[3],
                        const float fxfycxcy[4], asuna_camera* out);
/* Builds the env-map importance tables exactly as EnvMap::EnvMap
 * (src/core/texture.cpp:144-226): marginal/conditional are width*height*2
 * floats (.x = inverse CDF, .y = pdf). */
int asuna_envmap_tables(uint32_t width, uint32_t height, const float* rgba, float* marginal_xy,
                        float* conditional_xy);
/* Diffuse Fresnel reflectance fdrInt (src/loader/material.cpp:25-37). */
float asuna_diffuse_fresnel(float ior, int sample_count);
/* Complex index of refraction (eta, k at R, G, B) of a named conductor, as
 * brdf_conductor / brdf_rough_conductor select it (complexIorListLookup,
 * src/loader/material.cpp:290-300); ASUNA_ERR_PARSE for an unknown name. */
int asuna_complex_ior(const char* name, float* eta, float* k);

/* ---- render server (continuous batching) -------------------------------------
 * No counterpart in the reference (an addition for serving).  Requests on
 * the server's scenes arrive at any time; `slots` worker contexts render
 * them concurrently on the device, each slot batching the active requests of
 * one scene into one multi-shot wavefront per chunk of frames, with requests
 * leaving and joining at chunk boundaries.  Admission is by memory
 * footprint under the budget: a request is admitted when its result films
 * fit (else it waits), and the pending queue must have room (else it is
 * rejected with ASUNA_ERR_BUSY, reported by poll).  A scene registered with
 * asuna_server_register_scene is built on the device when its first request
 * is admitted, charged to the budget, and dropped again (least recently used
 * first) when an admission needs the memory and no request uses it. */
typedef struct asuna_server asuna_server;
typedef struct asuna_server_opts {
  int32_t device;
  uint32_t slots;            /* concurrent worker slots (each a context + stream) */
  uint32_t frames_per_chunk; /* frames per wavefront pass of an active set */
  uint32_t max_batch;        /* requests per active set (0 = 8) */
  uint32_t max_queue;        /* pending requests before arrivals are rejected (0 = unbounded) */
  uint32_t reserved;
  uint64_t memory_budget;    /* bytes for scenes + result films (0 = 150 GiB) */
  uint64_t path_budget;      /* wavefront state per slot, bytes (0 = default) */
} asuna_server_opts;
enum {
  /* the result's image 0 is the denoised radiance: the request renders two
   * halves of its frames into two films and asuna_denoise_blended combines
   * them (needs asuna_server_set_denoiser and albedo + normal channels) */
  ASUNA_REQUEST_DENOISE = 1u << 0
};
typedef struct asuna_request {
  uint32_t scene; /* id from asuna_server_add_scene / _register_scene */
  uint32_t flags; /* ASUNA_REQUEST_* */
  asuna_shot shot; /* shot.frames = spp */
} asuna_request;
typedef struct asuna_request_result {
  uint64_t id;
  int32_t status; /* ASUNA_OK, or why the request was rejected / failed */
  uint32_t scene;
  double arrival_s, start_s, finish_s; /* server clock */
  uint64_t samples;
} asuna_request_result;
typedef struct asuna_server_stats {
  uint64_t admitted, rejected, pending, samples, memory_used;
  double elapsed_s;
  uint64_t scenes_built;    /* device builds of registered scenes (admission time) */
  uint64_t scenes_evicted;  /* registered scenes dropped to make room */
  uint64_t denoised;        /* requests finished through the denoiser */
  uint64_t scene_bytes;     /* device bytes of the scenes resident now */
} asuna_server_stats;
int asuna_server_create(const asuna_server_opts* opts, asuna_server** out);
/* Builds the scene now; it stays resident for the server's lifetime. */
int asuna_server_add_scene(asuna_server* server, const asuna_scene_desc* desc, uint32_t* scene_id);
/* Registers a scene built on demand (see above).  The description's arrays
 * must stay valid until the server is destroyed. */
int asuna_server_register_scene(asuna_server* server, const asuna_scene_desc* desc, uint32_t* scene_id);
/* One denoiser per slot with `opts`' network and the trained parameters
 * `params` (n floats, asuna_denoiser_get_params); opts->max_pixels bounds
 * the padded size of a denoised request. */
struct asuna_denoiser_opts;
int asuna_server_set_denoiser(asuna_server* server, const struct asuna_denoiser_opts* opts, const float* params,
                              uint64_t n);
int asuna_server_submit(asuna_server* server, const asuna_request* req, uint64_t* id);
/* Finished (or rejected) requests since the last poll, oldest first. */
int asuna_server_poll(asuna_server* server, asuna_request_result* out, uint32_t max, uint32_t* n);
/* Film image `image` of a finished request (image 0 of a denoised request:
 * the denoised radiance).  Safe to call from any thread; a release of the
 * same request waits for the read, and a read after it fails with
 * ASUNA_ERR_INVALID (unknown request). */
int asuna_server_read(asuna_server* server, uint64_t id, int image, float* host_rgba);
/* Frees a finished request's film (returns its memory to the budget). */
int asuna_server_release(asuna_server* server, uint64_t id);
int asuna_server_drain(asuna_server* server, double timeout_s);
int asuna_server_get_stats(asuna_server* server, asuna_server_stats* out);
int asuna_server_destroy(asuna_server* server);

/* ---- image files ----------------------------------------------------------- */
/* RGBA32F images: .exr (uncompressed FLOAT scanlines), .png (8-bit, clamped,
 * gamma 1), .pfm.  Readers: .hdr (Radiance RGBE, env maps) and .pfm; with
 * rgba NULL only the size is returned; capacity counts floats. */
int asuna_image_write(const char* path, uint32_t width, uint32_t height, const float* rgba);
int asuna_image_read(const char* path, uint32_t* width, uint32_t* height, float* rgba, uint64_t capacity);

/* ---- post pass: tone mapping --------------------------------------------------
 * GpuPushConstantPost (src/shared/pushconstant.h:50-62) and the operators of
 * ToneMappingType (:37-46) as src/shaders/post.idle.frag:71-133 applies them. */
enum {
  ASUNA_TONEMAP_NONE = 0,
  ASUNA_TONEMAP_GAMMA = 1,
  ASUNA_TONEMAP_REINHARD = 2,
  ASUNA_TONEMAP_ACES = 3,
  ASUNA_TONEMAP_FILMIC = 4,
  ASUNA_TONEMAP_PBRT = 5,
  ASUNA_TONEMAP_CUSTOM = 6,
  ASUNA_TONEMAP_NUM = 7
};
typedef struct asuna_post_state {
  float brightness, contrast, saturation, vignette;
  float avg_lum, zoom;
  float rendering_ratio[2];
  int32_t auto_exposure; /* bit 0: exposure from the mean luminance, bit 1: local */
  float y_white, key;
  uint32_t tm_type;      /* ASUNA_TONEMAP_* */
} asuna_post_state;
/* The defaults of PipelineState (src/core/state.h:46-58): filmic. */
void asuna_post_default(asuna_post_state* post);
/* Tone-maps film image `image` into `out` (device, width*height RGBA32F):
 * the LDR color of the offline output before its 8-bit conversion. */
int asuna_tonemap(asuna_ctx* ctx, asuna_film* film, int image, const asuna_post_state* post, float* out);

/* ---- offline tracer ------------------------------------------------------- */
/* Renders every shot of a scene file and writes <out_prefix>_shot_%04d.exr
 * (output_hdr) or the tone-mapped _shot_%04d.png, + _channel_%04d.exr/.png
 * per AOV: the offline mode of Tracer::runOffline. */
int asuna_tracer_run_offline(asuna_ctx* ctx, const char* scene_json, const char* out_prefix);
/* The same with the CLI's --output_scanline (src/main.cpp:21,
 * tracer.cpp:347-395): each AOV channel is written as a [n, 3] float32 NumPy
 * array of the pixels whose channel-0 .z is 1 (a hit, for the uv channel),
 * with that channel's .z replaced by the pixel index; the file keeps its
 * _channel_%04d.exr / .png name, as the reference's does. */
int asuna_tracer_run_offline_scanline(asuna_ctx* ctx, const char* scene_json, const char* out_prefix,
                                      int output_scanline);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* ASUNA_RT_H */
