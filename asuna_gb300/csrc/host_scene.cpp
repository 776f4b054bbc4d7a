// host_scene.cpp — the host side of the render path: scene-file loader,
// scene assembly, camera matrices, env-map importance tables, file IO and
// the library's error plumbing.
//
// Follows (file:line of the reference):
//   HostState defaults      src/core/state.h:15-63
//   HostScene::reset        src/scene/scene.cpp:87-130 (dummy texture,
//                           material and light 0)
//   HostScene::addLight     src/scene/scene.cpp:220-283 (rect lights become
//                           two-triangle emitter instances, mesh lights one
//                           triangle light + instance per facet)
//   HostScene::submit       src/scene/scene.cpp:26-85 (numLights = lights - 1)
//   loadSceneJson           src/loader/loader.cpp:91-468,
//                           src/loader/material.cpp:54-231
//   camera matrices         src/core/camera.cpp:28-99, src/core/camera.h:124-126
//   env tables              src/core/texture.cpp:144-226
//   fdrInt                  src/loader/material.cpp:6-37
//   OBJ de-indexing         src/core/mesh.cpp:112-145
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include <cuda_runtime.h>
#include <fstream>
#include <sstream>

#include "common.h"
#include "json.h"

namespace asuna {

// ---- errors -------------------------------------------------------------------
static thread_local std::string gLastError;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  gLastError = buf;
  return code;
}
void clearError() { gLastError.clear(); }

// ---- scene validation ---------------------------------------------------------
int validateSceneDesc(const asuna_scene_desc* d) {
  if (d->num_meshes && !d->meshes) return fail(ASUNA_ERR_INVALID, "meshes is NULL");
  if (d->num_instances && !d->instances) return fail(ASUNA_ERR_INVALID, "instances is NULL");
  if (d->num_materials && !d->materials) return fail(ASUNA_ERR_INVALID, "materials is NULL");
  if (d->num_lights && !d->lights) return fail(ASUNA_ERR_INVALID, "lights is NULL");
  for (uint32_t m = 0; m < d->num_meshes; ++m) {
    const asuna_mesh_desc& md = d->meshes[m];
    if (md.num_triangles && (!md.indices || !md.vertices))
      return fail(ASUNA_ERR_INVALID, "mesh %u: NULL vertex or index array", m);
    for (uint64_t i = 0; i < uint64_t(md.num_triangles) * 3; ++i)
      if (md.indices[i] >= md.num_vertices)
        return fail(ASUNA_ERR_INVALID, "mesh %u: index %u out of range (%u vertices)", m, md.indices[i],
                    md.num_vertices);
  }
  for (uint32_t i = 0; i < d->num_materials; ++i) {
    uint32_t t = d->materials[i].type;
    if (t != ASUNA_MAT_LAMBERTIAN && t != ASUNA_MAT_ROUGH_PLASTIC && t != ASUNA_MAT_DIELECTRIC &&
        t != ASUNA_MAT_EMISSIVE && t != ASUNA_MAT_PLASTIC && t != ASUNA_MAT_MIRROR && t != ASUNA_MAT_CONDUCTOR &&
        t != ASUNA_MAT_ROUGH_CONDUCTOR && t != ASUNA_MAT_PHONG && t != ASUNA_MAT_PBR_METALNESS_ROUGHNESS &&
        t != ASUNA_MAT_DISNEY && t != ASUNA_MAT_KANG18)
      return fail(ASUNA_ERR_UNSUPPORTED, "material %u: type %u is not implemented", i, t);
    const asuna_material& m = d->materials[i];
    const int32_t ids[7] = {m.diffuse_texture_id,  m.roughness_texture_id, m.metalness_texture_id,
                            m.radiance_texture_id, m.normal_texture_id,    m.tangent_texture_id,
                            m.opacity_texture_id};
    for (int32_t id : ids)
      if (id >= int32_t(d->num_textures))
        return fail(ASUNA_ERR_INVALID, "material %u: texture %d out of range (%u textures)", i, id, d->num_textures);
  }
  for (uint32_t i = 0; i < d->num_instances; ++i) {
    const asuna_instance_desc& in = d->instances[i];
    if (in.mesh_id >= d->num_meshes) return fail(ASUNA_ERR_INVALID, "instance %u: mesh %u out of range", i, in.mesh_id);
    if (in.light_id >= 0) {
      if (uint32_t(in.light_id) >= d->num_lights)
        return fail(ASUNA_ERR_INVALID, "instance %u: light %d out of range", i, in.light_id);
    } else if (in.material_id < 0 || uint32_t(in.material_id) >= d->num_materials) {
      return fail(ASUNA_ERR_INVALID, "instance %u: material %d out of range", i, in.material_id);
    }
  }
  for (uint32_t i = 0; i < d->num_lights; ++i)
    if (d->lights[i].type < 0 || d->lights[i].type > ASUNA_LIGHT_POINT)
      return fail(ASUNA_ERR_UNSUPPORTED, "light %u: type %d", i, d->lights[i].type);
  if (d->envmap.rgba && (!d->envmap.width || !d->envmap.height))
    return fail(ASUNA_ERR_INVALID, "envmap has zero size");
  if (d->num_textures && !d->textures) return fail(ASUNA_ERR_INVALID, "textures is NULL");
  uint64_t texels = 0;
  for (uint32_t i = 0; i < d->num_textures; ++i) {
    const asuna_texture_desc& t = d->textures[i];
    if (!t.rgba || !t.width || !t.height || t.width > 65536 || t.height > 65536)
      return fail(ASUNA_ERR_INVALID, "texture %u: bad size %u x %u or no texels", i, t.width, t.height);
    texels += uint64_t(t.width) * t.height;
  }
  if (texels >= (1ull << 32)) return fail(ASUNA_ERR_INVALID, "textures hold %llu texels (limit 2^32)",
                                          (unsigned long long)texels);
  return ASUNA_OK;
}

void invert3x4(const float* m, float* out) {
  double a[3][3], t[3];
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) a[r][c] = m[r * 4 + c];
    t[r] = m[r * 4 + 3];
  }
  double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
               a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
  double inv[3][3];
  inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
  inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
  inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
  inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
  inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
  inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
  inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
  inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
  inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
  for (int r = 0; r < 3; ++r) {
    double tt = -(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]);
    for (int c = 0; c < 3; ++c) out[r * 4 + c] = float(inv[r][c]);
    out[r * 4 + 3] = float(tt);
  }
}

// ---- 4x4 helpers (row-major double here; stored column-major in GpuCamera) ----
namespace {
struct M4 {
  double m[4][4];
  static M4 id() {
    M4 r{};
    for (int i = 0; i < 4; ++i) r.m[i][i] = 1;
    return r;
  }
  M4 operator*(const M4& b) const {
    M4 r{};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k) r.m[i][j] += m[i][k] * b.m[k][j];
    return r;
  }
};
bool invert4(const M4& a, M4& out) {
  double inv[16], s[16];
  for (int i = 0; i < 16; ++i) s[i] = a.m[i / 4][i % 4];
  inv[0] = s[5] * s[10] * s[15] - s[5] * s[11] * s[14] - s[9] * s[6] * s[15] + s[9] * s[7] * s[14] + s[13] * s[6] * s[11] - s[13] * s[7] * s[10];
  inv[4] = -s[4] * s[10] * s[15] + s[4] * s[11] * s[14] + s[8] * s[6] * s[15] - s[8] * s[7] * s[14] - s[12] * s[6] * s[11] + s[12] * s[7] * s[10];
  inv[8] = s[4] * s[9] * s[15] - s[4] * s[11] * s[13] - s[8] * s[5] * s[15] + s[8] * s[7] * s[13] + s[12] * s[5] * s[11] - s[12] * s[7] * s[9];
  inv[12] = -s[4] * s[9] * s[14] + s[4] * s[10] * s[13] + s[8] * s[5] * s[14] - s[8] * s[6] * s[13] - s[12] * s[5] * s[10] + s[12] * s[6] * s[9];
  inv[1] = -s[1] * s[10] * s[15] + s[1] * s[11] * s[14] + s[9] * s[2] * s[15] - s[9] * s[3] * s[14] - s[13] * s[2] * s[11] + s[13] * s[3] * s[10];
  inv[5] = s[0] * s[10] * s[15] - s[0] * s[11] * s[14] - s[8] * s[2] * s[15] + s[8] * s[3] * s[14] + s[12] * s[2] * s[11] - s[12] * s[3] * s[10];
  inv[9] = -s[0] * s[9] * s[15] + s[0] * s[11] * s[13] + s[8] * s[1] * s[15] - s[8] * s[3] * s[13] - s[12] * s[1] * s[11] + s[12] * s[3] * s[9];
  inv[13] = s[0] * s[9] * s[14] - s[0] * s[10] * s[13] - s[8] * s[1] * s[14] + s[8] * s[2] * s[13] + s[12] * s[1] * s[10] - s[12] * s[2] * s[9];
  inv[2] = s[1] * s[6] * s[15] - s[1] * s[7] * s[14] - s[5] * s[2] * s[15] + s[5] * s[3] * s[14] + s[13] * s[2] * s[7] - s[13] * s[3] * s[6];
  inv[6] = -s[0] * s[6] * s[15] + s[0] * s[7] * s[14] + s[4] * s[2] * s[15] - s[4] * s[3] * s[14] - s[12] * s[2] * s[7] + s[12] * s[3] * s[6];
  inv[10] = s[0] * s[5] * s[15] - s[0] * s[7] * s[13] - s[4] * s[1] * s[15] + s[4] * s[3] * s[13] + s[12] * s[1] * s[7] - s[12] * s[3] * s[5];
  inv[14] = -s[0] * s[5] * s[14] + s[0] * s[6] * s[13] + s[4] * s[1] * s[14] - s[4] * s[2] * s[13] - s[12] * s[1] * s[6] + s[12] * s[2] * s[5];
  inv[3] = -s[1] * s[6] * s[11] + s[1] * s[7] * s[10] + s[5] * s[2] * s[11] - s[5] * s[3] * s[10] - s[9] * s[2] * s[7] + s[9] * s[3] * s[6];
  inv[7] = s[0] * s[6] * s[11] - s[0] * s[7] * s[10] - s[4] * s[2] * s[11] + s[4] * s[3] * s[10] + s[8] * s[2] * s[7] - s[8] * s[3] * s[6];
  inv[11] = -s[0] * s[5] * s[11] + s[0] * s[7] * s[9] + s[4] * s[1] * s[11] - s[4] * s[3] * s[9] - s[8] * s[1] * s[7] + s[8] * s[3] * s[5];
  inv[15] = s[0] * s[5] * s[10] - s[0] * s[6] * s[9] - s[4] * s[1] * s[10] + s[4] * s[2] * s[9] + s[8] * s[1] * s[6] - s[8] * s[2] * s[5];
  double det = s[0] * inv[0] + s[1] * inv[4] + s[2] * inv[8] + s[3] * inv[12];
  if (det == 0) return false;
  for (int i = 0; i < 16; ++i) out.m[i / 4][i % 4] = inv[i] / det;
  return true;
}
void storeColMajor(const M4& a, float* dst) {
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) dst[c * 4 + r] = float(a.m[r][c]);
}
M4 fromRowMajor16(const float* v) {
  M4 r{};
  for (int i = 0; i < 16; ++i) r.m[i / 4][i % 4] = v[i];
  return r;
}
void norm3(double v[3]) {
  double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (l > 0)
    for (int k = 0; k < 3; ++k) v[k] /= l;
}
void cross3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
// camera -> world of the reference's view = scale(1,-1,-1) * lookAt(eye, at, up)
// (src/core/camera.h:124-126): columns x, -y, -z, eye of the look-at frame.
M4 cameraToWorld(const float eye[3], const float at[3], const float up[3]) {
  double z[3] = {double(eye[0]) - at[0], double(eye[1]) - at[1], double(eye[2]) - at[2]};
  norm3(z);
  double u[3] = {up[0], up[1], up[2]}, x[3], y[3];
  cross3(u, z, x);
  norm3(x);
  cross3(z, x, y);
  norm3(y);
  M4 c = M4::id();
  for (int k = 0; k < 3; ++k) {
    c.m[k][0] = x[k];
    c.m[k][1] = -y[k];
    c.m[k][2] = -z[k];
    c.m[k][3] = eye[k];
  }
  return c;
}
// src/core/camera.cpp:28-62
M4 cameraToRaster(uint32_t w, uint32_t h, float fov, float nearz, float farz) {
  float aspect = float(w) / float(h);
  M4 persp{};
  float recip = 1.0f / (farz - nearz);
  float ctot = float(1.0 / double(tanf(fov * 0.017453292519943295f * 0.5f)));
  persp.m[0][0] = ctot;
  persp.m[1][1] = ctot;
  persp.m[2][2] = farz * recip;
  persp.m[2][3] = -nearz * farz * recip;
  persp.m[3][2] = 1;
  M4 s1 = M4::id();
  s1.m[1][1] = aspect;
  M4 t1 = M4::id();
  t1.m[0][3] = 1;
  t1.m[1][3] = 1;
  M4 s2 = M4::id();
  s2.m[0][0] = 0.5;
  s2.m[1][1] = 0.5;
  M4 s3 = M4::id();
  s3.m[0][0] = w;
  s3.m[1][1] = h;
  return s3 * (s2 * (t1 * (s1 * persp)));
}
}  // namespace

// ---- state / scene assembly -------------------------------------------------------
HostState::HostState() {
  std::memset(&rtx, 0, sizeof(rtx));
  rtx.cur_frame = -1;
  rtx.spp = 1;
  rtx.max_path_depth = 3;
  rtx.env_map_intensity = 1.0f;
  rtx.diffuse_out_channel = rtx.specular_out_channel = rtx.roughness_out_channel = -1;
  rtx.normal_out_channel = rtx.position_out_channel = rtx.tangent_out_channel = rtx.uv_out_channel = -1;
}

static asuna_material defaultMaterial() {
  // Material() of src/core/material.h:9-35
  asuna_material m;
  std::memset(&m, 0, sizeof(m));
  m.ior = 1.5f;
  m.roughness = 0.5f;
  for (int k = 0; k < 3; ++k) m.radiance_factor[k] = 1.0f;
  m.diffuse_texture_id = m.radiance_texture_id = m.metalness_texture_id = m.normal_texture_id = -1;
  m.roughness_texture_id = m.tangent_texture_id = m.opacity_texture_id = -1;
  m.type = ASUNA_MAT_LAMBERTIAN;
  return m;
}

void HostScene::reset() {
  *this = HostScene();
  // src/scene/scene.cpp:87-130: a 1 x 1 dummy texture (its texels are left
  // unset there; zero here)
  textureNames.push_back("add_by_default_dummy_texture");
  textures.push_back(Texture{1, 1, std::vector<float>(4, 0.0f)});
  materialNames.push_back("add_by_default_dummy_material");
  materials.push_back(defaultMaterial());
  asuna_light d;
  std::memset(&d, 0, sizeof(d));
  d.type = ASUNA_LIGHT_DIRECTIONAL;
  d.double_side = 1;
  addLight(d);
}

static void identity3x4(float* t) {
  std::memset(t, 0, 12 * sizeof(float));
  t[0] = t[5] = t[10] = 1.0f;
}

int HostScene::addLight(const asuna_light& l) {
  const int lightId = int(lights.size());
  if (l.type == ASUNA_LIGHT_RECT) {
    // src/core/mesh.cpp:18-33: 0=p, 1=p+u, 2=p+u+v, 3=p+v; indices 0,1,2,0,2,3
    HostMesh m;
    m.name = "__rectLight:" + std::to_string(lightId);
    m.v.assign(4, asuna_vertex{});
    for (int k = 0; k < 3; ++k) {
      m.v[0].pos[k] = l.position[k];
      m.v[1].pos[k] = l.position[k] + l.u[k];
      m.v[2].pos[k] = l.position[k] + l.u[k] + l.v[k];
      m.v[3].pos[k] = l.position[k] + l.v[k];
    }
    m.idx = {0, 1, 2, 0, 2, 3};
    asuna_instance_desc in{};
    identity3x4(in.transform);
    in.mesh_id = uint32_t(meshes.size());
    in.material_id = 0;
    in.light_id = lightId;
    meshes.push_back(std::move(m));
    instances.push_back(in);
  }
  lights.push_back(l);
  return ASUNA_OK;
}

int HostScene::addMeshLight(const asuna_light& l, const std::vector<asuna_vertex>& v,
                            const std::vector<uint32_t>& idx) {
  for (size_t i = 0; i + 2 < idx.size(); i += 3) {
    const asuna_vertex &a = v[idx[i]], &b = v[idx[i + 1]], &c = v[idx[i + 2]];
    asuna_light t = l;
    t.type = ASUNA_LIGHT_TRIANGLE;
    for (int k = 0; k < 3; ++k) {
      t.position[k] = a.pos[k];
      t.u[k] = b.pos[k] - a.pos[k];
      t.v[k] = c.pos[k] - a.pos[k];
    }
    float cx = t.u[1] * t.v[2] - t.u[2] * t.v[1], cy = t.u[2] * t.v[0] - t.u[0] * t.v[2],
          cz = t.u[0] * t.v[1] - t.u[1] * t.v[0];
    t.area = std::sqrt(cx * cx + cy * cy + cz * cz) * 0.5f;
    t.double_side = 0;
    const int lightId = int(lights.size());
    HostMesh m;
    m.name = "__meshLight:" + std::to_string(lightId);
    m.v.assign(3, asuna_vertex{});
    for (int k = 0; k < 3; ++k) {
      m.v[0].pos[k] = t.position[k];
      m.v[1].pos[k] = t.position[k] + t.u[k];
      m.v[2].pos[k] = t.position[k] + t.v[k];
    }
    m.idx = {0, 1, 2};
    asuna_instance_desc in{};
    identity3x4(in.transform);
    in.mesh_id = uint32_t(meshes.size());
    in.material_id = 0;
    in.light_id = lightId;
    meshes.push_back(std::move(m));
    instances.push_back(in);
    lights.push_back(t);
  }
  return ASUNA_OK;
}

int HostScene::materialId(const std::string& name) const {
  for (size_t i = 0; i < materialNames.size(); ++i)
    if (materialNames[i] == name) return int(i);
  return -1;
}
int HostScene::meshId(const std::string& name) const {
  for (size_t i = 0; i < meshes.size(); ++i)
    if (meshes[i].name == name) return int(i);
  return -1;
}

void HostScene::submit() {
  state.rtx.num_lights = int32_t(lights.size()) - 1;
  if (shots.empty()) {
    // Autofit (the reference calls nvpro_core's CameraManipulator::fit, whose
    // source is not in the reference tree): frame the bounding sphere of all
    // instances from the manipulator's default direction (1,1,1).
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (auto& in : instances) {
      for (auto& v : meshes[in.mesh_id].v) {
        for (int r = 0; r < 3; ++r) {
          double p = double(in.transform[r * 4]) * v.pos[0] + double(in.transform[r * 4 + 1]) * v.pos[1] +
                     double(in.transform[r * 4 + 2]) * v.pos[2] + double(in.transform[r * 4 + 3]);
          lo[r] = std::min(lo[r], p);
          hi[r] = std::max(hi[r], p);
        }
      }
    }
    if (!(lo[0] < hi[0] && lo[1] < hi[1] && lo[2] < hi[2])) {
      for (int k = 0; k < 3; ++k) {
        lo[k] = -1;
        hi[k] = 1;
      }
    }
    double c[3], r2 = 0;
    for (int k = 0; k < 3; ++k) {
      c[k] = 0.5 * (lo[k] + hi[k]);
      r2 += 0.25 * (hi[k] - lo[k]) * (hi[k] - lo[k]);
    }
    double fovr = double(fov) * 0.017453292519943295;
    double aspect = height ? double(width) / height : 1.0;
    double half = aspect > 1.0 ? fovr * 0.5 : fovr * aspect * 0.5;
    double dist = std::sqrt(r2) / std::sin(std::max(half, 1e-3));
    HostShot s{};
    const double dir = 1.0 / std::sqrt(3.0);
    for (int k = 0; k < 3; ++k) {
      s.lookat[k] = float(c[k]);
      s.eye[k] = float(c[k] + dir * dist);
      s.up[k] = k == 1 ? 1.0f : 0.0f;
    }
    std::memset(s.envTransform, 0, sizeof(s.envTransform));
    s.envTransform[0] = s.envTransform[5] = s.envTransform[10] = s.envTransform[15] = 1.0f;
    s.state = state;
    shots.push_back(s);
  }
  meshDescs.resize(meshes.size());
  for (size_t i = 0; i < meshes.size(); ++i) {
    meshDescs[i].num_vertices = uint32_t(meshes[i].v.size());
    meshDescs[i].num_triangles = uint32_t(meshes[i].idx.size() / 3);
    meshDescs[i].vertices = meshes[i].v.data();
    meshDescs[i].indices = meshes[i].idx.data();
  }
  texDescs.resize(textures.size());
  for (size_t i = 0; i < textures.size(); ++i)
    texDescs[i] = asuna_texture_desc{textures[i].w, textures[i].h, textures[i].rgba.data()};
}

void HostScene::desc(asuna_scene_desc* o) const {
  std::memset(o, 0, sizeof(*o));
  o->num_meshes = uint32_t(meshDescs.size());
  o->meshes = meshDescs.data();
  o->num_instances = uint32_t(instances.size());
  o->instances = instances.data();
  o->num_materials = uint32_t(materials.size());
  o->materials = materials.data();
  o->num_lights = uint32_t(lights.size());
  o->lights = lights.data();
  if (envW && envH) {
    o->envmap.width = envW;
    o->envmap.height = envH;
    o->envmap.rgba = env.data();
  }
  o->num_textures = uint32_t(texDescs.size());
  o->textures = texDescs.data();
}

int HostScene::shot(uint32_t i, asuna_shot* out) const {
  if (i >= shots.size()) return fail(ASUNA_ERR_INVALID, "shot %u out of range (%zu shots)", i, shots.size());
  const HostShot& s = shots[i];
  std::memset(out, 0, sizeof(*out));
  int rc;
  if (camType == ASUNA_CAMERA_OPENCV)
    rc = asuna_camera_opencv(s.eye, s.lookat, s.up, fxfycxcy, &out->camera);
  else
    rc = asuna_camera_perspective(s.eye, s.lookat, s.up, fov, aperture, focalDistance, width, height, &out->camera);
  if (rc) return rc;
  std::memcpy(out->camera.env_transform, s.envTransform, sizeof(s.envTransform));
  // Scene::setShot (src/scene/scene.cpp:439-453): per-shot overrides
  out->state = state.rtx;
  out->state.spp = s.state.rtx.spp;
  out->state.max_path_depth = s.state.rtx.max_path_depth;
  out->state.use_face_normal = s.state.rtx.use_face_normal;
  out->state.ignore_emissive = s.state.rtx.ignore_emissive;
  out->state.env_map_intensity = s.state.rtx.env_map_intensity;
  for (int k = 0; k < 3; ++k) out->state.bg_color[k] = s.state.rtx.bg_color[k];
  out->state.cur_frame = 0;
  out->width = width;
  out->height = height;
  out->frames = uint32_t(std::max(1, s.state.rtx.spp));
  out->frame0 = 0;
  out->seed = 0;
  out->flags = 0;
  out->rr_depth = 0;
  out->depth_out_channel = state.depthSlot;
  return ASUNA_OK;
}

// ---- file IO ------------------------------------------------------------------------
static bool readFile(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

int loadObj(const std::string& path, std::vector<asuna_vertex>& verts, std::vector<uint32_t>& idx) {
  std::string text;
  if (!readFile(path, text)) return fail(ASUNA_ERR_IO, "cannot read OBJ file %s", path.c_str());
  std::vector<float> P, T, N;
  std::istringstream in(text);
  std::string line;
  size_t lineNo = 0;
  while (std::getline(in, line)) {
    ++lineNo;
    if (line.size() < 2 || line[0] == '#') continue;
    std::istringstream ls(line);
    std::string tag;
    ls >> tag;
    if (tag == "v") {
      float x, y, z;
      if (!(ls >> x >> y >> z)) return fail(ASUNA_ERR_PARSE, "%s:%zu: bad vertex", path.c_str(), lineNo);
      P.insert(P.end(), {x, y, z});
    } else if (tag == "vt") {
      float u, v = 0;
      if (!(ls >> u)) return fail(ASUNA_ERR_PARSE, "%s:%zu: bad texcoord", path.c_str(), lineNo);
      ls >> v;
      T.insert(T.end(), {u, v});
    } else if (tag == "vn") {
      float x, y, z;
      if (!(ls >> x >> y >> z)) return fail(ASUNA_ERR_PARSE, "%s:%zu: bad normal", path.c_str(), lineNo);
      N.insert(N.end(), {x, y, z});
    } else if (tag == "f") {
      std::vector<asuna_vertex> poly;
      std::string tok;
      while (ls >> tok) {
        int vi = 0, ti = 0, ni = 0;
        const char* s = tok.c_str();
        char* e;
        vi = int(std::strtol(s, &e, 10));
        if (*e == '/') {
          s = e + 1;
          if (*s != '/') ti = int(std::strtol(s, &e, 10));
          else e = const_cast<char*>(s);
          if (*e == '/') ni = int(std::strtol(e + 1, &e, 10));
        }
        auto fix = [](int i, size_t n) { return i < 0 ? int(n) + i : i - 1; };
        vi = fix(vi, P.size() / 3);
        if (vi < 0 || size_t(vi) >= P.size() / 3)
          return fail(ASUNA_ERR_PARSE, "%s:%zu: vertex index out of range", path.c_str(), lineNo);
        asuna_vertex v{};
        for (int k = 0; k < 3; ++k) v.pos[k] = P[3 * vi + k];
        if (ti) {
          ti = fix(ti, T.size() / 2);
          if (ti >= 0 && size_t(ti) < T.size() / 2) {
            v.uv[0] = T[2 * ti];
            v.uv[1] = 1.0f - T[2 * ti + 1];
          }
        }
        if (ni) {
          ni = fix(ni, N.size() / 3);
          if (ni >= 0 && size_t(ni) < N.size() / 3)
            for (int k = 0; k < 3; ++k) v.normal[k] = N[3 * ni + k];
        }
        poly.push_back(v);
      }
      // triangle fan, de-indexed: every corner is its own vertex
      for (size_t k = 2; k < poly.size(); ++k) {
        for (const asuna_vertex* c : {&poly[0], &poly[k - 1], &poly[k]}) {
          idx.push_back(uint32_t(verts.size()));
          verts.push_back(*c);
        }
      }
    }
  }
  return ASUNA_OK;
}

static int loadPfm(const std::string& path, const std::string& data, uint32_t& w, uint32_t& h,
                   std::vector<float>& rgba) {
  std::istringstream in(data);
  std::string magic;
  double scale;
  in >> magic >> w >> h >> scale;
  in.get();
  int ch = magic == "PF" ? 3 : (magic == "Pf" ? 1 : 0);
  if (!ch || !w || !h) return fail(ASUNA_ERR_PARSE, "%s: not a PFM file", path.c_str());
  size_t off = size_t(in.tellg());
  if (data.size() < off + size_t(w) * h * ch * 4) return fail(ASUNA_ERR_PARSE, "%s: truncated PFM", path.c_str());
  const float* px = reinterpret_cast<const float*>(data.data() + off);
  rgba.assign(size_t(w) * h * 4, 1.0f);
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const float* s = px + (size_t(h - 1 - y) * w + x) * ch;  // PFM rows are bottom-up
      float* d = &rgba[(size_t(y) * w + x) * 4];
      for (int k = 0; k < 3; ++k) d[k] = s[ch == 3 ? k : 0];
    }
  return ASUNA_OK;
}

static int loadHdr(const std::string& path, const std::string& data, uint32_t& w, uint32_t& h,
                   std::vector<float>& rgba) {
  // Radiance RGBE (.hdr), flat or new-style run-length rows.
  size_t p = 0;
  auto line = [&]() {
    size_t e = data.find('\n', p);
    if (e == std::string::npos) e = data.size();
    std::string l = data.substr(p, e - p);
    p = e + 1;
    return l;
  };
  std::string first = line();
  if (first.rfind("#?", 0) != 0) return fail(ASUNA_ERR_PARSE, "%s: not a Radiance HDR file", path.c_str());
  for (;;) {
    if (p >= data.size()) return fail(ASUNA_ERR_PARSE, "%s: truncated header", path.c_str());
    std::string l = line();
    if (l.empty()) break;
  }
  std::string res = line();
  char ya[3], xa[3];
  int H = 0, W = 0;
  if (std::sscanf(res.c_str(), "%2s %d %2s %d", ya, &H, xa, &W) != 4 || std::string(ya) != "-Y" || W <= 0 || H <= 0)
    return fail(ASUNA_ERR_PARSE, "%s: unsupported resolution line", path.c_str());
  w = uint32_t(W);
  h = uint32_t(H);
  std::vector<unsigned char> scan(size_t(W) * 4);
  rgba.assign(size_t(W) * H * 4, 1.0f);
  const unsigned char* d = reinterpret_cast<const unsigned char*>(data.data());
  for (int y = 0; y < H; ++y) {
    if (p + 4 > data.size()) return fail(ASUNA_ERR_PARSE, "%s: truncated data", path.c_str());
    if (W >= 8 && W < 32768 && d[p] == 2 && d[p + 1] == 2 && ((d[p + 2] << 8) | d[p + 3]) == W) {
      p += 4;
      for (int c = 0; c < 4; ++c) {
        int x = 0;
        while (x < W) {
          if (p >= data.size()) return fail(ASUNA_ERR_PARSE, "%s: truncated run", path.c_str());
          int cnt = d[p++];
          if (cnt > 128) {
            cnt -= 128;
            if (p >= data.size() || x + cnt > W) return fail(ASUNA_ERR_PARSE, "%s: bad run", path.c_str());
            unsigned char v = d[p++];
            for (int k = 0; k < cnt; ++k) scan[size_t(x++) * 4 + c] = v;
          } else {
            if (cnt == 0 || p + cnt > data.size() || x + cnt > W) return fail(ASUNA_ERR_PARSE, "%s: bad run", path.c_str());
            for (int k = 0; k < cnt; ++k) scan[size_t(x++) * 4 + c] = d[p++];
          }
        }
      }
    } else {
      if (p + size_t(W) * 4 > data.size()) return fail(ASUNA_ERR_PARSE, "%s: truncated data", path.c_str());
      std::memcpy(scan.data(), d + p, size_t(W) * 4);
      p += size_t(W) * 4;
    }
    for (int x = 0; x < W; ++x) {
      const unsigned char* e = &scan[size_t(x) * 4];
      float* o = &rgba[(size_t(y) * W + x) * 4];
      if (e[3] == 0) {
        o[0] = o[1] = o[2] = 0.0f;
      } else {
        float f = std::ldexp(1.0f, int(e[3]) - (128 + 8));
        o[0] = e[0] * f;
        o[1] = e[1] * f;
        o[2] = e[2] * f;
      }
    }
  }
  return ASUNA_OK;
}

int loadImageRGBA(const std::string& path, uint32_t& w, uint32_t& h, std::vector<float>& rgba) {
  std::string data;
  if (!readFile(path, data)) return fail(ASUNA_ERR_IO, "cannot read image %s", path.c_str());
  std::string ext = path.substr(path.find_last_of('.') + 1);
  for (auto& ch : ext) ch = char(std::tolower(ch));
  if (ext == "pfm") return loadPfm(path, data, w, h, rgba);
  if (ext == "hdr") return loadHdr(path, data, w, h, rgba);
  return fail(ASUNA_ERR_UNSUPPORTED, "%s: image format .%s not supported (use .hdr or .pfm)", path.c_str(),
              ext.c_str());
}

// NumPy .npy, format 1.0: magic, little-endian header dict padded with
// spaces to a 64-byte boundary, then the float32 rows (C order).
int writeNpy(const std::string& path, uint64_t rows, uint32_t cols, const float* data) {
  std::string hdr = "{'descr': '<f4', 'fortran_order': False, 'shape': (" + std::to_string(rows) + ", " +
                    std::to_string(cols) + "), }";
  const size_t pre = 10;  // magic (6) + version (2) + header length (2)
  size_t total = pre + hdr.size() + 1;
  hdr.append((64 - total % 64) % 64, ' ');
  hdr.push_back('\n');
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(ASUNA_ERR_IO, "cannot write %s", path.c_str());
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  f.write(reinterpret_cast<const char*>(magic), 8);
  const uint16_t n = uint16_t(hdr.size());
  const unsigned char len[2] = {static_cast<unsigned char>(n & 0xff), static_cast<unsigned char>(n >> 8)};
  f.write(reinterpret_cast<const char*>(len), 2);
  f.write(hdr.data(), std::streamsize(hdr.size()));
  f.write(reinterpret_cast<const char*>(data), std::streamsize(rows * cols * sizeof(float)));
  return f ? ASUNA_OK : fail(ASUNA_ERR_IO, "write failed: %s", path.c_str());
}

int writePfm(const std::string& path, uint32_t w, uint32_t h, const float* rgba) {
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(ASUNA_ERR_IO, "cannot write %s", path.c_str());
  f << "PF\n" << w << " " << h << "\n-1.0\n";
  std::vector<float> row(size_t(w) * 3);
  for (uint32_t y = 0; y < h; ++y) {
    const float* s = rgba + size_t(h - 1 - y) * w * 4;
    for (uint32_t x = 0; x < w; ++x)
      for (int k = 0; k < 3; ++k) row[size_t(x) * 3 + k] = s[size_t(x) * 4 + k];
    f.write(reinterpret_cast<const char*>(row.data()), std::streamsize(row.size() * 4));
  }
  return f ? ASUNA_OK : fail(ASUNA_ERR_IO, "write failed: %s", path.c_str());
}

// OpenEXR (scanline, no compression, FLOAT R,G,B,A): the layout of the
// public OpenEXR file-format description (magic, attribute header, offset
// table, one chunk per scanline with channels in alphabetical order).
int writeExr(const std::string& path, uint32_t w, uint32_t h, const float* rgba) {
  std::string hdr;
  auto u8 = [&](uint8_t v) { hdr.push_back(char(v)); };
  auto i32 = [&](int32_t v) {
    for (int k = 0; k < 4; ++k) u8(uint8_t(uint32_t(v) >> (8 * k)));
  };
  auto f32 = [&](float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    i32(int32_t(b));
  };
  auto str = [&](const char* s) { hdr.append(s, std::strlen(s) + 1); };
  auto attr = [&](const char* name, const char* type, int32_t size) {
    str(name);
    str(type);
    i32(size);
  };
  i32(20000630);  // magic
  i32(2);         // version 2, single-part scanline
  attr("channels", "chlist", 4 * 18 + 1);
  for (const char* c : {"A", "B", "G", "R"}) {
    str(c);
    i32(2);  // FLOAT
    u8(0);
    u8(0);
    u8(0);
    u8(0);
    i32(1);
    i32(1);
  }
  u8(0);
  attr("compression", "compression", 1);
  u8(0);
  attr("dataWindow", "box2i", 16);
  i32(0);
  i32(0);
  i32(int32_t(w) - 1);
  i32(int32_t(h) - 1);
  attr("displayWindow", "box2i", 16);
  i32(0);
  i32(0);
  i32(int32_t(w) - 1);
  i32(int32_t(h) - 1);
  attr("lineOrder", "lineOrder", 1);
  u8(0);
  attr("pixelAspectRatio", "float", 4);
  f32(1.0f);
  attr("screenWindowCenter", "v2f", 8);
  f32(0.0f);
  f32(0.0f);
  attr("screenWindowWidth", "float", 4);
  f32(1.0f);
  u8(0);  // end of header
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(ASUNA_ERR_IO, "cannot write %s", path.c_str());
  f.write(hdr.data(), std::streamsize(hdr.size()));
  const uint64_t lineBytes = 8 + uint64_t(w) * 4 * 4;
  const uint64_t first = hdr.size() + uint64_t(h) * 8;
  for (uint32_t y = 0; y < h; ++y) {
    uint64_t off = first + y * lineBytes;
    f.write(reinterpret_cast<const char*>(&off), 8);  // little-endian hosts
  }
  std::vector<float> line(size_t(w) * 4);
  for (uint32_t y = 0; y < h; ++y) {
    int32_t hy[2] = {int32_t(y), int32_t(w * 16)};
    f.write(reinterpret_cast<const char*>(hy), 8);
    const float* src = rgba + size_t(y) * w * 4;
    for (uint32_t x = 0; x < w; ++x) {
      line[x] = src[x * 4 + 3];
      line[w + x] = src[x * 4 + 2];
      line[2 * size_t(w) + x] = src[x * 4 + 1];
      line[3 * size_t(w) + x] = src[x * 4 + 0];
    }
    f.write(reinterpret_cast<const char*>(line.data()), std::streamsize(line.size() * 4));
  }
  return f ? ASUNA_OK : fail(ASUNA_ERR_IO, "write failed: %s", path.c_str());
}

// PNG, 8-bit RGBA, clamp(v, 0, 1) * 255 with gamma 1 (the reference writes LDR
// channels through stbi with stbi_hdr_to_ldr_gamma(1.0)); zlib stream of
// stored (uncompressed) deflate blocks, as the PNG and zlib specifications allow.
int writePng(const std::string& path, uint32_t w, uint32_t h, const float* rgba) {
  auto crcTable = [] {
    std::vector<uint32_t> t(256);
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[n] = c;
    }
    return t;
  }();
  auto crc = [&](const std::string& d) {
    uint32_t c = 0xFFFFFFFFu;
    for (unsigned char b : d) c = crcTable[(c ^ b) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
  };
  auto be32 = [](std::string& o, uint32_t v) {
    for (int k = 3; k >= 0; --k) o.push_back(char((v >> (8 * k)) & 0xFF));
  };
  std::string raw;
  raw.reserve(size_t(h) * (1 + size_t(w) * 4));
  for (uint32_t y = 0; y < h; ++y) {
    raw.push_back(0);  // filter: none
    for (uint32_t x = 0; x < w * 4; ++x) {
      float v = rgba[size_t(y) * w * 4 + x];
      v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
      raw.push_back(char(uint8_t(v * 255.0f + 0.5f)));
    }
  }
  std::string z;
  z.push_back(char(0x78));
  z.push_back(char(0x01));
  uint32_t a = 1, b = 0;
  for (size_t p = 0; p < raw.size() || p == 0; p += 65535) {
    size_t n = std::min<size_t>(65535, raw.size() - p);
    z.push_back(char(p + n >= raw.size() ? 1 : 0));
    z.push_back(char(n & 0xFF));
    z.push_back(char(n >> 8));
    z.push_back(char(~n & 0xFF));
    z.push_back(char((~n >> 8) & 0xFF));
    z.append(raw, p, n);
    if (n == 0) break;
  }
  for (unsigned char c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  be32(z, (b << 16) | a);
  std::string png("\x89PNG\r\n\x1a\n", 8);
  auto chunk = [&](const char* type, const std::string& data) {
    be32(png, uint32_t(data.size()));
    std::string td = std::string(type, 4) + data;
    png += td;
    be32(png, crc(td));
  };
  std::string ihdr;
  be32(ihdr, w);
  be32(ihdr, h);
  ihdr += std::string("\x08\x06\x00\x00\x00", 5);
  chunk("IHDR", ihdr);
  chunk("IDAT", z);
  chunk("IEND", std::string());
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(ASUNA_ERR_IO, "cannot write %s", path.c_str());
  f.write(png.data(), std::streamsize(png.size()));
  return f ? ASUNA_OK : fail(ASUNA_ERR_IO, "write failed: %s", path.c_str());
}

// ---- scene-file loader ------------------------------------------------------------------
namespace {

struct LoadCtx {
  HostScene& S;
  std::string dir;
};

std::string joinPath(const std::string& dir, const std::string& p) {
  if (p.empty() || p[0] == '/' || dir.empty()) return p;
  return dir + "/" + p;
}

bool vecN(const Json& j, int n, float* out) {
  if (!j.isArr() || int(j.size()) < n) return false;
  for (int i = 0; i < n; ++i) {
    if (!j[size_t(i)].isNum()) return false;
    out[i] = float(j[size_t(i)].num);
  }
  return true;
}

#define REQUIRE(cond, ...) \
  do {                     \
    if (!(cond)) return fail(ASUNA_ERR_PARSE, __VA_ARGS__); \
  } while (0)

int checkKeys(const Json& j, std::initializer_list<const char*> keys, const char* where) {
  for (const char* k : keys) REQUIRE(j.has(k), "%s: missing key \"%s\"", where, k);
  return ASUNA_OK;
}

// src/loader/loader.cpp:148-234
int parseState(const Json& sj, HostState& st) {
  if (sj.has("path_tracing")) {
    const Json& pt = sj["path_tracing"];
    asuna_rt_state& r = st.rtx;
    if (pt.has("spp")) r.spp = int32_t(pt["spp"].num);
    if (pt.has("max_path_depth")) r.max_path_depth = int32_t(pt["max_path_depth"].num);
    if (pt.has("use_face_normal")) r.use_face_normal = pt["use_face_normal"].b ? 1u : 0u;
    if (pt.has("ignore_emissive")) r.ignore_emissive = pt["ignore_emissive"].b ? 1u : 0u;
    if (pt.has("background_color")) REQUIRE(vecN(pt["background_color"], 3, r.bg_color), "bad background_color");
    if (pt.has("envmap_intensity")) r.env_map_intensity = float(pt["envmap_intensity"].num);
    if (pt.has("multi_channel")) {
      const Json& mc = pt["multi_channel"];
      REQUIRE(mc.isArr(), "multi_channel must be an array");
      REQUIRE(mc.size() <= ASUNA_MAX_CHANNELS, "channel numbers can not exceed %d", ASUNA_MAX_CHANNELS);
      r.n_multi_channel = uint32_t(mc.size());
      st.channelKinds.assign(mc.size(), -1);
      for (uint32_t c = 0; c < mc.size(); ++c) {
        REQUIRE(mc[c].isStr(), "multi_channel entries must be strings");
        const std::string& t = mc[c].str;
        int kind = -1;
        if (t == "diffuse" || t == "albedo") r.diffuse_out_channel = int32_t(c), kind = ASUNA_CH_DIFFUSE;
        if (t == "normal") r.normal_out_channel = int32_t(c), kind = ASUNA_CH_NORMAL;
        if (t == "specular") r.specular_out_channel = int32_t(c), kind = ASUNA_CH_SPECULAR;
        if (t == "tangent") r.tangent_out_channel = int32_t(c), kind = ASUNA_CH_TANGENT;
        if (t == "roughness") r.roughness_out_channel = int32_t(c), kind = ASUNA_CH_ROUGHNESS;
        if (t == "position") r.position_out_channel = int32_t(c), kind = ASUNA_CH_POSITION;
        if (t == "uv") r.uv_out_channel = int32_t(c), kind = ASUNA_CH_UV;
        if (t == "depth") st.depthSlot = int32_t(c), kind = ASUNA_CH_DEPTH;
        st.channelKinds[c] = kind;
      }
    }
    st.channelLdr.assign(st.rtx.n_multi_channel, false);
    if (pt.has("multi_channel_ldr")) {
      const Json& ml = pt["multi_channel_ldr"];
      for (uint32_t c = 0; c < std::min<uint32_t>(st.rtx.n_multi_channel, uint32_t(ml.size())); ++c)
        st.channelLdr[c] = ml[c].b;
    }
  }
  if (sj.has("post_processing")) {
    const Json& pp = sj["post_processing"];
    std::string tm = pp.has("tone_mapping") ? pp["tone_mapping"].str : "";
    static const char* names[] = {"none", "gamma", "reinhard", "Aces", "filmic", "pbrt", "custom"};
    st.toneMapping = 0;
    for (uint32_t i = 0; i < 7; ++i)
      if (tm == names[i]) st.toneMapping = i;
  }
  if (sj.has("output_render_result")) st.outputRenderResult = sj["output_render_result"].b;
  if (sj.has("output_hdr")) st.outputHdr = sj["output_hdr"].b;
  return ASUNA_OK;
}

// src/loader/loader.cpp:366-396 (row-major JSON matrices, left-multiplied chain)
int parseToWorld(const Json& tw, M4& out, bool banTranslation) {
  out = M4::id();
  REQUIRE(tw.isArr(), "toworld must be an array");
  const double d2r = 0.017453292519943295;
  auto rot = [](int axis, double a) {
    M4 r = M4::id();
    double c = std::cos(a), s = std::sin(a);
    int i = (axis + 1) % 3, j = (axis + 2) % 3;
    r.m[i][i] = c;
    r.m[i][j] = -s;
    r.m[j][i] = s;
    r.m[j][j] = c;
    return r;
  };
  for (size_t k = 0; k < tw.size(); ++k) {
    const Json& s = tw[k];
    int rc = checkKeys(s, {"type", "value"}, "toworld");
    if (rc) return rc;
    const std::string& t = s["type"].str;
    M4 m = M4::id();
    float v[16];
    if (t == "matrix") {
      REQUIRE(vecN(s["value"], 16, v), "toworld matrix needs 16 numbers");
      m = fromRowMajor16(v);
    } else if (t == "translate") {
      REQUIRE(vecN(s["value"], 3, v), "translate needs 3 numbers");
      if (!banTranslation)
        for (int i = 0; i < 3; ++i) m.m[i][3] = v[i];
    } else if (t == "scale") {
      REQUIRE(vecN(s["value"], 3, v), "scale needs 3 numbers");
      for (int i = 0; i < 3; ++i) m.m[i][i] = v[i];
    } else if (t == "rotx" || t == "roty" || t == "rotz") {
      REQUIRE(s["value"].isNum(), "rotation needs a number");
      m = rot(t == "rotx" ? 0 : (t == "roty" ? 1 : 2), d2r * float(s["value"].num));
    } else if (t == "rotate") {
      REQUIRE(vecN(s["value"], 3, v), "rotate needs 3 numbers");
      m = rot(2, d2r * v[2]) * rot(1, d2r * v[1]) * rot(0, d2r * v[0]);
    } else {
      return fail(ASUNA_ERR_PARSE, "unrecognized toworld singleton type [%s]", t.c_str());
    }
    out = m * out;
  }
  return ASUNA_OK;
}

float dielectricReflectance(float eta, float cosThetaI, float& cosThetaT) {
  if (cosThetaI < 0.0f) {
    eta = 1.0f / eta;
    cosThetaI = -cosThetaI;
  }
  float sinThetaTSq = eta * eta * (1.0f - cosThetaI * cosThetaI);
  if (sinThetaTSq > 1.0f) {
    cosThetaT = 0.0f;
    return 1.0f;
  }
  cosThetaT = std::sqrt(std::max(1.0f - sinThetaTSq, 0.0f));
  float Rs = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  float Rp = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
  return (Rs * Rs + Rp * Rp) * 0.5f;
}

int addMaterial(LoadCtx& L, const Json& mj) {
  int rc = checkKeys(mj, {"type", "name"}, "material");
  if (rc) return rc;
  const std::string& name = mj["name"].str;
  REQUIRE(L.S.materialId(name) < 0, "material [%s] defined twice", name.c_str());
  asuna_material m = defaultMaterial();
  const std::string& t = mj["type"].str;
  auto tex = [&](const char* key, int32_t& id) -> int {
    if (!mj.has(key)) return ASUNA_OK;
    const std::string& tn = mj[key].str;
    for (size_t i = 0; i < L.S.textureNames.size(); ++i)
      if (L.S.textureNames[i] == tn) {
        id = int32_t(i);
        return ASUNA_OK;
      }
    return fail(ASUNA_ERR_PARSE, "texture [\"%s\"] does not exist", tn.c_str());
  };
  if (t == "brdf_lambertian") {
    m.type = ASUNA_MAT_LAMBERTIAN;
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id)) || (rc = tex("normal_texture", m.normal_texture_id)))
      return rc;
  } else if (t == "bsdf_dielectric") {
    m.type = ASUNA_MAT_DIELECTRIC;
    if ((rc = tex("normal_texture", m.normal_texture_id))) return rc;
    if (mj.has("ior")) m.ior = float(mj["ior"].num);
  } else if (t == "brdf_rough_plastic") {
    m.type = ASUNA_MAT_ROUGH_PLASTIC;
    if (mj.has("ior")) m.ior = float(mj["ior"].num);
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id)) || (rc = tex("normal_texture", m.normal_texture_id)))
      return rc;
    if (mj.has("alpha")) REQUIRE(vecN(mj["alpha"], 2, m.aniso_alpha), "bad alpha");
    if ((rc = tex("alpha_texture", m.roughness_texture_id))) return rc;
    m.radiance[0] = asuna_diffuse_fresnel(m.ior, 1000);
  } else if (t == "brdf_plastic") {
    // src/loader/material.cpp:197-210
    m.type = ASUNA_MAT_PLASTIC;
    if (mj.has("ior")) m.ior = float(mj["ior"].num);
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id)) || (rc = tex("normal_texture", m.normal_texture_id)))
      return rc;
    m.radiance[0] = asuna_diffuse_fresnel(m.ior, 1000);
  } else if (t == "brdf_mirror") {
    // src/loader/material.cpp:233-243
    m.type = ASUNA_MAT_MIRROR;
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id)) || (rc = tex("normal_texture", m.normal_texture_id)))
      return rc;
  } else if (t == "brdf_conductor" || t == "brdf_rough_conductor") {
    // src/loader/material.cpp:306-347: eta in radiance, k in radiance_factor
    const bool rough = t == "brdf_rough_conductor";
    m.type = rough ? ASUNA_MAT_ROUGH_CONDUCTOR : ASUNA_MAT_CONDUCTOR;
    std::string metal = "Cu";
    if (mj.has("material")) metal = mj["material"].str;
    if ((rc = asuna_complex_ior(metal.c_str(), m.radiance, m.radiance_factor))) return rc;
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id)) || (rc = tex("normal_texture", m.normal_texture_id)))
      return rc;
    if (rough) {
      if (mj.has("alpha")) REQUIRE(vecN(mj["alpha"], 2, m.aniso_alpha), "bad alpha");
      if ((rc = tex("alpha_texture", m.roughness_texture_id))) return rc;
    }
  } else if (t == "brdf_phong") {
    // src/loader/material.cpp:391-405: specular reflectance in rho_spec, the
    // exponent in specular
    m.type = ASUNA_MAT_PHONG;
    if ((rc = tex("normal_texture", m.normal_texture_id))) return rc;
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id))) return rc;
    if (mj.has("specular_reflectance"))
      REQUIRE(vecN(mj["specular_reflectance"], 3, m.rho_spec), "bad specular_reflectance");
    if (mj.has("shininess")) m.specular = float(mj["shininess"].num);
  } else if (t == "brdf_pbr_metalness_roughness") {
    // src/loader/material.cpp:116-143: opacity (specular) is always 0
    m.type = ASUNA_MAT_PBR_METALNESS_ROUGHNESS;
    if ((rc = tex("normal_texture", m.normal_texture_id))) return rc;
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id))) return rc;
    if (mj.has("metalness")) m.metalness = float(mj["metalness"].num);
    if ((rc = tex("metalness_texture", m.metalness_texture_id))) return rc;
    if (mj.has("roughness")) m.roughness = float(mj["roughness"].num);
    if ((rc = tex("roughness_texture", m.roughness_texture_id))) return rc;
    m.specular = 0.0f;
    if ((rc = tex("opacity_texture", m.opacity_texture_id))) return rc;
  } else if (t == "brdf_disney") {
    // src/loader/material.cpp:359-389: opacity in rho_spec[0]; the other
    // Disney parameters keep their defaults (0) on this path
    m.type = ASUNA_MAT_DISNEY;
    if ((rc = tex("normal_texture", m.normal_texture_id))) return rc;
    if (mj.has("diffuse_reflectance")) REQUIRE(vecN(mj["diffuse_reflectance"], 3, m.diffuse), "bad diffuse_reflectance");
    if ((rc = tex("diffuse_texture", m.diffuse_texture_id))) return rc;
    if (mj.has("metallic")) m.metalness = float(mj["metallic"].num);
    if ((rc = tex("metallic_texture", m.metalness_texture_id))) return rc;
    if (mj.has("roughness")) m.roughness = float(mj["roughness"].num);
    if ((rc = tex("roughness_texture", m.roughness_texture_id))) return rc;
    m.rho_spec[0] = 0.0f;
    if (mj.has("opacity")) m.rho_spec[0] = float(mj["opacity"].num);
    if ((rc = tex("opacity_texture", m.opacity_texture_id))) return rc;
  } else if (t == "brdf_kang18") {
    // src/loader/material.cpp:156-187: each of diffuse, specular and alpha
    // comes from its texture or else its (required) value; specular in
    // rho_spec, alpha in aniso_alpha, opacity (metalness) 0
    m.type = ASUNA_MAT_KANG18;
    if ((rc = tex("normal_texture", m.normal_texture_id)) || (rc = tex("tangent_texture", m.tangent_texture_id)))
      return rc;
    if (mj.has("diffuse_texture")) {
      if ((rc = tex("diffuse_texture", m.diffuse_texture_id))) return rc;
    } else {
      REQUIRE(mj.has("diffuse_reflectance") && vecN(mj["diffuse_reflectance"], 3, m.diffuse),
              "brdf_kang18 needs diffuse_reflectance or diffuse_texture");
    }
    if (mj.has("specular_texture")) {
      if ((rc = tex("specular_texture", m.metalness_texture_id))) return rc;
    } else {
      REQUIRE(mj.has("specular_reflectance") && vecN(mj["specular_reflectance"], 3, m.rho_spec),
              "brdf_kang18 needs specular_reflectance or specular_texture");
    }
    if (mj.has("alpha_texture")) {
      if ((rc = tex("alpha_texture", m.roughness_texture_id))) return rc;
    } else {
      REQUIRE(mj.has("alpha") && vecN(mj["alpha"], 2, m.aniso_alpha), "brdf_kang18 needs alpha or alpha_texture");
    }
    m.metalness = 0.0f;
    if ((rc = tex("opacity_texture", m.opacity_texture_id))) return rc;
  } else if (t == "brdf_emissive") {
    // src/loader/material.cpp:145-155
    m.type = ASUNA_MAT_EMISSIVE;
    if (mj.has("radiance")) REQUIRE(vecN(mj["radiance"], 3, m.radiance), "bad radiance");
    if (mj.has("radiance_factor")) REQUIRE(vecN(mj["radiance_factor"], 3, m.radiance_factor), "bad radiance_factor");
    if ((rc = tex("radiance_texture", m.radiance_texture_id))) return rc;
  } else {
    return fail(ASUNA_ERR_PARSE, "unrecognized material type [%s]", t.c_str());
  }
  L.S.materialNames.push_back(name);
  L.S.materials.push_back(m);
  return ASUNA_OK;
}

// src/loader/loader.cpp:270-332
int addLight(LoadCtx& L, const Json& lj) {
  int rc = checkKeys(lj, {"type", "radiance"}, "light");
  if (rc) return rc;
  asuna_light l;
  std::memset(&l, 0, sizeof(l));
  l.type = ASUNA_LIGHT_UNDEFINED;
  REQUIRE(vecN(lj["radiance"], 3, l.radiance), "bad light radiance");
  const std::string& t = lj["type"].str;
  if (t == "rect" || t == "triangle") {
    if ((rc = checkKeys(lj, {"position", "v1", "v2"}, "light"))) return rc;
    float v1[3], v2[3];
    REQUIRE(vecN(lj["v1"], 3, v1) && vecN(lj["v2"], 3, v2) && vecN(lj["position"], 3, l.position), "bad light geometry");
    for (int k = 0; k < 3; ++k) {
      l.u[k] = v1[k] - l.position[k];
      l.v[k] = v2[k] - l.position[k];
    }
    float cx = l.u[1] * l.v[2] - l.u[2] * l.v[1], cy = l.u[2] * l.v[0] - l.u[0] * l.v[2],
          cz = l.u[0] * l.v[1] - l.u[1] * l.v[0];
    l.area = std::sqrt(cx * cx + cy * cy + cz * cz);
    // JSON "triangle" lights stay LightTypeRect with half the area
    // (src/loader/loader.cpp:284-296): meshed and sampled as a parallelogram.
    l.type = ASUNA_LIGHT_RECT;
    if (lj.has("double_side")) l.double_side = lj["double_side"].b ? 1u : 0u;
    if (t == "triangle") l.area *= 0.5f;
  } else if (t == "point") {
    if ((rc = checkKeys(lj, {"position"}, "light"))) return rc;
    REQUIRE(vecN(lj["position"], 3, l.position), "bad light position");
    l.type = ASUNA_LIGHT_POINT;
  } else if (t == "distant") {
    if ((rc = checkKeys(lj, {"direction"}, "light"))) return rc;
    REQUIRE(vecN(lj["direction"], 3, l.direction), "bad light direction");
    l.type = ASUNA_LIGHT_DIRECTIONAL;
  } else if (t == "mesh") {
    if ((rc = checkKeys(lj, {"path"}, "light"))) return rc;
    std::vector<asuna_vertex> v;
    std::vector<uint32_t> idx;
    if ((rc = loadObj(joinPath(L.dir, lj["path"].str), v, idx))) return rc;
    l.type = ASUNA_LIGHT_TRIANGLE;
    return L.S.addMeshLight(l, v, idx);
  } else {
    return fail(ASUNA_ERR_PARSE, "unrecognized light type [%s]", t.c_str());
  }
  return L.S.addLight(l);
}

int addShot(LoadCtx& L, const Json& sj) {
  int rc = checkKeys(sj, {"type"}, "shot");
  if (rc) return rc;
  HostShot s{};
  const std::string& t = sj["type"].str;
  float m16[16];
  if (t == "lookat") {
    if ((rc = checkKeys(sj, {"eye", "lookat", "up"}, "shot"))) return rc;
    REQUIRE(vecN(sj["eye"], 3, s.eye) && vecN(sj["lookat"], 3, s.lookat) && vecN(sj["up"], 3, s.up), "bad lookat shot");
  } else if (t == "toworld" || t == "opencv") {
    if ((rc = checkKeys(sj, {"matrix"}, "shot"))) return rc;
    REQUIRE(vecN(sj["matrix"], 16, m16), "shot matrix needs 16 numbers");
    M4 c2w = fromRowMajor16(m16);
    if (t == "opencv") {
      M4 inv;
      REQUIRE(invert4(c2w, inv), "singular opencv extrinsic");
      c2w = inv;
    }
    const double upy = t == "opencv" ? -1.0 : 1.0;
    for (int k = 0; k < 3; ++k) {
      s.eye[k] = float(c2w.m[k][3]);
      s.up[k] = float(c2w.m[k][1] * upy);
      s.lookat[k] = float(c2w.m[k][2] + c2w.m[k][3]);
    }
  } else {
    return fail(ASUNA_ERR_PARSE, "unrecognized shot type [%s]", t.c_str());
  }
  s.state = L.S.state;
  if (sj.has("state") && (rc = parseState(sj["state"], s.state))) return rc;
  M4 env = M4::id();
  if (sj.has("env_toworld") && (rc = parseToWorld(sj["env_toworld"], env, true))) return rc;
  storeColMajor(env, s.envTransform);
  L.S.shots.push_back(s);
  return ASUNA_OK;
}

}  // namespace

int loadSceneJson(const std::string& text, const std::string& baseDir, HostScene& S) {
  Json root;
  std::string err;
  if (!parseJson(text, root, err)) return fail(ASUNA_ERR_PARSE, "scene JSON: %s", err.c_str());
  int rc = checkKeys(root, {"state", "camera", "meshes", "instances"}, "scene");
  if (rc) return rc;
  S.reset();
  LoadCtx L{S, baseDir};
  if ((rc = parseState(root["state"], S.state))) return rc;
  // camera (loader.cpp:242-268)
  const Json& cj = root["camera"];
  if ((rc = checkKeys(cj, {"type", "film"}, "camera"))) return rc;
  if ((rc = checkKeys(cj["film"], {"resolution"}, "camera.film"))) return rc;
  float res[2];
  REQUIRE(vecN(cj["film"]["resolution"], 2, res) && res[0] >= 1 && res[1] >= 1, "bad film resolution");
  S.width = uint32_t(res[0]);
  S.height = uint32_t(res[1]);
  if (cj["type"].str == "perspective") {
    S.camType = ASUNA_CAMERA_PERSPECTIVE;
    if (cj.has("fov")) S.fov = float(cj["fov"].num);
    if (cj.has("aperture")) S.aperture = float(cj["aperture"].num);
    if (cj.has("focal_distance")) S.focalDistance = float(cj["focal_distance"].num);
  } else if (cj["type"].str == "opencv") {
    if ((rc = checkKeys(cj, {"fx", "fy", "cx", "cy"}, "camera"))) return rc;
    S.camType = ASUNA_CAMERA_OPENCV;
    S.fxfycxcy[0] = float(cj["fx"].num);
    S.fxfycxcy[1] = float(cj["fy"].num);
    S.fxfycxcy[2] = float(cj["cx"].num);
    S.fxfycxcy[3] = float(cj["cy"].num);
  } else {
    return fail(ASUNA_ERR_PARSE, "unrecognized camera type [%s]", cj["type"].str.c_str());
  }
  if (root.has("textures")) {
    // src/loader/loader.cpp:334-347.  Decoding image files is not this
    // library's job: .hdr and .pfm are read; other formats are reported
    // (callers can pass decoded RGBA32F through asuna_scene_desc.textures).
    // "gamma" applies only to 8-bit formats, none of which is read here.
    for (size_t i = 0; i < root["textures"].size(); ++i) {
      const Json& tj = root["textures"][i];
      if ((rc = checkKeys(tj, {"name", "path"}, "texture"))) return rc;
      HostScene::Texture t;
      if ((rc = loadImageRGBA(joinPath(baseDir, tj["path"].str), t.w, t.h, t.rgba))) return rc;
      S.textureNames.push_back(tj["name"].str);
      S.textures.push_back(std::move(t));
    }
  }
  if (root.has("materials"))
    for (size_t i = 0; i < root["materials"].size(); ++i)
      if ((rc = addMaterial(L, root["materials"][i]))) return rc;
  if (root.has("lights"))
    for (size_t i = 0; i < root["lights"].size(); ++i)
      if ((rc = addLight(L, root["lights"][i]))) return rc;
  if (root.has("envmap")) {
    const Json& ej = root["envmap"];
    if ((rc = checkKeys(ej, {"path"}, "envmap"))) return rc;
    if ((rc = loadImageRGBA(joinPath(baseDir, ej["path"].str), S.envW, S.envH, S.env))) return rc;
    S.state.rtx.has_env_map = 1;
    S.state.rtx.env_map_resolution[0] = float(S.envW);
    S.state.rtx.env_map_resolution[1] = float(S.envH);
  }
  const Json& mj = root["meshes"];
  for (size_t i = 0; i < mj.size(); ++i) {
    const Json& m = mj[i];
    if ((rc = checkKeys(m, {"name", "path"}, "mesh"))) return rc;
    REQUIRE(S.meshId(m["name"].str) < 0, "mesh [%s] defined twice", m["name"].str.c_str());
    HostMesh hm;
    hm.name = m["name"].str;
    if ((rc = loadObj(joinPath(baseDir, m["path"].str), hm.v, hm.idx))) return rc;
    bool recompute = m.has("recompute_normal") && m["recompute_normal"].b;
    float uvs[2] = {1.0f, 1.0f};
    if (m.has("uv_scale")) REQUIRE(vecN(m["uv_scale"], 2, uvs), "bad uv_scale");
    for (size_t t = 0; t + 2 < hm.idx.size(); t += 3) {
      asuna_vertex* v[3] = {&hm.v[hm.idx[t]], &hm.v[hm.idx[t + 1]], &hm.v[hm.idx[t + 2]]};
      if (recompute) {
        float e1[3], e2[3];
        for (int k = 0; k < 3; ++k) {
          e1[k] = v[1]->pos[k] - v[0]->pos[k];
          e2[k] = v[2]->pos[k] - v[0]->pos[k];
        }
        float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) v[j]->normal[k] = n[k] / l;
      }
      for (int j = 0; j < 3; ++j) {
        v[j]->uv[0] *= uvs[0];
        v[j]->uv[1] *= uvs[1];
      }
    }
    S.meshes.push_back(std::move(hm));
  }
  const Json& ij = root["instances"];
  for (size_t i = 0; i < ij.size(); ++i) {
    const Json& in = ij[i];
    if ((rc = checkKeys(in, {"mesh"}, "instance"))) return rc;
    int mesh = S.meshId(in["mesh"].str);
    REQUIRE(mesh >= 0, "mesh [\"%s\"] does not exist", in["mesh"].str.c_str());
    // Without "material" the reference reads a key absent from its defaults
    // (loader.cpp:401-404); the dummy material 0 is used here.
    int mat = 0;
    if (in.has("material")) {
      mat = S.materialId(in["material"].str);
      REQUIRE(mat >= 0, "material [\"%s\"] does not exist", in["material"].str.c_str());
    }
    M4 tw = M4::id();
    if (in.has("toworld") && (rc = parseToWorld(in["toworld"], tw, false))) return rc;
    asuna_instance_desc d{};
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) d.transform[r * 4 + c] = float(tw.m[r][c]);
    d.mesh_id = uint32_t(mesh);
    d.material_id = mat;
    d.light_id = -1;
    S.instances.push_back(d);
  }
  if (root.has("shots"))
    for (size_t i = 0; i < root["shots"].size(); ++i)
      if ((rc = addShot(L, root["shots"][i]))) return rc;
  S.submit();
  return ASUNA_OK;
}

}  // namespace asuna

// ============================================================================
using namespace asuna;

struct asuna_json_scene {
  HostScene scene;
};

namespace {

// Named complex indices of refraction (eta, k) at R, G, B of the conductor
// materials: the values of the reference's table (src/loader/material.cpp:
// 245-289), which JSON scene files select by name.
struct NamedIor {
  const char* name;
  float eta[3], k[3];
};
const NamedIor kConductorIors[] = {
    {"a-C", {2.9440999183f, 2.2271502925f, 1.9681668794f}, {0.8874329109f, 0.7993216383f, 0.8152862927f}},
    {"Ag", {0.1552646489f, 0.1167232965f, 0.1383806959f}, {4.8283433224f, 3.1222459278f, 2.1469504455f}},
    {"Al", {1.6574599595f, 0.8803689579f, 0.5212287346f}, {9.2238691996f, 6.2695232477f, 4.8370012281f}},
    {"AlAs", {3.6051023902f, 3.2329365777f, 2.2175611545f}, {0.0006670247f, -0.0004999400f, 0.0074261204f}},
    {"AlSb", {-0.0485225705f, 4.1427547893f, 4.6697691348f}, {-0.0363741915f, 0.0937665154f, 1.3007390124f}},
    {"Au", {0.1431189557f, 0.3749570432f, 1.4424785571f}, {3.9831604247f, 2.3857207478f, 1.6032152899f}},
    {"Be", {4.1850592788f, 3.1850604423f, 2.7840913457f}, {3.8354398268f, 3.0101260162f, 2.8690088743f}},
    {"Cr", {4.3696828663f, 2.9167024892f, 1.6547005413f}, {5.2064337956f, 4.2313645277f, 3.7549467933f}},
    {"CsI", {2.1449030413f, 1.7023164587f, 1.6624194173f}, {0.0000000000f, 0.0000000000f, 0.0000000000f}},
    {"Cu", {0.2004376970f, 0.9240334304f, 1.1022119527f}, {3.9129485033f, 2.4528477015f, 2.1421879552f}},
    {"Cu2O", {3.5492833755f, 2.9520622449f, 2.7369202137f}, {0.1132179294f, 0.1946659670f, 0.6001681264f}},
    {"CuO", {3.2453822204f, 2.4496293965f, 2.1974114493f}, {0.5202739621f, 0.5707372756f, 0.7172250613f}},
    {"d-C", {2.7112524747f, 2.3185812849f, 2.2288565009f}, {0.0000000000f, 0.0000000000f, 0.0000000000f}},
    {"Hg", {2.3989314904f, 1.4400254917f, 0.9095512090f}, {6.3276269444f, 4.3719414152f, 3.4217899270f}},
    {"HgTe", {4.7795267752f, 3.2309984581f, 2.6600252401f}, {1.6319827058f, 1.5808189339f, 1.7295753852f}},
    {"Ir", {3.0864098394f, 2.0821938440f, 1.6178866805f}, {5.5921510077f, 4.0671757150f, 3.2672611269f}},
    {"K", {0.0640493070f, 0.0464100621f, 0.0381842017f}, {2.1042155920f, 1.3489364357f, 0.9132113889f}},
    {"Li", {0.2657871942f, 0.1956102432f, 0.2209198538f}, {3.5401743407f, 2.3111306542f, 1.6685930000f}},
    {"MgO", {2.0895885542f, 1.6507224525f, 1.5948759692f}, {0.0000000000f, -0.0000000000f, 0.0000000000f}},
    {"Mo", {4.4837010280f, 3.5254578255f, 2.7760769438f}, {4.1111307988f, 3.4208716252f, 3.1506031404f}},
    {"Na", {0.0602665320f, 0.0561412435f, 0.0619909494f}, {3.1792906496f, 2.1124800781f, 1.5790940266f}},
    {"Nb", {3.4201353595f, 2.7901921379f, 2.3955856658f}, {3.4413817900f, 2.7376437930f, 2.5799132708f}},
    {"Ni", {2.3672753521f, 1.6633583302f, 1.4670554172f}, {4.4988329911f, 3.0501643957f, 2.3454274399f}},
    {"Rh", {2.5857954933f, 1.8601866068f, 1.5544279524f}, {6.7822927110f, 4.7029501026f, 3.9760892461f}},
    {"Se-e", {5.7242724833f, 4.1653992967f, 4.0816099264f}, {0.8713747439f, 1.1052845009f, 1.5647788766f}},
    {"Se", {4.0592611085f, 2.8426947380f, 2.8207582835f}, {0.7543791750f, 0.6385150558f, 0.5215872029f}},
    {"SiC", {3.1723450205f, 2.5259677964f, 2.4793623897f}, {0.0000007284f, -0.0000006859f, 0.0000100150f}},
    {"SnTe", {4.5251865890f, 1.9811525984f, 1.2816819226f}, {0.0000000000f, 0.0000000000f, 0.0000000000f}},
    {"Ta", {2.0625846607f, 2.3930915569f, 2.6280684948f}, {2.4080467973f, 1.7413705864f, 1.9470377016f}},
    {"Te-e", {7.5090397678f, 4.2964603080f, 2.3698732430f}, {5.5842076830f, 4.9476231084f, 3.9975145063f}},
    {"Te", {7.3908396088f, 4.4821028985f, 2.6370708478f}, {3.2561412892f, 3.5273908133f, 3.2921683116f}},
    {"ThF4", {1.8307187117f, 1.4422274283f, 1.3876488528f}, {0.0000000000f, 0.0000000000f, 0.0000000000f}},
    {"TiC", {3.7004673762f, 2.8374356509f, 2.5823030278f}, {3.2656905818f, 2.3515586388f, 2.1727857800f}},
    {"TiN", {1.6484691607f, 1.1504482522f, 1.3797795097f}, {3.3684596226f, 1.9434888540f, 1.1020123347f}},
    {"TiO2-e", {3.1065574823f, 2.5131551146f, 2.5823844157f}, {0.0000289537f, -0.0000251484f, 0.0001775555f}},
    {"TiO2", {3.4566203131f, 2.8017076558f, 2.9051485020f}, {0.0001026662f, -0.0000897534f, 0.0006356902f}},
    {"VC", {3.6575665991f, 2.7527298065f, 2.5326814570f}, {3.0683516659f, 2.1986687713f, 1.9631816252f}},
    {"VN", {2.8656011588f, 2.1191817791f, 1.9400767149f}, {3.0323264950f, 2.0561075580f, 1.6162930914f}},
    {"V", {4.2775126218f, 3.5131538236f, 2.7611257461f}, {3.4911844504f, 2.8893580874f, 3.1116965117f}},
    {"W", {4.3707029924f, 3.3002972445f, 2.9982666528f}, {3.5006778591f, 2.6048652781f, 2.2731930614f}},
};
}  // namespace

extern "C" {

int asuna_abi_version(void) { return ASUNA_ABI_VERSION; }

// Scene::reset's sun & sky (src/scene/scene.cpp:112-129)
void asuna_sun_and_sky_default(asuna_sun_and_sky* out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  for (int k = 0; k < 3; ++k) {
    out->rgb_unit_conversion[k] = 1.0f;
    out->ground_color[k] = 0.4f;
  }
  out->multiplier = 0.0000101320f;
  out->haze = 0.0f;
  out->redblueshift = 0.0f;
  out->saturation = 1.0f;
  out->horizon_height = 0.0f;
  out->horizon_blur = 0.1f;
  out->night_color[2] = 0.01f;
  out->sun_disk_intensity = 0.8f;
  out->sun_direction[1] = 0.78f;
  out->sun_direction[2] = 0.62f;
  out->sun_disk_scale = 5.0f;
  out->sun_glow_intensity = 1.0f;
  out->y_is_up = 1;
  out->physically_scaled_sun = 1;
  out->in_use = 0;
}

int asuna_scene_validate(const asuna_scene_desc* desc) {
  clearError();
  if (!desc) return fail(ASUNA_ERR_INVALID, "null argument");
  return validateSceneDesc(desc);
}
const char* asuna_last_error(void) { return gLastError.c_str(); }

int asuna_camera_perspective(const float eye[3], const float lookat[3], const float up[3], float fov_deg,
                             float aperture, float focal_distance, uint32_t width, uint32_t height, asuna_camera* out) {
  if (!eye || !lookat || !up || !out || !width || !height) return fail(ASUNA_ERR_INVALID, "camera: bad argument");
  if (!(fov_deg > 0.0f && fov_deg < 180.0f)) return fail(ASUNA_ERR_INVALID, "camera: fov %g out of (0, 180)", fov_deg);
  std::memset(out, 0, sizeof(*out));
  out->type = ASUNA_CAMERA_PERSPECTIVE;
  storeColMajor(cameraToWorld(eye, lookat, up), out->camera_to_world);
  M4 inv;
  if (!invert4(cameraToRaster(width, height, fov_deg, 0.1f, 100.0f), inv))
    return fail(ASUNA_ERR_INVALID, "camera: singular projection");
  storeColMajor(inv, out->raster_to_camera);
  storeColMajor(M4::id(), out->env_transform);
  out->aperture = aperture;
  out->focal_distance = focal_distance;
  return ASUNA_OK;
}

int asuna_camera_opencv(const float eye[3], const float lookat[3], const float up[3], const float fxfycxcy[4],
                        asuna_camera* out) {
  if (!eye || !lookat || !up || !fxfycxcy || !out) return fail(ASUNA_ERR_INVALID, "camera: bad argument");
  std::memset(out, 0, sizeof(*out));
  out->type = ASUNA_CAMERA_OPENCV;
  storeColMajor(cameraToWorld(eye, lookat, up), out->camera_to_world);
  storeColMajor(M4::id(), out->env_transform);
  for (int k = 0; k < 4; ++k) out->fxfycxcy[k] = fxfycxcy[k];
  return ASUNA_OK;
}

// Environment-map importance tables, following EnvMap::EnvMap
// (src/core/texture.cpp:144-226) step for step: texel weights 0.3 r + 0.6 g
// + 0.1 b, per-row conditional and marginal pdf/cdf with the 1e-7 guards,
// and the inverse-CDF lookup by lower bound, with its double literals and
// float storage.  The tables must equal the reference's
// bit for bit, or the environment samples of the two diverge.
int asuna_envmap_tables(uint32_t width, uint32_t height, const float* px, float* marg, float* cond) {
  if (!width || !height || !px || !marg || !cond) return fail(ASUNA_ERR_INVALID, "envmap tables: bad argument");
  const int W = int(width), H = int(height);
  std::vector<float> pdf2D(size_t(W) * H), cdf2D(size_t(W) * H), pdf1D(H), cdf1D(H);
  std::memset(marg, 0, size_t(W) * H * 2 * sizeof(float));
  std::memset(cond, 0, size_t(W) * H * 2 * sizeof(float));
  float weightSum = 0.0f;
  for (int j = 0; j < H; ++j) {
    float rowWeightSum = 0.0f;
    for (int i = 0; i < W; ++i) {
      const float* c = px + (size_t(j) * W + i) * 4;
      float weight = float(0.3 * c[0] + 0.6 * c[1] + 0.1 * c[2]);
      rowWeightSum += weight;
      pdf2D[size_t(j) * W + i] = weight;
      cdf2D[size_t(j) * W + i] = rowWeightSum;
    }
    for (int i = 0; i < W; ++i) {
      pdf2D[size_t(j) * W + i] = float(pdf2D[size_t(j) * W + i] / (rowWeightSum + 1e-7));
      cdf2D[size_t(j) * W + i] = float(cdf2D[size_t(j) * W + i] / (rowWeightSum + 1e-7));
    }
    weightSum += rowWeightSum;
    pdf1D[j] = rowWeightSum;
    cdf1D[j] = weightSum;
  }
  for (int j = 0; j < H; ++j) {
    cdf1D[j] = float(cdf1D[j] / (weightSum + 1e-7));
    pdf1D[j] = float(pdf1D[j] / (weightSum + 1e-7));
  }
  auto lowerBound = [](const float* a, int lo, int hi, float v) {
    while (lo < hi) {
      int mid = (lo + hi) / 2;
      if (a[mid] < v)
        lo = mid + 1;
      else
        hi = mid;
    }
    return lo;
  };
  for (int j = 0; j < H; ++j) {
    float invHeight = float(j + 1) / float(H);
    float row = float(lowerBound(cdf1D.data(), 0, H, invHeight));
    marg[size_t(j) * W * 2] = row / float(H);
    marg[size_t(j) * W * 2 + 1] = pdf1D[j];
  }
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      float invWidth = float(i + 1) / float(W);
      float col = float(lowerBound(cdf2D.data(), j * W, (j + 1) * W, invWidth) - j * W);
      cond[(size_t(j) * W + i) * 2] = col / float(W);
      cond[(size_t(j) * W + i) * 2 + 1] = pdf2D[size_t(j) * W + i];
    }
  return ASUNA_OK;
}

// src/loader/material.cpp:290-300 (complexIorListLookup)
int asuna_complex_ior(const char* name, float* eta, float* k) {
  if (!name || !eta || !k) return fail(ASUNA_ERR_INVALID, "asuna_complex_ior: null argument");
  for (const NamedIor& e : kConductorIors)
    if (std::strcmp(e.name, name) == 0) {
      for (int c = 0; c < 3; ++c) {
        eta[c] = e.eta[c];
        k[c] = e.k[c];
      }
      return ASUNA_OK;
    }
  return fail(ASUNA_ERR_PARSE, "unrecognized conductor material [%s]", name);
}

// src/loader/material.cpp:25-37
float asuna_diffuse_fresnel(float ior, int sampleCount) {
  double diffuseFresnel = 0.0;
  float ct;
  float fb = dielectricReflectance(ior, 0.0f, ct);
  for (int i = 1; i <= sampleCount; ++i) {
    float cosThetaSq = float(i) / float(sampleCount);
    float fa = dielectricReflectance(ior, std::min(std::sqrt(cosThetaSq), 1.0f), ct);
    diffuseFresnel += double(fa + fb) * (0.5 / sampleCount);
    fb = fa;
  }
  return float(diffuseFresnel);
}

int asuna_image_write(const char* path, uint32_t width, uint32_t height, const float* rgba) {
  clearError();
  if (!path || !rgba || !width || !height) return fail(ASUNA_ERR_INVALID, "asuna_image_write: bad argument");
  std::string p(path);
  std::string ext = p.substr(p.find_last_of('.') + 1);
  if (ext == "exr") return writeExr(p, width, height, rgba);
  if (ext == "png") return writePng(p, width, height, rgba);
  if (ext == "pfm") return writePfm(p, width, height, rgba);
  return fail(ASUNA_ERR_UNSUPPORTED, "asuna_image_write: .%s (use .exr, .png or .pfm)", ext.c_str());
}

int asuna_image_read(const char* path, uint32_t* width, uint32_t* height, float* rgba, uint64_t capacity) {
  clearError();
  if (!path || !width || !height) return fail(ASUNA_ERR_INVALID, "asuna_image_read: bad argument");
  std::vector<float> px;
  int rc = loadImageRGBA(path, *width, *height, px);
  if (rc) return rc;
  if (rgba) {
    if (capacity < px.size()) return fail(ASUNA_ERR_INVALID, "asuna_image_read: buffer holds %llu of %zu floats",
                                          (unsigned long long)capacity, px.size());
    std::memcpy(rgba, px.data(), px.size() * sizeof(float));
  }
  return ASUNA_OK;
}

int asuna_json_load_string(const char* text, const char* base_dir, asuna_json_scene** out) {
  clearError();
  if (!text || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  asuna_json_scene* js = new (std::nothrow) asuna_json_scene;
  if (!js) return fail(ASUNA_ERR_OOM, "host allocation failed");
  int rc = loadSceneJson(text, base_dir ? base_dir : "", js->scene);
  if (rc) {
    delete js;
    return rc;
  }
  *out = js;
  return ASUNA_OK;
}

int asuna_json_load(const char* path, asuna_json_scene** out) {
  clearError();
  if (!path || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  std::string text;
  if (!readFile(path, text)) return fail(ASUNA_ERR_IO, "failed to load scene from file [%s]", path);
  std::string p(path);
  size_t slash = p.find_last_of('/');
  std::string dir = slash == std::string::npos ? "." : p.substr(0, slash);
  return asuna_json_load_string(text.c_str(), dir.c_str(), out);
}

int asuna_json_free(asuna_json_scene* js) {
  delete js;
  return ASUNA_OK;
}

int asuna_json_scene_desc(const asuna_json_scene* js, asuna_scene_desc* out) {
  if (!js || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  js->scene.desc(out);
  return ASUNA_OK;
}

int asuna_json_num_shots(const asuna_json_scene* js, uint32_t* out) {
  if (!js || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  *out = uint32_t(js->scene.shots.size());
  return ASUNA_OK;
}

int asuna_json_get_shot(const asuna_json_scene* js, uint32_t index, asuna_shot* out) {
  if (!js || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  return js->scene.shot(index, out);
}

int asuna_json_post_state(const asuna_json_scene* js, asuna_post_state* out) {
  if (!js || !out) return fail(ASUNA_ERR_INVALID, "null argument");
  asuna_post_default(out);
  out->tm_type = js->scene.state.toneMapping;
  return ASUNA_OK;
}

int asuna_json_channels(const asuna_json_scene* js, uint32_t* n, int32_t* kinds) {
  if (!js || !n) return fail(ASUNA_ERR_INVALID, "null argument");
  const auto& k = js->scene.state.channelKinds;
  *n = uint32_t(k.size());
  if (kinds)
    for (size_t i = 0; i < k.size(); ++i) kinds[i] = k[i];
  return ASUNA_OK;
}

// Tracer::runOffline + callSavingImage (src/tracer/tracer.cpp:177-291): every
// shot rendered for its spp frames; radiance written as <prefix>_shot_%04d.exr,
// AOV channel c as <prefix>_shot_%04d_channel_%04d.exr (or .png where the
// scene's multi_channel_ldr asks for it).  The reference's LDR radiance output
// goes through its tonemapping post pass, which is outside this path, so the
// radiance is always written as HDR.
int asuna_tracer_run_offline(asuna_ctx* ctx, const char* scene_json, const char* out_prefix) {
  return asuna_tracer_run_offline_scanline(ctx, scene_json, out_prefix, 0);
}

int asuna_tracer_run_offline_scanline(asuna_ctx* ctx, const char* scene_json, const char* out_prefix,
                                      int output_scanline) {
  clearError();
  if (!ctx || !scene_json || !out_prefix) return fail(ASUNA_ERR_INVALID, "null argument");
  asuna_json_scene* js = nullptr;
  int rc = asuna_json_load(scene_json, &js);
  if (rc) return rc;
  std::unique_ptr<asuna_json_scene, int (*)(asuna_json_scene*)> g(js, asuna_json_free);
  asuna_scene_desc d;
  js->scene.desc(&d);
  asuna_scene* scene = nullptr;
  if ((rc = asuna_scene_create(ctx, &d, &scene))) return rc;
  std::unique_ptr<asuna_scene, int (*)(asuna_scene*)> gs(scene, asuna_scene_destroy);
  const HostScene& S = js->scene;
  std::vector<float> px(size_t(S.width) * S.height * 4);
  for (uint32_t i = 0; i < S.shots.size(); ++i) {
    asuna_shot shot;
    if ((rc = S.shot(i, &shot))) return rc;
    asuna_film* film = nullptr;
    if ((rc = asuna_film_create(ctx, S.width, S.height, &film))) return rc;
    std::unique_ptr<asuna_film, int (*)(asuna_film*)> gf(film, asuna_film_destroy);
    if ((rc = asuna_render(ctx, scene, &shot, film, nullptr))) return rc;
    if (!S.state.outputRenderResult) continue;
    char name[64];
    if (S.state.outputHdr) {
      std::snprintf(name, sizeof(name), "_shot_%04u.exr", i);
      if ((rc = asuna_film_read(ctx, film, 0, px.data())) ||
          (rc = writeExr(out_prefix + std::string(name), S.width, S.height, px.data())))
        return rc;
    } else {
      // the post pass's LDR color (tone mapping of the scene file)
      asuna_post_state post;
      if ((rc = asuna_json_post_state(js, &post))) return rc;
      float* dev = nullptr;
      if (cudaMalloc(&dev, px.size() * sizeof(float)) != cudaSuccess)
        return fail(ASUNA_ERR_OOM, "offline output: device allocation failed");
      std::unique_ptr<float, cudaError_t (*)(void*)> gd(dev, cudaFree);
      if ((rc = asuna_tonemap(ctx, film, 0, &post, dev))) return rc;
      cudaStream_t stream = static_cast<cudaStream_t>(asuna_ctx_stream(ctx));
      if (cudaMemcpyAsync(px.data(), dev, px.size() * sizeof(float), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
          cudaStreamSynchronize(stream) != cudaSuccess)
        return fail(ASUNA_ERR_CUDA, "offline output: read-back of the tone-mapped image failed");
      std::snprintf(name, sizeof(name), "_shot_%04u.png", i);
      if ((rc = writePng(out_prefix + std::string(name), S.width, S.height, px.data()))) return rc;
    }
    std::vector<uint32_t> valid;  // scanline mode: pixels whose first channel has .z == 1
    for (uint32_t c = 0; c < S.state.rtx.n_multi_channel; ++c) {
      const bool ldr = c < S.state.channelLdr.size() && S.state.channelLdr[c];
      std::snprintf(name, sizeof(name), "_shot_%04u_channel_%04u.%s", i, c, ldr ? "png" : "exr");
      if ((rc = asuna_film_read(ctx, film, int(c + 1), px.data()))) return rc;
      if (output_scanline) {
        if (c == 0) {
          valid.clear();
          for (uint32_t k = 0; k < S.width * S.height; ++k)
            if (px[size_t(k) * 4 + 2] == 1.0f) {
              valid.push_back(k);
              px[size_t(k) * 4 + 2] = float(k);
            }
        }
        std::vector<float> rows(valid.size() * 3);
        for (size_t k = 0; k < valid.size(); ++k)
          for (int j = 0; j < 3; ++j) rows[k * 3 + j] = px[size_t(valid[k]) * 4 + j];
        rc = writeNpy(out_prefix + std::string(name), uint64_t(valid.size()), 3, rows.data());
      } else {
        rc = ldr ? writePng(out_prefix + std::string(name), S.width, S.height, px.data())
                 : writeExr(out_prefix + std::string(name), S.width, S.height, px.data());
      }
      if (rc) return rc;
    }
  }
  return ASUNA_OK;
}

}  // extern "C"
