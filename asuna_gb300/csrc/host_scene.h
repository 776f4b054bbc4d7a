// host_scene.h — host-side scene description: the Scene / Loader / Camera /
// EnvMap logic of the reference (src/scene/, src/loader/, src/core/) that
// assembles the device-ABI arrays the render path consumes.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/asuna_rt.h"

namespace asuna {

int validateSceneDesc(const asuna_scene_desc* d);
// world->object of an object->world 3x4 (row-major): double inverse, rounded once.
void invert3x4(const float* m, float* out);

// Pipeline state of one shot (src/core/state.h:15-63 plus the depth channel).
struct HostState {
  asuna_rt_state rtx{};
  int32_t depthSlot = -1;
  uint32_t toneMapping = 4;  // ToneMappingTypeFilmic
  bool outputHdr = false;
  bool outputRenderResult = true;
  std::vector<bool> channelLdr;
  std::vector<int32_t> channelKinds;
  HostState();
};

struct HostShot {
  float eye[3], lookat[3], up[3];
  float envTransform[16];
  HostState state;
};

struct HostMesh {
  std::string name;
  std::vector<asuna_vertex> v;
  std::vector<uint32_t> idx;
};

struct HostScene {
  // camera (src/loader/loader.cpp:242-268)
  uint32_t camType = ASUNA_CAMERA_PERSPECTIVE;
  uint32_t width = 0, height = 0;
  float fov = 45.0f, aperture = 0.0f, focalDistance = 0.1f;
  float fxfycxcy[4] = {0, 0, 0, 0};
  HostState state;
  std::vector<HostMesh> meshes;
  std::vector<std::string> materialNames, textureNames;
  std::vector<asuna_material> materials;
  std::vector<asuna_light> lights;
  std::vector<asuna_instance_desc> instances;
  std::vector<HostShot> shots;
  uint32_t envW = 0, envH = 0;
  std::vector<float> env;
  struct Texture {
    uint32_t w = 1, h = 1;
    std::vector<float> rgba;
  };
  std::vector<Texture> textures;  // parallel to textureNames
  // views for asuna_scene_desc
  std::vector<asuna_mesh_desc> meshDescs;
  std::vector<asuna_texture_desc> texDescs;

  void reset();
  int addLight(const asuna_light& l);
  int addMeshLight(const asuna_light& l, const std::vector<asuna_vertex>& v, const std::vector<uint32_t>& idx);
  int materialId(const std::string& name) const;
  int meshId(const std::string& name) const;
  void submit();  // numLights, autofit shot, descriptor views
  void desc(asuna_scene_desc* out) const;
  int shot(uint32_t i, asuna_shot* out) const;
};

// File loaders.
int loadObj(const std::string& path, std::vector<asuna_vertex>& v, std::vector<uint32_t>& idx);
int loadImageRGBA(const std::string& path, uint32_t& w, uint32_t& h, std::vector<float>& rgba);
int writePfm(const std::string& path, uint32_t w, uint32_t h, const float* rgba);
int writeExr(const std::string& path, uint32_t w, uint32_t h, const float* rgba);
int writePng(const std::string& path, uint32_t w, uint32_t h, const float* rgba);
int writeNpy(const std::string& path, uint64_t rows, uint32_t cols, const float* data);

// Scene-file loader (src/loader/loader.cpp:67-468, src/loader/material.cpp).
int loadSceneJson(const std::string& text, const std::string& baseDir, HostScene& scene);

}  // namespace asuna
