// post_harness.cpp — runs the reference's post-pass fragment shader on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Includes src/shaders/post.idle.frag (with
// utils/tonemapping.glsl and utils/random.glsl) as translated by
// oracle/gen_ref.py into oracle/_ref/gen/, and supplies what the graphics
// pipeline gives the shader: the input image sampler (inImage, mip-mapped),
// the push constant (tm, GpuPushConstantPost), the interpolated uvCoords of
// the full-screen triangle (post.idle.vert), gl_FragCoord and the output
// fragColor.  One invocation per pixel: gl_FragCoord = (x + 0.5, y + 0.5),
// uvCoords = gl_FragCoord / (width, height).
//
// The sampler's filtering and the mip chain are the graphics driver's, not
// the shader's: here they are the oracle's (bilinear with clamp to edge, each
// level a 2x2 box average of the one below), so the comparison with the
// oracle's restatement (oracle_tonemap) tests the shader's own arithmetic.
// Built into oracle/_ref/libasuna_ref.so by oracle/build_oracle.py.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "asuna_oracle.h"
#include "glsl_shim.h"
#include <shared/binding.h>
#include <shared/pushconstant.h>

static_assert(sizeof(GpuPushConstantPost) == sizeof(asuna_post_state), "GpuPushConstantPost layout");

namespace glslx {
namespace postfx {

// The input image with its mip chain (2x2 box levels), and the image's mean
// for a read past the chain's end (textureLod at level 20: the exposure's
// average, which the oracle and the GPU take as the exact mean).
struct MipImage {
  struct Level {
    std::vector<float> p;  // RGBA
    int w, h;
  };
  std::vector<Level> lv;
  vec4 mean;
};

inline vec4 sampleLevel(const MipImage::Level& L, vec2 uv) {
  const float x = uv.x * float(L.w) - 0.5f, y = uv.y * float(L.h) - 0.5f;
  const float fx = std::floor(x), fy = std::floor(y), tx = x - fx, ty = y - fy;
  auto at = [&](int i, int j, int c) {
    i = std::min(std::max(i, 0), L.w - 1);
    j = std::min(std::max(j, 0), L.h - 1);
    return L.p[(size_t(j) * L.w + i) * 4 + c];
  };
  const int i0 = int(fx), j0 = int(fy);
  float r[4];
  for (int c = 0; c < 4; ++c) {
    const float a = at(i0, j0, c), b = at(i0 + 1, j0, c), cc = at(i0, j0 + 1, c), d = at(i0 + 1, j0 + 1, c);
    const float p = a + (b - a) * tx, q = cc + (d - cc) * tx;
    r[c] = p + (q - p) * ty;
  }
  return vec4(r[0], r[1], r[2], r[3]);
}
// texture(): the base level (a full-screen pass at the image's size has
// implicit level 0); with a bias, that level; textureLod: that level, capped
inline vec4 texture(const MipImage& m, vec2 uv) { return sampleLevel(m.lv[0], uv); }
inline vec4 texture(const MipImage& m, vec2 uv, int bias) {
  return sampleLevel(m.lv[std::min<size_t>(size_t(std::max(bias, 0)), m.lv.size() - 1)], uv);
}
inline vec4 textureLod(const MipImage& m, vec2 uv, int lod) {
  return size_t(lod) >= m.lv.size() ? m.mean : texture(m, uv, lod);
}

struct FragOut {
  vec3 c;
  float a = 0.0f;
  vec3& rgb() { return c; }
  float& r() { return c.x; }
};

static MipImage inImage;
static GpuPushConstantPost tm;
static vec2 uvCoords;
static vec4 gl_FragCoord;
static FragOut fragColor;

#include "post.idle.frag.h"

}  // namespace postfx
}  // namespace glslx

extern "C" {

// The reference's post.idle.frag over a whole image (width x height RGBA);
// writes the fragment colours (RGBA) into `out`.
int ref_post(const float* rgba, uint32_t w, uint32_t h, const asuna_post_state* post, float* out) {
  using namespace glslx::postfx;
  if (!rgba || !post || !out || !w || !h) return ASUNA_ERR_INVALID;
  inImage.lv.clear();
  inImage.lv.push_back({std::vector<float>(rgba, rgba + size_t(w) * h * 4), int(w), int(h)});
  while (!(inImage.lv.back().w == 1 && inImage.lv.back().h == 1)) {
    const MipImage::Level& p = inImage.lv.back();
    MipImage::Level q{{}, std::max(1, p.w / 2), std::max(1, p.h / 2)};
    q.p.resize(size_t(q.w) * q.h * 4);
    for (int y = 0; y < q.h; ++y)
      for (int x = 0; x < q.w; ++x) {
        const int x0 = std::min(2 * x, p.w - 1), x1 = std::min(2 * x + 1, p.w - 1);
        const int y0 = std::min(2 * y, p.h - 1), y1 = std::min(2 * y + 1, p.h - 1);
        for (int c = 0; c < 4; ++c)
          q.p[(size_t(y) * q.w + x) * 4 + c] =
              0.25f * (p.p[(size_t(y0) * p.w + x0) * 4 + c] + p.p[(size_t(y0) * p.w + x1) * 4 + c] +
                       p.p[(size_t(y1) * p.w + x0) * 4 + c] + p.p[(size_t(y1) * p.w + x1) * 4 + c]);
      }
    inImage.lv.push_back(std::move(q));
  }
  {
    double sum[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < size_t(w) * h; ++i)
      for (int c = 0; c < 4; ++c) sum[c] += rgba[i * 4 + c];
    const double n = double(size_t(w) * h);
    inImage.mean = glslx::vec4(float(sum[0] / n), float(sum[1] / n), float(sum[2] / n), float(sum[3] / n));
  }
  std::memcpy(&tm, post, sizeof(tm));
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      gl_FragCoord = glslx::vec4(float(x) + 0.5f, float(y) + 0.5f, 0.0f, 1.0f);
      uvCoords = glslx::vec2((float(x) + 0.5f) / float(w), (float(y) + 0.5f) / float(h));
      fragColor = FragOut{};
      stage_post::main();
      float* o = out + (size_t(y) * w + x) * 4;
      o[0] = fragColor.c.x;
      o[1] = fragColor.c.y;
      o[2] = fragColor.c.z;
      o[3] = fragColor.a;
    }
  return ASUNA_OK;
}

}  // extern "C"
