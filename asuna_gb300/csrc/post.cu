// post.cu — the tone-mapping post pass of the offline output
// (src/shaders/post.idle.frag:71-133 with utils/tonemapping.glsl), as CUDA
// kernels over a film image: the operators None, Gamma, Reinhard (Hejl /
// Burgess-Dawson), ACES (Narkowicz fit), Filmic, Pbrt (sRGB transfer curve)
// and Custom (auto exposure, Uncharted 2 curve, dithering, contrast,
// brightness, saturation, vignette).  The fragment shader samples the HDR
// image at pixel centres (uv * zoom); Custom's exposure reads the image's
// mip chain (textureLod level 20 = the 1x1 level, texture(.., bias i) =
// level i), here a 2x2 box pyramid.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "common.h"
#include "handles.h"
#include "../../include/asuna_math.h"

namespace asuna {
namespace {

struct Level {
  const float4* p;
  int w, h;
};
constexpr int kMips = 9;  // levels 0..8 (local exposure reads levels 0..7)
struct Pyramid {
  Level l[kMips];
  int n;
};

__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return a * s; }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator+(float3 a, float s) { return make_float3(a.x + s, a.y + s, a.z + s); }
__device__ __forceinline__ float3 operator-(float3 a, float s) { return make_float3(a.x - s, a.y - s, a.z - s); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 max3(float3 a, float s) { return make_float3(fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)); }
__device__ __forceinline__ float3 clamp3(float3 a, float lo, float hi) {
  return make_float3(fminf(fmaxf(a.x, lo), hi), fminf(fmaxf(a.y, lo), hi), fminf(fmaxf(a.z, lo), hi));
}
// the shared transcendentals (include/asuna_math.h), as the CPU oracle
__device__ __forceinline__ float3 pow3(float3 a, float e) {
  return make_float3(asuna_math::powf_(a.x, e), asuna_math::powf_(a.y, e), asuna_math::powf_(a.z, e));
}
// GLSL mix as the specification writes it: x (1 - a) + y a
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float3 t) {
  return make_float3(a.x * (1.0f - t.x) + b.x * t.x, a.y * (1.0f - t.y) + b.y * t.y, a.z * (1.0f - t.z) + b.z * t.z);
}

constexpr float kGamma = 2.2f;
__device__ __forceinline__ float3 linearTosRGB(float3 c) { return pow3(c, 1.0f / kGamma); }
__device__ __forceinline__ float3 sRGBToLinear(float3 c) { return pow3(c, kGamma); }

// luminance of post.idle.frag:40-46 (Rec. 709 weights)
__device__ __forceinline__ float lum709(float3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

// Uncharted 2 filmic curve (J. Hable, "Filmic tonemapping operators", 2010)
__device__ __forceinline__ float3 uncharted2(float3 c) {
  const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
  return ((c * (c * A + C * B) + D * E) / (c * (c * A + B) + D * F)) - E / F;
}
__device__ __forceinline__ float3 toneMapUncharted(float3 c) {
  const float W = 11.2f;
  c = uncharted2(c * 2.0f);
  const float3 white = uncharted2(make_float3(W, W, W));
  return linearTosRGB(c * (make_float3(1.0f, 1.0f, 1.0f) / white));
}
// Hejl / Burgess-Dawson curve (the "reinhard" and "filmic" operators)
__device__ __forceinline__ float3 hejl(float3 c) {
  c = max3(c - 0.004f, 0.0f);
  return (c * (c * 6.2f + 0.5f)) / (c * (c * 6.2f + 1.7f) + 0.06f);
}
// ACES filmic fit (K. Narkowicz, 2016)
__device__ __forceinline__ float3 aces(float3 c) {
  const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
  return linearTosRGB(clamp3((c * (c * A + B)) / (c * (c * C + D) + E), 0.0f, 1.0f));
}
__device__ __forceinline__ float srgbCurve(float c) {
  return c < 0.0031308f ? 12.92f * c : 1.055f * asuna_math::powf_(c, 1.0f / 2.4f) - 0.055f;
}

// PCG3D hash (M. Jarzynski and M. Olano, "Hash functions for GPU
// rendering", JCGT 2020)
__device__ __forceinline__ uint3 pcg3d(uint3 v) {
  v.x = v.x * 1664525u + 1013904223u;
  v.y = v.y * 1664525u + 1013904223u;
  v.z = v.z * 1664525u + 1013904223u;
  v.x += v.y * v.z;
  v.y += v.z * v.x;
  v.z += v.x * v.y;
  v.x ^= v.x >> 16u;
  v.y ^= v.y >> 16u;
  v.z ^= v.z >> 16u;
  v.x += v.y * v.z;
  v.y += v.z * v.x;
  v.z += v.x * v.y;
  return v;
}

// bilinear sample of one level at uv (texel centres at (i + 0.5) / w), edges clamped
__device__ float4 sample(const Level& L, float u, float v) {
  const float x = u * float(L.w) - 0.5f, y = v * float(L.h) - 0.5f;
  const float fx = floorf(x), fy = floorf(y);
  const float tx = x - fx, ty = y - fy;
  auto at = [&](int i, int j) {
    i = min(max(i, 0), L.w - 1);
    j = min(max(j, 0), L.h - 1);
    return L.p[size_t(j) * L.w + i];
  };
  const int i0 = int(fx), j0 = int(fy);
  const float4 a = at(i0, j0), b = at(i0 + 1, j0), c = at(i0, j0 + 1), d = at(i0 + 1, j0 + 1);
  auto lerp4 = [](float4 p, float4 q, float t) {
    return make_float4(p.x + (q.x - p.x) * t, p.y + (q.y - p.y) * t, p.z + (q.z - p.z) * t, p.w + (q.w - p.w) * t);
  };
  return lerp4(lerp4(a, b, tx), lerp4(c, d, tx), ty);
}

// RGB -> XYZ as post.idle.frag:36-37 builds it: the nine values fill the
// GLSL mat3 column by column, so Y = 0.3575761 R + 0.7151522 G + 0.1191920 B
__device__ __forceinline__ float xyzY(float3 c) { return 0.3575761f * c.x + 0.7151522f * c.y + 0.1191920f * c.z; }

__global__ void __launch_bounds__(256) k_tonemap(Pyramid pyr, asuna_post_state tm, float avgLum2, float4* out) {
  const Level& L0 = pyr.l[0];
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= L0.w || y >= L0.h) return;
  const float u = (float(x) + 0.5f) / float(L0.w) * tm.zoom, v = (float(y) + 0.5f) / float(L0.h) * tm.zoom;
  const float4 hdr4 = tm.zoom == 1.0f ? L0.p[size_t(y) * L0.w + x] : sample(L0, u, v);
  const float3 hdr = f3(hdr4);
  float3 c = hdr;
  switch (tm.tm_type) {
    case ASUNA_TONEMAP_NONE:
      break;
    case ASUNA_TONEMAP_GAMMA:
      c = linearTosRGB(hdr / (hdr / 1.5f + 1.0f));
      break;
    case ASUNA_TONEMAP_REINHARD:
    case ASUNA_TONEMAP_FILMIC:
      c = hejl(hdr);
      break;
    case ASUNA_TONEMAP_ACES:
      c = aces(hdr);
      break;
    case ASUNA_TONEMAP_PBRT:
      c = make_float3(srgbCurve(hdr.x), srgbCurve(hdr.y), srgbCurve(hdr.z));
      break;
    default: {  // custom
      float3 h = hdr;
      if (tm.auto_exposure & 1) {
        const float XYZy = xyzY(h);
        const float factor = tm.key / avgLum2;
        const float Y = factor * XYZy;
        if ((tm.auto_exposure >> 1) & 1) {
          // local exposure: the finest mip level whose luminance stays close to the next one
          const float scale[7] = {1, 2, 4, 8, 16, 32, 64};
          const float epsilon = 0.05f, phi = 2.0f;
          float La = 0.0f;
          for (int i = 0; i < 7; ++i) {
            const Level& a = pyr.l[min(i, pyr.n - 1)];
            const Level& b = pyr.l[min(i + 1, pyr.n - 1)];
            const float v1 = lum709(f3(sample(a, u, v))) * factor;
            const float v2 = lum709(f3(sample(b, u, v))) * factor;
            if (fabsf(v1 - v2) / ((tm.key * asuna_math::powf_(2.0f, phi) / (scale[i] * scale[i])) + v1) > epsilon) {
              La = v1;
              break;
            }
            La = v2;
          }
          h = h / XYZy * (Y / (1.0f + La));
        } else {
          const float Yd = (Y * (1.0f + Y / (tm.y_white * tm.y_white))) / (1.0f + Y);
          h = h / XYZy * Yd;
        }
      }
      float3 col = toneMapUncharted(h * tm.avg_lum);
      // dithering against banding (http://www.thetenthplanet.de/archives/5367)
      const uint3 r = pcg3d(make_uint3(uint32_t(x), uint32_t(y), 0u));
      const float3 noise = make_float3(__uint_as_float(0x3f800000u | (r.x >> 9)) - 1.0f,
                                       __uint_as_float(0x3f800000u | (r.y >> 9)) - 1.0f,
                                       __uint_as_float(0x3f800000u | (r.z >> 9)) - 1.0f);
      {
        const float quant = 1.0f / 255.0f;
        const float3 lin = sRGBToLinear(col);
        const float3 s = linearTosRGB(lin);
        const float3 c0 = make_float3(floorf(s.x / quant) * quant, floorf(s.y / quant) * quant,
                                      floorf(s.z / quant) * quant);
        const float3 c1 = c0 + quant;
        const float3 discr = mix3(sRGBToLinear(c0), sRGBToLinear(c1), noise);
        col = make_float3(discr.x < lin.x ? c1.x : c0.x, discr.y < lin.y ? c1.y : c0.y, discr.z < lin.z ? c1.z : c0.z);
      }
      col = clamp3(mix3(make_float3(0.5f, 0.5f, 0.5f), col, tm.contrast), 0.0f, 1.0f);
      col = pow3(col, 1.0f / tm.brightness);
      const float gray = col.x * 0.299f + col.y * 0.587f + col.z * 0.114f;
      col = mix3(make_float3(gray, gray, gray), col, tm.saturation);
      const float vx = ((float(x) + 0.5f) / float(L0.w) * tm.rendering_ratio[0] - 0.5f) * 2.0f;
      const float vy = ((float(y) + 0.5f) / float(L0.h) * tm.rendering_ratio[1] - 0.5f) * 2.0f;
      col = col * (1.0f - (vx * vx + vy * vy) * tm.vignette);
      c = col;
    }
  }
  out[size_t(y) * L0.w + x] = make_float4(c.x, c.y, c.z, hdr4.w);
}

// next mip level: 2x2 box (odd edges clamp)
__global__ void k_mip(const float4* in, int w, int h, float4* out, int w2, int h2) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w2 || y >= h2) return;
  const int x0 = min(2 * x, w - 1), x1 = min(2 * x + 1, w - 1), y0 = min(2 * y, h - 1), y1 = min(2 * y + 1, h - 1);
  const float4 a = in[size_t(y0) * w + x0], b = in[size_t(y0) * w + x1], c = in[size_t(y1) * w + x0],
               d = in[size_t(y1) * w + x1];
  out[size_t(y) * w2 + x] = make_float4(0.25f * (a.x + b.x + c.x + d.x), 0.25f * (a.y + b.y + c.y + d.y),
                                        0.25f * (a.z + b.z + c.z + d.z), 0.25f * (a.w + b.w + c.w + d.w));
}

// mean RGB of the image (the 1x1 mip level): per-block partial sums in double
__global__ void k_mean(const float4* in, size_t n, double* sum) {
  double s[3] = {0, 0, 0};
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float4 v = in[i];
    s[0] += v.x;
    s[1] += v.y;
    s[2] += v.z;
  }
  for (int k = 0; k < 3; ++k) {
    for (int off = 16; off; off >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sum[k], s[k]);
  }
}

}  // namespace
}  // namespace asuna

using namespace asuna;

extern "C" {

void asuna_post_default(asuna_post_state* p) {
  if (!p) return;
  // PipelineState::PipelineState, src/core/state.h:46-58
  p->brightness = 1.0f;
  p->contrast = 1.0f;
  p->saturation = 1.0f;
  p->vignette = 0.0f;
  p->avg_lum = 1.0f;
  p->zoom = 1.0f;
  p->rendering_ratio[0] = p->rendering_ratio[1] = 1.0f;
  p->auto_exposure = 0;
  p->y_white = 0.5f;
  p->key = 0.5f;
  p->tm_type = ASUNA_TONEMAP_FILMIC;
}

int asuna_tonemap(asuna_ctx* c, asuna_film* f, int image, const asuna_post_state* post, float* out) {
  clearError();
  if (!c || !f || !post || !out) return fail(ASUNA_ERR_INVALID, "asuna_tonemap: null argument");
  if (image < 0 || image >= ASUNA_NUM_OUTPUT_IMAGES) return fail(ASUNA_ERR_INVALID, "image %d out of range", image);
  if (post->tm_type >= ASUNA_TONEMAP_NUM) return fail(ASUNA_ERR_INVALID, "tone mapping type %u", post->tm_type);
  ASUNA_CUDA_TRY(cudaSetDevice(c->device));
  const size_t np = size_t(f->width) * f->height;
  const float4* src = image == 0 ? f->rad : (image == 8 ? f->w : f->ch + size_t(image - 1) * np);
  Pyramid pyr{};
  pyr.l[0] = {src, int(f->width), int(f->height)};
  pyr.n = 1;
  std::vector<void*> tmp;
  auto cleanup = [&] {
    for (void* p : tmp) cudaFreeAsync(p, c->stream);
  };
  float avgLum2 = 1.0f;
  const bool custom = post->tm_type == ASUNA_TONEMAP_CUSTOM && (post->auto_exposure & 1);
  if (custom) {
    double* sum = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&sum), 3 * sizeof(double), c->stream) != cudaSuccess)
      return fail(ASUNA_ERR_OOM, "asuna_tonemap: allocation failed");
    tmp.push_back(sum);
    cudaMemsetAsync(sum, 0, 3 * sizeof(double), c->stream);
    k_mean<<<int(std::min<size_t>((np + 255) / 256, 1024)), 256, 0, c->stream>>>(src, np, sum);
    double h[3];
    cudaMemcpyAsync(h, sum, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
      cleanup();
      return fail(ASUNA_ERR_CUDA, "asuna_tonemap: %s", cudaGetErrorString(cudaGetLastError()));
    }
    const float mean[3] = {float(h[0] / double(np)), float(h[1] / double(np)), float(h[2] / double(np))};
    avgLum2 = mean[0] * 0.2126f + mean[1] * 0.7152f + mean[2] * 0.0722f;
    if ((post->auto_exposure >> 1) & 1) {
      for (int lv = 1; lv < kMips; ++lv) {
        const Level& p = pyr.l[lv - 1];
        if (p.w == 1 && p.h == 1) break;
        const int w2 = std::max(1, p.w / 2), h2 = std::max(1, p.h / 2);
        float4* q = nullptr;
        if (cudaMallocAsync(reinterpret_cast<void**>(&q), size_t(w2) * h2 * 16, c->stream) != cudaSuccess) {
          cleanup();
          return fail(ASUNA_ERR_OOM, "asuna_tonemap: allocation failed");
        }
        tmp.push_back(q);
        k_mip<<<dim3((w2 + 255) / 256, h2), 256, 0, c->stream>>>(p.p, p.w, p.h, q, w2, h2);
        pyr.l[lv] = {q, w2, h2};
        pyr.n = lv + 1;
      }
    }
  }
  k_tonemap<<<dim3((f->width + 255) / 256, f->height), 256, 0, c->stream>>>(pyr, *post, avgLum2,
                                                                           reinterpret_cast<float4*>(out));
  const cudaError_t e = cudaGetLastError();
  cleanup();
  if (e != cudaSuccess) return fail(ASUNA_ERR_CUDA, "asuna_tonemap: %s", cudaGetErrorString(e));
  return ASUNA_OK;
}

}  // extern "C"
