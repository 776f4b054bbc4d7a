// dev_math.cuh — device math of the path integrator.
//
// Restates, per function, the reference's GLSL (src/shaders/utils/math.glsl,
// sample_light.glsl, rchit_layouts.glsl and the three in-scope bxdf/*.rchit)
// with the same operation order.  The translation unit that includes this is
// compiled with -fmad=false, so every + - * / sqrt rounds as the GLSL source
// spells it; transcendental functions are CUDA's.
#pragma once
#include <cstdint>

#include "../../include/asuna_math.h"
#include "../../include/asuna_sunsky.h"
#include "dev_types.h"

namespace asuna {
namespace dm {

struct f3 {
  float x, y, z;
};
struct f2 {
  float x, y;
};

__device__ __forceinline__ f3 mk(float a, float b, float c) { return f3{a, b, c}; }
__device__ __forceinline__ f3 splat(float a) { return f3{a, a, a}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) {
  float l = length(a);
  return {a.x / l, a.y / l, a.z / l};
}
__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ float gsign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ f3 reflect(f3 I, f3 N) { return I - 2.0f * dot(N, I) * N; }
__device__ __forceinline__ f3 refract(f3 I, f3 N, float eta) {
  float d = dot(N, I);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return splat(0.0f);
  return eta * I - (eta * d + sqrtf(k)) * N;
}
__device__ __forceinline__ f3 ld3(float4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ f3 ld3(const float* a) { return {a[0], a[1], a[2]}; }

// Transcendentals: the shared implementation of include/asuna_math.h, so the
// CPU oracle computes the same bits.
__device__ __forceinline__ float msin(float x) { return asuna_math::sinf_(x); }
__device__ __forceinline__ float mcos(float x) { return asuna_math::cosf_(x); }
__device__ __forceinline__ float macos(float x) { return asuna_math::acosf_(x); }
__device__ __forceinline__ float mpow(float x, float y) { return asuna_math::powf_(x, y); }
__device__ __forceinline__ float mlog(float x) { return asuna_math::logf_(x); }
__device__ __forceinline__ float matan2(float y, float x) { return asuna_math::atan2f_(y, x); }
__device__ __forceinline__ float mexp(float x) { return asuna_math::expf_(x); }

constexpr float PI = 3.14159265358979323846f;
constexpr float TWO_PI = 6.28318530717958647692f;
constexpr float INV_PI = 0.31830988618379067154f;
constexpr float INV_2PI = 0.15915494309189533577f;
constexpr float INV_4PI = 0.07957747154594766788f;
constexpr float PI_OVER_2 = 1.57079632679489661923f;
constexpr float PI_OVER_4 = 0.78539816339744830961f;
constexpr float EPS = 0.001f;
constexpr float INF = 10000000000.0f;
constexpr float MINIMUM = 0.00001f;

// structs.glsl:7-20
enum : uint32_t {
  EBsdfNull = 0,
  EDiffuseReflection = 1,
  EGlossyReflection = 4,
  ESpecularReflection = 16,
  ESpecularTransmission = 32,
  ESmooth = 1 | 2 | 4 | 8,
  EDelta = 1,
  EArea = 2
};
__device__ __forceinline__ bool isNonSpecular(uint32_t f) { return (f & ESmooth) != 0; }

// math.glsl:20-30
__host__ __device__ __forceinline__ uint32_t xxhash32(uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t p0 = 2246822519u, p1 = 3266489917u, p2 = 668265263u, p3 = 374761393u;
  uint32_t h = z + p3 + x * p1;
  h = p2 * ((h << 17) | (h >> 15));
  h += y * p1;
  h = p2 * ((h << 17) | (h >> 15));
  h = p0 * (h ^ (h >> 15));
  h = p1 * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
// math.glsl:34-44
__device__ __forceinline__ uint32_t pcg(uint32_t& state) {
  uint32_t prev = state * 747796405u + 2891336453u;
  uint32_t word = ((prev >> ((prev >> 28u) + 4u)) ^ prev) * 277803737u;
  state = prev;
  return (word >> 22u) ^ word;
}
__device__ __forceinline__ float rnd(uint32_t& s) { return __uint2float_rn(pcg(s)) * 2.3283064365386963e-10f; }
__device__ __forceinline__ f2 rnd2(uint32_t& s) {
  float a = rnd(s);
  float b = rnd(s);
  return f2{a, b};
}
__host__ __device__ __forceinline__ uint32_t hashFrame(uint32_t frame, uint32_t seed) {
  return frame + seed * 0x9E3779B9u;
}

// math.glsl:58-66 (matrices column-major, m[c*4+r])
__device__ __forceinline__ f3 makeNormal(f3 n) {
  if (length(n) == 0.0f) return n;
  return normalize(n);
}
__device__ __forceinline__ void mat4mul(const float* m, float x, float y, float z, float w, float o[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) o[r] = m[0 * 4 + r] * x + m[1 * 4 + r] * y + m[2 * 4 + r] * z + m[3 * 4 + r] * w;
}
__device__ __forceinline__ void mat4Tmul(const float* m, float x, float y, float z, float w, float o[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) o[r] = m[r * 4 + 0] * x + m[r * 4 + 1] * y + m[r * 4 + 2] * z + m[r * 4 + 3] * w;
}
__device__ __forceinline__ f3 transformPoint(const float* m, f3 p) {
  float o[4];
  mat4mul(m, p.x, p.y, p.z, 1.0f, o);
  return {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
}
__device__ __forceinline__ f3 transformDirection(const float* m, f3 d) {
  float o[4];
  mat4mul(m, d.x, d.y, d.z, 0.0f, o);
  return makeNormal(f3{o[0], o[1], o[2]});
}
__device__ __forceinline__ f3 transformDirectionT(const float* m, f3 d) {
  float o[4];
  mat4Tmul(m, d.x, d.y, d.z, 0.0f, o);
  return makeNormal(f3{o[0], o[1], o[2]});
}
// math.glsl:148-174
__device__ __forceinline__ f2 concentricSampleDisk(f2 u) {
  float ox = 2.0f * u.x - 1.0f, oy = 2.0f * u.y - 1.0f;
  if (ox == 0.0f && oy == 0.0f) return f2{0.0f, 0.0f};
  float theta, r;
  if (fabsf(ox) > fabsf(oy)) {
    r = ox;
    theta = PI_OVER_4 * (oy / ox);
  } else {
    r = oy;
    theta = PI_OVER_2 - PI_OVER_4 * (ox / oy);
  }
  return f2{r * mcos(theta), r * msin(theta)};
}
__device__ __forceinline__ f3 cosineSampleHemisphere(f2 u) {
  f2 d = concentricSampleDisk(u);
  float z = sqrtf(gmax(0.0f, 1.0f - d.x * d.x - d.y * d.y));
  return {d.x, d.y, z};
}
__device__ __forceinline__ float cosineHemispherePdf(float c) { return c <= 0.0f ? 0.0f : c * INV_PI; }
// math.glsl:184-189
__device__ __forceinline__ float powerHeuristic(float a, float b) {
  a = a * a;
  b = b * b + a;
  if (b == 0.0f) return 0.0f;
  return a / b;
}
// math.glsl:199-216
__device__ __forceinline__ void basis(f3 n, f3& f, f3& r) {
  if (n.z < -0.999999f) {
    f = {0.0f, -1.0f, 0.0f};
    r = {-1.0f, 0.0f, 0.0f};
  } else {
    float a = 1.0f / (1.0f + n.z);
    float b = -n.x * n.y * a;
    f = {1.0f - n.x * n.x * a, b, -n.x};
    r = {b, 1.0f - n.y * n.y * a, -n.y};
  }
}
__device__ __forceinline__ f3 toWorld(f3 X, f3 Y, f3 Z, f3 v) { return v.x * X + v.y * Y + v.z * Z; }
__device__ __forceinline__ f3 toLocal(f3 X, f3 Y, f3 Z, f3 v) { return {dot(v, X), dot(v, Y), dot(v, Z)}; }
// math.glsl:241-266
__device__ __forceinline__ float offsetComp(float p, float n) {
  int32_t ofi = __float2int_rz(256.0f * n);
  int32_t bits = __float_as_int(p);
  bits += (p < 0.0f) ? -ofi : ofi;
  float pi = __int_as_float(bits);
  return fabsf(p) < (1.0f / 32.0f) ? p + (1.0f / 65536.0f) * n : pi;
}
__device__ __forceinline__ f3 offsetPositionAlongNormal(f3 p, f3 n) {
  return {offsetComp(p.x, n.x), offsetComp(p.y, n.y), offsetComp(p.z, n.z)};
}
// sun_and_sky.glsl:29-31
__device__ __forceinline__ float luminance(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// Bilinear REPEAT fetch at the base level (the reference's env samplers).
__device__ __forceinline__ int wrapIndex(int i, int n) {
  // REPEAT: i mod n in [0, n); the common in-range case costs one compare
  if (unsigned(i) >= unsigned(n)) {
    i %= n;
    if (i < 0) i += n;
  }
  return i;
}
__device__ __forceinline__ void texCoords(int w, int h, float u, float v, int& i0, int& i1, int& j0, int& j1, float& a,
                                          float& b) {
  float x = u * float(w) - 0.5f, y = v * float(h) - 0.5f;
  float fx0 = floorf(x), fy0 = floorf(y);
  a = x - fx0;
  b = y - fy0;
  const int ii = __float2int_rd(fx0), jj = __float2int_rd(fy0);
  i0 = wrapIndex(ii, w);
  i1 = wrapIndex(ii + 1, w);
  j0 = wrapIndex(jj, h);
  j1 = wrapIndex(jj + 1, h);
}
__device__ __forceinline__ float blerp(float a, float b, float t00, float t10, float t01, float t11) {
  return (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
}
__device__ __forceinline__ f2 tex2(const float2* t, int w, int h, float u, float v) {
  int i0, i1, j0, j1;
  float a, b;
  texCoords(w, h, u, v, i0, i1, j0, j1, a, b);
  float2 t00 = __ldg(t + size_t(j0) * w + i0), t10 = __ldg(t + size_t(j0) * w + i1);
  float2 t01 = __ldg(t + size_t(j1) * w + i0), t11 = __ldg(t + size_t(j1) * w + i1);
  return f2{blerp(a, b, t00.x, t10.x, t01.x, t11.x), blerp(a, b, t00.y, t10.y, t01.y, t11.y)};
}
__device__ __forceinline__ f3 tex4rgb(const float4* t, int w, int h, float u, float v) {
  int i0, i1, j0, j1;
  float a, b;
  texCoords(w, h, u, v, i0, i1, j0, j1, a, b);
  float4 t00 = __ldg(t + size_t(j0) * w + i0), t10 = __ldg(t + size_t(j0) * w + i1);
  float4 t01 = __ldg(t + size_t(j1) * w + i0), t11 = __ldg(t + size_t(j1) * w + i1);
  return f3{blerp(a, b, t00.x, t10.x, t01.x, t11.x), blerp(a, b, t00.y, t10.y, t01.y, t11.y),
            blerp(a, b, t00.z, t10.z, t01.z, t11.z)};
}

// math.glsl:134-139
__device__ __forceinline__ f3 uniformSampleSphere(f2 u) {
  float z = 1.0f - 2.0f * u.x;
  float r = sqrtf(gmax(0.0f, 1.0f - z * z));
  float phi = TWO_PI * u.y;
  return f3{r * mcos(phi), r * msin(phi), z};
}
// sun_and_sky.glsl:405-533 (include/asuna_sunsky.h) in world direction L
__device__ __noinline__ f3 evalSunSky(const SceneDev& S, f3 L) {
  const asuna_sky::Params<float> p = asuna_sky::paramsOf<float>(S.sky);
  const asuna_sky::V<float> r = asuna_sky::sunAndSky<float>(p, asuna_sky::V<float>{L.x, L.y, L.z});
  return f3{r.x, r.y, r.z};
}
// sample_light.glsl:84-95
__device__ __forceinline__ float pdfEnvmap(const SceneDev& S, const ShotDev& sh, f3 L) {
  L = transformDirectionT(sh.cam.env_transform, L);
  float theta = macos(gclamp(L.y, -1.0f, 1.0f));
  float u = (PI + matan2(L.z, L.x)) * INV_2PI, v = theta * INV_PI;
  f2 c = tex2(S.cond, S.envW, S.envH, u, v);
  f2 m = tex2(S.marg, S.envW, S.envH, 0.0f, v);
  float pdf = c.y * m.y;
  float sinTheta = msin(theta);
  if (sinTheta == 0.0f) return 0.0f;
  return (pdf * sh.state.env_map_resolution[0] * sh.state.env_map_resolution[1]) / (TWO_PI * PI * sinTheta);
}
// sample_light.glsl:97-104
__device__ __forceinline__ f3 evalEnvmap(const SceneDev& S, const ShotDev& sh, f3 L) {
  L = transformDirectionT(sh.cam.env_transform, L);
  float theta = macos(gclamp(L.y, -1.0f, 1.0f));
  float u = (PI + matan2(L.z, L.x)) * INV_2PI, v = theta * INV_PI;
  f3 e = tex4rgb(S.env, S.envW, S.envH, u, v);
  float k = sh.state.env_map_intensity;
  return f3{k * e.x, k * e.y, k * e.z};
}
// sample_light.glsl:106-129
__device__ __forceinline__ f3 sampleEnvmap(const SceneDev& S, const ShotDev& sh, f2 r, f3& L, float& pdf) {
  f2 m = tex2(S.marg, S.envW, S.envH, 0.0f, r.x);
  float uvy = m.x;
  f2 c = tex2(S.cond, S.envW, S.envH, r.y, uvy);
  float uvx = c.x;
  c = tex2(S.cond, S.envW, S.envH, uvx, uvy);
  m = tex2(S.marg, S.envW, S.envH, 0.0f, uvy);
  pdf = c.y * m.y;
  float phi = uvx * TWO_PI;
  float theta = uvy * PI;
  if (msin(theta) == 0.0f) pdf = 0.0f;
  pdf = (pdf * sh.state.env_map_resolution[0] * sh.state.env_map_resolution[1]) / (TWO_PI * PI * msin(theta));
  L = f3{-msin(theta) * mcos(phi), mcos(theta), -msin(theta) * msin(phi)};
  L = transformDirection(sh.cam.env_transform, L);
  f3 e = tex4rgb(S.env, S.envW, S.envH, uvx, uvy);
  float k = sh.state.env_map_intensity;
  return f3{k * e.x, k * e.y, k * e.z};
}

struct LRec {
  f3 d, n;
  float dist, pdf;
  uint32_t flags;
};

// sample_light.glsl:10-82
__device__ __forceinline__ f3 sampleOneLight(f2 r, const LightDev& l, f3 P, LRec& rec) {
  const int type = __float_as_int(l.pos.w);
  if (type == ASUNA_LIGHT_RECT || type == ASUNA_LIGHT_TRIANGLE) {
    float r1 = r.x, r2 = (type == ASUNA_LIGHT_TRIANGLE) ? (1.0f - r1) * r.y : r.y;
    f3 U = ld3(l.u), V = ld3(l.v);
    f3 pos = ld3(l.pos) + U * r1 + V * r2;
    rec.d = pos - P;
    rec.dist = length(rec.d);
    float distSq = rec.dist * rec.dist;
    rec.d = rec.d / rec.dist;
    rec.n = makeNormal(cross(U, V));
    rec.pdf = distSq / (l.u.w * fabsf(dot(rec.n, rec.d)) + EPS);
    rec.flags = EArea;
    return ld3(l.rad);
  } else if (type == ASUNA_LIGHT_DIRECTIONAL) {
    rec.d = makeNormal(ld3(l.dir));
    rec.n = -rec.d;
    rec.dist = INF;
    rec.pdf = 1.0f;
    rec.flags = EDelta;
    return ld3(l.rad);
  } else if (type == ASUNA_LIGHT_POINT) {
    rec.d = ld3(l.pos) - P;
    rec.n = -rec.d;
    rec.dist = length(rec.d);
    float distSq = rec.dist * rec.dist;
    rec.d = rec.d / (rec.dist + EPS);
    rec.pdf = 1.0f;
    rec.flags = EDelta;
    return ld3(l.rad) / (distSq + EPS);
  }
  return splat(0.0f);
}

// brdf_rough_plastic.rchit:12-80
__device__ __forceinline__ float fresnelDielectricExt(float cosThetaI_, float& cosThetaT_, float eta) {
  if (eta == 1.0f) {
    cosThetaT_ = -cosThetaI_;
    return 0.0f;
  }
  float scale = (cosThetaI_ > 0.0f) ? 1.0f / eta : eta;
  float cosThetaTSqr = 1.0f - (1.0f - cosThetaI_ * cosThetaI_) * (scale * scale);
  if (cosThetaTSqr <= 0.0f) {
    cosThetaT_ = 0.0f;
    return 1.0f;
  }
  float cosThetaI = fabsf(cosThetaI_);
  float cosThetaT = sqrtf(cosThetaTSqr);
  float Rs = (cosThetaI - eta * cosThetaT) / (cosThetaI + eta * cosThetaT);
  float Rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  cosThetaT_ = (cosThetaI_ > 0.0f) ? -cosThetaT : cosThetaT;
  return 0.5f * (Rs * Rs + Rp * Rp);
}
__device__ __forceinline__ float sqr(float x) { return x * x; }
// Conductor Fresnel reflectance (P. Shirley, "Physically based lighting
// calculations for computer graphics", 1991), brdf_conductor.rchit:14-36
__device__ __forceinline__ float conductorReflectance(float eta, float k, float cosThetaI) {
  const float cosThetaISq = cosThetaI * cosThetaI;
  const float sinThetaISq = fmaxf(1.0f - cosThetaISq, 0.0f);
  const float sinThetaIQu = sinThetaISq * sinThetaISq;
  const float innerTerm = eta * eta - k * k - sinThetaISq;
  const float aSqPlusBSq = sqrtf(fmaxf(innerTerm * innerTerm + 4.0f * eta * eta * k * k, 0.0f));
  const float a = sqrtf(fmaxf((aSqPlusBSq + innerTerm) * 0.5f, 0.0f));
  const float Rs = ((aSqPlusBSq + cosThetaISq) - (2.0f * a * cosThetaI)) /
                   ((aSqPlusBSq + cosThetaISq) + (2.0f * a * cosThetaI));
  const float Rp = ((cosThetaISq * aSqPlusBSq + sinThetaIQu) - (2.0f * a * cosThetaI * sinThetaISq)) /
                   ((cosThetaISq * aSqPlusBSq + sinThetaIQu) + (2.0f * a * cosThetaI * sinThetaISq));
  return 0.5f * (Rs + Rs * Rp);
}
__device__ __forceinline__ f3 conductorReflectance3(f3 eta, f3 k, float cosThetaI) {
  return {conductorReflectance(eta.x, k.x, cosThetaI), conductorReflectance(eta.y, k.y, cosThetaI),
          conductorReflectance(eta.z, k.z, cosThetaI)};
}

__device__ __forceinline__ float dAnisoGGX(float HdotN, float HdotX, float HdotY, float ax, float ay) {
  return 1.0f / (PI * ax * ay * sqr(sqr(HdotX / ax) + sqr(HdotY / ay) + sqr(HdotN)) + EPS);
}
__device__ __forceinline__ f3 importanceSampleAnisoGGX(f2 u, f3 wo, float ax, float ay) {
  float factor = sqrtf(gmax(0.0f, u.x / gmax(1.0f - u.x, EPS)));
  float phi = TWO_PI * u.y;
  f3 wh{0.0f, 0.0f, 1.0f};
  wh.x = -ax * factor * mcos(phi);
  wh.y = -ay * factor * msin(phi);
  wh = makeNormal(wh);
  return reflect(-wo, wh);
}
__device__ __forceinline__ float importanceAnisoGGXPdf(f3 wh, f3 wo, float ax, float ay) {
  float pdf = 0.0f, HdotV = dot(wh, wo);
  f3 wi = reflect(-wo, wh);
  if (wi.z > 0.0f && wo.z > 0.0f && wh.z > 0.0f) pdf = dAnisoGGX(wh.z, wh.x, wh.y, ax, ay) * fabsf(wh.z) / (4.0f * HdotV + EPS);
  return pdf;
}
__device__ __forceinline__ float g1SmithAnisoGGX(float NdotV, float VdotX, float VdotY, float ax, float ay) {
  if (NdotV <= 0.0f) return 0.0f;
  f3 f{ax * VdotX, ay * VdotY, NdotV};
  return 1.0f / (NdotV + length(f));
}
// brdf_rough_plastic.rchit:82-111 (definition's parameter order)
__device__ __forceinline__ f3 rpEval(f3 L, f3 V, f3 N, f3 X, f3 Y, f3 kd, f3 ks, float eta, float fdrInt, float invEta2,
                                     float ax, float ay, uint32_t flags) {
  f3 weight = splat(0.0f);
  float NdotL = dot(L, N), NdotV = dot(V, N);
  if (((flags & EArea) == 0) || NdotL < 0.0f || NdotV < 0.0f) return weight;
  {
    f3 H = makeNormal(L + V);
    float ct;
    float Fs = fresnelDielectricExt(dot(H, V), ct, eta);
    float Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
    Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
    float Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
    weight = weight + ks * Fs * Gs * Ds * NdotL;
  }
  {
    float c1, c2;
    float Fo = fresnelDielectricExt(NdotV, c1, eta);
    float Fi = fresnelDielectricExt(NdotL, c2, eta);
    f3 diff = kd;
    diff = diff / (splat(1.0f) - diff * fdrInt);
    weight = weight + (1.0f - Fi) * (1.0f - Fo) * diff * invEta2 * INV_PI * NdotL;
  }
  return weight;
}
// brdf_rough_plastic.rchit:113-136 (definition's parameter order)
__device__ __forceinline__ float rpPdf(f3 L, f3 V, f3 N, f3 X, f3 Y, float ax, float ay, float eta, float ssw,
                                       uint32_t flags) {
  float pdf = 0.0f;
  float NdotL = dot(L, N), NdotV = dot(V, N);
  if (NdotL < 0.0f || NdotV < 0.0f || ((flags & EArea) == 0)) return pdf;
  float ct;
  float Fo = fresnelDielectricExt(NdotV, ct, eta);
  float substrateWeight = ssw * (1.0f - Fo);
  float specularWeight = Fo;
  float probSpecular = specularWeight / (specularWeight + substrateWeight);
  f3 wi = toLocal(X, Y, N, L), wo = toLocal(X, Y, N, V);
  f3 wh = makeNormal(wi + wo);
  float glossyPdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
  pdf = pdf + probSpecular * glossyPdf;
  float diffusePdf = cosineHemispherePdf(wi.z);
  pdf = pdf + (1.0f - probSpecular) * diffusePdf;
  return pdf;
}
// bsdf_dielectric.rchit:12-24
__device__ __forceinline__ float dielectricFresnel(float cosThetaI, float eta) {
  float sinThetaTSq = eta * eta * (1.0f - cosThetaI * cosThetaI);
  if (sinThetaTSq > 1.0f) return 1.0f;
  float cosThetaT = sqrtf(gmax(1.0f - sinThetaTSq, 0.0f));
  float rs = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
  float rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  return 0.5f * (rs * rs + rp * rp);
}

}  // namespace dm
}  // namespace asuna
