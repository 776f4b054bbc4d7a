// glsl_shim.h — just enough GLSL 4.60 for the reference's ray-tracing shader
// source to compile as host C++ (TEST INFRASTRUCTURE ONLY: the reference
// shaders translated by oracle/gen_ref.py are the pin of the CPU oracle).
//
// Semantics follow the GLSL 4.60 specification: float vectors, column-major
// matrices, left-to-right component arithmetic, implicit int->float in mixed
// expressions, min/max/clamp as defined in §8.3, reflect/refract as in §8.5.
// texture() is bilinear, REPEAT-wrapped, base level (what a ray-tracing stage
// samples with the reference's samplers).  Vectors value-initialise to zero so
// reads of unset shader locals are deterministic.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "../include/asuna_math.h"

namespace glslx {

using uint = unsigned int;

template <class T>
constexpr bool is_num = std::is_arithmetic<T>::value;

struct uvec2 {
  uint x = 0, y = 0;
};
struct vec2 {
  float x = 0, y = 0;
  vec2() = default;
  template <class A, class = std::enable_if_t<is_num<A>>>
  explicit vec2(A s) : x(float(s)), y(float(s)) {}
  template <class A, class B, class = std::enable_if_t<is_num<A> && is_num<B>>>
  vec2(A a, B b) : x(float(a)), y(float(b)) {}
  explicit vec2(uvec2 v) : x(float(v.x)), y(float(v.y)) {}
};
struct vec4;
struct vec3 {
  float x = 0, y = 0, z = 0;
  vec3() = default;
  template <class A, class = std::enable_if_t<is_num<A>>>
  explicit vec3(A s) : x(float(s)), y(float(s)), z(float(s)) {}
  template <class A, class B, class C, class = std::enable_if_t<is_num<A> && is_num<B> && is_num<C>>>
  vec3(A a, B b, C c) : x(float(a)), y(float(b)), z(float(c)) {}
  template <class B, class = std::enable_if_t<is_num<B>>>
  vec3(vec2 v, B b) : x(v.x), y(v.y), z(float(b)) {}
  vec2 xy() const { return vec2(x, y); }
  vec2 rg() const { return vec2(x, y); }
  vec3 rgb() const { return *this; }
  vec3 xyz() const { return *this; }
};
struct vec4 {
  float x = 0, y = 0, z = 0, w = 0;
  vec4() = default;
  template <class A, class = std::enable_if_t<is_num<A>>>
  explicit vec4(A s) : x(float(s)), y(float(s)), z(float(s)), w(float(s)) {}
  template <class A, class B, class C, class D>
  vec4(A a, B b, C c, D d) : x(float(a)), y(float(b)), z(float(c)), w(float(d)) {}
  template <class B, class = std::enable_if_t<is_num<B>>>
  vec4(vec3 v, B b) : x(v.x), y(v.y), z(v.z), w(float(b)) {}
  vec3 xyz() const { return vec3(x, y, z); }
  vec3 rgb() const { return vec3(x, y, z); }
  float r() const { return x; }
  vec2 xy() const { return vec2(x, y); }
  vec2 rg() const { return vec2(x, y); }
  vec4 rgba() const { return *this; }
};
struct ivec2 {
  int x = 0, y = 0;
  ivec2() = default;
  explicit ivec2(uvec2 v) : x(int(v.x)), y(int(v.y)) {}
};
struct ivec3 {
  int x = 0, y = 0, z = 0;
  ivec3() = default;
  ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  explicit ivec3(vec3 v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}  // truncation
};
struct uvec3 {
  uint x = 0, y = 0, z = 0;
  uvec3() = default;
  explicit uvec3(uint s) : x(s), y(s), z(s) {}
  uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
  template <class C>
  uvec3(uvec2 v, C c) : x(v.x), y(v.y), z(uint(c)) {}
  template <class C>
  uvec3(vec2 v, C c) : x(uint(v.x)), y(uint(v.y)), z(uint(c)) {}  // float -> uint conversion
  uvec2 xy() const { return uvec2{x, y}; }
};
// unsigned vector arithmetic (wrapping, as GLSL's uint)
inline uvec2 operator*(uvec2 a, uint s) { return uvec2{a.x * s, a.y * s}; }
inline uvec2 operator+(uvec2 a, uint s) { return uvec2{a.x + s, a.y + s}; }
inline uvec2 operator^(uvec2 a, uvec2 b) { return uvec2{a.x ^ b.x, a.y ^ b.y}; }
inline uvec2 operator>>(uvec2 a, uint s) { return uvec2{a.x >> s, a.y >> s}; }
inline uvec3 operator*(uvec3 a, uint s) { return uvec3(a.x * s, a.y * s, a.z * s); }
inline uvec3 operator+(uvec3 a, uvec3 b) { return uvec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline uvec3 operator^(uvec3 a, uvec3 b) { return uvec3(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z); }
inline uvec3 operator>>(uvec3 a, uvec3 b) { return uvec3(a.x >> b.x, a.y >> b.y, a.z >> b.z); }
inline uvec3 operator>>(uvec3 a, int s) { return uvec3(a.x >> s, a.y >> s, a.z >> s); }
inline uvec3 operator|(int s, uvec3 a) { return uvec3(uint(s) | a.x, uint(s) | a.y, uint(s) | a.z); }
inline uvec3& operator^=(uvec3& a, uvec3 b) { return a = a ^ b; }
struct uvec4 {
  uint x = 0, y = 0, z = 0, w = 0;
  uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

// mat4: four vec4 columns (column-major, like the reference's nvmath mat4f).
struct mat4 {
  vec4 c[4];
};
struct mat3 {
  vec3 c[3];
  mat3() = default;
  // GLSL's column-major constructor: the first three values are column 0
  template <class... A, class = std::enable_if_t<sizeof...(A) == 9>>
  explicit mat3(A... v) {
    const float f[9] = {float(v)...};
    for (int k = 0; k < 3; ++k) c[k] = vec3(f[3 * k], f[3 * k + 1], f[3 * k + 2]);
  }
};
// mat4x3: four vec3 columns (gl_ObjectToWorldEXT / gl_WorldToObjectEXT).
struct mat4x3 {
  vec3 c[4];
};

// ---- arithmetic ------------------------------------------------------------
#define GLSLX_V2(op)                                                                        \
  inline vec2 operator op(vec2 a, vec2 b) { return vec2(a.x op b.x, a.y op b.y); }        \
  template <class S, class = std::enable_if_t<is_num<S>>>                                 \
  inline vec2 operator op(vec2 a, S s) { return vec2(a.x op float(s), a.y op float(s)); } \
  template <class S, class = std::enable_if_t<is_num<S>>>                                 \
  inline vec2 operator op(S s, vec2 a) { return vec2(float(s) op a.x, float(s) op a.y); }
#define GLSLX_V3(op)                                                                      \
  inline vec3 operator op(vec3 a, vec3 b) { return vec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
  template <class S, class = std::enable_if_t<is_num<S>>>                               \
  inline vec3 operator op(vec3 a, S s) {                                                \
    return vec3(a.x op float(s), a.y op float(s), a.z op float(s));                     \
  }                                                                                     \
  template <class S, class = std::enable_if_t<is_num<S>>>                               \
  inline vec3 operator op(S s, vec3 a) {                                                \
    return vec3(float(s) op a.x, float(s) op a.y, float(s) op a.z);                     \
  }
#define GLSLX_V4(op)                                                                             \
  inline vec4 operator op(vec4 a, vec4 b) { return vec4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w); } \
  template <class S, class = std::enable_if_t<is_num<S>>>                                      \
  inline vec4 operator op(vec4 a, S s) {                                                       \
    return vec4(a.x op float(s), a.y op float(s), a.z op float(s), a.w op float(s));           \
  }                                                                                            \
  template <class S, class = std::enable_if_t<is_num<S>>>                                      \
  inline vec4 operator op(S s, vec4 a) {                                                       \
    return vec4(float(s) op a.x, float(s) op a.y, float(s) op a.z, float(s) op a.w);           \
  }
GLSLX_V2(+) GLSLX_V2(-) GLSLX_V2(*) GLSLX_V2(/)
GLSLX_V3(+) GLSLX_V3(-) GLSLX_V3(*) GLSLX_V3(/)
GLSLX_V4(+) GLSLX_V4(-) GLSLX_V4(*) GLSLX_V4(/)
#undef GLSLX_V2
#undef GLSLX_V3
#undef GLSLX_V4

inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec4 operator-(vec4 a) { return vec4(-a.x, -a.y, -a.z, -a.w); }
template <class T> inline vec2& operator+=(vec2& a, T b) { return a = a + b; }
template <class T> inline vec2& operator-=(vec2& a, T b) { return a = a - b; }
template <class T> inline vec2& operator*=(vec2& a, T b) { return a = a * b; }
template <class T> inline vec2& operator/=(vec2& a, T b) { return a = a / b; }
template <class T> inline vec3& operator+=(vec3& a, T b) { return a = a + b; }
template <class T> inline vec3& operator-=(vec3& a, T b) { return a = a - b; }
template <class T> inline vec3& operator*=(vec3& a, T b) { return a = a * b; }
template <class T> inline vec3& operator/=(vec3& a, T b) { return a = a / b; }

inline vec4 operator*(const mat4& m, vec4 v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w; }
inline vec3 operator*(const mat4x3& m, vec4 v) {
  return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w;
}

// ---- scalar built-ins (float) -----------------------------------------------
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sqrt(float x) { return std::sqrt(x); }
// The driver's transcendentals are implementation-defined in GLSL; the
// project's shared implementation stands in for them (include/asuna_math.h).
inline float exp(float x) { return asuna_math::expf_(x); }
inline float sin(float x) { return asuna_math::sinf_(x); }
inline float cos(float x) { return asuna_math::cosf_(x); }
inline float acos(float x) { return asuna_math::acosf_(x); }
inline float atan(float y, float x) { return asuna_math::atan2f_(y, x); }
inline float pow(float x, float y) { return asuna_math::powf_(x, y); }
inline float tan(float x) { return asuna_math::tanf_(x); }
inline float log(float x) { return asuna_math::logf_(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }
inline int floatBitsToInt(float f) {
  int i;
  std::memcpy(&i, &f, 4);
  return i;
}
inline float intBitsToFloat(int i) {
  float f;
  std::memcpy(&f, &i, 4);
  return f;
}

// min/max/clamp with GLSL's implicit int->float promotion in mixed calls.
template <class A, class B>
using num_t = std::conditional_t<std::is_floating_point<A>::value || std::is_floating_point<B>::value, float, A>;
template <class A, class B, class = std::enable_if_t<is_num<A> && is_num<B>>>
inline num_t<A, B> min(A a, B b) {
  num_t<A, B> x = num_t<A, B>(a), y = num_t<A, B>(b);
  return y < x ? y : x;
}
template <class A, class B, class = std::enable_if_t<is_num<A> && is_num<B>>>
inline num_t<A, B> max(A a, B b) {
  num_t<A, B> x = num_t<A, B>(a), y = num_t<A, B>(b);
  return x < y ? y : x;
}
template <class A, class B, class C, class = std::enable_if_t<is_num<A>>>
inline float clamp(A x, B lo, C hi) {
  return min(max(float(x), float(lo)), float(hi));
}
template <class B, class C>
inline vec3 clamp(vec3 v, B lo, C hi) {
  return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi));
}
// GLSL mix as the specification writes it: x * (1 - a) + y * a
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(vec3 x, vec3 y, vec3 a) { return x * (1.0f - a) + y * a; }
template <class A, class B, class T, class = std::enable_if_t<is_num<A> && is_num<B>>>
inline float mix(A x, B y, T a) {
  return float(x) * (1.0f - float(a)) + float(y) * float(a);
}

inline vec3 operator*(const mat3& m, vec3 v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
// component-wise max (GLSL 4.60 §8.3: y if x < y, else x)
inline vec3 max(vec3 a, vec3 b) { return vec3(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z); }
struct bvec3 {
  bool x, y, z;
};
inline bvec3 lessThan(vec3 a, vec3 b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline vec3 mix(vec3 x, vec3 y, bvec3 a) { return vec3(a.x ? y.x : x.x, a.y ? y.y : x.y, a.z ? y.z : x.z); }
inline vec3 floor(vec3 v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline vec3 uintBitsToFloat(uvec3 u) {
  float f[3];
  std::memcpy(&f[0], &u.x, 4);
  std::memcpy(&f[1], &u.y, 4);
  std::memcpy(&f[2], &u.z, 4);
  return vec3(f[0], f[1], f[2]);
}
inline float uintBitsToFloat(uint u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// component-wise exp / pow (GLSL 4.60 §8.2)
inline vec3 exp(vec3 v) { return vec3(exp(v.x), exp(v.y), exp(v.z)); }
inline vec3 pow(vec3 a, vec3 b) { return vec3(pow(a.x, b.x), pow(a.y, b.y), pow(a.z, b.z)); }
// smoothstep as the specification writes it (GLSL 4.60 §8.3)
template <class A, class B, class X, class = std::enable_if_t<is_num<A> && is_num<B> && is_num<X>>>
inline float smoothstep(A e0, B e1, X x) {
  float t = clamp((float(x) - float(e0)) / (float(e1) - float(e0)), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

// ---- geometric built-ins ----------------------------------------------------
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline float length(vec2 a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) {
  float l = length(a);
  return vec3(a.x / l, a.y / l, a.z / l);
}
inline vec3 reflect(vec3 I, vec3 N) { return I - 2.0f * dot(N, I) * N; }
inline vec3 refract(vec3 I, vec3 N, float eta) {
  float d = dot(N, I);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return vec3(0.0f);
  return eta * I - (eta * d + std::sqrt(k)) * N;
}
inline mat4 transpose(const mat4& m) {
  mat4 t;
  const float* s = &m.c[0].x;
  float* d = &t.c[0].x;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) d[c * 4 + r] = s[r * 4 + c];
  return t;
}
// row vector times matrix: (v * M)[j] = dot(v, column j)
inline vec4 operator*(vec3 v, const mat4x3& m) { return vec4(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2]), dot(v, m.c[3])); }

// ---- textures / images / ray tracing stubs ----------------------------------
struct sampler2D {
  int w = 1, h = 1, comps = 4;
  const float* data = nullptr;
};
inline vec4 texture(const sampler2D& t, vec2 uv) {
  float x = uv.x * float(t.w) - 0.5f, y = uv.y * float(t.h) - 0.5f;
  float fx0 = std::floor(x), fy0 = std::floor(y);
  float a = x - fx0, b = y - fy0;
  long i0 = long(fx0), j0 = long(fy0);
  auto wrap = [](long i, int n) {
    long m = i % n;
    return int(m < 0 ? m + n : m);
  };
  int i0w = wrap(i0, t.w), i1w = wrap(i0 + 1, t.w), j0w = wrap(j0, t.h), j1w = wrap(j0 + 1, t.h);
  float out[4] = {0, 0, 0, 0};
  for (int k = 0; k < t.comps; ++k) {
    float t00 = t.data[(size_t(j0w) * t.w + i0w) * t.comps + k];
    float t10 = t.data[(size_t(j0w) * t.w + i1w) * t.comps + k];
    float t01 = t.data[(size_t(j1w) * t.w + i0w) * t.comps + k];
    float t11 = t.data[(size_t(j1w) * t.w + i1w) * t.comps + k];
    out[k] = (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
  }
  return vec4(out[0], out[1], out[2], out[3]);
}
template <class T> inline T nonuniformEXT(T x) { return x; }

struct image2D {
  float* data = nullptr;
  int w = 0, h = 0;
};
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
  float* d = im.data + (size_t(p.y) * im.w + p.x) * 4;
  d[0] = v.x;
  d[1] = v.y;
  d[2] = v.z;
  d[3] = v.w;
}
inline vec4 imageLoad(const image2D& im, ivec2 p) {
  const float* d = im.data + (size_t(p.y) * im.w + p.x) * 4;
  return vec4(d[0], d[1], d[2], d[3]);
}

struct accelerationStructureEXT {};
constexpr uint gl_RayFlagsNoneEXT = 0u;
constexpr uint gl_RayFlagsOpaqueEXT = 1u;
constexpr uint gl_RayFlagsTerminateOnFirstHitEXT = 4u;
constexpr uint gl_RayFlagsSkipClosestHitShaderEXT = 8u;
constexpr uint gl_RayFlagsCullBackFacingTrianglesEXT = 16u;

}  // namespace glslx
