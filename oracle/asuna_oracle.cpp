// asuna_oracle.cpp — CPU oracle of the path-tracer hot path.
//
// TEST INFRASTRUCTURE ONLY (the checker of the CUDA path; never linked into
// the library).  A scalar restatement of the reference's GLSL ray-tracing
// path, templated on the arithmetic type: float reproduces the reference's
// FP32 streams for per-path parity, double gives the quality reference.
// Each function names the reference lines it follows.  Compile with
// -ffp-contract=off so the float instantiation rounds every operation the way
// the GLSL source spells it.
#include "asuna_oracle.h"
#include "../include/asuna_math.h"
#include "../include/asuna_sunsky.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

namespace ora {

// ----------------------------------------------------------------------------
// Scalar/vector helpers with GLSL semantics (GLSL 4.60 §8).
template <class R>
struct V2 {
  R x, y;
};
template <class R>
struct V3 {
  R x, y, z;
};

// Transcendentals: float uses the shared implementation of
// include/asuna_math.h (the same bits as the CUDA kernels), double the C library.
inline float msin(float x) { return asuna_math::sinf_(x); }
inline float mcos(float x) { return asuna_math::cosf_(x); }
inline float macos(float x) { return asuna_math::acosf_(x); }
inline float matan2(float y, float x) { return asuna_math::atan2f_(y, x); }
inline float mexp(float x) { return asuna_math::expf_(x); }
inline double msin(double x) { return std::sin(x); }
inline double mcos(double x) { return std::cos(x); }
inline double macos(double x) { return std::acos(x); }
inline double matan2(double y, double x) { return std::atan2(y, x); }
inline float mpow(float x, float y) { return asuna_math::powf_(x, y); }
inline double mpow(double x, double y) { return std::pow(x, y); }
inline float mlog(float x) { return asuna_math::logf_(x); }
inline double mlog(double x) { return std::log(x); }
inline double mexp(double x) { return std::exp(x); }

template <class R> inline V3<R> mk(R a, R b, R c) { return V3<R>{a, b, c}; }
template <class R> inline V3<R> splat(R a) { return V3<R>{a, a, a}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a) {
  R l = length(a);
  return {a.x / l, a.y / l, a.z / l};
}
template <class R> inline R gmin(R a, R b) { return b < a ? b : a; }  // GLSL min
template <class R> inline R gmax(R a, R b) { return a < b ? b : a; }  // GLSL max
template <class R> inline R gclamp(R x, R lo, R hi) { return gmin(gmax(x, lo), hi); }
template <class R> inline R gsign(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
// reflect/refract, GLSL 4.60 §8.5
template <class R> inline V3<R> reflect(V3<R> I, V3<R> N) { return I - R(2) * dot(N, I) * N; }
template <class R> inline V3<R> refract(V3<R> I, V3<R> N, R eta) {
  R d = dot(N, I);
  R k = R(1) - eta * eta * (R(1) - d * d);
  if (k < R(0)) return splat(R(0));
  return eta * I - (eta * d + std::sqrt(k)) * N;
}

template <class R>
struct K {
  static constexpr R PI = R(3.14159265358979323846);
  static constexpr R TWO_PI = R(6.28318530717958647692);
  static constexpr R INV_PI = R(0.31830988618379067154);
  static constexpr R INV_2PI = R(0.15915494309189533577);
  static constexpr R INV_4PI = R(0.07957747154594766788);
  static constexpr R PI_OVER_2 = R(1.57079632679489661923);
  static constexpr R PI_OVER_4 = R(0.78539816339744830961);
  static constexpr R EPS = R(0.001);
  static constexpr R INF = R(10000000000.0);
  static constexpr R MINIMUM = R(0.00001);
};

// math.glsl:20-30
inline uint32_t xxhash32(uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t p0 = 2246822519u, p1 = 3266489917u, p2 = 668265263u, p3 = 374761393u;
  uint32_t h = z + p3 + x * p1;
  h = p2 * ((h << 17) | (h >> 15));
  h += y * p1;
  h = p2 * ((h << 17) | (h >> 15));
  h = p0 * (h ^ (h >> 15));
  h = p1 * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
// math.glsl:34-39
inline uint32_t pcg(uint32_t& state) {
  uint32_t prev = state * 747796405u + 2891336453u;
  uint32_t word = ((prev >> ((prev >> 28u) + 4u)) ^ prev) * 277803737u;
  state = prev;
  return (word >> 22u) ^ word;
}
// math.glsl:42 — uint -> float rounds to nearest, times 2^-32 (exact).
template <class R> inline R rnd(uint32_t& s) { return R(float(pcg(s))) * R(2.3283064365386963e-10); }
template <> inline double rnd<double>(uint32_t& s) { return double(pcg(s)) * 2.3283064365386963e-10; }
template <class R> inline V2<R> rnd2(uint32_t& s) {
  R a = rnd<R>(s);
  R b = rnd<R>(s);
  return V2<R>{a, b};
}

// math.glsl:58-61
template <class R> inline V3<R> makeNormal(V3<R> n) {
  if (length(n) == R(0)) return n;
  return normalize(n);
}
// column-major mat4 * vec4 (m[c*4+r])
template <class R> inline void mat4mul(const float* m, R x, R y, R z, R w, R out[4]) {
  for (int r = 0; r < 4; ++r)
    out[r] = R(m[0 * 4 + r]) * x + R(m[1 * 4 + r]) * y + R(m[2 * 4 + r]) * z + R(m[3 * 4 + r]) * w;
}
template <class R> inline void mat4Tmul(const float* m, R x, R y, R z, R w, R out[4]) {
  // transpose(m) * v
  for (int r = 0; r < 4; ++r)
    out[r] = R(m[r * 4 + 0]) * x + R(m[r * 4 + 1]) * y + R(m[r * 4 + 2]) * z + R(m[r * 4 + 3]) * w;
}
// math.glsl:46-50
template <class R> inline V3<R> transformPoint(const float* m, V3<R> p) {
  R o[4];
  mat4mul<R>(m, p.x, p.y, p.z, R(1), o);
  return {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
}
// math.glsl:52-66
template <class R> inline V3<R> transformDirection(const float* m, V3<R> d) {
  R o[4];
  mat4mul<R>(m, d.x, d.y, d.z, R(0), o);
  return makeNormal(V3<R>{o[0], o[1], o[2]});
}
template <class R> inline V3<R> transformDirectionT(const float* m, V3<R> d) {
  R o[4];
  mat4Tmul<R>(m, d.x, d.y, d.z, R(0), o);
  return makeNormal(V3<R>{o[0], o[1], o[2]});
}
// math.glsl:133-138
template <class R> inline V3<R> uniformSampleSphere(V2<R> u) {
  R z = R(1) - R(2) * u.x;
  R r = std::sqrt(gmax(R(0), R(1) - z * z));
  R phi = K<R>::TWO_PI * u.y;
  return {r * mcos(phi), r * msin(phi), z};
}
// math.glsl:148-163
template <class R> inline V2<R> concentricSampleDisk(V2<R> u) {
  R ox = R(2) * u.x - R(1), oy = R(2) * u.y - R(1);
  if (ox == R(0) && oy == R(0)) return V2<R>{R(0), R(0)};
  R theta, r;
  if (std::fabs(ox) > std::fabs(oy)) {
    r = ox;
    theta = K<R>::PI_OVER_4 * (oy / ox);
  } else {
    r = oy;
    theta = K<R>::PI_OVER_2 - K<R>::PI_OVER_4 * (ox / oy);
  }
  return V2<R>{r * mcos(theta), r * msin(theta)};
}
// math.glsl:165-174
template <class R> inline V3<R> cosineSampleHemisphere(V2<R> u) {
  V2<R> d = concentricSampleDisk(u);
  R z = std::sqrt(gmax(R(0), R(1) - d.x * d.x - d.y * d.y));
  return {d.x, d.y, z};
}
template <class R> inline R cosineHemispherePdf(R c) { return c <= R(0) ? R(0) : c * K<R>::INV_PI; }
// math.glsl:184-189
template <class R> inline R powerHeuristic(R a, R b) {
  a = a * a;
  b = b * b + a;
  if (b == R(0)) return R(0);
  return a / b;
}
// math.glsl:199-216
template <class R> inline void basis(V3<R> n, V3<R>& f, V3<R>& r) {
  if (n.z < R(-0.999999)) {
    f = {R(0), R(-1), R(0)};
    r = {R(-1), R(0), R(0)};
  } else {
    R a = R(1) / (R(1) + n.z);
    R b = -n.x * n.y * a;
    f = {R(1) - n.x * n.x * a, b, -n.x};
    r = {b, R(1) - n.y * n.y * a, -n.y};
  }
}
template <class R> inline V3<R> toWorld(V3<R> X, V3<R> Y, V3<R> Z, V3<R> v) { return v.x * X + v.y * Y + v.z * Z; }
template <class R> inline V3<R> toLocal(V3<R> X, V3<R> Y, V3<R> Z, V3<R> v) {
  return {dot(v, X), dot(v, Y), dot(v, Z)};
}
// math.glsl:241-266 — integer ulp offset on the float bits.
inline float offsetComp(float p, float n) {
  int32_t ofi = int32_t(256.0f * n);
  int32_t bits;
  std::memcpy(&bits, &p, 4);
  bits += (p < 0.0f) ? -ofi : ofi;
  float pi;
  std::memcpy(&pi, &bits, 4);
  return std::fabs(p) < (1.0f / 32.0f) ? p + (1.0f / 65536.0f) * n : pi;
}
inline double offsetComp(double p, double n) {
  // FP64 instantiation: same rule on the float image of the point.
  return double(offsetComp(float(p), float(n))) + (p - double(float(p)));
}
template <class R> inline V3<R> offsetPositionAlongNormal(V3<R> p, V3<R> n) {
  return {offsetComp(p.x, n.x), offsetComp(p.y, n.y), offsetComp(p.z, n.z)};
}
// sun_and_sky.glsl:29-31
template <class R> inline R luminance(V3<R> c) {
  return R(0.2126f) * c.x + R(0.7152f) * c.y + R(0.0722f) * c.z;
}

// structs.glsl:7-20
enum : uint32_t {
  EBsdfNull = 0,
  EDiffuseReflection = 1,
  EDiffuseTransmission = 2,
  EGlossyReflection = 4,
  EGlossyTransmission = 8,
  ESpecularReflection = 16,
  ESpecularTransmission = 32,
  ESmooth = 1 | 2 | 4 | 8,
  EDelta = 1,
  EArea = 2
};
inline bool isNonSpecular(uint32_t f) { return (f & ESmooth) != 0; }

// ----------------------------------------------------------------------------
// Bilinear, REPEAT-wrapped fetch at the base level: what texture() returns in
// a ray-tracing stage for the reference's samplers (linear filter, default
// address mode 0 = REPEAT; src/core/texture.cpp:244-248).
struct Tex {
  int w = 0, h = 0, c = 0;
  std::vector<float> d;
};
template <class R> inline void texFetch(const Tex& t, R u, R v, R out[4]) {
  R x = u * R(t.w) - R(0.5), y = v * R(t.h) - R(0.5);
  R fx0 = std::floor(x), fy0 = std::floor(y);
  R a = x - fx0, b = y - fy0;
  long i0 = long(fx0), j0 = long(fy0);
  auto wrap = [](long i, int n) { long m = i % n; return int(m < 0 ? m + n : m); };
  int i0w = wrap(i0, t.w), i1w = wrap(i0 + 1, t.w), j0w = wrap(j0, t.h), j1w = wrap(j0 + 1, t.h);
  for (int k = 0; k < t.c; ++k) {
    R t00 = t.d[(size_t(j0w) * t.w + i0w) * t.c + k], t10 = t.d[(size_t(j0w) * t.w + i1w) * t.c + k];
    R t01 = t.d[(size_t(j1w) * t.w + i0w) * t.c + k], t11 = t.d[(size_t(j1w) * t.w + i1w) * t.c + k];
    out[k] = (R(1) - a) * (R(1) - b) * t00 + a * (R(1) - b) * t10 + (R(1) - a) * b * t01 + a * b * t11;
  }
}

// ----------------------------------------------------------------------------
// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013), float.
struct RayPre {
  int kx, ky, kz;
  float Sx, Sy, Sz;
  float o[3], d[3];
};
inline RayPre precompute(const float o[3], const float d[3]) {
  RayPre r;
  float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  if (d[kz] < 0.0f) std::swap(kx, ky);
  r.kx = kx;
  r.ky = ky;
  r.kz = kz;
  r.Sx = d[kx] / d[kz];
  r.Sy = d[ky] / d[kz];
  r.Sz = 1.0f / d[kz];
  for (int i = 0; i < 3; ++i) {
    r.o[i] = o[i];
    r.d[i] = d[i];
  }
  return r;
}
// Returns true and (t, b1, b2) for a hit with tmin <= t <= tmax.
inline bool intersectTri(const RayPre& r, const float* p0, const float* p1, const float* p2, float tmin,
                         float tmax, float& t, float& b1, float& b2) {
  float A[3], B[3], C[3];
  for (int i = 0; i < 3; ++i) {
    A[i] = p0[i] - r.o[i];
    B[i] = p1[i] - r.o[i];
    C[i] = p2[i] - r.o[i];
  }
  float Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
  float Bx = B[r.kx] - r.Sx * B[r.kz], By = B[r.ky] - r.Sy * B[r.kz];
  float Cx = C[r.kx] - r.Sx * C[r.kz], Cy = C[r.ky] - r.Sy * C[r.kz];
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
    V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
    W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  float det = U + V + W;
  if (det == 0.0f) return false;
  float Az = r.Sz * A[r.kz], Bz = r.Sz * B[r.kz], Cz = r.Sz * C[r.kz];
  float T = U * Az + V * Bz + W * Cz;
  float rcp = 1.0f / det;
  float tt = T * rcp;
  if (!(tt >= tmin && tt <= tmax)) return false;
  t = tt;
  b1 = V * rcp;
  b2 = W * rcp;
  return true;
}

// ----------------------------------------------------------------------------
// Scene: per-mesh BVH (object-median split, <= 4 triangles per leaf) and a
// flat list of instances.  Independent of the library's builder.
struct BNode {
  float lo[3], hi[3];
  uint32_t left;   // inner: index of left child (right = left + 1)
  uint32_t start;  // leaf: first triangle in `order`
  uint32_t count;  // 0 = inner
};
struct Mesh {
  std::vector<asuna_vertex> v;
  std::vector<uint32_t> idx;
  uint32_t ntri = 0;
  std::vector<BNode> nodes;
  std::vector<uint32_t> order;
  std::vector<float> tri;  // 9 floats per triangle in `order`
  float lo[3], hi[3];
};
struct Inst {
  asuna_instance_desc d;
  float w2o[12];
  float lo[3], hi[3];
};

struct Scene {
  std::vector<Mesh> meshes;
  std::vector<Inst> insts;
  std::vector<asuna_material> mats;
  std::vector<asuna_light> lights;
  bool hasEnv = false;
  Tex env, marg, cond;
  std::vector<Tex> texs;  // material textures (RGBA)
  // sun & sky (GpuSunAndSky.in_use = 1), in both precisions
  bool sky = false;
  asuna_sky::Params<float> skyF{};
  asuna_sky::Params<double> skyD{};
};

// sun_and_sky.glsl:405-533 through include/asuna_sunsky.h
template <class R> V3<R> sunSky(const Scene& s, V3<R> d);
template <> V3<float> sunSky(const Scene& s, V3<float> d) {
  const auto r = asuna_sky::sunAndSky<float>(s.skyF, asuna_sky::V<float>{d.x, d.y, d.z});
  return {r.x, r.y, r.z};
}
template <> V3<double> sunSky(const Scene& s, V3<double> d) {
  const auto r = asuna_sky::sunAndSky<double>(s.skyD, asuna_sky::V<double>{d.x, d.y, d.z});
  return {r.x, r.y, r.z};
}

static void buildBvh(Mesh& m) {
  const uint32_t n = m.ntri;
  std::vector<float> cen(size_t(n) * 3), blo(size_t(n) * 3), bhi(size_t(n) * 3);
  for (uint32_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      float a = m.v[m.idx[3 * i]].pos[k], b = m.v[m.idx[3 * i + 1]].pos[k], c = m.v[m.idx[3 * i + 2]].pos[k];
      blo[3 * i + k] = std::min(a, std::min(b, c));
      bhi[3 * i + k] = std::max(a, std::max(b, c));
      cen[3 * i + k] = 0.5f * (blo[3 * i + k] + bhi[3 * i + k]);
    }
  }
  m.order.resize(n);
  for (uint32_t i = 0; i < n; ++i) m.order[i] = i;
  m.nodes.clear();
  m.nodes.reserve(2 * size_t(n) + 1);
  struct Item {
    uint32_t node, start, count;
  };
  std::vector<Item> stack;
  m.nodes.push_back(BNode{});
  if (n) stack.push_back({0, 0, n});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    BNode nd;
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 3; ++k) {
      nd.lo[k] = INFINITY;
      nd.hi[k] = -INFINITY;
    }
    for (uint32_t i = it.start; i < it.start + it.count; ++i) {
      uint32_t t = m.order[i];
      for (int k = 0; k < 3; ++k) {
        nd.lo[k] = std::min(nd.lo[k], blo[3 * t + k]);
        nd.hi[k] = std::max(nd.hi[k], bhi[3 * t + k]);
        clo[k] = std::min(clo[k], cen[3 * t + k]);
        chi[k] = std::max(chi[k], cen[3 * t + k]);
      }
    }
    // Conservative expansion so the slab test never rejects a triangle the
    // watertight test would accept.
    for (int k = 0; k < 3; ++k) {
      float e = 1e-6f * std::max(std::fabs(nd.lo[k]), std::fabs(nd.hi[k])) + 1e-30f;
      nd.lo[k] -= e;
      nd.hi[k] += e;
    }
    if (it.count <= 4) {
      nd.left = 0;
      nd.start = it.start;
      nd.count = it.count;
      m.nodes[it.node] = nd;
      continue;
    }
    int axis = 0;
    float ext = chi[0] - clo[0];
    for (int k = 1; k < 3; ++k)
      if (chi[k] - clo[k] > ext) {
        ext = chi[k] - clo[k];
        axis = k;
      }
    uint32_t mid = it.start + it.count / 2;
    std::nth_element(m.order.begin() + it.start, m.order.begin() + mid, m.order.begin() + it.start + it.count,
                     [&](uint32_t a, uint32_t b) {
                       float ca = cen[3 * a + axis], cb = cen[3 * b + axis];
                       return ca < cb || (ca == cb && a < b);
                     });
    uint32_t l = uint32_t(m.nodes.size());
    m.nodes.push_back(BNode{});
    m.nodes.push_back(BNode{});
    nd.left = l;
    nd.start = 0;
    nd.count = 0;
    m.nodes[it.node] = nd;
    stack.push_back({l, it.start, mid - it.start});
    stack.push_back({l + 1, mid, it.start + it.count - mid});
  }
  m.tri.resize(size_t(n) * 9);
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t t = m.order[i];
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < 3; ++k) m.tri[size_t(i) * 9 + c * 3 + k] = m.v[m.idx[3 * t + c]].pos[k];
  }
  if (n) {
    for (int k = 0; k < 3; ++k) {
      m.lo[k] = m.nodes[0].lo[k];
      m.hi[k] = m.nodes[0].hi[k];
    }
  } else {
    for (int k = 0; k < 3; ++k) {
      m.lo[k] = INFINITY;
      m.hi[k] = -INFINITY;
    }
  }
}

// 3x4 row-major inverse, computed in double and rounded once to float.  The
// library computes gl_WorldToObjectEXT the same way so both traverse with the
// same object-space rays.
static void invert3x4(const float* m, float* out) {
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

// Object-space ray: o' = W2O (o,1), d' = W2O (d,0); fixed operation order
// (the CUDA traversal uses the same order with non-contracted ops).
inline void xformRay(const float* w, const float o[3], const float d[3], float oo[3], float dd[3]) {
  for (int r = 0; r < 3; ++r) {
    oo[r] = ((w[r * 4 + 0] * o[0] + w[r * 4 + 1] * o[1]) + w[r * 4 + 2] * o[2]) + w[r * 4 + 3];
    dd[r] = (w[r * 4 + 0] * d[0] + w[r * 4 + 1] * d[1]) + w[r * 4 + 2] * d[2];
  }
}

// Box test.  The box is widened in space when built; the far distance is
// widened by 2^-20 here as well, so that the rounding of the distances
// (relative to t, not to the box's coordinates) never rejects a box whose
// triangle the watertight test would accept, as where a ray meets several
// triangles at the corner of their boxes.
inline bool slab(const float lo[3], const float hi[3], const float o[3], const float inv[3], float tmin, float tmax) {
  float t0 = tmin, t1 = tmax;
  for (int k = 0; k < 3; ++k) {
    float a = (lo[k] - o[k]) * inv[k], b = (hi[k] - o[k]) * inv[k];
    if (a > b) std::swap(a, b);
    if (std::isnan(a) || std::isnan(b)) {
      // 0 * inf: the ray lies in the slab plane; keep it (conservative).
      continue;
    }
    t0 = std::max(t0, a);
    t1 = std::min(t1, b);
  }
  return t0 <= t1 * 1.00000095367431640625f;  // 1 + 2^-20
}

struct Hit {
  float t;
  uint32_t inst, prim;
  float u, v;
};

struct TravStats {
  uint64_t nodes = 0, tris = 0;
};

// Closest hit (anyHit=false) or any hit (anyHit=true) in [tmin, tmax].
static bool traceScene(const Scene& s, const float o[3], const float d[3], float tmin, float tmax, bool anyHit,
                       Hit& hit, TravStats* st) {
  bool found = false;
  float best = tmax;
  for (uint32_t ii = 0; ii < s.insts.size(); ++ii) {
    const Inst& in = s.insts[ii];
    const Mesh& m = s.meshes[in.d.mesh_id];
    if (!m.ntri) continue;
    float oo[3], dd[3];
    xformRay(in.w2o, o, d, oo, dd);
    float inv[3] = {1.0f / dd[0], 1.0f / dd[1], 1.0f / dd[2]};
    if (!slab(m.lo, m.hi, oo, inv, tmin, best)) continue;
    RayPre rp = precompute(oo, dd);
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const BNode& nd = m.nodes[stack[--sp]];
      if (st) st->nodes++;
      if (!slab(nd.lo, nd.hi, oo, inv, tmin, best)) continue;
      if (nd.count) {
        for (uint32_t k = 0; k < nd.count; ++k) {
          const float* tv = &m.tri[size_t(nd.start + k) * 9];
          float t, b1, b2;
          if (st) st->tris++;
          if (intersectTri(rp, tv, tv + 3, tv + 6, tmin, best, t, b1, b2)) {
            if (anyHit) {
              hit = Hit{t, ii, m.order[nd.start + k], b1, b2};
              return true;
            }
            const uint32_t prim = m.order[nd.start + k];
            // exact ties resolve to the lowest (instance, primitive): the
            // closest hit does not depend on traversal order
            if (!found || t < best || ii < hit.inst || (ii == hit.inst && prim < hit.prim)) {
              found = true;
              best = t;
              hit = Hit{t, ii, prim, b1, b2};
            }
          }
        }
      } else {
        stack[sp++] = nd.left + 1;
        stack[sp++] = nd.left;
      }
    }
  }
  return found;
}

// ----------------------------------------------------------------------------
// Env map importance tables, restating EnvMap::EnvMap (src/core/texture.cpp:
// 144-226) including its double-precision literals and float storage.
static void envTables(int width, int height, const float* px, float* marg, float* cond) {
  std::vector<float> pdf2D(size_t(width) * height), cdf2D(size_t(width) * height), pdf1D(height), cdf1D(height);
  for (size_t i = 0; i < size_t(width) * height * 2; ++i) marg[i] = cond[i] = 0.0f;
  float weightSum = 0.0f;
  for (int j = 0; j < height; j++) {
    float rowWeightSum = 0.0f;
    for (int i = 0; i < width; i++) {
      const float* c = &px[(size_t(j) * width + i) * 4];
      float weight = float(0.3 * c[0] + 0.6 * c[1] + 0.1 * c[2]);
      rowWeightSum += weight;
      pdf2D[size_t(j) * width + i] = weight;
      cdf2D[size_t(j) * width + i] = rowWeightSum;
    }
    for (int i = 0; i < width; i++) {
      pdf2D[size_t(j) * width + i] = float(pdf2D[size_t(j) * width + i] / (rowWeightSum + 1e-7));
      cdf2D[size_t(j) * width + i] = float(cdf2D[size_t(j) * width + i] / (rowWeightSum + 1e-7));
    }
    weightSum += rowWeightSum;
    pdf1D[j] = rowWeightSum;
    cdf1D[j] = weightSum;
  }
  for (int j = 0; j < height; j++) {
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
  for (int j = 0; j < height; j++) {
    float invHeight = float(j + 1) / float(height);
    float row = float(lowerBound(cdf1D.data(), 0, height, invHeight));
    marg[(size_t(j) * width) * 2 + 0] = row / float(height);
    marg[(size_t(j) * width) * 2 + 1] = pdf1D[j];
  }
  for (int j = 0; j < height; j++)
    for (int i = 0; i < width; i++) {
      float invWidth = float(i + 1) / float(width);
      float col = float(lowerBound(cdf2D.data(), j * width, (j + 1) * width, invWidth) - j * width);
      cond[(size_t(j) * width + i) * 2 + 0] = col / float(width);
      cond[(size_t(j) * width + i) * 2 + 1] = pdf2D[size_t(j) * width + i];
    }
}

// ----------------------------------------------------------------------------
// The path (one sample of one pixel of one frame).
template <class R>
struct Ctx {
  const Scene* s;
  const asuna_shot* shot;
  TravStats* st;
  uint64_t* shadowRays;
  uint64_t* extendRays;
};

template <class R> inline V3<R> L3(const float* a) { return V3<R>{R(a[0]), R(a[1]), R(a[2])}; }

// sample_light.glsl:84-95
template <class R> R pdfEnvmap(const Scene& s, const asuna_shot& sh, V3<R> L) {
  L = transformDirectionT<R>(sh.camera.env_transform, L);
  R theta = macos(gclamp(L.y, R(-1), R(1)));
  R u = (K<R>::PI + matan2(L.z, L.x)) * K<R>::INV_2PI, v = theta * K<R>::INV_PI;
  R c[4], m[4];
  texFetch<R>(s.cond, u, v, c);
  texFetch<R>(s.marg, R(0), v, m);
  R pdf = c[1] * m[1];
  R sinTheta = msin(theta);
  if (sinTheta == R(0)) return R(0);
  return (pdf * R(sh.state.env_map_resolution[0]) * R(sh.state.env_map_resolution[1])) /
         (K<R>::TWO_PI * K<R>::PI * sinTheta);
}
// sample_light.glsl:97-104
template <class R> V3<R> evalEnvmap(const Scene& s, const asuna_shot& sh, V3<R> L) {
  L = transformDirectionT<R>(sh.camera.env_transform, L);
  R theta = macos(gclamp(L.y, R(-1), R(1)));
  R u = (K<R>::PI + matan2(L.z, L.x)) * K<R>::INV_2PI, v = theta * K<R>::INV_PI;
  R e[4];
  texFetch<R>(s.env, u, v, e);
  R k = R(sh.state.env_map_intensity);
  return V3<R>{k * e[0], k * e[1], k * e[2]};
}
// sample_light.glsl:106-129
template <class R> V3<R> sampleEnvmap(const Scene& s, const asuna_shot& sh, V2<R> r, V3<R>& L, R& pdf) {
  R m[4], c[4];
  texFetch<R>(s.marg, R(0), r.x, m);
  R uvy = m[0];
  texFetch<R>(s.cond, r.y, uvy, c);
  R uvx = c[0];
  texFetch<R>(s.cond, uvx, uvy, c);
  texFetch<R>(s.marg, R(0), uvy, m);
  pdf = c[1] * m[1];
  R phi = uvx * K<R>::TWO_PI;
  R theta = uvy * K<R>::PI;
  if (msin(theta) == R(0)) pdf = R(0);
  pdf = (pdf * R(sh.state.env_map_resolution[0]) * R(sh.state.env_map_resolution[1])) /
        (K<R>::TWO_PI * K<R>::PI * msin(theta));
  L = V3<R>{-msin(theta) * mcos(phi), mcos(theta), -msin(theta) * msin(phi)};
  L = transformDirection<R>(sh.camera.env_transform, L);
  R e[4];
  texFetch<R>(s.env, uvx, uvy, e);
  R k = R(sh.state.env_map_intensity);
  return V3<R>{k * e[0], k * e[1], k * e[2]};
}

template <class R>
struct LRec {
  V3<R> d{R(0), R(0), R(0)}, n{R(0), R(0), R(0)};
  R dist = R(0), pdf = R(0);
  uint32_t flags = 0;
};

// sample_light.glsl:10-82
template <class R> V3<R> sampleOneLight(V2<R> r, const asuna_light& l, V3<R> P, LRec<R>& rec) {
  if (l.type == ASUNA_LIGHT_RECT || l.type == ASUNA_LIGHT_TRIANGLE) {
    R r1 = r.x, r2 = (l.type == ASUNA_LIGHT_TRIANGLE) ? (R(1) - r1) * r.y : r.y;
    V3<R> pos = L3<R>(l.position) + L3<R>(l.u) * r1 + L3<R>(l.v) * r2;
    rec.d = pos - P;
    rec.dist = length(rec.d);
    R distSq = rec.dist * rec.dist;
    rec.d = rec.d / rec.dist;
    rec.n = makeNormal(cross(L3<R>(l.u), L3<R>(l.v)));
    rec.pdf = distSq / (R(l.area) * std::fabs(dot(rec.n, rec.d)) + K<R>::EPS);
    rec.flags = EArea;
    return L3<R>(l.radiance);
  } else if (l.type == ASUNA_LIGHT_DIRECTIONAL) {
    rec.d = makeNormal(L3<R>(l.direction));
    rec.n = -rec.d;
    rec.dist = K<R>::INF;
    rec.pdf = R(1);
    rec.flags = EDelta;
    return L3<R>(l.radiance);
  } else if (l.type == ASUNA_LIGHT_POINT) {
    rec.d = L3<R>(l.position) - P;
    rec.n = -rec.d;
    rec.dist = length(rec.d);
    R distSq = rec.dist * rec.dist;
    rec.d = rec.d / (rec.dist + K<R>::EPS);
    rec.pdf = R(1);
    rec.flags = EDelta;
    return L3<R>(l.radiance) / (distSq + K<R>::EPS);
  }
  return splat(R(0));  // undefined type: the reference returns nothing
}

template <class R>
struct PathState {
  V3<R> ro, rd;
  V3<R> radiance, throughput;
  uint32_t depth, seed;
  bool stop;
  bool passed;  // this hit passed the ray through (opacity): no bounce counted
  uint32_t bflags;
  R bpdf;
  V3<R> ch[ASUNA_MAX_CHANNELS];
  // NEE record of the current bounce
  bool dskip;
  V3<R> drad, dro, drd;
  R ddist;
  uint32_t sig;
};

inline uint32_t sigMix(uint32_t h, uint32_t v) {
  h ^= v + 0x9e3779b9u + (h << 6) + (h >> 2);
  return h;
}

// rchit_layouts.glsl:118-167
template <class R>
V3<R> sampleLights(const Scene& s, const asuna_shot& sh, PathState<R>& p, V3<R> pos, V3<R> nrm, bool& visible,
                   LRec<R>& lRec) {
  bool allowDoubleSide = false;
  V3<R> radiance = splat(R(0));
  bool hasEnv = sh.state.has_env_map == 1 || s.sky;
  bool hasLight = sh.state.num_lights > 0;
  R envSel, anaSel;
  if (hasEnv && hasLight)
    envSel = anaSel = R(0.5);
  else if (hasEnv)
    envSel = R(1), anaSel = R(0);
  else if (hasLight)
    envSel = R(0), anaSel = R(1);
  else
    envSel = anaSel = R(0);
  R sel = rnd<R>(p.seed);
  if (sel < envSel) {
    // rchit_layouts.glsl:98-116: sun & sky (sample_light.glsl:137-141,
    // uniform sphere) or the environment map
    lRec.flags = EArea;
    lRec.dist = K<R>::INF;
    lRec.n = -makeNormal(p.rd);
    V2<R> u = rnd2<R>(p.seed);
    if (s.sky) {
      lRec.d = uniformSampleSphere<R>(u);
      lRec.pdf = K<R>::INV_4PI;
      radiance = sunSky<R>(s, lRec.d) / envSel;
    } else {
      radiance = sampleEnvmap<R>(s, sh, u, lRec.d, lRec.pdf) / envSel;
    }
    allowDoubleSide = true;
  } else if (sel < envSel + anaSel) {
    int n = sh.state.num_lights;
    int idx = std::min(1 + int(rnd<R>(p.seed) * R(n)), n);
    const asuna_light& l = s.lights[idx];
    V2<R> u = rnd2<R>(p.seed);
    radiance = sampleOneLight<R>(u, l, pos, lRec) * R(n) / anaSel;
    allowDoubleSide = (l.double_side == 1);
  }
  p.dro = offsetPositionAlongNormal(pos, nrm);
  p.drd = lRec.d;
  p.ddist = lRec.dist;
  visible = (dot(lRec.d, nrm) > R(0) && lRec.pdf > R(0));
  visible = visible && (dot(lRec.n, lRec.d) < R(0) || allowDoubleSide);
  return radiance;
}

template <class R>
struct HitState {
  int lightId;
  V2<R> uv;
  V3<R> pos, V, N, geoN, ffN, X, Y;
  asuna_material mat;
  const float* w2o;  // the instance's world-to-object rows
};

// rchit_layouts.glsl:61-95
template <class R> HitState<R> getHitState(const Scene& s, const asuna_shot& sh, const PathState<R>& p, const Hit& h) {
  HitState<R> st;
  const Inst& in = s.insts[h.inst];
  const Mesh& m = s.meshes[in.d.mesh_id];
  const asuna_vertex& v0 = m.v[m.idx[3 * h.prim]];
  const asuna_vertex& v1 = m.v[m.idx[3 * h.prim + 1]];
  const asuna_vertex& v2 = m.v[m.idx[3 * h.prim + 2]];
  R bx = R(1) - R(h.u) - R(h.v), by = R(h.u), bz = R(h.v);
  st.lightId = in.d.light_id;
  st.uv = V2<R>{R(v0.uv[0]) * bx + R(v1.uv[0]) * by + R(v2.uv[0]) * bz,
                R(v0.uv[1]) * bx + R(v1.uv[1]) * by + R(v2.uv[1]) * bz};
  V3<R> po = L3<R>(v0.pos) * bx + L3<R>(v1.pos) * by + L3<R>(v2.pos) * bz;
  const float* o = in.d.transform;
  st.pos = V3<R>{R(o[0]) * po.x + R(o[1]) * po.y + R(o[2]) * po.z + R(o[3]),
                 R(o[4]) * po.x + R(o[5]) * po.y + R(o[6]) * po.z + R(o[7]),
                 R(o[8]) * po.x + R(o[9]) * po.y + R(o[10]) * po.z + R(o[11])};
  const float* w = in.w2o;
  st.w2o = w;
  auto nxf = [&](V3<R> n) {
    return makeNormal(V3<R>{n.x * R(w[0]) + n.y * R(w[4]) + n.z * R(w[8]),
                            n.x * R(w[1]) + n.y * R(w[5]) + n.z * R(w[9]),
                            n.x * R(w[2]) + n.y * R(w[6]) + n.z * R(w[10])});
  };
  V3<R> n = L3<R>(v0.normal) * bx + L3<R>(v1.normal) * by + L3<R>(v2.normal) * bz;
  st.N = nxf(n);
  // The reference stores this in ffN and never sets geoN; the geometric
  // normal is kept here for use_face_normal (reference reads geoN unset).
  st.geoN = nxf(cross(L3<R>(v1.pos) - L3<R>(v0.pos), L3<R>(v2.pos) - L3<R>(v0.pos)));
  st.V = makeNormal(-p.rd);
  if (st.lightId < 0) st.mat = s.mats[in.d.material_id];
  // configureShadingFrame, rchit_layouts.glsl:61-65
  if (sh.state.use_face_normal == 1) st.N = st.geoN;
  basis(st.N, st.X, st.Y);
  st.ffN = dot(st.N, st.V) > R(0) ? st.N : -st.N;
  return st;
}

// The "Fetch textures" block of each material's hit shader (textureEval,
// rchit_layouts.glsl:169-171, bilinear REPEAT at the base level):
// brdf_lambertian.rchit:80-90 diffuse + tangent-space normal map (likewise
// plastic, mirror, conductor, Phong); brdf_rough_plastic.rchit:196-208 and
// brdf_rough_conductor.rchit:152-164 add alpha (.rg); bsdf_dielectric.rchit:
// 79-86 normal only; brdf_pbr_metalness_roughness.rchit:136-149 and
// brdf_disney.rchit:380-391 add metalness and roughness (.r);
// brdf_kang18.rchit:140-175 specular (.rgb), alpha (.rg), object-space
// normal and tangent maps; brdf_emissive.rchit:20-23 radiance = factor * texel.
template <class R> V3<R> texRGB(const Scene& s, int id, V2<R> uv) {
  R o[4];
  texFetch(s.texs[size_t(id)], uv.x, uv.y, o);
  return V3<R>{o[0], o[1], o[2]};
}
template <class R> void applyTextures(const Scene& s, const asuna_shot& sh, HitState<R>& st) {
  asuna_material& m = st.mat;
  const uint32_t t = m.type;
  auto put3 = [](float* f, V3<R> v) {
    f[0] = float(v.x);
    f[1] = float(v.y);
    f[2] = float(v.z);
  };
  if (t == ASUNA_MAT_EMISSIVE) {
    if (m.radiance_texture_id >= 0) put3(m.radiance, L3<R>(m.radiance_factor) * texRGB(s, m.radiance_texture_id, st.uv));
    return;
  }
  if (t != ASUNA_MAT_DIELECTRIC && m.diffuse_texture_id >= 0) put3(m.diffuse, texRGB(s, m.diffuse_texture_id, st.uv));
  if (t == ASUNA_MAT_PBR_METALNESS_ROUGHNESS || t == ASUNA_MAT_DISNEY) {
    if (m.metalness_texture_id >= 0) m.metalness = float(texRGB(s, m.metalness_texture_id, st.uv).x);
    if (m.roughness_texture_id >= 0) m.roughness = float(texRGB(s, m.roughness_texture_id, st.uv).x);
  }
  if (t == ASUNA_MAT_KANG18 && m.metalness_texture_id >= 0) put3(m.rho_spec, texRGB(s, m.metalness_texture_id, st.uv));
  if ((t == ASUNA_MAT_ROUGH_PLASTIC || t == ASUNA_MAT_ROUGH_CONDUCTOR || t == ASUNA_MAT_KANG18) &&
      m.roughness_texture_id >= 0) {
    V3<R> c = texRGB(s, m.roughness_texture_id, st.uv);
    m.aniso_alpha[0] = float(c.x);
    m.aniso_alpha[1] = float(c.y);
  }
  auto objToWorld = [&](V3<R> n) {
    const float* w = st.w2o;
    return V3<R>{n.x * R(w[0]) + n.y * R(w[4]) + n.z * R(w[8]), n.x * R(w[1]) + n.y * R(w[5]) + n.z * R(w[9]),
                 n.x * R(w[2]) + n.y * R(w[6]) + n.z * R(w[10])};
  };
  if (m.normal_texture_id >= 0) {
    V3<R> c = texRGB(s, m.normal_texture_id, st.uv);
    V3<R> n{R(2) * c.x - R(1), R(2) * c.y - R(1), R(2) * c.z - R(1)};
    st.N = makeNormal(t == ASUNA_MAT_KANG18 ? objToWorld(n) : toWorld(st.X, st.Y, st.N, n));
    // configureShadingFrame, rchit_layouts.glsl:61-65
    if (sh.state.use_face_normal == 1) st.N = st.geoN;
    basis(st.N, st.X, st.Y);
    st.ffN = dot(st.N, st.V) > R(0) ? st.N : -st.N;
  }
  if (t == ASUNA_MAT_KANG18 && m.tangent_texture_id >= 0) {
    V3<R> c = texRGB(s, m.tangent_texture_id, st.uv);
    st.X = makeNormal(objToWorld(V3<R>{R(2) * c.x - R(1), R(2) * c.y - R(1), R(2) * c.z - R(1)}));
  }
}

// brdf_lambertian.rchit:44-68
template <class R> void hitLight(const Scene& s, PathState<R>& p, int lightId, V3<R> hitPos) {
  const asuna_light& l = s.lights[lightId];
  V3<R> ldir = makeNormal(p.rd);
  V3<R> lnrm = makeNormal(cross(L3<R>(l.u), L3<R>(l.v)));
  R proj = dot(lnrm, ldir);
  p.stop = true;
  if (proj > R(0) && l.double_side == 0) return;
  R mis = R(1);
  if (isNonSpecular(p.bflags) && p.depth != 1) {
    R dist = length(hitPos - p.ro);
    R d2 = dist * dist;
    R lpdf = d2 / (R(l.area) * std::fabs(proj) + K<R>::EPS);
    mis = powerHeuristic(p.bpdf, lpdf);
  }
  p.radiance = p.radiance + p.throughput * L3<R>(l.radiance) * mis;
}

// AOVs at depth 1 (brdf_lambertian.rchit:93-108), plus the depth channel.
template <class R> void writeAovs(const asuna_rt_state& ps, PathState<R>& p, const HitState<R>& st) {
  if (ps.diffuse_out_channel >= 0) p.ch[ps.diffuse_out_channel] = L3<R>(st.mat.diffuse);
  if (ps.normal_out_channel >= 0) p.ch[ps.normal_out_channel] = st.N;
  if (ps.specular_out_channel >= 0) p.ch[ps.specular_out_channel] = splat(R(0));
  if (ps.tangent_out_channel >= 0) p.ch[ps.tangent_out_channel] = st.X;
  if (ps.roughness_out_channel >= 0) p.ch[ps.roughness_out_channel] = V3<R>{R(1), R(1), R(0)};
  if (ps.position_out_channel >= 0) p.ch[ps.position_out_channel] = st.pos;
  if (ps.uv_out_channel >= 0) p.ch[ps.uv_out_channel] = V3<R>{st.uv.x, st.uv.y, R(1)};
}

// brdf_lambertian.rchit:70-151
template <class R> void shadeLambertian(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  const asuna_rt_state& ps = sh.state;
  V3<R> kd = L3<R>(st.mat.diffuse);
  if (p.depth == 1) writeAovs(ps, p, st);
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      // eval (12-21) with flag EArea, pdf (23-29) with lRec.flags
      V3<R> w = splat(R(0));
      R NdotL = dot(st.ffN, lRec.d), NdotV = dot(st.ffN, st.V);
      if (!(NdotL < R(0) || NdotV < R(0))) w = kd * K<R>::INV_PI * NdotL;
      R bpdf = (lRec.flags & EArea) ? cosineHemispherePdf(dot(st.ffN, lRec.d)) : R(0);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  // sampleBsdf (31-42)
  V2<R> u = rnd2<R>(p.seed);
  V3<R> wi = cosineSampleHemisphere(u);
  R pdf = cosineHemispherePdf(wi.z);
  V3<R> d = toWorld(st.X, st.Y, st.ffN, wi);
  V3<R> w = kd * K<R>::INV_PI * std::fabs(wi.z);
  if (pdf <= R(0) || length(w) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = EDiffuseReflection;
  p.bpdf = pdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = d;
  p.throughput = p.throughput * (w / pdf);
}

// brdf_rough_plastic.rchit:12-41
template <class R> R fresnelDielectricExt(R cosThetaI_, R& cosThetaT_, R eta) {
  if (eta == R(1)) {
    cosThetaT_ = -cosThetaI_;
    return R(0);
  }
  R scale = (cosThetaI_ > R(0)) ? R(1) / eta : eta;
  R cosThetaTSqr = R(1) - (R(1) - cosThetaI_ * cosThetaI_) * (scale * scale);
  if (cosThetaTSqr <= R(0)) {
    cosThetaT_ = R(0);
    return R(1);
  }
  R cosThetaI = std::fabs(cosThetaI_);
  R cosThetaT = std::sqrt(cosThetaTSqr);
  R Rs = (cosThetaI - eta * cosThetaT) / (cosThetaI + eta * cosThetaT);
  R Rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  cosThetaT_ = (cosThetaI_ > R(0)) ? -cosThetaT : cosThetaT;
  return R(0.5) * (Rs * Rs + Rp * Rp);
}
template <class R> inline R sqr(R x) { return x * x; }
// 45-50
template <class R> R dAnisoGGX(R HdotN, R HdotX, R HdotY, R ax, R ay) {
  return R(1) / (K<R>::PI * ax * ay * sqr(sqr(HdotX / ax) + sqr(HdotY / ay) + sqr(HdotN)) + K<R>::EPS);
}
// 52-65
template <class R> V3<R> importanceSampleAnisoGGX(V2<R> u, V3<R> wo, R ax, R ay) {
  R factor = std::sqrt(gmax(R(0), u.x / gmax(R(1) - u.x, K<R>::EPS)));
  R phi = K<R>::TWO_PI * u.y;
  V3<R> wh{R(0), R(0), R(1)};
  wh.x = -ax * factor * mcos(phi);
  wh.y = -ay * factor * msin(phi);
  wh = makeNormal(wh);
  return reflect(-wo, wh);
}
// 67-73
template <class R> R importanceAnisoGGXPdf(V3<R> wh, V3<R> wo, R ax, R ay) {
  R pdf = R(0), HdotV = dot(wh, wo);
  V3<R> wi = reflect(-wo, wh);
  if (wi.z > R(0) && wo.z > R(0) && wh.z > R(0))
    pdf = dAnisoGGX(wh.z, wh.x, wh.y, ax, ay) * std::fabs(wh.z) / (R(4) * HdotV + K<R>::EPS);
  return pdf;
}
// 75-80
template <class R> R g1SmithAnisoGGX(R NdotV, R VdotX, R VdotY, R ax, R ay) {
  if (NdotV <= R(0)) return R(0);
  V3<R> f{ax * VdotX, ay * VdotY, NdotV};
  return R(1) / (NdotV + length(f));
}
// 82-111 (parameter order of the definition)
template <class R>
V3<R> rpEval(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, V3<R> kd, V3<R> ks, R eta, R fdrInt, R invEta2, R ax, R ay,
             uint32_t flags) {
  V3<R> weight = splat(R(0));
  R NdotL = dot(L, N), NdotV = dot(V, N);
  if (((flags & EArea) == 0) || NdotL < R(0) || NdotV < R(0)) return weight;
  {
    V3<R> H = makeNormal(L + V);
    R ct;
    R Fs = fresnelDielectricExt(dot(H, V), ct, eta);
    R Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
    Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
    R Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
    weight = weight + ks * Fs * Gs * Ds * NdotL;
  }
  {
    R c1, c2;
    R Fo = fresnelDielectricExt(NdotV, c1, eta);
    R Fi = fresnelDielectricExt(NdotL, c2, eta);
    V3<R> diff = kd;
    diff = diff / (splat(R(1)) - diff * fdrInt);
    weight = weight + (R(1) - Fi) * (R(1) - Fo) * diff * invEta2 * K<R>::INV_PI * NdotL;
  }
  return weight;
}
// 113-136 (parameter order of the definition)
template <class R>
R rpPdf(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, R ax, R ay, R eta, R ssw, uint32_t flags) {
  R pdf = R(0);
  R NdotL = dot(L, N), NdotV = dot(V, N);
  if (NdotL < R(0) || NdotV < R(0) || ((flags & EArea) == 0)) return pdf;
  R ct;
  R Fo = fresnelDielectricExt(NdotV, ct, eta);
  R substrateWeight = ssw * (R(1) - Fo);
  R specularWeight = Fo;
  R probSpecular = specularWeight / (specularWeight + substrateWeight);
  V3<R> wi = toLocal(X, Y, N, L), wo = toLocal(X, Y, N, V);
  V3<R> wh = makeNormal(wi + wo);
  R glossyPdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
  pdf = pdf + probSpecular * glossyPdf;
  R diffusePdf = cosineHemispherePdf(wi.z);
  pdf = pdf + (R(1) - probSpecular) * diffusePdf;
  return pdf;
}

// brdf_rough_plastic.rchit:191-269
template <class R> void shadeRoughPlastic(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  R eta = R(st.mat.ior);
  R fdrInt = R(st.mat.radiance[0]);
  R invEta2 = R(1) / (eta * eta);
  R ax = gmax(K<R>::EPS, R(st.mat.aniso_alpha[0]));
  R ay = gmax(K<R>::EPS, R(st.mat.aniso_alpha[1]));
  V3<R> kd = L3<R>(st.mat.diffuse);
  R ssw = luminance(kd);
  const V3<R> ks = splat(R(1));
  if (p.depth == 1 && sh.state.n_multi_channel > 0) {
    // The reference writes no AOV here (219-222 are commented out).
  }
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      // Reference call sites 234-240 pass (.., fdrInt, ax, ay, invEta2, ..)
      // into (.., fdrInt, invEta2, ax, ay, ..) and (.., eta, ax, ay, ..) into
      // (.., ax, ay, eta, ..): kept as written.
      V3<R> w = rpEval<R>(lRec.d, st.V, st.ffN, st.X, st.Y, kd, ks, eta, fdrInt, ax, ay, invEta2, EArea);
      R bpdf = rpPdf<R>(lRec.d, st.V, st.ffN, st.X, st.Y, eta, ax, ay, ssw, lRec.flags);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  // sampleBsdf 138-189
  V2<R> u = rnd2<R>(p.seed);
  V3<R> V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  V3<R> weight = splat(R(0));
  R bpdf = R(0);
  uint32_t bflags = EBsdfNull;
  V3<R> bd = splat(R(0));
  R NdotV = dot(V, N);
  if (NdotV > R(0)) {
    R ct;
    R Fo = fresnelDielectricExt(NdotV, ct, eta);
    R substrateWeight = ssw * (R(1) - Fo);
    R specularWeight = Fo;
    R probSpecular = specularWeight / (specularWeight + substrateWeight);
    if (u.x < probSpecular) {
      u.x = u.x / probSpecular;
      V3<R> wo = toLocal(X, Y, N, V);
      V3<R> wi = importanceSampleAnisoGGX(u, wo, ax, ay);
      V3<R> L = toWorld(X, Y, N, wi);
      bd = L;
      V3<R> H = makeNormal(V + L);
      V3<R> wh = makeNormal(wi + wo);
      R NdotL = dot(N, L);
      R ct2;
      R Fs = fresnelDielectricExt(dot(H, V), ct2, eta);
      R Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
      Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
      R Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
      bflags = EGlossyReflection;
      bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay) * probSpecular;
      weight = ks * Fs * Gs * Ds * NdotL;
    } else {
      u.x = (u.x - probSpecular) / (R(1) + K<R>::EPS - probSpecular);
      V3<R> wi = cosineSampleHemisphere(u);
      R ct2;
      R Fi = fresnelDielectricExt(wi.z, ct2, eta);
      V3<R> diff = kd;
      diff = diff / (splat(R(1)) - diff * fdrInt);
      bpdf = (R(1) - probSpecular) * cosineHemispherePdf(wi.z);
      bd = toWorld(X, Y, N, wi);
      bflags = EDiffuseReflection;
      weight = (R(1) - Fi) * (R(1) - Fo) * invEta2 * diff * K<R>::INV_PI * std::fabs(wi.z);
    }
  }
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

// bsdf_dielectric.rchit:12-24
template <class R> R dielectricFresnel(R cosThetaI, R eta) {
  R sinThetaTSq = eta * eta * (R(1) - cosThetaI * cosThetaI);
  if (sinThetaTSq > R(1)) return R(1);
  R cosThetaT = std::sqrt(gmax(R(1) - sinThetaTSq, R(0)));
  R rs = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
  R rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  return R(0.5) * (rs * rs + rp * rp);
}

// bsdf_dielectric.rchit:74-139
template <class R> void shadeDielectric(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  R eta = dot(st.V, st.N) > R(0) ? (R(1) / R(st.mat.ior)) : R(st.mat.ior);
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      // eval (26-38) with EArea: (EArea & EDelta) == 0 -> weight 0.
      V3<R> w = splat(R(0));
      // pdf (41-52)
      R bpdf = R(0);
      if (lRec.flags & EDelta) {
        V3<R> L = lRec.d, V = st.V, N = st.ffN;
        R F = dielectricFresnel(std::fabs(dot(V, N)), eta);
        if (dot(L, N) > R(0)) {
          if (std::fabs(dot(reflect(-V, N), L) - R(1)) < K<R>::EPS) bpdf = F;
        } else {
          if (std::fabs(dot(refract(-V, N, eta), L) - R(1)) < K<R>::EPS) bpdf = R(1) - F;
        }
      }
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  // sampleBsdf 54-72
  R u = rnd<R>(p.seed);
  V3<R> V = st.V, N = st.ffN;
  R F = dielectricFresnel(std::fabs(dot(V, N)), eta);
  V3<R> bd, weight;
  R bpdf;
  uint32_t bflags;
  if (u < F) {
    bd = makeNormal(reflect(-V, N));
    bpdf = F;
    bflags = ESpecularReflection;
    weight = F * splat(R(1));
  } else {
    bd = makeNormal(refract(-V, N, eta));
    bpdf = R(1) - F;
    bflags = ESpecularTransmission;
    weight = (R(1) - F) * splat(R(1)) * eta * eta;
  }
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, gsign(dot(bd, st.N)) * st.N);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

// brdf_plastic.rchit:43-61 (eval; the same fresnelDielectricExt as rough plastic)
template <class R>
V3<R> plEval(V3<R> L, V3<R> V, V3<R> N, V3<R> kd, R eta, R fdrInt, R invEta2, uint32_t flags) {
  V3<R> weight = splat(R(0));
  R NdotL = dot(L, N), NdotV = dot(V, N);
  if (NdotL < R(0) || NdotV < R(0)) return weight;
  R c0;
  R Fo = fresnelDielectricExt(NdotV, c0, eta);
  const bool hasSpecular = (flags & EDelta) != 0, hasDiffuse = (flags & EArea) != 0;
  if (hasSpecular) {
    if (std::fabs(dot(reflect(-V, N), L) - R(1)) < K<R>::EPS) weight = Fo * splat(R(1));
  } else if (hasDiffuse) {
    R c1;
    R Fi = fresnelDielectricExt(NdotL, c1, eta);
    V3<R> diff = kd;
    diff = diff / (splat(R(1)) - diff * fdrInt);
    weight = (R(1) - Fi) * (R(1) - Fo) * diff * invEta2 * K<R>::INV_PI * NdotL;
  }
  return weight;
}
// 63-84
template <class R> R plPdf(V3<R> L, V3<R> V, V3<R> N, R eta, R ssw, uint32_t flags) {
  R pdf = R(0);
  R NdotL = dot(L, N), NdotV = dot(V, N);
  if (NdotL < R(0) || NdotV < R(0)) return pdf;
  R c0;
  R Fo = fresnelDielectricExt(NdotV, c0, eta);
  const bool hasSpecular = (flags & EDelta) != 0, hasDiffuse = (flags & EArea) != 0;
  R probSpecular = (Fo * ssw) / (Fo * ssw + (R(1) - Fo) * (R(1) - ssw));
  if (hasSpecular) {
    if (std::fabs(dot(reflect(-V, N), L) - R(1)) < K<R>::EPS) pdf = probSpecular;
  } else if (hasDiffuse) {
    pdf = NdotL * (R(1) - probSpecular);  // no 1/pi, as in the reference
  }
  return pdf;
}

// brdf_plastic.rchit:122-205 (main) with sampleBsdf 86-120
template <class R> void shadePlastic(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  R eta = R(st.mat.ior);
  R fdrInt = R(st.mat.radiance[0]);
  V3<R> kd = L3<R>(st.mat.diffuse);
  R dAvg = luminance(kd), sAvg = luminance(splat(R(1)));
  R ssw = sAvg / (dAvg + sAvg);
  R invEta2 = R(1) / (eta * eta);
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> w = plEval<R>(lRec.d, st.V, st.ffN, kd, eta, fdrInt, invEta2, EArea);
      R bpdf = plPdf<R>(lRec.d, st.V, st.ffN, eta, ssw, lRec.flags);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  V2<R> u = rnd2<R>(p.seed);
  V3<R> V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  V3<R> weight = splat(R(0));
  R bpdf = R(0);
  uint32_t bflags = EBsdfNull;
  V3<R> bd = splat(R(0));
  R NdotV = dot(V, N);
  if (NdotV > R(0)) {
    R c0;
    R Fo = fresnelDielectricExt(NdotV, c0, eta);
    R probSpecular = (Fo * ssw) / (Fo * ssw + (R(1) - Fo) * (R(1) - ssw));
    if (u.x < probSpecular) {
      bd = makeNormal(reflect(-V, N));
      bflags = ESpecularReflection;
      bpdf = probSpecular;
      weight = splat(R(1)) * Fo;
    } else {
      u.x = (u.x - probSpecular) / (R(1) + K<R>::EPS - probSpecular);
      V3<R> wi = cosineSampleHemisphere(u);
      R c1;
      R Fi = fresnelDielectricExt(wi.z, c1, eta);
      V3<R> diff = kd;
      diff = diff / (splat(R(1)) - diff * fdrInt);
      bpdf = (R(1) - probSpecular) * cosineHemispherePdf(wi.z);
      bd = toWorld(X, Y, N, wi);
      bflags = EDiffuseReflection;
      weight = (R(1) - Fi) * (R(1) - Fo) * invEta2 * diff * K<R>::INV_PI * std::fabs(wi.z);
    }
  }
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

// brdf_mirror.rchit:40-106 (main): eval (12-19) is zero for area samples,
// pdf (21-26) is 1 on the mirror direction of a delta light; sampleBsdf 28-37.
template <class R> void shadeMirror(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  V3<R> kd = L3<R>(st.mat.diffuse);
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> w = splat(R(0));
      R bpdf = R(0);
      if ((lRec.flags & EDelta) != 0 && std::fabs(dot(reflect(-st.V, st.ffN), lRec.d) - R(1)) < K<R>::EPS)
        bpdf = R(1);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  const R bpdf = R(1);
  const V3<R> bd = reflect(-st.V, st.ffN);
  const V3<R> weight = kd;
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = ESpecularReflection;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / bpdf);
}

// brdf_phong.rchit:12-30 (flag is EArea at every call site)
template <class R> V3<R> phEval(V3<R> L, V3<R> V, V3<R> N, V3<R> kd, V3<R> ks, R n, uint32_t flags) {
  V3<R> weight = splat(R(0));
  if ((flags & EArea) == 0) return weight;
  R NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL < R(0) || NdotV < R(0)) return weight;
  V3<R> H = normalize(L + V);
  V3<R> diffuseLobe = kd * K<R>::INV_PI;
  V3<R> specularLobe = ks * mpow(gmax(dot(H, N), R(0)), n) * (n + R(2)) * K<R>::INV_2PI;
  R db = luminance(kd), sb = luminance(ks);
  R dw = db / (db + sb), sw = R(1) - dw;
  return (dw * diffuseLobe + sw * specularLobe) * NdotL;
}
// 32-37
template <class R> R phLobePdf(V3<R> L, V3<R> V, V3<R> N, R n) {
  V3<R> H = normalize(L + V);
  R NdotH = gmax(dot(H, N), R(0)), VdotH = gmax(dot(H, V), R(0));
  return (n + R(1)) * K<R>::INV_2PI * mpow(NdotH, n) * R(0.25) / (VdotH + K<R>::EPS);
}
// 39-52
template <class R> R phPdf(V3<R> L, V3<R> V, V3<R> N, V3<R> kd, V3<R> ks, R n, uint32_t flags) {
  if ((flags & EArea) == 0) return R(0);
  R db = luminance(kd), sb = luminance(ks);
  R dw = db / (db + sb), sw = R(1) - dw;
  return dw * cosineHemispherePdf(dot(N, L)) + sw * phLobePdf(L, V, N, n);
}

// brdf_phong.rchit:112-194 (main) with sampleBsdf 54-84; AOVs at depth 1
// (135-150) carry the shading-side normal and the specular reflectance.
template <class R> void shadePhong(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  const asuna_rt_state& ps = sh.state;
  V3<R> kd = L3<R>(st.mat.diffuse), ks = L3<R>(st.mat.rho_spec);
  R n = R(st.mat.specular);
  if (p.depth == 1) {
    if (ps.diffuse_out_channel >= 0) p.ch[ps.diffuse_out_channel] = kd;
    if (ps.normal_out_channel >= 0) p.ch[ps.normal_out_channel] = st.ffN;
    if (ps.specular_out_channel >= 0) p.ch[ps.specular_out_channel] = ks;
    if (ps.tangent_out_channel >= 0) p.ch[ps.tangent_out_channel] = st.X;
    if (ps.roughness_out_channel >= 0) p.ch[ps.roughness_out_channel] = V3<R>{R(1), R(1), R(0)};
    if (ps.position_out_channel >= 0) p.ch[ps.position_out_channel] = st.pos;
    if (ps.uv_out_channel >= 0) p.ch[ps.uv_out_channel] = V3<R>{st.uv.x, st.uv.y, R(1)};
  }
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> w = phEval<R>(lRec.d, st.V, st.ffN, kd, ks, n, EArea);
      R bpdf = phPdf<R>(lRec.d, st.V, st.ffN, kd, ks, n, lRec.flags);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  V2<R> u = rnd2<R>(p.seed);
  V3<R> V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  R db = luminance(kd), sb = luminance(ks);
  R dw = db / (db + sb), sw = R(1) - dw;
  V3<R> bd;
  R bpdf;
  uint32_t bflags;
  if (u.x < dw) {
    u.x = u.x / dw;
    V3<R> wi = cosineSampleHemisphere(u);
    bpdf = cosineHemispherePdf(wi.z);
    bd = toWorld(X, Y, N, wi);
    bflags = EDiffuseReflection;
  } else {
    u.x = (u.x - dw) / sw;
    R cosTheta = mpow(u.x, R(1) / (n + R(1)));
    R phi = K<R>::TWO_PI * u.y;
    R sinTheta = std::sqrt(gmax(R(0), R(1) - cosTheta * cosTheta));
    V3<R> wh{sinTheta * msin(phi), sinTheta * mcos(phi), cosTheta};
    V3<R> H = toWorld(X, Y, N, wh);
    bd = reflect(-V, H);
    bpdf = phLobePdf(bd, V, N, n);
    bflags = EGlossyReflection;
  }
  V3<R> weight = phEval<R>(bd, V, N, kd, ks, n, EArea);
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / bpdf);
}

// brdf_pbr_metalness_roughness.rchit:151-160 (brdf_disney.rchit:408-417,
// brdf_kang18.rchit:150-187 alike): with probability `opacity` the ray goes
// on from the far side of the surface in the same direction and the bounce
// is not counted (depth--); nothing else of the hit runs.
template <class R> bool passThrough(const Scene& s, PathState<R>& p, HitState<R>& st, R opacity) {
  if (st.mat.opacity_texture_id >= 0) opacity = texRGB(s, st.mat.opacity_texture_id, st.uv).x;
  if (!(rnd<R>(p.seed) < opacity)) return false;
  p.ro = offsetPositionAlongNormal(st.pos, -st.ffN);
  p.depth--;
  p.passed = true;
  return true;
}

// brdf_pbr_metalness_roughness.rchit:14-16 (GLSL mix: x (1 - a) + y a)
template <class R> V3<R> fresnelSchlick(R cosThetaI, V3<R> f0) {
  return f0 + (splat(R(1)) - f0) * mpow(gclamp(R(1) - cosThetaI, R(0), R(1)), R(5));
}
// 57-86 (the flags argument is unused: its test is commented out)
template <class R> V3<R> pbrEval(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, V3<R> albedo, R ax, R ay, R metalness,
                                 R eta) {
  V3<R> weight = splat(R(0));
  R NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= R(0) || NdotV <= R(0)) return weight;
  V3<R> H = makeNormal(L + V);
  R HdotN = dot(H, N), HdotX = dot(H, X), HdotY = dot(H, Y), HdotV = dot(H, V);
  R F0 = sqr((eta - R(1)) / (eta + R(1)));
  V3<R> f0 = splat(F0) * (R(1) - metalness) + albedo * metalness;
  V3<R> Fs = fresnelSchlick(HdotV, f0);
  R Ds = dAnisoGGX(HdotN, HdotX, HdotY, ax, ay);
  R Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
  Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
  V3<R> diffuse = albedo * (R(1) - metalness) * K<R>::INV_PI;
  V3<R> specular = Fs * Ds * Gs;
  weight = weight + diffuse;
  weight = weight + specular;
  weight = weight * NdotL;
  return weight;
}
// 88-105: a fixed 0.2 / 0.8 mixture of the cosine and GGX pdfs
template <class R> R pbrPdf(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, R ax, R ay, uint32_t flags) {
  R pdf = R(0);
  if ((flags & EArea) == 0) return pdf;
  R NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= R(0) || NdotV <= R(0)) return pdf;
  V3<R> H = makeNormal(L + V);
  V3<R> wh = makeNormal(toLocal(X, Y, N, H)), wo = makeNormal(toLocal(X, Y, N, V)),
        wi = makeNormal(toLocal(X, Y, N, L));
  pdf = pdf + R(0.2f) * cosineHemispherePdf(wi.z);
  pdf = pdf + (R(1) - R(0.2f)) * importanceAnisoGGXPdf(wh, wo, ax, ay);
  return pdf;
}

// brdf_pbr_metalness_roughness.rchit:131-219 (main) with sampleBsdf 107-129.
// Random numbers in order: the opacity test, the light sample, the direction
// pair, then the lobe choice.  The sampled direction's pdf is that of the
// chosen lobe alone and its weight carries a second |cos| (as written).
// AOVs at depth 1: albedo and the face-forward normal only.
template <class R> void shadePbr(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  const asuna_rt_state& ps = sh.state;
  V3<R> albedo = L3<R>(st.mat.diffuse);
  R metalness = R(st.mat.metalness), roughness = R(st.mat.roughness);
  R opacity = R(st.mat.specular);
  if (passThrough(s, p, st, opacity)) return;
  R ax = gmax(sqr(roughness), R(0.001f)), ay = ax;
  R eta = R(st.mat.ior);
  if (p.depth == 1) {
    if (ps.diffuse_out_channel >= 0) p.ch[ps.diffuse_out_channel] = albedo;
    if (ps.normal_out_channel >= 0) p.ch[ps.normal_out_channel] = st.ffN;
  }
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> w = pbrEval<R>(lRec.d, st.V, st.ffN, st.X, st.Y, albedo, ax, ay, metalness, eta);
      R bpdf = pbrPdf<R>(lRec.d, st.V, st.ffN, st.X, st.Y, ax, ay, lRec.flags);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  V2<R> u = rnd2<R>(p.seed);
  V3<R> V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  V3<R> wo = makeNormal(toLocal(X, Y, N, V));
  V3<R> wi;
  R bpdf = R(0);
  uint32_t bflags;
  if (rnd<R>(p.seed) < R(0.2f)) {
    wi = cosineSampleHemisphere(u);
    bflags = EDiffuseReflection;
    bpdf = cosineHemispherePdf(wi.z);
  } else {
    wi = importanceSampleAnisoGGX(u, wo, ax, ay);
    V3<R> wh = makeNormal(wi + wo);
    bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
    bflags = EGlossyReflection;
  }
  V3<R> bd = toWorld(X, Y, N, wi);
  V3<R> weight = pbrEval<R>(bd, V, N, X, Y, albedo, ax, ay, metalness, eta) * std::fabs(wi.z);
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

// ---- brdf_disney.rchit -------------------------------------------------------
// GLSL mix of scalars: x (1 - a) + y a
template <class R> inline R gmix(R x, R y, R a) { return x * (R(1) - a) + y * a; }
template <class R> inline V3<R> gmix3(V3<R> x, V3<R> y, R a) { return x * (R(1) - a) + y * a; }
// 31-48
template <class R> struct DisneyMat {
  V3<R> baseColor;
  R anisotropic, metallic, roughness, subsurface, specularTint, sheen, sheenTint, clearcoat, clearcoatRoughness, ior,
      opacity, ax, ay;
};
// 50-52
template <class R> R dLuminance(V3<R> c) { return R(0.212671f) * c.x + R(0.715160f) * c.y + R(0.072169f) * c.z; }
// 54-59
template <class R> R GTR1(R NDotH, R a) {
  if (a >= R(1)) return K<R>::INV_PI;
  R a2 = a * a;
  R t = R(1) + (a2 - R(1)) * NDotH * NDotH;
  return (a2 - R(1)) / (K<R>::PI * mlog(a2) * t);
}
// 61-74: the polar angle uses r1 as well (r2 is unused, as written)
template <class R> V3<R> SampleGTR1(R rgh, R r1, R r2) {
  (void)r2;
  R a = gmax(R(0.001f), rgh);
  R a2 = a * a;
  R phi = r1 * K<R>::TWO_PI;
  R cosTheta = std::sqrt((R(1) - mpow(a2, R(1) - r1)) / (R(1) - a2));
  R sinTheta = gclamp(std::sqrt(R(1) - (cosTheta * cosTheta)), R(0), R(1));
  R sinPhi = msin(phi), cosPhi = mcos(phi);
  return V3<R>{sinTheta * cosPhi, sinTheta * sinPhi, cosTheta};
}
// 95-114 (Heitz 2018, visible normals)
template <class R> V3<R> SampleGGXVNDF(V3<R> V, R ax, R ay, R r1, R r2) {
  V3<R> Vh = normalize(V3<R>{ax * V.x, ay * V.y, V.z});
  R lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  V3<R> T1 = lensq > R(0) ? V3<R>{-Vh.y, Vh.x, R(0)} * (R(1) / std::sqrt(lensq)) : V3<R>{R(1), R(0), R(0)};
  V3<R> T2 = cross(Vh, T1);
  R r = std::sqrt(r1);
  R phi = R(2.0f * 3.14159265358979323846f) * r2;
  R t1 = r * mcos(phi);
  R t2 = r * msin(phi);
  R sv = R(0.5f) * (R(1) + Vh.z);
  t2 = (R(1) - sv) * std::sqrt(R(1) - t1 * t1) + sv * t2;
  V3<R> Nh = t1 * T1 + t2 * T2 + std::sqrt(gmax(R(0), R(1) - t1 * t1 - t2 * t2)) * Vh;
  return normalize(V3<R>{ax * Nh.x, ay * Nh.y, gmax(R(0), Nh.z)});
}
// 116-121
template <class R> R GTR2Aniso(R NDotH, R HDotX, R HDotY, R ax, R ay) {
  R a = HDotX / ax, b = HDotY / ay;
  R c = a * a + b * b + NDotH * NDotH;
  return R(1) / (K<R>::PI * ax * ay * c * c);
}
// 133-137
template <class R> R SmithG(R NDotV, R alphaG) {
  R a = alphaG * alphaG, b = NDotV * NDotV;
  return (R(2) * NDotV) / (NDotV + std::sqrt(a + b - a * b));
}
// 139-144
template <class R> R SmithGAniso(R NDotV, R VDotX, R VDotY, R ax, R ay) {
  R a = VDotX * ax, b = VDotY * ay, c = NDotV;
  return (R(2) * NDotV) / (NDotV + std::sqrt(a * a + b * b + c * c));
}
// 146-150
template <class R> R SchlickFresnel(R u) {
  R m = gclamp(R(1) - u, R(0), R(1));
  R m2 = m * m;
  return m2 * m2 * m;
}
// 152-164
template <class R> R DisneyDielectricFresnel(R cosThetaI, R eta) {
  R sinThetaTSq = eta * eta * (R(1) - cosThetaI * cosThetaI);
  if (sinThetaTSq > R(1)) return R(1);
  R cosThetaT = std::sqrt(gmax(R(1) - sinThetaTSq, R(0)));
  R rs = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
  R rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
  return R(0.5f) * (rs * rs + rp * rp);
}
// 166-170
template <class R> R DisneyFresnel(R metallic, R eta, R LDotH, R VDotH) {
  R metallicFresnel = SchlickFresnel(LDotH);
  R dielectricFresnel = DisneyDielectricFresnel(std::fabs(VDotH), eta);
  return gmix(dielectricFresnel, metallicFresnel, metallic);
}
// 172-195
template <class R> V3<R> EvalDiffuse(const DisneyMat<R>& mat, V3<R> Csheen, V3<R> V, V3<R> L, V3<R> H, R& pdf) {
  pdf = R(0);
  if (L.z <= R(0)) return splat(R(0));
  R FL = SchlickFresnel(L.z), FV = SchlickFresnel(V.z), FH = SchlickFresnel(dot(L, H));
  R Fd90 = R(0.5f) + R(2) * dot(L, H) * dot(L, H) * mat.roughness;
  R Fd = gmix(R(1), Fd90, FL) * gmix(R(1), Fd90, FV);
  R Fss90 = dot(L, H) * dot(L, H) * mat.roughness;
  R Fss = gmix(R(1), Fss90, FL) * gmix(R(1), Fss90, FV);
  R ss = R(1.25f) * (Fss * (R(1) / (L.z + V.z) - R(0.5f)) + R(0.5f));
  V3<R> Fsheen = FH * mat.sheen * Csheen;
  pdf = L.z * K<R>::INV_PI;
  return (R(1) - mat.metallic) * (K<R>::INV_PI * gmix(Fd, ss, mat.subsurface) * mat.baseColor + Fsheen);
}
// 197-211
template <class R>
V3<R> EvalSpecReflection(const DisneyMat<R>& mat, R eta, V3<R> specCol, V3<R> V, V3<R> L, V3<R> H, R& pdf) {
  pdf = R(0);
  if (L.z <= R(0)) return splat(R(0));
  R FM = DisneyFresnel(mat.metallic, eta, dot(L, H), dot(V, H));
  V3<R> F = gmix3(specCol, splat(R(1)), FM);
  R D = GTR2Aniso(H.z, H.x, H.y, mat.ax, mat.ay);
  R G1 = SmithGAniso(std::fabs(V.z), V.x, V.y, mat.ax, mat.ay);
  R G2 = G1 * SmithGAniso(std::fabs(L.z), L.x, L.y, mat.ax, mat.ay);
  pdf = G1 * D / (R(4) * V.z);
  return F * D * G2 / (R(4) * L.z * V.z);
}
// 213-226
template <class R> V3<R> EvalClearcoat(const DisneyMat<R>& mat, V3<R> V, V3<R> L, V3<R> H, R& pdf) {
  pdf = R(0);
  if (L.z <= R(0)) return splat(R(0));
  R FH = DisneyDielectricFresnel(dot(V, H), R(1.0f / 1.5f));
  R F = gmix(R(0.04f), R(1), FH);
  R D = GTR1(H.z, mat.clearcoatRoughness);
  R G = SmithG(L.z, R(0.25f)) * SmithG(V.z, R(0.25f));
  R jacobian = R(1) / (R(4) * dot(V, H));
  pdf = D * H.z * jacobian;
  return splat(R(0.25f)) * mat.clearcoat * F * D * G / (R(4) * L.z * V.z);
}
// 228-236
template <class R> void GetSpecColor(const DisneyMat<R>& mat, R eta, V3<R>& specCol, V3<R>& sheenCol) {
  R lum = dLuminance(mat.baseColor);
  V3<R> ctint = lum > R(0) ? mat.baseColor / lum : splat(R(1));
  R F0 = (R(1) - eta) / (R(1) + eta);
  specCol = gmix3(F0 * F0 * gmix3(splat(R(1)), ctint, mat.specularTint), mat.baseColor, mat.metallic);
  sheenCol = gmix3(splat(R(1)), ctint, mat.sheenTint);
}
// 238-250
template <class R>
void GetLobeProbabilities(const DisneyMat<R>& mat, V3<R> specCol, R approxFresnel, R& diffuseWt, R& specReflectWt,
                          R& clearcoatWt) {
  diffuseWt = dLuminance(mat.baseColor) * (R(1) - mat.metallic);
  specReflectWt = dLuminance(gmix3(specCol, splat(R(1)), approxFresnel));
  clearcoatWt = R(0.25f) * mat.clearcoat * (R(1) - mat.metallic);
  R totalWt = diffuseWt + specReflectWt + clearcoatWt;
  diffuseWt = diffuseWt / totalWt;
  specReflectWt = specReflectWt / totalWt;
  clearcoatWt = clearcoatWt / totalWt;
}
// 252-300 (flags is EArea at both call sites)
template <class R>
V3<R> disneyEval(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, const DisneyMat<R>& mat, R eta, R& bsdfPdf) {
  V3<R> weight = splat(R(0));
  bsdfPdf = R(0);
  V = toLocal(X, Y, N, V);
  L = toLocal(X, Y, N, L);
  if (L.z <= R(0) || V.z <= R(0)) return weight;
  V3<R> H = normalize(L + V);
  if (H.z < R(0)) H = -H;
  V3<R> specCol, sheenCol;
  GetSpecColor(mat, eta, specCol, sheenCol);
  R diffuseWt, specReflectWt, clearcoatWt;
  R fresnel = DisneyFresnel(mat.metallic, eta, dot(L, H), dot(V, H));
  GetLobeProbabilities(mat, specCol, fresnel, diffuseWt, specReflectWt, clearcoatWt);
  R pdf = R(0);
  if (diffuseWt > R(0) && L.z > R(0)) {
    weight = weight + EvalDiffuse(mat, sheenCol, V, L, H, pdf);
    bsdfPdf = bsdfPdf + pdf * diffuseWt;
  }
  if (specReflectWt > R(0) && L.z > R(0) && V.z > R(0)) {
    weight = weight + EvalSpecReflection(mat, eta, specCol, V, L, H, pdf);
    bsdfPdf = bsdfPdf + pdf * specReflectWt;
  }
  if (clearcoatWt > R(0) && L.z > R(0) && V.z > R(0)) {
    weight = weight + EvalClearcoat(mat, V, L, H, pdf);
    bsdfPdf = bsdfPdf + pdf * clearcoatWt;
  }
  return weight * L.z;
}

// brdf_disney.rchit:380-477 (main) with sampleBsdf 302-378.  Random numbers:
// the opacity test, the light sample, the direction pair.  No AOVs (the
// depth-1 block is commented out).  The sampled weight is scaled by
// |dot(N, L)| with N in world and L in the local frame, as written.
template <class R> void shadeDisney(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  const asuna_material& m = st.mat;
  R opacity = R(m.rho_spec[0]);
  if (passThrough(s, p, st, opacity)) return;
  DisneyMat<R> mat;
  {
    R rough = R(m.roughness);
    R aspect = std::sqrt(R(1) - R(m.anisotropic) * R(0.9f));
    mat.ax = gmax(R(0.001f), rough * rough / aspect);
    mat.ay = gmax(R(0.001f), rough * rough * aspect);
    mat.baseColor = L3<R>(m.diffuse);
    mat.anisotropic = R(m.anisotropic);
    mat.metallic = R(m.metalness);
    mat.roughness = gmax(rough * rough, R(0.001f));
    mat.subsurface = R(m.subsurface);
    mat.specularTint = R(m.specular_tint);
    mat.sheen = R(m.sheen);
    mat.sheenTint = R(m.sheen_tint);
    mat.clearcoat = R(m.clearcoat);
    mat.clearcoatRoughness = gmix(R(0.1f), R(0.001f), R(m.clearcoat_gloss));
    mat.ior = R(m.ior);
    mat.opacity = opacity;
  }
  R eta = dot(st.V, st.N) > R(0) ? (R(1) / mat.ior) : mat.ior;
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      R bpdf;
      V3<R> w = disneyEval<R>(lRec.d, st.V, st.ffN, st.X, st.Y, mat, eta, bpdf);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  V2<R> u = rnd2<R>(p.seed);
  R pdf = R(0);
  V3<R> f = splat(R(0));
  R r1 = u.x, r2 = u.y;
  V3<R> N = st.ffN, X = st.X, Y = st.Y;
  V3<R> V = toLocal(X, Y, N, st.V);
  V3<R> L;
  V3<R> specCol, sheenCol;
  GetSpecColor(mat, eta, specCol, sheenCol);
  R diffuseWt, specReflectWt, clearcoatWt;
  R approxFresnel = DisneyFresnel(mat.metallic, eta, V.z, V.z);
  GetLobeProbabilities(mat, specCol, approxFresnel, diffuseWt, specReflectWt, clearcoatWt);
  R cdf0 = diffuseWt;
  R cdf1 = cdf0 + clearcoatWt;
  uint32_t bflags;
  if (r1 < cdf0) {
    r1 = r1 / cdf0;
    L = cosineSampleHemisphere(V2<R>{r1, r2});
    V3<R> H = normalize(L + V);
    f = EvalDiffuse(mat, sheenCol, V, L, H, pdf);
    pdf = pdf * diffuseWt;
    bflags = EDiffuseReflection;
  } else if (r1 < cdf1) {
    r1 = (r1 - cdf0) / (cdf1 - cdf0);
    V3<R> H = SampleGTR1(mat.clearcoatRoughness, r1, r2);
    if (H.z < R(0)) H = -H;
    L = normalize(reflect(-V, H));
    f = EvalClearcoat(mat, V, L, H, pdf);
    pdf = pdf * clearcoatWt;
    bflags = EGlossyReflection;
  } else {
    r1 = (r1 - cdf1) / (R(1) - cdf1);
    V3<R> H = SampleGGXVNDF(V, mat.ax, mat.ay, r1, r2);
    if (H.z < R(0)) H = -H;
    L = normalize(reflect(-V, H));
    f = EvalSpecReflection(mat, eta, specCol, V, L, H, pdf);
    pdf = pdf * specReflectWt;
    bflags = EGlossyReflection;
  }
  V3<R> bd = toWorld(X, Y, N, L);
  V3<R> weight = f * std::fabs(dot(N, L));
  if (pdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = pdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / pdf);
}

// ---- brdf_kang18.rchit ------------------------------------------------------
// 57-86 (flags unused): anisotropic GGX with Schlick Fresnel plus Lambertian
template <class R>
V3<R> kangEval(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, V3<R> kd, V3<R> ks, R ax, R ay, R eta) {
  V3<R> weight = splat(R(0));
  R NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= R(0) || NdotV <= R(0)) return weight;
  V3<R> H = makeNormal(L + V);
  R HdotN = dot(H, N), HdotX = dot(H, X), HdotY = dot(H, Y), HdotV = dot(H, V);
  R F0 = sqr((eta - R(1)) / (eta + R(1)));
  R Fs = F0 + (R(1) - F0) * mpow(gclamp(R(1) - HdotV, R(0), R(1)), R(5));
  R Ds = dAnisoGGX(HdotN, HdotX, HdotY, ax, ay);
  R Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
  Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
  V3<R> diffuse = kd * K<R>::INV_PI;
  V3<R> specular = ks * Fs * Ds * Gs;
  weight = weight + diffuse;
  weight = weight + specular;
  weight = weight * NdotL;
  return weight;
}
// 88-111: lobe probability pd / (pd + ps + EPS) from the two luminances
template <class R> R kangDiffuseProb(V3<R> kd, V3<R> ks) {
  R pd = dLuminance(kd), ps = dLuminance(ks);
  return pd / (pd + ps + K<R>::EPS);
}
template <class R>
R kangPdf(V3<R> L, V3<R> V, V3<R> N, V3<R> X, V3<R> Y, R ax, R ay, V3<R> kd, V3<R> ks, uint32_t flags) {
  R pdf = R(0);
  if ((flags & EArea) == 0) return pdf;
  R NdotL = dot(N, L), NdotV = dot(N, V);
  if (NdotL <= R(0) || NdotV <= R(0)) return pdf;
  V3<R> H = makeNormal(L + V);
  V3<R> wh = makeNormal(toLocal(X, Y, N, H)), wo = makeNormal(toLocal(X, Y, N, V)),
        wi = makeNormal(toLocal(X, Y, N, L));
  R dp = kangDiffuseProb(kd, ks);
  pdf = pdf + dp * cosineHemispherePdf(wi.z);
  pdf = pdf + (R(1) - dp) * importanceAnisoGGXPdf(wh, wo, ax, ay);
  return pdf;
}

// brdf_kang18.rchit:137-249 (main) with sampleBsdf 113-135.  The tangent
// frame is rebuilt from N and X before anything else (178-181); random
// numbers: the opacity test, the light sample, the direction pair, the lobe
// choice; the sampled pdf is that of the chosen lobe.
template <class R> void shadeKang18(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  const asuna_rt_state& ps = sh.state;
  V3<R> kd = L3<R>(st.mat.diffuse), ks = L3<R>(st.mat.rho_spec);
  R opacity = R(st.mat.metalness);
  st.Y = makeNormal(cross(st.N, st.X));
  st.X = makeNormal(cross(st.Y, st.N));
  st.ffN = dot(st.N, st.V) > R(0) ? st.N : -st.N;
  if (passThrough(s, p, st, opacity)) return;
  R ax = gmax(R(st.mat.aniso_alpha[0]), K<R>::EPS), ay = gmax(R(st.mat.aniso_alpha[1]), K<R>::EPS);
  R eta = R(st.mat.ior);
  if (p.depth == 1) {
    if (ps.diffuse_out_channel >= 0) p.ch[ps.diffuse_out_channel] = kd;
    if (ps.normal_out_channel >= 0) p.ch[ps.normal_out_channel] = st.ffN;
    if (ps.specular_out_channel >= 0) p.ch[ps.specular_out_channel] = ks;
    if (ps.tangent_out_channel >= 0) p.ch[ps.tangent_out_channel] = st.X;
    if (ps.roughness_out_channel >= 0) p.ch[ps.roughness_out_channel] = V3<R>{ax, ay, R(0)};
    if (ps.position_out_channel >= 0) p.ch[ps.position_out_channel] = st.pos;
    if (ps.uv_out_channel >= 0) p.ch[ps.uv_out_channel] = V3<R>{st.uv.x, st.uv.y, R(1)};
  }
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> w = kangEval<R>(lRec.d, st.V, st.ffN, st.X, st.Y, kd, ks, ax, ay, eta);
      R bpdf = kangPdf<R>(lRec.d, st.V, st.ffN, st.X, st.Y, ax, ay, kd, ks, lRec.flags);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  V2<R> u = rnd2<R>(p.seed);
  V3<R> V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  V3<R> wo = makeNormal(toLocal(X, Y, N, V));
  R dp = kangDiffuseProb(kd, ks);
  V3<R> wi;
  R bpdf = R(0);
  uint32_t bflags;
  if (rnd<R>(p.seed) < dp) {
    wi = cosineSampleHemisphere(u);
    bflags = EDiffuseReflection;
    bpdf = cosineHemispherePdf(wi.z);
  } else {
    wi = importanceSampleAnisoGGX(u, wo, ax, ay);
    V3<R> wh = makeNormal(wi + wo);
    bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
    bflags = EGlossyReflection;
  }
  V3<R> bd = toWorld(X, Y, N, wi);
  V3<R> weight = kangEval<R>(bd, V, N, X, Y, kd, ks, ax, ay, eta);
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = bflags;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

// brdf_conductor.rchit:14-36 (P. Shirley's conductor Fresnel)
template <class R> R conductorReflectance(R eta, R k, R cosThetaI) {
  R cosThetaISq = cosThetaI * cosThetaI;
  R sinThetaISq = gmax(R(1) - cosThetaISq, R(0));
  R sinThetaIQu = sinThetaISq * sinThetaISq;
  R innerTerm = eta * eta - k * k - sinThetaISq;
  R aSqPlusBSq = std::sqrt(gmax(innerTerm * innerTerm + R(4) * eta * eta * k * k, R(0)));
  R a = std::sqrt(gmax((aSqPlusBSq + innerTerm) * R(0.5), R(0)));
  R Rs = ((aSqPlusBSq + cosThetaISq) - (R(2) * a * cosThetaI)) / ((aSqPlusBSq + cosThetaISq) + (R(2) * a * cosThetaI));
  R Rp = ((cosThetaISq * aSqPlusBSq + sinThetaIQu) - (R(2) * a * cosThetaI * sinThetaISq)) /
         ((cosThetaISq * aSqPlusBSq + sinThetaIQu) + (R(2) * a * cosThetaI * sinThetaISq));
  return R(0.5) * (Rs + Rs * Rp);
}
template <class R> V3<R> conductorReflectance3(V3<R> eta, V3<R> k, R c) {
  return V3<R>{conductorReflectance(eta.x, k.x, c), conductorReflectance(eta.y, k.y, c),
               conductorReflectance(eta.z, k.z, c)};
}

// brdf_conductor.rchit:83-164 (main), eval 38-51, pdf 53-63, sampleBsdf 65-80
template <class R> void shadeConductor(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  V3<R> kd = L3<R>(st.mat.diffuse), eta = L3<R>(st.mat.radiance), k = L3<R>(st.mat.radiance_factor);
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> w = splat(R(0));  // eval with EArea is zero
      R bpdf = R(0);
      R NdotL = dot(lRec.d, st.ffN), NdotV = dot(st.V, st.ffN);
      if (!(NdotL < R(0) || NdotV < R(0) || ((lRec.flags & EDelta) == 0)))
        if (std::fabs(dot(reflect(-st.V, st.ffN), lRec.d) - R(1)) < K<R>::EPS) bpdf = R(1);
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  rnd2<R>(p.seed);  // drawn and unused (sampleBsdf ignores u)
  V3<R> weight = splat(R(0));
  R bpdf = R(0);
  V3<R> bd = splat(R(0));
  if (dot(st.V, st.ffN) > R(0)) {
    bd = reflect(-st.V, st.ffN);
    bpdf = R(1);
    weight = kd * conductorReflectance3(eta, k, dot(st.ffN, bd));
  }
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = ESpecularReflection;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

// brdf_rough_conductor.rchit:133-206 (main), eval 72-88, pdf 90-101,
// sampleBsdf 103-131; the Fresnel term is taken at N.L, as written there
template <class R> void shadeRoughConductor(const Scene& s, const asuna_shot& sh, PathState<R>& p, HitState<R>& st) {
  V3<R> kd = L3<R>(st.mat.diffuse), eta = L3<R>(st.mat.radiance), k = L3<R>(st.mat.radiance_factor);
  R ax = gmax(R(st.mat.aniso_alpha[0]), K<R>::EPS);
  R ay = gmax(R(st.mat.aniso_alpha[1]), K<R>::EPS);
  V3<R> V = st.V, N = st.ffN, X = st.X, Y = st.Y;
  {
    bool visible;
    LRec<R> lRec;
    V3<R> Ld = splat(R(0));
    V3<R> rad = sampleLights<R>(s, sh, p, st.pos, st.ffN, visible, lRec);
    if (visible) {
      V3<R> L = lRec.d;
      V3<R> w = splat(R(0));
      R NdotL = dot(L, N), NdotV = dot(V, N);
      if (!(NdotL < R(0) || NdotV < R(0))) {
        V3<R> H = makeNormal(L + V);
        V3<R> Fs = conductorReflectance3(eta, k, NdotL);
        R Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
        Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
        R Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
        w = w + kd * Fs * Gs * Ds * NdotL;
      }
      R bpdf = R(0);
      if (!(NdotL < R(0) || NdotV < R(0) || ((lRec.flags & EArea) == 0))) {
        V3<R> wi = toLocal(X, Y, N, L), wo = toLocal(X, Y, N, V);
        V3<R> wh = makeNormal(wi + wo);
        bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
      }
      R mis = powerHeuristic(lRec.pdf, bpdf);
      Ld = Ld + mis * w * rad * p.throughput / (lRec.pdf + K<R>::EPS);
    }
    p.drad = Ld;
    p.dskip = !visible;
  }
  V2<R> u = rnd2<R>(p.seed);
  V3<R> weight = splat(R(0));
  R bpdf = R(0);
  V3<R> bd = splat(R(0));
  R NdotV = dot(V, N);
  if (NdotV > R(0)) {
    V3<R> wo = toLocal(X, Y, N, V);
    V3<R> wi = importanceSampleAnisoGGX(u, wo, ax, ay);
    V3<R> L = toWorld(X, Y, N, wi);
    bd = L;
    V3<R> H = makeNormal(V + L);
    V3<R> wh = makeNormal(wi + wo);
    R NdotL = dot(N, L);
    V3<R> Fs = conductorReflectance3(eta, k, NdotL);
    R Gs = g1SmithAnisoGGX(NdotV, dot(V, X), dot(V, Y), ax, ay);
    Gs = Gs * g1SmithAnisoGGX(NdotL, dot(L, X), dot(L, Y), ax, ay);
    R Ds = dAnisoGGX(dot(H, N), dot(H, X), dot(H, Y), ax, ay);
    bpdf = importanceAnisoGGXPdf(wh, wo, ax, ay);
    weight = kd * Fs * Gs * Ds * NdotL;
  }
  if (bpdf <= R(0) || length(weight) == R(0)) {
    p.stop = true;
    return;
  }
  p.bflags = EGlossyReflection;
  p.bpdf = bpdf;
  p.ro = offsetPositionAlongNormal(st.pos, st.ffN);
  p.rd = bd;
  p.throughput = p.throughput * (weight / (bpdf + K<R>::EPS));
}

struct PathOut {
  float rad[3];
  float fw;
  uint32_t depth, sig, events, shadows;
  float t1;
  float ch[ASUNA_MAX_CHANNELS][3];
  double radd[3];
};

inline uint32_t hashFrame(uint32_t frame, uint32_t seed) { return frame + seed * 0x9E3779B9u; }

template <class R>
void tracePath(const Scene& s, const asuna_shot& sh, uint32_t x, uint32_t y, uint32_t frame, PathOut& out,
               TravStats* st, uint64_t& nExt, uint64_t& nShadow) {
  const asuna_camera& cam = sh.camera;
  const asuna_rt_state& ps = sh.state;
  PathState<R> p;
  // raytrace.projective.rgen:26-100
  p.seed = xxhash32(x, y, hashFrame(frame, sh.seed));
  V3<R> origin = transformPoint<R>(cam.camera_to_world, splat(R(0)));
  V2<R> jitter = (frame == 0) ? V2<R>{R(0.5), R(0.5)} : rnd2<R>(p.seed);
  V2<R> pixel{R(x) + jitter.x, R(y) + jitter.y};
  V3<R> ro = origin, rd = splat(R(0));
  if (cam.type == ASUNA_CAMERA_PERSPECTIVE) {
    V3<R> pCamera = transformPoint<R>(cam.raster_to_camera, V3<R>{pixel.x, pixel.y, R(0)});
    V3<R> r = makeNormal(pCamera);
    if (cam.aperture > 0.0f) {
      V2<R> uLens = rnd2<R>(p.seed);
      V2<R> d = concentricSampleDisk(uLens);
      V2<R> pLens{R(cam.aperture) * d.x, R(cam.aperture) * d.y};
      R ft = R(cam.focal_distance) / r.z;
      V3<R> pFocus = ft * r;
      V3<R> o{pLens.x, pLens.y, R(0)};
      ro = transformPoint<R>(cam.camera_to_world, o);
      r = pFocus - o;
    }
    rd = transformDirection<R>(cam.camera_to_world, r);
  } else if (cam.type == ASUNA_CAMERA_OPENCV) {
    R px = (pixel.x - R(cam.fxfycxcy[2])) / R(cam.fxfycxcy[0]);
    R py = (pixel.y - R(cam.fxfycxcy[3])) / R(cam.fxfycxcy[1]);
    rd = transformDirection<R>(cam.camera_to_world, V3<R>{px, py, R(1)});
  }
  p.ro = ro;
  p.rd = rd;
  p.stop = false;
  p.radiance = splat(R(0));
  p.throughput = splat(R(1));
  p.bflags = EBsdfNull;
  p.bpdf = R(0);
  for (int i = 0; i < ASUNA_MAX_CHANNELS; ++i) p.ch[i] = splat(R(0));
  p.sig = 0;
  uint32_t events = 0, shadows = 0;
  R t1 = R(0);  // primary-hit distance (depth channel, an extension)
  const bool rr = (sh.flags & ASUNA_SHOT_RR) != 0;
  // rgen:102-132; the wavefront runs at most max_path_depth +
  // ASUNA_MAX_PASS_THROUGH passes, and so does this loop
  uint32_t iters = 0;
  for (p.depth = 1; p.depth <= uint32_t(ps.max_path_depth);) {
    if (++iters > uint32_t(ps.max_path_depth) + ASUNA_MAX_PASS_THROUGH) break;
    p.dskip = true;
    p.passed = false;
    p.drad = splat(R(0));
    float of[3] = {float(p.ro.x), float(p.ro.y), float(p.ro.z)}, df[3] = {float(p.rd.x), float(p.rd.y), float(p.rd.z)};
    Hit h;
    nExt++;
    bool hit = traceScene(s, of, df, float(K<float>::MINIMUM), float(K<float>::INF), false, h, st);
    if (!hit) {
      // raytrace.default.rmiss:24-56
      p.stop = true;
      V3<R> env;
      if (s.sky)
        env = sunSky<R>(s, p.rd);
      else if (ps.has_env_map == 1)
        env = evalEnvmap<R>(s, sh, p.rd);
      else
        env = L3<R>(ps.bg_color);
      R mis = R(1);
      if (p.depth != 1 && isNonSpecular(p.bflags)) {
        R envPdf = s.sky ? K<R>::INV_4PI : (ps.has_env_map == 1) ? pdfEnvmap<R>(s, sh, p.rd) : K<R>::INV_4PI;
        mis = powerHeuristic(p.bpdf, envPdf);
      }
      p.radiance = p.radiance + p.throughput * env * mis;
      p.sig = sigMix(p.sig, 0xffffffffu);
    } else {
      HitState<R> hs = getHitState<R>(s, sh, p, h);
      p.sig = sigMix(p.sig, (h.inst << 20) ^ h.prim);
      if (p.depth == 1) t1 = R(h.t);
      if (hs.lightId >= 0) {
        hitLight<R>(s, p, hs.lightId, hs.pos);
      } else {
        applyTextures<R>(s, sh, hs);
        uint32_t type = hs.mat.type;
        if (type == ASUNA_MAT_EMISSIVE) {
          // brdf_emissive.rchit:12-27
          p.stop = true;
          if (ps.ignore_emissive == 0) p.radiance = p.radiance + L3<R>(hs.mat.radiance) * p.throughput;
        } else if (type == ASUNA_MAT_ROUGH_PLASTIC)
          shadeRoughPlastic<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_DIELECTRIC)
          shadeDielectric<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_PLASTIC)
          shadePlastic<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_MIRROR)
          shadeMirror<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_CONDUCTOR)
          shadeConductor<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_ROUGH_CONDUCTOR)
          shadeRoughConductor<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_PHONG)
          shadePhong<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_PBR_METALNESS_ROUGHNESS)
          shadePbr<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_DISNEY)
          shadeDisney<R>(s, sh, p, hs);
        else if (type == ASUNA_MAT_KANG18)
          shadeKang18<R>(s, sh, p, hs);
        else
          shadeLambertian<R>(s, sh, p, hs);
        p.sig = sigMix(p.sig, p.stop ? 0xfffu : p.bflags);
      }
    }
    // rgen:111-127
    if (!p.dskip) {
      float o2[3] = {float(p.dro.x), float(p.dro.y), float(p.dro.z)},
            d2[3] = {float(p.drd.x), float(p.drd.y), float(p.drd.z)};
      float maxDist = float(p.ddist - R(2) * K<R>::EPS);
      nShadow++;
      shadows |= 1u << (p.depth - 1);
      Hit sh2;
      if (!traceScene(s, o2, d2, 0.0f, maxDist, true, sh2, st)) {
        p.radiance = p.radiance + p.drad;
        events |= 1u << (p.depth - 1);
      }
    }
    if (p.stop) break;
    // Russian roulette (extension, off for the reference's streams).
    if (rr && !p.passed && p.depth >= sh.rr_depth) {
      R q = gmin(R(0.95), gmax(p.throughput.x, gmax(p.throughput.y, p.throughput.z)));
      R u = rnd<R>(p.seed);
      if (!(u < q)) break;
      p.throughput = p.throughput / q;
    }
    p.depth++;
  }
  if (p.depth > uint32_t(ps.max_path_depth)) p.depth = ps.max_path_depth;
  // rgen:134-149
  const R alpha = R(-2);
  const R expXY = mexp(alpha * R(2) * R(2));
  R ox = jitter.x - R(0.5), oy = jitter.y - R(0.5);
  R fw = gmax(R(0), mexp(alpha * ox * ox) - expXY) * gmax(R(0), mexp(alpha * oy * oy) - expXY);
  out.rad[0] = float(p.radiance.x);
  out.rad[1] = float(p.radiance.y);
  out.rad[2] = float(p.radiance.z);
  out.radd[0] = double(p.radiance.x);
  out.radd[1] = double(p.radiance.y);
  out.radd[2] = double(p.radiance.z);
  out.fw = float(fw);
  out.depth = p.depth;
  out.sig = p.sig;
  out.events = events;
  out.shadows = shadows;
  out.t1 = float(t1);
  for (int i = 0; i < ASUNA_MAX_CHANNELS; ++i) {
    out.ch[i][0] = float(p.ch[i].x);
    out.ch[i][1] = float(p.ch[i].y);
    out.ch[i][2] = float(p.ch[i].z);
  }
}

}  // namespace ora

using namespace ora;

struct oracle_scene {
  Scene s;
};


// ---- post pass (src/shaders/post.idle.frag:71-133, utils/tonemapping.glsl) --
namespace post {
struct F3 {
  float x, y, z;
};
inline F3 op(F3 a, F3 b, float (*f)(float, float)) { return {f(a.x, b.x), f(a.y, b.y), f(a.z, b.z)}; }
inline F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 mul(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline F3 div(F3 a, F3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline F3 s3(float v) { return {v, v, v}; }
// pow of the shared transcendentals (include/asuna_math.h), as the pinned
// shader translation evaluates it
inline F3 pw(F3 a, float e) { return {asuna_math::powf_(a.x, e), asuna_math::powf_(a.y, e), asuna_math::powf_(a.z, e)}; }
// GLSL mix as the specification writes it: x (1 - a) + y a
inline float mixs(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline F3 lin2s(F3 c) { return pw(c, 1.0f / 2.2f); }
inline F3 s2lin(F3 c) { return pw(c, 2.2f); }
inline float lum709(F3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
inline F3 unch(F3 c) {
  const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
  F3 num = add(mul(c, add(mul(c, s3(A)), s3(C * B))), s3(D * E));
  F3 den = add(mul(c, add(mul(c, s3(A)), s3(B))), s3(D * F));
  return sub(div(num, den), s3(E / F));
}
inline F3 hejl(F3 c) {
  c = {std::max(c.x - 0.004f, 0.0f), std::max(c.y - 0.004f, 0.0f), std::max(c.z - 0.004f, 0.0f)};
  return div(mul(c, add(mul(c, s3(6.2f)), s3(0.5f))), add(mul(c, add(mul(c, s3(6.2f)), s3(1.7f))), s3(0.06f)));
}
inline float clamp01(float v) { return std::min(std::max(v, 0.0f), 1.0f); }
inline float srgb(float c) { return c < 0.0031308f ? 12.92f * c : 1.055f * asuna_math::powf_(c, 1.0f / 2.4f) - 0.055f; }
struct Lv {
  std::vector<float> p;
  int w, h;
};
inline F3 sample(const Lv& L, float u, float v, float* alpha = nullptr) {
  const float x = u * float(L.w) - 0.5f, y = v * float(L.h) - 0.5f;
  const float fx = std::floor(x), fy = std::floor(y), tx = x - fx, ty = y - fy;
  auto at = [&](int i, int j, int c) {
    i = std::min(std::max(i, 0), L.w - 1);
    j = std::min(std::max(j, 0), L.h - 1);
    return L.p[(size_t(j) * L.w + i) * 4 + c];
  };
  const int i0 = int(fx), j0 = int(fy);
  float r[4];
  for (int c = 0; c < 4; ++c) {
    float a = at(i0, j0, c), b = at(i0 + 1, j0, c), cc = at(i0, j0 + 1, c), d = at(i0 + 1, j0 + 1, c);
    float p = a + (b - a) * tx, q = cc + (d - cc) * tx;
    r[c] = p + (q - p) * ty;
  }
  if (alpha) *alpha = r[3];
  return {r[0], r[1], r[2]};
}
inline uint32_t pcg3dc(uint32_t v[3]) {
  for (int k = 0; k < 3; ++k) v[k] = v[k] * 1664525u + 1013904223u;
  v[0] += v[1] * v[2];
  v[1] += v[2] * v[0];
  v[2] += v[0] * v[1];
  for (int k = 0; k < 3; ++k) v[k] ^= v[k] >> 16u;
  v[0] += v[1] * v[2];
  v[1] += v[2] * v[0];
  v[2] += v[0] * v[1];
  return 0;
}
}  // namespace post

extern "C" {

uint32_t oracle_xxhash32(uint32_t x, uint32_t y, uint32_t z) { return xxhash32(x, y, z); }
void oracle_invert3x4(const float* m, float* out) { invert3x4(m, out); }
float oracle_math(int which, float x, float y) {
  switch (which) {
    case 0: return msin(x);
    case 1: return mcos(x);
    case 2: return mexp(x);
    case 3: return macos(x);
    case 5: return asuna_math::log2f_(x);
    case 6: return asuna_math::exp2f_(x);
    case 7: return asuna_math::powf_(x, y);
    case 8: return asuna_math::logf_(x);
    case 9: return asuna_math::tanf_(x);
    default: return matan2(x, y);
  }
}
uint32_t oracle_pcg(uint32_t* state) { return pcg(*state); }

// src/loader/material.cpp:6-22 (dielectricReflectance) and :24-37: the
// trapezoid rule over cos^2 theta in [0, 1], float terms summed in double.
static float oraDielectricReflectance(float eta, float cosI, float& cosT) {
  if (cosI < 0.0f) {
    eta = 1.0f / eta;
    cosI = -cosI;
  }
  const float sin2T = eta * eta * (1.0f - cosI * cosI);
  if (sin2T > 1.0f) {
    cosT = 0.0f;
    return 1.0f;
  }
  cosT = std::sqrt(std::max(1.0f - sin2T, 0.0f));
  const float rs = (eta * cosI - cosT) / (eta * cosI + cosT);
  const float rp = (eta * cosT - cosI) / (eta * cosT + cosI);
  return (rs * rs + rp * rp) * 0.5f;
}
float oracle_diffuse_fresnel(float ior, int samples) {
  float unused;
  double acc = 0.0;
  float prev = oraDielectricReflectance(ior, 0.0f, unused);
  for (int i = 1; i <= samples; ++i) {
    const float c2 = float(i) / samples;
    const float cur = oraDielectricReflectance(ior, std::min(std::sqrt(c2), 1.0f), unused);
    acc += double(cur + prev) * (0.5 / samples);
    prev = cur;
  }
  return float(acc);
}

// The camera's two matrices, column-major as GpuCamera stores them
// (src/shared/camera.h).  camera -> world: the look-at frame (x right,
// y up, z back from the target) with y and z negated, translated to the eye
// (view = scale(1,-1,-1) * lookAt).  raster -> camera: the inverse of
// raster <- NDC <- screen <- camera (camera.cpp:28-62) in closed form: with
// c = 1/tan(fov/2), aspect = w/h, a = f/(f-n), b = -n f/(f-n), raster =
// (w c/2 x + w/2 z, h aspect c/2 y + h/2 z, a z + b, z), so x = 2/(w c) X -
// W/c, y = 2/(h aspect c) Y - W/(aspect c), z = W, 1 = (Z - a W)/b.
int oracle_camera_perspective(const float eye[3], const float at[3], const float up[3], float fov_deg,
                              float aperture, float focal_distance, uint32_t width, uint32_t height,
                              asuna_camera* out) {
  if (!eye || !at || !up || !out || !width || !height || !(fov_deg > 0.0f && fov_deg < 180.0f))
    return ASUNA_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  out->type = ASUNA_CAMERA_PERSPECTIVE;
  auto unit = [](double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0)
      for (int k = 0; k < 3; ++k) v[k] /= l;
  };
  double z[3] = {double(eye[0]) - at[0], double(eye[1]) - at[1], double(eye[2]) - at[2]};
  unit(z);
  double x[3] = {up[1] * z[2] - up[2] * z[1], up[2] * z[0] - up[0] * z[2], up[0] * z[1] - up[1] * z[0]};
  unit(x);
  double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
  unit(y);
  double c2w[4][4] = {};  // [row][col]
  for (int k = 0; k < 3; ++k) {
    c2w[k][0] = x[k];
    c2w[k][1] = -y[k];
    c2w[k][2] = -z[k];
    c2w[k][3] = eye[k];
  }
  c2w[3][3] = 1.0;
  const float nearz = 0.1f, farz = 100.0f;
  const float aspect = float(width) / float(height);
  const double c = double(float(1.0 / double(tanf(fov_deg * 0.017453292519943295f * 0.5f))));
  const float recip = 1.0f / (farz - nearz);
  const double a = double(farz * recip), b = double(-nearz * farz * recip);
  double r2c[4][4] = {};
  r2c[0][0] = 2.0 / (double(width) * c);
  r2c[0][3] = -1.0 / c;
  r2c[1][1] = 2.0 / (double(height) * double(aspect) * c);
  r2c[1][3] = -1.0 / (double(aspect) * c);
  r2c[2][3] = 1.0;
  r2c[3][2] = 1.0 / b;
  r2c[3][3] = -a / b;
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      out->camera_to_world[col * 4 + row] = float(c2w[row][col]);
      out->raster_to_camera[col * 4 + row] = float(r2c[row][col]);
      out->env_transform[col * 4 + row] = row == col ? 1.0f : 0.0f;
    }
  out->aperture = aperture;
  out->focal_distance = focal_distance;
  return ASUNA_OK;
}
float oracle_rand(uint32_t* state) { return rnd<float>(*state); }


// Post pass of one image (rgba w*h) into out, as the GPU's k_tonemap
// (the same box mip pyramid and exact mean for Custom's exposure).
int oracle_tonemap(const float* rgba, uint32_t w, uint32_t h, const asuna_post_state* tm, float* out) {
  using namespace post;
  if (!rgba || !tm || !out || !w || !h) return ASUNA_ERR_INVALID;
  std::vector<Lv> pyr;
  pyr.push_back({std::vector<float>(rgba, rgba + size_t(w) * h * 4), int(w), int(h)});
  float avgLum2 = 1.0f;
  if (tm->tm_type == ASUNA_TONEMAP_CUSTOM && (tm->auto_exposure & 1)) {
    double s[3] = {0, 0, 0};
    for (size_t i = 0; i < size_t(w) * h; ++i)
      for (int c = 0; c < 3; ++c) s[c] += rgba[i * 4 + c];
    const float m[3] = {float(s[0] / double(size_t(w) * h)), float(s[1] / double(size_t(w) * h)),
                        float(s[2] / double(size_t(w) * h))};
    avgLum2 = m[0] * 0.2126f + m[1] * 0.7152f + m[2] * 0.0722f;
    if ((tm->auto_exposure >> 1) & 1)
      while (pyr.size() < 9 && !(pyr.back().w == 1 && pyr.back().h == 1)) {
        const Lv& p = pyr.back();
        Lv q{{}, std::max(1, p.w / 2), std::max(1, p.h / 2)};
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
        pyr.push_back(std::move(q));
      }
  }
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const float u = (float(x) + 0.5f) / float(w) * tm->zoom, v = (float(y) + 0.5f) / float(h) * tm->zoom;
      float alpha;
      F3 hdr;
      if (tm->zoom == 1.0f) {
        const float* p = rgba + (size_t(y) * w + x) * 4;
        hdr = {p[0], p[1], p[2]};
        alpha = p[3];
      } else {
        hdr = sample(pyr[0], u, v, &alpha);
      }
      F3 c = hdr;
      switch (tm->tm_type) {
        case ASUNA_TONEMAP_NONE:
          break;
        case ASUNA_TONEMAP_GAMMA:
          c = lin2s(div(hdr, add(div(hdr, s3(1.5f)), s3(1.0f))));
          break;
        case ASUNA_TONEMAP_REINHARD:
        case ASUNA_TONEMAP_FILMIC:
          c = hejl(hdr);
          break;
        case ASUNA_TONEMAP_ACES: {
          const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
          F3 t = div(mul(hdr, add(mul(hdr, s3(A)), s3(B))), add(mul(hdr, add(mul(hdr, s3(C)), s3(D))), s3(E)));
          c = lin2s({clamp01(t.x), clamp01(t.y), clamp01(t.z)});
          break;
        }
        case ASUNA_TONEMAP_PBRT:
          c = {srgb(hdr.x), srgb(hdr.y), srgb(hdr.z)};
          break;
        default: {
          F3 hh = hdr;
          if (tm->auto_exposure & 1) {
            const float XYZy = 0.3575761f * hh.x + 0.7151522f * hh.y + 0.1191920f * hh.z;
            const float factor = tm->key / avgLum2, Y = factor * XYZy;
            if ((tm->auto_exposure >> 1) & 1) {
              const float scale[7] = {1, 2, 4, 8, 16, 32, 64};
              float La = 0.0f;
              for (int i = 0; i < 7; ++i) {
                const Lv& a = pyr[std::min<size_t>(i, pyr.size() - 1)];
                const Lv& b = pyr[std::min<size_t>(i + 1, pyr.size() - 1)];
                const float v1 = lum709(sample(a, u, v)) * factor, v2 = lum709(sample(b, u, v)) * factor;
                if (std::fabs(v1 - v2) / ((tm->key * asuna_math::powf_(2.0f, 2.0f) / (scale[i] * scale[i])) + v1) >
                    0.05f) {
                  La = v1;
                  break;
                }
                La = v2;
              }
              const float k = Y / (1.0f + La);
              hh = mul(div(hh, s3(XYZy)), s3(k));
            } else {
              const float Yd = (Y * (1.0f + Y / (tm->y_white * tm->y_white))) / (1.0f + Y);
              hh = mul(div(hh, s3(XYZy)), s3(Yd));
            }
          }
          F3 col = mul(hh, s3(tm->avg_lum));
          {
            const F3 cu = unch(mul(col, s3(2.0f))), white = unch(s3(11.2f));
            col = lin2s(mul(cu, div(s3(1.0f), white)));
          }
          uint32_t r[3] = {x, y, 0u};
          pcg3dc(r);
          float noise[3];
          for (int k = 0; k < 3; ++k) {
            uint32_t bits = 0x3f800000u | (r[k] >> 9);
            float f;
            std::memcpy(&f, &bits, 4);
            noise[k] = f - 1.0f;
          }
          {
            const float quant = 1.0f / 255.0f;
            const F3 lin = s2lin(col), sv = lin2s(lin);
            const F3 c0 = {std::floor(sv.x / quant) * quant, std::floor(sv.y / quant) * quant,
                           std::floor(sv.z / quant) * quant};
            const F3 c1 = add(c0, s3(quant));
            const F3 l0 = s2lin(c0), l1 = s2lin(c1);
            const F3 discr = {mixs(l0.x, l1.x, noise[0]), mixs(l0.y, l1.y, noise[1]), mixs(l0.z, l1.z, noise[2])};
            col = {discr.x < lin.x ? c1.x : c0.x, discr.y < lin.y ? c1.y : c0.y, discr.z < lin.z ? c1.z : c0.z};
          }
          // GLSL clamp as NVIDIA hardware evaluates it (and fminf / fmaxf):
          // IEEE 754 minNum / maxNum, so a NaN (0/0 on a black pixel under
          // auto exposure, post.idle.frag:45,68) clamps to 0
          auto clampNum = [](float v) { return std::fmin(std::fmax(v, 0.0f), 1.0f); };
          col = {clampNum(mixs(0.5f, col.x, tm->contrast)), clampNum(mixs(0.5f, col.y, tm->contrast)),
                 clampNum(mixs(0.5f, col.z, tm->contrast))};
          col = pw(col, 1.0f / tm->brightness);
          const float g = col.x * 0.299f + col.y * 0.587f + col.z * 0.114f;
          col = {mixs(g, col.x, tm->saturation), mixs(g, col.y, tm->saturation), mixs(g, col.z, tm->saturation)};
          const float vx = ((float(x) + 0.5f) / float(w) * tm->rendering_ratio[0] - 0.5f) * 2.0f;
          const float vy = ((float(y) + 0.5f) / float(h) * tm->rendering_ratio[1] - 0.5f) * 2.0f;
          const float vg = 1.0f - (vx * vx + vy * vy) * tm->vignette;
          c = {col.x * vg, col.y * vg, col.z * vg};
        }
      }
      float* o = out + (size_t(y) * w + x) * 4;
      o[0] = c.x;
      o[1] = c.y;
      o[2] = c.z;
      o[3] = alpha;
    }
  return ASUNA_OK;
}

int oracle_envmap_tables(uint32_t w, uint32_t h, const float* rgba, float* marg, float* cond) {
  if (!w || !h || !rgba || !marg || !cond) return ASUNA_ERR_INVALID;
  envTables(int(w), int(h), rgba, marg, cond);
  return ASUNA_OK;
}

int oracle_scene_create(const asuna_scene_desc* d, oracle_scene** out) {
  if (!d || !out) return ASUNA_ERR_INVALID;
  oracle_scene* os = new (std::nothrow) oracle_scene;
  if (!os) return ASUNA_ERR_OOM;
  Scene& s = os->s;
  s.meshes.resize(d->num_meshes);
  for (uint32_t i = 0; i < d->num_meshes; ++i) {
    const asuna_mesh_desc& md = d->meshes[i];
    Mesh& m = s.meshes[i];
    m.v.assign(md.vertices, md.vertices + md.num_vertices);
    m.idx.assign(md.indices, md.indices + size_t(md.num_triangles) * 3);
    m.ntri = md.num_triangles;
    for (uint32_t k = 0; k < m.idx.size(); ++k)
      if (m.idx[k] >= md.num_vertices) {
        delete os;
        return ASUNA_ERR_INVALID;
      }
  }
  {
    std::vector<std::thread> th;
    std::atomic<uint32_t> next{0};
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (unsigned t = 0; t < nt; ++t)
      th.emplace_back([&] {
        for (uint32_t i; (i = next++) < s.meshes.size();) buildBvh(s.meshes[i]);
      });
    for (auto& t : th) t.join();
  }
  s.insts.resize(d->num_instances);
  for (uint32_t i = 0; i < d->num_instances; ++i) {
    s.insts[i].d = d->instances[i];
    if (d->instances[i].mesh_id >= d->num_meshes) {
      delete os;
      return ASUNA_ERR_INVALID;
    }
    invert3x4(d->instances[i].transform, s.insts[i].w2o);
  }
  s.mats.assign(d->materials, d->materials + d->num_materials);
  s.lights.assign(d->lights, d->lights + d->num_lights);
  s.texs.resize(d->num_textures);
  for (uint32_t i = 0; i < d->num_textures; ++i) {
    const asuna_texture_desc& t = d->textures[i];
    s.texs[i].w = int(t.width);
    s.texs[i].h = int(t.height);
    s.texs[i].c = 4;
    s.texs[i].d.assign(t.rgba, t.rgba + size_t(t.width) * t.height * 4);
  }
  if (d->sun_and_sky && d->sun_and_sky->in_use == 1) {
    s.sky = true;
    s.skyF = asuna_sky::paramsOf<float>(*d->sun_and_sky);
    s.skyD = asuna_sky::paramsOf<double>(*d->sun_and_sky);
  }
  if (d->envmap.rgba && d->envmap.width && d->envmap.height) {
    int w = int(d->envmap.width), h = int(d->envmap.height);
    s.hasEnv = true;
    s.env.w = s.marg.w = s.cond.w = w;
    s.env.h = s.marg.h = s.cond.h = h;
    s.env.c = 4;
    s.marg.c = s.cond.c = 2;
    s.env.d.assign(d->envmap.rgba, d->envmap.rgba + size_t(w) * h * 4);
    s.marg.d.resize(size_t(w) * h * 2);
    s.cond.d.resize(size_t(w) * h * 2);
    envTables(w, h, d->envmap.rgba, s.marg.d.data(), s.cond.d.data());
  } else {
    // Dummy 1x1 env of the reference (src/core/texture.cpp:137-142).
    s.env.w = s.marg.w = s.cond.w = 1;
    s.env.h = s.marg.h = s.cond.h = 1;
    s.env.c = 4;
    s.marg.c = s.cond.c = 2;
    s.env.d.assign(4, 0.0f);
    s.marg.d.assign(2, 0.0f);
    s.cond.d.assign(2, 0.0f);
  }
  *out = os;
  return ASUNA_OK;
}

void oracle_scene_destroy(oracle_scene* s) { delete s; }

int oracle_trace(const oracle_scene* s, const float o[3], const float d[3], float tmin, float tmax, float* t,
                 uint32_t* inst, uint32_t* prim, float* bu, float* bv) {
  Hit h;
  if (!traceScene(s->s, o, d, tmin, tmax, false, h, nullptr)) return 0;
  *t = h.t;
  *inst = h.inst;
  *prim = h.prim;
  *bu = h.u;
  *bv = h.v;
  return 1;
}

int oracle_occluded(const oracle_scene* s, const float o[3], const float d[3], float tmin, float tmax) {
  Hit h;
  return traceScene(s->s, o, d, tmin, tmax, true, h, nullptr) ? 1 : 0;
}

int oracle_render(const oracle_scene* os, const asuna_shot* shot, float* film, asuna_path_record* records,
                  const uint32_t* pixels, uint32_t npixels, int nthreads, int precision, oracle_stats* stats) {
  if (!os || !shot || (!film && !records)) return ASUNA_ERR_INVALID;
  const Scene& s = os->s;
  const uint32_t W = shot->width, H = shot->height;
  if (!W || !H || shot->state.max_path_depth < 1 || shot->state.max_path_depth > 32) return ASUNA_ERR_INVALID;
  const uint32_t npix = pixels ? npixels : W * H;
  if (pixels)
    for (uint32_t i = 0; i < npix; ++i)
      if (pixels[i] >= W * H) return ASUNA_ERR_INVALID;
  if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
  const size_t img = size_t(W) * H * 4;
  const asuna_rt_state& ps = shot->state;
  const int depthSlot = shot->depth_out_channel;
  std::atomic<uint32_t> next{0};
  std::atomic<uint64_t> gExt{0}, gSh{0}, gNodes{0}, gTris{0};
  auto t0 = std::chrono::steady_clock::now();
  auto worker = [&] {
    TravStats st;
    uint64_t nExt = 0, nSh = 0;
    const uint32_t chunk = 64;
    for (;;) {
      uint32_t b = next.fetch_add(chunk);
      if (b >= npix) break;
      uint32_t e = std::min(npix, b + chunk);
      for (uint32_t i = b; i < e; ++i) {
        uint32_t pix = pixels ? pixels[i] : i;
        uint32_t x = pix % W, y = pix / W;
        float* rad0 = film ? film + size_t(pix) * 4 : nullptr;
        float* wimg = film ? film + 8 * img + size_t(pix) * 4 : nullptr;
        for (uint32_t f = 0; f < shot->frames; ++f) {
          uint32_t frame = shot->frame0 + f;
          PathOut po;
          if (precision == 64)
            tracePath<double>(s, *shot, x, y, frame, po, &st, nExt, nSh);
          else
            tracePath<float>(s, *shot, x, y, frame, po, &st, nExt, nSh);
          if (records) {
            asuna_path_record& r = records[size_t(f) * npix + i];
            r.radiance[0] = po.rad[0];
            r.radiance[1] = po.rad[1];
            r.radiance[2] = po.rad[2];
            r.filter_weight = po.fw;
            r.depth = po.depth;
            r.signature = po.sig;
            r.events = po.events;
            r.shadows = po.shadows;
          }
          if (film) {
            // rgen:147-179 (spp = 1 per frame)
            float rc[3];
            for (int c = 0; c < 3; ++c) rc[c] = gclamp(po.rad[c], 0.0f, 10.0f);
            float rws[3] = {po.fw * rc[0], po.fw * rc[1], po.fw * rc[2]};
            float fws = po.fw;
            if (frame == 0) {
              for (int c = 0; c < 3; ++c) rad0[c] = rws[c] / fws;
              rad0[3] = 1.0f;
              for (uint32_t cid = 0; cid < ps.n_multi_channel && cid < ASUNA_MAX_CHANNELS; ++cid) {
                float* ch = film + size_t(cid + 1) * img + size_t(pix) * 4;
                if (int(cid) == depthSlot) {
                  ch[0] = ch[1] = ch[2] = po.t1;
                } else {
                  ch[0] = po.ch[cid][0];
                  ch[1] = po.ch[cid][1];
                  ch[2] = po.ch[cid][2];
                }
                ch[3] = 1.0f;
              }
              wimg[0] = wimg[1] = wimg[2] = wimg[3] = fws;
            } else {
              float ow = wimg[0];
              float nw = ow + fws;
              for (int c = 0; c < 3; ++c) rad0[c] = (rad0[c] * ow + rws[c]) / nw;
              rad0[3] = 1.0f;
              wimg[0] = wimg[1] = wimg[2] = wimg[3] = nw;
            }
          }
        }
      }
    }
    gExt += nExt;
    gSh += nSh;
    gNodes += st.nodes;
    gTris += st.tris;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
  worker();
  for (auto& t : th) t.join();
  if (stats) {
    stats->paths = uint64_t(npix) * shot->frames;
    stats->extend_rays = gExt;
    stats->shadow_rays = gSh;
    stats->nodes_visited = gNodes;
    stats->tris_tested = gTris;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats->threads = nthreads;
  }
  return ASUNA_OK;
}

int oracle_render_pixels_f64(const oracle_scene* os, const asuna_shot* shot, const uint32_t* pixels, uint32_t npixels,
                             int nthreads, double* out_rgb, double* out_var, oracle_stats* stats) {
  if (!os || !shot || !out_rgb) return ASUNA_ERR_INVALID;
  const Scene& s = os->s;
  const uint32_t W = shot->width, H = shot->height;
  const uint32_t npix = pixels ? npixels : W * H;
  if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<uint32_t> next{0};
  std::atomic<uint64_t> gExt{0}, gSh{0};
  auto t0 = std::chrono::steady_clock::now();
  auto worker = [&] {
    uint64_t nExt = 0, nSh = 0;
    for (;;) {
      uint32_t i = next.fetch_add(1);
      if (i >= npix) break;
      uint32_t pix = pixels ? pixels[i] : i;
      uint32_t x = pix % W, y = pix / W;
      // weighted mean of the clamped samples; for its variance also
      // sum fw^2 x^2, sum fw^2 x and sum fw^2
      double acc[3] = {0, 0, 0}, s2[3] = {0, 0, 0}, s3[3] = {0, 0, 0}, wsum = 0, w2 = 0;
      for (uint32_t f = 0; f < shot->frames; ++f) {
        PathOut po;
        tracePath<double>(s, *shot, x, y, shot->frame0 + f, po, nullptr, nExt, nSh);
        double fw = po.fw;
        for (int c = 0; c < 3; ++c) {
          const double v = std::min(std::max(po.radd[c], 0.0), 10.0);
          acc[c] += fw * v;
          s2[c] += fw * fw * v * v;
          s3[c] += fw * fw * v;
        }
        wsum += fw;
        w2 += fw * fw;
      }
      for (int c = 0; c < 3; ++c) {
        const double m = acc[c] / wsum;
        out_rgb[size_t(i) * 3 + c] = m;
        // variance of the weighted mean: sum fw^2 (x - m)^2 / (sum fw)^2 / (1 - sum fw^2 / (sum fw)^2)
        if (out_var) {
          const double ss = std::max(0.0, s2[c] - 2.0 * m * s3[c] + m * m * w2);
          const double corr = 1.0 - w2 / (wsum * wsum);
          out_var[size_t(i) * 3 + c] = corr > 0.0 ? ss / (wsum * wsum) / corr : 0.0;
        }
      }
    }
    gExt += nExt;
    gSh += nSh;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
  worker();
  for (auto& t : th) t.join();
  if (stats) {
    stats->paths = uint64_t(npix) * shot->frames;
    stats->extend_rays = gExt;
    stats->shadow_rays = gSh;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats->threads = nthreads;
  }
  return ASUNA_OK;
}

}  // extern "C"
