/*
 * asuna_sunsky.h — the sun & sky environment model of the path tracer.
 *
 * A restatement of src/shaders/utils/sun_and_sky.glsl (the analytic daylight
 * model the reference's miss shader and environment light sample use when
 * GpuSunAndSky.in_use = 1: raytrace.default.rmiss:24-56,
 * rchit_layouts.glsl:98-116, sample_light.glsl:137-141), written once for
 * the CUDA kernels and the CPU oracle, with the shader's float operations in
 * the shader's order: compile with -fmad=false (device) / -ffp-contract=off
 * (host).  The transcendentals are those of include/asuna_math.h for float;
 * the double instantiation (the oracle's quality reference) uses the C
 * library.  GLSL constants are float: M_PI is the file's own 3.1415926535f.
 *
 * Parity with the reference's shader source compiled as host C++ is pinned
 * bit for bit by the oracle tests.
 */
#ifndef ASUNA_SUNSKY_H
#define ASUNA_SUNSKY_H

#include "asuna_math.h"

#if !defined(__CUDACC__)
#include <cmath>
#endif

#ifdef __cplusplus
extern "C++" {
namespace asuna_sky {

/* Fields of GpuSunAndSky (src/shared/sun_and_sky.h), by value. */
template <class R>
struct Params {
  R rgb[3];
  R multiplier, haze, redblueshift, saturation, horizon_height;
  R ground[3];
  R horizon_blur;
  R night[3];
  R sun_disk_intensity;
  R sun_dir[3];
  R sun_disk_scale, sun_glow_intensity;
  int y_is_up, physically_scaled_sun;
};

template <class R>
struct V {
  R x, y, z;
};

/* Params from a GpuSunAndSky-shaped struct (asuna_sun_and_sky) */
template <class R, class G>
ASUNA_MATH_FN Params<R> paramsOf(const G& g) {
  Params<R> p;
  for (int k = 0; k < 3; ++k) {
    p.rgb[k] = R(g.rgb_unit_conversion[k]);
    p.ground[k] = R(g.ground_color[k]);
    p.night[k] = R(g.night_color[k]);
    p.sun_dir[k] = R(g.sun_direction[k]);
  }
  p.multiplier = R(g.multiplier);
  p.haze = R(g.haze);
  p.redblueshift = R(g.redblueshift);
  p.saturation = R(g.saturation);
  p.horizon_height = R(g.horizon_height);
  p.horizon_blur = R(g.horizon_blur);
  p.sun_disk_intensity = R(g.sun_disk_intensity);
  p.sun_disk_scale = R(g.sun_disk_scale);
  p.sun_glow_intensity = R(g.sun_glow_intensity);
  p.y_is_up = g.y_is_up;
  p.physically_scaled_sun = g.physically_scaled_sun;
  return p;
}

/* math: float = the shared implementation, double = the C library */
ASUNA_MATH_FN float m_sqrt(float x) { return asuna_math::fl_sqrt(x); }
ASUNA_MATH_FN float m_sin(float x) { return asuna_math::sinf_(x); }
ASUNA_MATH_FN float m_cos(float x) { return asuna_math::cosf_(x); }
ASUNA_MATH_FN float m_tan(float x) { return asuna_math::tanf_(x); }
ASUNA_MATH_FN float m_acos(float x) { return asuna_math::acosf_(x); }
ASUNA_MATH_FN float m_exp(float x) { return asuna_math::expf_(x); }
ASUNA_MATH_FN float m_pow(float x, float y) { return asuna_math::powf_(x, y); }
#if !defined(__CUDACC__)
static inline double m_sqrt(double x) { return std::sqrt(x); }
static inline double m_sin(double x) { return std::sin(x); }
static inline double m_cos(double x) { return std::cos(x); }
static inline double m_tan(double x) { return std::tan(x); }
static inline double m_acos(double x) { return std::acos(x); }
static inline double m_exp(double x) { return std::exp(x); }
static inline double m_pow(double x, double y) { return std::pow(x, y); }
#endif

#define ASUNA_SKY_FN template <class R> ASUNA_MATH_FN

ASUNA_SKY_FN R m_abs_(R x) { return x < R(0) ? -x : x; }
ASUNA_SKY_FN V<R> v3(R a, R b, R c) { return V<R>{a, b, c}; }
ASUNA_SKY_FN V<R> vadd(V<R> a, V<R> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
ASUNA_SKY_FN V<R> vmul(V<R> a, V<R> b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
ASUNA_SKY_FN V<R> vscale(V<R> a, R s) { return v3(a.x * s, a.y * s, a.z * s); }
ASUNA_SKY_FN R vdot(V<R> a, V<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ASUNA_SKY_FN R vlength(V<R> a) { return m_sqrt(vdot(a, a)); }
ASUNA_SKY_FN V<R> vnormalize(V<R> a) {
  const R l = vlength(a);
  return v3(a.x / l, a.y / l, a.z / l);
}
ASUNA_SKY_FN V<R> vcross(V<R> a, V<R> b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
/* GLSL smoothstep as the specification writes it */
ASUNA_SKY_FN R smoothstep_(R e0, R e1, R x) {
  R t = (x - e0) / (e1 - e0);
  t = t < R(0) ? R(0) : t;
  t = t > R(1) ? R(1) : t;
  return t * t * (R(3) - R(2) * t);
}
ASUNA_SKY_FN R kPi() { return R(3.1415926535f); }

/* sun_and_sky.glsl:29-31 */
ASUNA_SKY_FN R luminance(V<R> c) { return R(0.2126f) * c.x + R(0.7152f) * c.y + R(0.0722f) * c.z; }

/* sun_and_sky.glsl:33-57: an orthonormal frame around `n`, then x u + y v + z n */
ASUNA_SKY_FN V<R> xyz2dir(V<R> n, R x, R y, R z) {
  V<R> u = (m_abs_(n.x) < m_abs_(n.y)) ? v3(R(0), -n.z, n.y) : v3(n.z, R(0), -n.x);
  if (vlength(u) == R(0)) u = (m_abs_(n.x) < m_abs_(n.y)) ? v3(R(0), -n.z, n.y) : v3(n.z, R(0), -n.x);
  u = vnormalize(u);
  const V<R> v = vcross(n, u);
  return vadd(vadd(vscale(u, x), vscale(v, y)), vscale(n, z));
}

/* sun_and_sky.glsl:59-86: Shirley's concentric square -> disk, (r, phi) */
ASUNA_SKY_FN void squareToDisk(R sx, R sy, R& r, R& phi) {
  const R lx = R(2) * sx - R(1), ly = R(2) * sy - R(1);
  const R q = kPi<R>() / R(4.0f);
  if (lx == R(0) && ly == R(0)) {
    r = R(0);
    phi = R(0);
  } else if (lx > -ly) {
    if (lx > ly) {
      r = lx;
      phi = q * (R(1.0f) + ly / lx);
    } else {
      r = ly;
      phi = q * (R(3.0f) - lx / ly);
    }
  } else {
    if (lx < ly) {
      r = -lx;
      phi = q * (R(5.0f) + ly / lx);
    } else {
      r = -ly;
      phi = q * (R(7.0f) - lx / ly);
    }
  }
}

/* sun_and_sky.glsl:88-104: cosine-distributed direction about n */
ASUNA_SKY_FN V<R> diffuseDir(V<R> n, R sx, R sy) {
  R r, phi;
  squareToDisk(sx, sy, r, phi);
  const R x = r * m_cos(phi), y = r * m_sin(phi);
  const R z2 = R(1.0f) - x * x - y * y;
  const R z = z2 > R(0) ? m_sqrt(z2) : R(0);
  return xyz2dir(n, x, y, z);
}

/* sun_and_sky.glsl:106-132: direct sun colour through the atmosphere */
ASUNA_SKY_FN V<R> sunColor(V<R> sd, R turbidity) {
  V<R> out = v3(R(0), R(0), R(0));
  if (sd.z > R(0)) {
    const R ko[3] = {R(12.0f), R(8.5f), R(0.9f)};
    const R wl[3] = {R(0.610f), R(0.550f), R(0.470f)};
    const R sol[3] = {R(1.0f) * R(127500) / R(0.9878f), R(0.992f) * R(127500) / R(0.9878f),
                      R(0.911f) * R(127500) / R(0.9878f)};
    const R m = R(1.0f) / (sd.z + R(0.15f) * m_pow(R(93.885f) - m_acos(sd.z) * R(180) / kPi<R>(), R(-1.253f)));
    const R beta = R(0.04608f) * turbidity - R(0.04586f);
    const R alpha = R(1.3f);
    const R l = R(0.0035f);
    R c[3];
    for (int k = 0; k < 3; ++k) {
      const R ta = m_exp(-m * beta * m_pow(wl[k], -alpha));
      const R to = m_exp(-m * ko[k] * l);
      const R tr = m_exp(-m * R(0.008735f) * m_pow(wl[k], R(-4.08f)));
      c[k] = tr * ta * to * sol[k];
    }
    out = v3(c[0], c[1], c[2]);
  }
  return out;
}

/* the Perez distribution term shared by sky_color_xyz and sky_luminance:
 * ((1 + A e^{B / cos theta}) (1 + C e^{D gamma} + E cos^2 gamma)) /
 * ((1 + A e^{B}) (1 + C e^{D theta_s} + E cos^2 theta_s)) */
ASUNA_SKY_FN R perez(R A, R B, R C, R D, R E, R cosTheta, R gamma, R cosGamma, R thetaSun, R cosThetaSun) {
  return ((R(1) + A * m_exp(B / cosTheta)) * (R(1) + C * m_exp(D * gamma) + E * cosGamma * cosGamma)) /
         ((R(1) + A * m_exp(B / R(1.0f))) * (R(1) + C * m_exp(D * thetaSun) + E * cosThetaSun * cosThetaSun));
}

/* sun_and_sky.glsl:134-200: CIE XYZ of the sky in direction d */
ASUNA_SKY_FN V<R> skyXYZ(V<R> d, V<R> sun, R T, R lum) {
  R cg = vdot(sun, d);
  if (cg > R(1.0f)) cg = R(2.0f) - cg;
  const R gamma = m_acos(cg);
  const R ct = d.z, cts = sun.z;
  const R ts = m_acos(cts);
  const R t2 = T * T, ts2 = ts * ts, ts3 = ts2 * ts;
  const R zx = (R(0.001650f) * ts3 - R(0.003742f) * ts2 + R(0.002088f) * ts + R(0)) * t2 +
               (R(-0.029028f) * ts3 + R(0.063773f) * ts2 - R(0.032020f) * ts + R(0.003948f)) * T +
               (R(0.116936f) * ts3 - R(0.211960f) * ts2 + R(0.060523f) * ts + R(0.258852f));
  const R zy = (R(0.002759f) * ts3 - R(0.006105f) * ts2 + R(0.003162f) * ts + R(0)) * t2 +
               (R(-0.042149f) * ts3 + R(0.089701f) * ts2 - R(0.041536f) * ts + R(0.005158f)) * T +
               (R(0.153467f) * ts3 - R(0.267568f) * ts2 + R(0.066698f) * ts + R(0.266881f));
  R A = R(-0.019257f) * T - (R(0.29f) - m_pow(cts, R(0.5f)) * R(0.09f));
  R B = R(-0.066513f) * T + R(0.000818f);
  R C = R(-0.000417f) * T + R(0.212479f);
  R D = R(-0.064097f) * T - R(0.898875f);
  R E = R(-0.003251f) * T + R(0.045178f);
  R x = perez(A, B, C, D, E, ct, gamma, cg, ts, cts);
  A = R(-0.016698f) * T - R(0.260787f);
  B = R(-0.094958f) * T + R(0.009213f);
  C = R(-0.007928f) * T + R(0.210230f);
  D = R(-0.044050f) * T - R(1.653694f);
  E = R(-0.010922f) * T + R(0.052919f);
  R y = perez(A, B, C, D, E, ct, gamma, cg, ts, cts);
  const R sat = R(1.0f);
  x = zx * ((x * sat) + (R(1.0f) - sat));
  y = zy * ((y * sat) + (R(1.0f) - sat));
  return v3((x / y) * lum, lum, ((R(1.0f) - x - y) / y) * lum);
}

/* sun_and_sky.glsl:202-227: relative sky luminance (Perez, Y) */
ASUNA_SKY_FN R skyLuminance(V<R> d, V<R> sun, R T) {
  R cg = vdot(sun, d);
  if (cg < R(0.0f)) cg = R(0.0f);
  if (cg > R(1.0f)) cg = R(2.0f) - cg;
  const R gamma = m_acos(cg);
  const R ct = d.z, cts = sun.z;
  const R ts = m_acos(cts);
  const R A = R(0.178721f) * T - R(1.463037f);
  const R B = R(-0.355402f) * T + R(0.427494f);
  const R C = R(-0.022669f) * T + R(5.325056f);
  const R D = R(0.120647f) * T - R(2.577052f);
  const R E = R(-0.066967f) * T + R(0.370275f);
  return perez(A, B, C, D, E, ct, gamma, cg, ts, cts);
}

/* sun_and_sky.glsl:229-245: sky radiance (linear RGB) in direction d */
ASUNA_SKY_FN V<R> envColor(V<R> sun, V<R> d, R T) {
  const R ts = m_acos(sun.z);
  const R chi = (R(4.0f) / R(9.0f) - T / R(120.0f)) * (kPi<R>() - R(2) * ts);
  R lum = R(1000.0f) * ((R(4.0453f) * T - R(4.9710f)) * m_tan(chi) - R(0.2155f) * T + R(2.4192f));
  lum = lum * skyLuminance(d, sun, T);
  const V<R> X = skyXYZ(d, sun, T, lum);
  const V<R> c = v3(R(3.241f) * X.x - R(1.537f) * X.y - R(0.499f) * X.z,
                    R(-0.969f) * X.x + R(1.876f) * X.y + R(0.042f) * X.z,
                    R(0.056f) * X.x - R(0.204f) * X.y + R(1.057f) * X.z);
  return vscale(c, kPi<R>());
}

/* sun_and_sky.glsl:247-264: ground irradiance, 5 x 5 cosine-distributed
 * sky samples (the sample grid stepped in float as the shader steps it) */
ASUNA_SKY_FN V<R> irradiance(V<R> sun, R haze) {
  V<R> acc = v3(R(0), R(0), R(0));
  const V<R> n = v3(R(0), R(0), R(1.0f));
  for (float u = 1.0f / 10.0f; u < 1.0f; u += 1.0f / 5.0f)
    for (float v = 1.0f / 10.0f; v < 1.0f; v += 1.0f / 5.0f)
      acc = vadd(acc, envColor(sun, diffuseDir(n, R(u), R(v)), haze));
  return v3(acc.x / R(25.0f), acc.y / R(25.0f), acc.z / R(25.0f));
}

/* sun_and_sky.glsl:266-278 */
ASUNA_SKY_FN R tweakSaturation(R s, R haze) {
  const R lowsat = m_pow(s, R(3.0f));
  if (s <= R(1.0f)) {
    R h = haze;
    h = h - R(2.0f);
    h = h / R(15.0f);
    if (h < R(0.0f)) h = R(0.0f);
    if (h > R(1.0f)) h = R(1.0f);
    h = m_pow(h, R(3.0f));
    return (s * (R(1.0f) - h)) + lowsat * h;
  }
  return R(1.0f);
}

/* sun_and_sky.glsl:280-290: z up (y_is_up swaps y and z), lowered horizon */
ASUNA_SKY_FN V<R> vectorTweak(V<R> d, int yIsUp, R hh) {
  V<R> o = d;
  if (yIsUp == 1) o = v3(d.x, d.z, d.y);
  if (hh != R(0)) {
    o.z = o.z - hh;
    o = vnormalize(o);
  }
  return o;
}

/* sun_and_sky.glsl:292-313: saturation and red/blue shift (the clamp of
 * negatives there writes a variable that is not read again: no effect) */
ASUNA_SKY_FN V<R> colorTweak(V<R> tint, R sat, R red) {
  const R I = luminance(tint);
  V<R> o;
  if (sat <= R(0.0f))
    o = v3(I, I, I);
  else
    o = vadd(vscale(tint, sat), v3(I * (R(1.0f) - sat), I * (R(1.0f) - sat), I * (R(1.0f) - sat)));
  return vmul(o, v3(R(1.0f) + red, R(1.0f), R(1.0f) - red));
}

/* sun_and_sky.glsl:315-393: disk and glow scales of a physically scaled sun */
ASUNA_SKY_FN void physicalScale(R diskScale, R glowIntensity, R diskIntensity, R& diskOut, R& glowOut) {
  const R angular = R(0.00465f);
  const R diskRadius = angular * diskScale;
  const R glowRadius = diskRadius * R(10.0f);
  const R pi = kPi<R>();
  const R glowIntegral =
      glowIntensity * ((R(4.0f) * pi) - (R(24.0f) * pi) / (glowRadius * glowRadius) +
                       (R(24.0f) * pi) * m_sin(glowRadius) / (glowRadius * glowRadius * glowRadius));
  R target = diskIntensity * pi;
  R glowScale = R(1.0f);
  const R maxGlow = R(0.5f) * target;
  if (glowIntegral > maxGlow) {
    glowScale = glowScale * (maxGlow / glowIntegral);
    target = target - maxGlow;
  } else {
    target = target - glowIntegral;
  }
  const R area = R(2) * pi * (R(1) - m_cos(diskRadius));
  const R targetIntensity = target / area;
  const R actualIntegral = R(1.0f) * area;
  const R actualIntensity = diskIntensity * R(100.0f) * actualIntegral / area;
  diskOut = (targetIntensity == R(0.0f)) ? R(0.0f) : targetIntensity / actualIntensity;
  glowOut = glowScale;
}

/* sun_and_sky.glsl:395-403 */
ASUNA_SKY_FN R nightAdjust(V<R> sd) {
  const R lmt = R(0.30901699437494742410229341718282f);
  if (sd.z <= -lmt) return R(0.0f);
  R f = (sd.z + lmt) / lmt;
  f = f * f;
  f = f * f;
  return f;
}

/* sun_and_sky.glsl:405-533: radiance of the sun & sky in direction d */
ASUNA_SKY_FN V<R> sunAndSky(const Params<R>& ss, V<R> inDir) {
  R factor = R(1.0f), nightFactor = R(1.0f);
  V<R> rgbScale = v3(ss.rgb[0], ss.rgb[1], ss.rgb[2]);
  const R hh = ss.horizon_height / R(10.0f);
  V<R> dir = vectorTweak(inDir, ss.y_is_up, hh);
  R haze = R(2.0f) + ss.haze;
  if (haze < R(2.0f)) haze = R(2.0f);
  const R sat = tweakSaturation(ss.saturation, haze);
  if (luminance(rgbScale) < R(0.0f)) {
    const R s = R(1.0f) / R(80000.0f);
    rgbScale = v3(s, s, s);
  }
  rgbScale = vscale(rgbScale, ss.multiplier);
  if (ss.multiplier <= R(0.0f)) return v3(R(0), R(0), R(0));
  const R downness = dir.z;
  const V<R> realDir = dir;
  if (dir.z < R(0.001f)) {
    dir.z = R(0.001f);
    dir = vnormalize(dir);
  }
  V<R> sun = vnormalize(v3(ss.sun_dir[0], ss.sun_dir[1], ss.sun_dir[2]));
  sun = vectorTweak(sun, ss.y_is_up, hh);
  const V<R> realSun = sun;
  if (sun.z < R(0.001f)) {
    if (sun.z < R(0.0f)) factor = nightAdjust(sun);
    sun.z = R(0.001f);
    sun = vnormalize(sun);
  }
  V<R> tint;
  if (factor > R(0.0f)) {
    tint = envColor(sun, dir, haze);
    if (factor < R(1.0f)) tint = vscale(tint, factor);
  } else {
    tint = v3(R(0), R(0), R(0));
  }
  const V<R> sunCol = sunColor(sun, downness > R(0) ? haze : R(2.0f));
  if (ss.sun_disk_intensity > R(0.0f) && ss.sun_disk_scale > R(0.0f)) {
    const R angle = m_acos(vdot(realDir, realSun));
    const R radius = R(0.00465f) * ss.sun_disk_scale * R(10.0f);
    if (angle < radius) {
      R diskScale = R(1.0f), glowScale = R(1.0f);
      if (ss.physically_scaled_sun == 1)
        physicalScale(ss.sun_disk_scale, ss.sun_glow_intensity, ss.sun_disk_intensity, diskScale, glowScale);
      R f = (R(1.0f) - angle / radius) * R(10.0f);
      f = (m_pow(f / R(10.0f), R(3.0f)) * R(2.0f) * ss.sun_glow_intensity * glowScale +
           smoothstep_(R(8.5f), R(9.5f) + (haze / R(50.0f)), f) * R(100.0f) * ss.sun_disk_intensity * diskScale);
      tint = vadd(tint, vscale(sunCol, f));
    }
  }
  V<R> out = vmul(tint, rgbScale);
  if (downness <= R(0.0f)) {
    const V<R> irr = irradiance(sun, R(2.0f));
    V<R> down = v3(ss.ground[0], ss.ground[1], ss.ground[2]);
    down = vmul(down, vmul(vadd(irr, vscale(sunCol, sun.z)), rgbScale));
    if (factor < R(1)) down = vscale(down, factor);
    const R blur = ss.horizon_blur / R(10.0f);
    if (blur > R(0.0f)) {
      R dn = -downness;
      dn = dn / blur;
      if (dn > R(1.0f)) dn = R(1.0f);
      dn = smoothstep_(R(0.0f), R(1.0f), dn);
      out = vadd(vscale(out, R(1.0f) - dn), vscale(down, dn));
      nightFactor = R(1.0f) - dn;
    } else {
      out = down;
      nightFactor = R(0.0f);
    }
  }
  out = colorTweak(out, sat, ss.redblueshift);
  V<R> res = out;
  if (nightFactor > R(0.0f)) {
    const V<R> night = vscale(v3(ss.night[0], ss.night[1], ss.night[2]), nightFactor);
    if (res.x < night.x) res.x = night.x;
    if (res.y < night.y) res.y = night.y;
    if (res.z < night.z) res.z = night.z;
  }
  return vscale(res, kPi<R>());
}

#undef ASUNA_SKY_FN

}  // namespace asuna_sky
}  // extern "C++"
#endif /* __cplusplus */

#endif /* ASUNA_SUNSKY_H */
