// ssf_glsl.hpp — the slice of GLSL the reference's SSF shaders use, in C++,
// so that their source (fluids/shader/SSF*.glsl) compiles and runs on the CPU.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE: part of the reference harness that
// pins the SSF oracle (oracle/ssf_oracle.c) to the reference's own shader
// code.  build_ref.py rewrites each shader only where GLSL and C++ differ in
// syntax (the #version / #extension lines, in/out/uniform/layout qualifiers,
// float literals, read-only swizzles .xyz .rgb .xy become calls, .r becomes
// .x) and wraps it in a namespace; the statements and their order are the
// shader's.  ssf_ref.cpp supplies what fixed-function OpenGL does around the
// shaders (clipping, point rasterisation, depth test, blending, texture
// addressing) by the rules include/pbf_ssf.h states.
//
// Arithmetic is float, as GLSL's; vector and matrix products sum left to right.
#pragma once

#include <cmath>

namespace glsl {

struct vec2;
struct vec3;
struct vec4;

struct vec2 {
  float x = 0.f, y = 0.f;
  vec2() = default;
  vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
  float x = 0.f, y = 0.f, z = 0.f;
  vec3() = default;
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(const vec4& v);
  vec2 xy() const { return vec2(x, y); }
};

struct vec4 {
  float x = 0.f, y = 0.f, z = 0.f, w = 0.f;
  vec4() = default;
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3 xyz() const { return vec3(x, y, z); }
  vec2 xy() const { return vec2(x, y); }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct ivec2 {
  int x = 0, y = 0;
  ivec2(int a, int b) : x(a), y(b) {}
};

inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator/(vec2 a, float s) { return vec2(a.x / s, a.y / s); }

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

// column-major, element [c * 4 + r]
struct mat4 {
  float m[16] = {};
};
struct mat3 {
  float m[9] = {};
  mat3() = default;
  explicit mat3(const mat4& a) {
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) m[c * 3 + r] = a.m[c * 4 + r];
  }
};

inline vec4 operator*(const mat4& a, vec4 v) {
  const float* m = a.m;
  return vec4(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w,
              m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
              m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w,
              m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w);
}
inline vec3 operator*(const mat3& a, vec3 v) {
  const float* m = a.m;
  return vec3(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
              m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

// the built-in functions the shaders call, float only
inline float abs(float a) { return std::fabs(a); }
inline float sqrt(float a) { return std::sqrt(a); }
inline float exp(float a) { return std::exp(a); }
inline float pow(float a, float b) { return std::pow(a, b); }
inline float floor(float a) { return std::floor(a); }
inline float max(float a, float b) { return a < b ? b : a; }  // GLSL max: y if x < y else x
inline float mod(float a, float b) { return a - b * std::floor(a / b); }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline vec3 mix(vec3 a, vec3 b, float t) { return a * (1.f - t) + b * t; }

// textures: 2D float images (row 0 at the bottom), GL_REPEAT addressing (the
// textures' default wrap mode, never changed by the reference), nearest or
// bilinear filtering as the reference sets them (fluids/SSFRenderer.cpp:45-69)
struct sampler2D {
  const float* data = nullptr;
  int W = 0, H = 0, comps = 1;
  bool linear = false;
};
inline int wrap(int i, int n) { return ((i % n) + n) % n; }
inline vec4 texel(const sampler2D& s, int i, int j) {
  const float* p = s.data + ((size_t)j * s.W + i) * s.comps;
  return vec4(p[0], s.comps > 1 ? p[1] : 0.f, s.comps > 2 ? p[2] : 0.f, s.comps > 3 ? p[3] : 1.f);
}
inline vec4 texture(const sampler2D& s, vec2 uv) {
  if (!s.linear) {
    const int i = wrap((int)std::floor(uv.x * (float)s.W), s.W);
    const int j = wrap((int)std::floor(uv.y * (float)s.H), s.H);
    return texel(s, i, j);
  }
  const float u = uv.x * (float)s.W - 0.5f, v = uv.y * (float)s.H - 0.5f;
  const float fu = std::floor(u), fv = std::floor(v);
  const float a = u - fu, b = v - fv;
  const int i0 = wrap((int)fu, s.W), i1 = wrap((int)fu + 1, s.W);
  const int j0 = wrap((int)fv, s.H), j1 = wrap((int)fv + 1, s.H);
  const vec4 t00 = texel(s, i0, j0), t01 = texel(s, i1, j0), t10 = texel(s, i0, j1), t11 = texel(s, i1, j1);
  const float w00 = (1.f - a) * (1.f - b), w01 = a * (1.f - b), w10 = (1.f - a) * b, w11 = a * b;
  return vec4(w00 * t00.x + w01 * t01.x + w10 * t10.x + w11 * t11.x, w00 * t00.y + w01 * t01.y + w10 * t10.y + w11 * t11.y,
              w00 * t00.z + w01 * t01.z + w10 * t10.z + w11 * t11.z, w00 * t00.w + w01 * t01.w + w10 * t10.w + w11 * t11.w);
}
// texelFetch outside the image reads 0
inline vec4 texelFetch(const sampler2D& s, ivec2 p, int) {
  if (p.x < 0 || p.x >= s.W || p.y < 0 || p.y >= s.H) return vec4(0.f, 0.f, 0.f, 0.f);
  return texel(s, p.x, p.y);
}

// an r32f image (imageStore writes the first component)
struct image2D {
  float* data = nullptr;
  int W = 0, H = 0;
};
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
  if (p.x >= 0 && p.x < im.W && p.y >= 0 && p.y < im.H) im.data[(size_t)p.y * im.W + p.x] = v.x;
}

// the sky cube map: GL face table, bilinear, clamped to each face's edge
// (fluids/Renderer.cpp:460-464); no faces: a uniform colour
struct samplerCube {
  const float* faces = nullptr;  // [6][S][S][3]
  int S = 0;
  vec3 uniform_color;
};
inline vec4 texture(const samplerCube& c, vec3 d) {
  if (!c.faces || c.S <= 0) return vec4(c.uniform_color, 1.f);
  const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  int face;
  float sc, tc, ma;
  if (ax >= ay && ax >= az) {
    face = d.x >= 0.f ? 0 : 1, ma = ax, sc = d.x >= 0.f ? -d.z : d.z, tc = -d.y;
  } else if (ay >= az) {
    face = d.y >= 0.f ? 2 : 3, ma = ay, sc = d.x, tc = d.y >= 0.f ? d.z : -d.z;
  } else {
    face = d.z >= 0.f ? 4 : 5, ma = az, sc = d.z >= 0.f ? d.x : -d.x, tc = -d.y;
  }
  if (!(ma > 0.f) || !std::isfinite(ma)) return vec4(c.uniform_color, 1.f);
  const int S = c.S;
  const float s = 0.5f * (sc / ma + 1.f), t = 0.5f * (tc / ma + 1.f);
  const float u = s * (float)S - 0.5f, v = t * (float)S - 0.5f;
  const float fu = std::floor(u), fv = std::floor(v), a = u - fu, b = v - fv;
  auto cl = [S](int i) { return i < 0 ? 0 : (i > S - 1 ? S - 1 : i); };
  const int i0 = cl((int)fu), i1 = cl((int)fu + 1), j0 = cl((int)fv), j1 = cl((int)fv + 1);
  const float* F = c.faces + (size_t)face * S * S * 3;
  float o[3];
  for (int ch = 0; ch < 3; ++ch)
    o[ch] = (1.f - a) * (1.f - b) * F[((size_t)j0 * S + i0) * 3 + ch] + a * (1.f - b) * F[((size_t)j0 * S + i1) * 3 + ch] +
            (1.f - a) * b * F[((size_t)j1 * S + i0) * 3 + ch] + a * b * F[((size_t)j1 * S + i1) * 3 + ch];
  return vec4(o[0], o[1], o[2], 1.f);
}

// built-in variables (set and read by ssf_ref.cpp around each invocation)
inline vec2 gl_PointCoord;
inline vec4 gl_FragCoord;
inline float gl_FragDepth;
inline vec4 gl_Position;
inline float gl_PointSize;
struct DepthRange {
  float near, far, diff;
};
inline DepthRange gl_DepthRange = {0.f, 1.f, 1.f};
inline bool gl_discarded = false;

}  // namespace glsl

