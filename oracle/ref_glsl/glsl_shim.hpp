// glsl_shim.hpp — the subset of GLSL 4.50 that the reference's compute shaders
// and sky-rendering headers use, written as C++ so that their unmodified math
// compiles on the host.
//
// TEST INFRASTRUCTURE ONLY (oracle pinning). Compile with
// -fsingle-precision-constant (GLSL float literals are single precision) and
// -ffp-contract=off (no fused multiply-add).
//
// Samplers emulate the one sampler of src/precompute.rs:85-98: LINEAR filter,
// CLAMP_TO_EDGE, texel coordinate u*size-0.5, exact weights, summed in the
// order the Vulkan specification gives. Images may round stores to half
// precision, as the reference's RGBA16F images do (src/precompute.rs:1215).
#pragma once
#include <cmath>
#include <cstdint>

namespace glsl {

typedef unsigned int uint;

struct vec4;
struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  vec2(float a, float b) : x(a), y(b) {}
};
struct vec3 {
  union { float x; float r; };
  union { float y; float g; };
  union { float z; float b; };
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b_, float c) : x(a), y(b_), z(c) {}
  explicit vec3(const vec4& v);
  vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
};
struct vec4 {
  union { float x; float r; };
  union { float y; float g; };
  union { float z; float b; };
  union { float w; float a; };
  vec4() : x(0), y(0), z(0), w(0) {}
  explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3 rgb() const { return vec3(x, y, z); }
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct uvec2 { uint x, y; uvec2(uint a, uint b) : x(a), y(b) {} };
struct uvec3 {
  uint x, y, z;
  uvec3() : x(0), y(0), z(0) {}
  uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
  uvec2 xy() const { return uvec2(x, y); }
};
struct ivec2 {
  int x, y;
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}
  explicit ivec2(const uvec3& v) : x((int)v.x), y((int)v.y) {}
};
struct ivec3 {
  int x, y, z;
  explicit ivec3(const uvec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
};
struct bvec2 { bool x, y; };
struct bvec3 { bool x, y, z; };

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(const vec4& a, const vec4& b) { return vec4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }

// GLSL built-ins (GLSL 4.50 spec, section 8), single precision.
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float exp(float x) { return std::exp(x); }
inline vec3 exp(const vec3& v) { return vec3(std::exp(v.x), std::exp(v.y), std::exp(v.z)); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float floor(float x) { return std::floor(x); }
inline float mod(float x, float y) { return x - y * floor(x / y); }
inline float smoothstep(float e0, float e1, float x) {
  float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 normalize(const vec3& v) { return v / std::sqrt(dot(v, v)); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec4 mix(const vec4& x, const vec4& y, float t) {
  return vec4(x.x * (1.0f - t) + y.x * t, x.y * (1.0f - t) + y.y * t, x.z * (1.0f - t) + y.z * t,
              x.w * (1.0f - t) + y.w * t);
}
inline bool isinf(float x) { return std::isinf(x); }
inline bvec2 greaterThanEqual(const uvec2& a, const uvec2& b) { return {a.x >= b.x, a.y >= b.y}; }
inline bvec3 greaterThanEqual(const uvec3& a, const uvec3& b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bool any(const bvec2& v) { return v.x || v.y; }
inline bool any(const bvec3& v) { return v.x || v.y || v.z; }

// ---- images and samplers over host RGBA float arrays ----------------------
struct image2D { float* data; int w, h; bool half; };
struct image3D { float* data; int w, h, d; bool half; };
struct sampler2D { const float* data; int w, h; };
struct sampler3D { const float* data; int w, h, d; };

inline float store_rounding(float v, bool half) { return half ? (float)(_Float16)v : v; }
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
  float* t = im.data + 4 * ((size_t)p.y * im.w + p.x);
  t[0] = store_rounding(v.x, im.half); t[1] = store_rounding(v.y, im.half);
  t[2] = store_rounding(v.z, im.half); t[3] = store_rounding(v.w, im.half);
}
inline void imageStore(image3D& im, ivec3 p, vec4 v) {
  float* t = im.data + 4 * (((size_t)p.z * im.h + p.y) * im.w + p.x);
  t[0] = store_rounding(v.x, im.half); t[1] = store_rounding(v.y, im.half);
  t[2] = store_rounding(v.z, im.half); t[3] = store_rounding(v.w, im.half);
}
inline vec4 imageLoad(const image2D& im, ivec2 p) {
  const float* t = im.data + 4 * ((size_t)p.y * im.w + p.x);
  return vec4(t[0], t[1], t[2], t[3]);
}
inline vec4 imageLoad(const image3D& im, ivec3 p) {
  const float* t = im.data + 4 * (((size_t)p.z * im.h + p.y) * im.w + p.x);
  return vec4(t[0], t[1], t[2], t[3]);
}

inline void filter_axis(float coord, int n, int& i0, int& i1, float& frac) {
  float x = coord * (float)n - 0.5f;
  float fl = std::floor(x);
  frac = x - fl;
  if (!(fl >= -1.0f)) fl = -1.0f;
  if (fl > (float)n) fl = (float)n;
  int i = (int)fl;
  i0 = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
  i1 = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
}
inline vec4 texel(const float* p) { return vec4(p[0], p[1], p[2], p[3]); }
inline vec4 texture(const sampler2D& s, vec2 uv) {
  int x0, x1, y0, y1;
  float a, b;
  filter_axis(uv.x, s.w, x0, x1, a);
  filter_axis(uv.y, s.h, y0, y1, b);
  const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
  const float* p00 = s.data + 4 * ((size_t)y0 * s.w + x0);
  const float* p10 = s.data + 4 * ((size_t)y0 * s.w + x1);
  const float* p01 = s.data + 4 * ((size_t)y1 * s.w + x0);
  const float* p11 = s.data + 4 * ((size_t)y1 * s.w + x1);
  vec4 o;
  float* out[4] = {&o.x, &o.y, &o.z, &o.w};
  for (int c = 0; c < 4; ++c) *out[c] = w00 * p00[c] + w10 * p10[c] + w01 * p01[c] + w11 * p11[c];
  return o;
}
inline vec4 texture(const sampler3D& s, vec3 uvw) {
  int x0, x1, y0, y1, z0, z1;
  float a, b, c;
  filter_axis(uvw.x, s.w, x0, x1, a);
  filter_axis(uvw.y, s.h, y0, y1, b);
  filter_axis(uvw.z, s.d, z0, z1, c);
  const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
  const float w[8] = {ia * ib * ic, a * ib * ic, ia * b * ic, a * b * ic,
                      ia * ib * c,  a * ib * c,  ia * b * c,  a * b * c};
  const int xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
  float acc[4] = {0, 0, 0, 0};
  for (int k = 0; k < 8; ++k) {
    const float* p = s.data + 4 * (((size_t)zs[k >> 2] * s.h + ys[(k >> 1) & 1]) * s.w + xs[k & 1]);
    for (int ch = 0; ch < 4; ++ch) acc[ch] = (k == 0) ? w[k] * p[ch] : acc[ch] + w[k] * p[ch];
  }
  return vec4(acc[0], acc[1], acc[2], acc[3]);
}

}  // namespace glsl
