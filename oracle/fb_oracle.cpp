// fb_oracle.cpp — CPU oracle for the atmosphere LUT precompute.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA library, never part of it.
// It restates the algorithm of the reference's compute shaders with the same
// arithmetic, one function per shader routine; each cites the file:line it
// follows. Build with -ffp-contract=off so that float results follow the
// shaders' operation order term by term (see oracle/build.py).
//
// Texture fetches replace the Vulkan sampler of src/precompute.rs:85-98
// (LINEAR min/mag filter, CLAMP_TO_EDGE on u, v, w, unnormalised coordinate
// u*size-0.5) with exact interpolation weights, combined in the order the
// Vulkan specification writes the bilinear/trilinear sums.
#include "fb_oracle.h"

#include <omp.h>

#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

namespace {

// ---------------------------------------------------------------- scalars ---
template <class T> struct Num;
template <> struct Num<float> {
  static float sqrt(float x) { return std::sqrt(x); }
  static float exp(float x) { return std::exp(x); }
  static float pow(float x, float y) { return std::pow(x, y); }
  static float cos(float x) { return std::cos(x); }
  static float sin(float x) { return std::sin(x); }
  static float floor(float x) { return std::floor(x); }
};
template <> struct Num<double> {
  static double sqrt(double x) { return std::sqrt(x); }
  static double exp(double x) { return std::exp(x); }
  static double pow(double x, double y) { return std::pow(x, y); }
  static double cos(double x) { return std::cos(x); }
  static double sin(double x) { return std::sin(x); }
  static double floor(double x) { return std::floor(x); }
};

// --------------------------------------------------------- op counting ---
// CF: an FP32 scalar that tallies the arithmetic done on it, used only by
// fbo_count_ops to measure the FLOPs per texel of each pass of the reference's
// algorithm. Operations whose operands are all compile-time literals are folded
// (not counted), as a shader compiler folds them; operations that involve a
// uniform (atmosphere parameter), a texel coordinate or a table value count.
struct OpTally {
  uint64_t add = 0, mul = 0, div = 0, sqrt = 0, transc = 0;
  bool on = true;
};
thread_local OpTally g_tally;

struct CF {
  float v = 0.f;
  bool lit = true;  // value of literals only
  CF() = default;
  CF(double x) : v((float)x) {}
  CF(float x) : v(x) {}
  CF(int x) : v((float)x) {}
  CF(unsigned x) : v((float)x) {}
  static CF var(float x) {
    CF c(x);
    c.lit = false;
    return c;
  }
  explicit operator float() const { return v; }
  explicit operator double() const { return v; }
  explicit operator int() const { return (int)v; }
};
inline CF tallied(uint64_t& n, float v, const CF& a, const CF& b) {
  CF o(v);
  o.lit = a.lit && b.lit;
  if (!o.lit && g_tally.on) ++n;
  return o;
}
inline CF operator+(CF a, CF b) { return tallied(g_tally.add, a.v + b.v, a, b); }
inline CF operator-(CF a, CF b) { return tallied(g_tally.add, a.v - b.v, a, b); }
inline CF operator*(CF a, CF b) { return tallied(g_tally.mul, a.v * b.v, a, b); }
inline CF operator/(CF a, CF b) { return tallied(g_tally.div, a.v / b.v, a, b); }
inline CF operator-(CF a) {
  CF o(-a.v);
  o.lit = a.lit;
  return o;
}
inline bool operator<(CF a, CF b) { return a.v < b.v; }
inline bool operator>(CF a, CF b) { return a.v > b.v; }
inline bool operator<=(CF a, CF b) { return a.v <= b.v; }
inline bool operator>=(CF a, CF b) { return a.v >= b.v; }
inline bool operator==(CF a, CF b) { return a.v == b.v; }
inline CF tallied1(uint64_t& n, float v, const CF& a) {
  CF o(v);
  o.lit = a.lit;
  if (!o.lit && g_tally.on) ++n;
  return o;
}
template <> struct Num<CF> {
  static CF sqrt(CF x) { return tallied1(g_tally.sqrt, std::sqrt(x.v), x); }
  static CF exp(CF x) { return tallied1(g_tally.transc, std::exp(x.v), x); }
  static CF pow(CF x, CF y) { return tallied(g_tally.transc, std::pow(x.v, y.v), x, y); }
  static CF cos(CF x) { return tallied1(g_tally.transc, std::cos(x.v), x); }
  static CF sin(CF x) { return tallied1(g_tally.transc, std::sin(x.v), x); }
  static CF floor(CF x) {
    CF o(std::floor(x.v));
    o.lit = x.lit;
    return o;
  }
};
// A value that is uniform over a dispatch (an atmosphere parameter).
template <class T> inline T uni(float x) { return T(x); }
template <> inline CF uni<CF>(float x) { return CF::var(x); }
// Texture filtering is fixed-function sampler work in the reference, not
// shader arithmetic: it is not counted.
template <class T> struct SamplerWork {};
template <> struct SamplerWork<CF> {
  bool saved;
  SamplerWork() : saved(g_tally.on) { g_tally.on = false; }
  ~SamplerWork() { g_tally.on = saved; }
};

// GLSL min/max/clamp as specified (min: y < x ? y : x; max: x < y ? y : x).
template <class T> inline T gmin(T x, T y) { return y < x ? y : x; }
template <class T> inline T gmax(T x, T y) { return x < y ? y : x; }
template <class T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline T kPi() { return T(3.14159265358979323846); }

template <class T> struct V3 {
  T x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(T a, T b, T c) : x(a), y(b), z(c) {}
  static V3 splat(T s) { return V3(s, s, s); }
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot3(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// ------------------------------------------------------------- parameters ---
template <class T> struct Layer { T width, exp_term, exp_scale, linear_term, constant_term; };
template <class T> struct Profile { Layer<T> lo, hi; };

template <class T> struct Atmo {
  V3<T> solar, rayleigh, mie_sca, mie_ext, albedo, absorption;
  T sun_radius, bottom, top, g, mu_s_min;
  Profile<T> ray_d, mie_d, abs_d;
  int tr_mu, tr_r, sc_r, sc_mu, sc_mus, sc_nu, ir_mus, ir_r;
  int tr_steps, ss_steps, ms_steps, dens_n, irr_n, order;
  bool f16;
  bool exact_altitude;  // FP64 oracle: clamp rounding-negative altitudes (see optical_length)
};

template <class T> V3<T> v3(const float* f) { return V3<T>(uni<T>(f[0]), uni<T>(f[1]), uni<T>(f[2])); }
template <class T> Profile<T> prof(const fb_density_profile& p) {
  Profile<T> o;
  const fb_density_profile_layer* L[2] = {&p.layers[0], &p.layers[1]};
  Layer<T>* D[2] = {&o.lo, &o.hi};
  for (int i = 0; i < 2; ++i) {
    D[i]->width = uni<T>(L[i]->width);
    D[i]->exp_term = uni<T>(L[i]->exp_term);
    D[i]->exp_scale = uni<T>(L[i]->exp_scale);
    D[i]->linear_term = uni<T>(L[i]->linear_term);
    D[i]->constant_term = uni<T>(L[i]->constant_term);
  }
  return o;
}

template <class T> Atmo<T> load(const fb_params* p) {
  const fb_params_raw& r = p->raw;
  Atmo<T> a;
  a.solar = v3<T>(r.solar_irradiance);
  a.rayleigh = v3<T>(r.rayleigh_scattering);
  a.mie_sca = v3<T>(r.mie_scattering);
  a.mie_ext = v3<T>(r.mie_extinction);
  a.albedo = v3<T>(r.ground_albedo);
  a.absorption = v3<T>(r.absorption_extinction);
  a.sun_radius = uni<T>(r.sun_angular_radius);
  a.bottom = uni<T>(r.bottom_radius);
  a.top = uni<T>(r.top_radius);
  a.g = uni<T>(r.mie_phase_function_g);
  a.mu_s_min = uni<T>(r.mu_s_min);
  a.ray_d = prof<T>(r.rayleigh_density);
  a.mie_d = prof<T>(r.mie_density);
  a.abs_d = prof<T>(r.absorption_density);
  a.tr_mu = (int)r.transmittance_mu_size;
  a.tr_r = (int)r.transmittance_r_size;
  a.sc_r = (int)r.scattering_r_size;
  a.sc_mu = (int)r.scattering_mu_size;
  a.sc_mus = (int)r.scattering_mu_s_size;
  a.sc_nu = (int)r.scattering_nu_size;
  a.ir_mus = (int)r.irradiance_mu_s_size;
  a.ir_r = (int)r.irradiance_r_size;
  a.tr_steps = (int)p->transmittance_steps;
  a.ss_steps = (int)p->single_scattering_steps;
  a.ms_steps = (int)p->multiple_scattering_steps;
  a.dens_n = (int)p->density_samples;
  a.irr_n = (int)p->irradiance_samples;
  a.order = (int)p->order;
  a.f16 = p->storage == FB_STORAGE_F16;
  a.exact_altitude = std::is_same<T, double>::value;
  return a;
}

bool valid(const fb_params* p) {
  if (!p) return false;
  const fb_params_raw& r = p->raw;
  const uint32_t sizes[8] = {r.transmittance_mu_size, r.transmittance_r_size, r.scattering_r_size,
                             r.scattering_mu_size, r.scattering_mu_s_size, r.scattering_nu_size,
                             r.irradiance_mu_s_size, r.irradiance_r_size};
  for (uint32_t s : sizes)
    if (s < 2 || s > 65536) return false;
  if (r.scattering_mu_size % 2) return false;
  if (!(r.top_radius > r.bottom_radius) || !(r.bottom_radius > 0.f)) return false;
  if (p->order < 1 || p->order > 64) return false;
  if (p->transmittance_steps < 1 || p->single_scattering_steps < 1 || p->multiple_scattering_steps < 1)
    return false;
  if (p->density_samples < 2 || p->density_samples % 2 || p->density_samples > 64) return false;
  if (p->irradiance_samples < 2 || p->irradiance_samples % 2 || p->irradiance_samples > 64) return false;
  return true;
}

// ------------------------------------------------------------ util.h:6-45 ---
template <class T> inline T clamp_cosine(T mu) { return gclamp(mu, T(-1), T(1)); }   // util.h:6-8
template <class T> inline T clamp_distance(T d) { return gmax(d, T(0)); }          // util.h:10-12
template <class T> inline T safe_sqrt(T a) { return Num<T>::sqrt(gmax(a, T(0))); }  // util.h:14-16
// util.h:18-20
template <class T> inline T coord_from_unit(T x, int n) {
  return T(0.5) / T(n) + x * (T(1) - T(1) / T(n));
}
// util.h:22-24
template <class T> inline T unit_from_coord(T u, int n) {
  return (u - T(0.5) / T(n)) / (T(1) - T(1) / T(n));
}
// util.h:26-29
template <class T> inline T phase_rayleigh(T nu) {
  T k = T(3) / (T(16) * kPi<T>());
  return k * (T(1) + nu * nu);
}
// util.h:31-34
template <class T> inline T phase_mie(T g, T nu) {
  T k = T(3) / (T(8) * kPi<T>()) * (T(1) - g * g) / (T(2) + g * g);
  return k * (T(1) + nu * nu) / Num<T>::pow(T(1) + g * g - T(2) * g * nu, T(1.5));
}
// util.h:36-38: texel centre in "fragment" units, size * coord(i / (size - 1)).
template <class T> inline T frag_from_texel(uint32_t i, uint32_t n) {
  return T(n) * coord_from_unit(T(i) / T(n - 1), int(n));
}

// ---------------------------------------------------------- params.h:89-133 ---
template <class T> inline T layer_density(const Layer<T>& L, T h) {  // params.h:89-93
  T d = L.exp_term * Num<T>::exp(L.exp_scale * h) + L.linear_term * h + L.constant_term;
  return gclamp(d, T(0), T(1));
}
template <class T> inline T profile_density(const Profile<T>& P, T h) {  // params.h:95-99
  return h < P.lo.width ? layer_density(P.lo, h) : layer_density(P.hi, h);
}
template <class T> inline T clamp_radius(const Atmo<T>& a, T r) { return gclamp(r, a.bottom, a.top); }  // :101-103
template <class T> inline T dist_top(const Atmo<T>& a, T r, T mu) {  // params.h:105-110
  T disc = r * r * (mu * mu - T(1)) + a.top * a.top;
  return clamp_distance(-r * mu + safe_sqrt(disc));
}
template <class T> inline T dist_bottom(const Atmo<T>& a, T r, T mu) {  // params.h:112-117
  T disc = r * r * (mu * mu - T(1)) + a.bottom * a.bottom;
  return clamp_distance(-r * mu - safe_sqrt(disc));
}
template <class T> inline bool hits_ground(const Atmo<T>& a, T r, T mu) {  // params.h:119-124
  return mu < T(0) && r * r * (mu * mu - T(1)) + a.bottom * a.bottom >= T(0);
}
template <class T> inline T dist_nearest(const Atmo<T>& a, T r, T mu, bool ground) {  // :126-133
  return ground ? dist_bottom(a, r, mu) : dist_top(a, r, mu);
}

// ------------------------------------------------------- table sampling ---
// A read-only RGBA table; `f` points at w*h*d*4 values.
template <class T> struct Tab {
  const T* f;
  int w, h, d;
};

template <class T> inline void axis(T coord, int n, int& i0, int& i1, T& frac) {
  T x = coord * T(n) - T(0.5);
  T fl = Num<T>::floor(x);
  frac = x - fl;
  if (!(fl >= T(-1))) fl = T(-1);  // also catches NaN
  if (fl > T(n)) fl = T(n);
  int i = (int)fl;
  i0 = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
  i1 = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
}

// Bilinear RGB fetch (src/precompute.rs:85-98 sampler; Vulkan weight order).
template <class T> V3<T> fetch2(const Tab<T>& t, T u, T v) {
  SamplerWork<T> not_shader_work;
  int x0, x1, y0, y1;
  T a, b;
  axis(u, t.w, x0, x1, a);
  axis(v, t.h, y0, y1, b);
  const T w00 = (T(1) - a) * (T(1) - b), w10 = a * (T(1) - b), w01 = (T(1) - a) * b, w11 = a * b;
  const T* p00 = t.f + 4 * ((size_t)y0 * t.w + x0);
  const T* p10 = t.f + 4 * ((size_t)y0 * t.w + x1);
  const T* p01 = t.f + 4 * ((size_t)y1 * t.w + x0);
  const T* p11 = t.f + 4 * ((size_t)y1 * t.w + x1);
  V3<T> o;
  T* out[3] = {&o.x, &o.y, &o.z};
  for (int c = 0; c < 3; ++c) *out[c] = w00 * p00[c] + w10 * p10[c] + w01 * p01[c] + w11 * p11[c];
  return o;
}

// Trilinear RGB fetch.
template <class T> V3<T> fetch3(const Tab<T>& t, T u, T v, T s) {
  SamplerWork<T> not_shader_work;
  int x0, x1, y0, y1, z0, z1;
  T a, b, c;
  axis(u, t.w, x0, x1, a);
  axis(v, t.h, y0, y1, b);
  axis(s, t.d, z0, z1, c);
  const T ia = T(1) - a, ib = T(1) - b, ic = T(1) - c;
  const T w[8] = {ia * ib * ic, a * ib * ic, ia * b * ic, a * b * ic,
                  ia * ib * c,  a * ib * c,  ia * b * c,  a * b * c};
  const int xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
  V3<T> o;
  T acc[3] = {0, 0, 0};
  for (int k = 0; k < 8; ++k) {
    const T* p = t.f + 4 * (((size_t)zs[k >> 2] * t.h + ys[(k >> 1) & 1]) * t.w + xs[k & 1]);
    for (int ch = 0; ch < 3; ++ch) acc[ch] = (k == 0) ? w[k] * p[ch] : acc[ch] + w[k] * p[ch];
  }
  o.x = acc[0];
  o.y = acc[1];
  o.z = acc[2];
  return o;
}

// ----------------------------------------------------- transmittance.h ---
template <class T> struct UV { T u, v; };
template <class T> UV<T> tr_uv(const Atmo<T>& a, T r, T mu) {  // transmittance.h:7-24
  T H = Num<T>::sqrt(a.top * a.top - a.bottom * a.bottom);
  T rho = safe_sqrt(r * r - a.bottom * a.bottom);
  T d = dist_top(a, r, mu);
  T d_min = a.top - r;
  T d_max = rho + H;
  T x_mu = (d - d_min) / (d_max - d_min);
  T x_r = rho / H;
  return {coord_from_unit(x_mu, a.tr_mu), coord_from_unit(x_r, a.tr_r)};
}
template <class T> V3<T> tr_to_top(const Atmo<T>& a, const Tab<T>& tr, T r, T mu) {  // :26-33
  UV<T> uv = tr_uv(a, r, mu);
  return fetch2(tr, uv.u, uv.v);
}
template <class T> V3<T> tr_segment(const Atmo<T>& a, const Tab<T>& tr, T r, T mu, T d,
                                    bool ground) {  // transmittance.h:35-61
  T r_d = clamp_radius(a, Num<T>::sqrt(d * d + T(2) * r * mu * d + r * r));
  T mu_d = clamp_cosine((r * mu + d) / r_d);
  V3<T> q = ground ? tr_to_top(a, tr, r_d, -mu_d) / tr_to_top(a, tr, r, -mu)
                   : tr_to_top(a, tr, r, mu) / tr_to_top(a, tr, r_d, mu_d);
  return V3<T>(gmin(q.x, T(1)), gmin(q.y, T(1)), gmin(q.z, T(1)));
}
template <class T> inline T smoothstep(T e0, T e1, T x) {
  T t = gclamp((x - e0) / (e1 - e0), T(0), T(1));
  return t * t * (T(3) - T(2) * t);
}
template <class T> V3<T> tr_to_sun(const Atmo<T>& a, const Tab<T>& tr, T r, T mu_s) {  // :63-74
  T sin_h = a.bottom / r;
  T cos_h = -Num<T>::sqrt(gmax(T(1) - sin_h * sin_h, T(0)));
  return tr_to_top(a, tr, r, mu_s) *
         smoothstep(-sin_h * a.sun_radius, sin_h * a.sun_radius, mu_s - cos_h);
}

// -------------------------------------------------------- irradiance.h ---
template <class T> void irr_r_mus(const Atmo<T>& a, T x_mu_s, T x_r, T& r, T& mu_s) {  // :7-18
  r = a.bottom + x_r * (a.top - a.bottom);
  mu_s = clamp_cosine(T(2) * x_mu_s - T(1));
}
template <class T> V3<T> irr_lookup(const Atmo<T>& a, const Tab<T>& ir, T r, T mu_s) {  // :20-38
  T x_r = (r - a.bottom) / (a.top - a.bottom);
  T x_mu_s = mu_s * T(0.5) + T(0.5);
  return fetch2(ir, coord_from_unit(x_mu_s, a.ir_mus), coord_from_unit(x_r, a.ir_r));
}

// -------------------------------------------------------- scattering.h ---
template <class T> struct Uvwz { T x, y, z, w; };
template <class T> Uvwz<T> sc_uvwz(const Atmo<T>& a, T r, T mu, T mu_s, T nu, bool ground) {  // :7-60
  T H = Num<T>::sqrt(a.top * a.top - a.bottom * a.bottom);
  T rho = safe_sqrt(r * r - a.bottom * a.bottom);
  T u_r = coord_from_unit(rho / H, a.sc_r);
  T r_mu = r * mu;
  T disc = r_mu * r_mu - r * r + a.bottom * a.bottom;
  T u_mu;
  if (ground) {
    T d = -r_mu - safe_sqrt(disc);
    T d_min = r - a.bottom;
    T d_max = rho;
    u_mu = T(0.5) - T(0.5) * coord_from_unit(d_max == d_min ? T(0) : (d - d_min) / (d_max - d_min),
                                             a.sc_mu / 2);
  } else {
    T d = -r_mu + safe_sqrt(disc + H * H);
    T d_min = a.top - r;
    T d_max = rho + H;
    u_mu = T(0.5) + T(0.5) * coord_from_unit((d - d_min) / (d_max - d_min), a.sc_mu / 2);
  }
  T d = dist_top(a, a.bottom, mu_s);
  T d_min = a.top - a.bottom;
  T d_max = H;
  T aa = (d - d_min) / (d_max - d_min);
  T A = T(-2) * a.mu_s_min * a.bottom / (d_max - d_min);
  T u_mu_s = coord_from_unit(gmax(T(1) - aa / A, T(0)) / (T(1) + aa), a.sc_mus);
  T u_nu = (nu + T(1)) / T(2);
  return {u_nu, u_mu_s, u_mu, u_r};
}

template <class T> struct Rmmn { T r, mu, mu_s, nu; bool ground; };
template <class T> Rmmn<T> sc_from_uvwz(const Atmo<T>& a, Uvwz<T> q) {  // scattering.h:62-114
  Rmmn<T> o;
  T H = Num<T>::sqrt(a.top * a.top - a.bottom * a.bottom);
  T rho = H * unit_from_coord(q.w, a.sc_r);
  o.r = Num<T>::sqrt(rho * rho + a.bottom * a.bottom);
  if (q.z < T(0.5)) {
    T d_min = o.r - a.bottom;
    T d_max = rho;
    T d = d_min + (d_max - d_min) * unit_from_coord(T(1) - T(2) * q.z, a.sc_mu / 2);
    o.mu = d == T(0) ? T(-1) : clamp_cosine(-(rho * rho + d * d) / (T(2) * o.r * d));
    o.ground = true;
  } else {
    T d_min = a.top - o.r;
    T d_max = rho + H;
    T d = d_min + (d_max - d_min) * unit_from_coord(T(2) * q.z - T(1), a.sc_mu / 2);
    o.mu = d == T(0) ? T(1) : clamp_cosine((H * H - rho * rho - d * d) / (T(2) * o.r * d));
    o.ground = false;
  }
  T x_mu_s = unit_from_coord(q.y, a.sc_mus);
  T d_min = a.top - a.bottom;
  T d_max = H;
  T A = T(-2) * a.mu_s_min * a.bottom / (d_max - d_min);
  T aa = (A - x_mu_s * A) / (T(1) + x_mu_s * A);
  T d = d_min + gmin(aa, A) * (d_max - d_min);
  o.mu_s = d == T(0) ? T(1) : clamp_cosine((H * H - d * d) / (T(2) * a.bottom * d));
  o.nu = clamp_cosine(q.x * T(2) - T(1));
  return o;
}

// scattering.h:116-137 (texel centre -> parameters, with the nu clamp) and
// scattering.h:181-190 / util.h:36-45 (texel index -> texel centre).
template <class T> Rmmn<T> sc_from_texel(const Atmo<T>& a, uint32_t ix, uint32_t iy, uint32_t iz) {
  const uint32_t W = (uint32_t)(a.sc_nu * a.sc_mus), Hh = (uint32_t)a.sc_mu, D = (uint32_t)a.sc_r;
  T fx = frag_from_texel<T>(ix, W), fy = frag_from_texel<T>(iy, Hh), fz = frag_from_texel<T>(iz, D);
  T nmus = T(a.sc_mus);
  T f_nu = Num<T>::floor(fx / nmus);
  T f_mus = fx - nmus * Num<T>::floor(fx / nmus);  // GLSL mod
  Uvwz<T> q = {f_nu / T(a.sc_nu - 1), f_mus / nmus, fy / T(a.sc_mu), fz / T(a.sc_r)};
  Rmmn<T> o = sc_from_uvwz(a, q);
  T s = Num<T>::sqrt((T(1) - o.mu * o.mu) * (T(1) - o.mu_s * o.mu_s));
  o.nu = gclamp(o.nu, o.mu * o.mu_s - s, o.mu * o.mu_s + s);
  return o;
}

// scattering.h:139-155: 4D lookup = two trilinear fetches in neighbouring nu
// slices, blended linearly.
template <class T> V3<T> sc_lookup(const Atmo<T>& a, const Tab<T>& t, T r, T mu, T mu_s, T nu,
                                   bool ground) {
  Uvwz<T> q = sc_uvwz(a, r, mu, mu_s, nu, ground);
  T tcx = q.x * T(a.sc_nu - 1);
  T tex_x = Num<T>::floor(tcx);
  T lerp = tcx - tex_x;
  T x0 = (tex_x + q.y) / T(a.sc_nu);
  T x1 = (tex_x + T(1) + q.y) / T(a.sc_nu);
  V3<T> f0 = fetch3(t, x0, q.z, q.w);
  V3<T> f1 = fetch3(t, x1, q.z, q.w);
  return f0 * (T(1) - lerp) + f1 * lerp;
}
// scattering.h:157-179: order 1 combines the single Rayleigh and Mie tables
// with their phase functions; higher orders read one table.
template <class T> V3<T> sc_lookup_order(const Atmo<T>& a, const Tab<T>& sr, const Tab<T>& sm,
                                         const Tab<T>& ms, T r, T mu, T mu_s, T nu, bool ground,
                                         int order) {
  if (order == 1) {
    V3<T> ray = sc_lookup(a, sr, r, mu, mu_s, nu, ground);
    V3<T> mie = sc_lookup(a, sm, r, mu, mu_s, nu, ground);
    return ray * phase_rayleigh(nu) + mie * phase_mie(a.g, nu);
  }
  return sc_lookup(a, ms, r, mu, mu_s, nu, ground);
}

// ------------------------------------------------------------ render_sky.h ---
// The renderer's shading (the consumer of the tables): RGBA trilinear fetch,
// the combined scattering lookup, sky radiance to a point, surface lighting.
template <class T> struct V4 { T x, y, z, w; };
template <class T> V4<T> fetch3_rgba(const Tab<T>& t, T u, T v, T s) {
  int x0, x1, y0, y1, z0, z1;
  T a, b, c;
  {
    SamplerWork<T> not_shader_work;
    axis(u, t.w, x0, x1, a);
    axis(v, t.h, y0, y1, b);
    axis(s, t.d, z0, z1, c);
  }
  const T ia = T(1) - a, ib = T(1) - b, ic = T(1) - c;
  const T w[8] = {ia * ib * ic, a * ib * ic, ia * b * ic, a * b * ic,
                  ia * ib * c,  a * ib * c,  ia * b * c,  a * b * c};
  const int xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
  T acc[4] = {T(0), T(0), T(0), T(0)};
  for (int k = 0; k < 8; ++k) {
    const T* p = t.f + 4 * (((size_t)zs[k >> 2] * t.h + ys[(k >> 1) & 1]) * t.w + xs[k & 1]);
    for (int ch = 0; ch < 4; ++ch) acc[ch] = (k == 0) ? w[k] * p[ch] : acc[ch] + w[k] * p[ch];
  }
  return V4<T>{acc[0], acc[1], acc[2], acc[3]};
}
template <class T> V3<T> extrapolated_single_mie(const Atmo<T>& a, V4<T> s) {  // render_sky.h:9-19
  if (s.x <= T(0)) return V3<T>();
  return V3<T>(s.x, s.y, s.z) * s.w / s.x * (a.rayleigh.x / a.mie_sca.x) * (a.mie_sca / a.rayleigh);
}
template <class T>
V3<T> combined_scattering(const Atmo<T>& a, const Tab<T>& sc, T r, T mu, T mu_s, T nu, bool ground,
                          V3<T>& single_mie) {  // render_sky.h:21-43
  Uvwz<T> q = sc_uvwz(a, r, mu, mu_s, nu, ground);
  T tcx = q.x * T(a.sc_nu - 1);
  T tex_x = Num<T>::floor(tcx);
  T lerp = tcx - tex_x;
  V4<T> s0 = fetch3_rgba(sc, (tex_x + q.y) / T(a.sc_nu), q.z, q.w);
  V4<T> s1 = fetch3_rgba(sc, (tex_x + T(1) + q.y) / T(a.sc_nu), q.z, q.w);
  V4<T> m{s0.x * (T(1) - lerp) + s1.x * lerp, s0.y * (T(1) - lerp) + s1.y * lerp,
          s0.z * (T(1) - lerp) + s1.z * lerp, s0.w * (T(1) - lerp) + s1.w * lerp};
  single_mie = extrapolated_single_mie(a, m);
  return V3<T>(m.x, m.y, m.z);
}
template <class T> inline T len3(V3<T> v) { return Num<T>::sqrt(dot3(v, v)); }
// render_sky.h:111-191 (no light shafts: shadow_length 0)
template <class T>
V3<T> sky_radiance_to_point(const Atmo<T>& a, const Tab<T>& tr, const Tab<T>& sc, V3<T> camera, V3<T> view,
                            V3<T> point, V3<T> sun, V3<T>& transmittance) {
  T r = len3(camera);
  T rmu = dot3(camera, view);
  T to_top = -rmu - Num<T>::sqrt(rmu * rmu - r * r + a.top * a.top);
  if (to_top > T(0)) {
    camera = camera + view * to_top;
    r = a.top;
    rmu = rmu + to_top;
  } else if (r > a.top) {
    transmittance = V3<T>::splat(T(1));
    return V3<T>();
  }
  T mu = rmu / r;
  T mu_s = dot3(camera, sun) / r;
  T nu = dot3(view, sun);
  T d = len3(point - camera);
  bool ground = hits_ground(a, r, mu);
  transmittance = tr_segment(a, tr, r, mu, d, ground);
  V3<T> single_mie;
  V3<T> scattering = combined_scattering(a, sc, r, mu, mu_s, nu, ground, single_mie);
  if (!std::isinf((double)d)) {
    T r_p = clamp_radius(a, Num<T>::sqrt(d * d + T(2) * r * mu * d + r * r));
    T mu_p = (r * mu + d) / r_p;
    T mu_s_p = (r * mu_s + d * nu) / r_p;
    V3<T> single_mie_p;
    V3<T> scattering_p = combined_scattering(a, sc, r_p, mu_p, mu_s_p, nu, ground, single_mie_p);
    V3<T> shadow = transmittance;
    scattering = scattering - shadow * scattering_p;
    single_mie = single_mie - shadow * single_mie_p;
    single_mie = extrapolated_single_mie(a, V4<T>{scattering.x, scattering.y, scattering.z, single_mie.x});
    single_mie = single_mie * smoothstep(T(0), T(0.01), mu_s);
  }
  return scattering * phase_rayleigh(nu) + single_mie * phase_mie(a.g, nu);
}
// render_lighting.h:10-28
template <class T>
V3<T> sun_and_sky_irradiance(const Atmo<T>& a, const Tab<T>& tr, const Tab<T>& ir, V3<T> point, V3<T> normal,
                             V3<T> sun, V3<T>& sky) {
  T r = len3(point);
  T mu_s = dot3(point, sun) / r;
  sky = irr_lookup(a, ir, r, mu_s) * ((T(1) + dot3(normal, point) / r) * T(0.5));
  return a.solar * tr_to_sun(a, tr, r, mu_s) * gmax(dot3(normal, sun), T(0));
}

template <class T>
int render_sky(const fb_params* p, const T* tr, const T* sc, const fb_draw_parameters* d, const T* depth,
               uint32_t width, uint32_t height, T* color, T* trans) {
  if (!valid(p) || !tr || !sc || !d || !color || width == 0 || height == 0) return FB_ERR_INVALID_ARGUMENT;
  const Atmo<T> a = load<T>(p);
  const Tab<T> ttr{tr, a.tr_mu, a.tr_r, 1}, tsc{sc, a.sc_nu * a.sc_mus, a.sc_mu, a.sc_r};
  T m[4][4];
  for (int c = 0; c < 4; ++c)
    for (int row = 0; row < 4; ++row) m[c][row] = T(d->inverse_viewproj[c][row]);
  const V3<T> camera = v3<T>(d->camera_position), sun = v3<T>(d->sun_direction);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < (int64_t)width * height; ++k) {
    const uint32_t x = (uint32_t)(k % width), y = (uint32_t)(k / width);
    // render_sky.frag:24-34
    const T sx = T(2) * ((T(x) + T(0.5)) / T(width)) - T(1), sy = T(2) * ((T(y) + T(0.5)) / T(height)) - T(1);
    const T dz = depth ? depth[k] : T(0);
    T v[4], w[4];
    for (int row = 0; row < 4; ++row) {
      v[row] = m[0][row] * sx + m[1][row] * sy + m[2][row] * T(0) + m[3][row] * T(1);
      w[row] = m[0][row] * sx + m[1][row] * sy + m[2][row] * dz + m[3][row] * T(1);
    }
    V3<T> view(v[0], v[1], v[2]);
    view = view / len3(view);
    const V3<T> world = (V3<T>(w[0], w[1], w[2]) / w[3]) * T(1e-3);
    V3<T> t;
    const V3<T> c = sky_radiance_to_point(a, ttr, tsc, camera, view, world, sun, t);
    color[4 * k] = c.x;
    color[4 * k + 1] = c.y;
    color[4 * k + 2] = c.z;
    color[4 * k + 3] = T(0);
    if (trans) {
      trans[4 * k] = t.x;
      trans[4 * k + 1] = t.y;
      trans[4 * k + 2] = t.z;
      trans[4 * k + 3] = T(1);
    }
  }
  return FB_OK;
}

template <class T>
int lighting(const fb_params* p, const T* tr, const T* ir, const T* points, const T* normals, const T* sun_dir,
             int64_t n, T* sun_out, T* sky_out) {
  if (!valid(p) || !tr || !ir || !points || !normals || !sun_dir || !sun_out || !sky_out)
    return FB_ERR_INVALID_ARGUMENT;
  const Atmo<T> a = load<T>(p);
  const Tab<T> ttr{tr, a.tr_mu, a.tr_r, 1}, tir{ir, a.ir_mus, a.ir_r, 1};
  const V3<T> sun(sun_dir[0], sun_dir[1], sun_dir[2]);
#pragma omp parallel for
  for (int64_t k = 0; k < n; ++k) {
    V3<T> sky;
    const V3<T> direct = sun_and_sky_irradiance(a, ttr, tir, V3<T>(points[3 * k], points[3 * k + 1], points[3 * k + 2]),
                                                V3<T>(normals[3 * k], normals[3 * k + 1], normals[3 * k + 2]), sun, sky);
    sun_out[3 * k] = direct.x;
    sun_out[3 * k + 1] = direct.y;
    sun_out[3 * k + 2] = direct.z;
    sky_out[3 * k] = sky.x;
    sky_out[3 * k + 1] = sky.y;
    sky_out[3 * k + 2] = sky.z;
  }
  return FB_OK;
}

// ------------------------------------------------------------- the passes ---
template <class T> inline T store_round(T v, bool f16) {
  if (!f16) return v;
  return T((float)(_Float16)(float)v);
}

// transmittance.comp:8-32 — trapezoidal optical length to the top boundary.
template <class T> T optical_length(const Atmo<T>& a, const Profile<T>& P, T r, T mu) {
  const int N = a.tr_steps;
  T dx = dist_top(a, r, mu) / T(N);
  T result = T(0);
  for (int i = 0; i <= N; ++i) {
    T d_i = T(i) * dx;
    T r_i = Num<T>::sqrt(d_i * d_i + T(2) * r * mu * d_i + r * r);
    T h_i = r_i - a.bottom;
    // Every ray of the transmittance table stays above the ground in exact
    // arithmetic (mu is at or above the horizon), so a negative altitude is a
    // rounding artefact; the FP64 oracle evaluates the exact-arithmetic value
    // (h = 0 at a tangent sample). The FP32 oracle keeps the reference's
    // unclamped arithmetic.
    if (a.exact_altitude && h_i < T(0)) h_i = T(0);
    T y_i = profile_density(P, h_i);
    T w = (i == 0 || i == N) ? T(0.5) : T(1);
    result = result + y_i * w * dx;
  }
  return result;
}

// transmittance.comp:34-80
template <class T> void transmittance_texel(const Atmo<T>& a, int64_t t, T* out) {
  const int i = (int)(t % a.tr_mu), j = (int)(t / a.tr_mu);
  T x_mu = T(i) / T(a.tr_mu - 1);
  T x_r = T(j) / T(a.tr_r - 1);
  // transmittance.comp:48-64
  T H = Num<T>::sqrt(a.top * a.top - a.bottom * a.bottom);
  T rho = H * x_r;
  T r = Num<T>::sqrt(rho * rho + a.bottom * a.bottom);
  T d_min = a.top - r;
  T d_max = rho + H;
  T d = d_min + x_mu * (d_max - d_min);
  T mu = d == T(0) ? T(1) : (H * H - rho * rho - d * d) / (T(2) * r * d);
  mu = clamp_cosine(mu);
  T lr = optical_length(a, a.ray_d, r, mu);
  T lm = optical_length(a, a.mie_d, r, mu);
  T la = optical_length(a, a.abs_d, r, mu);
  V3<T> tau = a.rayleigh * lr + a.mie_ext * lm + a.absorption * la;
  out[0] = Num<T>::exp(-tau.x);
  out[1] = Num<T>::exp(-tau.y);
  out[2] = Num<T>::exp(-tau.z);
  out[3] = T(1);
}

// direct_irradiance.comp:10-46
template <class T> void direct_irradiance_texel(const Atmo<T>& a, const Tab<T>& tr, int64_t t, T* out) {
  const int i = (int)(t % a.ir_mus), j = (int)(t / a.ir_mus);
  T r, mu_s;
  irr_r_mus(a, T(i) / T(a.ir_mus - 1), T(j) / T(a.ir_r - 1), r, mu_s);
  T al = a.sun_radius;
  T avg = mu_s < -al ? T(0) : (mu_s > al ? mu_s : (mu_s + al) * (mu_s + al) / (T(4) * al));
  V3<T> v = a.solar * tr_to_top(a, tr, r, mu_s) * avg;
  out[0] = v.x;
  out[1] = v.y;
  out[2] = v.z;
  out[3] = T(0);
}

template <class T> void texel_xyz(const Atmo<T>& a, int64_t t, uint32_t& x, uint32_t& y, uint32_t& z) {
  const int64_t W = (int64_t)a.sc_nu * a.sc_mus;
  x = (uint32_t)(t % W);
  y = (uint32_t)((t / W) % a.sc_mu);
  z = (uint32_t)(t / (W * a.sc_mu));
}

// single_scattering.comp:10-101
template <class T> void single_scattering_texel(const Atmo<T>& a, const Tab<T>& tr, int64_t t,
                                                T* out_r, T* out_m) {
  uint32_t x, y, z;
  texel_xyz(a, t, x, y, z);
  Rmmn<T> s = sc_from_texel(a, x, y, z);
  const int N = a.ss_steps;
  T dx = dist_nearest(a, s.r, s.mu, s.ground) / T(N);
  V3<T> ray_sum, mie_sum;
  for (int i = 0; i <= N; ++i) {
    T d = T(i) * dx;
    // single_scattering.comp:10-28
    T r_d = clamp_radius(a, Num<T>::sqrt(d * d + T(2) * s.r * s.mu * d + s.r * s.r));
    T mu_s_d = clamp_cosine((s.r * s.mu_s + d * s.nu) / r_d);
    V3<T> tt = tr_segment(a, tr, s.r, s.mu, d, s.ground) * tr_to_sun(a, tr, r_d, mu_s_d);
    V3<T> ray_i = tt * profile_density(a.ray_d, r_d - a.bottom);
    V3<T> mie_i = tt * profile_density(a.mie_d, r_d - a.bottom);
    T w = (i == 0 || i == N) ? T(0.5) : T(1);
    ray_sum = ray_sum + ray_i * w;
    mie_sum = mie_sum + mie_i * w;
  }
  V3<T> ray = ray_sum * dx * a.solar * a.rayleigh;
  V3<T> mie = mie_sum * dx * a.solar * a.mie_sca;
  out_r[0] = ray.x; out_r[1] = ray.y; out_r[2] = ray.z; out_r[3] = T(0);
  out_m[0] = mie.x; out_m[1] = mie.y; out_m[2] = mie.z; out_m[3] = T(0);
}

// scattering_density.comp:10-107
template <class T> void density_texel(const Atmo<T>& a, int order, const Tab<T>& tr, const Tab<T>& sr,
                                      const Tab<T>& sm, const Tab<T>& ms, const Tab<T>& irr, int64_t t,
                                      T* out) {
  uint32_t x, y, z;
  texel_xyz(a, t, x, y, z);
  Rmmn<T> s = sc_from_texel(a, x, y, z);
  const T r = s.r, mu = s.mu, mu_s = s.mu_s, nu = s.nu;
  V3<T> omega(Num<T>::sqrt(T(1) - mu * mu), T(0), mu);
  T sun_x = omega.x == T(0) ? T(0) : (nu - mu * mu_s) / omega.x;
  T sun_y = Num<T>::sqrt(gmax(T(1) - sun_x * sun_x - mu_s * mu_s, T(0)));
  V3<T> omega_s(sun_x, sun_y, mu_s);
  const int N = a.dens_n;
  const T dphi = kPi<T>() / T(N);
  const T dtheta = kPi<T>() / T(N);
  const T ray_rho = profile_density(a.ray_d, r - a.bottom);
  const T mie_rho = profile_density(a.mie_d, r - a.bottom);
  V3<T> acc;
  for (int l = 0; l < N; ++l) {
    T theta = (T(l) + T(0.5)) * dtheta;
    T ct = Num<T>::cos(theta);
    T st = Num<T>::sin(theta);
    bool g = hits_ground(a, r, ct);
    T dist_g = T(0);
    V3<T> t_g, alb;
    if (g) {
      dist_g = dist_bottom(a, r, ct);
      t_g = tr_segment(a, tr, r, ct, dist_g, true);
      alb = a.albedo;
    }
    for (int m = 0; m < 2 * N; ++m) {
      T phi = (T(m) + T(0.5)) * dphi;
      V3<T> wi(Num<T>::cos(phi) * st, Num<T>::sin(phi) * st, ct);
      T domega = dtheta * dphi * Num<T>::sin(theta);
      T nu1 = dot3(omega_s, wi);
      V3<T> inc = sc_lookup_order(a, sr, sm, ms, r, wi.z, mu_s, nu1, g, order - 1);
      // Ground bounce: n = normalize(zenith * r + wi * dist_g).
      V3<T> gp(T(0) * r + wi.x * dist_g, T(0) * r + wi.y * dist_g, T(1) * r + wi.z * dist_g);
      T len = Num<T>::sqrt(dot3(gp, gp));
      V3<T> gn = gp / len;
      V3<T> girr = irr_lookup(a, irr, a.bottom, dot3(gn, omega_s));
      inc = inc + t_g * alb * (T(1) / kPi<T>()) * girr;
      T nu2 = dot3(omega, wi);
      V3<T> coef = a.rayleigh * ray_rho * phase_rayleigh(nu2) + a.mie_sca * mie_rho * phase_mie(a.g, nu2);
      acc = acc + inc * coef * domega;
    }
  }
  out[0] = acc.x; out[1] = acc.y; out[2] = acc.z; out[3] = T(0);
}

// indirect_irradiance.comp:10-74
template <class T> void indirect_texel(const Atmo<T>& a, int order, const Tab<T>& sr, const Tab<T>& sm,
                                       const Tab<T>& ms, int64_t t, T* out) {
  const int i = (int)(t % a.ir_mus), j = (int)(t / a.ir_mus);
  T r, mu_s;
  irr_r_mus(a, T(i) / T(a.ir_mus - 1), T(j) / T(a.ir_r - 1), r, mu_s);
  const int N = a.irr_n;
  const T dphi = kPi<T>() / T(N);
  const T dtheta = kPi<T>() / T(N);
  V3<T> res;
  V3<T> omega_s(Num<T>::sqrt(T(1) - mu_s * mu_s), T(0), mu_s);
  for (int jj = 0; jj < N / 2; ++jj) {
    T theta = (T(jj) + T(0.5)) * dtheta;
    for (int ii = 0; ii < 2 * N; ++ii) {
      T phi = (T(ii) + T(0.5)) * dphi;
      V3<T> w(Num<T>::cos(phi) * Num<T>::sin(theta), Num<T>::sin(phi) * Num<T>::sin(theta),
              Num<T>::cos(theta));
      T domega = dtheta * dphi * Num<T>::sin(theta);
      T nu = dot3(w, omega_s);
      res = res + sc_lookup_order(a, sr, sm, ms, r, w.z, mu_s, nu, false, order) * w.z * domega;
    }
  }
  out[0] = res.x; out[1] = res.y; out[2] = res.z; out[3] = T(0);
}

// multiple_scattering.comp:9-93
template <class T> void multiple_texel(const Atmo<T>& a, const Tab<T>& tr, const Tab<T>& dens, int64_t t,
                                       T* out, T* phase) {
  uint32_t x, y, z;
  texel_xyz(a, t, x, y, z);
  Rmmn<T> s = sc_from_texel(a, x, y, z);
  const int N = a.ms_steps;
  T dx = dist_nearest(a, s.r, s.mu, s.ground) / T(N);
  V3<T> sum;
  for (int i = 0; i <= N; ++i) {
    T d_i = T(i) * dx;
    T r_i = clamp_radius(a, Num<T>::sqrt(d_i * d_i + T(2) * s.r * s.mu * d_i + s.r * s.r));
    T mu_i = clamp_cosine((s.r * s.mu + d_i) / r_i);
    T mu_s_i = clamp_cosine((s.r * s.mu_s + d_i * s.nu) / r_i);
    V3<T> v = sc_lookup(a, dens, r_i, mu_i, mu_s_i, s.nu, s.ground) *
              tr_segment(a, tr, s.r, s.mu, d_i, s.ground) * dx;
    T w = (i == 0 || i == N) ? T(0.5) : T(1);
    sum = sum + v * w;
  }
  out[0] = sum.x; out[1] = sum.y; out[2] = sum.z; out[3] = T(0);
  if (phase) *phase = phase_rayleigh(s.nu);
}

// ------------------------------------------------------------------ driver ---
struct Threads {
  explicit Threads(int n) : saved(omp_get_max_threads()) {
    if (n > 0) omp_set_num_threads(n);
  }
  ~Threads() { omp_set_num_threads(saved); }
  int saved;
};

template <class F> void for_texels(const int64_t* idx, int64_t n, F&& f) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < n; ++k) f(k, idx ? idx[k] : k);
}

template <class T> Tab<T> tab(const T* f, int w, int h, int d = 1) { return Tab<T>{f, w, h, d}; }

template <class T> int precompute(const fb_params* p, int nthreads, T* tr, T* irr, T* sc, T* orders_ms,
                                  T* orders_irr, T* single_r, T* single_m) {
  if (!valid(p) || !tr || !irr || !sc) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  const int64_t ntr = (int64_t)a.tr_mu * a.tr_r, nir = (int64_t)a.ir_mus * a.ir_r;
  const int64_t nsc = (int64_t)a.sc_nu * a.sc_mus * a.sc_mu * a.sc_r;
  const int W = a.sc_nu * a.sc_mus;
  std::vector<T> dirr(4 * nir), dr(4 * nsc), dm(4 * nsc), dms(4 * nsc, T(0)), dens(4 * nsc);
  // Pass order of src/precompute.rs:1726-1999.
  for_texels(nullptr, ntr, [&](int64_t k, int64_t t) { transmittance_texel(a, t, tr + 4 * k); });
  const Tab<T> ttr = tab<T>(tr, a.tr_mu, a.tr_r);
  for_texels(nullptr, nir, [&](int64_t k, int64_t t) { direct_irradiance_texel(a, ttr, t, dirr.data() + 4 * k); });
  for_texels(nullptr, nsc, [&](int64_t k, int64_t t) {
    T* r = dr.data() + 4 * k;
    T* m = dm.data() + 4 * k;
    single_scattering_texel(a, ttr, t, r, m);
    T* s = sc + 4 * k;
    s[0] = r[0]; s[1] = r[1]; s[2] = r[2]; s[3] = m[0];  // single_scattering.comp:100
    for (int c = 0; c < 4; ++c) {
      r[c] = store_round(r[c], a.f16);
      m[c] = store_round(m[c], a.f16);
      s[c] = store_round(s[c], a.f16);
    }
  });
  std::memset(irr, 0, sizeof(T) * 4 * nir);  // src/precompute.rs:1802-1816
  const Tab<T> tsr = tab<T>(dr.data(), W, a.sc_mu, a.sc_r), tsm = tab<T>(dm.data(), W, a.sc_mu, a.sc_r);
  const Tab<T> tms = tab<T>(dms.data(), W, a.sc_mu, a.sc_r), tde = tab<T>(dens.data(), W, a.sc_mu, a.sc_r);
  const Tab<T> tdi = tab<T>(dirr.data(), a.ir_mus, a.ir_r);
  std::vector<T> next_irr(4 * nir);
  for (int order = 2; order <= a.order; ++order) {
    for_texels(nullptr, nsc, [&](int64_t k, int64_t t) {
      T* o = dens.data() + 4 * k;
      density_texel(a, order, ttr, tsr, tsm, tms, tdi, t, o);
      for (int c = 0; c < 4; ++c) o[c] = store_round(o[c], a.f16);
    });
    for_texels(nullptr, nir, [&](int64_t k, int64_t t) { indirect_texel(a, order - 1, tsr, tsm, tms, t, next_irr.data() + 4 * k); });
    for (int64_t k = 0; k < 4 * nir; ++k) {
      dirr[k] = next_irr[k];
      irr[k] = next_irr[k] + irr[k];  // indirect_irradiance.comp:72-73
    }
    if (orders_irr) std::memcpy(orders_irr + (size_t)(order - 2) * 4 * nir, dirr.data(), sizeof(T) * 4 * nir);
    for_texels(nullptr, nsc, [&](int64_t k, int64_t t) {
      T v[4], phase;
      multiple_texel(a, ttr, tde, t, v, &phase);
      T* o = dms.data() + 4 * k;
      T* s = sc + 4 * k;
      for (int c = 0; c < 3; ++c) s[c] = store_round(v[c] / phase + s[c], a.f16);  // :91-92
      s[3] = store_round(T(0) + s[3], a.f16);
      for (int c = 0; c < 4; ++c) o[c] = store_round(v[c], a.f16);
    });
    if (orders_ms) std::memcpy(orders_ms + (size_t)(order - 2) * 4 * nsc, dms.data(), sizeof(T) * 4 * nsc);
  }
  if (single_r) std::memcpy(single_r, dr.data(), sizeof(T) * 4 * nsc);
  if (single_m) std::memcpy(single_m, dm.data(), sizeof(T) * 4 * nsc);
  return FB_OK;
}

template <class T>
int density_impl(const fb_params* p, int nthreads, int order, const T* tr, const T* sr, const T* sm,
                        const T* ms, const T* dirr, const int64_t* idx, int64_t n, T* out) {
  if (!valid(p) || !tr || !dirr || !out || order < 2) return FB_ERR_INVALID_ARGUMENT;
  if (order == 2 && (!sr || !sm)) return FB_ERR_INVALID_ARGUMENT;
  if (order > 2 && !ms) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  const int W = a.sc_nu * a.sc_mus;
  if (!idx) n = (int64_t)W * a.sc_mu * a.sc_r;
  const Tab<T> ttr = tab<T>(tr, a.tr_mu, a.tr_r), tdi = tab<T>(dirr, a.ir_mus, a.ir_r);
  const Tab<T> tsr = tab<T>(sr ? sr : ms, W, a.sc_mu, a.sc_r), tsm = tab<T>(sm ? sm : ms, W, a.sc_mu, a.sc_r);
  const Tab<T> tms = tab<T>(ms ? ms : sr, W, a.sc_mu, a.sc_r);
  for_texels(idx, n, [&](int64_t k, int64_t x) { density_texel(a, order, ttr, tsr, tsm, tms, tdi, x, out + 4 * k); });
  return FB_OK;
}

template <class T>
int multiple_impl(const fb_params* p, int nthreads, const T* tr, const T* dens, const int64_t* idx,
                         int64_t n, T* out, T* phase) {
  if (!valid(p) || !tr || !dens || !out) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  const int W = a.sc_nu * a.sc_mus;
  if (!idx) n = (int64_t)W * a.sc_mu * a.sc_r;
  const Tab<T> ttr = tab<T>(tr, a.tr_mu, a.tr_r), tde = tab<T>(dens, W, a.sc_mu, a.sc_r);
  for_texels(idx, n, [&](int64_t k, int64_t x) { multiple_texel(a, ttr, tde, x, out + 4 * k, phase ? phase + k : nullptr); });
  return FB_OK;
}

template <class T> int transmittance_impl(const fb_params* p, int nthreads, const int64_t* idx, int64_t n, T* out) {
  if (!valid(p) || !out) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  if (!idx) n = (int64_t)a.tr_mu * a.tr_r;
  for_texels(idx, n, [&](int64_t k, int64_t t) { transmittance_texel(a, t, out + 4 * k); });
  return FB_OK;
}

template <class T>
int direct_impl(const fb_params* p, int nthreads, const T* tr, const int64_t* idx, int64_t n, T* out) {
  if (!valid(p) || !out || !tr) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  if (!idx) n = (int64_t)a.ir_mus * a.ir_r;
  const Tab<T> t = tab<T>(tr, a.tr_mu, a.tr_r);
  for_texels(idx, n, [&](int64_t k, int64_t x) { direct_irradiance_texel(a, t, x, out + 4 * k); });
  return FB_OK;
}

template <class T>
int single_impl(const fb_params* p, int nthreads, const T* tr, const int64_t* idx, int64_t n, T* out_r, T* out_m) {
  if (!valid(p) || !tr || !out_r || !out_m) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  if (!idx) n = (int64_t)a.sc_nu * a.sc_mus * a.sc_mu * a.sc_r;
  const Tab<T> t = tab<T>(tr, a.tr_mu, a.tr_r);
  for_texels(idx, n, [&](int64_t k, int64_t x) { single_scattering_texel(a, t, x, out_r + 4 * k, out_m + 4 * k); });
  return FB_OK;
}

template <class T>
int indirect_impl(const fb_params* p, int nthreads, int order, const T* sr, const T* sm, const T* ms,
                  const int64_t* idx, int64_t n, T* out) {
  if (!valid(p) || !out || order < 1) return FB_ERR_INVALID_ARGUMENT;
  if (order == 1 && (!sr || !sm)) return FB_ERR_INVALID_ARGUMENT;
  if (order > 1 && !ms) return FB_ERR_INVALID_ARGUMENT;
  Threads th(nthreads);
  const Atmo<T> a = load<T>(p);
  const int W = a.sc_nu * a.sc_mus;
  if (!idx) n = (int64_t)a.ir_mus * a.ir_r;
  const Tab<T> tsr = tab<T>(sr ? sr : ms, W, a.sc_mu, a.sc_r), tsm = tab<T>(sm ? sm : ms, W, a.sc_mu, a.sc_r);
  const Tab<T> tms = tab<T>(ms ? ms : sr, W, a.sc_mu, a.sc_r);
  for_texels(idx, n, [&](int64_t k, int64_t x) { indirect_texel(a, order, tsr, tsm, tms, x, out + 4 * k); });
  return FB_OK;
}

}  // namespace

// Op counts of the reference's algorithm: runs one pass's texel routine over
// `n` texels drawn uniformly (fixed LCG from `seed`) with CF scalars on zero
// tables (the arithmetic does not depend on table values), and returns the
// mean per texel of: adds/subs, muls, divs, sqrts, transcendentals (exp, pow,
// cos, sin). Sampler filtering is excluded (see SamplerWork).
int count_ops(const fb_params* p, int pass, int order, int64_t n, uint64_t seed, double* out) {
  if (!valid(p) || !out || n <= 0 || pass < 0 || pass > 5) return FB_ERR_INVALID_ARGUMENT;
  const Atmo<CF> a = load<CF>(p);
  const int64_t ntr = (int64_t)a.tr_mu * a.tr_r, nir = (int64_t)a.ir_mus * a.ir_r;
  const int64_t nsc = (int64_t)a.sc_nu * a.sc_mus * a.sc_mu * a.sc_r;
  const int W = a.sc_nu * a.sc_mus;
  std::vector<CF> tr(4 * ntr, CF::var(0.f)), ir(4 * nir, CF::var(0.f)), sc(4 * nsc, CF::var(0.f));
  const Tab<CF> ttr = tab<CF>(tr.data(), a.tr_mu, a.tr_r), tir = tab<CF>(ir.data(), a.ir_mus, a.ir_r);
  const Tab<CF> tsc = tab<CF>(sc.data(), W, a.sc_mu, a.sc_r);
  const int64_t count[6] = {ntr, nir, nsc, nsc, nir, nsc};
  g_tally = OpTally();
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  CF o[4], o2[4], ph;
  for (int64_t k = 0; k < n; ++k) {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    const int64_t t = (int64_t)((st >> 17) % (uint64_t)count[pass]);
    switch (pass) {
      case 0: transmittance_texel(a, t, o); break;
      case 1: direct_irradiance_texel(a, ttr, t, o); break;
      case 2: single_scattering_texel(a, ttr, t, o, o2); break;
      case 3: density_texel(a, order, ttr, tsc, tsc, tsc, tir, t, o); break;
      case 4: indirect_texel(a, order, tsc, tsc, tsc, t, o); break;
      default: multiple_texel(a, ttr, tsc, t, o, &ph); break;
    }
  }
  const double dn = (double)n;
  out[0] = g_tally.add / dn;
  out[1] = g_tally.mul / dn;
  out[2] = g_tally.div / dn;
  out[3] = g_tally.sqrt / dn;
  out[4] = g_tally.transc / dn;
  return FB_OK;
}

extern "C" {

int fbo_precompute_f32(const fb_params* p, int nthreads, float* tr, float* ir, float* sc, float* oms,
                       float* oirr, float* sr, float* sm) {
  return precompute<float>(p, nthreads, tr, ir, sc, oms, oirr, sr, sm);
}
int fbo_precompute_f64(const fb_params* p, int nthreads, double* tr, double* ir, double* sc, double* oms,
                       double* oirr, double* sr, double* sm) {
  return precompute<double>(p, nthreads, tr, ir, sc, oms, oirr, sr, sm);
}

int fbo_transmittance_f32(const fb_params* p, int nthreads, const int64_t* idx, int64_t n, float* out) {
  return transmittance_impl<float>(p, nthreads, idx, n, out);
}
int fbo_transmittance_f64(const fb_params* p, int nthreads, const int64_t* idx, int64_t n, double* out) {
  return transmittance_impl<double>(p, nthreads, idx, n, out);
}
int fbo_direct_irradiance_f32(const fb_params* p, int nthreads, const float* tr, const int64_t* idx, int64_t n,
                              float* out) {
  return direct_impl<float>(p, nthreads, tr, idx, n, out);
}
int fbo_direct_irradiance_f64(const fb_params* p, int nthreads, const double* tr, const int64_t* idx, int64_t n,
                              double* out) {
  return direct_impl<double>(p, nthreads, tr, idx, n, out);
}
int fbo_single_scattering_f32(const fb_params* p, int nthreads, const float* tr, const int64_t* idx, int64_t n,
                              float* out_r, float* out_m) {
  return single_impl<float>(p, nthreads, tr, idx, n, out_r, out_m);
}
int fbo_single_scattering_f64(const fb_params* p, int nthreads, const double* tr, const int64_t* idx, int64_t n,
                              double* out_r, double* out_m) {
  return single_impl<double>(p, nthreads, tr, idx, n, out_r, out_m);
}

int fbo_scattering_density_f32(const fb_params* p, int nthreads, int order, const float* tr, const float* sr,
                               const float* sm, const float* ms, const float* dirr, const int64_t* idx,
                               int64_t n, float* out) {
  return density_impl<float>(p, nthreads, order, tr, sr, sm, ms, dirr, idx, n, out);
}
int fbo_scattering_density_f64(const fb_params* p, int nthreads, int order, const double* tr, const double* sr,
                               const double* sm, const double* ms, const double* dirr, const int64_t* idx,
                               int64_t n, double* out) {
  return density_impl<double>(p, nthreads, order, tr, sr, sm, ms, dirr, idx, n, out);
}

int fbo_indirect_irradiance_f32(const fb_params* p, int nthreads, int order, const float* sr, const float* sm,
                                const float* ms, const int64_t* idx, int64_t n, float* out) {
  return indirect_impl<float>(p, nthreads, order, sr, sm, ms, idx, n, out);
}
int fbo_indirect_irradiance_f64(const fb_params* p, int nthreads, int order, const double* sr, const double* sm,
                                const double* ms, const int64_t* idx, int64_t n, double* out) {
  return indirect_impl<double>(p, nthreads, order, sr, sm, ms, idx, n, out);
}

int fbo_multiple_scattering_f32(const fb_params* p, int nthreads, const float* tr, const float* dens,
                                const int64_t* idx, int64_t n, float* out, float* phase) {
  return multiple_impl<float>(p, nthreads, tr, dens, idx, n, out, phase);
}
int fbo_multiple_scattering_f64(const fb_params* p, int nthreads, const double* tr, const double* dens,
                                const int64_t* idx, int64_t n, double* out, double* phase) {
  return multiple_impl<double>(p, nthreads, tr, dens, idx, n, out, phase);
}

void fbo_params_default(fb_params* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  fb_params_raw& r = o->raw;
  // src/precompute.rs:849-935
  const float solar[3] = {1.474f, 1.850f, 1.91198f};
  const float ray[3] = {0.005802f, 0.013558f, 0.033100f};
  const float absorb[3] = {6.5e-4f, 1.881e-3f, 8.5e-5f};
  for (int c = 0; c < 3; ++c) {
    r.solar_irradiance[c] = solar[c];
    r.rayleigh_scattering[c] = ray[c];
    r.mie_scattering[c] = 0.003996f;
    r.mie_extinction[c] = 0.004440f;
    r.ground_albedo[c] = 0.1f;
    r.absorption_extinction[c] = absorb[c];
  }
  r.sun_angular_radius = 0.004675f;
  r.bottom_radius = 6360.0f;
  r.top_radius = 6420.0f;
  r.mie_phase_function_g = 0.8f;
  r.mu_s_min = -0.207912f;
  r.transmittance_mu_size = 256;
  r.transmittance_r_size = 64;
  r.scattering_r_size = 32;
  r.scattering_mu_size = 128;
  r.scattering_mu_s_size = 32;
  r.scattering_nu_size = 8;
  r.irradiance_mu_s_size = 64;
  r.irradiance_r_size = 16;
  r.rayleigh_density.layers[1].exp_term = 1.0f;
  r.rayleigh_density.layers[1].exp_scale = -0.125f;
  r.mie_density.layers[1].exp_term = 1.0f;
  r.mie_density.layers[1].exp_scale = -0.833333f;
  r.absorption_density.layers[0].width = 25.0f;
  r.absorption_density.layers[0].linear_term = 0.066667f;
  r.absorption_density.layers[0].constant_term = -0.666667f;
  r.absorption_density.layers[1].linear_term = -0.066667f;
  r.absorption_density.layers[1].constant_term = 2.666667f;
  o->order = 4;
  o->transmittance_steps = 500;
  o->single_scattering_steps = 50;
  o->multiple_scattering_steps = 50;
  o->density_samples = 16;
  o->irradiance_samples = 32;
  o->precision = FB_PRECISION_PLAIN;
  o->storage = FB_STORAGE_F32;
}

// Shader arithmetic per texel of pass `pass` (0 transmittance, 1 direct
// irradiance, 2 single scattering, 3 scattering density of `order`, 4 indirect
// irradiance of `order`, 5 multiple scattering): out[5] = adds, muls, divs,
// sqrts, transcendentals, averaged over n sampled texels.
int fbo_count_ops(const fb_params* p, int pass, int order, int64_t n, uint64_t seed, double* out) {
  return count_ops(p, pass, order, n, seed, out);
}

int fbo_render_sky_f32(const fb_params* p, const float* tr, const float* sc, const fb_draw_parameters* d,
                       const float* depth, uint32_t width, uint32_t height, float* color, float* trans) {
  return render_sky<float>(p, tr, sc, d, depth, width, height, color, trans);
}
int fbo_render_sky_f64(const fb_params* p, const double* tr, const double* sc, const fb_draw_parameters* d,
                       const double* depth, uint32_t width, uint32_t height, double* color, double* trans) {
  return render_sky<double>(p, tr, sc, d, depth, width, height, color, trans);
}
int fbo_sun_and_sky_irradiance_f32(const fb_params* p, const float* tr, const float* ir, const float* points,
                                   const float* normals, const float* sun, int64_t n, float* sun_out,
                                   float* sky_out) {
  return lighting<float>(p, tr, ir, points, normals, sun, n, sun_out, sky_out);
}
int fbo_sun_and_sky_irradiance_f64(const fb_params* p, const double* tr, const double* ir, const double* points,
                                   const double* normals, const double* sun, int64_t n, double* sun_out,
                                   double* sky_out) {
  return lighting<double>(p, tr, ir, points, normals, sun, n, sun_out, sky_out);
}

}  // extern "C"
