// fb_device.cuh — device-side data of one atmosphere and the shared math of
// the six precompute passes (sm_103a).
//
// Two arithmetic modes are compiled from the same templates:
//   PLAIN (MX = false): FP32, operation for operation the arithmetic of the
//     reference's shaders (shaders/*.h, *.comp). The translation unit that
//     instantiates it is compiled with --fmad=false, so products and sums round
//     separately as in the shaders; fmaf() is used only in interpolation and
//     accumulation, where it changes nothing but the last bit.
//   MIXED (MX = true): a point on a ray is carried as (q, s) = (r^2 - R^2, r*mu)
//     in FP64, which removes the cancellations at the horizon (ground altitude,
//     ray/sphere discriminants, the horizon seam of the mu coordinate); quadrature
//     sums are Kahan-compensated; orders accumulate in FP64.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace fb {

struct Layer {
  float width, exp_term, exp_scale, linear_term, constant_term;
};

// One axis of the LINEAR + CLAMP_TO_EDGE sampler of src/precompute.rs:85-98:
// the two neighbouring texels and the weight of the second.
struct Axis {
  int i0, i1;
  float f;
};

// ---------------------------------------------------- geometry tables
// Order-independent geometry of one atmosphere, computed once per build (the
// FP64 decodes of the mixed mode cost 64 FP32 issue slots each on this part,
// so no pass repeats them per tile or per order).

// One (mu, r) row of the packed scattering table (texel y, z): the view ray.
struct RowGeo {
  float r, mu, dist, rr, two_r_mu, r_mu;  // PLAIN: the reference's float values; dist to the ground or the top
  double q, s, distd, one_m_mu2, mud;     // MIXED: q = r^2 - R^2, s = r mu, FP64 distance, 1 - mu^2, mu
  int ground, pad;
};

// Plane stride of the density table, so that every plane row starts 16-byte aligned.
__host__ __device__ inline int dens_stride(int W) { return (W + 3) & ~3; }

// One x column of the packed table (nu slice x / mu_s_size, mu_s index x % mu_s_size).
struct ColGeo {
  float mu_s, one_m_mus2, nu_raw, u_mus;  // PLAIN: reference float values; u_mus = u_mu_s texture coordinate
  double mu_sd, one_m_mus2d, nu_rawd, t_musd;  // MIXED: FP64 values; t_musd = texel coordinate within a slice
};

// One trapezoid sample of multiple scattering along the view ray of a row:
// distance, 1/r_i, transmittance x dx x trapezoid weight; the bilinear
// weights and 16-byte offsets ((z sc_mu + y) 3 Wd / 4) of the four density rows
// around the sample's (mu, r), corners (y0, z0), (y1, z0), (y0, z1), (y1, z1).
struct __align__(16) MSRec {
  float d, inv_r, tvwx, tvwy;
  float tvwz, pad0, pad1, pad2;
  float w[4];
  int off[4];
};

// Scattering density: per r slice, and per (r slice, theta row) of the sphere grid.
struct DensZ {
  float r;
  int pad;
  double q;
  Axis az;   // r axis of the 3D tables
  Axis irx;  // r axis of the irradiance table at the ground
};
struct DensTheta {
  float cos_t, domega, dg, tgx, tgy, tgz;  // tg = transmittance to the ground x albedo / pi
  int ground, pad;
};
struct ThetaRec {
  DensTheta th;
  Axis tay;  // mu axis of the lookup direction
  int pad;
};

// Indirect irradiance, MIXED (indirect_irradiance.comp:16-40 lookups): per
// irradiance r row the radius and the r axis of the 3D tables; the mu axes per
// (r row, theta row) and the x axes per (mu_s column, nu slice -1 .. nu_size)
// are separate arrays.
struct IrZ {
  float r;
  Axis az;
};

// One atmosphere as the kernels see it: parameters (ParamsRaw fields,
// src/precompute.rs:937-964), sizes, sample counts and its tables.
struct DevAtmo {
  float solar[3], rayleigh[3], mie_sca[3], mie_ext[3], albedo[3], absorption[3];
  float sun_radius, bottom, top, g, mu_s_min;
  Layer ray_d[2], mie_d[2], abs_d[2];
  int tr_mu, tr_r, sc_r, sc_mu, sc_mus, sc_nu, ir_mus, ir_r;
  int tr_steps, ss_steps, ms_steps, dens_n, irr_n, order;
  int f16;         // round the scattering-class tables to half on store
  int W;           // sc_nu * sc_mus, width of the packed 3D scattering tables
  int Wd;          // plane stride of the density table: W rounded up to a multiple of 4
  int dens_S, dens_chunk;  // scattering-density tile shape (0 = default; set by the autotuner)
  // Per-atmosphere constants of the MIXED geometry, computed on the host in
  // FP64 (correctly rounded, the values the device would compute) so that no
  // thread repeats an FP64 square root or division per tile.
  double H2d;                  // T^2 - R^2
  double Hd;                   // sqrt(T^2 - R^2)
  float Hf, inv_Hf;            // FP32 sqrt(T^2 - R^2) and its reciprocal
  float mus_inv_span, mus_inv_A;  // mu_s mapping (scattering.h:48-56): 1 / (H - (T - R)), (H - (T - R)) / A'
  // outputs
  float4* tr;
  float4* ir;
  float4* sc;
  // temporaries
  float* trp;       // transmittance pairs: per texel (mu i, r j) 32 bytes, the RGB of
                    // texels i and min(i + 1, tr_mu - 1) of row j and two zeros
  float4* dirr[2];  // delta irradiance, ping-pong by order parity
  float4* dr;       // delta Rayleigh (single)
  float4* dm;       // delta Mie (single)
  float4* dms;      // delta multiple scattering of the last order
  float* dens;      // scattering density of the current order: per (r, mu) row three
                    // planes (R, G, B) of Wd floats, the first W of each in use
  double* sc_acc;   // MIXED: FP64 running sum of scattering rgb (3 per texel)
  double* ir_acc;   // MIXED: FP64 running sum of irradiance rgb (3 per texel)
  // geometry tables (written by the transmittance and single-scattering launches)
  RowGeo* g_rows;   // sc_mu * sc_r
  ColGeo* g_cols;   // W
  MSRec* g_ms;      // sc_mu * sc_r * (ms_steps + 1)
  DensZ* g_z;       // sc_r
  ThetaRec* g_th;   // sc_r * dens_n
  IrZ* g_irz;       // MIXED: ir_r
  Axis* g_iry;      // MIXED: ir_r * irr_n / 2
  Axis* g_irx;      // MIXED: ir_mus * (sc_nu + 2)
  float* g_irmus;   // MIXED: ir_mus
};

constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPiD = 3.14159265358979323846;

// --------------------------------------------------------------- GLSL basics
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ double gmin(double x, double y) { return y < x ? y : x; }
__device__ __forceinline__ double gmax(double x, double y) { return x < y ? y : x; }
__device__ __forceinline__ double gclamp(double x, double lo, double hi) { return gmin(gmax(x, lo), hi); }

template <class T> __device__ __forceinline__ T clamp_cosine(T mu) { return gclamp(mu, T(-1), T(1)); }
__device__ __forceinline__ float safe_sqrt(float a) { return sqrtf(gmax(a, 0.0f)); }
// 1 / sqrt(x) for arguments that are positive and normal: the hardware
// reciprocal square root alone (PTX rsqrt.approx.ftz.f32). rsqrtf adds a test
// and a rescaling for subnormal arguments; for normal ones the result is the
// same. Callers pass only arguments bounded away from zero.
__device__ __forceinline__ float rsqrt_pos(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double safe_sqrt(double a) { return sqrt(gmax(a, 0.0)); }

// util.h:18-24
template <class T> __device__ __forceinline__ T coord_from_unit(T x, int n) {
  return T(0.5) / T(n) + x * (T(1) - T(1) / T(n));
}
template <class T> __device__ __forceinline__ T unit_from_coord(T u, int n) {
  return (u - T(0.5) / T(n)) / (T(1) - T(1) / T(n));
}
// util.h:26-34
__device__ __forceinline__ float phase_rayleigh(float nu) {
  const float k = 3.0f / (16.0f * kPiF);
  return k * (1.0f + nu * nu);
}
__device__ __forceinline__ float phase_mie(float g, float nu) {
  const float k = 3.0f / (8.0f * kPiF) * (1.0f - g * g) / (2.0f + g * g);
  return k * (1.0f + nu * nu) / powf(1.0f + g * g - 2.0f * g * nu, 1.5f);
}
// util.h:36-38
__device__ __forceinline__ float frag_from_texel(uint32_t i, uint32_t n) {
  return float(n) * coord_from_unit(float(i) / float(n - 1), int(n));
}
__device__ __forceinline__ double frag_from_texel_d(uint32_t i, uint32_t n) {
  return double(n) * coord_from_unit(double(i) / double(n - 1), int(n));
}
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
  float t = gclamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

// params.h:89-99 — density profiles.
__device__ __forceinline__ float layer_density(const Layer& L, float h) {
  float d = L.exp_term * expf(L.exp_scale * h) + L.linear_term * h + L.constant_term;
  return gclamp(d, 0.0f, 1.0f);
}
__device__ __forceinline__ float profile_density(const Layer* P, float h) {
  return h < P[0].width ? layer_density(P[0], h) : layer_density(P[1], h);
}

// ------------------------------------------------------------ table access
// make_axis: texel coordinate u*n - 0.5, neighbours clamped to [0, n-1].
__device__ __forceinline__ Axis make_axis(float coord, int n) {
  float x = coord * float(n) - 0.5f;
  float fl = floorf(x);
  Axis a;
  a.f = x - fl;
  fl = fminf(fmaxf(fl, -1.0f), float(n));  // fmaxf(NaN, -1) = -1
  int i = (int)fl;
  a.i0 = min(max(i, 0), n - 1);
  a.i1 = min(max(i + 1, 0), n - 1);
  return a;
}

// An axis read back from a geometry record, its indices bounded to [0, n - 1]
// so that a damaged record cannot address outside its table.
__device__ __forceinline__ Axis bounded_axis(Axis a, int n) {
  a.i0 = min(max(a.i0, 0), n - 1);
  a.i1 = min(max(a.i1, 0), n - 1);
  return a;
}

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// Bilinear RGB fetch with the Vulkan weight order (1-a)(1-b), a(1-b), (1-a)b, ab.
__device__ __forceinline__ float3 fetch2(const float4* t, int w, Axis x, Axis y) {
  const float4 p00 = ld4(t + y.i0 * w + x.i0), p10 = ld4(t + y.i0 * w + x.i1);
  const float4 p01 = ld4(t + y.i1 * w + x.i0), p11 = ld4(t + y.i1 * w + x.i1);
  const float w00 = (1.0f - x.f) * (1.0f - y.f), w10 = x.f * (1.0f - y.f);
  const float w01 = (1.0f - x.f) * y.f, w11 = x.f * y.f;
  float3 o;
  o.x = fmaf(w11, p11.x, fmaf(w01, p01.x, fmaf(w10, p10.x, w00 * p00.x)));
  o.y = fmaf(w11, p11.y, fmaf(w01, p01.y, fmaf(w10, p10.y, w00 * p00.y)));
  o.z = fmaf(w11, p11.z, fmaf(w01, p01.z, fmaf(w10, p10.z, w00 * p00.z)));
  return o;
}

// The same bilinear fetch from the transmittance pair table: one 32-byte load
// per row brings both x neighbours. Needs x.i1 = min(x.i0 + 1, w - 1), which
// axis_texel gives for coordinates t >= 0.
__device__ __forceinline__ void ld_pair(const float* p, float4& lo, float4& hi) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z), "=f"(hi.w)
      : "l"(p));
}
__device__ __forceinline__ float3 fetch2_pairs(const float* trp, int w, Axis x, Axis y) {
  float4 a0, a1, b0, b1;  // row y0: (p00.xyz, p10.x) (p10.yz, 0, 0); row y1 likewise
  ld_pair(trp + 8 * (size_t)(y.i0 * w + x.i0), a0, a1);
  ld_pair(trp + 8 * (size_t)(y.i1 * w + x.i0), b0, b1);
  const float w00 = (1.0f - x.f) * (1.0f - y.f), w10 = x.f * (1.0f - y.f);
  const float w01 = (1.0f - x.f) * y.f, w11 = x.f * y.f;
  float3 o;
  o.x = fmaf(w11, b0.w, fmaf(w01, b0.x, fmaf(w10, a0.w, w00 * a0.x)));
  o.y = fmaf(w11, b1.x, fmaf(w01, b0.y, fmaf(w10, a1.x, w00 * a0.y)));
  o.z = fmaf(w11, b1.y, fmaf(w01, b0.z, fmaf(w10, a1.y, w00 * a0.z)));
  return o;
}

// Trilinear RGB fetch from a packed 3D table (width w, height h), same weights.
__device__ __forceinline__ float3 fetch3(const float4* t, int w, int h, Axis x, Axis y, Axis z) {
  const float ia = 1.0f - x.f, ib = 1.0f - y.f, ic = 1.0f - z.f;
  const float wt[8] = {ia * ib * ic, x.f * ib * ic, ia * y.f * ic, x.f * y.f * ic,
                       ia * ib * z.f, x.f * ib * z.f, ia * y.f * z.f, x.f * y.f * z.f};
  const int xs[2] = {x.i0, x.i1}, ys[2] = {y.i0, y.i1}, zs[2] = {z.i0, z.i1};
  float3 o = make_float3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float4 p = ld4(t + ((size_t)zs[k >> 2] * h + ys[(k >> 1) & 1]) * w + xs[k & 1]);
    o.x = fmaf(wt[k], p.x, o.x);
    o.y = fmaf(wt[k], p.y, o.y);
    o.z = fmaf(wt[k], p.z, o.z);
  }
  return o;
}

__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 ld3(const float* v) { return make_float3(v[0], v[1], v[2]); }
__device__ __forceinline__ float3 min1(float3 q) { return make_float3(gmin(q.x, 1.f), gmin(q.y, 1.f), gmin(q.z, 1.f)); }

// Kahan-compensated accumulator of an RGB sum.
struct Kahan3 {
  float3 s, c;
  __device__ __forceinline__ void init() {
    s = make_float3(0.f, 0.f, 0.f);
    c = s;
  }
  __device__ __forceinline__ static void add1(float& sum, float& comp, float v) {
    float y = v - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
  }
  __device__ __forceinline__ void add(float3 v) {
    add1(s.x, c.x, v.x);
    add1(s.y, c.y, v.y);
    add1(s.z, c.z, v.z);
  }
  // add(u * v) with the product formed inside the first FMA (unrounded)
  __device__ __forceinline__ static void add1_prod(float& sum, float& comp, float u, float v) {
    float y = fmaf(u, v, -comp);
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
  }
  __device__ __forceinline__ void add_prod(float3 u, float3 v) {
    add1_prod(s.x, c.x, u.x, v.x);
    add1_prod(s.y, c.y, u.y, v.y);
    add1_prod(s.z, c.z, u.z, v.z);
  }
};
__device__ __forceinline__ float3 fma3(float3 a, float3 b, float3 c) {
  return make_float3(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z));
}

__device__ __forceinline__ float store_round(float v, int f16) {
  return f16 ? __half2float(__float2half_rn(v)) : v;
}
__device__ __forceinline__ float4 store_round4(float4 v, int f16) {
  if (!f16) return v;
  return make_float4(store_round(v.x, 1), store_round(v.y, 1), store_round(v.z, 1), store_round(v.w, 1));
}

// ------------------------------------------------------ PLAIN (FP32) geometry
// The reference's formulas, term by term.
struct Geo32 {
  float R, T, H;  // bottom, top, sqrt(T^2 - R^2)
  __device__ __forceinline__ void init(const DevAtmo& a) {
    R = a.bottom;
    T = a.top;
    H = sqrtf(T * T - R * R);
  }
  // params.h:105-124
  __device__ __forceinline__ float dist_top(float r, float mu) const {
    float disc = r * r * (mu * mu - 1.0f) + T * T;
    return gmax(-r * mu + safe_sqrt(disc), 0.0f);
  }
  __device__ __forceinline__ float dist_bottom(float r, float mu) const {
    float disc = r * r * (mu * mu - 1.0f) + R * R;
    return gmax(-r * mu - safe_sqrt(disc), 0.0f);
  }
  __device__ __forceinline__ bool hits_ground(float r, float mu) const {
    return mu < 0.0f && r * r * (mu * mu - 1.0f) + R * R >= 0.0f;
  }
  __device__ __forceinline__ float clamp_radius(float r) const { return gclamp(r, R, T); }
  // transmittance.h:7-24
  __device__ __forceinline__ void tr_coords(const DevAtmo& a, float r, float mu, float& u, float& v) const {
    float rho = safe_sqrt(r * r - R * R);
    float d = dist_top(r, mu);
    float d_min = T - r;
    float d_max = rho + H;
    float x_mu = (d - d_min) / (d_max - d_min);
    float x_r = rho / H;
    u = coord_from_unit(x_mu, a.tr_mu);
    v = coord_from_unit(x_r, a.tr_r);
  }
  // transmittance.h:26-33
  __device__ __forceinline__ float3 tr_to_top(const DevAtmo& a, float r, float mu) const {
    float u, v;
    tr_coords(a, r, mu, u, v);
    return fetch2(a.tr, a.tr_mu, make_axis(u, a.tr_mu), make_axis(v, a.tr_r));
  }
  // transmittance.h:35-61
  __device__ __forceinline__ float3 tr_segment(const DevAtmo& a, float r, float mu, float d, bool ground) const {
    float r_d = clamp_radius(sqrtf(d * d + 2.0f * r * mu * d + r * r));
    float mu_d = clamp_cosine((r * mu + d) / r_d);
    float3 q = ground ? tr_to_top(a, r_d, -mu_d) / tr_to_top(a, r, -mu)
                      : tr_to_top(a, r, mu) / tr_to_top(a, r_d, mu_d);
    return min1(q);
  }
  // scattering.h:15-46 — the r and mu texture coordinates (w and z).
  __device__ __forceinline__ float u_r(const DevAtmo& a, float r) const {
    float rho = safe_sqrt(r * r - R * R);
    return coord_from_unit(rho / H, a.sc_r);
  }
  __device__ __forceinline__ float u_mu(const DevAtmo& a, float r, float mu, bool ground) const {
    float rho = safe_sqrt(r * r - R * R);
    float r_mu = r * mu;
    float disc = r_mu * r_mu - r * r + R * R;
    if (ground) {
      float d = -r_mu - safe_sqrt(disc);
      float d_min = r - R;
      float d_max = rho;
      return 0.5f - 0.5f * coord_from_unit(d_max == d_min ? 0.0f : (d - d_min) / (d_max - d_min), a.sc_mu / 2);
    }
    float d = -r_mu + safe_sqrt(disc + H * H);
    float d_min = T - r;
    float d_max = rho + H;
    return 0.5f + 0.5f * coord_from_unit((d - d_min) / (d_max - d_min), a.sc_mu / 2);
  }
  // scattering.h:48-56 — the mu_s texture coordinate.
  __device__ __forceinline__ float u_mu_s(const DevAtmo& a, float mu_s) const {
    float d = dist_top(R, mu_s);
    float d_min = T - R;
    float d_max = H;
    float aa = (d - d_min) / (d_max - d_min);
    float A = -2.0f * a.mu_s_min * R / (d_max - d_min);
    return coord_from_unit(gmax(1.0f - aa / A, 0.0f) / (1.0f + aa), a.sc_mus);
  }
};

// ------------------------------------------------------ MIXED (FP64) geometry
// A point on a ray is (q, s) = (r^2 - R^2, r*mu). Moving a distance d along the
// ray gives q' = q + d (2 s + d) and s' = s + d exactly, so the altitude
// h = q / (r + R), the horizon distance rho = sqrt(q) and the ground
// discriminant s^2 - q never lose digits to cancellation.
//
// Sampler axes are built from texel coordinates. The reference maps a unit
// value y to u = 0.5/N + y (1 - 1/N) (util.h:18-20) and the sampler takes
// u N - 0.5, which is y (N - 1) exactly; evaluating y (N - 1) directly keeps
// texel-centred lookups exactly on the texel (no spurious weight on a
// neighbour that may be orders of magnitude larger).
template <class T> __device__ __forceinline__ Axis axis_texel(T t, int n) {
  T fl = floor(t);
  Axis a;
  a.f = (float)(t - fl);
  fl = fl < T(-1) ? T(-1) : (fl > T(n) ? T(n) : fl);
  if (!(fl == fl)) fl = T(-1);
  int i = (int)fl;
  a.i0 = min(max(i, 0), n - 1);
  a.i1 = min(max(i + 1, 0), n - 1);
  return a;
}

struct Geo64 {
  double R, T, H, H2;
  __device__ __forceinline__ void init(const DevAtmo& a) {
    R = a.bottom;
    T = a.top;
    H2 = a.H2d;  // T * T - R * R
    H = a.Hd;    // sqrt(H2)
  }
  __device__ __forceinline__ double radius(double q) const { return sqrt(q + R * R); }
  // params.h:105-110 with the discriminant T^2 - r^2 (1 - mu^2) = (H^2 - q) + s^2.
  __device__ __forceinline__ double dist_top(double q, double s) const {
    double e = H2 - q;  // T^2 - r^2
    double root = sqrt(gmax(e + s * s, 0.0));
    double d = s > 0.0 ? e / (s + root) : root - s;
    return gmax(d, 0.0);
  }
  // params.h:112-117 with the discriminant s^2 - q.
  __device__ __forceinline__ double dist_bottom(double q, double s) const {
    double root = sqrt(gmax(s * s - q, 0.0));
    double d = s < 0.0 ? q / (root - s) : -s - root;
    return gmax(d, 0.0);
  }
  __device__ __forceinline__ bool hits_ground(double q, double s) const { return s < 0.0 && s * s - q >= 0.0; }
  // ClampRadius on (q, s): r in [R, T] <=> q in [0, H^2]; mu in [-1, 1] <=> |s| <= r.
  __device__ __forceinline__ void clamp_point(double& q, double& s) const {
    q = gclamp(q, 0.0, H2);
    double r = radius(q);
    s = gclamp(s, -r, r);
  }
  // transmittance.h:7-24 as texel coordinates of the transmittance table.
  __device__ __forceinline__ void tr_texel(const DevAtmo& a, double q, double s, double& tx, double& ty) const {
    double rho = sqrt(gmax(q, 0.0));
    double r = radius(q);
    double d = dist_top(q, s);
    double d_min = (H2 - q) / (T + r);
    double d_max = rho + H;
    tx = (d - d_min) / (d_max - d_min) * double(a.tr_mu - 1);
    ty = rho / H * double(a.tr_r - 1);
  }
  __device__ __forceinline__ float3 tr_to_top(const DevAtmo& a, double q, double s) const {
    double tx, ty;
    tr_texel(a, q, s, tx, ty);
    return fetch2(a.tr, a.tr_mu, axis_texel(tx, a.tr_mu), axis_texel(ty, a.tr_r));
  }
  // transmittance.h:35-61: transmittance from (q, s) over distance d.
  __device__ __forceinline__ float3 tr_segment(const DevAtmo& a, double q, double s, double d, bool ground) const {
    double qd = q + d * (2.0 * s + d), sd = s + d;
    clamp_point(qd, sd);
    float3 num, den;
    if (ground) {
      num = tr_to_top(a, qd, -sd);
      den = tr_to_top(a, q, -s);
    } else {
      num = tr_to_top(a, q, s);
      den = tr_to_top(a, qd, sd);
    }
    return min1(num / den);
  }
  // scattering.h:15-21: texel coordinate along r (depth of the 3D table).
  __device__ __forceinline__ double sc_r_texel(const DevAtmo& a, double q) const {
    return sqrt(gmax(q, 0.0)) / H * double(a.sc_r - 1);
  }
  // scattering.h:23-46: texel coordinate along mu (height of the 3D table).
  // With M = mu_size / 2 the reference's u_mu maps to (M - 1)(1 - x) on the
  // ground half and M + x (M - 1) on the sky half.
  __device__ __forceinline__ double sc_mu_texel(const DevAtmo& a, double q, double s, bool ground) const {
    const int M = a.sc_mu / 2;
    double rho = sqrt(gmax(q, 0.0));
    double r = radius(q);
    if (ground) {
      double d = dist_bottom(q, s);
      double d_min = q / (r + R);
      double d_max = rho;
      double x = d_max == d_min ? 0.0 : (d - d_min) / (d_max - d_min);
      return double(M - 1) * (1.0 - x);
    }
    double d = dist_top(q, s);
    double d_min = (H2 - q) / (T + r);
    double d_max = rho + H;
    double x = (d - d_min) / (d_max - d_min);
    return double(M) + x * double(M - 1);
  }
  // scattering.h:48-56: the unit-range mu_s value y (texel coordinate within a
  // nu slice is y (mu_s_size - 1)). The distance from the ground to the top
  // along mu_s is H^2 / (s + sqrt(s^2 + H^2)) with s = R mu_s.
  __device__ __forceinline__ double mus_unit(const DevAtmo& a, double mu_s) const {
    double s = R * mu_s;
    double root = sqrt(s * s + H2);
    double d = s > 0.0 ? H2 / (s + root) : root - s;
    double d_min = T - R;
    double d_max = H;
    double aa = (d - d_min) / (d_max - d_min);
    double A = -2.0 * a.mu_s_min * R / (d_max - d_min);
    return gmax(1.0 - aa / A, 0.0) / (1.0 + aa);
  }
};

// The MIXED geometry used per trapezoid sample: FP64 only where cancellation
// happens (the sample state q, s; the ground discriminant s^2 - q; T^2 - r^2),
// every later step in FP32 on quantities that no longer cancel. Same results
// as Geo64 to FP32 precision, at a fraction of its FP64 instructions (FP64
// issues at 1/64 of the FP32 rate on this part).
// An axis of a table measured from its last texel: g >= 0 texels before
// texel n - 1, i.e. at texel coordinate n - 1 - g. The interpolation runs from
// the edge texel (i0) towards the inner one (i1) with weight f = frac(g), so
// that near the edge the position keeps the relative precision of g; an FP32
// coordinate near n - 1 itself has a resolution of ulp(n - 1) (1.5e-5 texels
// at n = 256). NaN maps to the edge texel.
__device__ __forceinline__ Axis edge_axis(float g, int n) {
  float k = floorf(g);
  Axis a;
  a.f = g - k;
  k = fminf(fmaxf(k, 0.0f), float(n));  // fmaxf(NaN, 0) = 0
  const int i = (int)k;
  a.i0 = max(n - 1 - i, 0);
  a.i1 = max(n - 2 - i, 0);
  return a;
}

// Geometry of the mixed mode's per-sample records: FP64 ray state (q = r^2 -
// R^2, s = r mu), the rest in FP32.
struct GeoMx {
  float R, T, H, H2f, inv_H, trm1, trr1, scr1, M1f, Mf;
  double H2;
  __device__ __forceinline__ void init(const DevAtmo& a) {
    R = a.bottom;
    T = a.top;
    H2 = a.H2d;
    H2f = (float)H2;
    H = a.Hf;
    inv_H = a.inv_Hf;
    trm1 = float(a.tr_mu - 1);
    trr1 = float(a.tr_r - 1);
    scr1 = float(a.sc_r - 1);
    Mf = float(a.sc_mu / 2);
    M1f = float(a.sc_mu / 2 - 1);
  }
  // distance to the top from (q, s): e = T^2 - r^2 in FP64, the rest in FP32
  __device__ __forceinline__ float dist_top(double q, double s, float& e_out) const {
    const double e = H2 - q;
    const float root = sqrtf((float)fmax(fma(s, s, e), 0.0));
    const float ef = (float)e, sf = (float)s;
    e_out = ef;
    return fmaxf(sf > 0.0f ? __fdividef(ef, sf + root) : root - sf, 0.0f);
  }
  // transmittance.h:7-24 as axes of the transmittance table, the mu axis
  // measured from its horizon edge. Along rays near the horizon the table
  // changes by large factors per texel (e^7 between the last two texels for
  // some atmospheres), so the texel position there must keep more than FP32's
  // absolute resolution near texel N - 1. With delta = s^2 - q (FP64), the gap
  // d_max - d between the horizon distance rho + H and the distance to the top
  // d = -s + sqrt(H^2 + delta) is (rho + s) + (H - sqrt(H^2 + delta)), each
  // part formed without cancellation: rho + s = -delta / (rho - s) for s < 0,
  // H - sqrt(H^2 + delta) = -delta / (H + sqrt(H^2 + delta)). The texel
  // position is N - 1 - g with g = (N - 1) gap / (d_max - d_min).
  __device__ __forceinline__ void tr_axes(double q, double s, int tr_mu, int tr_r, Axis& ax, Axis& ay) const {
    const float qf = fmaxf((float)q, 0.0f);
    const float rho = sqrtf(qf), r = sqrtf(qf + R * R);
    const float delta = (float)fma(s, s, -q), sf = (float)s;
    const float root = sqrtf(fmaxf(H2f + delta, 0.0f));
    const float rho_s = sf < 0.0f ? -delta / (rho - sf) : rho + sf;
    const float gap = fmaxf(rho_s - delta / (H + root), 0.0f);
    const float d_min = (float)(H2 - q) / (T + r);
    ax = edge_axis(gap / (rho + H - d_min) * trm1, tr_mu);
    ay = axis_texel(rho * inv_H * trr1, tr_r);
  }
  __device__ __forceinline__ float3 tr_to_top(const DevAtmo& a, double q, double s) const {
    Axis ax, ay;
    tr_axes(q, s, a.tr_mu, a.tr_r, ax, ay);
    return fetch2(a.tr, a.tr_mu, ax, ay);
  }
  __device__ __forceinline__ float3 tr_segment(const DevAtmo& a, double q, double s, double d, bool ground) const {
    double qd = fma(d, 2.0 * s + d, q), sd = s + d;
    qd = fmin(fmax(qd, 0.0), H2);
    const double rd = (double)sqrtf((float)qd + R * R);
    sd = fmin(fmax(sd, -rd), rd);
    float3 num, den;
    if (ground) {
      num = tr_to_top(a, qd, -sd);
      den = tr_to_top(a, q, -s);
    } else {
      num = tr_to_top(a, q, s);
      den = tr_to_top(a, qd, sd);
    }
    return min1(num / den);
  }
  __device__ __forceinline__ float sc_r_texel(double q) const {
    return sqrtf(fmaxf((float)q, 0.0f)) * inv_H * scr1;
  }
  // scattering.h:23-46 as a texel coordinate along mu
  __device__ __forceinline__ float sc_mu_texel(double q, double s, bool ground) const {
    const float qf = fmaxf((float)q, 0.0f);
    const float rho = sqrtf(qf), r = sqrtf(qf + R * R), sf = (float)s;
    if (ground) {
      const float root = sqrtf((float)fmax(fma(s, s, -q), 0.0));  // s^2 - q in FP64
      const float d = sf < 0.0f ? __fdividef(qf, root - sf) : fmaxf(-sf - root, 0.0f);
      const float d_min = __fdividef(qf, r + R);
      const float x = rho == d_min ? 0.0f : __fdividef(d - d_min, rho - d_min);
      return M1f * (1.0f - x);
    }
    float e;
    const float d = dist_top(q, s, e);
    const float d_min = __fdividef(e, T + r);
    const float x = __fdividef(d - d_min, rho + H - d_min);
    return fmaf(x, M1f, Mf);
  }
};

// FP32 form of Geo64::mus_unit for per-texel-sample use in the mixed mode: the
// same cancellation-free distance, single precision, constants precomputed.
struct MuS32 {
  float R, H2, dmin, inv_span, inv_A, scale;
  __device__ __forceinline__ void init(const DevAtmo& a) {
    R = a.bottom;
    H2 = (float)a.H2d;
    dmin = (float)((double)a.top - (double)a.bottom);
    inv_span = a.mus_inv_span;
    inv_A = a.mus_inv_A;
    scale = float(a.sc_mus - 1);
  }
  // texel coordinate within a nu slice. The distance to the top is d = P / Q
  // (rationalised where the ray points up); with a = (d - dmin) / span the
  // coordinate max(1 - a / A, 0) / (1 + a) is formed as one quotient,
  // max(Q - a Q / A, 0) / (Q + a Q).
  __device__ __forceinline__ float texel(float mu_s) const {
    float s = R * mu_s;
    const float disc = fmaf(s, s, H2);  // >= H^2 > 0
    float root = disc * rsqrt_pos(disc);  // disc >= H^2
    const bool up = s > 0.0f;
    const float P = up ? H2 : root - s, Q = up ? s + root : 1.0f;
    const float aQ = fmaf(-dmin, Q, P) * inv_span;
    return __fdividef(gmax(fmaf(-aQ, inv_A, Q), 0.0f), Q + aQ) * scale;
  }
};

// PLAIN form of the mu_s texture coordinate (scattering.h:48-56), the
// reference's float arithmetic with its per-atmosphere constants hoisted: the
// divisions by constants become products with reciprocals (last-bit
// differences only).
struct MuSRef32 {
  float R, RR, TT, dmin, inv_span, inv_A, c0, c1;
  __device__ __forceinline__ void init(const DevAtmo& a) {
    R = a.bottom;
    RR = R * R;
    const float T = a.top;
    TT = T * T;
    const float H = sqrtf(T * T - R * R);
    dmin = T - R;
    const float span = H - dmin;
    inv_span = 1.0f / span;
    const float A = -2.0f * a.mu_s_min * R / span;
    inv_A = 1.0f / A;
    c0 = 0.5f / float(a.sc_mus);
    c1 = 1.0f - 1.0f / float(a.sc_mus);
  }
  // the texture coordinate u_mu_s
  __device__ __forceinline__ float coord(float mu_s) const {
    float disc = RR * (mu_s * mu_s - 1.0f) + TT;
    float d = gmax(-R * mu_s + safe_sqrt(disc), 0.0f);
    float aa = (d - dmin) * inv_span;
    return c0 + gmax(1.0f - aa * inv_A, 0.0f) / (1.0f + aa) * c1;
  }
};

// --------------------------------------------------------- texel decoding
// scattering.h:62-137 + util.h:36-45: texel (x, y, z) of the packed 3D table
// to (r, mu, mu_s, nu, ground), nu clamped to its valid range.
struct TexelParams {
  double r, mu, mu_s, nu, q, s;  // q = r^2 - R^2, s = r mu
  bool ground;
};

// PLAIN: the reference's float arithmetic, split into the part that depends on
// the row (y, z) and the part that depends on the column x.
__device__ __forceinline__ void decode_yz32(const DevAtmo& a, const Geo32& G, uint32_t iy, uint32_t iz, float& r,
                                            float& mu, bool& ground) {
  float fy = frag_from_texel(iy, (uint32_t)a.sc_mu), fz = frag_from_texel(iz, (uint32_t)a.sc_r);
  float qz = fy / float(a.sc_mu), qw = fz / float(a.sc_r);
  float rho = G.H * unit_from_coord(qw, a.sc_r);
  r = sqrtf(rho * rho + G.R * G.R);
  if (qz < 0.5f) {
    float d_min = r - G.R;
    float d_max = rho;
    float d = d_min + (d_max - d_min) * unit_from_coord(1.0f - 2.0f * qz, a.sc_mu / 2);
    mu = d == 0.0f ? -1.0f : clamp_cosine(-(rho * rho + d * d) / (2.0f * r * d));
    ground = true;
  } else {
    float d_min = G.T - r;
    float d_max = rho + G.H;
    float d = d_min + (d_max - d_min) * unit_from_coord(2.0f * qz - 1.0f, a.sc_mu / 2);
    mu = d == 0.0f ? 1.0f : clamp_cosine((G.H * G.H - rho * rho - d * d) / (2.0f * r * d));
    ground = false;
  }
}
// mu_s and the nu of column x before the clamp of scattering.h:134-136.
__device__ __forceinline__ void decode_x32(const DevAtmo& a, const Geo32& G, uint32_t ix, float& mu_s,
                                           float& nu_raw) {
  float fx = frag_from_texel(ix, (uint32_t)a.W);
  float nmus = float(a.sc_mus);
  float f_nu = floorf(fx / nmus);
  float f_mus = fx - nmus * floorf(fx / nmus);
  float qx = f_nu / float(a.sc_nu - 1), qy = f_mus / nmus;
  float x_mu_s = unit_from_coord(qy, a.sc_mus);
  float d_min = G.T - G.R;
  float d_max = G.H;
  float A = -2.0f * a.mu_s_min * G.R / (d_max - d_min);
  float aa = (A - x_mu_s * A) / (1.0f + x_mu_s * A);
  float d = d_min + gmin(aa, A) * (d_max - d_min);
  mu_s = d == 0.0f ? 1.0f : clamp_cosine((G.H * G.H - d * d) / (2.0f * G.R * d));
  nu_raw = clamp_cosine(qx * 2.0f - 1.0f);
}
// scattering.h:134-136: nu limited to the range that mu and mu_s allow.
__device__ __forceinline__ float clamp_nu32(float nu_raw, float mu, float mu_s, float one_m_mus2) {
  float sq = sqrtf((1.0f - mu * mu) * one_m_mus2);
  return gclamp(nu_raw, mu * mu_s - sq, mu * mu_s + sq);
}

// MIXED: the same decode in FP64, producing q and s directly.
__device__ __forceinline__ void decode_yz64(const DevAtmo& a, const Geo64& G, uint32_t iy, uint32_t iz,
                                            TexelParams& o) {
  double fy = frag_from_texel_d(iy, (uint32_t)a.sc_mu), fz = frag_from_texel_d(iz, (uint32_t)a.sc_r);
  double qz = fy / double(a.sc_mu), qw = fz / double(a.sc_r);
  double rho = G.H * unit_from_coord(qw, a.sc_r);
  o.q = rho * rho;
  o.r = G.radius(o.q);
  if (qz < 0.5) {
    double d_min = o.q / (o.r + G.R);
    double d_max = rho;
    double d = d_min + (d_max - d_min) * unit_from_coord(1.0 - 2.0 * qz, a.sc_mu / 2);
    o.s = d == 0.0 ? -o.r : gmax(-(o.q + d * d) / (2.0 * d), -o.r);
    o.ground = true;
  } else {
    double d_min = (G.H2 - o.q) / (G.T + o.r);
    double d_max = rho + G.H;
    double d = d_min + (d_max - d_min) * unit_from_coord(2.0 * qz - 1.0, a.sc_mu / 2);
    o.s = d == 0.0 ? o.r : gclamp((G.H2 - o.q - d * d) / (2.0 * d), -o.r, o.r);
    o.ground = false;
  }
  o.mu = o.s / o.r;
}
// scattering.h:102-113 in FP64: mu_s and the raw nu of column x.
__device__ __forceinline__ void decode_x64(const DevAtmo& a, const Geo64& G, uint32_t ix, double& mu_s,
                                           double& nu_raw) {
  const double nmus = double(a.sc_mus);
  double fx = frag_from_texel_d(ix, (uint32_t)a.W);
  double f_nu = floor(fx / nmus);
  double f_mus = fx - nmus * floor(fx / nmus);
  double x_mu_s = unit_from_coord(f_mus / nmus, a.sc_mus);
  double d_min = G.T - G.R, d_max = G.H;
  double A = -2.0 * a.mu_s_min * G.R / (d_max - d_min);
  double aa = (A - x_mu_s * A) / (1.0 + x_mu_s * A);
  double d = d_min + gmin(aa, A) * (d_max - d_min);
  mu_s = d == 0.0 ? 1.0 : clamp_cosine((G.H2 - d * d) / (2.0 * G.R * d));
  nu_raw = clamp_cosine(f_nu / double(a.sc_nu - 1) * 2.0 - 1.0);
}
}  // namespace fb
