// fb_passes.cuh — the six precompute passes as persistent, work-list driven
// kernels (sm_103a). Included by fb_kernels_plain.cu (MX = false, compiled
// with --fmad=false) and fb_kernels_mixed.cu (MX = true).
//
// Launch structure (one launch per pass group, any number of atmospheres):
//   k_transmittance  transmittance.comp                      warp per texel, four per work item
//                    geometry tables: rows, x columns (seg 1) thread per entry
//   k_single         single_scattering.comp  (segment 0)     CTA per (mu, r) row(s), texels
//                                                            to threads nu slice fastest
//                    direct_irradiance.comp  (segment 1)     thread per texel
//                    multiple-scattering samples (seg 2)     thread per (row, sample)
//                    density r / theta records (segment 3)   thread per record
//   k_density        scattering_density.comp (segment 0)     CTA per (r, mu_s, mu-chunk)
//                    indirect_irradiance.comp (segment 1)    CTA per irradiance r row (up to 64 texels);
//                                                            order 1: four texels, a warp each
//   k_multiple       multiple_scattering.comp                CTA per (mu, r) row(s); variants 4
//                                                            and 5 compiled for the default layout
// CTAs take work items from a global atomic counter; an item is a tile of one
// atmosphere, located by binary search over per-atmosphere item offsets.
#pragma once

#include <cstddef>
#include "fb_device.cuh"

namespace fb {

constexpr int kThreads = 256;
constexpr int kMaxTexelsPerThread = 8;  // multiple scattering: W <= 2048
constexpr int kMaxThetas = 32;          // density_samples <= 32
constexpr int kMaxNuSlices = 66;        // scattering_nu_size <= 64 (+2 guard slices)

struct Segment {
  int njobs;
  int total;
  const int* job;  // atmosphere index per entry
  const int* off;  // first item of each entry (exclusive prefix sum)
};

constexpr int kMaxSegments = 4;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

struct LaunchArgs {
  const DevAtmo* atm;
  Segment seg[kMaxSegments];
  int nseg;
  int order;  // k_density / k_multiple: order n computed (indirect irradiance integrates n-1)
  unsigned int* counter;
  // Items a CTA takes before it exits (0: no limit, the CTA runs until the
  // work list is empty). A limit lets the block scheduler interleave CTAs of
  // other streams (by priority) between items; the grid then covers the work.
  int max_items;
};

// Takes the next work item of the launch for this CTA; `taken` counts the
// items this CTA has taken (for LaunchArgs::max_items).
__device__ __forceinline__ bool next_item(const LaunchArgs& L, int& seg, int& job, int& tile, int& taken) {
  __shared__ int s_item;
  if (L.max_items > 0 && taken >= L.max_items) return false;
  ++taken;
  __syncthreads();
  if (threadIdx.x == 0) s_item = (int)atomicAdd(L.counter, 1u);
  __syncthreads();
  int item = s_item;
  // segments are scanned with constant indices so that the launch arguments
  // stay in parameter space
  seg = -1;
  int njobs = 0;
  const int* jobs = nullptr;
  const int* offs = nullptr;
#pragma unroll
  for (int s = 0; s < kMaxSegments; ++s) {
    if (seg < 0 && s < L.nseg) {
      if (item < L.seg[s].total) {
        seg = s;
        njobs = L.seg[s].njobs;
        jobs = L.seg[s].job;
        offs = L.seg[s].off;
      } else {
        item -= L.seg[s].total;
      }
    }
  }
  if (seg < 0) return false;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (offs[mid] <= item) lo = mid; else hi = mid - 1;
  }
  job = jobs[lo];
  tile = item - offs[lo];
  return true;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ===================================================================== T ===
// transmittance.comp:8-80. One warp per texel; lanes split the trapezoid
// samples of the three optical lengths, then reduce with shuffles. A work
// item is kTrPerWarp texels per warp, so that the barriers with which a CTA
// takes an item are spread over more texels.
constexpr int kTrPerWarp = 4;
constexpr int kTrTexels = kThreads / 32 * kTrPerWarp;  // texels per work item
template <bool MX> __device__ void tile_transmittance(const DevAtmo& a, int tile) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t0 = tile * kTrTexels;
  const int ntr = a.tr_mu * a.tr_r;
  const int N = a.tr_steps;
  // MIXED: the ray state of the item's texels (transmittance.comp:48-64 in
  // FP64) is computed once per texel by one thread and shared: (q, 2 s, dx).
  __shared__ float3 s_ray[kTrTexels];
  if (MX) {
    if (threadIdx.x < kTrTexels && t0 + (int)threadIdx.x < ntr) {
      const int tt = t0 + threadIdx.x;
      const int i = tt % a.tr_mu, j = tt / a.tr_mu;
      Geo64 G;
      G.init(a);
      double x_mu = double(i) / double(a.tr_mu - 1), x_r = double(j) / double(a.tr_r - 1);
      double rho = G.H * x_r, q = rho * rho, r = G.radius(q);
      double d_min = (G.H2 - q) / (G.T + r), d_max = rho + G.H;
      double d = d_min + x_mu * (d_max - d_min);
      double s = d == 0.0 ? r : gclamp((G.H2 - q - d * d) / (2.0 * d), -r, r);
      s_ray[threadIdx.x] = make_float3((float)q, (float)(2.0 * s), (float)(G.dist_top(q, s) / double(N)));
    }
    __syncthreads();
  }
  for (int m = 0; m < kTrPerWarp; ++m) {
    const int tl = m * (kThreads / 32) + warp;  // texel of the item
    const int t = t0 + tl;
    if (t >= ntr) break;
    float sR, sM, sA;
    if (!MX) {
      const int i = t % a.tr_mu, j = t / a.tr_mu;
      Geo32 G;
      G.init(a);
      float x_mu = float(i) / float(a.tr_mu - 1), x_r = float(j) / float(a.tr_r - 1);
      // transmittance.comp:48-64
      float rho = G.H * x_r;
      float r = sqrtf(rho * rho + G.R * G.R);
      float d_min = G.T - r, d_max = rho + G.H;
      float d = d_min + x_mu * (d_max - d_min);
      float mu = d == 0.0f ? 1.0f : (G.H * G.H - rho * rho - d * d) / (2.0f * r * d);
      mu = clamp_cosine(mu);
      const float dx = G.dist_top(r, mu) / float(N);
      const float two_r_mu = 2.0f * r * mu, rr = r * r;
      sR = sM = sA = 0.0f;
      for (int k = lane; k <= N; k += 32) {
        float d_i = float(k) * dx;
        float r_i = sqrtf(d_i * d_i + two_r_mu * d_i + rr);
        float h = r_i - G.R;
        float w = (k == 0 || k == N) ? 0.5f : 1.0f;
        sR += profile_density(a.ray_d, h) * w * dx;
        sM += profile_density(a.mie_d, h) * w * dx;
        sA += profile_density(a.abs_d, h) * w * dx;
      }
      sR = warp_sum(sR);
      sM = warp_sum(sM);
      sA = warp_sum(sA);
    } else {
      // The march runs in FP32 on the FP64 ray state: r_k^2 - R^2 =
      // q + d_k (2 s + d_k) keeps the altitude q_k / (r_k + R) free of the
      // cancellation of r_k - R, to ~1e-5 km where the ray grazes the ground.
      const float3 ray = s_ray[tl];
      const float qf = ray.x, two_sf = ray.y, dxf = ray.z, Rf = a.bottom, R2f = Rf * Rf;
      float cR = 0.f, cM = 0.f, cA = 0.f;
      sR = sM = sA = 0.0f;
      for (int k = lane; k <= N; k += 32) {
        const float d_k = float(k) * dxf;
        const float q_k = fmaf(d_k, two_sf + d_k, qf);
        const float r_k = sqrtf(q_k + R2f);
        // every ray of this table stays at or above the ground: a negative
        // altitude here is rounding at a tangent sample
        float h = gmax(__fdividef(q_k, r_k + Rf), 0.0f);
        float w = (k == 0 || k == N) ? 0.5f : 1.0f;
        Kahan3::add1(sR, cR, profile_density(a.ray_d, h) * w);
        Kahan3::add1(sM, cM, profile_density(a.mie_d, h) * w);
        Kahan3::add1(sA, cA, profile_density(a.abs_d, h) * w);
      }
      // compensated lane sums, reduced in FP32 (32 terms)
      sR = warp_sum(sR - cR) * dxf;
      sM = warp_sum(sM - cM) * dxf;
      sA = warp_sum(sA - cA) * dxf;
    }
    if (lane == 0) {
      float4 o;
      o.x = expf(-(a.rayleigh[0] * sR + a.mie_ext[0] * sM + a.absorption[0] * sA));
      o.y = expf(-(a.rayleigh[1] * sR + a.mie_ext[1] * sM + a.absorption[1] * sA));
      o.z = expf(-(a.rayleigh[2] * sR + a.mie_ext[2] * sM + a.absorption[2] * sA));
      o.w = 1.0f;
      a.tr[t] = o;
      // the pair table: this texel's RGB first in its own record, second in the
      // record of texel i - 1 and, at the last mu, in its own
      const int i = t % a.tr_mu;
      float* own = a.trp + 8 * (size_t)t;
      own[0] = o.x;
      own[1] = o.y;
      own[2] = o.z;
      own[6] = own[7] = 0.f;
      if (i > 0) {
        own[-5] = o.x;
        own[-4] = o.y;
        own[-3] = o.z;
      }
      if (i == a.tr_mu - 1) {
        own[3] = o.x;
        own[4] = o.y;
        own[5] = o.z;
      }
    }
  }
}


// =========================================================== S: direct ===
// direct_irradiance.comp:10-46 plus the clear of the final irradiance table
// (src/precompute.rs:1802-1816).
template <bool MX> __device__ void tile_direct(const DevAtmo& a, int tile) {
  const int t = tile * kThreads + threadIdx.x;
  if (t >= a.ir_mus * a.ir_r) return;
  const int i = t % a.ir_mus, j = t / a.ir_mus;
  float3 T3;
  float mu_s;
  if (!MX) {
    Geo32 G;
    G.init(a);
    float x_mu_s = float(i) / float(a.ir_mus - 1), x_r = float(j) / float(a.ir_r - 1);
    float r = G.R + x_r * (G.T - G.R);
    mu_s = clamp_cosine(2.0f * x_mu_s - 1.0f);
    T3 = G.tr_to_top(a, r, mu_s);
  } else {
    Geo64 G;
    G.init(a);
    double x_mu_s = double(i) / double(a.ir_mus - 1), x_r = double(j) / double(a.ir_r - 1);
    double h = x_r * (G.T - G.R), r = G.R + h;
    double mus = clamp_cosine(2.0 * x_mu_s - 1.0);
    mu_s = (float)mus;
    T3 = G.tr_to_top(a, h * (r + G.R), r * mus);
  }
  const float al = a.sun_radius;
  const float avg = mu_s < -al ? 0.0f : (mu_s > al ? mu_s : (mu_s + al) * (mu_s + al) / (4.0f * al));
  float3 v = ld3(a.solar) * T3 * avg;
  a.dirr[0][t] = make_float4(v.x, v.y, v.z, 0.0f);
  a.ir[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (MX) {
    a.ir_acc[3 * t] = 0.0;
    a.ir_acc[3 * t + 1] = 0.0;
    a.ir_acc[3 * t + 2] = 0.0;
  }
}

// ============================================================ geometry ===
// Order-independent tables of one atmosphere (transmittance launch, segment
// 1): one thread per x column (ColGeo: mu_s and raw nu) and per (mu, r) row
// (RowGeo: the view ray). PLAIN values are the reference's float decode
// (scattering.h:62-137), MIXED values its FP64 form.
// Entry q of the indirect-irradiance records (MIXED; the FP64 decodes of
// indirect_irradiance.comp:16-40 that do not depend on the order).
__device__ inline void tile_irgeo(const DevAtmo& a, int q) {
  const int NT = a.irr_n / 2, NK = a.sc_nu + 2;
  Geo64 G;
  G.init(a);
  auto row_q = [&](int j) {
    const double h = (double(j) / double(a.ir_r - 1)) * (G.T - G.R), rd = G.R + h;
    return h * (rd + G.R);
  };
  auto col_mus = [&](int i) { return clamp_cosine(2.0 * (double(i) / double(a.ir_mus - 1)) - 1.0); };
  if (q < a.ir_r) {
    const int j = q;
    const double h = (double(j) / double(a.ir_r - 1)) * (G.T - G.R);
    IrZ o;
    o.r = (float)(G.R + h);
    o.az = axis_texel(G.sc_r_texel(a, row_q(j)), a.sc_r);
    a.g_irz[j] = o;
    return;
  }
  q -= a.ir_r;
  if (q < a.ir_r * NT) {
    const int j = q / NT, l = q % NT;
    const double qd = row_q(j);
    const double ct = cos((double(l) + 0.5) * (kPiD / double(a.irr_n)));
    a.g_iry[q] = axis_texel(G.sc_mu_texel(a, qd, G.radius(qd) * ct, false), a.sc_mu);
    return;
  }
  q -= a.ir_r * NT;
  if (q < a.ir_mus * NK) {
    const int i = q / NK, s = q % NK;
    const double ymus = G.mus_unit(a, col_mus(i));
    a.g_irx[q] = axis_texel(double(s - 1) * a.sc_mus + ymus * double(a.sc_mus - 1), a.W);
    return;
  }
  q -= a.ir_mus * NK;
  if (q < a.ir_mus) a.g_irmus[q] = (float)col_mus(q);
}

template <bool MX> __device__ void tile_geometry(const DevAtmo& a, int tile) {
  const int k = tile * kThreads + threadIdx.x;
  const int nrows = a.sc_mu * a.sc_r;
  if (k < a.W) {
    ColGeo c;
    if (!MX) {
      Geo32 G;
      G.init(a);
      decode_x32(a, G, (uint32_t)k, c.mu_s, c.nu_raw);
      c.one_m_mus2 = 1.0f - c.mu_s * c.mu_s;
      c.u_mus = G.u_mu_s(a, c.mu_s);
      c.mu_sd = c.one_m_mus2d = c.nu_rawd = c.t_musd = 0.0;
    } else {
      Geo64 G;
      G.init(a);
      decode_x64(a, G, (uint32_t)k, c.mu_sd, c.nu_rawd);
      c.one_m_mus2d = (1.0 - c.mu_sd) * (1.0 + c.mu_sd);
      c.t_musd = G.mus_unit(a, c.mu_sd) * double(a.sc_mus - 1);
      c.mu_s = (float)c.mu_sd;
      c.one_m_mus2 = (float)c.one_m_mus2d;
      c.nu_raw = (float)c.nu_rawd;
      c.u_mus = 0.f;
    }
    a.g_cols[k] = c;
  } else if (k < a.W + nrows) {
    const int row = k - a.W;
    const uint32_t y = (uint32_t)(row % a.sc_mu), z = (uint32_t)(row / a.sc_mu);
    RowGeo o;
    o.pad = 0;
    if (!MX) {
      Geo32 G;
      G.init(a);
      float r, mu;
      bool g;
      decode_yz32(a, G, y, z, r, mu, g);
      o.r = r;
      o.mu = mu;
      o.ground = g;
      o.dist = g ? G.dist_bottom(r, mu) : G.dist_top(r, mu);
      o.rr = r * r;
      o.two_r_mu = 2.0f * r * mu;
      o.r_mu = r * mu;
      o.q = o.s = o.distd = o.one_m_mu2 = o.mud = 0.0;
    } else {
      Geo64 G;
      G.init(a);
      TexelParams p;
      decode_yz64(a, G, y, z, p);
      o.q = p.q;
      o.s = p.s;
      o.r = (float)p.r;
      o.mu = (float)p.mu;
      o.ground = p.ground;
      o.distd = p.ground ? G.dist_bottom(p.q, p.s) : G.dist_top(p.q, p.s);
      o.dist = (float)o.distd;
      o.one_m_mu2 = (1.0 - p.mu) * (1.0 + p.mu);
      o.mud = p.mu;
      o.rr = o.two_r_mu = o.r_mu = 0.f;
    }
    a.g_rows[row] = o;
  } else if (MX) {
    tile_irgeo(a, k - a.W - nrows);
  }
}

// Entries of the indirect-irradiance records (MIXED), in the order tile_irgeo
// fills them.
__host__ __device__ inline int irgeo_entries(int ir_r, int ir_mus, int irr_n, int sc_nu) {
  return ir_r + ir_r * (irr_n / 2) + ir_mus * (sc_nu + 2) + ir_mus;
}
// Geometry work items of one atmosphere: x columns and (mu, r) rows, then in
// the mixed mode the indirect-irradiance records.
__host__ __device__ inline int tiles_geometry(int W, int sc_mu, int sc_r, int ir_entries) {
  return (W + sc_mu * sc_r + ir_entries + kThreads - 1) / kThreads;
}

template <bool MX> __global__ void __launch_bounds__(kThreads) k_transmittance(LaunchArgs L) {
  int seg, job, tile;
  int taken = 0;
  while (next_item(L, seg, job, tile, taken)) {
    if (seg == 0) tile_transmittance<MX>(L.atm[job], tile);
    else tile_geometry<MX>(L.atm[job], tile);
  }
}

// mu_s, nu (clamped to the range allowed by mu and mu_s, scattering.h:134-136)
// and r * mu_s of texel x of a row, from the geometry tables.
template <bool MX>
__device__ __forceinline__ void texel_mus_nu(const RowGeo& ri, const ColGeo& c, float& mu_s, float& nu,
                                             float& r_mu_s) {
  mu_s = c.mu_s;
  if (!MX) {
    nu = clamp_nu32(c.nu_raw, ri.mu, mu_s, c.one_m_mus2);
  } else {
    // 1 - mu^2 and 1 - mu_s^2 come from FP64 without cancellation; nothing
    // downstream of nu cancels, so the clamp runs in FP32.
    const float sq = sqrtf((float)ri.one_m_mu2 * c.one_m_mus2), mm = ri.mu * mu_s;
    nu = mm + gclamp(c.nu_raw - mm, -sq, sq);
  }
  r_mu_s = ri.r * mu_s;
}

__host__ __device__ inline int rows_per_tile(int W) { return W >= kThreads ? 1 : kThreads / W; }

// ======================================================= MS sample records ===
// multiple_scattering.comp:19-40, the parts that depend on the view ray and
// the sample only (single-scattering launch, segment 2): the sample distance
// and radius, the transmittance from the texel times dx and the trapezoid
// weight, and the four density rows around the sample's (mu, r) with their
// bilinear weights.
template <bool MX> __device__ void tile_msrec(const DevAtmo& a, int tile) {
  const int NS = a.ms_steps + 1;
  const int k = tile * kThreads + threadIdx.x;
  const int nrows = a.sc_mu * a.sc_r;
  if (k >= nrows * NS) return;
  const int row = k / NS, i = k % NS, N = a.ms_steps;
  const RowGeo ri = a.g_rows[row];
  MSRec o;
  o.pad0 = o.pad1 = o.pad2 = 0.f;
  const float w = (i == 0 || i == N) ? 0.5f : 1.0f;
  float3 tv;
  Axis ay, az;
  float dx;
  if (!MX) {
    Geo32 G;
    G.init(a);
    dx = ri.dist / float(N);
    const float d = float(i) * dx;
    const float r_i = G.clamp_radius(sqrtf(d * d + ri.two_r_mu * d + ri.rr));
    const float mu_i = clamp_cosine((ri.r_mu + d) / r_i);
    tv = G.tr_segment(a, ri.r, ri.mu, d, ri.ground);
    az = make_axis(G.u_r(a, r_i), a.sc_r);
    ay = make_axis(G.u_mu(a, r_i, mu_i, ri.ground), a.sc_mu);
    o.d = d;
    o.inv_r = 1.0f / r_i;
  } else {
    GeoMx G;
    G.init(a);
    const double dxd = ri.distd / double(N);
    dx = (float)dxd;
    const double d = double(i) * dxd;
    double q = fma(d, 2.0 * ri.s + d, ri.q), sd = ri.s + d;
    q = fmin(fmax(q, 0.0), G.H2);
    const float r_i = sqrtf((float)q + G.R * G.R);
    sd = fmin(fmax(sd, -(double)r_i), (double)r_i);
    tv = G.tr_segment(a, ri.q, ri.s, d, ri.ground);
    az = axis_texel(G.sc_r_texel(q), a.sc_r);
    ay = axis_texel(G.sc_mu_texel(q, sd, ri.ground), a.sc_mu);
    o.d = (float)d;
    o.inv_r = 1.0f / r_i;
  }
  const float wdx = dx * w;
  o.tvwx = tv.x * wdx;
  o.tvwy = tv.y * wdx;
  o.tvwz = tv.z * wdx;
  o.w[0] = (1.f - ay.f) * (1.f - az.f);
  o.w[1] = ay.f * (1.f - az.f);
  o.w[2] = (1.f - ay.f) * az.f;
  o.w[3] = ay.f * az.f;
  const int rs = 3 * a.Wd / 4;  // float4s per density row
  o.off[0] = (az.i0 * a.sc_mu + ay.i0) * rs;
  o.off[1] = (az.i0 * a.sc_mu + ay.i1) * rs;
  o.off[2] = (az.i1 * a.sc_mu + ay.i0) * rs;
  o.off[3] = (az.i1 * a.sc_mu + ay.i1) * rs;
  a.g_ms[k] = o;
}

__host__ __device__ inline int tiles_msrec(int sc_mu, int sc_r, int ms_steps) {
  return (sc_mu * sc_r * (ms_steps + 1) + kThreads - 1) / kThreads;
}

// =================================================== density r / theta ===
// scattering_density.comp:36-60, the parts that depend on r and the theta
// row only (single-scattering launch, segment 3): per r slice the r axis of
// the 3D tables; per (r slice, theta row) the direction's cosine, the solid
// angle of its row, the ground hit (distance, transmittance x albedo / pi)
// and the mu axis of the lookup.
template <bool MX> __device__ void tile_densgeo(const DevAtmo& a, int tile) {
  const int NT = a.dens_n;
  const int k = tile * kThreads + threadIdx.x;
  if (k >= a.sc_r * (NT + 1)) return;
  if (k < a.sc_r) {
    DensZ o;
    o.pad = 0;
    if (!MX) {
      Geo32 G;
      G.init(a);
      float r, mu;
      bool g;
      decode_yz32(a, G, 0u, (uint32_t)k, r, mu, g);
      o.r = r;
      o.q = 0.0;
      o.az = make_axis(G.u_r(a, r), a.sc_r);
      // irradiance at the ground: irradiance.h:20-30 with r = bottom (x_r = 0)
      o.irx = make_axis(coord_from_unit((a.bottom - a.bottom) / (a.top - a.bottom), a.ir_r), a.ir_r);
    } else {
      Geo64 G;
      G.init(a);
      TexelParams tp;
      decode_yz64(a, G, 0u, (uint32_t)k, tp);
      o.r = (float)tp.r;
      o.q = tp.q;
      o.az = axis_texel(G.sc_r_texel(a, tp.q), a.sc_r);
      o.irx = axis_texel(0.0f, a.ir_r);
    }
    a.g_z[k] = o;
    return;
  }
  const int zi = (k - a.sc_r) / NT, l = (k - a.sc_r) % NT;
  ThetaRec out;
  out.pad = 0;
  DensTheta& o = out.th;
  o.pad = 0;
  if (!MX) {
    Geo32 G;
    G.init(a);
    float r, mu;
    bool gg;
    decode_yz32(a, G, 0u, (uint32_t)zi, r, mu, gg);
    const float dtheta = kPiF / float(NT), dphi = kPiF / float(NT);
    const float theta = (float(l) + 0.5f) * dtheta;
    const float ct = cosf(theta);
    const bool g = G.hits_ground(r, ct);
    float3 tg = make_float3(0.f, 0.f, 0.f);
    float dg = 0.0f;
    if (g) {
      dg = G.dist_bottom(r, ct);
      tg = G.tr_segment(a, r, ct, dg, true) * ld3(a.albedo) * (1.0f / kPiF);
    }
    o.cos_t = ct;
    o.domega = dtheta * dphi * sinf(theta);
    o.dg = dg;
    o.ground = g;
    o.tgx = tg.x;
    o.tgy = tg.y;
    o.tgz = tg.z;
    out.tay = make_axis(G.u_mu(a, r, ct, g), a.sc_mu);
  } else {
    Geo64 G;
    G.init(a);
    TexelParams tp;
    decode_yz64(a, G, 0u, (uint32_t)zi, tp);
    const double dtheta = kPiD / double(NT), dphi = kPiD / double(NT);
    const double theta = (double(l) + 0.5) * dtheta;
    const double ct = cos(theta);
    const double q = tp.q, sv = G.radius(q) * ct;
    const bool g = G.hits_ground(q, sv);
    float3 tg = make_float3(0.f, 0.f, 0.f);
    double dg = 0.0;
    if (g) {
      dg = G.dist_bottom(q, sv);
      tg = G.tr_segment(a, q, sv, dg, true) * ld3(a.albedo) * (float)(1.0 / kPiD);
    }
    o.cos_t = (float)ct;
    o.domega = (float)(dtheta * dphi * sin(theta));
    o.dg = (float)dg;
    o.ground = g;
    o.tgx = tg.x;
    o.tgy = tg.y;
    o.tgz = tg.z;
    out.tay = axis_texel(G.sc_mu_texel(a, q, sv, g), a.sc_mu);
  }
  a.g_th[zi * NT + l] = out;
}

__host__ __device__ inline int tiles_densgeo(int sc_r, int dens_n) {
  return (sc_r * (dens_n + 1) + kThreads - 1) / kThreads;
}

// ============================================================ S: single ===
// Per (row, sample) of single scattering; 16-byte words in the order the
// texel loop reads them, so that each is one shared load. tr and tm are the
// transmittance from the texel times the trapezoid weight times the Rayleigh
// and Mie densities at the sample.
struct __align__(16) SSRec {
  float d, inv_r, r_d, rr_d;
  float e, dmin, inv_span, cos_h;
  float lo, inv_w, fy, trx;
  float try_, trz, tmx, tmy;
  float tmz;
  int y0, y1, pad;
};


template <bool MX>
__device__ void tile_single(const DevAtmo& a, int tile, unsigned char* smem) {
  const int W = a.W, nrows = a.sc_mu * a.sc_r;
  const int R = rows_per_tile(W);
  const int row0 = tile * R;
  const int nrow = min(R, nrows - row0);
  const int N = a.ss_steps, NS = N + 1;
  RowGeo* rows = (RowGeo*)smem;
  SSRec* rec = (SSRec*)(smem + align16(sizeof(RowGeo) * R));
  const int tid = threadIdx.x;
  if (tid < nrow) rows[tid] = a.g_rows[row0 + tid];
  __syncthreads();
  // Per (row, sample): the view ray point, the transmittance to it, the
  // densities there and the parts of the sun lookup that depend on it only.
  for (int k = tid; k < nrow * NS; k += kThreads) {
    const RowGeo& ri = rows[k / NS];
    const int i = k % NS;
    SSRec& o = rec[k];
    o.pad = 0;
    const float w = (i == 0 || i == N) ? 0.5f : 1.0f;
    float3 tv;
    float rho_r, rho_m;
    if (!MX) {
      Geo32 G;
      G.init(a);
      float v;
      // single_scattering.comp:16-23
      const float dx = ri.dist / float(N);
      float d = float(i) * dx;
      float r_d = G.clamp_radius(sqrtf(d * d + ri.two_r_mu * d + ri.rr));
      tv = G.tr_segment(a, ri.r, ri.mu, d, ri.ground);
      o.d = d;
      o.r_d = r_d;
      o.rr_d = r_d * r_d;
      float h = r_d - G.R;
      rho_r = profile_density(a.ray_d, h);
      rho_m = profile_density(a.mie_d, h);
      // transmittance.h:63-74 and :7-24
      float sin_h = G.R / r_d;
      o.cos_h = -sqrtf(gmax(1.0f - sin_h * sin_h, 0.0f));
      o.lo = -sin_h * a.sun_radius;
      o.inv_w = 1.0f / (sin_h * a.sun_radius - o.lo);
      o.inv_r = 1.0f / r_d;
      float rho = safe_sqrt(r_d * r_d - G.R * G.R);
      o.dmin = G.T - r_d;
      o.inv_span = 1.0f / ((rho + G.H) - o.dmin);
      v = coord_from_unit(rho / G.H, a.tr_r);
      o.e = 0.f;
      const Axis ay = make_axis(v, a.tr_r);
      o.y0 = ay.i0;
      o.y1 = ay.i1;
      o.fy = ay.f;
    } else {
      GeoMx G;
      G.init(a);
      const double d = double(i) * (ri.distd / double(N));
      double q = fma(d, 2.0 * ri.s + d, ri.q);
      q = fmin(fmax(q, 0.0), G.H2);
      const float qf = (float)q;
      const float r_d = sqrtf(qf + G.R * G.R);
      tv = G.tr_segment(a, ri.q, ri.s, d, ri.ground);
      o.d = (float)d;
      o.r_d = r_d;
      o.rr_d = 0.f;
      const float h = __fdividef(qf, r_d + G.R);
      rho_r = profile_density(a.ray_d, h);
      rho_m = profile_density(a.mie_d, h);
      const float rho = sqrtf(qf);
      o.inv_r = 1.0f / r_d;
      o.cos_h = -rho * o.inv_r;
      const float sin_h = G.R * o.inv_r;
      o.lo = -sin_h * a.sun_radius;
      o.inv_w = 1.0f / (2.0f * sin_h * a.sun_radius);
      o.e = (float)(G.H2 - q);  // T^2 - r_d^2
      const float dmin = __fdividef(o.e, G.T + r_d);
      o.dmin = dmin;
      o.inv_span = 1.0f / (rho + G.H - dmin);
      const Axis ay = axis_texel(rho * G.inv_H * G.trr1, a.tr_r);
      o.y0 = ay.i0;
      o.y1 = ay.i1;
      o.fy = ay.f;
    }
    const float wr = w * rho_r, wm = w * rho_m;
    o.trx = tv.x * wr;
    o.try_ = tv.y * wr;
    o.trz = tv.z * wr;
    o.tmx = tv.x * wm;
    o.tmy = tv.y * wm;
    o.tmz = tv.z * wm;
  }
  __syncthreads();
  const float TT = a.top * a.top;
  const float trc0 = 0.5f / float(a.tr_mu), trc1 = 1.0f - 1.0f / float(a.tr_mu), trn = float(a.tr_mu);
  // Texels go to threads nu slice fastest: a warp holds a few neighbouring
  // mu_s columns of every nu slice, whose sun directions at a sample (and so
  // transmittance lookups) lie closer together than those of a warp along
  // mu_s, so its lookups touch fewer cache sectors.
  const int NU = a.sc_nu, NMS = a.sc_mus;
  for (int k = tid; k < nrow * W; k += kThreads) {
    const int lr = k / W, kx = k - lr * W, kn = kx / NU;
    const int x = (kx - kn * NU) * NMS + kn;  // nu slice kx % NU, mu_s column kx / NU
    const RowGeo& ri = rows[lr];
    float mu_s, nu, r_mu_s;
    texel_mus_nu<MX>(ri, a.g_cols[x], mu_s, nu, r_mu_s);
    const SSRec* rr = rec + lr * NS;
    Kahan3 ray, mie;
    ray.init();
    mie.init();
    for (int i = 0; i < NS; ++i) {
      const SSRec& o = rr[i];
      float x_mu, mu_s_d;
      if (!MX) {
        // single_scattering.comp:17, transmittance.h:63-74
        mu_s_d = clamp_cosine((r_mu_s + o.d * nu) * o.inv_r);
        float disc = o.rr_d * (mu_s_d * mu_s_d - 1.0f) + TT;
        float dt = gmax(-o.r_d * mu_s_d + safe_sqrt(disc), 0.0f);
        x_mu = (dt - o.dmin) * o.inv_span;
      } else {
        // distance to the top from (r_d, mu_s_d): T^2 - r_d^2 + (r_d mu_s_d)^2
        // under the root, rationalised when the ray points up.
        float s_d = gclamp(fmaf(o.d, nu, r_mu_s), -o.r_d, o.r_d);
        mu_s_d = s_d * o.inv_r;
        // square root as x rsqrt(x) (a few ulp; 0 where the argument is 0,
        // on the top boundary)
        const float disc = fmaf(s_d, s_d, o.e);
        const float root = disc > 1e-30f ? disc * rsqrt_pos(disc) : 0.0f;
        float dt = s_d > 0.0f ? __fdividef(o.e, s_d + root) : root - s_d;
        x_mu = (dt - o.dmin) * o.inv_span;
      }
      // smoothstep(-sin_h alpha, sin_h alpha, mu_s_d - cos_h)
      const float st = gclamp((mu_s_d - o.cos_h - o.lo) * o.inv_w, 0.0f, 1.0f);
      const float sfac = st * st * (3.0f - 2.0f * st);
      // below the first texel centre (only by rounding) the sampler's clamp
      // gives texel 0 alone, as t = 0 does: the pair fetch needs t >= 0
      const Axis ax = MX ? axis_texel(fmaxf(x_mu * float(a.tr_mu - 1), 0.0f), a.tr_mu)
                         : axis_texel(fmaxf(fmaf(fmaf(x_mu, trc1, trc0), trn, -0.5f), 0.0f), a.tr_mu);
      Axis ay;
      ay.i0 = o.y0;
      ay.i1 = o.y1;
      ay.f = o.fy;
      const float3 ts = fetch2_pairs(a.trp, a.tr_mu, ax, ay) * sfac;
      const float3 tr3 = make_float3(o.trx, o.try_, o.trz), tm3 = make_float3(o.tmx, o.tmy, o.tmz);
      if (!MX) {
        ray.s = fma3(ts, tr3, ray.s);
        mie.s = fma3(ts, tm3, mie.s);
      } else {
        ray.add_prod(ts, tr3);
        mie.add_prod(ts, tm3);
      }
    }
    const float dx = MX ? (float)(ri.distd / double(N)) : ri.dist / float(N);
    const float3 rs = MX ? make_float3(ray.s.x - ray.c.x, ray.s.y - ray.c.y, ray.s.z - ray.c.z) : ray.s;
    const float3 ms = MX ? make_float3(mie.s.x - mie.c.x, mie.s.y - mie.c.y, mie.s.z - mie.c.z) : mie.s;
    const float3 R3 = rs * dx * ld3(a.solar) * ld3(a.rayleigh);
    const float3 M3 = ms * dx * ld3(a.solar) * ld3(a.mie_sca);
    const size_t t = (size_t)(row0 + lr) * W + x;
    a.dr[t] = store_round4(make_float4(R3.x, R3.y, R3.z, 0.f), a.f16);
    a.dm[t] = store_round4(make_float4(M3.x, M3.y, M3.z, 0.f), a.f16);
    a.sc[t] = store_round4(make_float4(R3.x, R3.y, R3.z, M3.x), a.f16);
    if (MX) {
      a.sc_acc[3 * t] = R3.x;
      a.sc_acc[3 * t + 1] = R3.y;
      a.sc_acc[3 * t + 2] = R3.z;
    }
  }
}

// Registers capped for 4 resident CTAs per SM (a few bytes of spills in the
// mixed kernel).
template <bool MX> __global__ void __launch_bounds__(kThreads, 4) k_single(LaunchArgs L) {
  extern __shared__ __align__(16) unsigned char smem[];
  int seg, job, tile;
  int taken = 0;
  while (next_item(L, seg, job, tile, taken)) {
    if (seg == 0) tile_single<MX>(L.atm[job], tile, smem);
    else if (seg == 1) tile_direct<MX>(L.atm[job], tile);
    else if (seg == 2) tile_msrec<MX>(L.atm[job], tile);
    else tile_densgeo<MX>(L.atm[job], tile);
  }
}

// ============================================================ density ===
// scattering_density.comp:10-155. A tile is a set of texels that share r (one
// z slice) and S mu_s columns; each thread owns a "nu group": G texels that
// share r, mu and mu_s and differ only in nu.
//  * The previous order's table is looked up at the tile's r and mu_s and at
//    one of the 16 theta rows only, so it is reduced once per tile by
//    trilinear interpolation to P[column][theta][nu slice] (stored with the
//    difference to the next slice): each 4D lookup becomes one linear blend.
//  * The phase functions of the scattering angle omega . omega_i depend on mu
//    and the direction only: they are evaluated once per thread and direction
//    for all G texels.
//  * Directions come in mirror pairs (phi, 2 pi - phi): same cos phi, opposite
//    sin phi, hence the same angle to the view direction (omega has no y
//    component), so each pair shares one phase evaluation.
constexpr int kDensThreads = 128;
constexpr int kDensMaxGroup = 8;

// Per-atmosphere tile shape of the density pass (host and device agree).
struct DensShape {
  int G;      // texels per thread (divides nu_size, <= kDensMaxGroup)
  int NG;     // nu groups per mu row
  int S;      // mu_s columns per tile
  int chunk;  // mu rows per tile
  int scols, ychunks, tiles;
};
// S_req / chunk_req: a tile shape chosen by the autotuner (0 = default rule:
// one mu_s column and every mu row that fits in the block).
__host__ __device__ inline DensShape dens_shape(int sc_r, int sc_mu, int sc_mus, int sc_nu, int S_req = 0,
                                                int chunk_req = 0) {
  DensShape d;
  d.G = (sc_nu % 8 == 0) ? 8 : (sc_nu % 4 == 0) ? 4 : (sc_nu % 2 == 0) ? 2 : 1;
  d.NG = sc_nu / d.G;
  const int per_col = sc_mu * d.NG;
  if (S_req > 0 && chunk_req > 0 && S_req * min(chunk_req, sc_mu) * d.NG <= kDensThreads) {
    d.S = min(S_req, sc_mus);
    d.chunk = min(chunk_req, sc_mu);
  } else if (per_col >= kDensThreads) {
    d.S = 1;
    d.chunk = max(1, kDensThreads / d.NG);
  } else {
    d.S = max(1, min(sc_mus, kDensThreads / per_col));
    d.chunk = sc_mu;
  }
  // the interval tables grow with S (nu + 2) records per theta row: with many
  // nu slices, fewer columns per tile, so that the tables of up to 32 theta
  // rows fit in shared memory
  d.S = max(1, min(d.S, 4096 / (32 * (sc_nu + 2))));
  d.scols = (sc_mus + d.S - 1) / d.S;
  d.ychunks = (sc_mu + d.chunk - 1) / d.chunk;
  d.tiles = sc_r * d.scols * d.ychunks;
  return d;
}

// One interval [k, k + 1] of a linearly interpolated RGB table, as the line
// through its two entries in the variable w = t - 1/2 (t the texel position):
// the line's value at w = 0 in a.xyz and its slope, the difference of the two
// entries, in (a.w, b.x, b.y); 32 bytes, read as one 16- and one 8-byte load
// from the same base address. The value at w in the interval is
// a.xyz + w (a.w, b.x, b.y): one FMA per channel, no offset within the
// interval to form. The line's value at 0 is left entry + (1/2 - k) slope,
// which rounds with the magnitude of k times the slope; k is at most the
// table size, so the error stays a few units in the last place of the
// table's largest values.
struct LerpRec {
  float4 a;
  float2 b;
  float2 pad;
};
// Order 2: the Rayleigh and Mie intervals of the same nu position in one
// 48-byte record, read as three 16-byte loads: a = (R value at 0, R slope x),
// b = (R slope y, R slope z, M value at 0 x, y), c = (M value at 0 z, M slope).
// Records 48 bytes apart also put the intervals 0-7 of a row on disjoint
// banks for each 16-byte load.
struct LerpRec2 {
  float4 a, b, c;
};

// The density tile's interval tables have a power-of-two number of records,
// addressed by k & (size - 1): intervals k >= 0 at position k, the interval
// k = -1 (below the first entry) at the last position, so that any k, even
// one derived from a NaN, stays inside the table. Where such tables do not
// fit in shared memory (CL: the largest nu and irradiance sizes), they hold
// exactly the intervals, k at position k + 1, and the position is clamped.
__host__ __device__ inline int pow2_at_least(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}
// nu intervals -1 .. nu_size of the reduced table (slices -1 .. nu_size + 1)
__host__ __device__ inline int dens_mk(int sc_nu, bool cl) { return cl ? sc_nu + 2 : pow2_at_least(sc_nu + 2); }
// ground irradiance intervals -1 .. ir_mus - 1
__host__ __device__ inline int dens_mke(int ir_mus, bool cl) { return cl ? ir_mus + 1 : pow2_at_least(ir_mus + 1); }
// Position of interval k in a table of n records, and the interval at position p.
template <bool CL> __device__ __forceinline__ int rec_pos(int k, int n) { return CL ? k + 1 : (k & (n - 1)); }
template <bool CL> __device__ __forceinline__ int rec_interval(int p, int n) {
  return CL ? p - 1 : (p == n - 1 ? -1 : p);
}

struct DensLayout {
  DensTheta* th;    // NT
  Axis* tay;        // NT: theta -> mu axis
  Axis* kax;        // S * NK: (column, nu slice) -> x axis
  float2* dir;      // NT * NT mirror pairs: (cos phi sin t, sin phi sin t) x (nu_size - 1) / 2
  float2* gw;       // NT: ground rows, the ground table position as a function of w: (A, B0)
  LerpRec* P;       // S * NT * MK: nu intervals of the previous order (dens_mk); order 2:
                    // LerpRec2 records of the Rayleigh and Mie tables
  LerpRec* E;       // MKE: intervals of the ground irradiance row, the two sampler rows pre-blended (dens_mke)
  float* col_mus;   // S
  double* col_musd; // S (MIXED)
  double2* ymu;     // chunk (MIXED): (mu, 1 - mu^2)
  double* nuraw;    // sc_nu (MIXED)
  float* acc;       // kDensThreads * kDensMaxGroup * 3 * 2 (MIXED: Kahan sum over theta rows)
};

__host__ __device__ inline size_t dens_layout(unsigned char* base, int dens_n, int sc_nu, int ir_mus, int S,
                                              int chunk, bool two, bool mixed, bool cl, DensLayout* L) {
  const int NT = dens_n, NK = sc_nu + 2;
  const size_t nP = (size_t)S * NT * dens_mk(sc_nu, cl);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align16(o + bytes);
    return at;
  };
  size_t o_th = take(sizeof(DensTheta) * NT), o_tay = take(sizeof(Axis) * NT), o_kax = take(sizeof(Axis) * S * NK);
  size_t o_dir = take(sizeof(float2) * NT * NT), o_gw = take(sizeof(float2) * NT);
  size_t o_P = take((two ? sizeof(LerpRec2) : sizeof(LerpRec)) * nP), o_E = take(sizeof(LerpRec) * dens_mke(ir_mus, cl));
  size_t o_cm = take(sizeof(float) * S), o_cmd = take(sizeof(double) * S);
  size_t o_ymu = take(mixed ? sizeof(double2) * chunk : 0), o_nu = take(mixed ? sizeof(double) * sc_nu : 0);
  size_t o_acc = take(mixed ? sizeof(float) * kDensThreads * kDensMaxGroup * 6 : 0);
  if (L) {
    L->th = (DensTheta*)(base + o_th);
    L->tay = (Axis*)(base + o_tay);
    L->kax = (Axis*)(base + o_kax);
    L->dir = (float2*)(base + o_dir);
    L->gw = (float2*)(base + o_gw);
    L->P = (LerpRec*)(base + o_P);
    L->E = (LerpRec*)(base + o_E);
    L->col_mus = (float*)(base + o_cm);
    L->col_musd = (double*)(base + o_cmd);
    L->ymu = (double2*)(base + o_ymu);
    L->nuraw = (double*)(base + o_nu);
    L->acc = (float*)(base + o_acc);
  }
  return o;
}

// Phase functions at the scattering angle nu, folded with the per-channel
// scattering coefficients: (kR kray + kM kmie (1 + g^2 - 2 g nu)^-3/2)(1 + nu^2),
// i.e. beta_R rho_R P_R(nu) + beta_M rho_M P_M(nu) (util.h:26-34).
struct PhaseCoef {
  float3 A, B;  // kR * 3/(16 pi), kM * k_mie
  float g1, g2;
  __device__ __forceinline__ float3 eval(float nu, float scale) const {
    const float t1 = fmaf(nu, nu, 1.0f) * scale;
    const float rs = rsqrt_pos(fmaf(-g2, nu, g1));
    const float rs3 = rs * rs * rs;
    return make_float3(fmaf(B.x, rs3, A.x) * t1, fmaf(B.y, rs3, A.y) * t1, fmaf(B.z, rs3, A.z) * t1);
  }
};

// Interval of a table position. For a cosine c in [-1, 1] the linear texel
// coordinate is t = (c + 1) / 2 (n - 1) in a table of n entries (the
// sampler's u n - 1/2 for u = coord_from_unit((c + 1) / 2)); the callers form
// w = t - 1/2 directly, with the scale folded into their direction tables.
// Rounding w to an integer k through the float adder (adding 1.5 * 2^23) gives
// the interval [k, k + 1] that holds t (or, where t is an integer, the
// neighbouring one: the same value) and its record position in a table of n
// records: k & (n - 1) (the float's low bits; 1.5 * 2^23 has none set), or for
// CL k + 1 clamped to [0, n - 1] (negative values wrap to large unsigned ones).
// Rounding excursions of c just beyond [-1, 1] give k = -1 or k = n - 1,
// whose records extrapolate by the excursion.
constexpr float kRoundMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kRoundMagicBits = 0x4B400000;
template <bool CL> __device__ __forceinline__ int line_pos(float w, int n) {
  const float y = w + kRoundMagic;
  if (CL) return (int)min((unsigned)(__float_as_int(y) - (kRoundMagicBits - 1)), (unsigned)(n - 1));
  return __float_as_int(y) & (n - 1);
}

// The directions of one theta row for the G texels of a thread (all sharing
// r, mu and mu_s): incident radiance of order n - 1 from the reduced table
// (scattering.h:139-179), plus for rows that meet the ground the ground
// bounce (scattering_density.comp:64-84), times the phase functions
// (scattering_density.comp:86-104). Table positions come as w = t - 1/2
// (line_pos): the direction table holds cos phi sin t and sin phi sin t scaled
// by (nu_size - 1) / 2, and the row and column terms carry the offsets.
//
// The ground bounce's lookup position is an affine function of the nu table's
// position w on a theta row: where omega_i meets the ground, at distance dg,
// the normal is n = (r zenith + dg omega_i) / R (the hit point lies on the
// sphere of radius R), so n . omega_s = (dg / R) nu_i + (r / R) mu_s with
// nu_i = omega_i . omega_s = (w + 1/2) / hP - 1. The position in the ground
// irradiance table, we = hE (n . omega_s + 1) - 1/2, is then A w + B with A =
// hE dg / (R hP) per row and B = B0 + hE (r / R) mu_s per row and texel column.
struct DensRowConst {
  float mu, muh, mu_s, oxs;  // mu; mu_s (nu_size - 1) / 2; mu_s; sqrt(1 - mu^2) / ((nu_size - 1) / 2)
  float offP, gmus;          // (n - 1) / 2 - 1/2 of the nu table; hE (r / R) mu_s
  float inv_h, c1;           // TWO: nu = w inv_h + c1
  int nP, nE;                 // records per nu table row and of the ground irradiance table
};
// GC: the texels per thread when known at compile time (kDensMaxGroup, the
// classes with nu a multiple of 8), else 0 and G at run time.
template <bool TWO, bool GROUND, bool CL, int GC>
__device__ __forceinline__ void dens_row(const DensLayout& S, const DensTheta& t, int l, int NT,
                                         const LerpRec* __restrict__ Pl,
                                         const DensRowConst& q, const float (&sx)[kDensMaxGroup],
                                         const float (&sy)[kDensMaxGroup], int G, const PhaseCoef& pc,
                                         float3 (&acc)[kDensMaxGroup]) {
  const float mus_ct = fmaf(q.muh, t.cos_t, q.offP), mu_ct = q.mu * t.cos_t;
  const float2* dirl = S.dir + l * NT;
  float gA = 0.f, gB = 0.f;
  if (GROUND) {
    const float2 g = S.gw[l];
    gA = g.x;
    gB = g.y + q.gmus;
  }
  for (int m = 0; m < NT; ++m) {
    const float2 d = dirl[m];
    // phase functions of omega . omega_i, shared by the pair and the group
    const float nu2 = fmaf(q.oxs, d.x, mu_ct);
    const float3 cf = pc.eval(nu2, t.domega);
#pragma unroll
    for (int j = 0; j < kDensMaxGroup; ++j) {
      if (j < (GC ? GC : G)) {
        const float base = fmaf(sx[j], d.x, mus_ct), dy = sy[j] * d.y;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const float w = side ? base - dy : base + dy;
          const int k = line_pos<CL>(w, q.nP);
          float3 inc;
          if (!TWO) {
            const float4 pa = Pl[k].a;
            const float2 pb = Pl[k].b;
            inc = make_float3(fmaf(pa.w, w, pa.x), fmaf(pb.x, w, pa.y), fmaf(pb.y, w, pa.z));
          } else {
            // R P_R(nu) + M P_M(nu) = (1 + nu^2) (kR R + kM (1 + g^2 - 2 g nu)^-3/2 M),
            // the constants kR, kM folded into the tables
            const LerpRec2& r2 = reinterpret_cast<const LerpRec2*>(Pl)[k];
            const float4 ra = r2.a, rb = r2.b, rc = r2.c;
            const float nu1 = fmaf(w, q.inv_h, q.c1);
            const float t1 = fmaf(nu1, nu1, 1.0f);
            const float rs = rsqrt_pos(fmaf(-pc.g2, nu1, pc.g1));
            const float rs3 = rs * rs * rs;
            inc.x = fmaf(fmaf(rc.y, w, rb.z), rs3, fmaf(ra.w, w, ra.x)) * t1;
            inc.y = fmaf(fmaf(rc.z, w, rb.w), rs3, fmaf(rb.x, w, ra.y)) * t1;
            inc.z = fmaf(fmaf(rc.w, w, rc.x), rs3, fmaf(rb.y, w, ra.z)) * t1;
          }
          if (GROUND) {
            // irradiance of order n - 2 where omega_i meets the ground
            const float we = fmaf(gA, w, gB);
            const int e = line_pos<CL>(we, q.nE);
            const float4 ea = S.E[e].a;
            const float2 eb = S.E[e].b;
            inc.x = fmaf(t.tgx, fmaf(ea.w, we, ea.x), inc.x);
            inc.y = fmaf(t.tgy, fmaf(eb.x, we, ea.y), inc.y);
            inc.z = fmaf(t.tgz, fmaf(eb.y, we, ea.z), inc.z);
          }
          acc[j].x = fmaf(inc.x, cf.x, acc[j].x);
          acc[j].y = fmaf(inc.y, cf.y, acc[j].y);
          acc[j].z = fmaf(inc.z, cf.z, acc[j].z);
        }
      }
    }
  }
}

// MIXED density: theta rows summed in FP32 between two Kahan steps.
constexpr int kDensKahanRows = 4;

// One Kahan step on a (sum, compensation) pair held in shared memory. The
// pointers are volatile so that the compiler keeps the pair in shared memory
// rather than forwarding it through registers across theta rows.
__device__ __forceinline__ void kahan_smem(volatile float* s, volatile float* c, float v) {
  float sum = *s, comp = *c;
  Kahan3::add1(sum, comp, v);
  *s = sum;
  *c = comp;
}

template <bool MX, bool TWO, bool CL>
__device__ void tile_density(const DevAtmo& a, int order, int tile, unsigned char* smem) {
  const int NT = a.dens_n, NNU = a.sc_nu, NK = NNU + 2;
  const DensShape sh = dens_shape(a.sc_r, a.sc_mu, a.sc_mus, a.sc_nu, a.dens_S, a.dens_chunk);
  const int zi = tile / (sh.scols * sh.ychunks);
  const int rem = tile % (sh.scols * sh.ychunks);
  const int s0 = (rem / sh.ychunks) * sh.S, y0 = (rem % sh.ychunks) * sh.chunk;
  const int ns = min(sh.S, a.sc_mus - s0), ny = min(sh.chunk, a.sc_mu - y0);
  const int tid = threadIdx.x, nth = blockDim.x;
  DensLayout S;
  dens_layout(smem, NT, NNU, a.ir_mus, sh.S, sh.chunk, TWO, MX, CL, &S);

  // --- tile scalars (r slice), theta rows, columns and mu rows from the
  // geometry tables
  const DensZ zr = a.g_z[zi];
  const float r = zr.r;
  const Axis s_az = bounded_axis(zr.az, a.sc_r), s_irx = bounded_axis(zr.irx, a.ir_r);
  const ThetaRec* thr = a.g_th + (size_t)zi * NT;
  for (int k = tid; k < NT + ns + (MX ? ny + NNU : 0); k += nth) {
    if (k < NT) {
      const ThetaRec t = thr[k];
      S.th[k] = t.th;
      S.tay[k] = bounded_axis(t.tay, a.sc_mu);
    } else if (k < NT + ns) {
      const int c = k - NT, si = s0 + c;
      const ColGeo cg = a.g_cols[si];
      S.col_mus[c] = cg.mu_s;
      if (!MX) {
        for (int j = 0; j < NK; ++j) S.kax[c * NK + j] = make_axis((float(j - 1) + cg.u_mus) / float(NNU), a.W);
      } else {
        S.col_musd[c] = cg.mu_sd;
        for (int j = 0; j < NK; ++j) S.kax[c * NK + j] = axis_texel(double(j - 1) * a.sc_mus + cg.t_musd, a.W);
      }
    } else if (MX) {
      const int k2 = k - NT - ns;
      if (k2 < ny) {
        const RowGeo& rg = a.g_rows[zi * a.sc_mu + y0 + k2];
        S.ymu[k2] = make_double2(rg.mud, rg.one_m_mu2);
      } else {
        S.nuraw[k2 - ny] = a.g_cols[(k2 - ny) * a.sc_mus].nu_rawd;
      }
    }
  }
  __syncthreads();
  // --- reduced tables: the previous order's table at this tile's r and mu_s
  // columns, on the theta rows, as nu intervals: the entries (pass 1), the
  // differences (pass 2, into the slope fields, which pass 2 readers do not touch),
  // then the line's value at w = 0 and its slope in place (pass 3); the same
  // for the ground irradiance row; direction pairs with ground normals,
  // pre-scaled for line_pos
  const int MK = dens_mk(NNU, CL), MKE = dens_mke(a.ir_mus, CL);
  const int per_col = NT * MK;
  LerpRec2* const P2 = reinterpret_cast<LerpRec2*>(S.P);  // order 2
  const float hP = 0.5f * float(NNU - 1), hE = 0.5f * float(a.ir_mus - 1);
  {
    const float4* src0 = TWO ? a.dr : a.dms;
    // order 2: the Rayleigh and Mie tables carry their phase functions'
    // constants, 3 / (16 pi) and 3 / (8 pi) (1 - g^2) / (2 + g^2)
    const float sR = TWO ? 3.0f / (16.0f * kPiF) : 1.0f;
    const float sM = 3.0f / (8.0f * kPiF) * (1.0f - a.g * a.g) / (2.0f + a.g * a.g);
    for (int k = tid; k < ns * per_col; k += nth) {
      const int c = k / per_col, l = (k % per_col) / MK, p = k % MK;
      // interval ki (-1 .. nu_size): left entry nu slice ki, kax index ki + 1
      const int ki = rec_interval<CL>(p, MK);
      const bool used = ki <= NNU;
      const int sl = ki + 1;
      float3 v = make_float3(0.f, 0.f, 0.f), m = v;
      if (used) {
        v = fetch3(src0, a.W, a.sc_mu, S.kax[c * NK + sl], S.tay[l], s_az) * sR;
        if (TWO) m = fetch3(a.dm, a.W, a.sc_mu, S.kax[c * NK + sl], S.tay[l], s_az) * sM;
      }
      if (!TWO) {
        S.P[k].a = make_float4(v.x, v.y, v.z, 0.f);
        S.P[k].b = S.P[k].pad = make_float2(0.f, 0.f);
      } else {
        P2[k].a = make_float4(v.x, v.y, v.z, 0.f);
        P2[k].b = make_float4(0.f, 0.f, m.x, m.y);
        P2[k].c = make_float4(m.z, 0.f, 0.f, 0.f);
      }
    }
    const float dtheta = kPiF / float(NT), dphi = kPiF / float(NT);
    for (int k = tid; k < NT * NT; k += nth) {
      const int l = k / NT, m = k % NT;
      const float st = sinf((float(l) + 0.5f) * dtheta);
      const float phi = (float(m) + 0.5f) * dphi;
      S.dir[k] = make_float2(cosf(phi) * st * hP, sinf(phi) * st * hP);
    }
    // ground rows: the ground table position we = A w + B0 + hE (r / R) mu_s
    for (int l = tid; l < NT; l += nth) {
      const float g = S.th[l].dg / a.bottom;
      S.gw[l] = make_float2(hE * g / hP, fmaf(hE, fmaf(g, 0.5f / hP - 1.0f, 1.0f), -0.5f));
    }
    // interval ki (entries ki, ki + 1) for ki < ir_mus; interval -1 (below
    // entry 0) holds entry 0's value
    const float4* E = a.dirr[order & 1];  // irradiance of order n-2
    const float fy = s_irx.f;
    for (int k = tid; k < MKE; k += nth) {
      const int ki = rec_interval<CL>(k, MKE);
      const bool used = ki < a.ir_mus;
      const int e = ki < 0 ? 0 : ki;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (used) {
        const float4 e0 = E[s_irx.i0 * a.ir_mus + e], e1 = E[s_irx.i1 * a.ir_mus + e];
        v = make_float4(fmaf(e1.x - e0.x, fy, e0.x), fmaf(e1.y - e0.y, fy, e0.y), fmaf(e1.z - e0.z, fy, e0.z), 0.f);
      }
      S.E[k].a = v;
      S.E[k].b = S.E[k].pad = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  {  // pass 2: differences of the two entries of each interval
    for (int k = tid; k < ns * per_col; k += nth) {
      const int p = k % MK, row0 = k - p, ki = rec_interval<CL>(p, MK);
      if (ki <= NNU - 1) {  // intervals -1 .. nu_size - 1
        const int right = row0 + rec_pos<CL>(ki + 1, MK);
        if (!TWO) {
          const float4 v0 = S.P[k].a, v1 = S.P[right].a;
          S.P[k].b = make_float2(v1.x - v0.x, v1.y - v0.y);
          S.P[k].pad = make_float2(v1.z - v0.z, 0.f);
        } else {
          // values only (the slope slots of `right` are being written by its owner)
          LerpRec2& r0 = P2[k];
          const LerpRec2& r1 = P2[right];
          r0.a.w = r1.a.x - r0.a.x;
          r0.b.x = r1.a.y - r0.a.y;
          r0.b.y = r1.a.z - r0.a.z;
          r0.c.y = r1.b.z - r0.b.z;
          r0.c.z = r1.b.w - r0.b.w;
          r0.c.w = r1.c.x - r0.c.x;
        }
      }
    }
    for (int k = tid; k < MKE; k += nth) {  // intervals 0 .. ir_mus - 2 (-1 and ir_mus - 1: flat)
      const int ki = rec_interval<CL>(k, MKE);
      if (ki >= 0 && ki <= a.ir_mus - 2) {
        const float4 v0 = S.E[k].a, v1 = S.E[rec_pos<CL>(ki + 1, MKE)].a;
        S.E[k].b = make_float2(v1.x - v0.x, v1.y - v0.y);
        S.E[k].pad = make_float2(v1.z - v0.z, 0.f);
      }
    }
  }
  __syncthreads();
  {  // pass 3: the line of interval ki, value at w = 0 and slope, in the record's own fields
    auto line = [](LerpRec& rec, int ki) {
      const float3 d = make_float3(rec.b.x, rec.b.y, rec.pad.x);
      const float c = 0.5f - float(ki);
      rec.a = make_float4(fmaf(c, d.x, rec.a.x), fmaf(c, d.y, rec.a.y), fmaf(c, d.z, rec.a.z), d.x);
      rec.b = make_float2(d.y, d.z);
    };
    for (int k = tid; k < ns * per_col; k += nth) {
      const int ki = rec_interval<CL>(k % MK, MK);
      if (!TWO) {
        line(S.P[k], ki);
      } else {
        LerpRec2& r = P2[k];
        const float c = 0.5f - float(ki);
        r.a.x = fmaf(c, r.a.w, r.a.x);
        r.a.y = fmaf(c, r.b.x, r.a.y);
        r.a.z = fmaf(c, r.b.y, r.a.z);
        r.b.z = fmaf(c, r.c.y, r.b.z);
        r.b.w = fmaf(c, r.c.z, r.b.w);
        r.c.x = fmaf(c, r.c.w, r.c.x);
      }
    }
    for (int k = tid; k < MKE; k += nth) line(S.E[k], rec_interval<CL>(k, MKE));
  }
  __syncthreads();

  // --- this thread's nu group
  const int per_s = sh.chunk * sh.NG;
  const int cl = tid / per_s, yl = (tid % per_s) / sh.NG, grp = tid % sh.NG;
  const bool active = tid < sh.S * per_s && cl < ns && yl < ny;
  if (active) {
    const int G = sh.G, y = y0 + yl, si = s0 + cl;
    float mu = 0.f, ox = 0.f, mu_s;
    float sx[kDensMaxGroup], sy[kDensMaxGroup];
    // MIXED: the texel frame in FP64 (scattering.h:134-136 clamp, frame of
    // scattering_density.comp:28-32): sq, mu mu_s and 1/(1-mu^2) are shared by
    // the group; per texel delta = nu - mu mu_s in [-sq, sq] and
    // sun_y^2 = (sq - delta)(sq + delta) / (1 - mu^2), exactly 0 in the plane.
    double mx_sq = 0.0, mx_mm = 0.0, mx_iom = 0.0, mx_isom = 0.0, mx_omus = 0.0;
    bool mx_pole = false;
    if (MX) {
      const double2 ym = S.ymu[yl];
      const double musd = S.col_musd[cl];
      mx_omus = (1.0 - musd) * (1.0 + musd);
      mx_sq = sqrt(ym.y * mx_omus);
      mx_mm = ym.x * musd;
      mx_pole = ym.y == 0.0;
      mx_iom = mx_pole ? 0.0 : 1.0 / ym.y;
      mx_isom = mx_pole ? 0.0 : 1.0 / sqrt(ym.y);
      mu = (float)ym.x;
      ox = (float)sqrt(ym.y);
    }
#pragma unroll
    for (int j = 0; j < kDensMaxGroup; ++j) {
      sx[j] = sy[j] = 0.f;
      if (j < G) {
        const int nu_i = grp * G + j, x = nu_i * a.sc_mus + si;
        if (!MX) {
          mu = a.g_rows[zi * a.sc_mu + y].mu;
          const ColGeo& cg = a.g_cols[x];
          const float ms = cg.mu_s, nu = clamp_nu32(cg.nu_raw, mu, ms, cg.one_m_mus2);
          // scattering_density.comp:28-32
          ox = sqrtf(1.0f - mu * mu);
          sx[j] = ox == 0.0f ? 0.0f : (nu - mu * ms) / ox;
          sy[j] = sqrtf(gmax(1.0f - sx[j] * sx[j] - ms * ms, 0.0f));
        } else {
          const double delta = gclamp(S.nuraw[nu_i] - mx_mm, -mx_sq, mx_sq);
          if (mx_pole) {
            sx[j] = 0.f;
            sy[j] = sqrtf((float)mx_omus);
          } else {
            sx[j] = (float)(delta * mx_isom);
            sy[j] = sqrtf((float)fmax((mx_sq - delta) * (mx_sq + delta) * mx_iom, 0.0));
          }
        }
      }
    }
    mu_s = S.col_mus[cl];
    const float h0 = r - a.bottom;
    const float rho_r = profile_density(a.ray_d, h0), rho_m = profile_density(a.mie_d, h0);
    const float g = a.g;
    const float kmie = 3.0f / (8.0f * kPiF) * (1.0f - g * g) / (2.0f + g * g);
    const float kray = 3.0f / (16.0f * kPiF);
    PhaseCoef pc;
    pc.A = make_float3(a.rayleigh[0] * rho_r * kray, a.rayleigh[1] * rho_r * kray, a.rayleigh[2] * rho_r * kray);
    pc.B = make_float3(a.mie_sca[0] * rho_m * kmie, a.mie_sca[1] * rho_m * kmie, a.mie_sca[2] * rho_m * kmie);
    pc.g1 = 1.0f + g * g;
    pc.g2 = 2.0f * g;
    DensRowConst q;
    q.mu = mu;
    q.muh = mu_s * hP;
    q.mu_s = mu_s;
    q.oxs = ox / hP;
    q.offP = hP - 0.5f;
    q.gmus = hE * (r / a.bottom) * mu_s;
    q.inv_h = 1.0f / hP;
    q.c1 = 0.5f / hP - 1.0f;
    q.nP = MK;
    q.nE = MKE;
    float3 acc[kDensMaxGroup];
#pragma unroll
    for (int j = 0; j < kDensMaxGroup; ++j) acc[j] = make_float3(0.f, 0.f, 0.f);
    // (sum, compensation) x 3 x G per thread, element e at accs[e * kDensThreads]:
    // consecutive threads use consecutive banks, offsets are immediates
    volatile float* accs = S.acc + tid;
    if (MX) {
#pragma unroll
      for (int e = 0; e < 6 * kDensMaxGroup; ++e) accs[e * kDensThreads] = 0.f;
    }
    for (int l = 0; l < NT; ++l) {
      const DensTheta t = S.th[l];
      const size_t row = (size_t)(cl * NT + l) * MK;
      const LerpRec* Pl = TWO ? reinterpret_cast<const LerpRec*>(reinterpret_cast<const LerpRec2*>(S.P) + row)
                              : S.P + row;
      if (G == kDensMaxGroup) {
        if (t.ground)
          dens_row<TWO, true, CL, kDensMaxGroup>(S, t, l, NT, Pl, q, sx, sy, G, pc, acc);
        else
          dens_row<TWO, false, CL, kDensMaxGroup>(S, t, l, NT, Pl, q, sx, sy, G, pc, acc);
      } else {
        if (t.ground)
          dens_row<TWO, true, CL, 0>(S, t, l, NT, Pl, q, sx, sy, G, pc, acc);
        else
          dens_row<TWO, false, CL, 0>(S, t, l, NT, Pl, q, sx, sy, G, pc, acc);
      }
      if (MX && ((l + 1) % kDensKahanRows == 0 || l == NT - 1)) {
        // Kahan sum over theta rows of the FP32 sums over kDensKahanRows rows
#pragma unroll
        for (int j = 0; j < kDensMaxGroup; ++j) {
          if (j < G) {
            kahan_smem(accs + (6 * j) * kDensThreads, accs + (6 * j + 3) * kDensThreads, acc[j].x);
            kahan_smem(accs + (6 * j + 1) * kDensThreads, accs + (6 * j + 4) * kDensThreads, acc[j].y);
            kahan_smem(accs + (6 * j + 2) * kDensThreads, accs + (6 * j + 5) * kDensThreads, acc[j].z);
            acc[j] = make_float3(0.f, 0.f, 0.f);
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kDensMaxGroup; ++j) {
      if (j < G) {
        const int x = (grp * G + j) * a.sc_mus + si;
        float* row = a.dens + ((size_t)zi * a.sc_mu + y) * 3 * a.Wd;
        float3 o = acc[j];
        if (MX)
          o = make_float3(accs[(6 * j) * kDensThreads] - accs[(6 * j + 3) * kDensThreads],
                          accs[(6 * j + 1) * kDensThreads] - accs[(6 * j + 4) * kDensThreads],
                          accs[(6 * j + 2) * kDensThreads] - accs[(6 * j + 5) * kDensThreads]);
        row[x] = store_round(o.x, a.f16);
        row[a.Wd + x] = store_round(o.y, a.f16);
        row[2 * a.Wd + x] = store_round(o.z, a.f16);
      }
    }
  }
}

// ================================================== indirect irradiance ===
// indirect_irradiance.comp:10-74. A work item is K irradiance texels (K = 4
// where shared memory allows, see ir_per_item), one warp per texel: the warp
// reduces the order's table to P[theta][nu slice] at its texel's (r, mu_s),
// its lanes split the 16 x 64 directions, and a warp shuffle sums them. The
// CTA first tabulates the directions once for its K texels: per direction
// cos phi sin theta, per theta row cos theta and the solid angle (the same
// float arithmetic as evaluating them per direction).
constexpr int kIrMaxPerItem = 4;  // texels per item: one per warp of a kDensThreads CTA
constexpr size_t kIrItemSmem = 64 * 1024;
__host__ __device__ inline size_t indirect_smem_k(int irr_n, int sc_nu, bool one, int k) {
  const size_t NT = irr_n / 2, NP = 2 * (size_t)irr_n;
  return align16(sizeof(float) * NT * NP) + align16(sizeof(float2) * NT) +
         (size_t)k * sizeof(float4) * NT * (sc_nu + 2) * (one ? 2 : 1);
}
// Texels per item: 4, 2 or 1, the most whose tables fit in kIrItemSmem (the
// order-1 layout, the larger one, decides for every order).
__host__ __device__ inline int ir_per_item(int irr_n, int sc_nu) {
  int k = kIrMaxPerItem;
  while (k > 1 && indirect_smem_k(irr_n, sc_nu, true, k) > kIrItemSmem) k >>= 1;
  return k;
}
// Row items (tile_indirect_rows): an item is up to KT irradiance texels of one
// irradiance r row. Shared memory: the direction table, the table blended in
// (mu, r) for one theta row over every x (B; order 1 blends the Rayleigh and
// Mie tables through it in turn), the texels' slice entries of that theta row
// (P, per table) and every thread's FP64 partial sums. KT is the largest of
// 64, 32, 16 whose layout fits in kIrRowsSmem (the order-1 layout, the larger,
// decides); 0 selects the per-texel items.
__host__ __device__ inline size_t ir_rows_smem(int irr_n, int sc_nu, int W, bool one, int kt) {
  const size_t NT = irr_n / 2, NP = 2 * (size_t)irr_n, f = one ? 2 : 1;
  return align16(sizeof(float) * NT * NP) + align16(sizeof(float2) * NT) + align16(sizeof(float4) * W) +
         align16(sizeof(float4) * (size_t)kt * (sc_nu + 2) * f) + sizeof(double) * 3 * kDensThreads;
}
constexpr size_t kIrRowsSmem = 48 * 1024;  // no more than the density tiles' own shared memory
__host__ __device__ inline int ir_rows_kt(int irr_n, int sc_nu, int W, int ir_mus) {
  for (int kt = 64; kt >= 16; kt >>= 1)
    if (ir_rows_smem(irr_n, sc_nu, W, true, kt) <= kIrRowsSmem) return kt < ir_mus ? kt : ir_mus;
  return 0;
}
// Row items integrate orders >= 2 (the multiple-scattering table); order 1
// (the Rayleigh and Mie tables with their phase functions) keeps the items of
// up to four texels, which measured faster there (173.3 against 175.3 ms per
// order-2 density launch of 256 default atmospheres).
__host__ __device__ inline int ir_items_kt(int irr_n, int sc_nu, int W, int ir_mus, bool one) {
  return one ? 0 : ir_rows_kt(irr_n, sc_nu, W, ir_mus);
}
__host__ __device__ inline size_t indirect_smem(int irr_n, int sc_nu, int W, int ir_mus, bool one) {
  const int kt = ir_items_kt(irr_n, sc_nu, W, ir_mus, one);
  return kt ? ir_rows_smem(irr_n, sc_nu, W, one, kt) : indirect_smem_k(irr_n, sc_nu, one, ir_per_item(irr_n, sc_nu));
}
__host__ __device__ inline int tiles_indirect(int ir_mus, int ir_r, int irr_n, int sc_nu, int W, bool one) {
  const int kt = ir_items_kt(irr_n, sc_nu, W, ir_mus, one);
  if (kt) return ir_r * ((ir_mus + kt - 1) / kt);
  const int k = ir_per_item(irr_n, sc_nu);
  return (ir_mus * ir_r + k - 1) / k;
}

template <bool MX>
__device__ void tile_indirect(const DevAtmo& a, int order, int tile, unsigned char* smem) {
  const int ord = order - 1;  // order integrated (the push constant order-1)
  const bool one = ord == 1;
  const int NT = a.irr_n / 2, NP = 2 * a.irr_n;
  const int NNU = a.sc_nu, NK = NNU + 2;
  const int K = ir_per_item(a.irr_n, a.sc_nu);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nth = blockDim.x;
  float* Dcx = (float*)smem;                                          // NT * NP: cos phi sin theta
  float2* Drow = (float2*)(smem + align16(sizeof(float) * NT * NP));  // NT: (cos theta, d omega)
  float4* Pall = (float4*)((unsigned char*)Drow + align16(sizeof(float2) * NT));
  const float dthetaf = kPiF / float(a.irr_n), dphif = kPiF / float(a.irr_n);
  for (int k = tid; k < NT * NP; k += nth) {
    const int l = k / NP, m = k % NP;
    const float theta = (float(l) + 0.5f) * dthetaf, phi = (float(m) + 0.5f) * dphif;
    Dcx[k] = cosf(phi) * sinf(theta);
    if (m == 0) Drow[l] = make_float2(cosf(theta), dthetaf * dphif * sinf(theta));
  }
  const int t = tile * K + warp;
  const bool active = warp < K && t < a.ir_mus * a.ir_r;
  const int PS = NT * NK;  // entries of one table
  float4* P = Pall + (size_t)(warp < K ? warp : 0) * PS * (one ? 2 : 1);
  const int i = t % a.ir_mus, j = t / a.ir_mus;
  float r = 0.f, mu_s = 0.f, u_ms = 0.f;
  Axis az;
  az.i0 = az.i1 = 0;
  az.f = 0.f;
  if (active) {
    if (!MX) {
      Geo32 G;
      G.init(a);
      const float x_mu_s = float(i) / float(a.ir_mus - 1), x_r = float(j) / float(a.ir_r - 1);
      r = G.R + x_r * (G.T - G.R);
      mu_s = clamp_cosine(2.0f * x_mu_s - 1.0f);
      az = make_axis(G.u_r(a, r), a.sc_r);
      u_ms = G.u_mu_s(a, mu_s);
    } else {
      // the FP64 decodes come from the records of the build (tile_irgeo)
      const IrZ z = a.g_irz[j];
      r = z.r;
      az = bounded_axis(z.az, a.sc_r);
      mu_s = a.g_irmus[i];
    }
    const float4* src0 = one ? a.dr : a.dms;
    for (int k = lane; k < PS; k += 32) {
      const int l = k / NK, sl = k % NK;
      Axis ay, ax;
      if (!MX) {
        Geo32 G;
        G.init(a);
        const float ct = cosf((float(l) + 0.5f) * dthetaf);
        ay = make_axis(G.u_mu(a, r, ct, false), a.sc_mu);
        ax = make_axis((float(sl - 1) + u_ms) / float(NNU), a.W);
      } else {
        ay = bounded_axis(a.g_iry[j * NT + l], a.sc_mu);
        ax = bounded_axis(a.g_irx[i * NK + sl], a.W);
      }
      const float3 v = fetch3(src0, a.W, a.sc_mu, ax, ay, az);
      P[k] = make_float4(v.x, v.y, v.z, 0.f);
      if (one) {
        const float3 m = fetch3(a.dm, a.W, a.sc_mu, ax, ay, az);
        P[PS + k] = make_float4(m.x, m.y, m.z, 0.f);
      }
    }
  }
  __syncthreads();
  if (!active) return;
  const float sxs = sqrtf(1.0f - mu_s * mu_s);
  const float g = a.g;
  const float kmie = 3.0f / (8.0f * kPiF) * (1.0f - g * g) / (2.0f + g * g);
  const float kray = 3.0f / (16.0f * kPiF);
  const float g1 = 1.0f + g * g, g2 = 2.0f * g;
  const float fnu = float(NNU - 1);
  // each lane sums its directions of a theta row in FP32 (NP / 32 of them),
  // then adds the row sum to a Kahan-compensated total
  Kahan3 acc;
  acc.init();
  for (int l = 0; l < NT; ++l) {
    const float2 row = Drow[l];
    const float ct = row.x, dom = row.y;
    const float4* Pl = P + l * NK;
    float3 part = make_float3(0.f, 0.f, 0.f);
    for (int m = lane; m < NP; m += 32) {
      // nu = dot(omega, omega_s) with omega_s = (sqrt(1 - mu_s^2), 0, mu_s)
      const float nu = Dcx[l * NP + m] * sxs + ct * mu_s;
      const float tcx = (nu + 1.0f) / 2.0f * fnu;
      float fk = floorf(tcx);
      const float lf = tcx - fk;
      fk = fminf(fmaxf(fk, -1.0f), float(NNU - 1));
      const int ks = (int)fk + 1;
      float3 L;
      if (one) {
        const float4* Ml = Pl + PS;
        const float4 r0 = Pl[ks], r1 = Pl[ks + 1], m0 = Ml[ks], m1 = Ml[ks + 1];
        const float pr = kray * (1.0f + nu * nu);
        const float rs = rsqrt_pos(g1 - g2 * nu);
        const float pm = kmie * (1.0f + nu * nu) * (rs * rs * rs);
        L.x = fmaf(r1.x - r0.x, lf, r0.x) * pr + fmaf(m1.x - m0.x, lf, m0.x) * pm;
        L.y = fmaf(r1.y - r0.y, lf, r0.y) * pr + fmaf(m1.y - m0.y, lf, m0.y) * pm;
        L.z = fmaf(r1.z - r0.z, lf, r0.z) * pr + fmaf(m1.z - m0.z, lf, m0.z) * pm;
      } else {
        const float4 r0 = Pl[ks], r1 = Pl[ks + 1];
        L.x = fmaf(r1.x - r0.x, lf, r0.x);
        L.y = fmaf(r1.y - r0.y, lf, r0.y);
        L.z = fmaf(r1.z - r0.z, lf, r0.z);
      }
      const float3 v = L * ct * dom;
      part.x += v.x;
      part.y += v.y;
      part.z += v.z;
    }
    if (!MX) {
      acc.s.x += part.x;
      acc.s.y += part.y;
      acc.s.z += part.z;
    } else {
      acc.add(part);
    }
  }
  // reduction over the warp's lanes, in FP64
  const double tx = warp_sum((double)acc.s.x - (double)acc.c.x);
  const double ty = warp_sum((double)acc.s.y - (double)acc.c.y);
  const double tz = warp_sum((double)acc.s.z - (double)acc.c.z);
  if (lane == 0) {
    const float3 res = make_float3((float)tx, (float)ty, (float)tz);
    a.dirr[(order + 1) & 1][t] = make_float4(res.x, res.y, res.z, 0.f);
    if (!MX) {
      const float4 old = a.ir[t];
      a.ir[t] = make_float4(res.x + old.x, res.y + old.y, res.z + old.z, 0.f + old.w);
    } else {
      double* acc3 = a.ir_acc + 3 * (size_t)t;
      acc3[0] += tx;
      acc3[1] += ty;
      acc3[2] += tz;
      a.ir[t] = make_float4((float)acc3[0], (float)acc3[1], (float)acc3[2], 0.f);
    }
  }
}

// Row items: KT irradiance texels of one irradiance r row. For each theta row
// the CTA first blends the order's table in (mu, r) at that row's lookup
// position for every x of the packed table (B; coalesced loads, each table
// row read once for the item), then every texel's slice entries are linear
// interpolations of B in x (P), then the texels' directions of that theta row
// are summed. The interpolation is the same trilinear one (blended in y and
// z, then in x). Each texel's directions are split over nth / KT threads
// whose FP64 partial sums meet in shared memory.
template <bool MX>
__device__ void tile_indirect_rows(const DevAtmo& a, int order, int tile, int KT, unsigned char* smem) {
  const int ord = order - 1;  // order integrated (the push constant order-1)
  const bool one = ord == 1;
  const int NT = a.irr_n / 2, NP = 2 * a.irr_n;
  const int NNU = a.sc_nu, NK = NNU + 2, W = a.W;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int segs = (a.ir_mus + KT - 1) / KT;
  const int j = tile / segs, i0 = (tile % segs) * KT;
  const int nt = min(KT, a.ir_mus - i0);
  float* Dcx = (float*)smem;                                          // NT * NP: cos phi sin theta
  float2* Drow = (float2*)(smem + align16(sizeof(float) * NT * NP));  // NT: (cos theta, d omega)
  float4* B = (float4*)((unsigned char*)Drow + align16(sizeof(float2) * NT));  // W
  float4* P = (float4*)((unsigned char*)B + align16(sizeof(float4) * W));        // KT * NK (x2 for order 1)
  double* X = (double*)((unsigned char*)P + align16(sizeof(float4) * (size_t)KT * NK * (one ? 2 : 1)));
  const float dthetaf = kPiF / float(a.irr_n), dphif = kPiF / float(a.irr_n);
  for (int k = tid; k < NT * NP; k += nth) {
    const int l = k / NP, m = k % NP;
    const float theta = (float(l) + 0.5f) * dthetaf, phi = (float(m) + 0.5f) * dphif;
    Dcx[k] = cosf(phi) * sinf(theta);
    if (m == 0) Drow[l] = make_float2(cosf(theta), dthetaf * dphif * sinf(theta));
  }
  // this irradiance row and the thread's texel (t) and share of its directions (h of H)
  const int H = nth / KT, t = tid % KT, h = tid / KT;
  const bool active = t < nt && h < H;
  const int i = i0 + (t < nt ? t : 0);
  float r = 0.f, mu_s, u_ms = 0.f;
  Axis az;
  if (!MX) {
    Geo32 G;
    G.init(a);
    const float x_mu_s = float(i) / float(a.ir_mus - 1), x_r = float(j) / float(a.ir_r - 1);
    r = G.R + x_r * (G.T - G.R);
    mu_s = clamp_cosine(2.0f * x_mu_s - 1.0f);
    az = make_axis(G.u_r(a, r), a.sc_r);
    u_ms = G.u_mu_s(a, mu_s);
  } else {
    const IrZ z = a.g_irz[j];
    r = z.r;
    az = bounded_axis(z.az, a.sc_r);
    mu_s = a.g_irmus[i];
  }
  const float4* src0 = one ? a.dr : a.dms;
  const float sxs = sqrtf(1.0f - mu_s * mu_s);
  const float g = a.g;
  const float kmie = 3.0f / (8.0f * kPiF) * (1.0f - g * g) / (2.0f + g * g);
  const float kray = 3.0f / (16.0f * kPiF);
  const float g1 = 1.0f + g * g, g2 = 2.0f * g;
  const float fnu = float(NNU - 1);
  const int PS = KT * NK;
  Kahan3 acc;
  acc.init();
  for (int l = 0; l < NT; ++l) {
    // B: the table at this theta row's (mu, r) position, every x
    Axis ay;
    if (!MX) {
      Geo32 G;
      G.init(a);
      ay = make_axis(G.u_mu(a, r, cosf((float(l) + 0.5f) * dthetaf), false), a.sc_mu);
    } else {
      ay = bounded_axis(a.g_iry[j * NT + l], a.sc_mu);
    }
    const float w00 = (1.0f - ay.f) * (1.0f - az.f), w10 = ay.f * (1.0f - az.f);
    const float w01 = (1.0f - ay.f) * az.f, w11 = ay.f * az.f;
    const size_t r00 = ((size_t)az.i0 * a.sc_mu + ay.i0) * W, r10 = ((size_t)az.i0 * a.sc_mu + ay.i1) * W;
    const size_t r01 = ((size_t)az.i1 * a.sc_mu + ay.i0) * W, r11 = ((size_t)az.i1 * a.sc_mu + ay.i1) * W;
    for (int tab = 0; tab < (one ? 2 : 1); ++tab) {
      const float4* T = tab ? a.dm : src0;
      for (int x = tid; x < W; x += nth) {
        const float4 p00 = ld4(T + r00 + x), p10 = ld4(T + r10 + x), p01 = ld4(T + r01 + x), p11 = ld4(T + r11 + x);
        B[x] = make_float4(fmaf(w11, p11.x, fmaf(w01, p01.x, fmaf(w10, p10.x, w00 * p00.x))),
                           fmaf(w11, p11.y, fmaf(w01, p01.y, fmaf(w10, p10.y, w00 * p00.y))),
                           fmaf(w11, p11.z, fmaf(w01, p01.z, fmaf(w10, p10.z, w00 * p00.z))), 0.f);
      }
      __syncthreads();
      // P: each texel's entries of the nu slices -1 .. nu_size at its mu_s
      float4* Pt = P + tab * PS;
      for (int e = tid; e < nt * NK; e += nth) {
        const int t2 = e / NK, sl = e - t2 * NK;
        Axis ax;
        if (!MX) {
          Geo32 G;
          G.init(a);
          const float ms2 = clamp_cosine(2.0f * (float(i0 + t2) / float(a.ir_mus - 1)) - 1.0f);
          ax = make_axis((float(sl - 1) + G.u_mu_s(a, ms2)) / float(NNU), a.W);
        } else {
          ax = bounded_axis(a.g_irx[(i0 + t2) * NK + sl], a.W);
        }
        const float4 b0 = B[ax.i0], b1 = B[ax.i1];
        const float f0 = 1.0f - ax.f;
        Pt[e] = make_float4(fmaf(ax.f, b1.x, f0 * b0.x), fmaf(ax.f, b1.y, f0 * b0.y), fmaf(ax.f, b1.z, f0 * b0.z), 0.f);
      }
      __syncthreads();
    }
    if (active) {
      const float2 row = Drow[l];
      const float ct = row.x, dom = row.y;
      const float4* Pl = P + t * NK;
      float3 part = make_float3(0.f, 0.f, 0.f);
      for (int m = h; m < NP; m += H) {
        // nu = dot(omega, omega_s) with omega_s = (sqrt(1 - mu_s^2), 0, mu_s)
        const float nu = Dcx[l * NP + m] * sxs + ct * mu_s;
        const float tcx = (nu + 1.0f) / 2.0f * fnu;
        float fk = floorf(tcx);
        const float lf = tcx - fk;
        fk = fminf(fmaxf(fk, -1.0f), float(NNU - 1));
        const int ks = (int)fk + 1;
        float3 L;
        if (one) {
          const float4* Ml = Pl + PS;
          const float4 r0 = Pl[ks], r1 = Pl[ks + 1], m0 = Ml[ks], m1 = Ml[ks + 1];
          const float pr = kray * (1.0f + nu * nu);
          const float rs = rsqrt_pos(g1 - g2 * nu);
          const float pm = kmie * (1.0f + nu * nu) * (rs * rs * rs);
          L.x = fmaf(r1.x - r0.x, lf, r0.x) * pr + fmaf(m1.x - m0.x, lf, m0.x) * pm;
          L.y = fmaf(r1.y - r0.y, lf, r0.y) * pr + fmaf(m1.y - m0.y, lf, m0.y) * pm;
          L.z = fmaf(r1.z - r0.z, lf, r0.z) * pr + fmaf(m1.z - m0.z, lf, m0.z) * pm;
        } else {
          const float4 r0 = Pl[ks], r1 = Pl[ks + 1];
          L.x = fmaf(r1.x - r0.x, lf, r0.x);
          L.y = fmaf(r1.y - r0.y, lf, r0.y);
          L.z = fmaf(r1.z - r0.z, lf, r0.z);
        }
        const float3 v = L * ct * dom;
        part.x += v.x;
        part.y += v.y;
        part.z += v.z;
      }
      if (!MX) {
        acc.s.x += part.x;
        acc.s.y += part.y;
        acc.s.z += part.z;
      } else {
        acc.add(part);
      }
    }
    __syncthreads();  // B and P are rebuilt for the next theta row
  }
  // the texel's partial sums, in FP64
  X[3 * tid] = (double)acc.s.x - (double)acc.c.x;
  X[3 * tid + 1] = (double)acc.s.y - (double)acc.c.y;
  X[3 * tid + 2] = (double)acc.s.z - (double)acc.c.z;
  __syncthreads();
  if (h == 0 && t < nt) {
    double tx = 0.0, ty = 0.0, tz = 0.0;
    for (int q = 0; q < H; ++q) {
      const int o = 3 * (q * KT + t);
      tx += X[o];
      ty += X[o + 1];
      tz += X[o + 2];
    }
    const int tt = j * a.ir_mus + i;
    const float3 res = make_float3((float)tx, (float)ty, (float)tz);
    a.dirr[(order + 1) & 1][tt] = make_float4(res.x, res.y, res.z, 0.f);
    if (!MX) {
      const float4 old = a.ir[tt];
      a.ir[tt] = make_float4(res.x + old.x, res.y + old.y, res.z + old.z, 0.f + old.w);
    } else {
      double* acc3 = a.ir_acc + 3 * (size_t)tt;
      acc3[0] += tx;
      acc3[1] += ty;
      acc3[2] += tz;
      a.ir[tt] = make_float4((float)acc3[0], (float)acc3[1], (float)acc3[2], 0.f);
    }
  }
}

// V selects the occupancy variant chosen by the autotuner: V = 0 caps the
// registers for 4 resident blocks per SM, V = 1 for 3, V = 2 for 5. TWO: the
// launch of order 2, whose lookups read the single-scattering Rayleigh and
// Mie tables. CL: clamped interval tables (the largest sizes).
template <bool MX, int V, bool TWO, bool CL>
__global__ void __launch_bounds__(kDensThreads, V == 0 ? 4 : (V == 1 ? 3 : 5)) k_density(LaunchArgs L) {
  extern __shared__ __align__(16) unsigned char smem[];
  int seg, job, tile;
  int taken = 0;
  while (next_item(L, seg, job, tile, taken)) {
    if (seg == 0) {
      tile_density<MX, TWO, CL>(L.atm[job], L.order, tile, smem);
    } else {
      const DevAtmo& a = L.atm[job];
      // order 2 (TWO) integrates order 1, which always takes the four-texel
      // items: its kernel does not contain the row items
      const int kt = TWO ? 0 : ir_items_kt(a.irr_n, a.sc_nu, a.W, a.ir_mus, false);
      if (!TWO && kt)
        tile_indirect_rows<MX>(a, L.order, tile, kt, smem);
      else
        tile_indirect<MX>(a, L.order, tile, smem);
    }
  }
}

// ================================================== multiple scattering ===
// multiple_scattering.comp:9-93. Every texel of a row shares the ray (r, mu)
// and hence, for each trapezoid sample, the sample radius, its mu, the
// transmittance from the texel and the (mu, r) coordinates of the density
// lookup: those come from the sample records (MSRec) computed once per build.
// For each sample the CTA interpolates the density table in (mu, r) once into
// a slab over x; each texel then blends four slab entries (two mu_s
// neighbours in two nu slices).
// Tile of multiple scattering: whole rows (a texel's lookups can reach any
// nu slice of its row: its clamped nu picks the slices), R = threads / W rows
// per CTA for rows of at most `threads` texels, else one row with TPT texels
// per thread. Launches use CTAs of kThreads threads; when a row of the launch
// is wider, CTAs of kMsMidThreads (two per SM, so that one runs while the
// other waits at its per-sample barrier) up to rows of 512 texels, else of
// kMsWideThreads (one texel per thread up to rows of 1024: measured faster
// than two per thread on kMsMidThreads, which spill). The slab of a row holds,
// like the density table, three planes (R, G, B): each the row plus a zero
// guard nu slice, read with weight 0 where nu = 1 selects the last slice. A
// thread builds four entries of one plane from four 16-byte loads (one per
// density row), so the unused fourth channel of an RGBA table is never moved.
constexpr int kMsMidThreads = 512;
// Slab buffers of a tile: two samples are taken per barrier while the next two
// are built.
constexpr int kMsSlabs = 4;
constexpr int kMsWideThreads = 1024;
// The default table layout (32 mu_s texels, 8 nu slices), for which the
// multiple-scattering kernels are also compiled with the sizes fixed (the
// slab offsets of the texel loads become constants).
constexpr int kMsFixedMuS = 32, kMsFixedW = 8 * kMsFixedMuS;
constexpr int kMsRowBytes = 96 * 1024;  // shared memory for the rows of a tile (records + slabs)
struct MSShape {
  int R;         // rows per tile
  int TPT;       // texels per thread
  int slab_row;  // floats per slab plane: W, a zero guard slice and one zero entry, rounded up to 4
};
__host__ __device__ inline MSShape ms_shape(int W, int sc_mus, int steps, int threads) {
  MSShape m;
  m.slab_row = (W + sc_mus + 1 + 3) & ~3;
  const int row_bytes = (int)sizeof(MSRec) * (steps + 1) + kMsSlabs * 3 * (int)sizeof(float) * m.slab_row;
  m.R = W <= threads ? min(threads / W, max(1, kMsRowBytes / row_bytes)) : 1;
  m.TPT = (m.R * W + threads - 1) / threads;
  return m;
}
// CTA size of a launch over rows of width W (the widest of the launch).
__host__ __device__ inline int ms_threads(int W) {
  return W <= kThreads ? kThreads : (W <= kMsMidThreads ? kMsMidThreads : kMsWideThreads);
}
// Kernel variant of a launch of `block` threads: 2 and 3 for the wide CTA
// sizes, -1 for kThreads (the tuned occupancy variant 0 or 1 applies).
__host__ __device__ inline int ms_block_variant(int block) {
  return block == kMsWideThreads ? 2 : (block == kMsMidThreads ? 3 : -1);
}
// An atmosphere of the fixed layout: with CTAs of kThreads (one texel per
// thread) its launches may take variants 4 and 5.
__host__ __device__ inline bool ms_fixed_layout(int W, int sc_mus) {
  return W == kMsFixedW && sc_mus == kMsFixedMuS;
}
__host__ __device__ inline int tiles_multiple(int W, int sc_mus, int steps, int sc_mu, int sc_r, int threads) {
  const MSShape m = ms_shape(W, sc_mus, steps, threads);
  return (sc_mu * sc_r + m.R - 1) / m.R;
}
__host__ __device__ inline size_t ms_smem(int W, int steps, int sc_mus, int threads) {
  const MSShape m = ms_shape(W, sc_mus, steps, threads);
  return align16(sizeof(MSRec) * (size_t)m.R * (steps + 1)) + kMsSlabs * 3 * sizeof(float) * (size_t)m.R * m.slab_row;
}

// Position t in [0, n - 1] within a row of n texels as (i0, f): texel i0 in
// [0, n - 1] and weight f of texel i0 + 1 (the value at t is p[i0] + f
// (p[i0 + 1] - p[i0])); the clamp also maps NaN to 0. Rounding t - 1/2 to an
// integer through the float adder gives floor(t), or floor(t) - 1 with f = 1
// where t is an integer: the same interpolated value.
__device__ __forceinline__ int row_pos(float t, float n_minus_1, float& f) {
  t = fminf(fmaxf(t, 0.0f), n_minus_1);
  const float y = (t - 0.5f) + kRoundMagic;
  f = t - (y - kRoundMagic);
  return max(__float_as_int(y) - kRoundMagicBits, 0);
}

// Compile-time switch of the multiple-scattering sample loop's lambdas.
template <bool B> struct MsFast {
  static constexpr bool value = B;
};

// NMC, WC: the mu_s size and row width when fixed at compile time (the slab
// offsets of the texel loads become constants), else 0; NTH: the CTA size.
template <bool MX, int TPT, int NMC, int WC, int NTH>
__device__ void tile_multiple(const DevAtmo& a, int order, int tile, unsigned char* smem) {
  const int W = WC ? WC : a.W, nrows = a.sc_mu * a.sc_r, NM = NMC ? NMC : a.sc_mus;
  const int nth = NTH;
  const MSShape sh = ms_shape(W, NM, a.ms_steps, nth);
  const int row0 = tile * sh.R;
  const int nrow = min(sh.R, nrows - row0);
  const int N = a.ms_steps, NS = N + 1;
  const int tid = threadIdx.x;
  const int SR = sh.slab_row;                      // slab plane stride
  MSRec* rec = (MSRec*)smem;
  float* slab = (float*)(smem + align16(sizeof(MSRec) * (size_t)sh.R * NS));
  const int nx_tex = nrow * W;                     // texels of the tile = slab entries built per sample
  const int slab_stride = sh.R * 3 * SR;
  // zero guard after each plane row: a nu slice (read with weight 0 where
  // nu = 1 selects the last slice) and one entry (read with weight 0 where the
  // mu_s position is the slice's last texel)
  const int ng = NM + 1;
  for (int k = tid; k < kMsSlabs * nrow * 3 * ng; k += nth) {
    const int pl = k / ng;  // plane row: slab pl / (3 nrow), row and plane pl % (3 nrow)
    slab[(pl / (3 * nrow)) * slab_stride + (pl % (3 * nrow)) * SR + W + k % ng] = 0.f;
  }
  {  // this tile's sample records, their density row offsets bounded to the table
    static_assert(sizeof(MSRec) == 4 * sizeof(int4) && offsetof(MSRec, off) == 3 * sizeof(int4),
                  "MSRec: four 16-byte words, the offsets last");
    const int4* src = reinterpret_cast<const int4*>(a.g_ms + (size_t)row0 * NS);
    int4* dst = reinterpret_cast<int4*>(rec);
    const int omax = (a.sc_r * a.sc_mu - 1) * (3 * a.Wd / 4);  // start of the table's last row
    for (int k = tid; k < nrow * NS; k += nth) {
      int4 o = __ldg(src + 4 * k + 3);
      o.x = min(max(o.x, 0), omax);
      o.y = min(max(o.y, 0), omax);
      o.z = min(max(o.z, 0), omax);
      o.w = min(max(o.w, 0), omax);
      dst[4 * k] = __ldg(src + 4 * k);
      dst[4 * k + 1] = __ldg(src + 4 * k + 1);
      dst[4 * k + 2] = __ldg(src + 4 * k + 2);
      dst[4 * k + 3] = o;
    }
  }
  // per-texel constants (TPT texels per thread): row, slab entry, texel x
  float c_rmus[TPT], c_nu[TPT], c_lerp[TPT];
  int c_lr[TPT], c_e[TPT], c_x[TPT], c_ro[TPT];
  // per-unit constants of the slab build (TPT units per thread; a unit is
  // four entries of one plane of a row, and a tile has at most as many units
  // as texels since rows are at least 4 entries wide): row's record offset,
  // float offset in the density row, slab offset, entries in use.
  //
  // The sample loop branches on warp-wide conditions only (warp votes), so
  // that it needs no divergence handling: warps without units or texels skip
  // that work, and in a warp with some, a lane without a unit repeats another
  // lane's unit (the same values stored to the same entries) and a lane
  // without a texel computes texel 0 of the tile and stores nothing.
  const int G4 = (W + 3) / 4, nunits = nrow * 3 * G4;
  int u_ro[TPT], u_src[TPT], u_dst[TPT], u_n[TPT];
  bool w_unit[TPT], w_tex[TPT], has_tex[TPT];
  bool all_full = true;
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    const int u0 = tid + j * nth, u = u0 < nunits ? u0 : u0 % nunits;
    const int lr = u / (3 * G4), rem = u - lr * 3 * G4, pl = rem / G4, g = rem - pl * G4;
    u_ro[j] = lr * NS;
    u_src[j] = pl * a.Wd + 4 * g;
    u_dst[j] = (lr * 3 + pl) * SR + 4 * g;
    u_n[j] = min(4, W - 4 * g);
    w_unit[j] = __any_sync(0xffffffffu, u0 < nunits);
    all_full = all_full && u_n[j] == 4;
  }
  all_full = __all_sync(0xffffffffu, all_full);
  Kahan3 acc[TPT];
  float3 part[TPT];
  MuS32 mus32;
  mus32.init(a);
  MuSRef32 musref;
  musref.init(a);
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    acc[j].init();
    part[j] = make_float3(0.f, 0.f, 0.f);
    c_rmus[j] = c_nu[j] = c_lerp[j] = 0.f;
    const int k0 = tid + j * nth;
    has_tex[j] = k0 < nx_tex;
    w_tex[j] = __any_sync(0xffffffffu, has_tex[j]);
    const int k = has_tex[j] ? k0 : 0;
    c_lr[j] = k / W;
    c_x[j] = k - c_lr[j] * W;
    c_e[j] = c_lr[j] * 3 * SR;
    c_ro[j] = c_lr[j] * NS;
    {
      float mu_s, nu, rmus;
      texel_mus_nu<MX>(a.g_rows[row0 + c_lr[j]], a.g_cols[c_x[j]], mu_s, nu, rmus);
      c_nu[j] = nu;
      c_rmus[j] = rmus;
      // scattering.h:146-148: slices tex_x and tex_x + 1 of the row
      const float tcx = (nu + 1.0f) / 2.0f * float(a.sc_nu - 1);
      const float fl = fminf(fmaxf(floorf(tcx), 0.0f), float(a.sc_nu - 1));
      c_lerp[j] = tcx - fl;
      c_e[j] += (int)fl * NM;
    }
  }
  __syncthreads();
  const float* dens = a.dens;
  // Slab of sample i: the density table interpolated in (mu, r) at the
  // sample, for the tile's slices of the row. With one texel per thread its
  // four loads are issued one sample ahead (load) and blended after the texel
  // work (blend); with more, the registers are not there and the loads
  // directly precede the blend. The last unit of a plane row reads up to
  // three entries of the density table's padding and stores only those in
  // use, leaving the zero guard alone.
  constexpr bool kAhead = TPT == 1;
  float4 q[TPT][4];
  // `fast` (MsFast<true>): the warp has a unit and a texel in every slot and
  // every unit is full, so the per-slot tests fold away
  // Samples are loaded in order. With one row per tile (the fixed layout) all
  // threads load the same four density rows, and a sample in the same (mu, r)
  // cell as the one before (the offsets of two opposite corners fix all four)
  // keeps the values already loaded.
  int prev0 = -1, prev3 = -1;
  auto load = [&](auto fast, int i) {
#pragma unroll
    for (int j = 0; j < TPT; ++j) {
      if (decltype(fast)::value || w_unit[j]) {
        const MSRec& o = rec[u_ro[j] + i];
        if (NMC) {
          const int o0 = o.off[0], o3 = o.off[3];
          if (o0 == prev0 && o3 == prev3) continue;
          prev0 = o0;
          prev3 = o3;
        }
        const float4* p = reinterpret_cast<const float4*>(dens + u_src[j]);
#pragma unroll
        for (int c = 0; c < 4; ++c) q[j][c] = ld4(p + o.off[c]);
      }
    }
  };
  auto blend = [&](auto fast, int i, float* dst) {
#pragma unroll
    for (int j = 0; j < TPT; ++j) {
      if (decltype(fast)::value || w_unit[j]) {
        const MSRec& o = rec[u_ro[j] + i];
        const float w00 = o.w[0], w10 = o.w[1], w01 = o.w[2], w11 = o.w[3];
        const float4 a00 = q[j][0], a10 = q[j][1], a01 = q[j][2], a11 = q[j][3];
        float4 v;
        v.x = fmaf(w11, a11.x, fmaf(w01, a01.x, fmaf(w10, a10.x, w00 * a00.x)));
        v.y = fmaf(w11, a11.y, fmaf(w01, a01.y, fmaf(w10, a10.y, w00 * a00.y)));
        v.z = fmaf(w11, a11.z, fmaf(w01, a01.z, fmaf(w10, a10.z, w00 * a00.z)));
        v.w = fmaf(w11, a11.w, fmaf(w01, a01.w, fmaf(w10, a10.w, w00 * a00.w)));
        float* d = dst + u_dst[j];
        if (decltype(fast)::value || all_full || u_n[j] == 4) {
          *reinterpret_cast<float4*>(d) = v;
        } else {
          d[0] = v.x;
          if (u_n[j] > 1) d[1] = v.y;
          if (u_n[j] > 2) d[2] = v.z;
        }
      }
    }
  };
  const float fmus = float(NM);
  // the texel work of sample i on its slab; `close`: sample i ends a run of
  // the mixed sums (i % 8 == 7 or the last sample)
  auto step = [&](auto fast, int i, const float* cur, bool close) {
#pragma unroll
    for (int j = 0; j < TPT; ++j) {
      if (decltype(fast)::value || w_tex[j]) {
        const MSRec& o = rec[c_ro[j] + i];
        const float nu = c_nu[j];
        // position within a nu slice, texel units (scattering.h:48-56, 149-151):
        // both slices of the lookup share it
        float t;
        if (!MX) {
          const float mu_s_i = clamp_cosine((c_rmus[j] + o.d * nu) * o.inv_r);
          t = fmaf(musref.coord(mu_s_i), fmus, -0.5f);
        } else {
          const float mu_s_i = clamp_cosine(fmaf(o.d, nu, c_rmus[j]) * o.inv_r);
          t = mus32.texel(mu_s_i);
        }
        float fx;
        const int i0 = row_pos(t, fmus - 1.0f, fx);
        const float* sl = cur + c_e[j] + i0;
        const float* sg = sl + SR;
        const float* sb = sl + 2 * SR;
        const float lf = c_lerp[j];
        const float ax = fmaf(sl[1] - sl[0], fx, sl[0]), bx = fmaf(sl[NM + 1] - sl[NM], fx, sl[NM]);
        const float ay = fmaf(sg[1] - sg[0], fx, sg[0]), by = fmaf(sg[NM + 1] - sg[NM], fx, sg[NM]);
        const float az = fmaf(sb[1] - sb[0], fx, sb[0]), bz = fmaf(sb[NM + 1] - sb[NM], fx, sb[NM]);
        const float3 J = make_float3(fmaf(bx - ax, lf, ax), fmaf(by - ay, lf, ay), fmaf(bz - az, lf, az));
        const float3 tvw = make_float3(o.tvwx, o.tvwy, o.tvwz);
        if (!MX) {
          acc[j].s = fma3(J, tvw, acc[j].s);
        } else {
          // plain sums over runs of 8 samples, Kahan-compensated across runs
          part[j] = fma3(J, tvw, part[j]);
          if (close) {
            acc[j].add(part[j]);
            part[j] = make_float3(0.f, 0.f, 0.f);
          }
        }
      }
    }
  };
  // sample i lives in slab buffer i % kMsSlabs; with one texel per thread the
  // mixed loop runs four samples per iteration so that every buffer is a
  // fixed pointer (with two, the longer body spills)
  float* const sb0 = slab;
  float* const sb1 = slab + slab_stride;
  float* const sb2 = slab + 2 * slab_stride;
  float* const sb3 = slab + 3 * slab_stride;
  static_assert(kMsSlabs == 4, "four slab buffers");
  // sample k from `cur` while sample k + A is built into `nxt`
  const MsFast<false> slow;
  const MsFast<true> quick;
  auto visit = [&](int k, const float* cur, float* nxt, int A) {
    if (k < NS) {
      if (kAhead && k + A < NS) load(slow, k + A);
      step(slow, k, cur, (k & 7) == 7 || k == N);
      if (k + A < NS) {
        if (!kAhead) load(slow, k + A);
        blend(slow, k + A, nxt);
      }
    }
  };
  // the same where samples k and k + A exist; sample k ends a run if `close`
  auto visit_full = [&](auto fast, int k, const float* cur, float* nxt, int A, bool close) {
    if (kAhead) load(fast, k + A);
    step(fast, k, cur, close);
    if (!kAhead) load(fast, k + A);
    blend(fast, k + A, nxt);
  };
  const bool fast = TPT == 1 && all_full && w_unit[0] && w_tex[0];  // warp-uniform
  int i = 0;
  if (MX) {
    // two samples per barrier: i and i + 1 from their slabs while i + 2 and
    // i + 3 are built (measured faster for the mixed kernels; the plain ones
    // run faster one sample per barrier). The loops first take the samples
    // whose successors two ahead exist, without bounds tests.
    load(slow, 0);
    blend(slow, 0, sb0);
    if (NS > 1) {
      load(slow, 1);
      blend(slow, 1, sb1);
    }
    __syncthreads();
    if (TPT == 1) {
      for (; i + 5 < NS; i += 4) {
        const bool c = (i & 4) != 0;  // sample i + 3 ends a run of 8
        if (fast) {
          visit_full(quick, i, sb0, sb2, 2, false);
          visit_full(quick, i + 1, sb1, sb3, 2, false);
        } else {
          visit_full(slow, i, sb0, sb2, 2, false);
          visit_full(slow, i + 1, sb1, sb3, 2, false);
        }
        __syncthreads();
        if (fast) {
          visit_full(quick, i + 2, sb2, sb0, 2, false);
          visit_full(quick, i + 3, sb3, sb1, 2, c);
        } else {
          visit_full(slow, i + 2, sb2, sb0, 2, false);
          visit_full(slow, i + 3, sb3, sb1, 2, c);
        }
        __syncthreads();
      }
      for (; i < NS; i += 4) {
        visit(i, sb0, sb2, 2);
        visit(i + 1, sb1, sb3, 2);
        __syncthreads();
        visit(i + 2, sb2, sb0, 2);
        visit(i + 3, sb3, sb1, 2);
        __syncthreads();
      }
    } else {
      for (; i + 3 < NS; i += 2) {
        float* const b0 = slab + (i % kMsSlabs) * slab_stride;
        float* const b1 = slab + ((i + 1) % kMsSlabs) * slab_stride;
        float* const b2 = slab + ((i + 2) % kMsSlabs) * slab_stride;
        float* const b3 = slab + ((i + 3) % kMsSlabs) * slab_stride;
        // (a second copy for `fast` warps spills at this width)
        const bool c = (i & 7) == 6;  // sample i + 1 ends a run of 8
        visit_full(slow, i, b0, b2, 2, false);
        visit_full(slow, i + 1, b1, b3, 2, c);
        __syncthreads();
      }
      for (; i < NS; i += 2) {
        visit(i, slab + (i % kMsSlabs) * slab_stride, slab + ((i + 2) % kMsSlabs) * slab_stride, 2);
        visit(i + 1, slab + ((i + 1) % kMsSlabs) * slab_stride, slab + ((i + 3) % kMsSlabs) * slab_stride, 2);
        __syncthreads();
      }
    }
  } else {
    // one sample per barrier: i from its slab while i + 1 is built (a
    // four-sample body with fixed buffers measured slower here)
    load(slow, 0);
    blend(slow, 0, sb0);
    __syncthreads();
    for (; i < NS; ++i) {
      visit(i, slab + (i % kMsSlabs) * slab_stride, slab + ((i + 1) % kMsSlabs) * slab_stride, 1);
      __syncthreads();
    }
  }
  // outputs: delta multiple scattering and the final table (:91-92)
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    if (has_tex[j]) {
      const size_t t = (size_t)(row0 + c_lr[j]) * W + c_x[j];
      const float3 ms = make_float3(acc[j].s.x - acc[j].c.x, acc[j].s.y - acc[j].c.y, acc[j].s.z - acc[j].c.z);
      a.dms[t] = store_round4(make_float4(ms.x, ms.y, ms.z, 0.f), a.f16);
      const float pr = phase_rayleigh(c_nu[j]);
      if (!MX) {
        const float4 old = a.sc[t];
        a.sc[t] = store_round4(make_float4(ms.x / pr + old.x, ms.y / pr + old.y, ms.z / pr + old.z, 0.f + old.w),
                               a.f16);
      } else {
        // orders accumulate in FP64; the FP32 table is written after the last
        double* s3 = a.sc_acc + 3 * t;
        const float ipr = 1.0f / pr;
        const double sx = s3[0] + (double)(ms.x * ipr), sy = s3[1] + (double)(ms.y * ipr),
                     sz = s3[2] + (double)(ms.z * ipr);
        s3[0] = sx;
        s3[1] = sy;
        s3[2] = sz;
        if (order == a.order) {
          const float w = a.sc[t].w;
          a.sc[t] = store_round4(make_float4((float)sx, (float)sy, (float)sz, w), a.f16);
        }
      }
    }
  }
}

// V = 0: CTAs of kThreads, registers capped for 4 resident CTAs per SM;
// V = 1: for 3; V = 2: CTAs of kMsWideThreads, one per SM; V = 3: CTAs of
// kMsMidThreads, two per SM; V = 4, 5: as 0, 1 for launches whose atmospheres
// all have the fixed layout (ms_fixed_layout), compiled with its sizes.
template <bool MX, int TPT, int V>
__global__ void __launch_bounds__(V == 2 ? kMsWideThreads : (V == 3 ? kMsMidThreads : kThreads),
                                  V == 2 ? 1 : (V == 3 ? 2 : (V == 0 || V == 4 ? 4 : 3)))
    k_multiple(LaunchArgs L) {
  extern __shared__ __align__(16) unsigned char smem[];
  int seg, job, tile;
  int taken = 0;
  constexpr int NTH = V == 2 ? kMsWideThreads : (V == 3 ? kMsMidThreads : kThreads);
  constexpr bool FIX = V >= 4;
  static_assert(!FIX || TPT == 1, "the fixed layout has one texel per thread");
  if (blockDim.x != NTH) return;  // the launch plans give each variant its CTA size
  while (next_item(L, seg, job, tile, taken)) {
    const DevAtmo& a = L.atm[job];
    if (FIX && !ms_fixed_layout(a.W, a.sc_mus)) continue;  // the launch plans never pair these
    tile_multiple<MX, TPT, FIX ? kMsFixedMuS : 0, FIX ? kMsFixedW : 0, NTH>(a, L.order, tile, smem);
  }
}

// ------------------------------------------------------ tile geometry ----
// Host and device agree on tile counts and shared-memory sizes through these.
__host__ __device__ inline int tiles_transmittance(int tr_mu, int tr_r) {
  return (tr_mu * tr_r + kTrTexels - 1) / kTrTexels;
}
__host__ __device__ inline int tiles_rows(int W, int sc_mu, int sc_r) {
  const int R = rows_per_tile(W);
  return (sc_mu * sc_r + R - 1) / R;
}
__host__ __device__ inline int tiles_direct(int ir_mus, int ir_r) { return (ir_mus * ir_r + kThreads - 1) / kThreads; }
__host__ __device__ inline int tiles_density(const DevAtmo& a) {
  return dens_shape(a.sc_r, a.sc_mu, a.sc_mus, a.sc_nu, a.dens_S, a.dens_chunk).tiles;
}
__host__ __device__ inline size_t ss_smem(int W, int steps, int sc_mus, int sc_nu) {
  (void)sc_mus;
  (void)sc_nu;
  const int R = rows_per_tile(W);
  return align16(sizeof(RowGeo) * R) + sizeof(SSRec) * (size_t)R * (steps + 1);
}
__host__ __device__ inline size_t density_smem(const DevAtmo& a, bool two, bool mixed, bool cl) {
  const DensShape d = dens_shape(a.sc_r, a.sc_mu, a.sc_mus, a.sc_nu, a.dens_S, a.dens_chunk);
  return dens_layout(nullptr, a.dens_n, a.sc_nu, a.ir_mus, d.S, d.chunk, two, mixed, cl, nullptr);
}
// Density variants: the occupancy variant (0..2), plus kDensClamped for the
// clamped interval tables.
constexpr int kDensClamped = 3;

}  // namespace fb
