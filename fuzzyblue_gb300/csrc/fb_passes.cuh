// fb_passes.cuh — the six precompute passes as persistent, work-list driven
// kernels (sm_103a). Included by fb_kernels_plain.cu (MX = false, compiled
// with --fmad=false) and fb_kernels_mixed.cu (MX = true).
//
// Launch structure (one launch per pass group, any number of atmospheres):
//   k_transmittance  transmittance.comp                      warp per texel
//   k_single         single_scattering.comp  (segment 0)     CTA per (mu, r) row(s)
//                    direct_irradiance.comp  (segment 1)     thread per texel
//   k_density        scattering_density.comp (segment 0)     CTA per (r, mu_s, mu-chunk)
//                    indirect_irradiance.comp (segment 1)    CTA per texel
//   k_multiple       multiple_scattering.comp                CTA per (mu, r) row(s)
// CTAs take work items from a global atomic counter; an item is a tile of one
// atmosphere, located by binary search over per-atmosphere item offsets.
#pragma once

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

struct LaunchArgs {
  const DevAtmo* atm;
  Segment seg[2];
  int nseg;
  int order;  // k_density: order n computed (indirect irradiance integrates n-1)
  unsigned int* counter;
};

__device__ __forceinline__ bool next_item(const LaunchArgs& L, int& seg, int& job, int& tile) {
  __shared__ int s_item;
  __syncthreads();
  if (threadIdx.x == 0) s_item = (int)atomicAdd(L.counter, 1u);
  __syncthreads();
  int item = s_item;
  const int total = L.seg[0].total + (L.nseg > 1 ? L.seg[1].total : 0);
  if (item >= total) return false;
  seg = 0;
  if (item >= L.seg[0].total) {
    seg = 1;
    item -= L.seg[0].total;
  }
  const Segment& S = L.seg[seg];
  int lo = 0, hi = S.njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (S.off[mid] <= item) lo = mid; else hi = mid - 1;
  }
  job = S.job[lo];
  tile = item - S.off[lo];
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
// samples of the three optical lengths, then reduce with shuffles.
template <bool MX> __device__ void tile_transmittance(const DevAtmo& a, int tile) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = tile * (kThreads / 32) + warp;
  if (t >= a.tr_mu * a.tr_r) return;
  const int i = t % a.tr_mu, j = t / a.tr_mu;
  const int N = a.tr_steps;
  float sR, sM, sA;
  if (!MX) {
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
    Geo64 G;
    G.init(a);
    double x_mu = double(i) / double(a.tr_mu - 1), x_r = double(j) / double(a.tr_r - 1);
    double rho = G.H * x_r, q = rho * rho, r = G.radius(q);
    double d_min = (G.H2 - q) / (G.T + r), d_max = rho + G.H;
    double d = d_min + x_mu * (d_max - d_min);
    double s = d == 0.0 ? r : gclamp((G.H2 - q - d * d) / (2.0 * d), -r, r);
    const double dx = G.dist_top(q, s) / double(N);
    const double two_s = 2.0 * s, R2 = G.R * G.R;
    const float Rf = a.bottom;
    float cR = 0.f, cM = 0.f, cA = 0.f;
    sR = sM = sA = 0.0f;
    for (int k = lane; k <= N; k += 32) {
      double d_k = double(k) * dx;
      double q_k = fma(d_k, two_s + d_k, q);  // r_k^2 - R^2, no cancellation
      float r_k = sqrtf((float)(q_k + R2));
      // every ray of this table stays at or above the ground: a negative
      // altitude here is rounding at a tangent sample
      float h = gmax((float)q_k / (r_k + Rf), 0.0f);
      float w = (k == 0 || k == N) ? 0.5f : 1.0f;
      Kahan3::add1(sR, cR, profile_density(a.ray_d, h) * w);
      Kahan3::add1(sM, cM, profile_density(a.mie_d, h) * w);
      Kahan3::add1(sA, cA, profile_density(a.abs_d, h) * w);
    }
    double dR = warp_sum((double)sR - (double)cR), dM = warp_sum((double)sM - (double)cM),
           dA = warp_sum((double)sA - (double)cA);
    sR = (float)(dR * dx);
    sM = (float)(dM * dx);
    sA = (float)(dA * dx);
  }
  if (lane == 0) {
    float4 o;
    o.x = expf(-(a.rayleigh[0] * sR + a.mie_ext[0] * sM + a.absorption[0] * sA));
    o.y = expf(-(a.rayleigh[1] * sR + a.mie_ext[1] * sM + a.absorption[1] * sA));
    o.z = expf(-(a.rayleigh[2] * sR + a.mie_ext[2] * sM + a.absorption[2] * sA));
    o.w = 1.0f;
    a.tr[t] = o;
  }
}

template <bool MX> __global__ void __launch_bounds__(kThreads) k_transmittance(LaunchArgs L) {
  int seg, job, tile;
  while (next_item(L, seg, job, tile)) tile_transmittance<MX>(L.atm[job], tile);
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

// ===================================================== row-tile helpers ===
// Single and multiple scattering run one CTA over one or more (mu, r) rows of
// the packed table: every texel of a row shares r, mu and the ground flag, so
// the ray geometry of each trapezoid sample is computed once per row.
struct RowInfo {
  float r, mu, dx, rr, two_r_mu, r_mu;  // PLAIN: the reference's float values
  double q, s, dxd, one_m_mu2, mud;     // MIXED: FP64 ray state
  int ground;
  int y, z;
};

template <bool MX> __device__ __forceinline__ void row_info(const DevAtmo& a, int row, int steps, RowInfo& o) {
  o.y = row % a.sc_mu;
  o.z = row / a.sc_mu;
  if (!MX) {
    Geo32 G;
    G.init(a);
    float r, mu, mu_s, nu;
    bool g;
    decode_texel32(a, G, 0, (uint32_t)o.y, (uint32_t)o.z, r, mu, mu_s, nu, g);
    o.r = r;
    o.mu = mu;
    o.ground = g;
    o.dx = (g ? G.dist_bottom(r, mu) : G.dist_top(r, mu)) / float(steps);
    o.rr = r * r;
    o.two_r_mu = 2.0f * r * mu;
    o.r_mu = r * mu;
  } else {
    Geo64 G;
    G.init(a);
    TexelParams p = decode_texel64(a, G, 0, (uint32_t)o.y, (uint32_t)o.z);
    o.q = p.q;
    o.s = p.s;
    o.r = (float)p.r;
    o.mu = (float)p.mu;
    o.ground = p.ground;
    o.dxd = (p.ground ? G.dist_bottom(p.q, p.s) : G.dist_top(p.q, p.s)) / double(steps);
    o.dx = (float)o.dxd;
    o.one_m_mu2 = (1.0 - p.mu) * (1.0 + p.mu);
    o.mud = p.mu;
  }
}

// MIXED: FP64 decode of the mu_s coordinate (scattering.h:102-111) and of the
// raw nu coordinate (scattering.h:113), tabulated per column class.
__device__ __forceinline__ void decode_mus_nu64(const DevAtmo& a, const Geo64& G, int x, double& mu_s,
                                                double& nu_raw) {
  const double nmus = double(a.sc_mus);
  double fx = frag_from_texel_d((uint32_t)x, (uint32_t)a.W);
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

// Column tables of a row tile (MIXED only): mu_s and 1 - mu_s^2 per mu_s index,
// raw nu per nu index.
struct ColTabs {
  double2* mus;  // sc_mus entries: (mu_s, 1 - mu_s^2)
  double* nu;    // sc_nu entries: raw nu
};
__device__ __forceinline__ void build_cols(const DevAtmo& a, ColTabs c) {
  Geo64 G;
  G.init(a);
  for (int k = threadIdx.x; k < a.sc_mus + a.sc_nu; k += kThreads) {
    double mu_s, nu;
    if (k < a.sc_mus) {
      decode_mus_nu64(a, G, k, mu_s, nu);
      c.mus[k] = make_double2(mu_s, (1.0 - mu_s) * (1.0 + mu_s));
    } else {
      const int n = k - a.sc_mus;
      decode_mus_nu64(a, G, n * a.sc_mus, mu_s, nu);
      c.nu[n] = nu;
    }
  }
}

// mu_s, nu (clamped to the range allowed by mu and mu_s, scattering.h:134-136)
// and r*mu_s of texel x of a row.
template <bool MX>
__device__ __forceinline__ void texel_mus_nu(const DevAtmo& a, const RowInfo& ri, const ColTabs& c, int x,
                                             float& mu_s, float& nu, float& r_mu_s) {
  if (!MX) {
    Geo32 G;
    G.init(a);
    float r, mu;
    bool g;
    decode_texel32(a, G, (uint32_t)x, (uint32_t)ri.y, (uint32_t)ri.z, r, mu, mu_s, nu, g);
    r_mu_s = ri.r * mu_s;
  } else {
    // the clamp in FP64 (scattering.h:134-136)
    const double2 ms = c.mus[x % a.sc_mus];
    const double sq = sqrt(ri.one_m_mu2 * ms.y), mm = ri.mud * ms.x;
    mu_s = (float)ms.x;
    nu = (float)(mm + gclamp(c.nu[x / a.sc_mus] - mm, -sq, sq));
    r_mu_s = ri.r * mu_s;
  }
}

// ============================================================ S: single ===
struct SSRec {
  float d, r_d, rr_d, dmin, span, tvx, tvy, tvz, rho_r, rho_m, w, cos_h, lo, hi, fy, e;
  int y0, y1;
};

__host__ __device__ inline int rows_per_tile(int W) { return W >= kThreads ? 1 : kThreads / W; }

template <bool MX>
__device__ void tile_single(const DevAtmo& a, int tile, unsigned char* smem) {
  const int W = a.W, nrows = a.sc_mu * a.sc_r;
  const int R = rows_per_tile(W);
  const int row0 = tile * R;
  const int nrow = min(R, nrows - row0);
  const int N = a.ss_steps, NS = N + 1;
  RowInfo* rows = (RowInfo*)smem;
  SSRec* rec = (SSRec*)(rows + R);
  ColTabs cols;
  cols.mus = (double2*)(((uintptr_t)(rec + (size_t)R * NS) + 15) & ~(uintptr_t)15);
  cols.nu = (double*)(cols.mus + a.sc_mus);
  const int tid = threadIdx.x;
  if (tid < nrow) row_info<MX>(a, row0 + tid, N, rows[tid]);
  if (MX) build_cols(a, cols);
  __syncthreads();
  // Per (row, sample): the view ray point, the transmittance to it, the
  // densities there and the parts of the sun lookup that depend on it only.
  for (int k = tid; k < nrow * NS; k += kThreads) {
    const RowInfo& ri = rows[k / NS];
    const int i = k % NS;
    SSRec& o = rec[k];
    o.w = (i == 0 || i == N) ? 0.5f : 1.0f;
    float3 tv;
    if (!MX) {
      Geo32 G;
      G.init(a);
      float v;
      // single_scattering.comp:16-23
      float d = float(i) * ri.dx;
      float r_d = G.clamp_radius(sqrtf(d * d + ri.two_r_mu * d + ri.rr));
      tv = G.tr_segment(a, ri.r, ri.mu, d, ri.ground);
      o.d = d;
      o.r_d = r_d;
      o.rr_d = r_d * r_d;
      float h = r_d - G.R;
      o.rho_r = profile_density(a.ray_d, h);
      o.rho_m = profile_density(a.mie_d, h);
      // transmittance.h:63-74 and :7-24
      float sin_h = G.R / r_d;
      o.cos_h = -sqrtf(gmax(1.0f - sin_h * sin_h, 0.0f));
      o.lo = -sin_h * a.sun_radius;
      o.hi = sin_h * a.sun_radius;
      float rho = safe_sqrt(r_d * r_d - G.R * G.R);
      o.dmin = G.T - r_d;
      o.span = (rho + G.H) - o.dmin;
      v = coord_from_unit(rho / G.H, a.tr_r);
      o.e = 0.f;
      const Axis ay = make_axis(v, a.tr_r);
      o.y0 = ay.i0;
      o.y1 = ay.i1;
      o.fy = ay.f;
    } else {
      Geo64 G;
      G.init(a);
      double d = double(i) * ri.dxd;
      double q = ri.q + d * (2.0 * ri.s + d), s = ri.s + d;
      G.clamp_point(q, s);
      double r_d = G.radius(q);
      tv = G.tr_segment(a, ri.q, ri.s, d, ri.ground);
      o.d = (float)d;
      o.r_d = (float)r_d;
      o.rr_d = 0.f;
      float h = (float)(q / (r_d + G.R));
      o.rho_r = profile_density(a.ray_d, h);
      o.rho_m = profile_density(a.mie_d, h);
      double rho = sqrt(q);
      o.cos_h = (float)(-rho / r_d);
      double sin_h = G.R / r_d;
      o.lo = (float)(-sin_h * a.sun_radius);
      o.hi = (float)(sin_h * a.sun_radius);
      o.e = (float)(G.H2 - q);  // T^2 - r_d^2
      const double dmin = (G.H2 - q) / (G.T + r_d);
      o.dmin = (float)dmin;
      o.span = (float)(rho + G.H - dmin);
      const Axis ay = axis_texel(rho / G.H * double(a.tr_r - 1), a.tr_r);
      o.y0 = ay.i0;
      o.y1 = ay.i1;
      o.fy = ay.f;
    }
    o.tvx = tv.x;
    o.tvy = tv.y;
    o.tvz = tv.z;
  }
  __syncthreads();
  const float TT = a.top * a.top;
  for (int k = tid; k < nrow * W; k += kThreads) {
    const int lr = k / W, x = k % W;
    const RowInfo& ri = rows[lr];
    float mu_s, nu, r_mu_s;
    texel_mus_nu<MX>(a, ri, cols, x, mu_s, nu, r_mu_s);
    const SSRec* rr = rec + lr * NS;
    Kahan3 ray, mie;
    ray.init();
    mie.init();
    for (int i = 0; i < NS; ++i) {
      const SSRec& o = rr[i];
      float x_mu, mu_s_d;
      if (!MX) {
        // single_scattering.comp:17, transmittance.h:63-74
        mu_s_d = clamp_cosine((r_mu_s + o.d * nu) / o.r_d);
        float disc = o.rr_d * (mu_s_d * mu_s_d - 1.0f) + TT;
        float dt = gmax(-o.r_d * mu_s_d + safe_sqrt(disc), 0.0f);
        x_mu = (dt - o.dmin) / o.span;
      } else {
        // distance to the top from (r_d, mu_s_d): T^2 - r_d^2 + (r_d mu_s_d)^2
        // under the root, rationalised when the ray points up.
        float s_d = gclamp(fmaf(o.d, nu, r_mu_s), -o.r_d, o.r_d);
        mu_s_d = s_d / o.r_d;
        float root = sqrtf(fmaf(s_d, s_d, o.e));
        float dt = s_d > 0.0f ? o.e / (s_d + root) : root - s_d;
        x_mu = (dt - o.dmin) / o.span;
      }
      const float sfac = smoothstepf(o.lo, o.hi, mu_s_d - o.cos_h);
      const Axis ax = MX ? axis_texel(x_mu * float(a.tr_mu - 1), a.tr_mu)
                         : make_axis(coord_from_unit(x_mu, a.tr_mu), a.tr_mu);
      Axis ay;
      ay.i0 = o.y0;
      ay.i1 = o.y1;
      ay.f = o.fy;
      const float3 ts = fetch2(a.tr, a.tr_mu, ax, ay) * sfac;
      const float3 t3 = make_float3(o.tvx, o.tvy, o.tvz) * ts;
      const float3 ri_ = t3 * o.rho_r, mi_ = t3 * o.rho_m;
      if (!MX) {
        ray.s = ray.s + ri_ * o.w;
        mie.s = mie.s + mi_ * o.w;
      } else {
        ray.add(ri_ * o.w);
        mie.add(mi_ * o.w);
      }
    }
    const float dx = ri.dx;
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

template <bool MX> __global__ void __launch_bounds__(kThreads) k_single(LaunchArgs L) {
  extern __shared__ __align__(16) unsigned char smem[];
  int seg, job, tile;
  while (next_item(L, seg, job, tile)) {
    if (seg == 0) tile_single<MX>(L.atm[job], tile, smem);
    else tile_direct<MX>(L.atm[job], tile);
  }
}

// ============================================================ density ===
// scattering_density.comp:10-155 for a tile of texels sharing (r, mu_s): all
// 4D lookups of the tile hit the previous order's table at the tile's r and
// mu_s and at one of the 16 theta rows, so the table is first reduced by
// trilinear interpolation to P[theta][nu slice]; each of the 512 directions of
// a texel is then a linear blend of two P entries.
struct DensTheta {
  float cos_t, domega, dg, tgx, tgy, tgz;
  int ground, pad;
};

struct DensLayout {
  DensTheta* th;
  Axis* tay;    // theta -> mu axis
  Axis* kax;    // nu slice -> x axis
  float2* dir;  // (cos phi sin theta, sin phi sin theta) per direction
  float4* gn;   // ground normal per direction (ground thetas)
  float4* P;    // reduced table(s)
  float4* irow; // two irradiance rows at the ground
  double2* ymu;  // MIXED: per mu row (mu, 1 - mu^2)
  double* nuraw; // MIXED: raw nu per nu index
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t dens_layout(unsigned char* base, int dens_n, int sc_nu, int ir_mus, int chunk,
                                              bool two, DensLayout* L) {
  const int NT = dens_n, ND = 2 * dens_n * dens_n, NK = sc_nu + 2;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align16(o + bytes);
    return at;
  };
  size_t o_th = take(sizeof(DensTheta) * NT), o_tay = take(sizeof(Axis) * NT), o_kax = take(sizeof(Axis) * NK);
  size_t o_dir = take(sizeof(float2) * ND), o_gn = take(sizeof(float4) * ND);
  size_t o_P = take(sizeof(float4) * (size_t)NT * NK * (two ? 2 : 1)), o_irow = take(sizeof(float4) * 2 * ir_mus);
  size_t o_ymu = take(sizeof(double2) * chunk), o_nu = take(sizeof(double) * sc_nu);
  if (L) {
    L->th = (DensTheta*)(base + o_th);
    L->tay = (Axis*)(base + o_tay);
    L->kax = (Axis*)(base + o_kax);
    L->dir = (float2*)(base + o_dir);
    L->gn = (float4*)(base + o_gn);
    L->P = (float4*)(base + o_P);
    L->irow = (float4*)(base + o_irow);
    L->ymu = (double2*)(base + o_ymu);
    L->nuraw = (double*)(base + o_nu);
  }
  return o;
}

template <bool MX>
__device__ void tile_density(const DevAtmo& a, int order, int chunk, int tile, unsigned char* smem) {
  const int NT = a.dens_n, NP = 2 * NT, ND = NT * NP;
  const int NNU = a.sc_nu, NK = NNU + 2;  // slices -1 .. NNU
  const int nchunks = (a.sc_mu + chunk - 1) / chunk;
  const int zi = tile / (a.sc_mus * nchunks);
  const int rem = tile % (a.sc_mus * nchunks);
  const int si = rem / nchunks, ci = rem % nchunks;
  const int y_begin = ci * chunk, y_end = min(a.sc_mu, y_begin + chunk);
  const bool two = (order - 1) == 1;  // order 2 reads the single Rayleigh/Mie tables
  const int tid = threadIdx.x;
  DensLayout S;
  dens_layout(smem, NT, NNU, a.ir_mus, chunk, two, &S);

  __shared__ Axis s_az, s_irx;
  __shared__ float s_r, s_mu_s, s_ums;
  __shared__ double s_q, s_ymus, s_musd, s_omus2;
  if (tid == 0) {
    float r, mu_s, u_ms;
    if (!MX) {
      Geo32 G;
      G.init(a);
      float mu, nu;
      bool g;
      decode_texel32(a, G, (uint32_t)si, 0u, (uint32_t)zi, r, mu, mu_s, nu, g);
      s_az = make_axis(G.u_r(a, r), a.sc_r);
      u_ms = G.u_mu_s(a, mu_s);
      s_omus2 = 0.0;
      s_musd = mu_s;
    } else {
      Geo64 G;
      G.init(a);
      TexelParams tp = decode_texel64(a, G, (uint32_t)si, 0u, (uint32_t)zi);
      r = (float)tp.r;
      mu_s = (float)tp.mu_s;
      s_q = tp.q;
      s_az = axis_texel(G.sc_r_texel(a, tp.q), a.sc_r);
      s_ymus = G.mus_unit(a, tp.mu_s);
      u_ms = 0.f;
      s_omus2 = (1.0 - tp.mu_s) * (1.0 + tp.mu_s);
      s_musd = tp.mu_s;
    }
    s_r = r;
    s_mu_s = mu_s;
    s_ums = u_ms;
    // irradiance at the ground: irradiance.h:20-30 with r = bottom (x_r = 0)
    s_irx = MX ? axis_texel(0.0f, a.ir_r)
               : make_axis(coord_from_unit((a.bottom - a.bottom) / (a.top - a.bottom), a.ir_r), a.ir_r);
  }
  __syncthreads();
  const float r = s_r;
  const Axis az = s_az;
  // --- per theta: ground flag, ground distance and transmittance, mu axis
  if (tid < NT) {
    const int l = tid;
    DensTheta& o = S.th[l];
    if (!MX) {
      Geo32 G;
      G.init(a);
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
      S.tay[l] = make_axis(G.u_mu(a, r, ct, g), a.sc_mu);
    } else {
      Geo64 G;
      G.init(a);
      const double dtheta = kPiD / double(NT), dphi = kPiD / double(NT);
      const double theta = (double(l) + 0.5) * dtheta;
      const double ct = cos(theta);
      const double q = s_q, s = G.radius(q) * ct;
      const bool g = G.hits_ground(q, s);
      float3 tg = make_float3(0.f, 0.f, 0.f);
      double dg = 0.0;
      if (g) {
        dg = G.dist_bottom(q, s);
        tg = G.tr_segment(a, q, s, dg, true) * ld3(a.albedo) * (float)(1.0 / kPiD);
      }
      o.cos_t = (float)ct;
      o.domega = (float)(dtheta * dphi * sin(theta));
      o.dg = (float)dg;
      o.ground = g;
      o.tgx = tg.x;
      o.tgy = tg.y;
      o.tgz = tg.z;
      S.tay[l] = axis_texel(G.sc_mu_texel(a, q, s, g), a.sc_mu);
    }
  }
  if (tid >= 64 && tid < 64 + NK) {
    const int k = tid - 64;
    S.kax[k] = MX ? axis_texel(double(k - 1) * a.sc_mus + s_ymus * double(a.sc_mus - 1), a.W)
                  : make_axis((float(k - 1) + s_ums) / float(NNU), a.W);
  }
  if (MX && tid >= 128) {
    Geo64 G;
    G.init(a);
    const int nk = (y_end - y_begin) + NNU;
    for (int k = tid - 128; k < nk; k += kThreads - 128) {
      if (k < y_end - y_begin) {
        TexelParams tp = decode_texel64(a, G, (uint32_t)si, (uint32_t)(y_begin + k), (uint32_t)zi);
        S.ymu[k] = make_double2(tp.mu, (1.0 - tp.mu) * (1.0 + tp.mu));
      } else {
        const int n = k - (y_end - y_begin);
        double mu_s, nu;
        decode_mus_nu64(a, G, n * a.sc_mus + si, mu_s, nu);
        S.nuraw[n] = nu;
      }
    }
  }
  __syncthreads();
  // --- reduced table P[theta][slice], directions, ground normals, ground irradiance
  {
    const float4* src0 = two ? a.dr : a.dms;
    for (int k = tid; k < NT * NK; k += kThreads) {
      const int l = k / NK, s = k % NK;
      const float3 v = fetch3(src0, a.W, a.sc_mu, S.kax[s], S.tay[l], az);
      S.P[k] = make_float4(v.x, v.y, v.z, 0.f);
      if (two) {
        const float3 m = fetch3(a.dm, a.W, a.sc_mu, S.kax[s], S.tay[l], az);
        S.P[NT * NK + k] = make_float4(m.x, m.y, m.z, 0.f);
      }
    }
    const float dtheta = kPiF / float(NT), dphi = kPiF / float(NT);
    for (int k = tid; k < ND; k += kThreads) {
      const int l = k / NP, m = k % NP;
      const float theta = (float(l) + 0.5f) * dtheta;
      const float st = sinf(theta);
      const float phi = (float(m) + 0.5f) * dphi;
      const float cx = cosf(phi) * st, cy = sinf(phi) * st;
      S.dir[k] = make_float2(cx, cy);
      // normalize(zenith * r + omega_i * distance_to_ground)
      const float dg = S.th[l].dg, ct = S.th[l].cos_t;
      const float gx = cx * dg, gy = cy * dg, gz = r + ct * dg;
      const float len = sqrtf(gx * gx + gy * gy + gz * gz);
      S.gn[k] = make_float4(gx / len, gy / len, gz / len, 0.f);
    }
    const float4* E = a.dirr[order & 1];  // irradiance of order n-2
    for (int k = tid; k < 2 * a.ir_mus; k += kThreads) {
      const int row = k < a.ir_mus ? s_irx.i0 : s_irx.i1;
      S.irow[k] = E[row * a.ir_mus + (k % a.ir_mus)];
    }
  }
  __syncthreads();

  // --- texels of the tile: (nu, mu) pairs at the tile's (r, mu_s)
  const float h0 = r - a.bottom;
  const float rho_r = profile_density(a.ray_d, h0), rho_m = profile_density(a.mie_d, h0);
  const float3 kR = make_float3(a.rayleigh[0] * rho_r, a.rayleigh[1] * rho_r, a.rayleigh[2] * rho_r);
  const float3 kM = make_float3(a.mie_sca[0] * rho_m, a.mie_sca[1] * rho_m, a.mie_sca[2] * rho_m);
  const float g = a.g;
  const float kmie = 3.0f / (8.0f * kPiF) * (1.0f - g * g) / (2.0f + g * g);
  const float kray = 3.0f / (16.0f * kPiF);
  const float g1 = 1.0f + g * g, g2 = 2.0f * g;
  const float fnu = float(NNU - 1);
  const Axis irx = s_irx;
  const int ntex = (y_end - y_begin) * NNU;
  for (int k = tid; k < ntex; k += kThreads) {
    const int nu_i = k % NNU, y = y_begin + k / NNU;
    const int x = nu_i * a.sc_mus + si;
    float mu, mu_s, ox, sx, sy;
    if (!MX) {
      Geo32 G;
      G.init(a);
      float rr, nu;
      bool gg;
      decode_texel32(a, G, (uint32_t)x, (uint32_t)y, (uint32_t)zi, rr, mu, mu_s, nu, gg);
      // scattering_density.comp:28-32
      ox = sqrtf(1.0f - mu * mu);
      sx = ox == 0.0f ? 0.0f : (nu - mu * mu_s) / ox;
      sy = sqrtf(gmax(1.0f - sx * sx - mu_s * mu_s, 0.0f));
    } else {
      // The same frame in FP64, with nu clamped (scattering.h:134-136) as
      // delta = nu - mu mu_s in [-sq, sq], sq = sqrt((1-mu^2)(1-mu_s^2)), and
      // sun_y^2 = (sq - delta)(sq + delta) / (1 - mu^2): exactly 0 when the sun
      // lies in the view plane, where 1 - sun_x^2 - mu_s^2 would cancel.
      const double2 ym = S.ymu[y - y_begin];
      const double mud = ym.x, om = ym.y, musd = s_musd;
      const double sq = sqrt(om * s_omus2), mm = mud * musd;
      const double delta = gclamp(S.nuraw[nu_i] - mm, -sq, sq);
      double sxd, syd;
      if (om == 0.0) {
        sxd = 0.0;
        syd = sqrt(gmax(s_omus2, 0.0));
      } else {
        sxd = delta / sqrt(om);
        syd = sqrt(gmax((sq - delta) * (sq + delta), 0.0) / om);
      }
      mu = (float)mud;
      mu_s = (float)musd;
      ox = (float)sqrt(om);
      sx = (float)sxd;
      sy = (float)syd;
    }
    Kahan3 acc;
    acc.init();
    for (int l = 0; l < NT; ++l) {
      const DensTheta t = S.th[l];
      const float4* Pl = S.P + l * NK;
      const float4* Ml = S.P + NT * NK + l * NK;
      const float mus_ct = mu_s * t.cos_t, mu_ct = mu * t.cos_t;
      Kahan3 accl;
      accl.init();
      for (int m = 0; m < NP; ++m) {
        const float2 c = S.dir[l * NP + m];
        // incident radiance of order n-1 (scattering.h:139-179)
        const float nu1 = sx * c.x + sy * c.y + mus_ct;
        const float tcx = (nu1 + 1.0f) / 2.0f * fnu;
        float fk = floorf(tcx);
        const float lf = tcx - fk;
        fk = fminf(fmaxf(fk, -1.0f), float(NNU - 1));
        const int ks = (int)fk + 1;
        float3 inc;
        if (two) {
          const float4 r0 = Pl[ks], r1 = Pl[ks + 1], m0 = Ml[ks], m1 = Ml[ks + 1];
          const float pr = kray * (1.0f + nu1 * nu1);
          const float rs = rsqrtf(g1 - g2 * nu1);
          const float pm = kmie * (1.0f + nu1 * nu1) * (rs * rs * rs);
          inc.x = fmaf(r1.x - r0.x, lf, r0.x) * pr + fmaf(m1.x - m0.x, lf, m0.x) * pm;
          inc.y = fmaf(r1.y - r0.y, lf, r0.y) * pr + fmaf(m1.y - m0.y, lf, m0.y) * pm;
          inc.z = fmaf(r1.z - r0.z, lf, r0.z) * pr + fmaf(m1.z - m0.z, lf, m0.z) * pm;
        } else {
          const float4 r0 = Pl[ks], r1 = Pl[ks + 1];
          inc.x = fmaf(r1.x - r0.x, lf, r0.x);
          inc.y = fmaf(r1.y - r0.y, lf, r0.y);
          inc.z = fmaf(r1.z - r0.z, lf, r0.z);
        }
        if (t.ground) {
          // ground bounce: irradiance of order n-2 at the ground point
          const float4 nrm = S.gn[l * NP + m];
          const float mg = nrm.x * sx + nrm.y * sy + nrm.z * mu_s;
          const Axis ax = MX ? axis_texel((mg * 0.5f + 0.5f) * float(a.ir_mus - 1), a.ir_mus)
                             : make_axis(coord_from_unit(mg * 0.5f + 0.5f, a.ir_mus), a.ir_mus);
          const float4 e00 = S.irow[ax.i0], e10 = S.irow[ax.i1];
          const float4 e01 = S.irow[a.ir_mus + ax.i0], e11 = S.irow[a.ir_mus + ax.i1];
          const float w00 = (1.f - ax.f) * (1.f - irx.f), w10 = ax.f * (1.f - irx.f);
          const float w01 = (1.f - ax.f) * irx.f, w11 = ax.f * irx.f;
          inc.x = fmaf(t.tgx, w00 * e00.x + w10 * e10.x + w01 * e01.x + w11 * e11.x, inc.x);
          inc.y = fmaf(t.tgy, w00 * e00.y + w10 * e10.y + w01 * e01.y + w11 * e11.y, inc.y);
          inc.z = fmaf(t.tgz, w00 * e00.z + w10 * e10.z + w01 * e01.z + w11 * e11.z, inc.z);
        }
        // phase functions of the scattering angle omega . omega_i
        const float nu2 = ox * c.x + mu_ct;
        const float pr2 = kray * (1.0f + nu2 * nu2);
        const float rs2 = rsqrtf(g1 - g2 * nu2);
        const float pm2 = kmie * (1.0f + nu2 * nu2) * (rs2 * rs2 * rs2);
        float3 v;
        v.x = inc.x * fmaf(kR.x, pr2, kM.x * pm2);
        v.y = inc.y * fmaf(kR.y, pr2, kM.y * pm2);
        v.z = inc.z * fmaf(kR.z, pr2, kM.z * pm2);
        if (!MX) {
          accl.s.x += v.x;
          accl.s.y += v.y;
          accl.s.z += v.z;
        } else {
          accl.add(v);
        }
      }
      const float3 part = make_float3(accl.s.x - accl.c.x, accl.s.y - accl.c.y, accl.s.z - accl.c.z);
      if (!MX) acc.s = acc.s + part * t.domega;
      else acc.add(part * t.domega);
    }
    const float3 o = make_float3(acc.s.x - acc.c.x, acc.s.y - acc.c.y, acc.s.z - acc.c.z);
    const size_t t = ((size_t)zi * a.sc_mu + y) * a.W + x;
    a.dens[t] = store_round4(make_float4(o.x, o.y, o.z, 0.f), a.f16);
  }
}

// ================================================== indirect irradiance ===
// indirect_irradiance.comp:10-74. One CTA per irradiance texel: the CTA
// reduces the order's table to P[theta][nu slice] at its (r, mu_s), threads
// split the 16 x 64 directions, and warp shuffles plus one shared-memory step
// sum them.
__host__ __device__ inline size_t indirect_smem(int irr_n, int sc_nu, bool one) {
  return sizeof(float4) * (size_t)(irr_n / 2) * (sc_nu + 2) * (one ? 2 : 1) + sizeof(double) * 3 * (kThreads / 32);
}

template <bool MX>
__device__ void tile_indirect(const DevAtmo& a, int order, int tile, unsigned char* smem) {
  const int ord = order - 1;  // order integrated (the push constant order-1)
  const bool one = ord == 1;
  const int NT = a.irr_n / 2, NP = 2 * a.irr_n;
  const int NNU = a.sc_nu, NK = NNU + 2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float4* P = (float4*)smem;
  double* red = (double*)(P + (size_t)NT * NK * (one ? 2 : 1));
  const int t = tile;
  const int i = t % a.ir_mus, j = t / a.ir_mus;
  float r, mu_s, u_ms = 0.f;
  Axis az;
  double qd = 0.0, ymus = 0.0;
  if (!MX) {
    Geo32 G;
    G.init(a);
    const float x_mu_s = float(i) / float(a.ir_mus - 1), x_r = float(j) / float(a.ir_r - 1);
    r = G.R + x_r * (G.T - G.R);
    mu_s = clamp_cosine(2.0f * x_mu_s - 1.0f);
    az = make_axis(G.u_r(a, r), a.sc_r);
    u_ms = G.u_mu_s(a, mu_s);
  } else {
    Geo64 G;
    G.init(a);
    const double x_mu_s = double(i) / double(a.ir_mus - 1), x_r = double(j) / double(a.ir_r - 1);
    const double h = x_r * (G.T - G.R), rd = G.R + h;
    qd = h * (rd + G.R);
    r = (float)rd;
    const double mus = clamp_cosine(2.0 * x_mu_s - 1.0);
    mu_s = (float)mus;
    az = axis_texel(G.sc_r_texel(a, qd), a.sc_r);
    ymus = G.mus_unit(a, mus);
  }
  const float4* src0 = one ? a.dr : a.dms;
  const float dthetaf = kPiF / float(a.irr_n), dphif = kPiF / float(a.irr_n);
  for (int k = tid; k < NT * NK; k += kThreads) {
    const int l = k / NK, s = k % NK;
    Axis ay, ax;
    if (!MX) {
      Geo32 G;
      G.init(a);
      const float ct = cosf((float(l) + 0.5f) * dthetaf);
      ay = make_axis(G.u_mu(a, r, ct, false), a.sc_mu);
      ax = make_axis((float(s - 1) + u_ms) / float(NNU), a.W);
    } else {
      Geo64 G;
      G.init(a);
      const double ct = cos((double(l) + 0.5) * (kPiD / double(a.irr_n)));
      ay = axis_texel(G.sc_mu_texel(a, qd, G.radius(qd) * ct, false), a.sc_mu);
      ax = axis_texel(double(s - 1) * a.sc_mus + ymus * double(a.sc_mus - 1), a.W);
    }
    const float3 v = fetch3(src0, a.W, a.sc_mu, ax, ay, az);
    P[k] = make_float4(v.x, v.y, v.z, 0.f);
    if (one) {
      const float3 m = fetch3(a.dm, a.W, a.sc_mu, ax, ay, az);
      P[NT * NK + k] = make_float4(m.x, m.y, m.z, 0.f);
    }
  }
  __syncthreads();
  const float sxs = sqrtf(1.0f - mu_s * mu_s);
  const float g = a.g;
  const float kmie = 3.0f / (8.0f * kPiF) * (1.0f - g * g) / (2.0f + g * g);
  const float kray = 3.0f / (16.0f * kPiF);
  const float g1 = 1.0f + g * g, g2 = 2.0f * g;
  const float fnu = float(NNU - 1);
  Kahan3 acc;
  acc.init();
  for (int k = tid; k < NT * NP; k += kThreads) {
    const int l = k / NP, m = k % NP;
    const float theta = (float(l) + 0.5f) * dthetaf, phi = (float(m) + 0.5f) * dphif;
    const float st = sinf(theta);
    const float cx = cosf(phi) * st, ct = cosf(theta);
    const float dom = dthetaf * dphif * st;
    // nu = dot(omega, omega_s) with omega_s = (sqrt(1 - mu_s^2), 0, mu_s)
    const float nu = cx * sxs + ct * mu_s;
    const float tcx = (nu + 1.0f) / 2.0f * fnu;
    float fk = floorf(tcx);
    const float lf = tcx - fk;
    fk = fminf(fmaxf(fk, -1.0f), float(NNU - 1));
    const int ks = (int)fk + 1;
    const float4* Pl = P + l * NK;
    float3 L;
    if (one) {
      const float4* Ml = P + NT * NK + l * NK;
      const float4 r0 = Pl[ks], r1 = Pl[ks + 1], m0 = Ml[ks], m1 = Ml[ks + 1];
      const float pr = kray * (1.0f + nu * nu);
      const float rs = rsqrtf(g1 - g2 * nu);
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
    if (!MX) {
      acc.s.x += v.x;
      acc.s.y += v.y;
      acc.s.z += v.z;
    } else {
      acc.add(v);
    }
  }
  // reduction: warp shuffles, then the 8 warp sums in FP64 through shared memory
  double sx = warp_sum((double)acc.s.x - (double)acc.c.x);
  double sy = warp_sum((double)acc.s.y - (double)acc.c.y);
  double sz = warp_sum((double)acc.s.z - (double)acc.c.z);
  if (lane == 0) {
    red[3 * warp] = sx;
    red[3 * warp + 1] = sy;
    red[3 * warp + 2] = sz;
  }
  __syncthreads();
  if (tid == 0) {
    double tx = 0, ty = 0, tz = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      tx += red[3 * w];
      ty += red[3 * w + 1];
      tz += red[3 * w + 2];
    }
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

template <bool MX> __global__ void __launch_bounds__(kThreads) k_density(LaunchArgs L) {
  extern __shared__ __align__(16) unsigned char smem[];
  int seg, job, tile;
  while (next_item(L, seg, job, tile)) {
    if (seg == 0) tile_density<MX>(L.atm[job], L.order, L.atm[job].dens_chunk, tile, smem);
    else tile_indirect<MX>(L.atm[job], L.order, tile, smem);
  }
}

// ================================================== multiple scattering ===
// multiple_scattering.comp:9-93. Every texel of a row shares the ray (r, mu)
// and hence, for each trapezoid sample, the sample radius, its mu, the
// transmittance from the texel and the (mu, r) coordinates of the density
// lookup. For each sample the CTA interpolates the density table in (mu, r)
// once into a slab over x; each texel then blends four slab entries (two
// mu_s neighbours in two nu slices).
struct MSRec {
  float d, r_i, wdx, tvx, tvy, tvz, fy, fz;
  int y0, y1, z0, z1;
};

__host__ __device__ inline size_t ms_smem(int W, int steps, int sc_mus, int sc_nu) {
  const int R = rows_per_tile(W);
  return align16(sizeof(RowInfo) * R) + align16(sizeof(MSRec) * (size_t)R * (steps + 1)) +
         2 * sizeof(float4) * (size_t)R * W + align16(sizeof(double2) * sc_mus) + align16(sizeof(double) * sc_nu);
}

template <bool MX, int TPT>
__device__ void tile_multiple(const DevAtmo& a, int tile, unsigned char* smem) {
  const int W = a.W, nrows = a.sc_mu * a.sc_r;
  const int R = rows_per_tile(W);
  const int row0 = tile * R;
  const int nrow = min(R, nrows - row0);
  const int N = a.ms_steps, NS = N + 1;
  const int tid = threadIdx.x;
  unsigned char* p = smem;
  RowInfo* rows = (RowInfo*)p;                 p += align16(sizeof(RowInfo) * R);
  MSRec* rec = (MSRec*)p;                      p += align16(sizeof(MSRec) * (size_t)R * NS);
  float4* slab = (float4*)p;                   p += 2 * sizeof(float4) * (size_t)R * W;
  ColTabs cols;
  cols.mus = (double2*)p;                      p += align16(sizeof(double2) * a.sc_mus);
  cols.nu = (double*)p;
  const int slab_n = nrow * W;
  const int slab_stride = R * W;
  if (tid < nrow) row_info<MX>(a, row0 + tid, N, rows[tid]);
  if (MX) build_cols(a, cols);
  __syncthreads();
  for (int k = tid; k < nrow * NS; k += kThreads) {
    const RowInfo& ri = rows[k / NS];
    const int i = k % NS;
    MSRec& o = rec[k];
    const float w = (i == 0 || i == N) ? 0.5f : 1.0f;
    float3 tv;
    Axis ay, az;
    if (!MX) {
      Geo32 G;
      G.init(a);
      const float d = float(i) * ri.dx;
      const float r_i = G.clamp_radius(sqrtf(d * d + ri.two_r_mu * d + ri.rr));
      const float mu_i = clamp_cosine((ri.r_mu + d) / r_i);
      tv = G.tr_segment(a, ri.r, ri.mu, d, ri.ground);
      az = make_axis(G.u_r(a, r_i), a.sc_r);
      ay = make_axis(G.u_mu(a, r_i, mu_i, ri.ground), a.sc_mu);
      o.d = d;
      o.r_i = r_i;
    } else {
      Geo64 G;
      G.init(a);
      const double d = double(i) * ri.dxd;
      double q = ri.q + d * (2.0 * ri.s + d), s = ri.s + d;
      G.clamp_point(q, s);
      tv = G.tr_segment(a, ri.q, ri.s, d, ri.ground);
      az = axis_texel(G.sc_r_texel(a, q), a.sc_r);
      ay = axis_texel(G.sc_mu_texel(a, q, s, ri.ground), a.sc_mu);
      o.d = (float)d;
      o.r_i = (float)G.radius(q);
    }
    o.wdx = ri.dx * w;
    o.tvx = tv.x;
    o.tvy = tv.y;
    o.tvz = tv.z;
    o.y0 = ay.i0;
    o.y1 = ay.i1;
    o.fy = ay.f;
    o.z0 = az.i0;
    o.z1 = az.i1;
    o.fz = az.f;
  }
  __syncthreads();
  // per-texel constants (TPT texels per thread)
  float c_rmus[TPT], c_nu[TPT], c_lerp[TPT], c_tex[TPT];
  Kahan3 acc[TPT];
  MuS32 mus32;
  mus32.init(a);
  Geo32 G32;
  G32.init(a);
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    acc[j].init();
    c_rmus[j] = c_nu[j] = c_lerp[j] = c_tex[j] = 0.f;
    const int k = tid + j * kThreads;
    if (k < slab_n) {
      const int lr = k / W, x = k % W;
      float mu_s, nu, rmus;
      texel_mus_nu<MX>(a, rows[lr], cols, x, mu_s, nu, rmus);
      c_nu[j] = nu;
      c_rmus[j] = rmus;
      // scattering.h:146-148
      const float tcx = (nu + 1.0f) / 2.0f * float(a.sc_nu - 1);
      const float fl = floorf(tcx);
      c_lerp[j] = tcx - fl;
      c_tex[j] = fl;
    }
  }
  const float4* dens = a.dens;
  const size_t plane = (size_t)a.sc_mu * W;
  auto build = [&](int i, float4* dst) {
    for (int k = tid; k < slab_n; k += kThreads) {
      const int lr = k / W, x = k % W;
      const MSRec& o = rec[lr * NS + i];
      const float4 a00 = ld4(dens + o.z0 * plane + (size_t)o.y0 * W + x);
      const float4 a10 = ld4(dens + o.z0 * plane + (size_t)o.y1 * W + x);
      const float4 a01 = ld4(dens + o.z1 * plane + (size_t)o.y0 * W + x);
      const float4 a11 = ld4(dens + o.z1 * plane + (size_t)o.y1 * W + x);
      const float w00 = (1.f - o.fy) * (1.f - o.fz), w10 = o.fy * (1.f - o.fz);
      const float w01 = (1.f - o.fy) * o.fz, w11 = o.fy * o.fz;
      float4 v;
      v.x = fmaf(w11, a11.x, fmaf(w01, a01.x, fmaf(w10, a10.x, w00 * a00.x)));
      v.y = fmaf(w11, a11.y, fmaf(w01, a01.y, fmaf(w10, a10.y, w00 * a00.y)));
      v.z = fmaf(w11, a11.z, fmaf(w01, a01.z, fmaf(w10, a10.z, w00 * a00.z)));
      v.w = 0.f;
      dst[k] = v;
    }
  };
  build(0, slab);
  __syncthreads();
  const float fnu = float(a.sc_nu);
  for (int i = 0; i < NS; ++i) {
    const float4* cur = slab + (i & 1) * slab_stride;
    if (i + 1 < NS) build(i + 1, slab + ((i + 1) & 1) * slab_stride);
#pragma unroll
    for (int j = 0; j < TPT; ++j) {
      const int k = tid + j * kThreads;
      if (k < slab_n) {
        const int lr = k / W;
        const MSRec& o = rec[lr * NS + i];
        const float nu = c_nu[j];
        // multiple_scattering.comp:38 and scattering.h:48-56
        const float tx = c_tex[j];
        Axis x0, x1;
        if (!MX) {
          const float mu_s_i = clamp_cosine((c_rmus[j] + o.d * nu) / o.r_i);
          const float u_ms = G32.u_mu_s(a, mu_s_i);
          x0 = make_axis((tx + u_ms) / fnu, W);
          x1 = make_axis((tx + 1.0f + u_ms) / fnu, W);
        } else {
          // texel coordinate of slice k: k * mu_s_size + y (mu_s_size - 1)
          const float mu_s_i = clamp_cosine(fmaf(o.d, nu, c_rmus[j]) / o.r_i);
          const float t = mus32.texel(mu_s_i);
          x0 = axis_texel(fmaf(tx, float(a.sc_mus), t), W);
          x1 = axis_texel(fmaf(tx + 1.0f, float(a.sc_mus), t), W);
        }
        const float4* sl = cur + lr * W;
        const float4 p00 = sl[x0.i0], p01 = sl[x0.i1], p10 = sl[x1.i0], p11 = sl[x1.i1];
        const float lf = c_lerp[j];
        const float ax = fmaf(p01.x - p00.x, x0.f, p00.x), bx = fmaf(p11.x - p10.x, x1.f, p10.x);
        const float ay = fmaf(p01.y - p00.y, x0.f, p00.y), by = fmaf(p11.y - p10.y, x1.f, p10.y);
        const float az = fmaf(p01.z - p00.z, x0.f, p00.z), bz = fmaf(p11.z - p10.z, x1.f, p10.z);
        const float3 J = make_float3(fmaf(bx - ax, lf, ax), fmaf(by - ay, lf, ay), fmaf(bz - az, lf, az));
        const float3 v = J * make_float3(o.tvx, o.tvy, o.tvz) * o.wdx;
        if (!MX) acc[j].s = acc[j].s + v;
        else acc[j].add(v);
      }
    }
    __syncthreads();
  }
  // outputs: delta multiple scattering and the final table (:91-92)
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    const int k = tid + j * kThreads;
    if (k < slab_n) {
      const int lr = k / W, x = k % W;
      const size_t t = (size_t)(row0 + lr) * W + x;
      const float3 ms = make_float3(acc[j].s.x - acc[j].c.x, acc[j].s.y - acc[j].c.y, acc[j].s.z - acc[j].c.z);
      a.dms[t] = store_round4(make_float4(ms.x, ms.y, ms.z, 0.f), a.f16);
      const float pr = phase_rayleigh(c_nu[j]);
      const float4 old = a.sc[t];
      if (!MX) {
        a.sc[t] = store_round4(make_float4(ms.x / pr + old.x, ms.y / pr + old.y, ms.z / pr + old.z, 0.f + old.w),
                               a.f16);
      } else {
        double* s3 = a.sc_acc + 3 * t;
        s3[0] += (double)ms.x / pr;
        s3[1] += (double)ms.y / pr;
        s3[2] += (double)ms.z / pr;
        a.sc[t] = store_round4(make_float4((float)s3[0], (float)s3[1], (float)s3[2], old.w), a.f16);
      }
    }
  }
}

template <bool MX, int TPT> __global__ void __launch_bounds__(kThreads) k_multiple(LaunchArgs L) {
  extern __shared__ __align__(16) unsigned char smem[];
  int seg, job, tile;
  while (next_item(L, seg, job, tile)) tile_multiple<MX, TPT>(L.atm[job], tile, smem);
}

// ------------------------------------------------------ tile geometry ----
// Host and device agree on tile counts and shared-memory sizes through these.
__host__ __device__ inline int tiles_transmittance(int tr_mu, int tr_r) {
  return (tr_mu * tr_r + kThreads / 32 - 1) / (kThreads / 32);
}
__host__ __device__ inline int tiles_rows(int W, int sc_mu, int sc_r) {
  const int R = rows_per_tile(W);
  return (sc_mu * sc_r + R - 1) / R;
}
__host__ __device__ inline int tiles_direct(int ir_mus, int ir_r) { return (ir_mus * ir_r + kThreads - 1) / kThreads; }
__host__ __device__ inline int tiles_indirect(int ir_mus, int ir_r) { return ir_mus * ir_r; }
__host__ __device__ inline int tiles_density(int sc_r, int sc_mus, int sc_mu, int chunk) {
  return sc_r * sc_mus * ((sc_mu + chunk - 1) / chunk);
}
__host__ __device__ inline size_t ss_smem(int W, int steps, int sc_mus, int sc_nu) {
  const int R = rows_per_tile(W);
  return sizeof(RowInfo) * R + sizeof(SSRec) * (size_t)R * (steps + 1) + 16 + sizeof(double2) * sc_mus +
         sizeof(double) * sc_nu + 16;
}
__host__ __device__ inline size_t density_smem(int dens_n, int sc_nu, int ir_mus, int chunk, bool two) {
  return dens_layout(nullptr, dens_n, sc_nu, ir_mus, chunk, two, nullptr);
}

}  // namespace fb
