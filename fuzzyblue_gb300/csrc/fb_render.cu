// fb_render.cu — the crate's sky pass and surface lighting on the precomputed
// tables, without a graphics API: fb_atmosphere_render_sky evaluates
// render_sky.frag:24-34 (GetSkyRadianceToPoint, render_sky.h:111-191) for
// every pixel of an image into device memory; fb_atmosphere_sun_and_sky_
// irradiance evaluates GetSunAndSkyIrradiance (render_lighting.h:10-28) at
// a batch of points. FP32 in the shaders' operation order (this translation
// unit is compiled with --fmad=false); the tables are sampled with the exact
// weights of the crate's LINEAR / CLAMP_TO_EDGE sampler. One thread per pixel
// or point; these are consumers of the tables, not part of the precompute.
#include <cuda_runtime.h>

#include "../../include/fuzzyblue.h"
#include "fb_device.cuh"
#include "fb_internal.h"

namespace {

using namespace fb;

struct DrawArgs {
  float m[4][4];  // (projection * view)^-1, m[column][row]
  float cam[3];
  float sun[3];
};

__device__ __forceinline__ float3 f3sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 f3add(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float f3dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float f3len(float3 a) { return sqrtf(f3dot(a, a)); }

// RGBA trilinear fetch (same weights and order as fetch3).
__device__ float4 fetch3_rgba(const float4* t, int w, int h, Axis x, Axis y, Axis z) {
  const float ia = 1.0f - x.f, ib = 1.0f - y.f, ic = 1.0f - z.f;
  const float wt[8] = {ia * ib * ic, x.f * ib * ic, ia * y.f * ic, x.f * y.f * ic,
                       ia * ib * z.f, x.f * ib * z.f, ia * y.f * z.f, x.f * y.f * z.f};
  const int xs[2] = {x.i0, x.i1}, ys[2] = {y.i0, y.i1}, zs[2] = {z.i0, z.i1};
  float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float4 p = ld4(t + ((size_t)zs[k >> 2] * h + ys[(k >> 1) & 1]) * w + xs[k & 1]);
    if (k == 0) {
      o = make_float4(wt[0] * p.x, wt[0] * p.y, wt[0] * p.z, wt[0] * p.w);
    } else {
      o.x = o.x + wt[k] * p.x;
      o.y = o.y + wt[k] * p.y;
      o.z = o.z + wt[k] * p.z;
      o.w = o.w + wt[k] * p.w;
    }
  }
  return o;
}

// render_sky.h:9-19
__device__ float3 extrapolated_single_mie(const DevAtmo& a, float4 s) {
  if (s.x <= 0.0f) return make_float3(0.f, 0.f, 0.f);
  const float q = a.rayleigh[0] / a.mie_sca[0];
  return make_float3(s.x * s.w / s.x * q * (a.mie_sca[0] / a.rayleigh[0]),
                     s.y * s.w / s.x * q * (a.mie_sca[1] / a.rayleigh[1]),
                     s.z * s.w / s.x * q * (a.mie_sca[2] / a.rayleigh[2]));
}

// render_sky.h:21-43 (scattering.h:7-60 for the coordinates)
__device__ float3 combined_scattering(const DevAtmo& a, const Geo32& G, float r, float mu, float mu_s, float nu,
                                      bool ground, float3& single_mie) {
  const float u_r = G.u_r(a, r), u_mu = G.u_mu(a, r, mu, ground), u_mu_s = G.u_mu_s(a, mu_s);
  const float u_nu = (nu + 1.0f) / 2.0f;
  const float tcx = u_nu * float(a.sc_nu - 1);
  const float tex_x = floorf(tcx);
  const float lerp = tcx - tex_x;
  const Axis ay = make_axis(u_mu, a.sc_mu), az = make_axis(u_r, a.sc_r);
  const float4 s0 = fetch3_rgba(a.sc, a.W, a.sc_mu, make_axis((tex_x + u_mu_s) / float(a.sc_nu), a.W), ay, az);
  const float4 s1 =
      fetch3_rgba(a.sc, a.W, a.sc_mu, make_axis((tex_x + 1.0f + u_mu_s) / float(a.sc_nu), a.W), ay, az);
  const float il = 1.0f - lerp;
  const float4 m = make_float4(s0.x * il + s1.x * lerp, s0.y * il + s1.y * lerp, s0.z * il + s1.z * lerp,
                               s0.w * il + s1.w * lerp);
  single_mie = extrapolated_single_mie(a, m);
  return make_float3(m.x, m.y, m.z);
}

// render_sky.h:111-191 without light shafts (shadow_length 0)
__device__ float3 sky_radiance_to_point(const DevAtmo& a, const Geo32& G, float3 camera, float3 view, float3 point,
                                        float3 sun, float3& transmittance) {
  float r = f3len(camera);
  float rmu = f3dot(camera, view);
  const float to_top = -rmu - sqrtf(rmu * rmu - r * r + a.top * a.top);
  if (to_top > 0.0f) {
    camera = f3add(camera, view * to_top);
    r = a.top;
    rmu += to_top;
  } else if (r > a.top) {
    transmittance = make_float3(1.f, 1.f, 1.f);
    return make_float3(0.f, 0.f, 0.f);
  }
  const float mu = rmu / r;
  const float mu_s = f3dot(camera, sun) / r;
  const float nu = f3dot(view, sun);
  const float d = f3len(f3sub(point, camera));
  const bool ground = G.hits_ground(r, mu);
  transmittance = G.tr_segment(a, r, mu, d, ground);
  float3 single_mie;
  float3 scattering = combined_scattering(a, G, r, mu, mu_s, nu, ground, single_mie);
  if (!isinf(d)) {
    const float r_p = G.clamp_radius(sqrtf(d * d + 2.0f * r * mu * d + r * r));
    const float mu_p = (r * mu + d) / r_p;
    const float mu_s_p = (r * mu_s + d * nu) / r_p;
    float3 single_mie_p;
    const float3 scattering_p = combined_scattering(a, G, r_p, mu_p, mu_s_p, nu, ground, single_mie_p);
    const float3 shadow = transmittance;
    scattering = f3sub(scattering, shadow * scattering_p);
    single_mie = f3sub(single_mie, shadow * single_mie_p);
    single_mie = extrapolated_single_mie(a, make_float4(scattering.x, scattering.y, scattering.z, single_mie.x));
    single_mie = single_mie * smoothstepf(0.0f, 0.01f, mu_s);
  }
  const float pr = phase_rayleigh(nu), pm = phase_mie(a.g, nu);
  return f3add(scattering * pr, single_mie * pm);
}

__global__ void __launch_bounds__(256) k_render_sky(DevAtmo a, DrawArgs d, const float* depth, uint32_t width,
                                                    uint32_t height, float4* color, float4* trans) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (uint64_t)width * height) return;
  const uint32_t x = (uint32_t)(k % width), y = (uint32_t)(k / width);
  Geo32 G;
  G.init(a);
  // render_sky.frag:24-34
  const float sx = 2.0f * ((float(x) + 0.5f) / float(width)) - 1.0f;
  const float sy = 2.0f * ((float(y) + 0.5f) / float(height)) - 1.0f;
  const float dz = depth ? depth[k] : 0.0f;
  float v[4], w[4];
#pragma unroll
  for (int row = 0; row < 4; ++row) {
    v[row] = d.m[0][row] * sx + d.m[1][row] * sy + d.m[2][row] * 0.0f + d.m[3][row] * 1.0f;
    w[row] = d.m[0][row] * sx + d.m[1][row] * sy + d.m[2][row] * dz + d.m[3][row] * 1.0f;
  }
  const float vl = f3len(make_float3(v[0], v[1], v[2]));
  const float3 view = make_float3(v[0] / vl, v[1] / vl, v[2] / vl);
  const float3 world = make_float3(w[0] / w[3] * 1e-3f, w[1] / w[3] * 1e-3f, w[2] / w[3] * 1e-3f);
  float3 t;
  const float3 c = sky_radiance_to_point(a, G, make_float3(d.cam[0], d.cam[1], d.cam[2]), view, world,
                                         make_float3(d.sun[0], d.sun[1], d.sun[2]), t);
  color[k] = make_float4(c.x, c.y, c.z, 0.0f);
  if (trans) trans[k] = make_float4(t.x, t.y, t.z, 1.0f);
}

// render_lighting.h:10-28 (irradiance.h:20-38, transmittance.h:63-74)
__global__ void __launch_bounds__(256) k_sun_and_sky(DevAtmo a, const float* points, const float* normals,
                                                     float3 sun, uint32_t n, float* sun_out, float* sky_out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Geo32 G;
  G.init(a);
  const float3 p = make_float3(points[3 * k], points[3 * k + 1], points[3 * k + 2]);
  const float3 nrm = make_float3(normals[3 * k], normals[3 * k + 1], normals[3 * k + 2]);
  const float r = f3len(p);
  const float mu_s = f3dot(p, sun) / r;
  // indirect: GetIrradiance(r, mu_s) * (1 + n . p / r) / 2
  const float x_r = (r - a.bottom) / (a.top - a.bottom);
  const float x_mu_s = mu_s * 0.5f + 0.5f;
  const float3 irr = fetch2(a.ir, a.ir_mus, make_axis(coord_from_unit(x_mu_s, a.ir_mus), a.ir_mus),
                            make_axis(coord_from_unit(x_r, a.ir_r), a.ir_r));
  const float3 sky = irr * ((1.0f + f3dot(nrm, p) / r) * 0.5f);
  // direct: solar * GetTransmittanceToSun(r, mu_s) * max(n . sun, 0)
  const float sin_h = a.bottom / r;
  const float cos_h = -sqrtf(gmax(1.0f - sin_h * sin_h, 0.0f));
  const float3 ts = G.tr_to_top(a, r, mu_s) *
                    smoothstepf(-sin_h * a.sun_radius, sin_h * a.sun_radius, mu_s - cos_h);
  const float3 direct = ld3(a.solar) * ts * gmax(f3dot(nrm, sun), 0.0f);
  sun_out[3 * k] = direct.x;
  sun_out[3 * k + 1] = direct.y;
  sun_out[3 * k + 2] = direct.z;
  sky_out[3 * k] = sky.x;
  sky_out[3 * k + 1] = sky.y;
  sky_out[3 * k + 2] = sky.z;
}

int record_of(const fb_atmosphere* atm, DevAtmo& d) {
  fbi::fill_atmo_record(d, fbi::atmosphere_params(atm));
  fbi::atmosphere_tables(atm, &d.tr, &d.ir, &d.sc);
  return FB_OK;
}

}  // namespace

extern "C" int fb_atmosphere_render_sky(const fb_atmosphere* a, void* stream, const fb_draw_parameters* dp,
                                        const float* depth, uint32_t width, uint32_t height, float* color,
                                        float* transmittance) {
  if (!a || !dp || !color) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 31))
    return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "image size out of range");
  if (((uintptr_t)color | (uintptr_t)transmittance) & 15u)
    return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "output images must be 16-byte aligned");
  DevAtmo d;
  record_of(a, d);
  DrawArgs args;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) args.m[c][r] = dp->inverse_viewproj[c][r];
  for (int i = 0; i < 3; ++i) {
    args.cam[i] = dp->camera_position[i];
    args.sun[i] = dp->sun_direction[i];
  }
  const uint64_t n = (uint64_t)width * height;
  k_render_sky<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d, args, depth, width, height,
                                                                             (float4*)color, (float4*)transmittance);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fbi::set_error(FB_ERR_CUDA, cudaGetErrorString(e));
  return FB_OK;
}

extern "C" int fb_atmosphere_sun_and_sky_irradiance(const fb_atmosphere* a, void* stream, const float* points,
                                                    const float* normals, const float* sun_direction, uint32_t n,
                                                    float* sun_irradiance, float* sky_irradiance) {
  if (!a || !points || !normals || !sun_direction || !sun_irradiance || !sky_irradiance)
    return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n == 0) return FB_OK;
  DevAtmo d;
  record_of(a, d);
  const float3 sun = make_float3(sun_direction[0], sun_direction[1], sun_direction[2]);
  k_sun_and_sky<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d, points, normals, sun, n, sun_irradiance,
                                                                   sky_irradiance);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fbi::set_error(FB_ERR_CUDA, cudaGetErrorString(e));
  return FB_OK;
}
