// ref_runner.cpp — runs the reference's own compute shaders, compiled as C++
// (oracle/ref_glsl/translate.py + glsl_shim.hpp), in the pass order of
// Atmosphere::build (src/precompute.rs:1726-1999).
//
// TEST INFRASTRUCTURE ONLY: it pins the CPU oracle and produces the golden
// vectors; nothing in the library links it. Built into oracle/_ref/ with
// -fsingle-precision-constant -ffp-contract=off (see oracle/build.py).
#include "glsl_shim.hpp"

namespace glsl {
#include "util.h"
#include "params.h"
#include "transmittance.h"
#include "irradiance.h"
#include "scattering.h"
namespace p_transmittance {
#include "transmittance.comp"
}
namespace p_direct {
#include "direct_irradiance.comp"
}
namespace p_single {
#include "single_scattering.comp"
}
namespace p_density {
#include "scattering_density.comp"
}
namespace p_indirect {
#include "indirect_irradiance.comp"
}
namespace p_multiple {
#include "multiple_scattering.comp"
}
namespace p_render {
#include "render_sky.h"
#include "render_lighting.h"
}
}  // namespace glsl

#include <cstring>
#include <vector>

#include "fuzzyblue.h"

namespace {
using namespace glsl;

void set_layer(DensityProfileLayer& d, const fb_density_profile_layer& s) {
  d.width = s.width;
  d.exp_term = s.exp_term;
  d.exp_scale = s.exp_scale;
  d.linear_term = s.linear_term;
  d.constant_term = s.constant_term;
}
void set_profile(DensityProfile& d, const fb_density_profile& s) {
  set_layer(d.layers[0], s.layers[0]);
  set_layer(d.layers[1], s.layers[1]);
}
vec3 v3(const float* f) { return vec3(f[0], f[1], f[2]); }

AtmosphereParameters convert(const fb_params_raw& r) {
  AtmosphereParameters a;
  a.solar_irradiance = v3(r.solar_irradiance);
  a.sun_angular_radius = r.sun_angular_radius;
  a.rayleigh_scattering = v3(r.rayleigh_scattering);
  a.bottom_radius = r.bottom_radius;
  a.mie_scattering = v3(r.mie_scattering);
  a.top_radius = r.top_radius;
  a.mie_extinction = v3(r.mie_extinction);
  a.mie_phase_function_g = r.mie_phase_function_g;
  a.ground_albedo = v3(r.ground_albedo);
  a.mu_s_min = r.mu_s_min;
  a.absorption_extinction = v3(r.absorption_extinction);
  a.transmittance_texture_mu_size = (int)r.transmittance_mu_size;
  a.transmittance_texture_r_size = (int)r.transmittance_r_size;
  a.scattering_texture_r_size = (int)r.scattering_r_size;
  a.scattering_texture_mu_size = (int)r.scattering_mu_size;
  a.scattering_texture_mu_s_size = (int)r.scattering_mu_s_size;
  a.scattering_texture_nu_size = (int)r.scattering_nu_size;
  a.irradiance_texture_mu_s_size = (int)r.irradiance_mu_s_size;
  a.irradiance_texture_r_size = (int)r.irradiance_r_size;
  set_profile(a.rayleigh_density, r.rayleigh_density);
  set_profile(a.mie_density, r.mie_density);
  set_profile(a.absorption_density, r.absorption_density);
  return a;
}

template <class F> void dispatch(uint w, uint h, uint d, F&& f) {
  const long n = (long)w * h * d;
#pragma omp parallel for schedule(dynamic, 16)
  for (long k = 0; k < n; ++k) {
    uint x = (uint)(k % w), y = (uint)((k / w) % h), z = (uint)(k / ((long)w * h));
    f(uvec3(x, y, z));
  }
}

}  // namespace

extern "C" {

// Same arguments as the oracle's fbo_precompute_f32; the reference's shader
// constants fix the sample counts (500/50/50/16/32), so other values are
// rejected.
int fbref_precompute(const fb_params* p, float* tr, float* ir, float* sc, float* orders_ms,
                     float* orders_irr, float* single_r, float* single_m) {
  if (!p || !tr || !ir || !sc) return FB_ERR_INVALID_ARGUMENT;
  if (p->transmittance_steps != 500 || p->single_scattering_steps != 50 ||
      p->multiple_scattering_steps != 50 || p->density_samples != 16 || p->irradiance_samples != 32)
    return FB_ERR_INVALID_PARAMS;
  const fb_params_raw& r = p->raw;
  const bool half = p->storage == FB_STORAGE_F16;
  const AtmosphereParameters atm = convert(r);
  const int trw = (int)r.transmittance_mu_size, trh = (int)r.transmittance_r_size;
  const int irw = (int)r.irradiance_mu_s_size, irh = (int)r.irradiance_r_size;
  const int scw = (int)(r.scattering_nu_size * r.scattering_mu_s_size), sch = (int)r.scattering_mu_size,
            scd = (int)r.scattering_r_size;
  const size_t nsc = (size_t)scw * sch * scd, nir = (size_t)irw * irh;
  std::vector<float> dirr(4 * nir), dr(4 * nsc), dm(4 * nsc), dms(4 * nsc), dens(4 * nsc);

  const sampler2D s_tr = {tr, trw, trh};
  const sampler2D s_dirr = {dirr.data(), irw, irh};
  const sampler3D s_dr = {dr.data(), scw, sch, scd}, s_dm = {dm.data(), scw, sch, scd};
  const sampler3D s_dms = {dms.data(), scw, sch, scd}, s_dens = {dens.data(), scw, sch, scd};

  p_transmittance::atmosphere = atm;
  p_transmittance::table = image2D{tr, trw, trh, false};
  dispatch(trw, trh, 1, [](uvec3 id) { p_transmittance::main_entry(id); });

  p_direct::atmosphere = atm;
  p_direct::transmittance_texture = s_tr;
  p_direct::delta_irradiance = image2D{dirr.data(), irw, irh, false};
  dispatch(irw, irh, 1, [](uvec3 id) { p_direct::main_entry(id); });

  p_single::atmosphere = atm;
  p_single::transmittance = s_tr;
  p_single::delta_rayleigh = image3D{dr.data(), scw, sch, scd, half};
  p_single::delta_mie = image3D{dm.data(), scw, sch, scd, half};
  p_single::scattering = image3D{sc, scw, sch, scd, half};
  dispatch(scw, sch, scd, [](uvec3 id) { p_single::main_entry(id); });

  std::memset(ir, 0, sizeof(float) * 4 * nir);  // src/precompute.rs:1802-1816

  p_density::atmosphere = atm;
  p_density::transmittance_texture = s_tr;
  p_density::single_rayleigh_scattering_texture = s_dr;
  p_density::single_mie_scattering_texture = s_dm;
  p_density::multiple_scattering_texture = s_dms;
  p_density::irradiance_texture = s_dirr;
  p_density::scattering_density = image3D{dens.data(), scw, sch, scd, half};

  p_indirect::atmosphere = atm;
  p_indirect::single_rayleigh_scattering_texture = s_dr;
  p_indirect::single_mie_scattering_texture = s_dm;
  p_indirect::multiple_scattering_texture = s_dms;
  p_indirect::delta_irradiance = image2D{dirr.data(), irw, irh, false};
  p_indirect::irradiance = image2D{ir, irw, irh, false};

  p_multiple::atmosphere = atm;
  p_multiple::transmittance_texture = s_tr;
  p_multiple::scattering_density_texture = s_dens;
  p_multiple::delta_multiple_scattering = image3D{dms.data(), scw, sch, scd, half};
  p_multiple::scattering = image3D{sc, scw, sch, scd, half};

  for (int order = 2; order <= (int)p->order; ++order) {
    p_density::scattering_order = order;  // push constant, src/precompute.rs:1892-1898
    dispatch(scw, sch, scd, [](uvec3 id) { p_density::main_entry(id); });
    p_indirect::scattering_order = order - 1;  // src/precompute.rs:1941-1947
    dispatch(irw, irh, 1, [](uvec3 id) { p_indirect::main_entry(id); });
    if (orders_irr) std::memcpy(orders_irr + (size_t)(order - 2) * 4 * nir, dirr.data(), sizeof(float) * 4 * nir);
    dispatch(scw, sch, scd, [](uvec3 id) { p_multiple::main_entry(id); });
    if (orders_ms) std::memcpy(orders_ms + (size_t)(order - 2) * 4 * nsc, dms.data(), sizeof(float) * 4 * nsc);
  }
  if (single_r) std::memcpy(single_r, dr.data(), sizeof(float) * 4 * nsc);
  if (single_m) std::memcpy(single_m, dm.data(), sizeof(float) * 4 * nsc);
  return FB_OK;
}

}  // extern "C"

extern "C" {

// Runs one pass of the reference's shaders for the listed invocations (linear
// ids x + width * (y + height * z) of the pass's output grid), reading and
// writing caller-owned full-size RGBA tables. Used to time a bounded sample of
// the reference's own code. pass: 0 transmittance, 1 direct irradiance,
// 2 single scattering, 3 scattering density, 4 indirect irradiance,
// 5 multiple scattering. `order` is the push constant of passes 3 and 4.
int fbref_run_pass(int pass, const fb_params* p, int order, float* tr, float* dirr, float* dr, float* dm,
                   float* dms, float* dens, float* ir, float* sc, const int64_t* ids, int64_t n) {
  if (!p || !ids) return FB_ERR_INVALID_ARGUMENT;
  const fb_params_raw& r = p->raw;
  const bool half = p->storage == FB_STORAGE_F16;
  const AtmosphereParameters atm = convert(r);
  const int trw = (int)r.transmittance_mu_size, trh = (int)r.transmittance_r_size;
  const int irw = (int)r.irradiance_mu_s_size, irh = (int)r.irradiance_r_size;
  const int scw = (int)(r.scattering_nu_size * r.scattering_mu_s_size), sch = (int)r.scattering_mu_size,
            scd = (int)r.scattering_r_size;
  const sampler2D s_tr = {tr, trw, trh}, s_dirr = {dirr, irw, irh};
  const sampler3D s_dr = {dr, scw, sch, scd}, s_dm = {dm, scw, sch, scd};
  const sampler3D s_dms = {dms, scw, sch, scd}, s_dens = {dens, scw, sch, scd};
  long w = 0, h = 0;
  void (*entry)(uvec3) = nullptr;
  switch (pass) {
    case 0:
      p_transmittance::atmosphere = atm;
      p_transmittance::table = image2D{tr, trw, trh, false};
      entry = p_transmittance::main_entry;
      w = trw; h = trh;
      break;
    case 1:
      p_direct::atmosphere = atm;
      p_direct::transmittance_texture = s_tr;
      p_direct::delta_irradiance = image2D{dirr, irw, irh, false};
      entry = p_direct::main_entry;
      w = irw; h = irh;
      break;
    case 2:
      p_single::atmosphere = atm;
      p_single::transmittance = s_tr;
      p_single::delta_rayleigh = image3D{dr, scw, sch, scd, half};
      p_single::delta_mie = image3D{dm, scw, sch, scd, half};
      p_single::scattering = image3D{sc, scw, sch, scd, half};
      entry = p_single::main_entry;
      w = scw; h = sch;
      break;
    case 3:
      p_density::atmosphere = atm;
      p_density::transmittance_texture = s_tr;
      p_density::single_rayleigh_scattering_texture = s_dr;
      p_density::single_mie_scattering_texture = s_dm;
      p_density::multiple_scattering_texture = s_dms;
      p_density::irradiance_texture = s_dirr;
      p_density::scattering_density = image3D{dens, scw, sch, scd, half};
      p_density::scattering_order = order;
      entry = p_density::main_entry;
      w = scw; h = sch;
      break;
    case 4:
      p_indirect::atmosphere = atm;
      p_indirect::single_rayleigh_scattering_texture = s_dr;
      p_indirect::single_mie_scattering_texture = s_dm;
      p_indirect::multiple_scattering_texture = s_dms;
      p_indirect::delta_irradiance = image2D{dirr, irw, irh, false};
      p_indirect::irradiance = image2D{ir, irw, irh, false};
      p_indirect::scattering_order = order;
      entry = p_indirect::main_entry;
      w = irw; h = irh;
      break;
    case 5:
      p_multiple::atmosphere = atm;
      p_multiple::transmittance_texture = s_tr;
      p_multiple::scattering_density_texture = s_dens;
      p_multiple::delta_multiple_scattering = image3D{dms, scw, sch, scd, half};
      p_multiple::scattering = image3D{sc, scw, sch, scd, half};
      entry = p_multiple::main_entry;
      w = scw; h = sch;
      break;
    default:
      return FB_ERR_INVALID_ARGUMENT;
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < n; ++k) {
    const int64_t id = ids[k];
    entry(uvec3((uint)(id % w), (uint)((id / w) % h), (uint)(id / (w * h))));
  }
  return FB_OK;
}

// The sky pass of the crate's renderer: render_sky.frag:24-34 per pixel with
// the reference's GetSkyRadianceToPoint (render_sky.h, compiled as C++).
// Screen coordinates are pixel centres; depth NULL reads 0 everywhere.
int fbref_render_sky(const fb_params* p, const float* tr, const float* sc, const fb_draw_parameters* d,
                     const float* depth, uint32_t width, uint32_t height, float* color, float* transmittance) {
  if (!p || !tr || !sc || !d || !color || width == 0 || height == 0) return FB_ERR_INVALID_ARGUMENT;
  const fb_params_raw& r = p->raw;
  const AtmosphereParameters atm = convert(r);
  const sampler2D s_tr = {tr, (int)r.transmittance_mu_size, (int)r.transmittance_r_size};
  const sampler3D s_sc = {sc, (int)(r.scattering_nu_size * r.scattering_mu_s_size), (int)r.scattering_mu_size,
                          (int)r.scattering_r_size};
  const float(*m)[4] = d->inverse_viewproj;
  // mat4 (columns m[c]) times vec4
  auto mul = [&](float x, float y, float z, float w, float out[4]) {
    for (int row = 0; row < 4; ++row) out[row] = m[0][row] * x + m[1][row] * y + m[2][row] * z + m[3][row] * w;
  };
  const vec3 camera(d->camera_position[0], d->camera_position[1], d->camera_position[2]);
  const vec3 sun(d->sun_direction[0], d->sun_direction[1], d->sun_direction[2]);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < (int64_t)width * height; ++k) {
    const uint32_t x = (uint32_t)(k % width), y = (uint32_t)(k / width);
    const vec2 screen((x + 0.5f) / (float)width, (y + 0.5f) / (float)height);
    const float sx = 2 * screen.x - 1, sy = 2 * screen.y - 1;
    float v[4], wp[4];
    mul(sx, sy, 0, 1, v);
    const vec3 view = normalize(vec3(v[0], v[1], v[2]));
    mul(sx, sy, depth ? depth[k] : 0.0f, 1, wp);
    const vec3 world = (vec3(wp[0], wp[1], wp[2]) / wp[3]) * 1e-3f;
    vec3 t;
    const vec3 c = p_render::GetSkyRadianceToPoint(atm, s_tr, s_sc, camera, view, world, sun, t);
    color[4 * k] = c.x;
    color[4 * k + 1] = c.y;
    color[4 * k + 2] = c.z;
    color[4 * k + 3] = 0.0f;
    if (transmittance) {
      transmittance[4 * k] = t.x;
      transmittance[4 * k + 1] = t.y;
      transmittance[4 * k + 2] = t.z;
      transmittance[4 * k + 3] = 1.0f;
    }
  }
  return FB_OK;
}

// GetSunAndSkyIrradiance (render_lighting.h) at n points.
int fbref_sun_and_sky_irradiance(const fb_params* p, const float* tr, const float* ir, const float* points,
                                 const float* normals, const float* sun_direction, int64_t n, float* sun_out,
                                 float* sky_out) {
  if (!p || !tr || !ir || !points || !normals || !sun_direction || !sun_out || !sky_out)
    return FB_ERR_INVALID_ARGUMENT;
  const fb_params_raw& r = p->raw;
  const AtmosphereParameters atm = convert(r);
  const sampler2D s_tr = {tr, (int)r.transmittance_mu_size, (int)r.transmittance_r_size};
  const sampler2D s_ir = {ir, (int)r.irradiance_mu_s_size, (int)r.irradiance_r_size};
  const vec3 sun(sun_direction[0], sun_direction[1], sun_direction[2]);
#pragma omp parallel for
  for (int64_t k = 0; k < n; ++k) {
    vec3 sky;
    const vec3 direct = p_render::GetSunAndSkyIrradiance(atm, s_tr, s_ir, v3(points + 3 * k), v3(normals + 3 * k),
                                                         sun, sky);
    sun_out[3 * k] = direct.x;
    sun_out[3 * k + 1] = direct.y;
    sun_out[3 * k + 2] = direct.z;
    sky_out[3 * k] = sky.x;
    sky_out[3 * k + 1] = sky.y;
    sky_out[3 * k + 2] = sky.z;
  }
  return FB_OK;
}

}  // extern "C"
