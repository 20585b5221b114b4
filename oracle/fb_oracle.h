/*
 * fb_oracle.h — CPU oracle for the atmosphere LUT precompute.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle restates, on the CPU, the algorithm of
 * the reference's six compute shaders (shaders/*.comp and the headers they
 * include) and the pass order of Atmosphere::build (src/precompute.rs:1726-1999).
 * Only tests, the smoke check and the CPU-baseline leg of bench.py may call it;
 * the library never links it.
 *
 * Two instantiations of one template:
 *   _f32  IEEE single precision, no FMA contraction: the arithmetic of the
 *         reference's GLSL (float literals, float intermediates), with exact
 *         bilinear/trilinear weights in place of the sampler's fixed-point ones.
 *   _f64  the same integrals in double precision: the accuracy oracle. In the
 *         transmittance march it evaluates the exact-arithmetic altitude of
 *         samples that rounding puts a hair below the ground (every ray of that
 *         table stays at or above the ground), so that tangent samples do not
 *         flip the width-0 layer test of params.h:95-99 at random.
 *
 * Texel layout of every table: RGBA (4 values per texel), x fastest, then y,
 * then z, exactly like the library's tables.
 */
#ifndef FB_ORACLE_H_
#define FB_ORACLE_H_

#include <stdint.h>
#include "../include/fuzzyblue.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Whole precompute in the reference's pass order. `nthreads` <= 0 uses all
 * OpenMP threads. Optional outputs may be NULL:
 *   orders_ms   (order-1) scattering-sized tables: delta_multiple_scattering of
 *               orders 2..order
 *   orders_irr  (order-1) irradiance-sized tables: delta_irradiance written by
 *               indirect irradiance of orders 1..order-1
 *   single_r / single_m  delta_rayleigh / delta_mie
 * p->storage == FB_STORAGE_F16 rounds the scattering-class tables to half on
 * every store, like the reference's RGBA16F images. */
int fbo_precompute_f32(const fb_params* p, int nthreads, float* transmittance,
                       float* irradiance, float* scattering, float* orders_ms,
                       float* orders_irr, float* single_r, float* single_m);
int fbo_precompute_f64(const fb_params* p, int nthreads, double* transmittance,
                       double* irradiance, double* scattering, double* orders_ms,
                       double* orders_irr, double* single_r, double* single_m);

/* Single passes over given inputs. `idx` lists linear texel indices of the
 * pass's output table (NULL = every texel); outputs are packed in idx order
 * (or table order when idx is NULL), 4 values per texel. */
int fbo_transmittance_f32(const fb_params* p, int nthreads, const int64_t* idx,
                          int64_t n, float* out);
int fbo_direct_irradiance_f32(const fb_params* p, int nthreads,
                              const float* transmittance, const int64_t* idx,
                              int64_t n, float* out);
int fbo_single_scattering_f32(const fb_params* p, int nthreads,
                              const float* transmittance, const int64_t* idx,
                              int64_t n, float* out_rayleigh, float* out_mie);
/* `order` is the order being computed (>= 2); order 2 reads single_r/single_m,
 * higher orders read multiple. */
int fbo_scattering_density_f32(const fb_params* p, int nthreads, int order,
                               const float* transmittance, const float* single_r,
                               const float* single_m, const float* multiple,
                               const float* delta_irradiance, const int64_t* idx,
                               int64_t n, float* out);
/* `order` is the scattering order integrated (>= 1, the push constant of
 * src/precompute.rs:1946). */
int fbo_indirect_irradiance_f32(const fb_params* p, int nthreads, int order,
                                const float* single_r, const float* single_m,
                                const float* multiple, const int64_t* idx,
                                int64_t n, float* out);
/* out: delta_multiple_scattering texels; out_phase (may be NULL): the
 * RayleighPhase(nu) the final scattering table divides it by
 * (multiple_scattering.comp:92). */
int fbo_multiple_scattering_f32(const fb_params* p, int nthreads,
                                const float* transmittance, const float* density,
                                const int64_t* idx, int64_t n, float* out,
                                float* out_phase);

/* Same single passes in double precision (inputs and outputs double). */
int fbo_transmittance_f64(const fb_params* p, int nthreads, const int64_t* idx,
                          int64_t n, double* out);
int fbo_direct_irradiance_f64(const fb_params* p, int nthreads,
                              const double* transmittance, const int64_t* idx,
                              int64_t n, double* out);
int fbo_single_scattering_f64(const fb_params* p, int nthreads,
                              const double* transmittance, const int64_t* idx,
                              int64_t n, double* out_rayleigh, double* out_mie);
int fbo_indirect_irradiance_f64(const fb_params* p, int nthreads, int order,
                                const double* single_r, const double* single_m,
                                const double* multiple, const int64_t* idx,
                                int64_t n, double* out);
int fbo_scattering_density_f64(const fb_params* p, int nthreads, int order,
                               const double* transmittance, const double* single_r,
                               const double* single_m, const double* multiple,
                               const double* delta_irradiance, const int64_t* idx,
                               int64_t n, double* out);
int fbo_multiple_scattering_f64(const fb_params* p, int nthreads,
                                const double* transmittance, const double* density,
                                const int64_t* idx, int64_t n, double* out,
                                double* out_phase);

/* Parameters::default() restated (src/precompute.rs:849-935) plus the
 * default sample counts, for callers that do not link the library. */
void fbo_params_default(fb_params* out);

/* The renderer's shading (render_sky.frag:24-34 with render_sky.h:111-191;
 * render_lighting.h:10-28) on the given tables: see fb_atmosphere_render_sky
 * and fb_atmosphere_sun_and_sky_irradiance in fuzzyblue.h for the arguments
 * (host arrays here). */
int fbo_render_sky_f32(const fb_params* p, const float* tr, const float* sc, const fb_draw_parameters* d,
                       const float* depth, uint32_t width, uint32_t height, float* color, float* trans);
int fbo_render_sky_f64(const fb_params* p, const double* tr, const double* sc, const fb_draw_parameters* d,
                       const double* depth, uint32_t width, uint32_t height, double* color, double* trans);
int fbo_sun_and_sky_irradiance_f32(const fb_params* p, const float* tr, const float* ir, const float* points,
                                   const float* normals, const float* sun, int64_t n, float* sun_out,
                                   float* sky_out);
int fbo_sun_and_sky_irradiance_f64(const fb_params* p, const double* tr, const double* ir, const double* points,
                                   const double* normals, const double* sun, int64_t n, double* sun_out,
                                   double* sky_out);

/* Reference shader arithmetic per texel of one pass (0 transmittance, 1 direct
 * irradiance, 2 single scattering, 3 scattering density of `order`, 4 indirect
 * irradiance of `order`, 5 multiple scattering), averaged over `n` sampled
 * texels: out[5] = adds/subs, muls, divs, sqrts, transcendentals. Sampler
 * filtering (fixed-function in the reference) is not counted; operations on
 * literals only are folded. */
int fbo_count_ops(const fb_params* p, int pass, int order, int64_t n,
                  uint64_t seed, double* out);

#ifdef __cplusplus
}
#endif
#endif
