// fb_capi.cu — the C ABI of include/fuzzyblue.h: parameters, builder,
// single and batched builds, pending handles and table access.
//
// A build (one atmosphere or a batch) is planned on the host: every atmosphere
// gets its output block and its temporaries, a DevAtmo record, and a place in
// the work lists of the launches. Launch order per precision group:
//   transmittance; single scattering + direct irradiance; then for each order
//   n = 2..max: scattering density(n) + indirect irradiance(n-1); multiple
//   scattering(n). An atmosphere whose order is below n has no items in the
//   launches of order n. This is the pass order of src/precompute.rs:1726-1999
//   with the two pairs of independent passes fused into one launch each.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fuzzyblue.h"
#include "fb_internal.h"
#include "fb_kernels.h"

using fb::DevAtmo;
using fb::LaunchArgs;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define FB_CU(expr)                                                                        \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess) return fail(FB_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// ------------------------------------------------------------ parameters ---
extern "C" void fb_params_default(fb_params* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  fb_params_raw& r = o->raw;
  // Parameters::default(), src/precompute.rs:849-935
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

extern "C" int fb_params_validate(const fb_params* p) {
  if (!p) return fail(FB_ERR_INVALID_ARGUMENT, "params is NULL");
  const fb_params_raw& r = p->raw;
  const uint32_t sizes[8] = {r.transmittance_mu_size, r.transmittance_r_size, r.scattering_r_size,
                             r.scattering_mu_size,    r.scattering_mu_s_size, r.scattering_nu_size,
                             r.irradiance_mu_s_size,  r.irradiance_r_size};
  const char* names[8] = {"transmittance_mu_size", "transmittance_r_size", "scattering_r_size",
                          "scattering_mu_size", "scattering_mu_s_size", "scattering_nu_size",
                          "irradiance_mu_s_size", "irradiance_r_size"};
  for (int i = 0; i < 8; ++i)
    if (sizes[i] < 2 || sizes[i] > 65536) return fail(FB_ERR_INVALID_PARAMS, "%s = %u is outside [2, 65536]", names[i], sizes[i]);
  if (r.scattering_mu_size % 2) return fail(FB_ERR_INVALID_PARAMS, "scattering_mu_size must be even");
  if (r.scattering_nu_size > 64) return fail(FB_ERR_INVALID_PARAMS, "scattering_nu_size must be <= 64");
  if ((uint64_t)r.scattering_nu_size * r.scattering_mu_s_size > 2048)
    return fail(FB_ERR_INVALID_PARAMS, "scattering_nu_size * scattering_mu_s_size must be <= 2048");
  if (r.irradiance_mu_s_size > 4096) return fail(FB_ERR_INVALID_PARAMS, "irradiance_mu_s_size must be <= 4096");
  if ((uint64_t)r.scattering_nu_size * r.scattering_mu_s_size * r.scattering_mu_size * r.scattering_r_size > (1ull << 30))
    return fail(FB_ERR_INVALID_PARAMS, "scattering table larger than 2^30 texels");
  if (!(r.bottom_radius > 0.0f) || !(r.top_radius > r.bottom_radius))
    return fail(FB_ERR_INVALID_PARAMS, "need 0 < bottom_radius < top_radius");
  if (p->order < 1 || p->order > 64) return fail(FB_ERR_INVALID_PARAMS, "order must be in [1, 64]");
  if (p->transmittance_steps < 1 || p->transmittance_steps > 1000000)
    return fail(FB_ERR_INVALID_PARAMS, "transmittance_steps must be in [1, 1e6]");
  if (p->single_scattering_steps < 1 || p->single_scattering_steps > 1024 || p->multiple_scattering_steps < 1 ||
      p->multiple_scattering_steps > 1024)
    return fail(FB_ERR_INVALID_PARAMS, "single/multiple scattering steps must be in [1, 1024]");
  if (p->density_samples < 2 || p->density_samples > 32 || p->density_samples % 2)
    return fail(FB_ERR_INVALID_PARAMS, "density_samples must be even, in [2, 32]");
  if (p->irradiance_samples < 2 || p->irradiance_samples > 64 || p->irradiance_samples % 2)
    return fail(FB_ERR_INVALID_PARAMS, "irradiance_samples must be even, in [2, 64]");
  if (p->precision > FB_PRECISION_MIXED) return fail(FB_ERR_INVALID_PARAMS, "unknown precision mode %u", p->precision);
  if (p->storage > FB_STORAGE_F16) return fail(FB_ERR_INVALID_PARAMS, "unknown storage mode %u", p->storage);
  return FB_OK;
}

extern "C" int fb_params_extents(const fb_params* p, fb_extent* tr, fb_extent* ir, fb_extent* sc) {
  if (!p) return fail(FB_ERR_INVALID_ARGUMENT, "params is NULL");
  const fb_params_raw& r = p->raw;
  if (tr) *tr = fb_extent{r.transmittance_mu_size, r.transmittance_r_size, 1};
  if (ir) *ir = fb_extent{r.irradiance_mu_s_size, r.irradiance_r_size, 1};
  if (sc) *sc = fb_extent{r.scattering_nu_size * r.scattering_mu_s_size, r.scattering_mu_size, r.scattering_r_size};
  return FB_OK;
}

namespace fbi {

// Geometry tables (order-independent, written by the first two launches):
// rows, x columns, multiple-scattering sample records, density r / theta records.
// Indirect-irradiance records of the mixed mode.
size_t irgeo_bytes(const fb_params& p) {
  const fb_params_raw& r = p.raw;
  const size_t ir_r = r.irradiance_r_size, ir_mus = r.irradiance_mu_s_size;
  return align256(sizeof(fb::IrZ) * ir_r) + align256(sizeof(fb::Axis) * ir_r * (p.irradiance_samples / 2)) +
         align256(sizeof(fb::Axis) * ir_mus * (r.scattering_nu_size + 2)) + align256(sizeof(float) * ir_mus);
}

size_t geometry_bytes(const fb_params& p) {
  const fb_params_raw& r = p.raw;
  const size_t rows = (size_t)r.scattering_mu_size * r.scattering_r_size;
  const size_t W = (size_t)r.scattering_nu_size * r.scattering_mu_s_size;
  return align256(sizeof(fb::RowGeo) * rows) + align256(sizeof(fb::ColGeo) * W) +
         align256(sizeof(fb::MSRec) * rows * (p.multiple_scattering_steps + 1)) +
         align256(sizeof(fb::DensZ) * r.scattering_r_size) +
         align256(sizeof(fb::ThetaRec) * r.scattering_r_size * p.density_samples) +
         (p.precision == FB_PRECISION_MIXED ? irgeo_bytes(p) : 0);
}

void place_geometry(fb::DevAtmo& d, char*& tp, bool mixed) {
  const size_t rows = (size_t)d.sc_mu * d.sc_r;
  d.g_rows = (fb::RowGeo*)tp;   tp += align256(sizeof(fb::RowGeo) * rows);
  d.g_cols = (fb::ColGeo*)tp;   tp += align256(sizeof(fb::ColGeo) * (size_t)d.W);
  d.g_ms = (fb::MSRec*)tp;      tp += align256(sizeof(fb::MSRec) * rows * (d.ms_steps + 1));
  d.g_z = (fb::DensZ*)tp;       tp += align256(sizeof(fb::DensZ) * (size_t)d.sc_r);
  d.g_th = (fb::ThetaRec*)tp;   tp += align256(sizeof(fb::ThetaRec) * (size_t)d.sc_r * d.dens_n);
  d.g_irz = nullptr;
  d.g_iry = d.g_irx = nullptr;
  d.g_irmus = nullptr;
  if (mixed) {
    d.g_irz = (fb::IrZ*)tp;   tp += align256(sizeof(fb::IrZ) * (size_t)d.ir_r);
    d.g_iry = (fb::Axis*)tp;  tp += align256(sizeof(fb::Axis) * (size_t)d.ir_r * (d.irr_n / 2));
    d.g_irx = (fb::Axis*)tp;  tp += align256(sizeof(fb::Axis) * (size_t)d.ir_mus * (d.sc_nu + 2));
    d.g_irmus = (float*)tp;   tp += align256(sizeof(float) * (size_t)d.ir_mus);
  }
}

TableSizes sizes_of(const fb_params& p) {
  const fb_params_raw& r = p.raw;
  TableSizes s;
  s.ntr = (size_t)r.transmittance_mu_size * r.transmittance_r_size;
  s.nir = (size_t)r.irradiance_mu_s_size * r.irradiance_r_size;
  s.nsc = (size_t)r.scattering_nu_size * r.scattering_mu_s_size * r.scattering_mu_size * r.scattering_r_size;
  s.out_bytes = align256(16 * s.ntr) + align256(16 * s.nir) + align256(16 * s.nsc);
  const size_t rows = (size_t)r.scattering_mu_size * r.scattering_r_size;
  s.dens_bytes = 12 * rows * (size_t)fb::dens_stride((int)(r.scattering_nu_size * r.scattering_mu_s_size));
  s.tmp_bytes = align256(32 * s.ntr) + 2 * align256(16 * s.nir) + 3 * align256(16 * s.nsc) + align256(s.dens_bytes);
  if (p.precision == FB_PRECISION_MIXED) s.tmp_bytes += align256(24 * s.nsc) + align256(24 * s.nir);
  s.tmp_bytes += geometry_bytes(p);
  return s;
}

}  // namespace fbi

extern "C" int fb_params_device_bytes(const fb_params* p, uint64_t* out_b, uint64_t* tmp_b) {
  int rc = fb_params_validate(p);
  if (rc) return rc;
  fbi::TableSizes s = fbi::sizes_of(*p);
  if (out_b) *out_b = s.out_bytes;
  if (tmp_b) *tmp_b = s.tmp_bytes;
  return FB_OK;
}

// --------------------------------------------------------------- builder ---
struct fb_builder {
  int device = 0;
  int sms = 0;
  int smem_optin = 0;
  cudaStream_t stream = nullptr;
  fb_alloc_fn alloc = nullptr;
  fb_free_fn release = nullptr;
  void* user = nullptr;
  cudaMemPool_t pool = nullptr;  // stream-ordered pool that keeps freed memory for reuse
  int profiling = 0;
  std::atomic<int> refs{1};
  std::mutex mu;
  fbi::Tuning tuning;
};

namespace fbi {

void builder_ref(fb_builder* b) { b->refs.fetch_add(1); }
void builder_unref(fb_builder* b) {
  if (b->refs.fetch_sub(1) == 1) {
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->pool) cudaMemPoolDestroy(b->pool);
    delete b;
  }
}

void* dev_alloc(fb_builder* b, size_t bytes, cudaStream_t s) {
  if (bytes == 0) bytes = 256;
  if (b->alloc) return b->alloc(b->user, bytes, (void*)s);
  void* p = nullptr;
  if (cudaMallocFromPoolAsync(&p, bytes, b->pool, s) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}
void dev_free(fb_builder* b, void* p, cudaStream_t s) {
  if (!p) return;
  if (b->release) {
    b->release(b->user, p, (void*)s);
    return;
  }
  cudaFreeAsync(p, s);
}

int builder_sms(const fb_builder* b) { return b->sms; }
int builder_device(const fb_builder* b) { return b->device; }
cudaStream_t builder_stream(const fb_builder* b) { return b->stream; }
Tuning& builder_tuning(fb_builder* b) { return b->tuning; }
std::mutex& builder_mutex(fb_builder* b) { return b->mu; }
int set_error(int code, const char* msg) { return fail(code, "%s", msg); }

}  // namespace fbi

extern "C" int fb_builder_create(int device, fb_builder** out) {
  if (!out) return fail(FB_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int n = 0;
  FB_CU(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(FB_ERR_INVALID_ARGUMENT, "device %d out of range (%d devices)", device, n);
  FB_CU(cudaSetDevice(device));
  cudaDeviceProp prop;
  FB_CU(cudaGetDeviceProperties(&prop, device));
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, fb::kernel_plain(fb::kPassDensity, 1, 0, false)) != cudaSuccess) {
    cudaGetLastError();
    return fail(FB_ERR_NO_KERNEL, "no sm_103a kernel image loads on device %d (%s, sm_%d%d)", device, prop.name,
                prop.major, prop.minor);
  }
  fb_builder* b = new fb_builder();
  b->device = device;
  b->sms = prop.multiProcessorCount;
  b->smem_optin = (int)prop.sharedMemPerBlockOptin;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return fail(FB_ERR_CUDA, "cudaStreamCreate failed");
  }
  {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    uint64_t keep = ~0ull;
    if (cudaMemPoolCreate(&b->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(b->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      cudaGetLastError();
      cudaStreamDestroy(b->stream);
      delete b;
      return fail(FB_ERR_CUDA, "cannot create the device memory pool");
    }
  }
  for (int mode = 0; mode < 2; ++mode)
    for (int pass = 0; pass < 4; ++pass)
      for (int tpt : {1, 2})
        for (int variant = 0; variant < 12; ++variant) {
        // variants 0..5 (density: occupancy + clamped tables), of order 2 or not
        const void* k = fb::kernel_for(mode == 1, pass, tpt, variant % 6, variant >= 6);
        cudaFuncAttributes kfa;
        if (cudaFuncGetAttributes(&kfa, k) != cudaSuccess ||
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 b->smem_optin - (int)kfa.sharedSizeBytes) != cudaSuccess) {
          cudaGetLastError();
          cudaStreamDestroy(b->stream);
          cudaMemPoolDestroy(b->pool);
          delete b;
          return fail(FB_ERR_CUDA, "cudaFuncSetAttribute failed");
        }
      }
  fbi::tuning_load_default(b->tuning);
  *out = b;
  return FB_OK;
}

extern "C" void fb_builder_destroy(fb_builder* b) {
  if (b) fbi::builder_unref(b);
}

extern "C" int fb_builder_device(const fb_builder* b, int* d) {
  if (!b || !d) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  *d = b->device;
  return FB_OK;
}

extern "C" int fb_builder_sm_count(const fb_builder* b, int* s) {
  if (!b || !s) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  *s = b->sms;
  return FB_OK;
}

extern "C" int fb_builder_set_profiling(fb_builder* b, int enabled) {
  if (!b) return fail(FB_ERR_INVALID_ARGUMENT, "builder is NULL");
  std::lock_guard<std::mutex> g(b->mu);
  b->profiling = enabled ? 1 : 0;
  return FB_OK;
}

extern "C" int fb_builder_set_allocator(fb_builder* b, fb_alloc_fn alloc, fb_free_fn release, void* user) {
  if (!b) return fail(FB_ERR_INVALID_ARGUMENT, "builder is NULL");
  if ((alloc == nullptr) != (release == nullptr))
    return fail(FB_ERR_INVALID_ARGUMENT, "alloc and release must both be set or both be NULL");
  std::lock_guard<std::mutex> g(b->mu);
  b->alloc = alloc;
  b->release = release;
  b->user = user;
  return FB_OK;
}

// ------------------------------------------------------------ atmosphere ---
struct fb_atmosphere {
  fb_builder* b = nullptr;
  fb_params params;
  void* block = nullptr;
  float4* tr = nullptr;
  float4* ir = nullptr;
  float4* sc = nullptr;
  cudaStream_t stream = nullptr;
};

namespace fbi {

fb_atmosphere* atmosphere_new(fb_builder* b, const fb_params& p, cudaStream_t s) {
  TableSizes z = sizes_of(p);
  void* blk = dev_alloc(b, z.out_bytes, s);
  if (!blk) return nullptr;
  fb_atmosphere* a = new fb_atmosphere();
  a->b = b;
  builder_ref(b);
  a->params = p;
  a->block = blk;
  a->stream = s;
  char* c = (char*)blk;
  a->tr = (float4*)c;
  c += align256(16 * z.ntr);
  a->ir = (float4*)c;
  c += align256(16 * z.nir);
  a->sc = (float4*)c;
  return a;
}

void atmosphere_free(fb_atmosphere* a) {
  if (!a) return;
  cudaSetDevice(a->b->device);
  dev_free(a->b, a->block, a->stream);
  builder_unref(a->b);
  delete a;
}

void atmosphere_tables(const fb_atmosphere* a, float4** tr, float4** ir, float4** sc) {
  *tr = a->tr;
  *ir = a->ir;
  *sc = a->sc;
}

const fb_params& atmosphere_params(const fb_atmosphere* a) { return a->params; }
void atmosphere_set_stream(fb_atmosphere* a, cudaStream_t s) { a->stream = s; }

}  // namespace fbi

extern "C" int fb_atmosphere_tables(const fb_atmosphere* a, fb_tables* o) {
  if (!a || !o) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  o->transmittance = a->tr;
  o->irradiance = a->ir;
  o->scattering = a->sc;
  fb_params_extents(&a->params, &o->transmittance_extent, &o->irradiance_extent, &o->scattering_extent);
  return FB_OK;
}

extern "C" int fb_atmosphere_params(const fb_atmosphere* a, fb_params* o) {
  if (!a || !o) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  *o = a->params;
  return FB_OK;
}

extern "C" int fb_atmosphere_copy_to_host(const fb_atmosphere* a, void* stream, float* tr, float* ir, float* sc) {
  if (!a) return fail(FB_ERR_INVALID_ARGUMENT, "atmosphere is NULL");
  FB_CU(cudaSetDevice(a->b->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : a->b->stream;
  fbi::TableSizes z = fbi::sizes_of(a->params);
  if (tr) FB_CU(cudaMemcpyAsync(tr, a->tr, 16 * z.ntr, cudaMemcpyDeviceToHost, s));
  if (ir) FB_CU(cudaMemcpyAsync(ir, a->ir, 16 * z.nir, cudaMemcpyDeviceToHost, s));
  if (sc) FB_CU(cudaMemcpyAsync(sc, a->sc, 16 * z.nsc, cudaMemcpyDeviceToHost, s));
  FB_CU(cudaStreamSynchronize(s));
  return FB_OK;
}

extern "C" int fb_atmosphere_copy_to_host_async(const fb_atmosphere* a, void* stream, float* tr, float* ir,
                                                float* sc) {
  if (!a) return fail(FB_ERR_INVALID_ARGUMENT, "atmosphere is NULL");
  FB_CU(cudaSetDevice(a->b->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : a->b->stream;
  fbi::TableSizes z = fbi::sizes_of(a->params);
  if (tr) FB_CU(cudaMemcpyAsync(tr, a->tr, 16 * z.ntr, cudaMemcpyDeviceToHost, s));
  if (ir) FB_CU(cudaMemcpyAsync(ir, a->ir, 16 * z.nir, cudaMemcpyDeviceToHost, s));
  if (sc) FB_CU(cudaMemcpyAsync(sc, a->sc, 16 * z.nsc, cudaMemcpyDeviceToHost, s));
  return FB_OK;
}

extern "C" int fb_atmosphere_export_scattering_f16(const fb_atmosphere* a, void* stream, uint16_t* out) {
  if (!a || !out) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  FB_CU(cudaSetDevice(a->b->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : a->b->stream;
  fbi::TableSizes z = fbi::sizes_of(a->params);
  void* tmp = fbi::dev_alloc(a->b, 8 * z.nsc, s);
  if (!tmp) return fail(FB_ERR_OUT_OF_MEMORY, "no device memory for the f16 export");
  cudaError_t e = fbi::launch_to_half((const float4*)a->sc, tmp, z.nsc, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp, 8 * z.nsc, cudaMemcpyDeviceToHost, s);
  fbi::dev_free(a->b, tmp, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(FB_ERR_CUDA, "f16 export: %s", cudaGetErrorString(e));
  return FB_OK;
}

extern "C" void fb_atmosphere_destroy(fb_atmosphere* a) { fbi::atmosphere_free(a); }

// ----------------------------------------------------------------- builds ---
struct fb_pending {
  fb_builder* b = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<fb_atmosphere*> atms;
  std::vector<DevAtmo> dev;  // host copy of the per-atmosphere records
  void* temp = nullptr;
  void* plan = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> marks;       // profiling: marks[k] before launch k, marks[k+1] after
  std::vector<fb_launch_profile> prof;  // one record per launch
};

namespace {

struct PlannedLaunch {
  int pass;
  bool mixed;
  int block;  // CTA size
  int tpt;
  int variant;
  int order;
  int nseg;
  int seg_njobs[fb::kMaxSegments];
  int seg_total[fb::kMaxSegments];
  size_t seg_job_off[fb::kMaxSegments];  // offsets (in ints) into the int pool
  size_t seg_off_off[fb::kMaxSegments];
  size_t smem;
  uint64_t texels;
};

struct Plan {
  std::vector<PlannedLaunch> launches;
  std::vector<int> ints;
};

void add_segment(Plan& P, PlannedLaunch& L, int s, const std::vector<int>& jobs, const std::vector<int>& tiles) {
  L.seg_njobs[s] = (int)jobs.size();
  L.seg_job_off[s] = P.ints.size();
  P.ints.insert(P.ints.end(), jobs.begin(), jobs.end());
  L.seg_off_off[s] = P.ints.size();
  int acc = 0;
  for (int t : tiles) {
    P.ints.push_back(acc);
    acc += t;
  }
  L.seg_total[s] = acc;
}

// Occupancy variant of a launch: the tuned variant of its largest atmosphere.
int launch_variant(const std::vector<DevAtmo>& A, const std::vector<int>& jobs, const fbi::Tuning& tun, bool mixed,
                   bool density) {
  int best = -1;
  size_t best_n = 0;
  for (int j : jobs) {
    const size_t n = (size_t)A[j].W * A[j].sc_mu * A[j].sc_r;
    if (best < 0 || n > best_n) {
      best = j;
      best_n = n;
    }
  }
  if (best < 0) return 0;
  const DevAtmo& a = A[best];
  const fbi::TuneEntry* e = fbi::tuning_find(tun, a.sc_r, a.sc_mu, a.sc_mus, a.sc_nu, mixed ? 1 : 0);
  return e ? (density ? e->dens_variant : e->ms_variant) : 0;
}

// smem_limit: dynamic shared memory a launch may use; density launches whose
// power-of-two interval tables would exceed it use the clamped tables.
void plan_group(Plan& P, const std::vector<DevAtmo>& A, const std::vector<int>& group, bool mixed,
                const fbi::Tuning& tun, size_t smem_limit) {
  if (group.empty()) return;
  int max_order = 1;
  for (int j : group) max_order = std::max(max_order, A[j].order);
  auto mk = [&](int pass, int order) {
    PlannedLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.pass = pass;
    L.mixed = mixed;
    L.block = pass == fb::kPassDensity ? fb::kDensThreads : fb::kThreads;
    L.tpt = 1;
    L.order = order;
    return L;
  };
  {  // transmittance + geometry tables
    PlannedLaunch L = mk(fb::kPassTransmittance, 0);
    std::vector<int> tiles, tg;
    for (int j : group) {
      tiles.push_back(fb::tiles_transmittance(A[j].tr_mu, A[j].tr_r));
      tg.push_back(fb::tiles_geometry(
          A[j].W, A[j].sc_mu, A[j].sc_r, mixed ? fb::irgeo_entries(A[j].ir_r, A[j].ir_mus, A[j].irr_n, A[j].sc_nu) : 0));
      L.texels += (uint64_t)A[j].tr_mu * A[j].tr_r;
    }
    add_segment(P, L, 0, group, tiles);
    add_segment(P, L, 1, group, tg);
    L.nseg = 2;
    P.launches.push_back(L);
  }
  {  // single scattering rows + direct irradiance + records for the orders >= 2
    PlannedLaunch L = mk(fb::kPassSingle, 0);
    std::vector<int> t0, t1, t2, t3, multi;
    for (int j : group) {
      const DevAtmo& a = A[j];
      t0.push_back(fb::tiles_rows(a.W, a.sc_mu, a.sc_r));
      t1.push_back(fb::tiles_direct(a.ir_mus, a.ir_r));
      if (a.order >= 2) {
        multi.push_back(j);
        t2.push_back(fb::tiles_msrec(a.sc_mu, a.sc_r, a.ms_steps));
        t3.push_back(fb::tiles_densgeo(a.sc_r, a.dens_n));
      }
      L.smem = std::max(L.smem, fb::ss_smem(a.W, a.ss_steps, a.sc_mus, a.sc_nu));
      L.texels += (uint64_t)a.W * a.sc_mu * a.sc_r + (uint64_t)a.ir_mus * a.ir_r;
    }
    add_segment(P, L, 0, group, t0);
    add_segment(P, L, 1, group, t1);
    add_segment(P, L, 2, multi, t2);
    add_segment(P, L, 3, multi, t3);
    L.nseg = 4;
    P.launches.push_back(L);
  }
  for (int n = 2; n <= max_order; ++n) {
    std::vector<int> jobs;
    for (int j : group)
      if (A[j].order >= n) jobs.push_back(j);
    PlannedLaunch D = mk(fb::kPassDensity, n);
    std::vector<int> t0, t1;
    // the tuned variant (occupancy, + kDensClamped for exact-size tables); the
    // exact-size tables also wherever the power-of-two ones do not fit
    const int tuned = launch_variant(A, jobs, tun, mixed, true);
    bool cl = tuned >= fb::kDensClamped;
    for (int j : jobs) cl |= fb::density_smem(A[j], n == 2, mixed, false) > smem_limit;
    for (int j : jobs) {
      const DevAtmo& a = A[j];
      t0.push_back(fb::tiles_density(a));
      t1.push_back(fb::tiles_indirect(a.ir_mus, a.ir_r, a.irr_n, a.sc_nu, a.W, n - 1 == 1));
      D.smem = std::max(D.smem, fb::density_smem(a, n == 2, mixed, cl));
      D.smem = std::max(D.smem, fb::indirect_smem(a.irr_n, a.sc_nu, a.W, a.ir_mus, n - 1 == 1));
      D.texels += (uint64_t)a.W * a.sc_mu * a.sc_r + (uint64_t)a.ir_mus * a.ir_r;
    }
    add_segment(P, D, 0, jobs, t0);
    add_segment(P, D, 1, jobs, t1);
    D.nseg = 2;
    D.variant = tuned % fb::kDensClamped + (cl ? fb::kDensClamped : 0);
    P.launches.push_back(D);
    PlannedLaunch M = mk(fb::kPassMultiple, n);
    std::vector<int> tm;
    for (int j : jobs) M.block = std::max(M.block, fb::ms_threads(A[j].W));
    for (int j : jobs) {
      const DevAtmo& a = A[j];
      tm.push_back(fb::tiles_multiple(a.W, a.sc_mus, a.ms_steps, a.sc_mu, a.sc_r, M.block));
      M.smem = std::max(M.smem, fb::ms_smem(a.W, a.ms_steps, a.sc_mus, M.block));
      M.tpt = std::max(M.tpt, fb::ms_shape(a.W, a.sc_mus, a.ms_steps, M.block).TPT);
      M.texels += (uint64_t)a.W * a.sc_mu * a.sc_r;
    }
    add_segment(P, M, 0, jobs, tm);
    M.nseg = 1;
    M.variant = fb::ms_block_variant(M.block) >= 0 ? fb::ms_block_variant(M.block)
                                                   : launch_variant(A, jobs, tun, mixed, false);
    bool fixed = M.block == fb::kThreads && M.tpt == 1;
    for (int j : jobs) fixed = fixed && fb::ms_fixed_layout(A[j].W, A[j].sc_mus);
    if (fixed) M.variant += 4;  // 0, 1 -> 4, 5
    P.launches.push_back(M);
  }
}

void fill_devatmo(DevAtmo& d, const fb_params& p, const fbi::Tuning& tun) {
  std::memset(&d, 0, sizeof(d));
  const fb_params_raw& r = p.raw;
  for (int c = 0; c < 3; ++c) {
    d.solar[c] = r.solar_irradiance[c];
    d.rayleigh[c] = r.rayleigh_scattering[c];
    d.mie_sca[c] = r.mie_scattering[c];
    d.mie_ext[c] = r.mie_extinction[c];
    d.albedo[c] = r.ground_albedo[c];
    d.absorption[c] = r.absorption_extinction[c];
  }
  d.sun_radius = r.sun_angular_radius;
  d.bottom = r.bottom_radius;
  d.top = r.top_radius;
  d.g = r.mie_phase_function_g;
  d.mu_s_min = r.mu_s_min;
  const fb_density_profile* src[3] = {&r.rayleigh_density, &r.mie_density, &r.absorption_density};
  fb::Layer* dst[3] = {d.ray_d, d.mie_d, d.abs_d};
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 2; ++l) {
      const fb_density_profile_layer& s = src[k]->layers[l];
      dst[k][l] = fb::Layer{s.width, s.exp_term, s.exp_scale, s.linear_term, s.constant_term};
    }
  d.tr_mu = (int)r.transmittance_mu_size;
  d.tr_r = (int)r.transmittance_r_size;
  d.sc_r = (int)r.scattering_r_size;
  d.sc_mu = (int)r.scattering_mu_size;
  d.sc_mus = (int)r.scattering_mu_s_size;
  d.sc_nu = (int)r.scattering_nu_size;
  d.ir_mus = (int)r.irradiance_mu_s_size;
  d.ir_r = (int)r.irradiance_r_size;
  d.tr_steps = (int)p.transmittance_steps;
  d.ss_steps = (int)p.single_scattering_steps;
  d.ms_steps = (int)p.multiple_scattering_steps;
  d.dens_n = (int)p.density_samples;
  d.irr_n = (int)p.irradiance_samples;
  d.order = (int)p.order;
  d.f16 = p.storage == FB_STORAGE_F16;
  d.W = d.sc_nu * d.sc_mus;
  d.Wd = fb::dens_stride(d.W);
  {
    const double R = d.bottom, T = d.top;
    d.H2d = T * T - R * R;
    d.Hd = std::sqrt(d.H2d);
    d.Hf = (float)d.Hd;
    d.inv_Hf = (float)(1.0 / d.Hd);
    const double span = d.Hd - (T - R);
    d.mus_inv_span = (float)(1.0 / span);
    d.mus_inv_A = (float)(span / (-2.0 * (double)d.mu_s_min * R));
  }
  const fbi::TuneEntry* te = fbi::tuning_find(tun, d.sc_r, d.sc_mu, d.sc_mus, d.sc_nu, (int)p.precision);
  d.dens_S = te ? te->dens_S : 0;
  d.dens_chunk = te ? te->dens_chunk : 0;
}

}  // namespace

namespace fbi {

void pending_destroy(fb_pending* p) {
  if (!p) return;
  cudaSetDevice(p->b->device);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  dev_free(p->b, p->temp, p->stream);
  dev_free(p->b, p->plan, p->stream);
  for (fb_atmosphere* a : p->atms) atmosphere_free(a);
  if (p->done) cudaEventDestroy(p->done);
  for (cudaEvent_t e : p->marks) cudaEventDestroy(e);
  builder_unref(p->b);
  delete p;
}

// Plans and enqueues a build of `count` atmospheres on `s`. With use_graph the
// launch sequence is captured into a CUDA graph and replayed.
int build(fb_builder* b, cudaStream_t s, const fb_params* params, uint32_t count, bool use_graph, fb_pending** out,
          int max_items_per_cta) {
  if (!b || !params || !out || count == 0) return fail(FB_ERR_INVALID_ARGUMENT, "invalid arguments");
  *out = nullptr;
  for (uint32_t i = 0; i < count; ++i) {
    int rc = fb_params_validate(&params[i]);
    if (rc) {
      std::string m = g_err;
      return fail(rc, "atmosphere %u: %s", i, m.c_str());
    }
  }
  FB_CU(cudaSetDevice(b->device));
  fb_pending* P = new fb_pending();
  P->b = b;
  builder_ref(b);
  P->stream = s;
  auto bail = [&](int code, const char* msg) {
    pending_destroy(P);
    return fail(code, "%s", msg);
  };
  if (cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming) != cudaSuccess) return bail(FB_ERR_CUDA, "cudaEventCreate failed");
  // outputs and temporaries
  size_t tmp_total = 0;
  std::vector<TableSizes> sz(count);
  for (uint32_t i = 0; i < count; ++i) {
    sz[i] = sizes_of(params[i]);
    tmp_total += sz[i].tmp_bytes;
  }
  P->temp = dev_alloc(b, tmp_total, s);
  if (!P->temp) return bail(FB_ERR_OUT_OF_MEMORY, "cannot allocate the temporaries");
  P->atms.resize(count, nullptr);
  P->dev.resize(count);
  char* tp = (char*)P->temp;
  Tuning tun;
  {
    std::lock_guard<std::mutex> g(b->mu);
    tun = b->tuning;
  }
  for (uint32_t i = 0; i < count; ++i) {
    fb_atmosphere* a = atmosphere_new(b, params[i], s);
    if (!a) return bail(FB_ERR_OUT_OF_MEMORY, "cannot allocate the output tables");
    P->atms[i] = a;
    DevAtmo& d = P->dev[i];
    fill_devatmo(d, params[i], tun);
    d.tr = a->tr;
    d.ir = a->ir;
    d.sc = a->sc;
    const TableSizes& z = sz[i];
    d.trp = (float*)tp;      tp += align256(32 * z.ntr);
    d.dirr[0] = (float4*)tp; tp += align256(16 * z.nir);
    d.dirr[1] = (float4*)tp; tp += align256(16 * z.nir);
    d.dr = (float4*)tp;      tp += align256(16 * z.nsc);
    d.dm = (float4*)tp;      tp += align256(16 * z.nsc);
    d.dms = (float4*)tp;     tp += align256(16 * z.nsc);
    d.dens = (float*)tp;     tp += align256(z.dens_bytes);
    if (params[i].precision == FB_PRECISION_MIXED) {
      d.sc_acc = (double*)tp; tp += align256(24 * z.nsc);
      d.ir_acc = (double*)tp; tp += align256(24 * z.nir);
    }
    place_geometry(d, tp, params[i].precision == FB_PRECISION_MIXED);
  }
  // work plan
  Plan plan;
  std::vector<int> g_plain, g_mixed;
  for (uint32_t i = 0; i < count; ++i) (params[i].precision == FB_PRECISION_MIXED ? g_mixed : g_plain).push_back((int)i);
  const size_t smem_limit = (size_t)std::max(0, b->smem_optin - 1024);
  plan_group(plan, P->dev, g_plain, false, tun, smem_limit);
  plan_group(plan, P->dev, g_mixed, true, tun, smem_limit);
  const size_t atm_bytes = align256(sizeof(DevAtmo) * count);
  const size_t int_bytes = align256(sizeof(int) * std::max<size_t>(plan.ints.size(), 1));
  const size_t cnt_bytes = align256(sizeof(unsigned) * plan.launches.size());
  P->plan = dev_alloc(b, atm_bytes + int_bytes + cnt_bytes, s);
  if (!P->plan) return bail(FB_ERR_OUT_OF_MEMORY, "cannot allocate the work plan");
  char* pb = (char*)P->plan;
  DevAtmo* d_atm = (DevAtmo*)pb;
  int* d_ints = (int*)(pb + atm_bytes);
  unsigned* d_cnt = (unsigned*)(pb + atm_bytes + int_bytes);
  if (cudaMemcpyAsync(d_atm, P->dev.data(), sizeof(DevAtmo) * count, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      (plan.ints.size() &&
       cudaMemcpyAsync(d_ints, plan.ints.data(), sizeof(int) * plan.ints.size(), cudaMemcpyHostToDevice, s) != cudaSuccess))
    return bail(FB_ERR_CUDA, "plan upload failed");
  // launch configurations
  struct Ready {
    const void* fn;
    LaunchArgs args;
    int grid;
    int block;
    size_t smem;
    fb_launch_profile info;
  };
  std::vector<Ready> ready;
  for (size_t li = 0; li < plan.launches.size(); ++li) {
    const PlannedLaunch& L = plan.launches[li];
    Ready R;
    R.fn = fb::kernel_for(L.mixed, L.pass, L.tpt, L.variant, L.order == 2);
    R.smem = L.smem;
    cudaFuncAttributes kfa;
    if (cudaFuncGetAttributes(&kfa, R.fn) != cudaSuccess) return bail(FB_ERR_CUDA, "cudaFuncGetAttributes failed");
    if ((int)(R.smem + kfa.sharedSizeBytes) > b->smem_optin)
      return bail(FB_ERR_INVALID_PARAMS, "shared memory of a pass exceeds the device limit");
    std::memset(&R.args, 0, sizeof(R.args));
    R.args.atm = d_atm;
    R.args.nseg = L.nseg;
    R.args.order = L.order;
    R.args.counter = d_cnt + li;
    int total = 0;
    for (int sidx = 0; sidx < L.nseg; ++sidx) {
      R.args.seg[sidx].njobs = L.seg_njobs[sidx];
      R.args.seg[sidx].total = L.seg_total[sidx];
      R.args.seg[sidx].job = d_ints + L.seg_job_off[sidx];
      R.args.seg[sidx].off = d_ints + L.seg_off_off[sidx];
      total += L.seg_total[sidx];
    }
    int per_sm = 0;
    R.block = L.block;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, R.fn, R.block, R.smem) != cudaSuccess || per_sm < 1)
      return bail(FB_ERR_CUDA, "occupancy query failed");
    R.args.max_items = std::max(0, max_items_per_cta);
    R.grid = max_items_per_cta > 0 ? std::max(1, (total + max_items_per_cta - 1) / max_items_per_cta)
                                   : std::max(1, std::min(total, per_sm * b->sms));
    std::memset(&R.info, 0, sizeof(R.info));
    R.info.kernel = (uint32_t)L.pass;
    R.info.order = (uint32_t)L.order;
    R.info.precision = L.mixed ? FB_PRECISION_MIXED : FB_PRECISION_PLAIN;
    R.info.grid = (uint32_t)R.grid;
    R.info.items = (uint64_t)total;
    R.info.texels = L.texels;
    if (total > 0) ready.push_back(R);
  }
  int profiling;
  {
    std::lock_guard<std::mutex> g(b->mu);
    profiling = b->profiling;
  }
  if (profiling) {
    P->marks.resize(ready.size() + 1, nullptr);
    for (auto& e : P->marks)
      if (cudaEventCreate(&e) != cudaSuccess) return bail(FB_ERR_CUDA, "cudaEventCreate failed");
    for (const Ready& R : ready) P->prof.push_back(R.info);
  }
  auto enqueue = [&](cudaStream_t st) -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(d_cnt, 0, sizeof(unsigned) * std::max<size_t>(plan.launches.size(), 1), st);
    if (e == cudaSuccess && profiling) e = cudaEventRecord(P->marks[0], st);
    for (size_t k = 0; e == cudaSuccess && k < ready.size(); ++k) {
      void* args[] = {(void*)&ready[k].args};
      e = cudaLaunchKernel(ready[k].fn, dim3(ready[k].grid), dim3(ready[k].block), args, ready[k].smem, st);
      if (e == cudaSuccess && profiling) e = cudaEventRecord(P->marks[k + 1], st);
    }
    return e;
  };
  // Timing events cannot be read back from inside a graph: profiled builds
  // launch the same sequence directly.
  if (use_graph && !profiling) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t e2 = enqueue(s);
      e = cudaStreamEndCapture(s, &graph);
      if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&P->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e == cudaSuccess) e = cudaGraphLaunch(P->exec, s);
    if (e != cudaSuccess) {
      std::string m = std::string("graph build/launch failed: ") + cudaGetErrorString(e);
      cudaGetLastError();
      return bail(FB_ERR_CUDA, m.c_str());
    }
  } else {
    cudaError_t e = enqueue(s);
    if (e != cudaSuccess) {
      std::string m = std::string("kernel launch failed: ") + cudaGetErrorString(e);
      cudaGetLastError();
      return bail(FB_ERR_CUDA, m.c_str());
    }
  }
  if (cudaEventRecord(P->done, s) != cudaSuccess) return bail(FB_ERR_CUDA, "cudaEventRecord failed");
  *out = P;
  return FB_OK;
}

void fill_atmo_record(fb::DevAtmo& d, const fb_params& p) {
  Tuning untuned;
  fill_devatmo(d, p, untuned);
}

fb_atmosphere* pending_detach(fb_pending* p, uint32_t i) {
  if (!p || i >= p->atms.size()) return nullptr;
  fb_atmosphere* a = p->atms[i];
  p->atms[i] = nullptr;
  return a;
}
cudaEvent_t pending_event(fb_pending* p) { return p->done; }
size_t atmosphere_bytes(const fb_atmosphere* a) { return sizes_of(a->params).out_bytes; }

}  // namespace fbi

extern "C" int fb_atmosphere_build(fb_builder* b, void* stream, const fb_params* p, fb_pending** out) {
  if (!b) return fail(FB_ERR_INVALID_ARGUMENT, "builder is NULL");
  return fbi::build(b, stream ? (cudaStream_t)stream : b->stream, p, 1, false, out);
}

extern "C" int fb_batch_build(fb_builder* b, void* stream, const fb_params* params, uint32_t count, fb_pending** out) {
  if (!b) return fail(FB_ERR_INVALID_ARGUMENT, "builder is NULL");
  return fbi::build(b, stream ? (cudaStream_t)stream : b->stream, params, count, true, out);
}

extern "C" int fb_pending_query(fb_pending* p) {
  if (!p) return fail(FB_ERR_INVALID_ARGUMENT, "pending is NULL");
  cudaError_t e = cudaEventQuery(p->done);
  if (e == cudaSuccess) return FB_OK;
  if (e == cudaErrorNotReady) return FB_NOT_READY;
  return fail(FB_ERR_CUDA, "build failed: %s", cudaGetErrorString(e));
}

extern "C" int fb_pending_wait(fb_pending* p) {
  if (!p) return fail(FB_ERR_INVALID_ARGUMENT, "pending is NULL");
  FB_CU(cudaEventSynchronize(p->done));
  return FB_OK;
}

extern "C" int fb_pending_acquire(fb_pending* p, void* consumer) {
  if (!p) return fail(FB_ERR_INVALID_ARGUMENT, "pending is NULL");
  FB_CU(cudaStreamWaitEvent((cudaStream_t)consumer, p->done, 0));
  return FB_OK;
}

extern "C" int fb_pending_count(const fb_pending* p, uint32_t* n) {
  if (!p || !n) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = (uint32_t)p->atms.size();
  return FB_OK;
}

extern "C" int fb_pending_atmosphere(fb_pending* p, uint32_t i, fb_atmosphere** out) {
  if (!p || !out) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (i >= p->atms.size()) return fail(FB_ERR_NOT_FOUND, "index %u out of range", i);
  if (!p->atms[i]) return fail(FB_ERR_NOT_FOUND, "atmosphere %u was taken", i);
  *out = p->atms[i];
  return FB_OK;
}

extern "C" int fb_pending_take(fb_pending* p, uint32_t i, fb_atmosphere** out) {
  int rc = fb_pending_atmosphere(p, i, out);
  if (rc) return rc;
  rc = fb_pending_wait(p);
  if (rc) return rc;
  p->atms[i] = nullptr;
  return FB_OK;
}

extern "C" int fb_pending_intermediates(fb_pending* p, uint32_t i, fb_intermediates* o) {
  if (!p || !o) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (i >= p->dev.size()) return fail(FB_ERR_NOT_FOUND, "index %u out of range", i);
  const DevAtmo& d = p->dev[i];
  o->delta_irradiance[0] = d.dirr[0];
  o->delta_irradiance[1] = d.dirr[1];
  o->delta_rayleigh = d.dr;
  o->delta_mie = d.dm;
  o->delta_multiple_scattering = d.dms;
  o->scattering_density = d.dens;
  o->scattering_density_stride = (uint32_t)d.Wd;
  return FB_OK;
}

extern "C" void fb_pending_release(fb_pending* p) { fbi::pending_destroy(p); }

extern "C" int fb_pending_profile(fb_pending* p, fb_launch_profile* out, uint32_t cap, uint32_t* count) {
  if (!p || !count) return fail(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (p->marks.empty()) return fail(FB_ERR_NOT_FOUND, "profiling was off for this build");
  FB_CU(cudaEventSynchronize(p->done));
  *count = (uint32_t)p->prof.size();
  for (uint32_t k = 0; k < p->prof.size() && k < cap && out; ++k) {
    fb_launch_profile r = p->prof[k];
    FB_CU(cudaEventElapsedTime(&r.ms, p->marks[k], p->marks[k + 1]));
    out[k] = r;
  }
  return FB_OK;
}

// ------------------------------------------------------------ diagnostics ---
extern "C" const char* fb_status_string(int s) {
  switch (s) {
    case FB_OK: return "ok";
    case FB_NOT_READY: return "not ready";
    case FB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FB_ERR_INVALID_PARAMS: return "invalid parameters";
    case FB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FB_ERR_CUDA: return "CUDA error";
    case FB_ERR_BUDGET: return "over the memory budget";
    case FB_ERR_CANCELLED: return "cancelled";
    case FB_ERR_NOT_FOUND: return "not found";
    case FB_ERR_SHUTDOWN: return "shut down";
    case FB_ERR_NO_KERNEL: return "no kernel image for this device";
  }
  return "unknown status";
}

extern "C" const char* fb_last_error(void) { return g_err.c_str(); }
extern "C" int fb_abi_version(void) { return FB_ABI_VERSION; }
