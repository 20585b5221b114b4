// fb_tune.cu — tile-shape autotuner (fb_builder_autotune) and its JSON cache.
//
// For one table class (scattering sizes + precision) the tuner builds a small
// batch of that class at order 3 with per-launch timing events, once per
// candidate: every valid scattering-density tile shape (mu_s columns x mu
// rows per 128-thread block) in the three occupancy variants of the density
// kernel (4, 3 or 5 resident blocks per SM), each with power-of-two and with
// exact-size interval tables, then both variants of the multiple-scattering
// kernel. The fastest of each is
// kept in the builder's tuning table, which every later build consults.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fuzzyblue.h"
#include "fb_internal.h"
#include "fb_passes.cuh"

namespace {

struct Cand {
  int S, chunk;
};

std::vector<Cand> density_candidates(const fb_params& p) {
  const fb_params_raw& r = p.raw;
  const fb::DensShape d0 = fb::dens_shape((int)r.scattering_r_size, (int)r.scattering_mu_size,
                                          (int)r.scattering_mu_s_size, (int)r.scattering_nu_size);
  std::vector<Cand> out;
  out.push_back({d0.S, d0.chunk});
  const int mu = (int)r.scattering_mu_size, mus = (int)r.scattering_mu_s_size;
  int chunk = std::min(mu, fb::kDensThreads / d0.NG);
  for (int k = 0; k < 4 && chunk >= 4; ++k, chunk /= 2) {
    const int S = std::max(1, std::min(mus, fb::kDensThreads / (chunk * d0.NG)));
    bool dup = false;
    for (const Cand& c : out) dup |= (c.S == S && c.chunk == chunk);
    if (!dup) out.push_back({S, chunk});
  }
  return out;
}

// Builds `batch` copies of p and returns the device time of the launch of
// `kernel` at `order` (min over `reps`), or a negative value on failure.
float time_launch(fb_builder* b, const std::vector<fb_params>& batch, int kernel, int order, int reps) {
  float best = -1.0f;
  for (int rep = 0; rep < reps; ++rep) {
    fb_pending* pend = nullptr;
    if (fbi::build(b, fbi::builder_stream(b), batch.data(), (uint32_t)batch.size(), false, &pend) != FB_OK)
      return -1.0f;
    fb_launch_profile prof[64];
    uint32_t n = 0;
    int rc = fb_pending_profile(pend, prof, 64, &n);
    fbi::pending_destroy(pend);
    if (rc != FB_OK) return -1.0f;
    for (uint32_t k = 0; k < n && k < 64; ++k)
      if ((int)prof[k].kernel == kernel && (int)prof[k].order == order && (best < 0 || prof[k].ms < best))
        best = prof[k].ms;
  }
  return best;
}

}  // namespace

extern "C" int fb_builder_autotune(fb_builder* b, const fb_params* classes, uint32_t count, uint32_t batch) {
  if (!b || !classes || count == 0) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "invalid arguments");
  for (uint32_t c = 0; c < count; ++c) {
    int rc = fb_params_validate(&classes[c]);
    if (rc) return rc;
  }
  if (batch == 0) batch = 8;
  if (cudaSetDevice(fbi::builder_device(b)) != cudaSuccess) return fbi::set_error(FB_ERR_CUDA, "cudaSetDevice");
  fb_builder_set_profiling(b, 1);
  int status = FB_OK;
  for (uint32_t c = 0; c < count && status == FB_OK; ++c) {
    fb_params p = classes[c];
    p.order = 3;
    const std::vector<fb_params> batchv(batch, p);
    const fb_params_raw& r = p.raw;
    fbi::TuneEntry e;
    std::memset(&e, 0, sizeof(e));
    e.sc_r = (int)r.scattering_r_size;
    e.sc_mu = (int)r.scattering_mu_size;
    e.sc_mus = (int)r.scattering_mu_s_size;
    e.sc_nu = (int)r.scattering_nu_size;
    e.precision = (int)p.precision;
    fbi::TuneEntry best = e;
    best.dens_ms = -1.0f;
    for (const Cand& cd : density_candidates(p)) {
      for (int v = 0; v < 2 * fb::kDensClamped; ++v) {  // occupancy variants, power-of-two and exact-size tables
        fbi::TuneEntry t = e;
        t.dens_S = cd.S;
        t.dens_chunk = cd.chunk;
        t.dens_variant = v;
        {
          std::lock_guard<std::mutex> g(fbi::builder_mutex(b));
          fbi::tuning_set(fbi::builder_tuning(b), t);
        }
        const float ms = time_launch(b, batchv, FB_KERNEL_DENSITY, 3, 2);
        if (ms < 0) continue;  // a candidate that cannot launch here (e.g. its shared memory) is skipped
        if (best.dens_ms < 0 || ms < best.dens_ms) {
          best = t;
          best.dens_ms = ms;
        }
      }
    }
    if (best.dens_ms < 0) {
      status = fbi::set_error(FB_ERR_CUDA, "autotune: no density candidate could be built");
      break;
    }
    best.ms_ms = -1.0f;
    for (int v = 0; v < 2; ++v) {
      fbi::TuneEntry t = best;
      t.ms_variant = v;
      {
        std::lock_guard<std::mutex> g(fbi::builder_mutex(b));
        fbi::tuning_set(fbi::builder_tuning(b), t);
      }
      const float ms = time_launch(b, batchv, FB_KERNEL_MULTIPLE, 3, 2);
      if (ms < 0) continue;
      if (best.ms_ms < 0 || ms < best.ms_ms) {
        best.ms_variant = v;
        best.ms_ms = ms;
      }
    }
    std::lock_guard<std::mutex> g(fbi::builder_mutex(b));
    fbi::tuning_set(fbi::builder_tuning(b), best);
  }
  fb_builder_set_profiling(b, 0);
  return status;
}

extern "C" int fb_builder_tuned_shape(const fb_builder* b, const fb_params* p, fb_tile_shape* out) {
  if (!b || !p || !out) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  fb_builder* mb = const_cast<fb_builder*>(b);
  std::lock_guard<std::mutex> g(fbi::builder_mutex(mb));
  const fb_params_raw& r = p->raw;
  const fbi::TuneEntry* e = fbi::tuning_find(fbi::builder_tuning(mb), (int)r.scattering_r_size,
                                             (int)r.scattering_mu_size, (int)r.scattering_mu_s_size,
                                             (int)r.scattering_nu_size, (int)p->precision);
  if (!e) return fbi::set_error(FB_ERR_NOT_FOUND, "class not tuned");
  out->density_columns = (uint32_t)e->dens_S;
  out->density_rows = (uint32_t)e->dens_chunk;
  out->density_variant = (uint32_t)e->dens_variant;
  out->multiple_variant = (uint32_t)e->ms_variant;
  out->density_ms = e->dens_ms;
  out->multiple_ms = e->ms_ms;
  return FB_OK;
}

extern "C" int fb_builder_save_tuning(fb_builder* b, const char* path) {
  if (!b || !path) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  std::vector<fbi::TuneEntry> v;
  {
    std::lock_guard<std::mutex> g(fbi::builder_mutex(b));
    v = fbi::builder_tuning(b).entries;
  }
  FILE* f = fopen(path, "w");
  if (!f) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "cannot open the tuning file for writing");
  fprintf(f, "{\"fuzzyblue_tuning\": 1, \"classes\": [\n");
  for (size_t i = 0; i < v.size(); ++i) {
    const fbi::TuneEntry& e = v[i];
    fprintf(f,
            "  {\"sc_r\": %d, \"sc_mu\": %d, \"sc_mus\": %d, \"sc_nu\": %d, \"precision\": %d, \"dens_S\": %d, "
            "\"dens_chunk\": %d, \"dens_variant\": %d, \"ms_variant\": %d, \"dens_ms\": %.6g, \"ms_ms\": %.6g}%s\n",
            e.sc_r, e.sc_mu, e.sc_mus, e.sc_nu, e.precision, e.dens_S, e.dens_chunk, e.dens_variant, e.ms_variant,
            e.dens_ms, e.ms_ms, i + 1 < v.size() ? "," : "");
  }
  fprintf(f, "]}\n");
  fclose(f);
  return FB_OK;
}

namespace {
// Reads `"key": number` from one JSON object's text.
bool json_num(const std::string& obj, const char* key, double* out) {
  const std::string k = std::string("\"") + key + "\"";
  size_t at = obj.find(k);
  if (at == std::string::npos) return false;
  at = obj.find(':', at + k.size());
  if (at == std::string::npos) return false;
  return sscanf(obj.c_str() + at + 1, "%lf", out) == 1;
}
}  // namespace

extern "C" int fb_builder_load_tuning(fb_builder* b, const char* path) {
  if (!b || !path) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  FILE* f = fopen(path, "r");
  if (!f) return fbi::set_error(FB_ERR_NOT_FOUND, "cannot open the tuning file");
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  fclose(f);
  if (text.find("\"fuzzyblue_tuning\"") == std::string::npos)
    return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "not a tuning file");
  const size_t cls = text.find("\"classes\"");
  if (cls == std::string::npos) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "no classes in the tuning file");
  std::vector<fbi::TuneEntry> got;
  size_t pos = cls;
  while ((pos = text.find('{', pos)) != std::string::npos) {
    const size_t end = text.find('}', pos);
    if (end == std::string::npos) break;
    const std::string obj = text.substr(pos, end - pos + 1);
    pos = end + 1;
    const char* keys[11] = {"sc_r", "sc_mu", "sc_mus", "sc_nu", "precision", "dens_S",
                            "dens_chunk", "dens_variant", "ms_variant", "dens_ms", "ms_ms"};
    double v[11];
    bool ok = true;
    for (int k = 0; k < 11 && ok; ++k) ok = json_num(obj, keys[k], &v[k]);
    if (!ok) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "malformed class in the tuning file");
    fbi::TuneEntry e;
    e.sc_r = (int)v[0];
    e.sc_mu = (int)v[1];
    e.sc_mus = (int)v[2];
    e.sc_nu = (int)v[3];
    e.precision = (int)v[4];
    e.dens_S = (int)v[5];
    e.dens_chunk = (int)v[6];
    e.dens_variant = std::min(2 * fb::kDensClamped - 1, std::max(0, (int)v[7]));
    e.ms_variant = std::min(1, std::max(0, (int)v[8]));
    e.dens_ms = (float)v[9];
    e.ms_ms = (float)v[10];
    if (e.dens_S < 0 || e.dens_chunk < 0) return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "bad tile shape");
    got.push_back(e);
  }
  std::lock_guard<std::mutex> g(fbi::builder_mutex(b));
  for (const fbi::TuneEntry& e : got) fbi::tuning_set(fbi::builder_tuning(b), e);
  return FB_OK;
}
