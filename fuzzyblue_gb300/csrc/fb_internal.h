// fb_internal.h — declarations shared by the host-side translation units.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "../../include/fuzzyblue.h"

namespace fbi {

struct TableSizes {
  size_t ntr, nir, nsc;   // texels
  size_t dens_bytes;      // the planar scattering-density table
  size_t out_bytes;       // transmittance + irradiance + scattering
  size_t tmp_bytes;       // temporaries of one build
};
TableSizes sizes_of(const fb_params& p);

// Tile shapes per scattering-table class, chosen by the autotuner
// (fb_builder_autotune) or by the default rule.
struct TuneEntry {
  int sc_r, sc_mu, sc_mus, sc_nu, precision;
  int dens_S, dens_chunk;  // scattering-density tile: mu_s columns x mu rows
  int dens_variant, ms_variant;
  float dens_ms, ms_ms;
};
struct Tuning {
  std::vector<TuneEntry> entries;
};
void tuning_load_default(Tuning& t);
// The entry of a class, or nullptr (default rule, variants 0).
const TuneEntry* tuning_find(const Tuning& t, int sc_r, int sc_mu, int sc_mus, int sc_nu, int precision);
void tuning_set(Tuning& t, const TuneEntry& e);

void builder_ref(fb_builder* b);
void builder_unref(fb_builder* b);
void* dev_alloc(fb_builder* b, size_t bytes, cudaStream_t s);
void dev_free(fb_builder* b, void* p, cudaStream_t s);
int builder_sms(const fb_builder* b);
int builder_device(const fb_builder* b);
cudaStream_t builder_stream(const fb_builder* b);
Tuning& builder_tuning(fb_builder* b);
std::mutex& builder_mutex(fb_builder* b);
int set_error(int code, const char* msg);

fb_atmosphere* atmosphere_new(fb_builder* b, const fb_params& p, cudaStream_t s);
void atmosphere_free(fb_atmosphere* a);
const fb_params& atmosphere_params(const fb_atmosphere* a);
void atmosphere_set_stream(fb_atmosphere* a, cudaStream_t s);
void atmosphere_tables(const fb_atmosphere* a, float4** tr, float4** ir, float4** sc);

// max_items_per_cta > 0: every CTA exits after that many work items and the
// grid covers the launch's items (the request loop uses it so that CTAs of
// concurrent batches on other streams interleave); 0: persistent grids.
int build(fb_builder* b, cudaStream_t s, const fb_params* params, uint32_t count, bool use_graph, fb_pending** out,
          int max_items_per_cta = 0);
void pending_destroy(fb_pending* p);
// Removes atmosphere `index` from the pending handle (ownership to the caller).
fb_atmosphere* pending_detach(fb_pending* p, uint32_t index);
cudaEvent_t pending_event(fb_pending* p);
size_t atmosphere_bytes(const fb_atmosphere* a);

cudaError_t launch_to_half(const float4* src, void* dst, size_t n, cudaStream_t s);

}  // namespace fbi

namespace fb {
struct DevAtmo;
}

namespace fbi {
// The kernels' record of one atmosphere with the default tile shapes (no
// tables set).
void fill_atmo_record(fb::DevAtmo& d, const fb_params& p);
// Points the record's geometry tables at `tp` and advances it past them
// (the last part of the temporaries, sizes_of(p).tmp_bytes counts them).
void place_geometry(fb::DevAtmo& d, char*& tp, bool mixed);

}  // namespace fbi
