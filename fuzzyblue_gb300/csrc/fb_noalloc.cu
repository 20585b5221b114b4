// fb_noalloc.cu — fb_atmosphere_build_noalloc: one atmosphere built without
// any device allocation.
//
// Who needs this: callers that may not allocate device memory, neither
// directly nor through a library. Examples are an engine that owns every
// device allocation through its own pool and forbids outside allocations, and
// a render loop in which the device-wide synchronisation that an allocation
// can imply would stall frames. They hand in the three output tables they own;
// every temporary of the build (work lists, the order-to-order tables, the
// FP64 accumulators of the mixed mode) lives in one fixed scratch array,
// g_scratch below, that every GPU which loads this library holds until the
// process exits.
//
// Limits and rules: the scratch holds kNoAllocScratchBytes (16 MiB), enough
// for the r16 mu64 mu_s16 nu4 class in either precision; larger builds are
// refused with FB_ERR_BUDGET. All calls share the array and it keeps the last
// call's contents, so each call clears what must start at zero (the work
// counters; every table is written before it is read), and calls whose GPU
// work overlaps race on it: serialise them (one stream, or events). The first
// call on a device sets that device up (looks up the scratch address and
// raises the kernels' shared-memory limits); make that first call before any
// stream capture.
//
// Every check (parameters, scratch size, each launch's shared memory and
// occupancy) runs before anything is enqueued, so a call that returns an error
// has enqueued nothing and left the output tables and the scratch untouched.
// The per-atmosphere record and the work lists are written on the device by a
// small kernel from its launch arguments: a call copies nothing from host
// memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/fuzzyblue.h"
#include "fb_internal.h"
#include "fb_kernels.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;
constexpr int kMaxDevices = 64;
constexpr int kMaxLaunches = 2 + 2 * 64;                       // T, S, then D and M for orders 2..64
constexpr int kNumInts = 2 * fb::kMaxSegments * kMaxLaunches;  // per launch and segment: a job id, an offset

static __device__ __align__(256) unsigned char g_scratch[kNoAllocScratchBytes];

// The record travels as a launch argument (copied by the launch itself).
static_assert(sizeof(fb::DevAtmo) <= 4000, "the atmosphere record must fit in a kernel's arguments");

// Writes the atmosphere record into the scratch and clears the work lists (one
// job, id 0, at offset 0) and the launches' work counters.
__global__ void k_noalloc_prepare(fb::DevAtmo d, fb::DevAtmo* dst, int* ints, unsigned* counters) {
  const int t = threadIdx.x;
  const int* src = reinterpret_cast<const int*>(&d);
  int* out = reinterpret_cast<int*>(dst);
  for (int i = t; i < (int)(sizeof(fb::DevAtmo) / sizeof(int)); i += blockDim.x) out[i] = src[i];
  for (int i = t; i < kNumInts; i += blockDim.x) ints[i] = 0;
  for (int i = t; i < kMaxLaunches; i += blockDim.x) counters[i] = 0u;
}
static_assert(sizeof(fb::DevAtmo) % sizeof(int) == 0, "the record is copied as ints");

struct DeviceSetup {
  bool done = false;
  unsigned char* scratch = nullptr;  // device address of g_scratch
  int sms = 0;
  int smem_optin = 0;
};

std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Once per device, with that device current: the scratch address and every
// pass kernel's dynamic shared-memory limit (the same kernels the builder sets
// up: variants 0..5, of order 2 or not).
int setup_device(int dev, DeviceSetup** out) {
  std::lock_guard<std::mutex> g(g_setup_mu);
  DeviceSetup& d = g_setup[dev];
  if (!d.done) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fbi::set_error(FB_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
      cudaGetLastError();
      return fbi::set_error(FB_ERR_CUDA, "cudaGetDeviceProperties failed");
    }
    for (int mode = 0; mode < 2; ++mode)
      for (int pass = 0; pass < 4; ++pass)
        for (int tpt : {1, 2})
          for (int variant = 0; variant < 12; ++variant) {
            const void* k = fb::kernel_for(mode == 1, pass, tpt, variant % 6, variant >= 6);
            cudaFuncAttributes fa;
            if (cudaFuncGetAttributes(&fa, k) != cudaSuccess ||
                cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)prop.sharedMemPerBlockOptin - (int)fa.sharedSizeBytes) != cudaSuccess) {
              cudaGetLastError();
              return fbi::set_error(FB_ERR_NO_KERNEL, "no sm_103a kernel image loads on this device");
            }
          }
    d.scratch = static_cast<unsigned char*>(ptr);
    d.sms = prop.multiProcessorCount;
    d.smem_optin = (int)prop.sharedMemPerBlockOptin;
    d.done = true;
  }
  *out = &d;
  return FB_OK;
}

// A launch with its grid decided and its checks passed.
struct Launch {
  const void* fn;
  fb::LaunchArgs args;
  int grid;
  int block;
  size_t smem;
};

}  // namespace

extern "C" int fb_atmosphere_build_noalloc(void* stream, const fb_params* p, void* transmittance, void* irradiance,
                                           void* scattering) {
  if (!p || !transmittance || !irradiance || !scattering)
    return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (((uintptr_t)transmittance | (uintptr_t)irradiance | (uintptr_t)scattering) & 15u)
    return fbi::set_error(FB_ERR_INVALID_ARGUMENT, "output tables must be 16-byte aligned");
  int rc = fb_params_validate(p);
  if (rc) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fbi::set_error(FB_ERR_CUDA, "no current CUDA device");
  }
  DeviceSetup* ds = nullptr;
  rc = setup_device(dev, &ds);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  // layout of the scratch: record, work lists, counters, temporaries
  const fbi::TableSizes z = fbi::sizes_of(*p);
  const bool mixed = p->precision == FB_PRECISION_MIXED;
  size_t off = 0;
  const size_t o_atm = off;
  off = align256(off + sizeof(fb::DevAtmo));
  const size_t o_ints = off;
  off = align256(off + sizeof(int) * kNumInts);
  const size_t o_cnt = off;
  off = align256(off + sizeof(unsigned) * kMaxLaunches);
  const size_t o_tmp = off;
  off += z.tmp_bytes;
  if (off > kNoAllocScratchBytes) {
    char msg[160];
    snprintf(msg, sizeof(msg), "this build needs %zu bytes of scratch; the fixed no-alloc scratch holds %zu", off,
             kNoAllocScratchBytes);
    return fbi::set_error(FB_ERR_BUDGET, msg);
  }
  unsigned char* base = ds->scratch;
  fb::DevAtmo d;
  fbi::fill_atmo_record(d, *p);
  d.tr = (float4*)transmittance;
  d.ir = (float4*)irradiance;
  d.sc = (float4*)scattering;
  unsigned char* tp = base + o_tmp;
  d.trp = (float*)tp;      tp += align256(32 * z.ntr);
  d.dirr[0] = (float4*)tp; tp += align256(16 * z.nir);
  d.dirr[1] = (float4*)tp; tp += align256(16 * z.nir);
  d.dr = (float4*)tp;      tp += align256(16 * z.nsc);
  d.dm = (float4*)tp;      tp += align256(16 * z.nsc);
  d.dms = (float4*)tp;     tp += align256(16 * z.nsc);
  d.dens = (float*)tp;     tp += align256(z.dens_bytes);
  if (mixed) {
    d.sc_acc = (double*)tp; tp += align256(24 * z.nsc);
    d.ir_acc = (double*)tp; tp += align256(24 * z.nir);
  }
  {
    char* gp = (char*)tp;
    fbi::place_geometry(d, gp, mixed);
  }
  fb::DevAtmo* d_atm = (fb::DevAtmo*)(base + o_atm);
  int* d_ints = (int*)(base + o_ints);
  unsigned* d_cnt = (unsigned*)(base + o_cnt);

  // launches of the pass order (src/precompute.rs:1726-1999), one job each;
  // launch k uses work counter k and work-list ints [2 kMaxSegments k, ...).
  // Each is checked and its grid decided here; launches without work items
  // (order 1 has none after the first two) are left out.
  std::vector<Launch> L;
  int slot = 0;
  auto add = [&](int pass, int order, std::vector<int> tiles, size_t smem, int tpt, int block,
                 int variant) -> int {
    const int k = slot++;
    Launch l;
    std::memset(&l, 0, sizeof(l));
    l.fn = fb::kernel_for(mixed, pass, tpt, variant, order == 2);
    l.block = block;
    l.smem = smem;
    l.args.atm = d_atm;
    l.args.nseg = (int)tiles.size();
    l.args.order = order;
    l.args.counter = d_cnt + k;
    int total = 0;
    for (int sgi = 0; sgi < (int)tiles.size(); ++sgi) {
      const size_t at = 2 * (fb::kMaxSegments * (size_t)k + sgi);
      l.args.seg[sgi].njobs = 1;
      l.args.seg[sgi].total = tiles[sgi];
      l.args.seg[sgi].job = d_ints + at;
      l.args.seg[sgi].off = d_ints + at + 1;
      total += tiles[sgi];
    }
    if (total == 0) return FB_OK;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, l.fn) != cudaSuccess) {
      cudaGetLastError();
      return fbi::set_error(FB_ERR_CUDA, "cudaFuncGetAttributes failed");
    }
    if ((int)(l.smem + fa.sharedSizeBytes) > ds->smem_optin)
      return fbi::set_error(FB_ERR_INVALID_PARAMS, "shared memory of a pass exceeds the device limit");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, l.fn, l.block, l.smem) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      return fbi::set_error(FB_ERR_CUDA, "occupancy query failed: a pass cannot be resident on this device");
    }
    l.grid = std::max(1, std::min(total, per_sm * ds->sms));
    L.push_back(l);
    return FB_OK;
  };
  const bool multi = d.order >= 2;
  rc = add(fb::kPassTransmittance, 0,
           {fb::tiles_transmittance(d.tr_mu, d.tr_r),
            fb::tiles_geometry(d.W, d.sc_mu, d.sc_r, mixed ? fb::irgeo_entries(d.ir_r, d.ir_mus, d.irr_n, d.sc_nu) : 0)},
           0, 1, fb::kThreads, 0);
  if (!rc)
    rc = add(fb::kPassSingle, 0,
             {fb::tiles_rows(d.W, d.sc_mu, d.sc_r), fb::tiles_direct(d.ir_mus, d.ir_r),
              multi ? fb::tiles_msrec(d.sc_mu, d.sc_r, d.ms_steps) : 0, multi ? fb::tiles_densgeo(d.sc_r, d.dens_n) : 0},
             fb::ss_smem(d.W, d.ss_steps, d.sc_mus, d.sc_nu), 1, fb::kThreads, 0);
  const int ms_block = fb::ms_threads(d.W);
  const int ms_tpt = fb::ms_shape(d.W, d.sc_mus, d.ms_steps, ms_block).TPT;
  const int ms_variant = fb::ms_block_variant(ms_block) >= 0 ? fb::ms_block_variant(ms_block)
                         : (ms_tpt == 1 && fb::ms_fixed_layout(d.W, d.sc_mus) ? 4 : 0);
  for (int n = 2; !rc && n <= d.order; ++n) {
    const bool cl = fb::density_smem(d, n == 2, mixed, false) > (size_t)std::max(0, ds->smem_optin - 1024);
    const size_t sm = std::max(fb::density_smem(d, n == 2, mixed, cl), fb::indirect_smem(d.irr_n, d.sc_nu, d.W, d.ir_mus, n - 1 == 1));
    rc = add(fb::kPassDensity, n, {fb::tiles_density(d), fb::tiles_indirect(d.ir_mus, d.ir_r, d.irr_n, d.sc_nu, d.W, n - 1 == 1)}, sm, 1,
             fb::kDensThreads, cl ? fb::kDensClamped : 0);
    if (!rc)
      rc = add(fb::kPassMultiple, n, {fb::tiles_multiple(d.W, d.sc_mus, d.ms_steps, d.sc_mu, d.sc_r, ms_block)},
               fb::ms_smem(d.W, d.ms_steps, d.sc_mus, ms_block), ms_tpt, ms_block, ms_variant);
  }
  if (rc) return rc;

  // enqueue: the record and cleared work lists, then the passes
  void* pargs[] = {(void*)&d, (void*)&d_atm, (void*)&d_ints, (void*)&d_cnt};
  cudaError_t e = cudaLaunchKernel((const void*)k_noalloc_prepare, dim3(1), dim3(256), pargs, 0, st);
  for (size_t k = 0; e == cudaSuccess && k < L.size(); ++k) {
    void* args[] = {(void*)&L[k].args};
    e = cudaLaunchKernel(L[k].fn, dim3(L[k].grid), dim3(L[k].block), args, L[k].smem, st);
  }
  if (e != cudaSuccess) {
    const char* m = cudaGetErrorString(e);
    cudaGetLastError();
    return fbi::set_error(FB_ERR_CUDA, m);
  }
  return FB_OK;
}
