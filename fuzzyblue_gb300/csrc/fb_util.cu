// fb_util.cu — small device utilities and the default tile-shape rule.
#include <cuda_fp16.h>

#include <algorithm>

#include "fb_internal.h"

namespace {

// RGBA32F -> RGBA16F, round to nearest even (the reference's scattering image
// format, src/precompute.rs:1215).
__global__ void k_to_half(const float4* __restrict__ src, uint2* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float4 v = src[i];
    __half2 lo = __floats2half2_rn(v.x, v.y), hi = __floats2half2_rn(v.z, v.w);
    uint2 o;
    o.x = *reinterpret_cast<unsigned*>(&lo);
    o.y = *reinterpret_cast<unsigned*>(&hi);
    dst[i] = o;
  }
}

}  // namespace

namespace fbi {

cudaError_t launch_to_half(const float4* src, void* dst, size_t n, cudaStream_t s) {
  const int threads = 256;
  const size_t blocks = std::min<size_t>((n + threads - 1) / threads, 65535);
  k_to_half<<<(unsigned)std::max<size_t>(blocks, 1), threads, 0, s>>>(src, (uint2*)dst, n);
  return cudaGetLastError();
}

void tuning_load_default(Tuning& t) { t.entries.clear(); }

const TuneEntry* tuning_find(const Tuning& t, int sc_r, int sc_mu, int sc_mus, int sc_nu, int precision) {
  for (const TuneEntry& e : t.entries)
    if (e.sc_r == sc_r && e.sc_mu == sc_mu && e.sc_mus == sc_mus && e.sc_nu == sc_nu && e.precision == precision)
      return &e;
  return nullptr;
}

void tuning_set(Tuning& t, const TuneEntry& e) {
  for (TuneEntry& x : t.entries)
    if (x.sc_r == e.sc_r && x.sc_mu == e.sc_mu && x.sc_mus == e.sc_mus && x.sc_nu == e.sc_nu &&
        x.precision == e.precision) {
      x = e;
      return;
    }
  t.entries.push_back(e);
}

}  // namespace fbi
