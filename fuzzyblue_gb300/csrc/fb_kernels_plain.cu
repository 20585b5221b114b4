// fb_kernels_plain.cu — PLAIN (FP32) instantiation of the passes. Compiled with
// --fmad=false: every product and sum rounds separately, as in the reference's
// shaders; explicit fmaf() remains only in interpolation and accumulation.
#include "fb_kernels.h"

namespace fb {

template __global__ void k_transmittance<false>(LaunchArgs);
template __global__ void k_single<false>(LaunchArgs);
template __global__ void k_density<false>(LaunchArgs);
template __global__ void k_multiple<false, 1>(LaunchArgs);
template __global__ void k_multiple<false, 2>(LaunchArgs);
template __global__ void k_multiple<false, 4>(LaunchArgs);
template __global__ void k_multiple<false, 8>(LaunchArgs);

const void* kernel_plain(int pass, int tpt) {
  switch (pass) {
    case kPassTransmittance: return (const void*)k_transmittance<false>;
    case kPassSingle: return (const void*)k_single<false>;
    case kPassDensity: return (const void*)k_density<false>;
    case kPassMultiple:
      switch (tpt) {
        case 1: return (const void*)k_multiple<false, 1>;
        case 2: return (const void*)k_multiple<false, 2>;
        case 4: return (const void*)k_multiple<false, 4>;
        default: return (const void*)k_multiple<false, 8>;
      }
  }
  return nullptr;
}

}  // namespace fb
