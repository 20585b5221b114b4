// fb_kernels_mixed.cu — MIXED instantiation of the passes (FP64 ray state,
// Kahan sums, FP64 order accumulation); default FMA contraction.
#include "fb_kernels.h"

namespace fb {

template __global__ void k_transmittance<true>(LaunchArgs);
template __global__ void k_single<true>(LaunchArgs);
template __global__ void k_density<true>(LaunchArgs);
template __global__ void k_multiple<true, 1>(LaunchArgs);
template __global__ void k_multiple<true, 2>(LaunchArgs);
template __global__ void k_multiple<true, 4>(LaunchArgs);
template __global__ void k_multiple<true, 8>(LaunchArgs);

const void* kernel_mixed(int pass, int tpt) {
  switch (pass) {
    case kPassTransmittance: return (const void*)k_transmittance<true>;
    case kPassSingle: return (const void*)k_single<true>;
    case kPassDensity: return (const void*)k_density<true>;
    case kPassMultiple:
      switch (tpt) {
        case 1: return (const void*)k_multiple<true, 1>;
        case 2: return (const void*)k_multiple<true, 2>;
        case 4: return (const void*)k_multiple<true, 4>;
        default: return (const void*)k_multiple<true, 8>;
      }
  }
  return nullptr;
}

}  // namespace fb
