// fb_kernels_mixed.cu — MIXED instantiation of the passes (FP64 ray state,
// Kahan sums, FP64 order accumulation); default FMA contraction.
#include "fb_kernels.h"

namespace fb {

template __global__ void k_transmittance<true>(LaunchArgs);
template __global__ void k_single<true>(LaunchArgs);
template __global__ void k_density<true, 0>(LaunchArgs);
template __global__ void k_density<true, 1>(LaunchArgs);
template __global__ void k_multiple<true, 1, 0>(LaunchArgs);
template __global__ void k_multiple<true, 2, 0>(LaunchArgs);
template __global__ void k_multiple<true, 4, 0>(LaunchArgs);
template __global__ void k_multiple<true, 8, 0>(LaunchArgs);
template __global__ void k_multiple<true, 1, 1>(LaunchArgs);
template __global__ void k_multiple<true, 2, 1>(LaunchArgs);
template __global__ void k_multiple<true, 4, 1>(LaunchArgs);
template __global__ void k_multiple<true, 8, 1>(LaunchArgs);

const void* kernel_mixed(int pass, int tpt, int variant) {
  const bool v1 = variant == 1;
  switch (pass) {
    case kPassTransmittance: return (const void*)k_transmittance<true>;
    case kPassSingle: return (const void*)k_single<true>;
    case kPassDensity: return v1 ? (const void*)k_density<true, 1> : (const void*)k_density<true, 0>;
    case kPassMultiple:
      switch (tpt) {
        case 1: return v1 ? (const void*)k_multiple<true, 1, 1> : (const void*)k_multiple<true, 1, 0>;
        case 2: return v1 ? (const void*)k_multiple<true, 2, 1> : (const void*)k_multiple<true, 2, 0>;
        case 4: return v1 ? (const void*)k_multiple<true, 4, 1> : (const void*)k_multiple<true, 4, 0>;
        default: return v1 ? (const void*)k_multiple<true, 8, 1> : (const void*)k_multiple<true, 8, 0>;
      }
  }
  return nullptr;
}

}  // namespace fb
