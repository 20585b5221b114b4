// fb_kernels_mixed.cu — MIXED instantiation of the passes (FP64 ray state,
// Kahan sums, FP64 order accumulation); default FMA contraction.
#include "fb_kernels.h"

namespace fb {

template __global__ void k_transmittance<true>(LaunchArgs);
template __global__ void k_single<true>(LaunchArgs);
template __global__ void k_multiple<true, 1, 0>(LaunchArgs);
template __global__ void k_multiple<true, 1, 1>(LaunchArgs);
template __global__ void k_multiple<true, 1, 2>(LaunchArgs);
template __global__ void k_multiple<true, 2, 2>(LaunchArgs);
template __global__ void k_multiple<true, 1, 3>(LaunchArgs);
template __global__ void k_multiple<true, 2, 3>(LaunchArgs);
template __global__ void k_multiple<true, 1, 4>(LaunchArgs);
template __global__ void k_multiple<true, 1, 5>(LaunchArgs);

template __global__ void k_density<true, 0, false, false>(LaunchArgs);
template __global__ void k_density<true, 1, false, false>(LaunchArgs);
template __global__ void k_density<true, 2, false, false>(LaunchArgs);
template __global__ void k_density<true, 0, true, false>(LaunchArgs);
template __global__ void k_density<true, 1, true, false>(LaunchArgs);
template __global__ void k_density<true, 2, true, false>(LaunchArgs);
template __global__ void k_density<true, 0, false, true>(LaunchArgs);
template __global__ void k_density<true, 1, false, true>(LaunchArgs);
template __global__ void k_density<true, 2, false, true>(LaunchArgs);
template __global__ void k_density<true, 0, true, true>(LaunchArgs);
template __global__ void k_density<true, 1, true, true>(LaunchArgs);
template __global__ void k_density<true, 2, true, true>(LaunchArgs);

const void* kernel_mixed(int pass, int tpt, int variant, bool order2) {
  const bool v1 = variant == 1;
  switch (pass) {
    case kPassTransmittance: return (const void*)k_transmittance<true>;
    case kPassSingle: return (const void*)k_single<true>;
    case kPassDensity: {
      // variant: occupancy variant (0..2) + kDensClamped for clamped tables
      static const void* const k[2][2][3] = {
          {{(const void*)k_density<true, 0, false, false>, (const void*)k_density<true, 1, false, false>,
            (const void*)k_density<true, 2, false, false>},
           {(const void*)k_density<true, 0, true, false>, (const void*)k_density<true, 1, true, false>,
            (const void*)k_density<true, 2, true, false>}},
          {{(const void*)k_density<true, 0, false, true>, (const void*)k_density<true, 1, false, true>,
            (const void*)k_density<true, 2, false, true>},
           {(const void*)k_density<true, 0, true, true>, (const void*)k_density<true, 1, true, true>,
            (const void*)k_density<true, 2, true, true>}}};
      const int v = variant < 0 ? 0 : variant;
      return k[v >= kDensClamped ? 1 : 0][order2 ? 1 : 0][(v % kDensClamped) % 3];
    }
    case kPassMultiple:
      if (variant == 2) return tpt >= 2 ? (const void*)k_multiple<true, 2, 2> : (const void*)k_multiple<true, 1, 2>;
      if (variant == 3) return tpt >= 2 ? (const void*)k_multiple<true, 2, 3> : (const void*)k_multiple<true, 1, 3>;
      if (variant == 4 && tpt == 1) return (const void*)k_multiple<true, 1, 4>;
      if (variant == 5 && tpt == 1) return (const void*)k_multiple<true, 1, 5>;
      return v1 || variant == 5 ? (const void*)k_multiple<true, 1, 1> : (const void*)k_multiple<true, 1, 0>;
  }
  return nullptr;
}

}  // namespace fb
