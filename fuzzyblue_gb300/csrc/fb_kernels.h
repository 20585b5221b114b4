// fb_kernels.h — host-side entry points of the pass kernels (internal).
#pragma once
#include <cuda_runtime.h>

#include "fb_passes.cuh"

namespace fb {

enum PassKind { kPassTransmittance = 0, kPassSingle = 1, kPassDensity = 2, kPassMultiple = 3 };

// Kernel of (mode, pass, texels-per-thread, occupancy variant, order 2); tpt
// is used by kPassMultiple only (1, 2, 4 or 8); variant (0 or 1) by the
// density and multiple-scattering passes; order2 by the density pass (the
// launch of order 2 reads the single-scattering tables).
const void* kernel_plain(int pass, int tpt, int variant, bool order2);
const void* kernel_mixed(int pass, int tpt, int variant, bool order2);

inline const void* kernel_for(bool mixed, int pass, int tpt, int variant = 0, bool order2 = false) {
  return mixed ? kernel_mixed(pass, tpt, variant, order2) : kernel_plain(pass, tpt, variant, order2);
}

inline int tpt_for_width(int W) {
  const int n = (W + kThreads - 1) / kThreads;
  return n <= 1 ? 1 : n <= 2 ? 2 : n <= 4 ? 4 : 8;
}

}  // namespace fb
