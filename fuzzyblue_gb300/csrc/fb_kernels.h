// fb_kernels.h — host-side entry points of the pass kernels (internal).
#pragma once
#include <cuda_runtime.h>

#include "fb_passes.cuh"

namespace fb {

enum PassKind { kPassTransmittance = 0, kPassSingle = 1, kPassDensity = 2, kPassMultiple = 3 };

// Kernel of (mode, pass, texels-per-thread, variant, order 2). Multiple
// scattering: variant 0 / 1 = CTAs of kThreads with registers for 4 / 3 CTAs
// per SM (tpt 1), variant 2 / 3 = CTAs of kMsWideThreads / kMsMidThreads
// (tpt 1 or 2). Density:
// variant 0 / 1 = registers for 4 / 3 CTAs per SM; order2 selects the launch
// of order 2 (it reads the single-scattering tables).
const void* kernel_plain(int pass, int tpt, int variant, bool order2);
const void* kernel_mixed(int pass, int tpt, int variant, bool order2);

inline const void* kernel_for(bool mixed, int pass, int tpt, int variant = 0, bool order2 = false) {
  return mixed ? kernel_mixed(pass, tpt, variant, order2) : kernel_plain(pass, tpt, variant, order2);
}

}  // namespace fb
