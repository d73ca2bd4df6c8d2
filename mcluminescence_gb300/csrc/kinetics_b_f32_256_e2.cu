// FP32 Bernoulli kernel, 256 threads per CTA, 2 slots per thread (one
// translation unit per variant so that the variants compile in parallel).
// Builds with and without the filling path; occupancy 0 = the default build; 4 = the build for 4
// resident CTAs per SM (fewer registers).
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_f32_256_e2(int occupancy, bool fills) {
  if (occupancy == 4) return fills ? kb_f32_occ<256, 2, 4, true> : kb_f32_occ<256, 2, 4, false>;
  if (occupancy == 0) return fills ? kb_f32<256, 2, true> : kb_f32<256, 2, false>;
  return nullptr;
}

}  // namespace mcl
