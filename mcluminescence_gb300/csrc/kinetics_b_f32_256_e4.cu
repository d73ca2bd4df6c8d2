// FP32 Bernoulli kernel, 256 threads per CTA, 4 slots per thread (one
// translation unit per variant so that the variants compile in parallel).
// Builds with and without the filling path; occupancy 0 = the default build; 3 = the build for 3
// resident CTAs per SM (fewer registers).
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_f32_256_e4(int occupancy, bool fills) {
  if (occupancy == 3) return fills ? kb_f32_occ<256, 4, 3, true> : kb_f32_occ<256, 4, 3, false>;
  if (occupancy == 0) return fills ? kb_f32<256, 4, true> : kb_f32<256, 4, false>;
  return nullptr;
}

}  // namespace mcl
