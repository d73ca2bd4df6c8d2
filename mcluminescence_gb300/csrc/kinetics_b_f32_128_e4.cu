// FP32 Bernoulli kernel, 128 threads per CTA, 4 slots per thread (one
// translation unit per variant so that the variants compile in parallel).
// Builds with and without the filling path; occupancy 0 = the default build; 6 = the build for 6
// resident CTAs per SM (fewer registers).
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_f32_128_e4(int occupancy, bool fills) {
  if (occupancy == 6) return fills ? kb_f32_occ<128, 4, 6, true> : kb_f32_occ<128, 4, 6, false>;
  if (occupancy == 0) return fills ? kb_f32<128, 4, true> : kb_f32<128, 4, false>;
  return nullptr;
}

}  // namespace mcl
