// FP32 Bernoulli kernel, 128 threads per CTA, 2 slots per thread (one
// translation unit per variant so that the variants compile in parallel).
// Builds with and without the filling path; occupancy 0 = the default build; 8 = the build for 8
// resident CTAs per SM (fewer registers).
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_f32_128_e2(int occupancy, bool fills) {
  if (occupancy == 8) return fills ? kb_f32_occ<128, 2, 8, true> : kb_f32_occ<128, 2, 8, false>;
  if (occupancy == 0) return fills ? kb_f32<128, 2, true> : kb_f32<128, 2, false>;
  return nullptr;
}

}  // namespace mcl
