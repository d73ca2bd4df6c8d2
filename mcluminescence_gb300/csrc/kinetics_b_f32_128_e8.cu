// FP32 Bernoulli kernel, 128 threads per CTA, 8 slots per thread (one
// translation unit per variant so that the variants compile in parallel).
// Builds with and without the filling path; occupancy 0 = the default build; 4 = the build for 4
// resident CTAs per SM (at most 128 registers).
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_f32_128_e8(int occupancy, bool fills) {
  if (occupancy == 4) return fills ? kb_f32_occ<128, 8, 4, true> : kb_f32_occ<128, 8, 4, false>;
  if (occupancy == 0) return fills ? kb_f32<128, 8, true> : kb_f32<128, 8, false>;
  return nullptr;
}

}  // namespace mcl
