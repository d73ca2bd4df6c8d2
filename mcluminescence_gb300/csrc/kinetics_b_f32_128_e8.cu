// FP32 Bernoulli kernel, 128 threads per CTA, 8 slots per thread (one
// translation unit per variant so that the variants compile in parallel).
// occupancy 0 = the default build; 4 = the build for 4 resident CTAs per SM (at most 128 registers).
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_f32_128_e8(int occupancy) {
  if (occupancy == 4) return kb_f32_occ<128, 8, 4>;
  return occupancy == 0 ? kb_f32<128, 8> : nullptr;
}

}  // namespace mcl
