// FP64 Bernoulli kernels (Philox or injected uniforms): the oracle-parity mode.
#include "kinetics_b_device.cuh"

namespace mcl {

KernelFn b_pick_f64(int block, int ept, bool injected) {
  if (block != 256) return nullptr;
  if (injected) {
    if (ept == 1) return kb_f64<256, 1, true>;
    if (ept == 2) return kb_f64<256, 2, true>;
  } else {
    if (ept == 1) return kb_f64<256, 1, false>;
    if (ept == 2) return kb_f64<256, 2, false>;
  }
  return nullptr;
}

}  // namespace mcl
