// Shared device helpers: Philox4x32-10, status reporting, CUDA error checks.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mclum.h"

namespace mcl {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Multipliers and Weyl key increments of that paper.
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

// Counter word 3 says which draw of a trap slot a block is for.
constexpr uint32_t kTagStep = 0;    // per-step Bernoulli uniforms
constexpr uint32_t kTagInit = 1;    // initial nearest-centre distance r'
constexpr uint32_t kTagRefill = 2;  // r' of a trap refilled at a step
constexpr uint32_t kTagLow = 3;     // low 16 bits of an FP32-mode uniform

__device__ __forceinline__ uint4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                               uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += kPhiloxW0;
      k1 += kPhiloxW1;
    }
    const uint64_t p0 = (uint64_t)kPhiloxM0 * c0;
    const uint64_t p1 = (uint64_t)kPhiloxM1 * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c1 = (uint32_t)p1;
    c3 = (uint32_t)p0;
    c0 = n0;
    c2 = n2;
  }
  return make_uint4(c0, c1, c2, c3);
}

// 53-bit double in [0, 1): ((a >> 5) * 2^26 + (b >> 6)) / 2^53.
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  const double hi = (double)(a >> 5);
  const double lo = (double)(b >> 6);
  return __dmul_rn(__dadd_rn(__dmul_rn(hi, 67108864.0), lo), 1.0 / 9007199254740992.0);
}

// First error wins; the host reads the word after the launch.
__device__ __forceinline__ void report(int32_t* status, int32_t code) {
  if (status) atomicCAS(status, 0, code);
}

}  // namespace mcl

#define MCL_CUDA_TRY(expr)                       \
  do {                                           \
    cudaError_t _e = (expr);                     \
    if (_e != cudaSuccess) {                     \
      mcl_set_last_cuda_error(_e);               \
      return MCL_ECUDA;                          \
    }                                            \
  } while (0)

extern "C" void mcl_set_last_cuda_error(cudaError_t e);
// Sets the text mcl_last_error() returns on this thread.
extern "C" void mcl_set_last_message(const char* msg);
