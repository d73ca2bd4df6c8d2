// Fixed-dt Bernoulli trap kinetics over ragged batches of parameter sets.
//
// Physics (dilute limit of src/class/engine.py:65-77 with the event loop of
// src/class/simulate.py:51-92): a filled trap whose electron sits at
// dimensionless distance r' from its nearest centre escapes in step j with
// probability p = 1 - exp(-c_j * w), w = exp(-alpha r'), c_j = dt_j * A_j,
// A_j = rate_const + s exp(-E / (k_b T_j)).  An empty trap fills with
// probability q_j = 1 - exp(-dt_j * fill_rate).  Each escape is one
// recombination photon, counted into the set's bin for that step.
//
// Execution:
// * a pre-pass (kb_tables) evaluates c_j and q_j once per step of every set,
//   in FP64, into a table in the workspace (the only FP64 work of a launch);
// * a persistent grid pulls work items (set, `block*ept` consecutive trap
//   slots) from an atomic ticket; items are packed longest-first on the host,
//   so the ticket order is a longest-processing-time schedule;
// * each thread owns `EPT` slots: their w and filled bits live in registers.
//   Electrons are never stored: r' comes from the Philox stream keyed by
//   (set, slot), every step's uniform from (set, slot, step).  The Philox key
//   schedule is precomputed on the host and read from the kernel's constant
//   parameter bank, so the rounds cost only the multiplies and 3-input XORs;
// * the CTA copies 256-step chunks of (c_j, q_j) into shared memory;
// * FP32 mode spends 16 random bits per electron-step in the common case: a
//   Philox block (four 32-bit words) covers 8 steps of a slot.  Per 8-step
//   block the CTA stores the bound cm = RU(max c16 (1 + 2^-20)) (c16 = c 2^16
//   from the step table); per slot one FFMA turns cm w into an integer
//   threshold TI > h of every trial that can escape, and each word tests its
//   two 16-bit fields against TI with one subtraction and one LOP3 (filling
//   segments use the refill bound for empty traps).  A slot with no flagged
//   field has no event in the block; a flagged one is drawn again out of
//   line and tested step by step: the float test d = 2^23 + h - c16 w <
//   2^23 + 1, then the exact test u32 < ceil(p 2^32), p = -expm1f(-c w),
//   drawing the uniform's low 16 bits from a separate Philox counter only
//   when h sits on the threshold's upper half.  Per trial the fast path is
//   about one instruction next to 1/8 of a Philox call (17 32x32->64
//   multiplies per block on the FMA-heavy pipe, 20 3-input XORs);
// * batches without filling segments (mcl_b_args.no_fill) run a build
//   without the filling path: fewer registers, more resident warps;
// * events are added to shared-memory bins (rare); at each bin end the warp
//   sums the filled-trap counts with one reduction; when an item ends the CTA
//   adds every non-zero bin to HBM with one atomic.
// HBM traffic: descriptors, the step table (L2-resident per set) and bins.

#include <algorithm>
#include <cstdio>

#include "kinetics_b_device.cuh"

namespace mcl {
namespace {

KernelFn pick_kernel(const mcl_b_args& a) {
  if (a.precision == MCL_FP32) {
    if (a.rng != MCL_RNG_PHILOX) return nullptr;
    const int o = a.occupancy;
    const bool f = a.no_fill == 0;
    if (a.block == 128)
      return a.ept == 2 ? b_f32_128_e2(o, f) : a.ept == 4 ? b_f32_128_e4(o, f) : a.ept == 8 ? b_f32_128_e8(o, f) : nullptr;
    if (a.block == 256)
      return a.ept == 2 ? b_f32_256_e2(o, f) : a.ept == 4 ? b_f32_256_e4(o, f) : a.ept == 8 ? b_f32_256_e8(o, f) : nullptr;
    return nullptr;
  }
  if (a.precision == MCL_FP64) return b_pick_f64(a.block, a.ept, a.rng == MCL_RNG_INJECTED);
  return nullptr;
}

size_t table_entry_bytes(int32_t precision) { return precision == MCL_FP64 ? 16 : 8; }

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" size_t mcl_b_workspace_size(const mcl_set* sets, int32_t n_sets, int32_t precision) {
  int64_t steps = 0;
  for (int32_t i = 0; sets && i < n_sets; ++i) steps += sets[i].total_steps;
  return (size_t)kHeaderBytes + (size_t)steps * table_entry_bytes(precision);
}

extern "C" size_t mcl_b_smem_bytes(int32_t max_bins, int32_t precision, int32_t want_alive) {
  const size_t chunk = (precision == MCL_FP64 ? 2 * sizeof(double) : 2 * sizeof(float)) * kChunk;
  return chunk + (size_t)max_bins * sizeof(uint32_t) * (want_alive ? 2 : 1);
}

extern "C" int mcl_b_run(const mcl_b_args* args, void* stream) {
  if (!args) return MCL_EINVAL;
  const mcl_b_args& a = *args;
  if (a.n_items < 0 || a.n_sets < 0 || a.max_bins < 0 || !a.workspace || !a.lum || !a.status)
    return MCL_EINVAL;
  if (a.table_steps < 0 ||
      a.workspace_bytes < (int64_t)kHeaderBytes + a.table_steps * (int64_t)table_entry_bytes(a.precision))
    return MCL_ECAPACITY;
  if (a.slots_per_item != a.block * a.ept) return MCL_EINVAL;
  if (a.rng == MCL_RNG_INJECTED && (!a.uniforms || a.n_uniforms < 0)) return MCL_EINVAL;
  KernelFn fn = pick_kernel(a);
  if (!fn) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int copies = a.bin_copies <= 0 ? 1 : a.bin_copies;
  if (copies != 1 && copies != 2 && copies != 4) return MCL_EINVAL;
  if (a.precision != MCL_FP32) copies = 1;
  size_t smem = mcl_b_smem_bytes(a.max_bins, a.precision, a.alive != nullptr);
  smem += (size_t)(copies - 1) * a.max_bins * sizeof(uint32_t);
  if (smem > 200 * 1024) return MCL_ECAPACITY;
  KParams P;
  P.a = a;
  P.a.bin_copies = copies;
  const uint32_t k0 = (uint32_t)a.seed, k1 = (uint32_t)(a.seed >> 32);
  for (int r = 0; r < 10; ++r) {
    P.ks0[r] = k0 + (uint32_t)r * kPhiloxW0;
    P.ks1[r] = k1 + (uint32_t)r * kPhiloxW1;
  }
  MCL_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (a.zero_outputs) {
    MCL_CUDA_TRY(cudaMemsetAsync(a.lum, 0, sizeof(uint32_t) * (size_t)a.n_bins_total, s));
    if (a.alive) MCL_CUDA_TRY(cudaMemsetAsync(a.alive, 0, sizeof(uint32_t) * (size_t)a.n_bins_total, s));
    if (a.fates) MCL_CUDA_TRY(cudaMemsetAsync(a.fates, 0xff, sizeof(int32_t) * (size_t)a.n_slots_total, s));
    MCL_CUDA_TRY(cudaMemsetAsync(a.status, 0, sizeof(int32_t), s));
  }
  MCL_CUDA_TRY(cudaMemsetAsync(a.workspace, 0, sizeof(Header), s));
  if (a.n_sets > 0) {
    if (a.precision == MCL_FP64)
      kb_tables<double><<<a.n_sets, 256, 0, s>>>(a);
    else
      kb_tables<float><<<a.n_sets, 256, 0, s>>>(a);
    MCL_CUDA_TRY(cudaGetLastError());
  }
  if (a.n_items == 0) return MCL_OK;
  int grid = a.grid;
  if (grid <= 0) {
    int dev = 0, sms = 0, per_sm = 0;
    MCL_CUDA_TRY(cudaGetDevice(&dev));
    MCL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MCL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, a.block, smem));
    grid = sms * std::max(per_sm, 1);
  }
  grid = std::min(grid, a.n_items);
  fn<<<grid, a.block, smem, s>>>(P);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

// ---------------------------------------------------------------------------
// Roofline microbenchmark: Philox4x32-10 block generation alone, with the same
// counter structure as the FP32 kernel (block index and set id warp-uniform,
// four slots per thread), XOR-folded into one word per thread.  The rate it
// reaches bounds the FP32 kernel, which consumes one block per 8 trials.
// ---------------------------------------------------------------------------
namespace mcl {
namespace {
__global__ void __launch_bounds__(256) philox_peak_kernel(const KParams P, int iters, uint32_t* sink) {
  const uint32_t slot0 = blockIdx.x * 1024u + threadIdx.x;
  uint32_t acc = 0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint4 r = philox_ks((uint32_t)it, slot0 + 256u * i, blockIdx.x, kTagStep, P);
      acc ^= r.x ^ r.y ^ r.z ^ r.w;
    }
  }
  sink[blockIdx.x * 256 + threadIdx.x] = acc;
}
}  // namespace
}  // namespace mcl

extern "C" int mcl_bench_philox(uint32_t* sink, int32_t grid, int32_t iters, uint64_t seed, void* stream) {
  if (!sink || grid <= 0 || iters <= 0) return MCL_EINVAL;
  KParams P{};
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    P.ks0[r] = k0 + (uint32_t)r * kPhiloxW0;
    P.ks1[r] = k1 + (uint32_t)r * kPhiloxW1;
  }
  philox_peak_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(P, iters, sink);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
