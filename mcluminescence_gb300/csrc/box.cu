// Step-level operations of the event-driven kinetics, for callers that drive
// the simulation loop themselves (the reference's driver calls them once per
// step: src/class/simulate.py:51-92 over src/class/engine.py:113-188 and
// src/class/tl_trap_lab.py:48-51).  The throughput path is mcl_k_run, which
// keeps the whole loop on the device; these entry points exist so that code
// written against the reference's TLTrapSim / Box surface runs unchanged.
//
// * mcl_k_box_nearest: per listed electron, the minimum and first argmin over
//   all holes of the Euclidean distance, evaluated as the reference's
//   np.linalg.norm(e - h) evaluates it: d = sqrt((dx*dx + dy*dy) + dz*dz)
//   with dx = e.x - h.x, every operation rounded once (no contraction).  A
//   NaN distance is the minimum, as in numpy (its first occurrence wins).
// * mcl_k_box_waits: lifetimes 1 / (s e^{-E_cb/kT} + b e^{-E_loc/kT - alpha d})
//   and exponential waits lifetime * (-log(1 - u)) from caller-drawn
//   uniforms (the Retrap choice E_loc = E_loc_2 if u_r < Retrap else E_loc_1).
// * mcl_k_box_distances: the full electron x hole distance matrix.
#include <algorithm>

#include "common.cuh"

namespace mcl {
namespace {

__device__ __forceinline__ double dist3(const double* e, const double* h) {
  const double dx = __dadd_rn(e[0], -h[0]);
  const double dy = __dadd_rn(e[1], -h[1]);
  const double dz = __dadd_rn(e[2], -h[2]);
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// Order key of a distance: NaN lowest, then non-negative doubles by their
// bit patterns (which order like their values).
__device__ __forceinline__ uint64_t dkey(double d) {
  return d != d ? 0ull : (uint64_t)__double_as_longlong(d) + 1ull;
}

// One warp per listed electron; lanes stride over the holes.
// Row indices outside [0, n_e) are skipped (nothing is read or written).
__global__ void __launch_bounds__(256) box_nearest(const double* __restrict__ el, int n_e,
                                                   const double* __restrict__ ho, int n_h,
                                                   const int32_t* __restrict__ rows, int n_rows,
                                                   double* __restrict__ min_d, int64_t* __restrict__ nearest) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= n_rows) return;
  const int r = rows ? rows[w] : w;
  if (r < 0 || r >= n_e) return;
  const double e[3] = {el[3 * (size_t)r], el[3 * (size_t)r + 1], el[3 * (size_t)r + 2]};
  uint64_t bk = ~0ull;
  int bi = 0x7fffffff;
  double bd = 0.0;
  for (int j = lane; j < n_h; j += 32) {
    const double d = dist3(e, ho + 3 * (size_t)j);
    const uint64_t k = dkey(d);
    if (k < bk) {  // strictly smaller: a lane meets its holes in increasing order
      bk = k;
      bi = j;
      bd = d;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t k2 = __shfl_xor_sync(0xffffffffu, bk, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
    const double d2 = __shfl_xor_sync(0xffffffffu, bd, o);
    if (k2 < bk || (k2 == bk && i2 < bi)) {
      bk = k2;
      bi = i2;
      bd = d2;
    }
  }
  if (lane == 0) {
    min_d[r] = bd;
    nearest[r] = bi;
  }
}

struct WaitPhys {
  double alpha, b, s, E_cb, E_loc_1, E_loc_2, Retrap, k_b;
};

__global__ void __launch_bounds__(256) box_waits(const WaitPhys P, double T, const double* __restrict__ d,
                                                 const double* __restrict__ ur, const double* __restrict__ uw, int n,
                                                 double* __restrict__ lifetime, double* __restrict__ wait) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double kT = __dmul_rn(P.k_b, T);
  const double rate_cb = __dmul_rn(P.s, exp(__ddiv_rn(-P.E_cb, kT)));
  const double E_loc = ur[i] < P.Retrap ? P.E_loc_2 : P.E_loc_1;
  const double arg = __dadd_rn(__ddiv_rn(-E_loc, kT), -__dmul_rn(P.alpha, d[i]));
  const double rate = __dmul_rn(P.b, exp(arg));
  const double lt = __ddiv_rn(1.0, __dadd_rn(rate_cb, rate));
  lifetime[i] = lt;
  wait[i] = __dmul_rn(lt, -log(__dadd_rn(1.0, -uw[i])));
}

__global__ void __launch_bounds__(256) box_distances(const double* __restrict__ el, int n_e,
                                                     const double* __restrict__ ho, int n_h, double* __restrict__ out) {
  const int64_t n = (int64_t)n_e * n_h;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k / n_h, j = k % n_h;
    out[k] = dist3(el + 3 * i, ho + 3 * j);
  }
}

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_k_box_nearest(const double* electrons, int32_t n_e, const double* holes, int32_t n_h,
                                 const int32_t* rows, int32_t n_rows, double* min_d, int64_t* nearest,
                                 void* stream) {
  if (n_e < 0 || n_h < 0 || n_rows < 0 || (!rows && n_rows > n_e)) return MCL_EINVAL;
  if (n_rows == 0) return MCL_OK;
  if (n_h == 0) return MCL_ENOHOLE;
  if (!electrons || !holes || !min_d || !nearest) return MCL_EINVAL;
  const int threads = 256, per_block = threads / 32;
  box_nearest<<<(n_rows + per_block - 1) / per_block, threads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      electrons, n_e, holes, n_h, rows, n_rows, min_d, nearest);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_k_box_waits(const mcl_k_sim* phys, double T, const double* min_d, const double* u_retrap,
                               const double* u_wait, int32_t n, double* lifetime, double* wait, void* stream) {
  if (!phys || n < 0) return MCL_EINVAL;
  if (n == 0) return MCL_OK;
  if (!min_d || !u_retrap || !u_wait || !lifetime || !wait) return MCL_EINVAL;
  const WaitPhys P{phys->alpha, phys->b, phys->s, phys->E_cb, phys->E_loc_1, phys->E_loc_2, phys->Retrap, phys->k_b};
  box_waits<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(P, T, min_d, u_retrap, u_wait, n,
                                                                                 lifetime, wait);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_k_box_distances(const double* electrons, int32_t n_e, const double* holes, int32_t n_h,
                                   double* out, void* stream) {
  if (n_e < 0 || n_h < 0) return MCL_EINVAL;
  if ((int64_t)n_e * n_h == 0) return MCL_OK;
  if (!electrons || !holes || !out) return MCL_EINVAL;
  const int64_t n = (int64_t)n_e * n_h;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  box_distances<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(electrons, n_e, holes, n_h, out);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
