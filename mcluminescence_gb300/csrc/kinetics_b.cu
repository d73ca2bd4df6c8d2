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
// * a persistent grid pulls work items (set, 'slots_per_item' consecutive
//   trap slots) from an atomic ticket; items are packed longest-first on the
//   host, so the ticket order is a longest-processing-time schedule;
// * each thread owns `EPT` slots: their w and filled bits live in registers,
//   and the electrons themselves are never stored in memory -- r' comes from
//   the Philox stream keyed by (set, slot), every step's uniform from
//   (set, slot, step);
// * per step, c_j (the same for every slot of the set) is read from a
//   shared-memory chunk the CTA precomputes in FP64;
// * FP32 mode tests every electron-step with three ALU ops: the top 23 bits
//   of the uniform form f in [1,2); if f >= 1 + c*w + 2^-21 the uniform is
//   provably >= c*w >= p and nothing happens.  Otherwise (probability
//   ~ c*w + 2^-21) the exact test u32 < ceil(p * 2^32) with p = -expm1f(-c*w)
//   decides;
// * events accumulate in a per-thread counter, are summed per warp with a
//   single reduction at every bin boundary, added to shared-memory bins, and
//   the CTA adds each non-zero bin to HBM with one atomic when the item ends.
// HBM traffic is therefore the set/segment/item descriptors in and the bins
// out; the kernel is bound by integer/FP32 issue (the Philox rounds).

#include <algorithm>
#include <cstdio>

#include "common.cuh"

namespace mcl {
namespace {

constexpr int kChunk = 256;  // steps whose c_j/q_j one shared-memory chunk holds

struct Workspace {
  int32_t ticket;
  int32_t pad[63];
};

// c_j and q_j of local step j of segment sg (FP64, no contraction so that the
// values match the oracle's numpy evaluation order).
__device__ __forceinline__ void step_constants(const mcl_set& st, const mcl_segment& sg, int j,
                                               double& c, double& q) {
  double dtj, t;
  if (sg.dt_growth == 1.0) {
    dtj = sg.dt;
    t = __dmul_rn(sg.dt, (double)j);
  } else {
    const double gj = pow(sg.dt_growth, (double)j);
    dtj = __dmul_rn(sg.dt, gj);
    t = __ddiv_rn(__dmul_rn(sg.dt, __dadd_rn(gj, -1.0)), __dadd_rn(sg.dt_growth, -1.0));
  }
  const double T = __dadd_rn(sg.T0, __dmul_rn(sg.beta, t));
  double A = sg.rate_const;
  if (sg.flags & MCL_SEG_THERMAL) {
    A = __dadd_rn(A, __dmul_rn(st.s, exp(__ddiv_rn(-st.E, __dmul_rn(st.k_b, T)))));
  }
  c = __dmul_rn(dtj, A);
  q = sg.fill_rate > 0.0 ? -expm1(__dmul_rn(-dtj, sg.fill_rate)) : 0.0;
}

__device__ __forceinline__ float r_prime_f(float u) { return cbrtf(-log1pf(-u)); }
__device__ __forceinline__ double r_prime_d(double u) { return cbrt(-log1p(-u)); }

// Sum `v` over the warp and add it to *dst from lane 0 (skipped if all zero).
__device__ __forceinline__ void warp_flush(uint32_t v, uint32_t* dst) {
  if (__any_sync(0xffffffffu, v != 0)) {
    const uint32_t tot = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, tot);
  }
}

template <int BLOCK>
__device__ __forceinline__ void zero_bins(uint32_t* s_lum, uint32_t* s_alive, int n_bins) {
  for (int b = threadIdx.x; b < n_bins; b += BLOCK) {
    s_lum[b] = 0;
    if (s_alive) s_alive[b] = 0;
  }
}

template <int BLOCK>
__device__ __forceinline__ void flush_bins(const mcl_b_args& a, const mcl_set& st,
                                           const uint32_t* s_lum, const uint32_t* s_alive) {
  for (int b = threadIdx.x; b < st.n_bins; b += BLOCK) {
    const uint32_t v = s_lum[b];
    if (v) atomicAdd(&a.lum[st.bin_offset + b], v);
    if (s_alive) {
      const uint32_t al = s_alive[b];
      if (al) atomicAdd(&a.alive[st.bin_offset + b], al);
    }
  }
}

__device__ __forceinline__ uint32_t word_of(const uint4& r, int q) {
  return q == 0 ? r.x : (q == 1 ? r.y : (q == 2 ? r.z : r.w));
}

// ---------------------------------------------------------------------------
// FP32 / Philox kernel
// ---------------------------------------------------------------------------
template <int BLOCK, int EPT>
__global__ void __launch_bounds__(BLOCK) kb_f32(const mcl_b_args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_c = reinterpret_cast<float*>(smem);
  float* s_q = s_c + kChunk;
  uint32_t* s_lum = reinterpret_cast<uint32_t*>(s_q + kChunk);
  uint32_t* s_alive = a.alive ? s_lum + a.max_bins : nullptr;
  __shared__ int s_item;

  Workspace* ws = reinterpret_cast<Workspace*>(a.workspace);
  const int tid = threadIdx.x;
  const uint32_t k0 = (uint32_t)a.seed;
  const uint32_t k1 = (uint32_t)(a.seed >> 32);
  constexpr float kMargin = 1.0f + 0x1p-21f;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(&ws->ticket, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= a.n_items) break;
    const mcl_item item = a.items[it];
    const mcl_set st = a.sets[item.set];
    if (st.n_bins > a.max_bins) {  // host validation makes this unreachable
      report(a.status, MCL_ECAPACITY);
      __syncthreads();
      continue;
    }
    zero_bins<BLOCK>(s_lum, s_alive, st.n_bins);

    // ---- slot initialisation: r' -> w, filled bits ----------------------
    const float alpha = (float)st.alpha;
    float w[EPT];
    uint32_t slot[EPT];
    uint32_t filled = 0;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = item.slot_begin + i * BLOCK + tid;
      slot[i] = (uint32_t)e;
      w[i] = 0.0f;
      if (e < st.n_slots) {
        const uint4 r = philox4x32_10(0u, (uint32_t)e, st.set_id, kTagInit, k0, k1);
        const float u = (float)(r.x >> 8) * 0x1p-24f;
        w[i] = expf(-alpha * r_prime_f(u));
        if (e < st.n_filled) filled |= 1u << i;
      }
    }
    float weff[EPT];  // w of a filled trap, 0 for an empty one
#pragma unroll
    for (int i = 0; i < EPT; ++i) weff[i] = (filled >> i & 1u) ? w[i] : 0.0f;

    uint32_t cnt = 0;
    int64_t kglob = 0;  // global step of the set (fates, refill counters)
    uint32_t qbase = 0;
    for (int g = 0; g < st.seg_count; ++g) {
      const mcl_segment sg = a.segs[st.seg_begin + g];
      const bool fill_on = sg.fill_rate > 0.0;
      const int spb = sg.steps_per_bin;
      int to_flush = spb;
      int bin = sg.bin_offset;
      for (int j0 = 0; j0 < sg.n_steps; j0 += kChunk) {
        const int nj = min(kChunk, sg.n_steps - j0);
        __syncthreads();
        for (int jj = tid; jj < nj; jj += BLOCK) {
          double c, q;
          step_constants(st, sg, j0 + jj, c, q);
          s_c[jj] = (float)c;
          s_q[jj] = (float)q;
        }
        __syncthreads();
        for (int jq = 0; jq < nj; jq += 4) {
          const uint32_t quad = qbase + (uint32_t)((j0 + jq) >> 2);
          uint4 r[EPT];
#pragma unroll
          for (int i = 0; i < EPT; ++i) r[i] = philox4x32_10(quad, slot[i], st.set_id, kTagStep, k0, k1);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (jq + q < nj) {
              const float c = s_c[jq + q];
              const float qf = s_q[jq + q];
#pragma unroll
              for (int i = 0; i < EPT; ++i) {
                const uint32_t wd = word_of(r[i], q);
                const float f = __uint_as_float((wd & 0x7fffffu) | 0x3f800000u);
                const bool is_filled = (filled >> i) & 1u;
                float y = __fmaf_rn(c, weff[i], kMargin);
                if (fill_on && !is_filled) y = __fadd_rn(qf, kMargin);
                if (f < y) {
                  // exact test on the full 32-bit uniform (rotated left 9)
                  const uint32_t u32 = __funnelshift_l(wd, wd, 9);
                  if (is_filled) {
                    const float p = -expm1f(-__fmul_rn(c, w[i]));
                    if (p >= 1.0f || u32 < __float2uint_ru(__fmul_rn(p, 4294967296.0f))) {
                      filled &= ~(1u << i);
                      weff[i] = 0.0f;
                      ++cnt;
                      if (a.fates) a.fates[st.slot_offset + slot[i]] = (int32_t)(kglob + j0 + jq + q);
                    }
                  } else if (fill_on && slot[i] < (uint32_t)st.n_slots) {
                    if (qf >= 1.0f || u32 < __float2uint_ru(__fmul_rn(qf, 4294967296.0f))) {
                      const uint4 rr = philox4x32_10((uint32_t)(kglob + j0 + jq + q), slot[i],
                                                     st.set_id, kTagRefill, k0, k1);
                      const float u = (float)(rr.x >> 8) * 0x1p-24f;
                      w[i] = expf(-alpha * r_prime_f(u));
                      weff[i] = w[i];
                      filled |= 1u << i;
                    }
                  }
                }
              }
              if (--to_flush == 0 || j0 + jq + q + 1 == sg.n_steps) {
                if (bin < st.n_bins) {
                  warp_flush(cnt, &s_lum[bin]);
                  if (s_alive) warp_flush((uint32_t)__popc(filled), &s_alive[bin]);
                } else {
                  report(a.status, MCL_ECAPACITY);
                }
                cnt = 0;
                ++bin;
                to_flush = spb;
              }
            }
          }
        }
      }
      qbase += (uint32_t)((sg.n_steps + 3) >> 2);
      kglob += sg.n_steps;
    }
    __syncthreads();
    flush_bins<BLOCK>(a, st, s_lum, s_alive);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// FP64 kernel (Philox or injected uniforms): the oracle-parity mode
// ---------------------------------------------------------------------------
template <int BLOCK, int EPT, bool INJ>
__global__ void __launch_bounds__(BLOCK) kb_f64(const mcl_b_args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_c = reinterpret_cast<double*>(smem);
  double* s_q = s_c + kChunk;
  uint32_t* s_lum = reinterpret_cast<uint32_t*>(s_q + kChunk);
  uint32_t* s_alive = a.alive ? s_lum + a.max_bins : nullptr;
  __shared__ int s_item;

  Workspace* ws = reinterpret_cast<Workspace*>(a.workspace);
  const int tid = threadIdx.x;
  const uint32_t k0 = (uint32_t)a.seed;
  const uint32_t k1 = (uint32_t)(a.seed >> 32);

  for (;;) {
    if (tid == 0) s_item = atomicAdd(&ws->ticket, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= a.n_items) break;
    const mcl_item item = a.items[it];
    const mcl_set st = a.sets[item.set];
    if (st.n_bins > a.max_bins) {
      report(a.status, MCL_ECAPACITY);
      __syncthreads();
      continue;
    }
    zero_bins<BLOCK>(s_lum, s_alive, st.n_bins);

    double w[EPT];
    uint32_t slot[EPT];
    uint32_t filled = 0;
    const int64_t n = st.n_slots;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = item.slot_begin + i * BLOCK + tid;
      slot[i] = (uint32_t)e;
      w[i] = 0.0;
      if (e < st.n_slots) {
        double u;
        if (INJ) {
          u = a.uniforms[st.u_offset + e];
        } else {
          const uint4 r = philox4x32_10(0u, (uint32_t)e, st.set_id, kTagInit, k0, k1);
          u = u53(r.x, r.y);
        }
        w[i] = exp(__dmul_rn(-st.alpha, r_prime_d(u)));
        if (e < st.n_filled) filled |= 1u << i;
      }
    }

    uint32_t cnt = 0;
    int64_t kglob = 0;
    uint32_t pbase = 0;
    for (int g = 0; g < st.seg_count; ++g) {
      const mcl_segment sg = a.segs[st.seg_begin + g];
      const bool fill_on = sg.fill_rate > 0.0;
      const int spb = sg.steps_per_bin;
      int to_flush = spb;
      int bin = sg.bin_offset;
      for (int j0 = 0; j0 < sg.n_steps; j0 += kChunk) {
        const int nj = min(kChunk, sg.n_steps - j0);
        __syncthreads();
        for (int jj = tid; jj < nj; jj += BLOCK) step_constants(st, sg, j0 + jj, s_c[jj], s_q[jj]);
        __syncthreads();
        uint4 r[EPT];
        for (int jj = 0; jj < nj; ++jj) {
          const int j = j0 + jj;
          const int64_t k = kglob + j;
          if (!INJ && (j & 1) == 0) {
#pragma unroll
            for (int i = 0; i < EPT; ++i)
              r[i] = philox4x32_10(pbase + (uint32_t)(j >> 1), slot[i], st.set_id, kTagStep, k0, k1);
          }
          const double c = s_c[jj];
          const double qv = s_q[jj];
#pragma unroll
          for (int i = 0; i < EPT; ++i) {
            if (slot[i] >= (uint32_t)st.n_slots) continue;
            double u;
            if (INJ) {
              u = a.uniforms[st.u_offset + n + k * n + slot[i]];
            } else {
              u = (j & 1) ? u53(r[i].z, r[i].w) : u53(r[i].x, r[i].y);
            }
            if ((filled >> i) & 1u) {
              const double p = -expm1(__dmul_rn(-c, w[i]));
              if (u < p) {
                filled &= ~(1u << i);
                ++cnt;
                if (a.fates) a.fates[st.slot_offset + slot[i]] = (int32_t)k;
              }
            } else if (fill_on && u < qv) {
              double ur;
              if (INJ) {
                ur = 0.0;  // host validation rejects fill segments in injected mode
              } else {
                const uint4 rr = philox4x32_10((uint32_t)k, slot[i], st.set_id, kTagRefill, k0, k1);
                ur = u53(rr.x, rr.y);
              }
              w[i] = exp(__dmul_rn(-st.alpha, r_prime_d(ur)));
              filled |= 1u << i;
            }
          }
          if (--to_flush == 0 || j + 1 == sg.n_steps) {
            if (bin < st.n_bins) {
              warp_flush(cnt, &s_lum[bin]);
              if (s_alive) warp_flush((uint32_t)__popc(filled), &s_alive[bin]);
            } else {
              report(a.status, MCL_ECAPACITY);
            }
            cnt = 0;
            ++bin;
            to_flush = spb;
          }
        }
      }
      pbase += (uint32_t)((sg.n_steps + 1) >> 1);
      kglob += sg.n_steps;
    }
    __syncthreads();
    flush_bins<BLOCK>(a, st, s_lum, s_alive);
    __syncthreads();
  }
}

using KernelFn = void (*)(const mcl_b_args);

template <int BLOCK>
KernelFn pick_f32(int ept) {
  switch (ept) {
    case 1: return kb_f32<BLOCK, 1>;
    case 2: return kb_f32<BLOCK, 2>;
    case 4: return kb_f32<BLOCK, 4>;
    case 8: return kb_f32<BLOCK, 8>;
  }
  return nullptr;
}

KernelFn pick_kernel(const mcl_b_args& a) {
  if (a.precision == MCL_FP32) {
    if (a.rng != MCL_RNG_PHILOX) return nullptr;
    switch (a.block) {
      case 128: return pick_f32<128>(a.ept);
      case 256: return pick_f32<256>(a.ept);
      case 512: return pick_f32<512>(a.ept);
    }
    return nullptr;
  }
  if (a.precision == MCL_FP64 && a.block == 256) {
    if (a.rng == MCL_RNG_INJECTED) {
      if (a.ept == 1) return kb_f64<256, 1, true>;
      if (a.ept == 2) return kb_f64<256, 2, true>;
    } else {
      if (a.ept == 1) return kb_f64<256, 1, false>;
      if (a.ept == 2) return kb_f64<256, 2, false>;
    }
  }
  return nullptr;
}

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" size_t mcl_b_workspace_size(void) { return sizeof(Workspace); }

extern "C" size_t mcl_b_smem_bytes(int32_t max_bins, int32_t precision, int32_t want_alive) {
  const size_t chunk = (precision == MCL_FP64 ? 2 * sizeof(double) : 2 * sizeof(float)) * kChunk;
  return chunk + (size_t)max_bins * sizeof(uint32_t) * (want_alive ? 2 : 1);
}

extern "C" int mcl_b_run(const mcl_b_args* args, void* stream) {
  if (!args) return MCL_EINVAL;
  const mcl_b_args& a = *args;
  if (a.n_items < 0 || a.max_bins < 0 || !a.workspace || !a.lum || !a.status) return MCL_EINVAL;
  if (a.slots_per_item != a.block * a.ept) return MCL_EINVAL;
  if (a.rng == MCL_RNG_INJECTED && !a.uniforms) return MCL_EINVAL;
  KernelFn fn = pick_kernel(a);
  if (!fn) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const size_t smem = mcl_b_smem_bytes(a.max_bins, a.precision, a.alive != nullptr);
  if (smem > 200 * 1024) return MCL_ECAPACITY;
  MCL_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (a.zero_outputs) {
    MCL_CUDA_TRY(cudaMemsetAsync(a.lum, 0, sizeof(uint32_t) * (size_t)a.n_bins_total, s));
    if (a.alive) MCL_CUDA_TRY(cudaMemsetAsync(a.alive, 0, sizeof(uint32_t) * (size_t)a.n_bins_total, s));
    if (a.fates) MCL_CUDA_TRY(cudaMemsetAsync(a.fates, 0xff, sizeof(int32_t) * (size_t)a.n_slots_total, s));
    MCL_CUDA_TRY(cudaMemsetAsync(a.status, 0, sizeof(int32_t), s));
  }
  MCL_CUDA_TRY(cudaMemsetAsync(a.workspace, 0, sizeof(Workspace), s));
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
  fn<<<grid, a.block, smem, s>>>(a);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
