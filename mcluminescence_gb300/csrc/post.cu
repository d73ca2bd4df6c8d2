// Presentation binning and smoothing of glow curves on the device.
//
// The reference turns its simulate() tables into plotted glow curves in
// src/class/plots.py: plot_TL (:52-74) takes, per run r, the first replica's
// time axis t = x_ax[:, 0, r] and the replica mean L = lum[:, :, r].mean(1),
// keeps the steps with t > 0, maps them to degC with T_start + T_rate t, and
// hist_and_smooth (:39-47) histograms L over [0, 1, 2, ...] * bin_width edges
// up to max(T) + bin_width, divides by bin_width and applies running_mean
// (:19-21), a 'valid' boxcar of width k = max(1, int(win_deg / bin_width)).
//
// Here the same curves come out of three small kernels:
// * glow_extent: one CTA per run reduces max(T) over the kept steps and
//   derives the edge count the way numpy's arange sizes its result,
//   ceil((max + bin_width) / bin_width);
// * glow_hist: each step adds its event count (sum of the 0/1 lum entries of
//   its replicas) to its bin with an integer atomic -- exact and independent
//   of the order -- and glow_finish divides by the replica count and the bin
//   width.  numpy sums the replica means, which is the same number whenever
//   count / sims is exact (sims a power of two) and within an ulp otherwise;
// * running_mean_seg: one thread per output, the window summed in order with
//   the weight 1/k (numpy's convolve sums the same products in BLAS order).
//   A curve shorter than the window gives k - n + 1 equal values (numpy's
//   convolve swaps its operands).
// All of it is a few reads per step and per bin: HBM/latency-bound work.

#include <cmath>

#include "common.cuh"

namespace mcl {
namespace {

__device__ __forceinline__ double temp_of(const double* T0, const double* rate, int r, double t) {
  return __dadd_rn(T0[r], __dmul_rn(rate[r], t));
}

__global__ void __launch_bounds__(256) glow_extent(const double* x_ax, int steps, int sims, int runs,
                                                   const double* T0, const double* rate, double bw,
                                                   int64_t* n_edges) {
  __shared__ double s_max[256];
  __shared__ int s_any[256];
  const int r = blockIdx.x;
  double m = -INFINITY;
  int any = 0;
  for (int i = threadIdx.x; i < steps; i += blockDim.x) {
    const double t = x_ax[((int64_t)i * sims) * runs + r];
    if (t > 0.0) {
      m = fmax(m, temp_of(T0, rate, r, t));
      any = 1;
    }
  }
  s_max[threadIdx.x] = m;
  s_any[threadIdx.x] = any;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + w]);
      s_any[threadIdx.x] |= s_any[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (!s_any[0]) {
      n_edges[r] = -1;  // no step with t > 0: the reference's max() raises
    } else {
      const double len = ceil(__ddiv_rn(__dadd_rn(s_max[0], bw), bw));
      n_edges[r] = len > 0.0 ? (int64_t)len : 0;
    }
  }
}

__global__ void __launch_bounds__(256) glow_hist(const double* x_ax, const double* lum, int steps, int sims,
                                                 int runs, const double* T0, const double* rate, double bw,
                                                 const int64_t* bin_offsets, uint32_t* counts, int32_t* status) {
  const int r = blockIdx.y;
  const int64_t b0 = bin_offsets[r], nb = bin_offsets[r + 1] - b0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < steps; i += gridDim.x * blockDim.x) {
    const double t = x_ax[((int64_t)i * sims) * runs + r];
    if (!(t > 0.0)) continue;
    double c = 0.0;
    for (int s = 0; s < sims; ++s) c += lum[((int64_t)i * sims + s) * runs + r];
    if (c != floor(c) || c < 0.0 || c > (double)sims) {  // lum entries must be 0/1 event flags
      report(status, MCL_EINVAL);
      continue;
    }
    if (c == 0.0) continue;
    const double T = temp_of(T0, rate, r, t);
    // bin j holds j*bw <= T < (j+1)*bw; the last bin also holds T == nb*bw
    int64_t j = (int64_t)floor(__ddiv_rn(T, bw));
    if (j >= 0 && __dmul_rn((double)j, bw) > T) --j;
    if (j + 1 >= 0 && __dmul_rn((double)(j + 1), bw) <= T) ++j;
    if (j == nb && __dmul_rn((double)nb, bw) == T) j = nb - 1;
    if (T < 0.0 || j < 0 || j >= nb) continue;
    atomicAdd(&counts[b0 + j], (uint32_t)c);
  }
}

__global__ void __launch_bounds__(256) glow_finish(const uint32_t* counts, int64_t n, int sims, double bw,
                                                   double* hist) {
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
    hist[i] = __ddiv_rn(__ddiv_rn((double)counts[i], (double)sims), bw);
}

template <typename T>
__global__ void __launch_bounds__(256) running_mean_seg(const T* in, const int64_t* in_off, int k, double divisor,
                                                        const int64_t* out_off, double* out) {
  const int c = blockIdx.y;
  const int64_t i0 = in_off[c], n = in_off[c + 1] - i0;
  const int64_t o0 = out_off[c], no = out_off[c + 1] - o0;
  const double inv = 1.0 / (double)k;
  for (int64_t j = blockIdx.x * 256ll + threadIdx.x; j < no; j += (int64_t)gridDim.x * 256) {
    double acc = 0.0;
    if (n >= k) {
      for (int m = 0; m < k; ++m) acc = __dadd_rn(acc, __dmul_rn(__ddiv_rn((double)in[i0 + j + m], divisor), inv));
    } else {
      for (int64_t m = 0; m < n; ++m) acc = __dadd_rn(acc, __dmul_rn(__ddiv_rn((double)in[i0 + m], divisor), inv));
    }
    out[o0 + j] = acc;
  }
}

int grid_for(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 4096); }

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_glow_extent(const double* x_ax, int32_t steps, int32_t sims, int32_t runs,
                               const double* T_start, const double* T_rate, double bin_width,
                               int64_t* n_edges, void* stream) {
  if (!x_ax || !T_start || !T_rate || !n_edges || steps < 0 || sims <= 0 || runs < 0) return MCL_EINVAL;
  if (!(bin_width > 0.0)) return MCL_EINVAL;
  if (runs == 0) return MCL_OK;
  glow_extent<<<runs, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(x_ax, steps, sims, runs, T_start, T_rate,
                                                                         bin_width, n_edges);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_glow_hist(const double* x_ax, const double* lum, int32_t steps, int32_t sims, int32_t runs,
                             const double* T_start, const double* T_rate, double bin_width,
                             const int64_t* bin_offsets, int64_t n_bins_total, uint32_t* counts, double* hist,
                             int32_t* status, void* stream) {
  if (!x_ax || !lum || !T_start || !T_rate || !bin_offsets || !counts || !hist || !status) return MCL_EINVAL;
  if (steps < 0 || sims <= 0 || runs < 0 || n_bins_total < 0 || !(bin_width > 0.0)) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  MCL_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int32_t), s));
  if (n_bins_total > 0) MCL_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (size_t)n_bins_total, s));
  if (runs > 0 && steps > 0) {
    dim3 grid((unsigned)std::min((steps + 255) / 256, 64), (unsigned)runs);
    glow_hist<<<grid, 256, 0, s>>>(x_ax, lum, steps, sims, runs, T_start, T_rate, bin_width, bin_offsets, counts,
                                   status);
    MCL_CUDA_TRY(cudaGetLastError());
  }
  if (n_bins_total > 0) {
    glow_finish<<<grid_for(n_bins_total), 256, 0, s>>>(counts, n_bins_total, sims, bin_width, hist);
    MCL_CUDA_TRY(cudaGetLastError());
  }
  return MCL_OK;
}

extern "C" int mcl_running_mean(int32_t in_type, const void* in, const int64_t* in_offsets, int32_t n_curves,
                                int32_t k, double divisor, const int64_t* out_offsets, int64_t max_out, double* out,
                                void* stream) {
  if (!in || !in_offsets || !out_offsets || !out || n_curves < 0 || k < 1 || !(divisor != 0.0) || max_out < 0)
    return MCL_EINVAL;
  if (n_curves == 0 || max_out == 0) return MCL_OK;
  if (n_curves > 65535) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  dim3 grid((unsigned)std::min<int64_t>((max_out + 255) / 256, 1024), (unsigned)n_curves);
  if (in_type == 0)
    running_mean_seg<double><<<grid, 256, 0, s>>>(static_cast<const double*>(in), in_offsets, k, divisor,
                                                  out_offsets, out);
  else if (in_type == 1)
    running_mean_seg<uint32_t><<<grid, 256, 0, s>>>(static_cast<const uint32_t*>(in), in_offsets, k, divisor,
                                                    out_offsets, out);
  else
    return MCL_EINVAL;
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
