// Host side of the C ABI: validation, the ragged packer, CUDA-graph capture,
// device queries and error strings.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace {
thread_local cudaError_t g_last_cuda = cudaSuccess;
thread_local char g_last_msg[256] = "";

bool is_fin(double x) { return std::isfinite(x); }
}  // namespace

extern "C" void mcl_set_last_cuda_error(cudaError_t e) {
  g_last_cuda = e;
  std::snprintf(g_last_msg, sizeof(g_last_msg), "CUDA error %d: %s", (int)e, cudaGetErrorString(e));
}

extern "C" void mcl_set_last_message(const char* msg) {
  std::snprintf(g_last_msg, sizeof(g_last_msg), "%s", msg ? msg : "");
}

extern "C" int mcl_abi_version(void) { return MCL_ABI_VERSION; }

extern "C" const char* mcl_last_error(void) { return g_last_msg; }

extern "C" int mcl_struct_sizes(size_t* out) {
  if (!out) return MCL_EINVAL;
  out[0] = sizeof(mcl_segment);
  out[1] = sizeof(mcl_set);
  out[2] = sizeof(mcl_item);
  out[3] = sizeof(mcl_b_args);
  out[4] = sizeof(mcl_k_sim);
  out[5] = sizeof(mcl_k_args);
  return MCL_OK;
}

extern "C" const char* mcl_status_string(int code) {
  switch (code) {
    case MCL_OK: return "ok";
    case MCL_EINVAL: return "invalid argument";
    case MCL_ECAPACITY: return "output table or on-chip buffer too small";
    case MCL_EBUDGET: return "step or iteration budget exhausted";
    case MCL_ECUDA: return "CUDA runtime error";
    case MCL_ENODEV: return "no usable sm_103 device";
    case MCL_ENOHOLE: return "nearest-centre search over zero recombination centres";
    case MCL_EOVERFLOW: return "more steps than rows in the output table";
  }
  return "unknown status";
}

extern "C" int mcl_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor) {
  int dev = 0, n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return MCL_ENODEV;
  MCL_CUDA_TRY(cudaGetDevice(&dev));
  int sms = 0, ma = 0, mi = 0;
  MCL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MCL_CUDA_TRY(cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, dev));
  MCL_CUDA_TRY(cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, dev));
  if (sm_count) *sm_count = sms;
  if (cc_major) *cc_major = ma;
  if (cc_minor) *cc_minor = mi;
  return MCL_OK;
}

// ---------------------------------------------------------------------------
// Bernoulli mode: validation and packing
// ---------------------------------------------------------------------------
extern "C" int mcl_b_validate(const mcl_set* sets, int32_t n_sets, const mcl_segment* segs,
                              int32_t n_segs, int64_t n_bins_total, int64_t n_slots_total,
                              int32_t precision, int32_t rng, int64_t n_uniforms) {
  if (n_sets < 0 || n_segs < 0 || (n_sets > 0 && !sets) || (n_segs > 0 && !segs)) return MCL_EINVAL;
  if (precision != MCL_FP32 && precision != MCL_FP64) return MCL_EINVAL;
  if (rng != MCL_RNG_PHILOX && rng != MCL_RNG_INJECTED) return MCL_EINVAL;
  if (rng == MCL_RNG_INJECTED && precision != MCL_FP64) return MCL_EINVAL;
  int64_t step_prefix = 0;
  for (int32_t i = 0; i < n_sets; ++i) {
    const mcl_set& s = sets[i];
    if (s.step_offset != step_prefix) return MCL_EINVAL;
    step_prefix += s.total_steps;
    if (s.n_slots < 0 || s.n_filled < 0 || s.n_filled > s.n_slots) return MCL_EINVAL;
    if (s.seg_count < 0 || s.seg_begin < 0 || (int64_t)s.seg_begin + s.seg_count > n_segs) return MCL_EINVAL;
    if (s.n_bins < 0 || s.bin_offset < 0 || s.bin_offset + s.n_bins > n_bins_total) return MCL_ECAPACITY;
    if (s.slot_offset < 0 || s.slot_offset + s.n_slots > n_slots_total) return MCL_ECAPACITY;
    if (!is_fin(s.E) || !is_fin(s.s) || s.s < 0 || !is_fin(s.alpha) || s.alpha < 0) return MCL_EINVAL;
    if (!is_fin(s.k_b) || s.k_b <= 0) return MCL_EINVAL;
    int64_t steps = 0, quads = 0;
    int32_t next_bin = 0;
    for (int32_t g = 0; g < s.seg_count; ++g) {
      const mcl_segment& sg = segs[s.seg_begin + g];
      if (sg.n_steps < 0 || sg.steps_per_bin < 1 || sg.bin_offset < 0) return MCL_EINVAL;
      if (!is_fin(sg.dt) || sg.dt <= 0 || !is_fin(sg.dt_growth) || sg.dt_growth <= 0) return MCL_EINVAL;
      if (!is_fin(sg.T0) || !is_fin(sg.beta) || !is_fin(sg.rate_const) || sg.rate_const < 0) return MCL_EINVAL;
      if (!is_fin(sg.fill_rate) || sg.fill_rate < 0) return MCL_EINVAL;
      if (rng == MCL_RNG_INJECTED && sg.fill_rate > 0) return MCL_EINVAL;
      const int64_t nb = (sg.n_steps + sg.steps_per_bin - 1) / sg.steps_per_bin;
      if (sg.bin_offset < next_bin || sg.bin_offset + nb > s.n_bins) return MCL_ECAPACITY;
      next_bin = (int32_t)(sg.bin_offset + nb);
      if (sg.flags & MCL_SEG_THERMAL) {
        double t_end;
        if (sg.dt_growth == 1.0) t_end = sg.dt * sg.n_steps;
        else t_end = sg.dt * (std::pow(sg.dt_growth, (double)sg.n_steps) - 1.0) / (sg.dt_growth - 1.0);
        if (!(sg.T0 > 0) || !(sg.T0 + sg.beta * t_end > 0) || !is_fin(t_end)) return MCL_EINVAL;
      }
      steps += sg.n_steps;
      quads += (sg.n_steps + 3) / 4;
    }
    if (steps != s.total_steps || steps > INT32_MAX || quads > UINT32_MAX) return MCL_EINVAL;
    if (rng == MCL_RNG_INJECTED) {
      const int64_t need = (int64_t)s.n_slots * (1 + steps);
      if (s.u_offset < 0 || s.u_offset + need > n_uniforms) return MCL_ECAPACITY;
    }
  }
  return MCL_OK;
}

extern "C" int64_t mcl_b_pack_items(const mcl_set* sets, int32_t n_sets, int32_t slots_per_item,
                                    mcl_item* items_out, int64_t items_cap) {
  if (n_sets < 0 || slots_per_item <= 0 || (n_sets > 0 && !sets)) return MCL_EINVAL;
  struct Cand {
    int64_t cost;
    mcl_item it;
  };
  std::vector<Cand> c;
  for (int32_t i = 0; i < n_sets; ++i) {
    for (int32_t b = 0; b < sets[i].n_slots; b += slots_per_item) {
      const int64_t n = std::min<int64_t>(slots_per_item, sets[i].n_slots - b);
      // the CTA walks every step for its whole slot range, full or not
      (void)n;
      c.push_back({sets[i].total_steps, {i, b}});
    }
  }
  std::stable_sort(c.begin(), c.end(), [](const Cand& x, const Cand& y) { return x.cost > y.cost; });
  if ((int64_t)c.size() > items_cap) return MCL_ECAPACITY;
  for (size_t k = 0; k < c.size(); ++k) items_out[k] = c[k].it;
  return (int64_t)c.size();
}

// ---------------------------------------------------------------------------
// CUDA graphs
// ---------------------------------------------------------------------------
extern "C" int mcl_b_graph_create(const mcl_b_args* args, void* stream, void** graph_out) {
  if (!args || !graph_out || !stream) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  MCL_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const int rc = mcl_b_run(args, stream);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc != MCL_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) {
    mcl_set_last_cuda_error(e);
    return MCL_ECUDA;
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    mcl_set_last_cuda_error(e);
    return MCL_ECUDA;
  }
  *graph_out = reinterpret_cast<void*>(x);
  return MCL_OK;
}

extern "C" int mcl_graph_launch(void* graph, void* stream) {
  if (!graph) return MCL_EINVAL;
  MCL_CUDA_TRY(cudaGraphLaunch(reinterpret_cast<cudaGraphExec_t>(graph),
                               reinterpret_cast<cudaStream_t>(stream)));
  return MCL_OK;
}

extern "C" int mcl_graph_destroy(void* graph) {
  if (!graph) return MCL_EINVAL;
  MCL_CUDA_TRY(cudaGraphExecDestroy(reinterpret_cast<cudaGraphExec_t>(graph)));
  return MCL_OK;
}
