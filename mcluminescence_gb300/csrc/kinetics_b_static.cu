// Bernoulli-mode launch whose scratch memory is a fixed device array of this
// library, for callers that must not allocate GPU memory.
//
// Who needs it: a host application that hands this library only its input
// and output buffers and owns every other byte of device memory itself --
// for example a service that reserves the whole GPU up front through its own
// memory pool, or a plugin host that forbids its plugins from calling
// cudaMalloc (which can block on, and synchronise with, work already queued
// on the device).  Such a caller cannot provide the workspace that
// mcl_b_run() needs, so this variant uses the file-scope array below instead.
//
// The array is part of the library's device image: every GPU that loads the
// library holds its MCL_B_STATIC_SCRATCH_BYTES until the process exits.  It
// holds the 256-byte work-ticket header plus the per-step rate table, so a
// batch may have at most (MCL_B_STATIC_SCRATCH_BYTES - 256) / 8 steps summed
// over its sets in FP32 mode, / 16 in FP64 mode; larger batches are rejected
// with MCL_ECAPACITY before anything is launched.
//
// All calls share the one array and it keeps the previous call's contents.
// The ticket is cleared and the whole table rewritten by every call, so no
// stale state leaks between calls; but two calls whose work overlaps on the
// GPU (different streams, or different host threads) race on the array and
// corrupt each other's results -- serialise them on one stream.  The kernels
// check every set's table rows against table_steps (which is checked against
// the array's size here), so sets that disagree with the declared sizes are
// refused on the device instead of writing past the array.
//
// The array's device address is looked up once per device and kept for the
// life of the process: a device reset (cudaDeviceReset) after the first call
// on that device is not supported, as the cached address would then be
// stale.
#include <cstdio>
#include <mutex>

#include "common.cuh"

namespace {

static __device__ __align__(256) unsigned char g_b_scratch[MCL_B_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

}  // namespace

extern "C" int mcl_b_run_static(const mcl_b_args* args, void* stream) {
  if (!args) return MCL_EINVAL;
  const int64_t entry = args->precision == MCL_FP64 ? 16 : 8;
  const int64_t capacity = ((int64_t)MCL_B_STATIC_SCRATCH_BYTES - 256) / entry;
  if (args->table_steps < 0 || args->table_steps > capacity) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "mcl_b_run_static: the batch has %lld steps over all sets; the static "
                  "scratch of %d bytes holds at most %lld in this precision",
                  (long long)args->table_steps, (int)MCL_B_STATIC_SCRATCH_BYTES, (long long)capacity);
    mcl_set_last_message(msg);
    return MCL_ECAPACITY;
  }
  // Set-up, once per device, with that device current: the host-side name of
  // the array is only a stand-in, so look up its device address.
  int dev = 0;
  MCL_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return MCL_ENODEV;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      MCL_CUDA_TRY(cudaGetSymbolAddress(&p, g_b_scratch));
      g_scratch_addr[dev] = p;
    }
    scratch = g_scratch_addr[dev];
  }
  mcl_b_args a = *args;
  a.workspace = scratch;
  a.workspace_bytes = MCL_B_STATIC_SCRATCH_BYTES;
  return mcl_b_run(&a, stream);
}
