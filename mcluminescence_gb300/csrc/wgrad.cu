// The surrogate network's weight gradients and Adam step in one launch (no
// counterpart in the reference, whose parameter fit runs the Monte Carlo for
// every candidate, src/class/optimizer.py:93-111).
//
// dW_l = dZ_l^T X_l reduces over the batch: M = the layer's outputs, N = its
// inputs, K = the batch.  Each 128 x 64 tile of dW_l belongs to a cluster of
// kSplits CTAs, CTA q taking the batch range [q K / kSplits, (q+1) K /
// kSplits).  Per CTA one thread (warp 1) streams 64-wide K slabs of dZ_l^T
// and X_l^T (both stored K-contiguous) with TMA (cp.async.bulk.tensor,
// 128-byte swizzle) into a ring of kStages shared-memory stages, each
// completing on its own mbarrier, and another (warp 0) issues tcgen05.mma
// (M 128, N 64, K 16, FP32 accumulator in tensor memory) as soon as a stage
// lands; an MMA commit frees the stage for the slab kStages further on.  The
// partial tiles then meet in distributed shared memory: every CTA pushes
// accumulator rows [32 q, 32 q + 32) (TMEM lane quadrant q) to CTA q, which
// sums them over the cluster in rank order (deterministic) and applies Adam
// to those weights right away (mcl_adam_multi_dev's arithmetic, operation
// for operation), refreshing the bf16 copy and its transpose.  One extra
// cluster applies Adam to the biases, whose gradients the fused forward /
// backward launch already summed.
//
// Every mbarrier wait is bounded; after a timeout the kernel records it in
// *err, writes nothing, waits (again bounded) for its copies and MMAs in
// flight, frees its tensor memory and returns.
#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "tcgen05.cuh"

namespace mcl {
namespace {
using namespace ::mcl::tcg;
namespace cg = cooperative_groups;

constexpr int kSplits = 4;               // CTAs per tile (cluster size)
constexpr int kStages = 7;               // slabs in flight per CTA
constexpr int kTM = 128, kTN = 64, kKS = 64;
constexpr int kStageA = kTM * kKS * 2;   // 16 KB: 128 rows x 128 bytes, 128-byte swizzled
constexpr int kStageB = kTN * kKS * 2;   // 8 KB
constexpr int kStage = kStageA + kStageB;
constexpr int kPS = kTN + 4;             // row stride (floats) of a received partial tile
constexpr int kRecv = kSplits * 32 * kPS * 4;   // partial rows received from every CTA of the cluster
constexpr int kSmem = kStages * kStage + kRecv + 1024;  // + slack to align the ring to 1,024 bytes
constexpr int kThreads = 256;  // 8 warps: two per TMEM lane quadrant
constexpr int kMaxLayers = 8;
constexpr int kMaxTiles = 64;

struct WgLayer {
  CUtensorMap mapA;  // dZt [out][ld], box 64 x 128
  CUtensorMap mapB;  // Xt [in][ld], box 64 x 64
  float* W;
  float* m1;
  float* m2;
  __nv_bfloat16* Wb;
  __nv_bfloat16* Wt;
  float* gW;
  float* b;
  const float* gb;
  float* mb;
  float* vb;
  int out, in;
};

struct WgParams {
  WgLayer L[kMaxLayers];
  uint8_t tile_layer[kMaxTiles], tile_m[kMaxTiles], tile_n[kMaxTiles];
  int n_layers, n_tiles, batch, step_offset;
  const float* lr;
  const int32_t* step_base;
  int32_t* err;
  float b1, b2, eps;
};

// Shared-memory descriptor of a K-major tile in the 128-byte swizzled layout
// (8-row atoms of 1,024 bytes; rows 128 bytes apart inside an atom): stride
// byte offset 1,024, leading byte offset unused (16), descriptor version 1,
// swizzle mode 2 (128 bytes).  Advancing K by 16 elements inside an atom
// moves the start address by 32 bytes.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}

// One Adam step on element i of a tensor (the arithmetic of adam_multi).
// When both new moments are +0 (the padded rows and columns of the network,
// whose gradient is always zero) that arithmetic gives p - (+0) = p: return p
// without the divisions and the square root, whose special-case paths are
// slow for zeros.
__device__ __forceinline__ float adam(float g, float& m1, float& m2, float p, float lr, float b1, float b2, float eps,
                                      float bc1, float bc2) {
  const float a = b1 * m1 + (1.0f - b1) * g;
  const float b = b2 * m2 + (1.0f - b2) * g * g;
  m1 = a;
  m2 = b;
  if ((__float_as_uint(a) | __float_as_uint(b)) == 0u) return p;
  const float mh = a / bc1, vh = b / bc2;
  return p - lr * mh / (sqrtf(vh) + eps);
}

__global__ void __launch_bounds__(kThreads, 1) wgrad_adam(const __grid_constant__ WgParams P) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ __nv_bfloat16 s_t[kTN][32 + 2];  // this CTA's 32 rows of the tile, transposed
  __shared__ int s_fail, s_loaded, s_consumed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tile = blockIdx.x / kSplits;
  const float lr = *P.lr;
  const float step = (float)(*P.step_base + P.step_offset);
  const float bc1 = 1.0f - powf(P.b1, step), bc2 = 1.0f - powf(P.b2, step);

  if (tile >= P.n_tiles) {
    // the bias cluster: Adam on every layer's bias
    for (int l = 0; l < P.n_layers; ++l) {
      const WgLayer& L = P.L[l];
      for (int i = rank * kThreads + tid; i < L.out; i += kSplits * kThreads) {
        float m1 = L.mb[i], m2 = L.vb[i];
        const float p = adam(L.gb[i], m1, m2, L.b[i], lr, P.b1, P.b2, P.eps, bc1, bc2);
        L.mb[i] = m1;
        L.vb[i] = m2;
        L.b[i] = p;
      }
    }
    return;
  }

  const WgLayer& L = P.L[P.tile_layer[tile]];
  const int m0 = P.tile_m[tile] * kTM, n0 = P.tile_n[tile] * kTN;
  const int kper = P.batch / kSplits, kbeg = rank * kper, nk = kper / kKS;
  const uint32_t ring = (smem_u32(smem_raw) + 1023u) & ~1023u;
  // received partial rows: [source rank][32 rows][kPS floats], after the ring
  const uint32_t recv = ring + (uint32_t)(kStages * kStage);
  const float* recv_ptr = reinterpret_cast<const float*>(smem_raw + (recv - smem_u32(smem_raw)));
  auto stA = [&](int s) { return ring + (uint32_t)(s * kStage); };
  auto stB = [&](int s) { return ring + (uint32_t)(s * kStage + kStageA); };
  const uint32_t mfull = smem_u32(&full[0]), mempty = smem_u32(&empty[0]), mdone = smem_u32(&done);

  if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), kTN);
  if (tid == 0) {
    s_fail = 0;
    s_loaded = s_consumed = 0;
    for (int s = 0; s < kStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mfull + 8 * s) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mempty + 8 * s) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mdone) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  // Warp 1 lane 0 streams slab j into stage j % kStages once the MMAs of
  // slab j - kStages are done; warp 0 lane 0 multiplies each slab as it
  // lands.  Neither waits for the other beyond what the data needs.
  constexpr uint32_t idesc = idesc_bf16(kTM, kTN);
  if (tid == 32) {
    int j = 0;
    for (; j < nk; ++j) {
      const int s = j % kStages;
      if (j >= kStages && !mbar_wait(mempty + 8 * s, (uint32_t)(j / kStages - 1) & 1u)) {
        atomicExch(&s_fail, 1);
        break;
      }
      expect_tx(mfull + 8 * s, kStage);
      tma_load_2d(stA(s), &L.mapA, kbeg + j * kKS, m0, mfull + 8 * s);
      tma_load_2d(stB(s), &L.mapB, kbeg + j * kKS, n0, mfull + 8 * s);
    }
    s_loaded = j;
  } else if (tid == 0) {
    int it = 0;
    for (; it < nk; ++it) {
      const int s = it % kStages;
      if (!mbar_wait(mfull + 8 * s, (uint32_t)(it / kStages) & 1u)) {
        atomicExch(&s_fail, 1);
        break;
      }
      fence_after();
#pragma unroll
      for (int kk = 0; kk < kKS / 16; ++kk)
        mma(tmem, sdesc_sw128(stA(s) + kk * 32), sdesc_sw128(stB(s) + kk * 32), idesc,
            (it > 0 || kk > 0) ? 1u : 0u);
      commit(mempty + 8 * s);
    }
    s_consumed = it;
    // every MMA issued, then the accumulator is complete
    commit(mdone);
    if (!mbar_wait(mdone, 0)) atomicExch(&s_fail, 1);
  }
  __syncthreads();
  const bool ok = *reinterpret_cast<volatile int*>(&s_fail) == 0;
  fence_after();
  if (!ok) {
    if (tid == 0) atomicExch(P.err, 1);
    // copies still in flight land before the CTA leaves (bounded waits)
    if (tid == 32)
      for (int j = s_consumed; j < s_loaded; ++j) mbar_wait(mfull + 8 * (j % kStages), (uint32_t)(j / kStages) & 1u);
  }

  // Accumulator rows 32 q .. 32 q + 31 (TMEM lane quadrant q) belong to CTA
  // q of the cluster: push them into its receive buffer (slot = this CTA's
  // rank) with distributed shared-memory stores, which nobody waits for.
  if (ok) {
    const int quad = warp & 3;  // TMEM lanes 32 quad .. +31; columns 32 (warp / 4) .. +31
#pragma unroll 1
    for (int c0 = 32 * (warp >> 2); c0 < 32 * (warp >> 2) + 32; c0 += 16) {
      float v[16];
      ld16(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)c0, v);
      const uint32_t local = recv + (uint32_t)(((rank * 32 + lane) * kPS + c0) * 4);
      uint32_t dst;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(dst) : "r"(local), "r"(quad));
#pragma unroll
      for (int j = 0; j < 4; ++j)
        asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(dst + 16 * j), "f"(v[4 * j]),
                     "f"(v[4 * j + 1]), "f"(v[4 * j + 2]), "f"(v[4 * j + 3])
                     : "memory");
    }
  }
  cluster.sync();  // every CTA's rows have arrived; no remote access follows
  if (ok) {
    // thread t: float4 column group t % 16 of rows t / 16 + 16 k (k = 0, 1);
    // every load is issued before any arithmetic
    constexpr int kRows = 32 * 16 / kThreads;  // rows per thread
    const int r0 = 32 * rank, c4 = 4 * (tid & 15), rr = tid >> 4;
    float4 pv[kRows][kSplits], wv[kRows], av[kRows], bv[kRows];
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
      const int off = (rr + 16 * k) * kPS + c4;
#pragma unroll
      for (int q = 0; q < kSplits; ++q) pv[k][q] = *reinterpret_cast<const float4*>(recv_ptr + q * 32 * kPS + off);
      const size_t i = (size_t)(m0 + r0 + rr + 16 * k) * L.in + n0 + c4;
      wv[k] = *reinterpret_cast<const float4*>(L.W + i);
      av[k] = *reinterpret_cast<const float4*>(L.m1 + i);
      bv[k] = *reinterpret_cast<const float4*>(L.m2 + i);
    }
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
      float4 g = pv[k][0];
#pragma unroll
      for (int q = 1; q < kSplits; ++q) {  // rank order
        g.x += pv[k][q].x;
        g.y += pv[k][q].y;
        g.z += pv[k][q].z;
        g.w += pv[k][q].w;
      }
      float4 w = wv[k], a = av[k], b = bv[k];
      w.x = adam(g.x, a.x, b.x, w.x, lr, P.b1, P.b2, P.eps, bc1, bc2);
      w.y = adam(g.y, a.y, b.y, w.y, lr, P.b1, P.b2, P.eps, bc1, bc2);
      w.z = adam(g.z, a.z, b.z, w.z, lr, P.b1, P.b2, P.eps, bc1, bc2);
      w.w = adam(g.w, a.w, b.w, w.w, lr, P.b1, P.b2, P.eps, bc1, bc2);
      const int r = rr + 16 * k;
      const size_t i = (size_t)(m0 + r0 + r) * L.in + n0 + c4;
      if (L.gW) *reinterpret_cast<float4*>(L.gW + i) = g;
      *reinterpret_cast<float4*>(L.m1 + i) = a;
      *reinterpret_cast<float4*>(L.m2 + i) = b;
      *reinterpret_cast<float4*>(L.W + i) = w;
      const __nv_bfloat16 h0 = __float2bfloat16_rn(w.x), h1 = __float2bfloat16_rn(w.y),
                          h2 = __float2bfloat16_rn(w.z), h3 = __float2bfloat16_rn(w.w);
      if (L.Wb) {
        const __nv_bfloat162 lo = __halves2bfloat162(h0, h1), hi = __halves2bfloat162(h2, h3);
        *reinterpret_cast<uint2*>(L.Wb + i) =
            make_uint2(*reinterpret_cast<const uint32_t*>(&lo), *reinterpret_cast<const uint32_t*>(&hi));
      }
      s_t[c4][r] = h0;
      s_t[c4 + 1][r] = h1;
      s_t[c4 + 2][r] = h2;
      s_t[c4 + 3][r] = h3;
    }
  }
  __syncthreads();
  if (ok && L.Wt) {
    // Wt[n0 + c][m0 + r0 .. + 31]: 64 rows of 32 bf16 (4 x 16 bytes each)
    for (int e = tid; e < kTN * 4; e += kThreads) {
      const int c = e >> 2, q = e & 3;
      uint32_t w[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 v = __halves2bfloat162(s_t[c][8 * q + 2 * k], s_t[c][8 * q + 2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t*>(&v);
      }
      *reinterpret_cast<uint4*>(L.Wt + (size_t)(n0 + c) * L.out + m0 + 32 * rank + 8 * q) =
          make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTN);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library), and a cache of encoded maps.
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

std::mutex g_map_mutex;
EncodeTiled g_encode = nullptr;
std::map<std::tuple<const void*, int, int, int, int>, CUtensorMap> g_maps;

// A bf16 [rows][ld] matrix (cols used), box cols x box_rows, 128-byte swizzle.
int make_map(const void* base, int rows, int cols, int ld, int box_rows, CUtensorMap* out) {
  std::lock_guard<std::mutex> lock(g_map_mutex);
  const auto key = std::make_tuple(base, rows, cols, ld, box_rows);
  auto it = g_maps.find(key);
  if (it != g_maps.end()) {
    *out = it->second;
    return MCL_OK;
  }
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    MCL_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn) return MCL_ECUDA;
    g_encode = reinterpret_cast<EncodeTiled>(fn);
  }
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kKS, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUtensorMap m;
  if (g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    mcl_set_last_message("cuTensorMapEncodeTiled refused a weight-gradient operand");
    return MCL_EINVAL;
  }
  if (g_maps.size() > 512) g_maps.clear();
  g_maps[key] = m;
  *out = m;
  return MCL_OK;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_wgrad_adam(const mcl_wgrad_layer* layers, int32_t n, int32_t batch, const float* lr,
                              const int32_t* step_base, int32_t step_offset, float b1, float b2, float eps,
                              int32_t* err, void* stream) {
  if (!layers || n < 1 || n > kMaxLayers || !lr || !step_base || !err) return MCL_EINVAL;
  if (batch <= 0 || batch % (kSplits * kKS)) return MCL_EINVAL;
  WgParams P;
  std::memset(&P, 0, sizeof(P));
  int tiles = 0;
  for (int l = 0; l < n; ++l) {
    const mcl_wgrad_layer& d = layers[l];
    if (d.out <= 0 || d.out % kTM || d.in <= 0 || d.in % kTN || d.ld < batch || d.ld % 8) return MCL_EINVAL;
    if (!d.dZt || !d.Xt || !d.W || !d.m1 || !d.m2 || !d.b || !d.gb || !d.mb || !d.vb) return MCL_EINVAL;
    if (!aligned16(d.dZt) || !aligned16(d.Xt) || (d.Wt && !aligned16(d.Wt))) return MCL_EINVAL;
    if (!aligned16(d.W) || !aligned16(d.m1) || !aligned16(d.m2) || (d.gW && !aligned16(d.gW)) ||
        ((uintptr_t)d.Wb & 7))
      return MCL_EINVAL;
    if (d.out / kTM > 255 || d.in / kTN > 255) return MCL_EINVAL;
    WgLayer& L = P.L[l];
    int rc = make_map(d.dZt, d.out, batch, d.ld, kTM, &L.mapA);
    if (rc != MCL_OK) return rc;
    rc = make_map(d.Xt, d.in, batch, d.ld, kTN, &L.mapB);
    if (rc != MCL_OK) return rc;
    L.W = d.W;
    L.m1 = d.m1;
    L.m2 = d.m2;
    L.Wb = reinterpret_cast<__nv_bfloat16*>(d.Wb);
    L.Wt = reinterpret_cast<__nv_bfloat16*>(d.Wt);
    L.gW = d.gW;
    L.b = d.b;
    L.gb = d.gb;
    L.mb = d.mb;
    L.vb = d.vb;
    L.out = d.out;
    L.in = d.in;
    for (int tm = 0; tm < d.out / kTM; ++tm)
      for (int tn = 0; tn < d.in / kTN; ++tn) {
        if (tiles >= kMaxTiles) return MCL_ECAPACITY;
        P.tile_layer[tiles] = (uint8_t)l;
        P.tile_m[tiles] = (uint8_t)tm;
        P.tile_n[tiles] = (uint8_t)tn;
        ++tiles;
      }
  }
  P.n_layers = n;
  P.n_tiles = tiles;
  P.batch = batch;
  P.step_offset = step_offset;
  P.lr = lr;
  P.step_base = step_base;
  P.err = err;
  P.b1 = b1;
  P.b2 = b2;
  P.eps = eps;
  MCL_CUDA_TRY(cudaFuncSetAttribute(wgrad_adam, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((tiles + 1) * kSplits), 1, 1);  // + the bias cluster
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = kSmem;
  cfg.stream = reinterpret_cast<cudaStream_t>(stream);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kSplits;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  MCL_CUDA_TRY(cudaLaunchKernelEx(&cfg, wgrad_adam, P));
  return MCL_OK;
}
