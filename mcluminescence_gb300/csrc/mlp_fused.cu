// The surrogate network in one persistent launch (no counterpart in the
// reference, whose parameter fit runs the Monte Carlo for every candidate,
// src/class/optimizer.py:93-111).
//
// 128 rows of the batch belong to a thread-block cluster of SPLIT CTAs (1, 2
// or 4), each of 16 warps.  CTA q of the cluster computes output columns
// [q N, q N + N), N = 256 / SPLIT, of every GEMM: its accumulator (128 x N
// fp32) lives in tensor memory, its B operand is the matching N rows of the
// weights, and its epilogue writes those N columns of the next GEMM's A
// operand (bf16, no-swizzle K-major core-matrix layout, 4 slabs of 64
// columns) into its own shared memory; after one CTA barrier thread 0 sends
// them to every partner with bulk copies (cp.async.bulk.shared::cluster) that
// complete on the partner's mbarrier, so each CTA holds the whole 128 x 256
// activation tile when the next GEMM starts.  A batch of 4,096 rows thus
// keeps 128 SMs busy instead of 32.  With SPLIT > 1 the A operand is
// double-buffered; the data dependencies keep it safe without a cluster
// barrier per GEMM: a partner sends GEMM g + 1's columns only after its GEMM
// g, which needed this CTA's columns of GEMM g, so nobody overwrites an A
// buffer a partner may still multiply.  With SPLIT 4 the B operand is
// double-buffered too, so the weights of GEMM g + 2 stream in (16-byte
// cp.async) while GEMM g's epilogue runs.
//
// Per GEMM one thread issues tcgen05.mma (M 128, N, K 16) over the K slabs,
// once the partners' columns have landed, and commits to an mbarrier; the
// epilogue reads the accumulator with tcgen05.ld (warp w reads TMEM lanes
// 32 (w % 4) .. +31, i.e. tile rows, and a quarter of the N columns picked
// by w / 4); its critical part (the next A operand) ends with the CTA
// barrier, and the stores nobody waits for come after it.  Transposed copies
// for the weight gradients go through a small per-warp shared tile so that
// global stores are 16-byte rows.  GELU' travels from a tile's forward
// epilogue to the same thread's backward epilogue (the same CTA owns the
// same columns in both), so it is kept in a layout private to the kernel in
// which each warp-wide float4 access covers 512 contiguous bytes.
//
// GEMM sequence (training): forward layers 0..4, then the input-gradient
// chain for layers 4..1.  Epilogues:
//   hidden layer l:   z = acc + b_l; Y = bf16(GELU(z)) -> A; GELU'(z) and Y^T
//                     to global memory (backward's inputs)
//   output layer:     z = acc + b_4 -> out; d = z - target on the 200 valid
//                     columns; loss += d^2; dZ_4 = 2 d scale -> A (bf16),
//                     dZ_4^T to global, bias gradient column sums
//   backward layer l: dY_{l-1} = acc; dZ_{l-1} = dY_{l-1} GELU'(z_{l-1}) ->
//                     A (bf16), dZ^T to global, bias gradient column sums
// The weight gradients dW_l = dZ_l^T X_l reduce over the whole batch and run
// afterwards in their own launch (mcl_wgrad_adam, or the grouped split-K
// GEMM mcl_gemm_nt_tc_grouped).
//
// Every mbarrier wait is bounded.  After a timeout the CTA records it in
// *err, issues no further MMAs and sends no further columns (its partners'
// waits then time out in turn), waits (again bounded) for its last committed
// MMAs and for its own bulk copies, takes part in the final cluster barrier,
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "tcgen05.cuh"

namespace mcl {
namespace {
using namespace ::mcl::tcg;

constexpr int kRows = 128;     // batch rows per cluster: the MMA's M
constexpr int kWidth = 256;    // hidden width = padded output width
constexpr int kIn = 64;        // padded input width
constexpr int kInValid = 6;
constexpr int kOutValid = 200;
constexpr int kThreads = 512;   // 16 warps: 4 per TMEM lane quadrant
constexpr int kWarps = kThreads / 32;
constexpr int kSlabK = 64;                       // K elements per slab
constexpr int kSlabA = kRows * kSlabK * 2;       // 16 KB
constexpr int kBufA = 4 * kSlabA;                // one A operand: 128 x 256 bf16

// Shared-memory plan of a CTA of a SPLIT-wide cluster.
template <int SPLIT>
struct Plan {
  static constexpr int kN = kWidth / SPLIT;        // output columns per CTA: the MMA's N
  static constexpr int kChunks = kN / 64;          // 16-column chunks per warp and epilogue
  static constexpr int kNA = SPLIT > 1 ? 2 : 1;    // A buffers
  static constexpr int kNB = SPLIT == 4 ? 2 : 1;   // B buffers
  static constexpr int kSlabB = kN * kSlabK * 2;   // N rows x 64 K
  static constexpr int kBufB = 4 * kSlabB;
  static constexpr int kOffB = kNA * kBufA;
  static constexpr int kOffCol = kOffB + kNB * kBufB;  // two bias-gradient column-sum buffers (parity)
  static constexpr int kOffBias = kOffCol + 2 * kN * 4;  // two bias buffers (GEMM parity)
  static constexpr int kOffT = kOffBias + 2 * kN * 4;  // per-warp 16 x 32 bf16 transpose tiles
  static constexpr int kSmem = kOffT + kWarps * 1024;  // 214,016 / 215,040 / 217,088 bytes
};

__device__ __forceinline__ void cp_async_wait_n(int n) {
  if (n <= 0)
    asm volatile("cp.async.wait_group 0;" ::: "memory");
  else
    asm volatile("cp.async.wait_group 1;" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// All threads of all CTAs of the cluster; stores before the arrive (to any
// CTA's shared memory) are visible to every thread after the wait.  Between
// the two a thread does work nobody waits for.  A lone CTA uses a plain
// CTA barrier at the arrive.
template <int SPLIT>
__device__ __forceinline__ void cluster_arrive() {
  if constexpr (SPLIT > 1)
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  else
    __syncthreads();
}
template <int SPLIT>
__device__ __forceinline__ void cluster_wait() {
  if constexpr (SPLIT > 1) asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
template <int SPLIT>
__device__ __forceinline__ void cluster_barrier() {
  cluster_arrive<SPLIT>();
  cluster_wait<SPLIT>();
}

// Byte offset of (row r, column c, c a multiple of 8) in a core-matrix slab
// set of 128 rows: slab c / 64, 8-row group r / 8 (1,024 bytes apart),
// 8-column chunk (c % 64) / 8 (128 bytes apart), row r % 8 (16 bytes apart).
__device__ __forceinline__ uint32_t a_offset(int r, int c) {
  return (uint32_t)((c >> 6) * kSlabA + ((r >> 3) * 8 + ((c & 63) >> 3)) * 128 + (r & 7) * 16);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__device__ __forceinline__ void load16(const float* p, float (&v)[16]) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float4 t = q[j];
    v[4 * j] = t.x;
    v[4 * j + 1] = t.y;
    v[4 * j + 2] = t.z;
    v[4 * j + 3] = t.w;
  }
}

// Store the warp's 32 rows x 16 columns (c0..c0+15; lane = row r0 + lane)
// transposed into dst[c][m] (bf16, row length ld): through the warp's shared
// tile [16][32], then as 16-byte pieces of 8 consecutive rows.
__device__ __forceinline__ void store_t(__nv_bfloat16* tile, __nv_bfloat16* dst, int ld, int c0, int r0, int lane,
                                        const float (&v)[16]) {
#pragma unroll
  for (int j = 0; j < 16; ++j) tile[j * 32 + lane] = __float2bfloat16_rn(v[j]);
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int k = lane + 32 * i, j = k >> 2, q = k & 3;
    *reinterpret_cast<uint4*>(dst + (size_t)(c0 + j) * ld + r0 + 8 * q) =
        *reinterpret_cast<const uint4*>(tile + j * 32 + 8 * q);
  }
  __syncwarp();
}

// Sum 16 columns over the warp's 32 rows (one value per lane and column):
// halving exchanges leave lane pair (2i, 2i + 1) with the total of column
// col = bits 4..1 of the lane.  16 shuffles instead of 80.
__device__ __forceinline__ float column_sums(const float (&v)[16], int lane, int& col) {
  float a[8], b[4], c[2];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const bool up = lane & 16;
    const float send = up ? v[i] : v[i + 8], keep = up ? v[i + 8] : v[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool up = lane & 8;
    const float send = up ? a[i] : a[i + 4], keep = up ? a[i + 4] : a[i];
    b[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool up = lane & 4;
    const float send = up ? b[i] : b[i + 2], keep = up ? b[i + 2] : b[i];
    c[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  const bool up = lane & 2;
  float d = (up ? c[1] : c[0]) + __shfl_xor_sync(0xffffffffu, up ? c[0] : c[1], 2);
  d += __shfl_xor_sync(0xffffffffu, d, 1);
  col = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
  return d;
}


// Write 16 values of row r, columns c0..c0+15, as bf16 into the A operand
// slabs at shared address sa.
__device__ __forceinline__ void store_a(uint32_t sa, int r, int c0, const float (&v)[16]) {
  st_shared_v4(sa + a_offset(r, c0), pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
               pack_bf16(v[6], v[7]));
  st_shared_v4(sa + a_offset(r, c0 + 8), pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]),
               pack_bf16(v[14], v[15]));
}

// Copy `bytes` of this CTA's shared memory at `src` to the same offset in CTA
// `rank` of the cluster, completing on that CTA's mbarrier at the same offset
// as `mbar` (bulk asynchronous copy, one commit group).
__device__ __forceinline__ void push_to(uint32_t src, uint32_t bytes, uint32_t mbar, uint32_t rank) {
  uint32_t dst, rmb;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(dst) : "r"(src), "r"(rank));
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rmb) : "r"(mbar), "r"(rank));
  asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   dst),
               "r"(src), "r"(bytes), "r"(rmb)
               : "memory");
}

// The B operand of GEMM g: W_g (forward, g = 0..4) or W_l^T (backward, g =
// 5..8, l = 9 - g), 256 rows of K = 64 (g = 0) or 256 columns.
__device__ __forceinline__ const __nv_bfloat16* b_operand(const mcl_mlp_args& a, int g, int& ld) {
  if (g < 5) {
    ld = g == 0 ? kIn : kWidth;
    return reinterpret_cast<const __nv_bfloat16*>(a.layer[g].W);
  }
  ld = kWidth;
  return reinterpret_cast<const __nv_bfloat16*>(a.layer[9 - g].Wt);
}

// Copy rows [rank N, rank N + N) of GEMM g's B operand into B buffer `buf`
// (16-byte cp.async, one commit group per GEMM).
template <int SPLIT>
__device__ __forceinline__ void issue_b(const mcl_mlp_args& a, int g, uint32_t sb, int buf, int rank) {
  using P = Plan<SPLIT>;
  int ld;
  const __nv_bfloat16* W = b_operand(a, g, ld);
  const __nv_bfloat16* Bm = W + (size_t)rank * P::kN * ld;
  const int nslab = g == 0 ? 1 : 4;
  const uint32_t base = sb + P::kOffB + buf * P::kBufB;
  for (int s = 0; s < nslab; ++s) {
#pragma unroll
    for (int i = 0; i < P::kN * 8 / kThreads; ++i) {
      const int c = threadIdx.x + kThreads * i, r = c >> 3, kc = c & 7;
      cp_async16(base + s * P::kSlabB + ((r >> 3) * 8 + kc) * 128 + (r & 7) * 16,
                 Bm + (size_t)r * ld + s * kSlabK + kc * 8);
    }
  }
  cp_async_commit();
}

// Stage this CTA's N bias values of GEMM g (forward layers only) into bias
// buffer g & 1; N / 4 threads copy a float4 each.
template <int SPLIT>
__device__ __forceinline__ void stage_bias(const mcl_mlp_args& a, int g, float* s_bias, int rank) {
  using P = Plan<SPLIT>;
  if (g < 5 && threadIdx.x < P::kN / 4)
    reinterpret_cast<float4*>(s_bias + (g & 1) * P::kN)[threadIdx.x] =
        reinterpret_cast<const float4*>(a.layer[g].bias + rank * P::kN)[threadIdx.x];
}

// GELU(z) = z Phi(z) and GELU'(z) = Phi(z) + z phi(z), with Phi the
// standard normal CDF and phi its density.  erf comes from Abramowitz &
// Stegun, Handbook of Mathematical Functions, formula 7.1.26 (|error| <=
// 1.5e-7): 1 - erf(x) = (a1 t + a2 t^2 + a3 t^3 + a4 t^4 + a5 t^5) e^{-x^2},
// t = 1 / (1 + p x), x >= 0.  With x = |z| / sqrt(2) the exponential is
// e^{-z^2 / 2}, shared with phi; h = (1 - erf(x)) / 2 gives Phi = h for z < 0
// and 1 - h otherwise, without cancellation in the lower tail.
__device__ __forceinline__ float gelu_and_grad(float z, float& grad) {
  const float t = __fdividef(1.0f, fmaf(0.3275911f * 0.70710678118654752f, fabsf(z), 1.0f));
  const float e = __expf(-0.5f * z * z);
  const float poly =
      ((((1.061405429f * t - 1.453152027f) * t + 1.421413741f) * t - 0.284496736f) * t + 0.254829592f) * t;
  const float h = 0.5f * poly * e;
  const float cdf = z < 0.0f ? h : 1.0f - h;
  grad = fmaf(z, 0.39894228040143268f * e, cdf);
  return z * cdf;
}

// GELU' of (CTA, warp quadrant, column part, chunk): 32 lanes x 16 floats at
// a private offset, float4 j of lane L at [j * 32 + L].  Each CTA owns
// 128 x N floats of the batch x 256 buffer.
template <int SPLIT>
__device__ __forceinline__ float4* gelu_grad_block(float* base, int quad, int part, int ch) {
  constexpr int kCh = Plan<SPLIT>::kChunks;
  return reinterpret_cast<float4*>(base) + ((((size_t)blockIdx.x * 4 + quad) * 4 + part) * kCh + ch) * 128;
}

template <bool TRAIN, int SPLIT>
__global__ void __launch_bounds__(kThreads, 1) mlp_fused(const __grid_constant__ mcl_mlp_args a) {
  using P = Plan<SPLIT>;
  constexpr int kN = P::kN;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t abar[2];  // A buffer b: the partners' slabs have landed
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, part = warp >> 2;
  const int row = 32 * quad + lane;  // the tile row this thread finishes in every epilogue
  const int rank = SPLIT > 1 ? (int)cluster_rank() : 0;
  const int m0 = (blockIdx.x / SPLIT) * kRows;
  const int n0 = rank * kN;          // this CTA's first output column
  const int B = a.batch;
  const uint32_t sb = smem_u32(smem);
  float* s_col = reinterpret_cast<float*>(smem + P::kOffCol);
  __nv_bfloat16* tile = reinterpret_cast<__nv_bfloat16*>(smem + P::kOffT + warp * 1024);
  float* s_bias = reinterpret_cast<float*>(smem + P::kOffBias);
  const uint32_t mb = smem_u32(&mbar);
  const uint32_t ab = smem_u32(&abar[0]);  // abar[b] at ab + 8 b
  constexpr int n_gemm = TRAIN ? 9 : 5;
  // bytes of A operand one CTA sends to each partner, and receives in all
  constexpr uint32_t kSlabsOwn = kN / kSlabK;
  constexpr uint32_t kBytesOut = kSlabsOwn * kSlabA, kBytesIn = (SPLIT - 1) * kBytesOut;

  if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), kN);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ab) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ab + 8) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < 2 * kN) s_col[tid] = 0.0f;
  // Layer 0's A operand (buffer 0, every CTA its own copy): the tile's
  // inputs (6 values, then zeros to 64).
  {
    const int r = tid >> 2, h = tid & 3, m = m0 + r;
    const int64_t src = a.idx ? a.idx[m] : (int64_t)m;
    float xv[kInValid];
#pragma unroll
    for (int c = 0; c < kInValid; ++c) xv[c] = a.x[src * kInValid + c];
#pragma unroll
    for (int kc = 2 * h; kc < 2 * h + 2; ++kc) {
      float v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = (8 * kc + e < kInValid) ? xv[8 * kc + e] : 0.0f;
      st_shared_v4(sb + a_offset(r, 8 * kc), pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                   pack_bf16(v[6], v[7]));
    }
    if (TRAIN && h == 0 && rank == 0) {
      __nv_bfloat16* xt = reinterpret_cast<__nv_bfloat16*>(a.xt);
#pragma unroll
      for (int c = 0; c < kInValid; ++c) xt[(size_t)c * B + m] = __float2bfloat16_rn(xv[c]);
    }
  }
  for (int g = 0; g < P::kNB; ++g) issue_b<SPLIT>(a, g, sb, g, rank);
  stage_bias<SPLIT>(a, 0, s_bias, rank);
  cp_async_wait_n(P::kNB - 1);  // this thread's copies of GEMM 0's B operand have landed
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before();
  // every CTA of the cluster has started (its shared memory may be written)
  cluster_barrier<SPLIT>();
  fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t t_row = tmem + ((uint32_t)(32 * quad) << 16);
  constexpr uint32_t idesc = idesc_bf16(kRows, kN);

  bool ok = true;
  int pending = -1;      // the last GEMM whose MMAs were committed when a wait timed out
  uint32_t aphase = 0;   // thread 0: parity bit b = the phase of abar[b] to wait for
  float loss = 0.0f;
  for (int g = 0; g < n_gemm; ++g) {
    const uint32_t sa = sb + (g % P::kNA) * kBufA;
    const uint32_t sbb = sb + P::kOffB + (g % P::kNB) * P::kBufB;
    bool issued = false;
    if (ok && tid == 0) {
      bool landed = true;
      if (SPLIT > 1 && g >= 1) {
        // the partners' columns of this A operand (bulk copies into buffer g % 2)
        const uint32_t b = (uint32_t)g & 1u, bar = ab + 8 * b;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kBytesIn) : "memory");
        landed = mbar_wait(bar, (aphase >> b) & 1u);
        aphase ^= 1u << b;
      }
      if (landed) issued = true;
    }
    if (issued) {
      fence_after();
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const int nslab = g == 0 ? 1 : 4;
      for (int s = 0; s < nslab; ++s) {
#pragma unroll
        for (int kk = 0; kk < kSlabK / 16; ++kk) {
          const uint64_t ad = sdesc(sa + s * kSlabA + kk * 256, 128, 1024);
          const uint64_t bd = sdesc(sbb + s * P::kSlabB + kk * 256, 128, 1024);
          mma(tmem, ad, bd, idesc, (s > 0 || kk > 0) ? 1u : 0u);
        }
      }
      commit(mb);
    }
    // one thread polls the barrier; the others wait at the CTA barrier
    const bool done = (tid == 0 && ok) ? (issued && mbar_wait(mb, (uint32_t)g & 1u)) : true;
    if (__syncthreads_and(done ? 1 : 0) == 0 && ok) {
      ok = false;
      pending = issued ? g : g - 1;
    }
    fence_after();
    if (TRAIN && ok && g >= 5 && tid < kN) {
      // the previous epilogue's bias-gradient sums (complete: every thread
      // added them before this CTA barrier), one atomic per column
      const int lz = g == 5 ? 4 : 9 - g;
      float* sc = s_col + ((g - 1) & 1) * kN;
      const float cs = sc[tid];
      if (cs != 0.0f) atomicAdd(&a.layer[lz].grad_b[n0 + tid], cs);
      sc[tid] = 0.0f;
    }
    // The next GEMM's operands are ready once every thread's A writes and B
    // copies have landed (and are ordered before the async proxy) and its
    // TMEM reads are done: one CTA barrier, after which thread 0 sends this
    // CTA's columns of the next A operand to the partners (bulk copies that
    // complete on their abar).  The stores nobody waits for come after.
    const uint32_t sa_next = sb + ((g + 1) % P::kNA) * kBufA;
    const bool feed = g + 1 < n_gemm;
    bool arrived = false;
    auto arrive = [&]() {
      cp_async_wait_n((P::kNB == 2 && g + 2 < n_gemm) ? 1 : 0);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      fence_before();
      __syncthreads();
      if (SPLIT > 1 && feed && ok && tid == 0) {
        const uint32_t src = sa_next + (uint32_t)rank * kBytesOut;
        const uint32_t bar = ab + 8 * ((uint32_t)(g + 1) & 1u);
        for (int q = 1; q < SPLIT; ++q) push_to(src, kBytesOut, bar, (uint32_t)((rank + q) % SPLIT));
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      }
      arrived = true;
    };
    float* s_colg = s_col + (g & 1) * kN;
    if (ok) {
      if (g + P::kNB < n_gemm)  // the B buffer GEMM g read is free
        issue_b<SPLIT>(a, g + P::kNB, sb, g % P::kNB, rank);
      stage_bias<SPLIT>(a, g + 1, s_bias, rank);  // read after the next barrier
    }

    if (!ok) {
      // no epilogue: keep pace with the partners' barriers only
    } else if (g < 4) {
      // hidden layer g: z = acc + b; GELU into the next A operand
      const float* bias = s_bias + (g & 1) * kN;
#pragma unroll 1
      for (int ch = 0; ch < P::kChunks; ++ch) {
        const int cl = part * (kN / 4) + 16 * ch, c0 = n0 + cl;
        float v[16], bv[16];
        load16(bias + cl, bv);
        ld16(t_row + (uint32_t)cl, v);
        float y[16], gp[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          y[j] = gelu_and_grad(v[j] + bv[j], gp[j]);
        }
        store_a(sa_next, row, c0, y);
        if (ch == P::kChunks - 1) arrive();
        if (TRAIN) {
          float4* G = gelu_grad_block<SPLIT>(a.layer[g].gelu_grad, quad, part, ch);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            G[j * 32 + lane] = make_float4(gp[4 * j], gp[4 * j + 1], gp[4 * j + 2], gp[4 * j + 3]);
          store_t(tile, reinterpret_cast<__nv_bfloat16*>(a.layer[g].Yt), B, c0, m0 + 32 * quad, lane, y);
        }
      }
    } else if (g == 4) {
      // output layer: z = acc + b; in training also the loss and dZ_4
      const float* bias = s_bias + (4 & 1) * kN;
      const int m = m0 + row;
      const float* trow = nullptr;
      if (TRAIN) trow = a.target + (size_t)(a.idx ? a.idx[m] : (int64_t)m) * a.target_ld;
#pragma unroll 1
      for (int ch = 0; ch < P::kChunks; ++ch) {
        const int cl = part * (kN / 4) + 16 * ch, c0 = n0 + cl;
        float v[16], bv[16], tv[16];
        if (TRAIN) {  // issued before the tensor-memory read, so the latencies overlap
          if (c0 + 16 <= kOutValid) {
            load16(trow + c0, tv);
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) tv[j] = c0 + j < kOutValid ? trow[c0 + j] : 0.0f;
          }
        }
        load16(bias + cl, bv);
        ld16(t_row + (uint32_t)cl, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] += bv[j];
        if (a.out) {
          float4* O = reinterpret_cast<float4*>(a.out + (size_t)m * kWidth + c0);
#pragma unroll
          for (int j = 0; j < 4; ++j) O[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
        if (TRAIN) {
          float dz[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int c = c0 + j;
            const float d = c < kOutValid ? v[j] - tv[j] : 0.0f;
            loss += d * d;
            dz[j] = 2.0f * d * a.loss_scale;
          }
          store_a(sa_next, row, c0, dz);
          if (ch == P::kChunks - 1) arrive();
          store_t(tile, reinterpret_cast<__nv_bfloat16*>(a.layer[4].dZt), B, c0, m0 + 32 * quad, lane, dz);
          int col;
          const float tot = column_sums(dz, lane, col);
          if ((lane & 1) == 0) atomicAdd(&s_colg[cl + col], tot);
        }
      }
    } else {
      // backward GEMM g for layer l = 9 - g gave dY_{l-1}: dZ_{l-1} = dY GELU'
      const int lz = 8 - g;
#pragma unroll 1
      for (int ch = 0; ch < P::kChunks; ++ch) {
        const int cl = part * (kN / 4) + 16 * ch, c0 = n0 + cl;
        float v[16];
        float4 gv[4];  // loaded before the tensor-memory read, so the latencies overlap
        const float4* G = gelu_grad_block<SPLIT>(a.layer[lz].gelu_grad, quad, part, ch);
#pragma unroll
        for (int j = 0; j < 4; ++j) gv[j] = G[j * 32 + lane];
        ld16(t_row + (uint32_t)cl, v);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          v[4 * j] *= gv[j].x;
          v[4 * j + 1] *= gv[j].y;
          v[4 * j + 2] *= gv[j].z;
          v[4 * j + 3] *= gv[j].w;
        }
        if (feed) store_a(sa_next, row, c0, v);
        if (ch == P::kChunks - 1) arrive();
        store_t(tile, reinterpret_cast<__nv_bfloat16*>(a.layer[lz].dZt), B, c0, m0 + 32 * quad, lane, v);
        int col;
        const float tot = column_sums(v, lane, col);
        if ((lane & 1) == 0) atomicAdd(&s_colg[cl + col], tot);
      }
    }
    if (!arrived) arrive();  // inference's output layer, or after a timeout
    fence_after();
  }
  // every bulk copy this CTA issued has completed, in every partner, before
  // any CTA of the cluster leaves
  if (SPLIT > 1 && tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  cluster_barrier<SPLIT>();
  if (TRAIN && ok && tid < kN) {  // the last epilogue's bias-gradient sums (layer 0)
    const float cs = s_col[((n_gemm - 1) & 1) * kN + tid];
    if (cs != 0.0f) atomicAdd(&a.layer[0].grad_b[n0 + tid], cs);
  }
  if (!ok) {
    if (tid == 0) {
      atomicExch(a.err, 1);
      // a second, again bounded, wait for the MMAs that timed out before the
      // tensor memory is freed
      mbar_wait(mb, (uint32_t)pending & 1u);
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (TRAIN) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0 && loss != 0.0f) atomicAdd(a.loss, loss);
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kN);
}

template <bool TRAIN, int SPLIT>
int launch(const mcl_mlp_args& a, cudaStream_t s) {
  auto kern = mlp_fused<TRAIN, SPLIT>;
  constexpr int smem = Plan<SPLIT>::kSmem;
  MCL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.batch / kRows * SPLIT), 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = SPLIT;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  MCL_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, a));
  return MCL_OK;
}

template <bool TRAIN>
int launch_split(const mcl_mlp_args& a, int split, cudaStream_t s) {
  if (split == 1) return launch<TRAIN, 1>(a, s);
  if (split == 2) return launch<TRAIN, 2>(a, s);
  return launch<TRAIN, 4>(a, s);
}

// Clusters of each size that fit on the device at once (queried once per
// device; index 0, 1, 2 for SPLIT 1, 2, 4).
constexpr int kMaxDevices = 64;
std::mutex g_fit_mutex;
int g_fit[kMaxDevices][3] = {};

template <int SPLIT>
int clusters_that_fit(int& out) {
  auto kern = mlp_fused<true, SPLIT>;
  constexpr int smem = Plan<SPLIT>::kSmem;
  MCL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(SPLIT, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = SPLIT;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  MCL_CUDA_TRY(cudaOccupancyMaxActiveClusters(&out, kern, &cfg));
  return MCL_OK;
}

// The split with the fewest waves of clusters per unit of work: with T
// tiles and C clusters of SPLIT resident at once, time ~ ceil(T / C) / SPLIT
// (each CTA does 1 / SPLIT of a tile's work); ties go to the smaller split.
int pick_split(int tiles) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
  std::lock_guard<std::mutex> lock(g_fit_mutex);
  int* fit = g_fit[dev];
  if (!fit[0]) {
    if (clusters_that_fit<1>(fit[0]) != MCL_OK || clusters_that_fit<2>(fit[1]) != MCL_OK ||
        clusters_that_fit<4>(fit[2]) != MCL_OK) {
      fit[0] = 0;
      return 1;
    }
  }
  int best = 1;
  double best_cost = 1e30;
  const int splits[3] = {1, 2, 4};
  for (int i = 0; i < 3; ++i) {
    if (fit[i] <= 0) continue;
    const double cost = (double)((tiles + fit[i] - 1) / fit[i]) / splits[i];
    if (cost < best_cost - 1e-9) {
      best_cost = cost;
      best = splits[i];
    }
  }
  return best;
}

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_mlp_fused(const mcl_mlp_args* args, void* stream) {
  if (!args) return MCL_EINVAL;
  const mcl_mlp_args& a = *args;
  if (a.batch <= 0 || a.batch % kRows || !a.x || !a.err) return MCL_EINVAL;
  if (a.split != 0 && a.split != 1 && a.split != 2 && a.split != 4) return MCL_EINVAL;
  for (int l = 0; l < 5; ++l) {
    const mcl_mlp_layer& L = a.layer[l];
    if (!L.W || !L.bias || ((uintptr_t)L.W & 15)) return MCL_EINVAL;
    if (a.training) {
      if (!L.grad_b || !L.dZt) return MCL_EINVAL;
      if (l < 4 && (!L.gelu_grad || !L.Yt || ((uintptr_t)L.gelu_grad & 15))) return MCL_EINVAL;
      if (l > 0 && (!L.Wt || ((uintptr_t)L.Wt & 15))) return MCL_EINVAL;
    }
  }
  if (a.training && (!a.target || !a.xt || !a.loss || a.target_ld < kOutValid || a.target_ld % 4 ||
                     ((uintptr_t)a.target & 15) || ((uintptr_t)a.xt & 15)))
    return MCL_EINVAL;
  for (int l = 0; a.training && l < 5; ++l)
    if (((uintptr_t)a.layer[l].dZt & 15) || (l < 4 && ((uintptr_t)a.layer[l].Yt & 15))) return MCL_EINVAL;
  if (((uintptr_t)a.x & 3) || ((uintptr_t)a.layer[0].bias & 15)) return MCL_EINVAL;
  for (int l = 1; l < 5; ++l)
    if ((uintptr_t)a.layer[l].bias & 15) return MCL_EINVAL;
  if (a.out && ((uintptr_t)a.out & 15)) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int split = a.split ? a.split : pick_split(a.batch / kRows);
  return a.training ? launch_split<true>(a, split, s) : launch_split<false>(a, split, s);
}
