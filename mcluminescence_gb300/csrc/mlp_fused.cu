// The surrogate network in one persistent launch (no counterpart in the
// reference, whose parameter fit runs the Monte Carlo for every candidate,
// src/class/optimizer.py:93-111).
//
// One CTA of 16 warps owns 128 rows of the batch.  Its activations stay in
// shared memory, as the next GEMM's A operand in the no-swizzle K-major
// core-matrix layout (4 slabs of 64 columns), and each GEMM's accumulator
// (128 x 256 fp32) lives in tensor memory.  Per GEMM one thread issues
// tcgen05.mma (M 128, N 256, K 16) slab by slab as the B operand's slabs land,
// then commits to an mbarrier; as soon as the GEMM has completed, the CTA
// starts copying the next GEMM's B operand into the freed slabs and runs the
// epilogue (tcgen05.ld: warp w reads TMEM lanes 32 (w % 4) .. +31, i.e. tile
// rows, and columns 64 (w / 4) .. +63), which writes the next A operand.
// Transposed copies for the weight gradients go through a small per-warp
// shared tile so that global stores are 16-byte rows.  GELU' travels from a
// tile's forward epilogue to the same thread's backward epilogue, so it is
// kept in a layout private to the kernel in which each warp-wide float4
// access covers 512 contiguous bytes.
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
// afterwards as one grouped split-K launch (mcl_gemm_nt_tc_grouped).
//
// Every mbarrier wait is bounded; after a timeout the kernel records it in
// *err, waits (again bounded) for its last committed MMAs, frees its tensor
// memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "tcgen05.cuh"

namespace mcl {
namespace {
using namespace ::mcl::tcg;

constexpr int kRows = 128;     // batch rows per CTA: the MMA's M
constexpr int kWidth = 256;    // hidden width = padded output width: the MMA's N
constexpr int kIn = 64;        // padded input width
constexpr int kInValid = 6;
constexpr int kOutValid = 200;
constexpr int kThreads = 512;   // 16 warps: 4 per TMEM lane quadrant
constexpr int kWarps = kThreads / 32;
constexpr int kSlabK = 64;                       // K elements per staged slab
constexpr int kSlabA = kRows * kSlabK * 2;       // 16 KB
constexpr int kSlabB = kWidth * kSlabK * 2;      // 32 KB
constexpr int kOffB = 4 * kSlabA;                // B slabs after the 4 A slabs
constexpr int kOffCol = kOffB + 4 * kSlabB;      // bias-gradient column sums
constexpr int kOffBias = kOffCol + kWidth * 4;   // two 256-float bias buffers (GEMM parity)
constexpr int kOffT = kOffBias + 2 * kWidth * 4; // per-warp 16 x 32 bf16 transpose tiles
constexpr int kSmem = kOffT + kWarps * 1024;     // 216,064 bytes

__device__ __forceinline__ void cp_async_wait_n(int n) {
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 3;" ::: "memory"); break;
  }
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

// Write 16 values of row r, columns c0..c0+15, as bf16 into the A slabs.
__device__ __forceinline__ void store_a(uint32_t sa, int r, int c0, const float (&v)[16]) {
  st_shared_v4(sa + a_offset(r, c0), pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
               pack_bf16(v[6], v[7]));
  st_shared_v4(sa + a_offset(r, c0 + 8), pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]),
               pack_bf16(v[14], v[15]));
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

// Copy GEMM g's B operand into the B slabs (16-byte cp.async, one commit
// group per slab; each thread copies 4 chunks per slab).
__device__ __forceinline__ void issue_b(const mcl_mlp_args& a, int g, uint32_t sb) {
  int ld;
  const __nv_bfloat16* Bm = b_operand(a, g, ld);
  const int nslab = g == 0 ? 1 : 4;
  for (int s = 0; s < nslab; ++s) {
#pragma unroll
    for (int i = 0; i < kWidth * 8 / kThreads; ++i) {
      const int c = threadIdx.x + kThreads * i, r = c >> 3, kc = c & 7;
      cp_async16(sb + kOffB + s * kSlabB + ((r >> 3) * 8 + kc) * 128 + (r & 7) * 16,
                 Bm + (size_t)r * ld + s * kSlabK + kc * 8);
    }
    cp_async_commit();
  }
}

// Stage the bias the epilogue of GEMM g adds (forward layers only) into its
// shared buffer (g & 1); 64 threads copy a float4 each.
__device__ __forceinline__ void stage_bias(const mcl_mlp_args& a, int g, float* s_bias) {
  if (g < 5 && threadIdx.x < kWidth / 4)
    reinterpret_cast<float4*>(s_bias + (g & 1) * kWidth)[threadIdx.x] =
        reinterpret_cast<const float4*>(a.layer[g].bias)[threadIdx.x];
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

// GELU' of (warp quadrant, column part, chunk): 32 lanes x 16 floats at a
// private offset, float4 j of lane L at [j * 32 + L].
__device__ __forceinline__ float4* gelu_grad_block(float* base, int quad, int part, int ch) {
  return reinterpret_cast<float4*>(base) + ((((size_t)blockIdx.x * 4 + quad) * 4 + part) * 4 + ch) * 128;
}

template <bool TRAIN>
__global__ void __launch_bounds__(kThreads, 1) mlp_fused(const __grid_constant__ mcl_mlp_args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, part = warp >> 2;
  const int row = 32 * quad + lane;  // the tile row this thread finishes in every epilogue
  const int m0 = blockIdx.x * kRows;
  const int B = a.batch;
  const uint32_t sb = smem_u32(smem);
  float* s_col = reinterpret_cast<float*>(smem + kOffCol);
  __nv_bfloat16* tile = reinterpret_cast<__nv_bfloat16*>(smem + kOffT + warp * 1024);
  float* s_bias = reinterpret_cast<float*>(smem + kOffBias);
  const uint32_t mb = smem_u32(&mbar);
  constexpr int n_gemm = TRAIN ? 9 : 5;

  if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), kWidth);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < kWidth) s_col[tid] = 0.0f;
  // Layer 0's A operand: the tile's inputs (6 values, then zeros to 64).
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
    if (TRAIN && h == 0) {
      __nv_bfloat16* xt = reinterpret_cast<__nv_bfloat16*>(a.xt);
#pragma unroll
      for (int c = 0; c < kInValid; ++c) xt[(size_t)c * B + m] = __float2bfloat16_rn(xv[c]);
    }
  }
  issue_b(a, 0, sb);
  stage_bias(a, 0, s_bias);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t t_row = tmem + ((uint32_t)(32 * quad) << 16);
  constexpr uint32_t idesc = idesc_bf16(kRows, kWidth);

  bool ok = true;
  int last = -1;
  float loss = 0.0f;
  for (int g = 0; g < n_gemm; ++g) {
    const int nslab = g == 0 ? 1 : 4;
    for (int s = 0; s < nslab; ++s) {
      cp_async_wait_n(nslab - 1 - s);  // this thread's copies of slab s have landed
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();  // everyone's copies (and the previous epilogue's A writes) are visible
      if (tid == 0) {
        fence_after();
#pragma unroll
        for (int kk = 0; kk < kSlabK / 16; ++kk) {
          const uint64_t ad = sdesc(sb + s * kSlabA + kk * 256, 128, 1024);
          const uint64_t bd = sdesc(sb + kOffB + s * kSlabB + kk * 256, 128, 1024);
          mma(tmem, ad, bd, idesc, (s > 0 || kk > 0) ? 1u : 0u);
        }
        if (s == nslab - 1) commit(mb);
      }
      __syncwarp();
    }
    last = g;
    // one thread polls the barrier; the others wait at the CTA barrier
    const bool done = tid == 0 ? mbar_wait(mb, (uint32_t)g & 1u) : true;
    ok = __syncthreads_and(done ? 1 : 0) != 0;
    fence_after();
    if (!ok) break;
    if (g + 1 < n_gemm) {  // the B slabs are idle until the next GEMM
      issue_b(a, g + 1, sb);
      stage_bias(a, g + 1, s_bias);  // read after the next GEMM's barriers
    }

    if (g < 4) {
      // hidden layer g: z = acc + b; GELU into the next A operand
      const float* bias = s_bias + (g & 1) * kWidth;
#pragma unroll 1
      for (int ch = 0; ch < 4; ++ch) {
        const int c0 = 64 * part + 16 * ch;
        float v[16], bv[16];
        load16(bias + c0, bv);
        ld16(t_row + (uint32_t)c0, v);
        float y[16], gp[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          y[j] = gelu_and_grad(v[j] + bv[j], gp[j]);
        }
        store_a(sb, row, c0, y);
        if (TRAIN) {
          float4* G = gelu_grad_block(a.layer[g].gelu_grad, quad, part, ch);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            G[j * 32 + lane] = make_float4(gp[4 * j], gp[4 * j + 1], gp[4 * j + 2], gp[4 * j + 3]);
          store_t(tile, reinterpret_cast<__nv_bfloat16*>(a.layer[g].Yt), B, c0, m0 + 32 * quad, lane, y);
        }
      }
    } else if (g == 4) {
      // output layer: z = acc + b; in training also the loss and dZ_4
      const float* bias = s_bias + (4 & 1) * kWidth;
      const int m = m0 + row;
      const float* trow = nullptr;
      if (TRAIN) trow = a.target + (size_t)(a.idx ? a.idx[m] : (int64_t)m) * a.target_ld;
#pragma unroll 1
      for (int ch = 0; ch < 4; ++ch) {
        const int c0 = 64 * part + 16 * ch;
        float v[16], bv[16], tv[16];
        if (TRAIN) {  // issued before the tensor-memory read, so the latencies overlap
          if (c0 + 16 <= kOutValid) {
            load16(trow + c0, tv);
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) tv[j] = c0 + j < kOutValid ? trow[c0 + j] : 0.0f;
          }
        }
        load16(bias + c0, bv);
        ld16(t_row + (uint32_t)c0, v);
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
          store_a(sb, row, c0, dz);
          store_t(tile, reinterpret_cast<__nv_bfloat16*>(a.layer[4].dZt), B, c0, m0 + 32 * quad, lane, dz);
          int col;
          const float tot = column_sums(dz, lane, col);
          if ((lane & 1) == 0) atomicAdd(&s_col[c0 + col], tot);
        }
      }
    } else {
      // backward GEMM g for layer l = 9 - g gave dY_{l-1}: dZ_{l-1} = dY GELU'
      const int lz = 8 - g;

#pragma unroll 1
      for (int ch = 0; ch < 4; ++ch) {
        const int c0 = 64 * part + 16 * ch;
        float v[16];
        float4 gv[4];  // loaded before the tensor-memory read, so the latencies overlap
        const float4* G = gelu_grad_block(a.layer[lz].gelu_grad, quad, part, ch);
#pragma unroll
        for (int j = 0; j < 4; ++j) gv[j] = G[j * 32 + lane];
        ld16(t_row + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          v[4 * j] *= gv[j].x;
          v[4 * j + 1] *= gv[j].y;
          v[4 * j + 2] *= gv[j].z;
          v[4 * j + 3] *= gv[j].w;
        }
        store_a(sb, row, c0, v);
        store_t(tile, reinterpret_cast<__nv_bfloat16*>(a.layer[lz].dZt), B, c0, m0 + 32 * quad, lane, v);
        int col;
        const float tot = column_sums(v, lane, col);
        if ((lane & 1) == 0) atomicAdd(&s_col[c0 + col], tot);
      }
    }
    // the A writes go to the tensor core next; the TMEM reads are complete
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    if (TRAIN && g >= 4 && tid < kWidth) {  // this CTA's bias-gradient sums, one atomic per column
      const int lz = g == 4 ? 4 : 8 - g;
      const float cs = s_col[tid];
      if (cs != 0.0f) atomicAdd(&a.layer[lz].grad_b[tid], cs);
      s_col[tid] = 0.0f;
    }
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.err, 1);
    // a second, again bounded, wait for the last committed MMAs before the
    // tensor memory is freed
    if (last >= 0) mbar_wait(mb, (uint32_t)last & 1u);
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (TRAIN) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0 && loss != 0.0f) atomicAdd(a.loss, loss);
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kWidth);
}

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_mlp_fused(const mcl_mlp_args* args, void* stream) {
  if (!args) return MCL_EINVAL;
  const mcl_mlp_args& a = *args;
  if (a.batch <= 0 || a.batch % kRows || !a.x || !a.err) return MCL_EINVAL;
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
  auto kern = a.training ? mlp_fused<true> : mlp_fused<false>;
  MCL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
  kern<<<a.batch / kRows, kThreads, kSmem, s>>>(a);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
