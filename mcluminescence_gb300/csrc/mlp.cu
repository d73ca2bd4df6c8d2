// Surrogate network kernels: BF16-input / FP32-accumulate GEMM with fused
// epilogues, GELU backward, MSE loss and Adam.  The network maps six physics
// parameters to a 200-bin glow curve (6 -> 256 -> 256 -> 256 -> 256 -> 200,
// GELU); it has no counterpart in the reference, whose parameter fit
// (src/class/optimizer.py:93-111) calls the Monte Carlo for every candidate.
//
// All GEMMs are "NT": C[m][n] = sum_k A[m][k] * B[n][k], both operands stored
// with k contiguous (row-major A, and B as an out x in weight matrix like
// torch.nn.Linear).  Tiles of 64 x 64 x 32 per CTA, four warps of 32 x 32,
// mma.sync m16n8k16 BF16 tensor-core instructions fed by ldmatrix from padded
// shared memory.  M and N must be multiples of 64, K a multiple of 32 (the
// host pads 6 -> 32 inputs and 200 -> 256 outputs with zeros).
#include <cuda_bf16.h>

#include "common.cuh"

namespace mcl {
namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int PAD = 8;              // bf16 elements of row padding (bank spread)
constexpr int LDS = BK + PAD;       // shared-memory row stride (elements)

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  return cdf + z * pdf;
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}

__device__ __forceinline__ void ldmatrix_x2(uint32_t (&r)[2], const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Epilogue modes
constexpr int EPI_F32 = 0;        // C (fp32) = acc
constexpr int EPI_BIAS = 1;       // C (fp32) = acc + bias
constexpr int EPI_BIAS_GELU = 2;  // Z (fp32) = acc + bias; Y = gelu(Z) as bf16 [M][N] and [N][M]

template <int EPI>
__global__ void __launch_bounds__(128) gemm_nt(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                               int lda, const __nv_bfloat16* __restrict__ B, int ldb,
                                               const float* __restrict__ bias, float* __restrict__ C, int ldc,
                                               __nv_bfloat16* __restrict__ Y, int ldy,
                                               __nv_bfloat16* __restrict__ Yt, int ldyt) {
  __shared__ __align__(16) __nv_bfloat16 sA[BM * LDS];
  __shared__ __align__(16) __nv_bfloat16 sB[BN * LDS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;

  for (int k0 = 0; k0 < K; k0 += BK) {
    // 64 rows x 32 cols of bf16 = 4 KB per operand; 128 threads x 2 x 16 B
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 128;   // 0..255: row = idx / 4, 8-element column group = idx % 4
      const int row = idx >> 2, cg = (idx & 3) * 8;
      *reinterpret_cast<uint4*>(&sA[row * LDS + cg]) =
          *reinterpret_cast<const uint4*>(&A[(size_t)(m0 + row) * lda + k0 + cg]);
      *reinterpret_cast<uint4*>(&sB[row * LDS + cg]) =
          *reinterpret_cast<const uint4*>(&B[(size_t)(n0 + row) * ldb + k0 + cg]);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        // rows wm + 16i + (lane & 15), columns kk + 8 * (lane >> 4)
        const int row = wm + 16 * i + (lane & 15);
        ldmatrix_x4(af[i], &sA[row * LDS + kk + 8 * (lane >> 4)]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        // B^T rows (n) wn + 8j + (lane & 7), k columns kk + 8 * ((lane >> 3) & 1)
        const int row = wn + 8 * j + (lane & 7);
        ldmatrix_x2(bfr[j], &sB[row * LDS + kk + 8 * ((lane >> 3) & 1)]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }

  // epilogue: acc[i][j][q] sits at row wm + 16i + g (+8 for q >= 2), column wn + 8j + 2t (+1 for odd q)
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = m0 + wm + 16 * i + g + (q >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * t + (q & 1);
        float v = acc[i][j][q];
        if (EPI != EPI_F32) v += bias[n];
        C[(size_t)m * ldc + n] = v;
        if (EPI == EPI_BIAS_GELU) {
          const __nv_bfloat16 y = __float2bfloat16_rn(gelu(v));
          Y[(size_t)m * ldy + n] = y;
          if (Yt) Yt[(size_t)n * ldyt + m] = y;
        }
      }
  (void)M;
}

// dZ = dY * gelu'(Z) (or dZ = dY for a linear layer) as bf16 in [M][N] and
// [N][M], and db[n] += sum over this CTA's rows of dZ (fp32 atomics).
__global__ void __launch_bounds__(256) act_backward(int M, int N, const float* __restrict__ dY, int lddy,
                                                    const float* __restrict__ Z, int ldz, int gelu_on,
                                                    __nv_bfloat16* __restrict__ dZ, int lddz,
                                                    __nv_bfloat16* __restrict__ dZt, int lddzt,
                                                    float* __restrict__ db) {
  // CTA: 32 rows x 256 columns chunk; each thread one column, loops the rows
  const int n = blockIdx.x * 256 + threadIdx.x;
  const int m0 = blockIdx.y * 32;
  if (n >= N) return;
  float colsum = 0.0f;
  for (int r = 0; r < 32; ++r) {
    const int m = m0 + r;
    if (m >= M) break;
    float d = dY[(size_t)m * lddy + n];
    if (gelu_on) d *= gelu_grad(Z[(size_t)m * ldz + n]);
    const __nv_bfloat16 b = __float2bfloat16_rn(d);
    dZ[(size_t)m * lddz + n] = b;
    dZt[(size_t)n * lddzt + m] = b;
    colsum += d;
  }
  atomicAdd(&db[n], colsum);
}

// loss += sum over valid columns of (out - target)^2; dOut = 2 (out - target) * scale
__global__ void __launch_bounds__(256) mse_loss(int M, int N, int n_valid, const float* __restrict__ out, int ldo,
                                                const float* __restrict__ target, int ldt, float scale,
                                                float* __restrict__ dout, int ldd, float* __restrict__ loss) {
  const int64_t total = (int64_t)M * N;
  float part = 0.0f;
  for (int64_t idx = blockIdx.x * 256ll + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * 256) {
    const int m = (int)(idx / N), n = (int)(idx % N);
    float d = 0.0f;
    if (n < n_valid) {
      d = out[(size_t)m * ldo + n] - target[(size_t)m * ldt + n];
      part += d * d;
    }
    dout[(size_t)m * ldd + n] = 2.0f * d * scale;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part);
}

// Adam on fp32 master weights; refreshes the bf16 copies W[rows][cols] and
// its transpose Wt[cols][rows] (either may be null).
__global__ void __launch_bounds__(256) adam_update(int rows, int cols, float* __restrict__ p,
                                                   const float* __restrict__ g, float* __restrict__ m1,
                                                   float* __restrict__ m2, float lr, float b1, float b2,
                                                   float eps, float bc1, float bc2,
                                                   __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ Wt) {
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.0f - b1) * gi;
    const float b = b2 * m2[i] + (1.0f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float mh = a / bc1, vh = b / bc2;
    const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
    p[i] = pi;
    const __nv_bfloat16 q = __float2bfloat16_rn(pi);
    if (W) W[i] = q;
    if (Wt) Wt[(size_t)(i % cols) * rows + i / cols] = q;
  }
}

__global__ void __launch_bounds__(256) f32_to_bf16(int64_t n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) y[i] = __float2bfloat16_rn(x[i]);
}

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_gemm_nt(int32_t epilogue, int32_t M, int32_t N, int32_t K, const void* A, int32_t lda,
                           const void* B, int32_t ldb, const float* bias, float* C, int32_t ldc, void* Y,
                           int32_t ldy, void* Yt, int32_t ldyt, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || M % BM || N % BN || K % BK) return MCL_EINVAL;
  if (!A || !B || !C || lda < K || ldb < K || ldc < N || (lda % 8) || (ldb % 8)) return MCL_EINVAL;
  if (((uintptr_t)A | (uintptr_t)B) & 15) return MCL_EINVAL;
  if (epilogue != EPI_F32 && !bias) return MCL_EINVAL;
  if (epilogue == EPI_BIAS_GELU && (!Y || ldy < N || (Yt && ldyt < M))) return MCL_EINVAL;
  dim3 grid(N / BN, M / BM);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const auto* a = reinterpret_cast<const __nv_bfloat16*>(A);
  const auto* b = reinterpret_cast<const __nv_bfloat16*>(B);
  auto* y = reinterpret_cast<__nv_bfloat16*>(Y);
  auto* yt = reinterpret_cast<__nv_bfloat16*>(Yt);
  switch (epilogue) {
    case EPI_F32: gemm_nt<EPI_F32><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt); break;
    case EPI_BIAS: gemm_nt<EPI_BIAS><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt); break;
    case EPI_BIAS_GELU: gemm_nt<EPI_BIAS_GELU><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt); break;
    default: return MCL_EINVAL;
  }
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_act_backward(int32_t M, int32_t N, const float* dY, int32_t lddy, const float* Z, int32_t ldz,
                                int32_t gelu_on, void* dZ, int32_t lddz, void* dZt, int32_t lddzt, float* db,
                                void* stream) {
  if (M <= 0 || N <= 0 || !dY || !dZ || !dZt || !db || (gelu_on && !Z)) return MCL_EINVAL;
  dim3 grid((N + 255) / 256, (M + 31) / 32);
  act_backward<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      M, N, dY, lddy, Z, ldz, gelu_on, reinterpret_cast<__nv_bfloat16*>(dZ), lddz,
      reinterpret_cast<__nv_bfloat16*>(dZt), lddzt, db);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_mse_loss(int32_t M, int32_t N, int32_t n_valid, const float* out, int32_t ldo,
                            const float* target, int32_t ldt, float scale, float* dout, int32_t ldd,
                            float* loss, void* stream) {
  if (M <= 0 || N <= 0 || n_valid > N || !out || !target || !dout || !loss) return MCL_EINVAL;
  const int64_t total = (int64_t)M * N;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 4096);
  mse_loss<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(M, N, n_valid, out, ldo, target, ldt,
                                                                      scale, dout, ldd, loss);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_adam(int32_t rows, int32_t cols, float* p, const float* g, float* m1, float* m2, float lr,
                        float b1, float b2, float eps, int32_t step, void* W, void* Wt, void* stream) {
  if (rows <= 0 || cols <= 0 || !p || !g || !m1 || !m2 || step < 1) return MCL_EINVAL;
  const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
  const int64_t n = (int64_t)rows * cols;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 2048);
  adam_update<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      rows, cols, p, g, m1, m2, lr, b1, b2, eps, bc1, bc2, reinterpret_cast<__nv_bfloat16*>(W),
      reinterpret_cast<__nv_bfloat16*>(Wt));
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_f32_to_bf16(int64_t n, const float* x, void* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return MCL_EINVAL;
  if (n == 0) return MCL_OK;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  f32_to_bf16<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(n, x, reinterpret_cast<__nv_bfloat16*>(y));
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
