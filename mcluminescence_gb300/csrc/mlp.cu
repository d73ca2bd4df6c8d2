// Surrogate network kernels: BF16-input / FP32-accumulate GEMM with fused
// epilogues, GELU backward, MSE loss and Adam.  The network maps six physics
// parameters to a 200-bin glow curve (6 -> 256 -> 256 -> 256 -> 256 -> 200,
// GELU); it has no counterpart in the reference, whose parameter fit
// (src/class/optimizer.py:93-111) calls the Monte Carlo for every candidate.
//
// All GEMMs are "NT": C[m][n] = sum_k A[m][k] * B[n][k], both operands stored
// with k contiguous (row-major A, and B as an out x in weight matrix like
// torch.nn.Linear).  Two implementations: gemm_nt_tc on the tcgen05 tensor
// cores with the accumulator in tensor memory (used whenever the shape tiles
// by 128 x 64 x 64, i.e. every GEMM of the surrogate at batch sizes that are
// multiples of 128), and gemm_nt with mma.sync m16n8k16 instructions fed by
// ldmatrix from padded shared memory (64 x 64 x 32 tiles) for other shapes.
// The host pads 6 -> 64 inputs and 200 -> 256 outputs with zeros.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "tcgen05.cuh"

namespace mcl {
namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int PAD = 8;              // bf16 elements of row padding (bank spread)
constexpr int LDS = BK + PAD;       // shared-memory row stride (elements)

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
// dZ = dY * GELU'(Z) (or dY) in bf16, both as dZ[M][N] and dZt[N][M], and
// the bias gradient db[n] += sum_m dZ.  CTA: 32 rows x 64 columns, 256
// threads (64 columns x 4 row groups of 8 rows); the transposed copy goes
// through shared memory so that both stores are row-contiguous, and the
// column sums meet in shared memory (one atomic per column per CTA).
__global__ void __launch_bounds__(256) act_backward(int M, int N, const float* __restrict__ dY, int lddy,
                                                    const float* __restrict__ Z, int ldz, int gelu_on,
                                                    __nv_bfloat16* __restrict__ dZ, int lddz,
                                                    __nv_bfloat16* __restrict__ dZt, int lddzt,
                                                    float* __restrict__ db) {
  __shared__ __nv_bfloat16 tile[64][34];  // [column][row], padded
  __shared__ float part[4][64];
  const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;
  const int n0 = blockIdx.x * 64, n = n0 + tx;
  const int m0 = blockIdx.y * 32;
  float colsum = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = ty + 4 * i, m = m0 + r;
    __nv_bfloat16 b = __float2bfloat16_rn(0.0f);
    if (m < M && n < N) {
      float d = dY[(size_t)m * lddy + n];
      if (gelu_on) d *= gelu_grad(Z[(size_t)m * ldz + n]);
      b = __float2bfloat16_rn(d);
      dZ[(size_t)m * lddz + n] = b;
      colsum += d;
    }
    tile[tx][r] = b;
  }
  part[ty][tx] = colsum;
  __syncthreads();
  if (ty == 0 && n < N) atomicAdd(&db[n], (part[0][tx] + part[1][tx]) + (part[2][tx] + part[3][tx]));
  for (int e = threadIdx.x; e < 64 * 32; e += 256) {
    const int c = e >> 5, r = e & 31;  // consecutive threads: consecutive m of one dZt row
    if (n0 + c < N && m0 + r < M) dZt[(size_t)(n0 + c) * lddzt + m0 + r] = tile[c][r];
  }
}

// loss += sum over valid columns of (out - target)^2; dOut = 2 (out - target) * scale.
// One atomic per CTA.
__global__ void __launch_bounds__(256) mse_loss(int M, int N, int n_valid, const float* __restrict__ out, int ldo,
                                                const float* __restrict__ target, int ldt, float scale,
                                                float* __restrict__ dout, int ldd, float* __restrict__ loss) {
  __shared__ float warp_part[8];
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
  if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < 8; ++w) t += warp_part[w];
    atomicAdd(loss, t);
  }
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

// Adam over up to 16 tensors in one launch (blockIdx.y = tensor).
struct AdamMulti {
  mcl_adam_tensor t[16];
};

__global__ void __launch_bounds__(256) adam_multi(const AdamMulti A, float lr, float b1, float b2, float eps,
                                                  float bc1, float bc2, const float* lr_dev,
                                                  const int32_t* step_base, int32_t step_offset) {
  if (lr_dev) {  // learning rate and step read on the device (graph replays)
    lr = *lr_dev;
    const float step = (float)(*step_base + step_offset);
    bc1 = 1.0f - powf(b1, step);
    bc2 = 1.0f - powf(b2, step);
  }
  const mcl_adam_tensor& T = A.t[blockIdx.y];
  const int64_t n = (int64_t)T.rows * T.cols;
  __nv_bfloat16* W = reinterpret_cast<__nv_bfloat16*>(T.W);
  __nv_bfloat16* Wt = reinterpret_cast<__nv_bfloat16*>(T.Wt);
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
    const float gi = T.g[i];
    const float a = b1 * T.m1[i] + (1.0f - b1) * gi;
    const float b = b2 * T.m2[i] + (1.0f - b2) * gi * gi;
    T.m1[i] = a;
    T.m2[i] = b;
    const float mh = a / bc1, vh = b / bc2;
    const float pi = T.p[i] - lr * mh / (sqrtf(vh) + eps);
    T.p[i] = pi;
    const __nv_bfloat16 q = __float2bfloat16_rn(pi);
    if (W) W[i] = q;
    if (Wt) Wt[(size_t)(i % T.cols) * T.rows + i / T.cols] = q;
  }
}

__global__ void __launch_bounds__(256) f32_to_bf16(int64_t n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
  for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) y[i] = __float2bfloat16_rn(x[i]);
}

// ---------------------------------------------------------------------------
// tcgen05 path: the same NT GEMM on the 5th-generation tensor cores.
// One CTA of 4 warps computes a 128 x NT tile.  Per 64-wide K slab the CTA
// stages A (128 x 64) and B (NT x 64) in shared memory in the no-swizzle
// K-major "core matrix" layout (8 rows x 16 bytes per core matrix, core
// matrices adjacent along K 128 bytes apart, 8-row groups 1024 bytes apart),
// one thread issues four tcgen05.mma (M = 128, N = NT, K = 16, BF16 inputs,
// FP32 accumulator in tensor memory) and commits them to an mbarrier; the
// epilogue reads the accumulator back with tcgen05.ld (warp w owns TMEM lanes
// 32w..32w+31 = rows) and applies the same fused bias / GELU as gemm_nt.
// Every mbarrier wait is bounded; on a timeout the kernel records an error
// and still releases its tensor memory.
// ---------------------------------------------------------------------------
namespace tc {

using namespace ::mcl::tcg;

constexpr int kM = 128;   // rows per CTA (one tcgen05.mma M)
constexpr int kKS = 64;   // K elements staged per slab


// Start copying rows [m0, m0 + 128) of A and [n0, n0 + NT) of B (k-contiguous
// bf16) x K slab [k0, k0 + 64) into the core-matrix layout at shared
// addresses dA / dB (16-byte asynchronous copies; no registers held).
template <int NT>
__device__ __forceinline__ void issue_slab(uint32_t dA, uint32_t dB, const __nv_bfloat16* A, int lda,
                                           const __nv_bfloat16* B, int ldb, int m0, int n0, int k0) {
  constexpr int PA = kM * (kKS / 8) / 128, PB = NT * (kKS / 8) / 128;
#pragma unroll
  for (int i = 0; i < PA; ++i) {
    const int c = threadIdx.x + 128 * i, r = c / (kKS / 8), kc = c % (kKS / 8);
    cp_async16(dA + ((r >> 3) * (kKS / 8) + kc) * 128 + (r & 7) * 16, &A[(size_t)(m0 + r) * lda + k0 + kc * 8]);
  }
#pragma unroll
  for (int i = 0; i < PB; ++i) {
    const int c = threadIdx.x + 128 * i, r = c / (kKS / 8), kc = c % (kKS / 8);
    cp_async16(dB + ((r >> 3) * (kKS / 8) + kc) * 128 + (r & 7) * 16, &B[(size_t)(n0 + r) * ldb + k0 + kc * 8]);
  }
}

constexpr int kStageA = kM * kKS * 2;  // bytes of one staged A slab
constexpr int kStages = 3;             // slabs in flight: two loading while one multiplies

// Dynamic shared memory: kStages A and B slabs for the main loop, reused by
// the epilogue for the fp32 tile [128][NT+1] and the bf16 tile [128][NT+2].
template <int NT>
constexpr int smem_bytes() {
  return kStages * (kStageA + NT * kKS * 2) > 128 * (NT + 1) * 4 + 128 * (NT + 2) * 2
             ? kStages * (kStageA + NT * kKS * 2)
             : 128 * (NT + 1) * 4 + 128 * (NT + 2) * 2;
}

// Split-K: gridDim.z CTAs, launched as one thread-block cluster along z, each
// accumulate a K/gridDim.z range of the same tile; the partial tiles meet in
// distributed shared memory and every CTA sums 128/gridDim.z of the rows over
// the cluster in rank order (deterministic).  Only the plain fp32 epilogue
// uses it (the weight gradients, whose K is the batch).
// One CTA's tile (tile_m, tile_n) of C, K range split `split` of `splits`.
template <int EPI, int NT>
__device__ __forceinline__ void gemm_tile(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                          const __nv_bfloat16* __restrict__ B, int ldb,
                                          const float* __restrict__ bias, float* __restrict__ C, int ldc,
                                          __nv_bfloat16* __restrict__ Y, int ldy, __nv_bfloat16* __restrict__ Yt,
                                          int ldyt, int32_t* err, int tile_m, int tile_n, int split, int splits) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[kStages];
  __shared__ uint32_t tmem_slot;
  // slab buffer q: A at smem + q * kStageA, B at smem + kStages * kStageA + q * NT * kKS * 2
  const uint32_t sbase = smem_u32(smem);
  auto slabA = [&](int q) { return sbase + q * kStageA; };
  auto slabB = [&](int q) { return sbase + kStages * kStageA + q * NT * kKS * 2; };
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = tile_m * kM, n0 = tile_n * NT;
  const int kper = K / splits, kbeg = split * kper, nk = kper / kKS;
  const uint32_t mb0 = smem_u32(&mbar[0]);  // barrier q at mb0 + 8 q; MMA j commits to barrier j % 3
  if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), NT);
  if (tid == 0) {
    for (int q = 0; q < kStages; ++q) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb0 + 8 * q) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // prologue: slabs 0 and 1 in flight (one commit group per slab, empty if absent)
  issue_slab<NT>(slabA(0), slabB(0), A, lda, B, ldb, m0, n0, kbeg);
  cp_async_commit();
  if (nk > 1) issue_slab<NT>(slabA(1), slabB(1), A, lda, B, ldb, m0, n0, kbeg + kKS);
  cp_async_commit();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = idesc_bf16(kM, NT);
  bool ok = true;
  int last_commit = -1;  // the last slab whose MMAs were committed (uniform over the CTA)
  for (int it = 0; it < nk; ++it) {
    const int q = it % kStages;
    cp_async_wait_1();  // this thread's copies of slab it have landed
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    ok = __syncthreads_and(ok ? 1 : 0) != 0;  // everyone's copies visible; all agree on ok
    if (!ok) break;
    if (tid == 0) {
      fence_after();
#pragma unroll
      for (int kk = 0; kk < kKS / 16; ++kk) {
        const uint64_t ad = sdesc(slabA(q) + kk * 256, 128, 1024);
        const uint64_t bd = sdesc(slabB(q) + kk * 256, 128, 1024);
        mma(tmem, ad, bd, idesc, (it > 0 || kk > 0) ? 1u : 0u);
      }
      commit(mb0 + 8 * q);
    }
    last_commit = it;
    __syncwarp();
    if (it + 2 < nk) {
      // slab it + 2 reuses the buffer of slab it - 1: wait for that MMA first
      if (it >= 1) {
        const int j = it - 1;
        if (!mbar_wait(mb0 + 8 * (j % kStages), (uint32_t)(j / kStages) & 1u)) ok = false;
        fence_after();
      }
      if (ok) issue_slab<NT>(slabA((it + 2) % kStages), slabB((it + 2) % kStages), A, lda, B, ldb, m0, n0,
                             kbeg + (it + 2) * kKS);
    }
    cp_async_commit();
  }
  // Whatever happened above, no MMA may still write tensor memory when it is
  // read or freed: wait for the last commit issued, which covers every MMA
  // before it.  After an earlier timeout this is the second, again bounded,
  // wait; the kernel then frees its tensor memory either way.
  if (last_commit >= 0) {
    const int j = last_commit;
    if (!mbar_wait(mb0 + 8 * (j % kStages), (uint32_t)(j / kStages) & 1u)) ok = false;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  fence_after();
  if (!ok && tid == 0) atomicExch(err, 1);

  // Accumulator -> fp32 tile in shared memory (thread = row, as tcgen05.ld
  // delivers it), then stores in row order (coalesced).
  constexpr int FS = NT + 1, HS = NT + 2;
  float* ftile = reinterpret_cast<float*>(smem);
  const int row = 32 * warp + lane;
  if (ok) {
#pragma unroll 1
    for (int c0 = 0; c0 < NT; c0 += 16) {
      float v[16];
      ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) ftile[row * FS + c0 + j] = v[j];
    }
  }
  if (splits > 1) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    cluster.sync();  // every partial tile is in its CTA's shared memory
    const int rows = kM / splits, r0 = (int)cluster.block_rank() * rows;
    for (int e = tid; e < rows * NT; e += blockDim.x) {
      const int r = r0 + e / NT, c = e % NT;
      float acc = 0.0f;
      for (int q = 0; q < splits; ++q) acc += cluster.map_shared_rank(ftile, q)[r * FS + c];
      if (ok) C[(size_t)(m0 + r) * ldc + n0 + c] = acc;
    }
    cluster.sync();  // no CTA leaves while another reads its tile
  } else {
    __syncthreads();
    __nv_bfloat16* htile = reinterpret_cast<__nv_bfloat16*>(smem + 128 * FS * 4);
    for (int e = tid; e < kM * NT; e += blockDim.x) {
      const int r = e / NT, c = e % NT;
      float x = ftile[r * FS + c];
      if (EPI != EPI_F32) x += bias[n0 + c];
      if (ok) C[(size_t)(m0 + r) * ldc + n0 + c] = x;
      if (EPI == EPI_BIAS_GELU) {
        const __nv_bfloat16 y = __float2bfloat16_rn(gelu(x));
        if (ok) Y[(size_t)(m0 + r) * ldy + n0 + c] = y;
        htile[r * HS + c] = y;
      }
    }
    if (EPI == EPI_BIAS_GELU && Yt) {
      __syncthreads();
      for (int e = tid; e < kM * NT; e += blockDim.x) {
        const int c = e / kM, r = e % kM;  // consecutive threads: consecutive m of Yt[n][m]
        if (ok) Yt[(size_t)(n0 + c) * ldyt + m0 + r] = htile[r * HS + c];
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, NT);
  (void)M;
  (void)N;
}

template <int EPI, int NT>
__global__ void __launch_bounds__(128) gemm_nt_tc(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                                  const __nv_bfloat16* __restrict__ B, int ldb,
                                                  const float* __restrict__ bias, float* __restrict__ C, int ldc,
                                                  __nv_bfloat16* __restrict__ Y, int ldy,
                                                  __nv_bfloat16* __restrict__ Yt, int ldyt, int32_t* err) {
  gemm_tile<EPI, NT>(M, N, K, A, lda, B, ldb, bias, C, ldc, Y, ldy, Yt, ldyt, err, blockIdx.y, blockIdx.x, blockIdx.z,
                     gridDim.z);
}

// Several independent plain (fp32 output) GEMMs in one launch: blockIdx.z =
// gemm * splits + split, the split-K cluster running along z inside one
// GEMM.  CTAs whose tile lies outside their GEMM leave at once; a cluster
// shares its (x, y), so its CTAs leave together.
struct Grouped {
  mcl_gemm_desc g[8];
};

__global__ void __launch_bounds__(128) gemm_nt_tc_grouped(const __grid_constant__ Grouped G, int splits,
                                                          int32_t* err) {
  const mcl_gemm_desc& d = G.g[blockIdx.z / splits];
  if ((int)blockIdx.x * 64 >= d.N || (int)blockIdx.y * kM >= d.M) return;
  gemm_tile<EPI_F32, 64>(d.M, d.N, d.K, reinterpret_cast<const __nv_bfloat16*>(d.A), d.lda,
                         reinterpret_cast<const __nv_bfloat16*>(d.B), d.ldb, nullptr, d.C, d.ldc, nullptr, 0, nullptr,
                         0, err, blockIdx.y, blockIdx.x, blockIdx.z % splits, splits);
}

}  // namespace tc

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
  dim3 grid((N + 63) / 64, (M + 31) / 32);
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
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 608);
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

extern "C" int mcl_adam_multi(const mcl_adam_tensor* tensors, int32_t n, float lr, float b1, float b2, float eps,
                              int32_t step, void* stream) {
  if (!tensors || n < 1 || n > 16 || step < 1) return MCL_EINVAL;
  AdamMulti A;
  int64_t most = 0;
  for (int i = 0; i < n; ++i) {
    const mcl_adam_tensor& t = tensors[i];
    if (t.rows <= 0 || t.cols <= 0 || !t.p || !t.g || !t.m1 || !t.m2) return MCL_EINVAL;
    A.t[i] = t;
    most = std::max<int64_t>(most, (int64_t)t.rows * t.cols);
  }
  const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
  dim3 grid((unsigned)std::min<int64_t>((most + 255) / 256, 256), (unsigned)n);
  adam_multi<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A, lr, b1, b2, eps, bc1, bc2, nullptr,
                                                                        nullptr, 0);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}

extern "C" int mcl_adam_multi_dev(const mcl_adam_tensor* tensors, int32_t n, const float* lr,
                                  const int32_t* step_base, int32_t step_offset, float b1, float b2, float eps,
                                  void* stream) {
  if (!tensors || n < 1 || n > 16 || !lr || !step_base) return MCL_EINVAL;
  AdamMulti A;
  int64_t most = 0;
  for (int i = 0; i < n; ++i) {
    const mcl_adam_tensor& t = tensors[i];
    if (t.rows <= 0 || t.cols <= 0 || !t.p || !t.g || !t.m1 || !t.m2) return MCL_EINVAL;
    A.t[i] = t;
    most = std::max<int64_t>(most, (int64_t)t.rows * t.cols);
  }
  dim3 grid((unsigned)std::min<int64_t>((most + 255) / 256, 256), (unsigned)n);
  adam_multi<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A, 0.0f, b1, b2, eps, 1.0f, 1.0f, lr,
                                                                        step_base, step_offset);
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

namespace mcl {
namespace {
template <int EPI>
int launch_tc(dim3 grid, int splits, int M, int N, int K, const __nv_bfloat16* a, int lda, const __nv_bfloat16* b,
              int ldb, const float* bias, float* C, int ldc, __nv_bfloat16* y, int ldy, __nv_bfloat16* yt,
              int ldyt, int32_t* err, cudaStream_t s) {
  constexpr int NT = 64;
  auto kern = tc::gemm_nt_tc<EPI, NT>;
  constexpr int smem = tc::smem_bytes<NT>();
  MCL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  if (splits == 1) {
    kern<<<grid, 128, smem, s>>>(M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt, err);
    MCL_CUDA_TRY(cudaGetLastError());
    return MCL_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid.x, grid.y, (unsigned)splits);
  cfg.blockDim = dim3(128, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 1;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = (unsigned)splits;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  MCL_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt, err));
  return MCL_OK;
}
}  // namespace
}  // namespace mcl

extern "C" int mcl_gemm_nt_tc_grouped(const mcl_gemm_desc* gemms, int32_t n, int32_t splits, int32_t* err,
                                      void* stream) {
  if (!gemms || n < 1 || n > 8 || !err || (splits != 1 && splits != 2 && splits != 4 && splits != 8))
    return MCL_EINVAL;
  tc::Grouped G;
  int gx = 0, gy = 0;
  for (int i = 0; i < n; ++i) {
    const mcl_gemm_desc& d = gemms[i];
    if (d.M <= 0 || d.N <= 0 || d.K <= 0 || d.M % tc::kM || d.N % 64 || d.K % (tc::kKS * splits)) return MCL_EINVAL;
    if (splits > 1 && d.K / splits < 2 * tc::kKS) return MCL_EINVAL;
    if (!d.A || !d.B || !d.C || d.lda < d.K || d.ldb < d.K || d.ldc < d.N || (d.lda % 8) || (d.ldb % 8))
      return MCL_EINVAL;
    if (((uintptr_t)d.A | (uintptr_t)d.B) & 15) return MCL_EINVAL;
    G.g[i] = d;
    gx = std::max(gx, d.N / 64);
    gy = std::max(gy, d.M / tc::kM);
  }
  constexpr int smem = tc::smem_bytes<64>();
  MCL_CUDA_TRY(cudaFuncSetAttribute(tc::gemm_nt_tc_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)gx, (unsigned)gy, (unsigned)(n * splits));
  cfg.blockDim = dim3(128, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = reinterpret_cast<cudaStream_t>(stream);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 1;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = (unsigned)splits;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  MCL_CUDA_TRY(cudaLaunchKernelEx(&cfg, tc::gemm_nt_tc_grouped, G, (int)splits, err));
  return MCL_OK;
}

extern "C" int mcl_gemm_nt_tc(int32_t epilogue, int32_t M, int32_t N, int32_t K, const void* A, int32_t lda,
                              const void* B, int32_t ldb, const float* bias, float* C, int32_t ldc, void* Y,
                              int32_t ldy, void* Yt, int32_t ldyt, int32_t* err, void* stream) {
  constexpr int NT = 64;
  if (M <= 0 || N <= 0 || K <= 0 || M % tc::kM || N % NT || K % tc::kKS) return MCL_EINVAL;
  if (!A || !B || !C || !err || lda < K || ldb < K || ldc < N || (lda % 8) || (ldb % 8)) return MCL_EINVAL;
  if (((uintptr_t)A | (uintptr_t)B) & 15) return MCL_EINVAL;
  if (epilogue != EPI_F32 && !bias) return MCL_EINVAL;
  if (epilogue == EPI_BIAS_GELU && (!Y || ldy < N || (Yt && ldyt < M))) return MCL_EINVAL;
  dim3 grid(N / NT, M / tc::kM);
  // Few output tiles and a long K (weight gradients, K = batch): split K over
  // a cluster of up to 8 CTAs, at least two 64-wide slabs each.
  int splits = 1;
  const int slabs = K / tc::kKS;
  if (epilogue == EPI_F32 && (int)(grid.x * grid.y) < 64) {
    for (int sp = 8; sp >= 2; sp >>= 1)
      if (slabs % sp == 0 && slabs / sp >= 2) {
        splits = sp;
        break;
      }
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const auto* a = reinterpret_cast<const __nv_bfloat16*>(A);
  const auto* b = reinterpret_cast<const __nv_bfloat16*>(B);
  auto* y = reinterpret_cast<__nv_bfloat16*>(Y);
  auto* yt = reinterpret_cast<__nv_bfloat16*>(Yt);
  switch (epilogue) {
    case EPI_F32: return launch_tc<EPI_F32>(grid, splits, M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt, err, s);
    case EPI_BIAS: return launch_tc<EPI_BIAS>(grid, 1, M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt, err, s);
    case EPI_BIAS_GELU: return launch_tc<EPI_BIAS_GELU>(grid, 1, M, N, K, a, lda, b, ldb, bias, C, ldc, y, ldy, yt, ldyt, err, s);
  }
  return MCL_EINVAL;
}
