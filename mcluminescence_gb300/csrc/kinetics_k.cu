// Event-driven (reference) trap kinetics: the loop of src/class/simulate.py:51-92
// over TLTrapSim / Box / Physics (src/class/tl_trap_lab.py:27-60,
// src/class/engine.py:65-188), one CTA per simulation, FP64.
//
// Per step, exactly as the reference:
//   T = T_start + T_rate t + 273.15                        (simulate.py:53-54)
//   per electron: E_loc = U < Retrap ? E_loc_2 : E_loc_1    (engine.py:72)
//                 wait = 1/(s e^{-E_cb/kT} + b e^{-E_loc/kT - alpha d}) * -log(1-U)
//                                                         (engine.py:65-77, tl_trap_lab.py:48-51)
//   fill wait: lambda = (D/D0)(N-n), or 1e-20 when n == N or D == 0;
//              one uniform whenever lambda > 0           (tl_trap_lab.py:53-60)
//   dt = min(dt_fill, min wait (if any wait != 0, else dt_fill), dt_cap)
//   one event: pair creation, recombination of the first electron with the
//   minimal wait and its nearest hole, or nothing        (simulate.py:56-84)
// with the reference's bookkeeping quirks (engine.py:133-175): a created
// electron searches the OLD holes only, existing electrons are not re-pointed
// to the new hole, and after a removal the hole indices above the removed one
// shift down BEFORE the electrons pointing at the removed index are rescanned
// (so the former h+1 owners are rescanned too).  Arrays are shifted like
// np.delete, so every index the kernel reports is the reference's index.
//
// Uniforms are consumed in the reference's order (engine.py:125,128; then per
// step engine.py:72, tl_trap_lab.py:51, :60, and engine.py:135-136 on a pair
// creation) from one of three sources:
//   MT19937   numpy's legacy RandomState stream, generated in shared memory
//             (the key array and position come from / go back to the host,
//             so np.random.seed(k); simulate(cfg) is reproduced draw by draw);
//   injected  a caller-provided array of doubles;
//   Philox    an independent counter-based stream per simulation.
// Distances follow np.linalg.norm's order sqrt((dx*dx + dy*dy) + dz*dz) with no
// contraction; nearest searches compare squared distances and take the square
// root only when it can decide (first index wins ties, like np.argmin).
// GB300 runs FP64 at ~1/64 of the FP32 rate, so the FP64 arithmetic is kept to
// what decides a result: nearest searches scan FP32 coordinates first and
// evaluate FP64 norms only for candidates within a proven margin, the wait
// filter scores electrons in FP32 and evaluates FP64 waits only near the
// minimum, generated uniforms stay 53-bit integers until a double is needed,
// reductions compare integer keys, and per-step scalars are computed once per
// CTA.  Every result stays the reference's FP64 result.
#include <climits>
#include <cmath>

#include "common.cuh"

namespace mcl {
namespace {

constexpr int kRing = 4096;          // MT19937 output ring (words), power of two
constexpr int kChunk = 1024;         // doubles consumed per chunk
constexpr uint32_t kTagK = 4;        // Philox tag of the event-driven draws
constexpr int kMtN = 624;
constexpr int kMtM = 397;

static_assert(2 * kChunk + 2 * kMtN <= kRing, "ring too small for a chunk");

__device__ __forceinline__ double dsq3(double ax, double ay, double az, double bx, double by, double bz) {
  const double dx = __dadd_rn(ax, -bx);
  const double dy = __dadd_rn(ay, -by);
  const double dz = __dadd_rn(az, -bz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// (v2, i2) beats (v1, i1) under np.argmin: NaN first, then smaller, then lower index.
__device__ __forceinline__ bool better(double v2, int i2, double v1, int i1) {
  const bool n1 = isnan(v1), n2 = isnan(v2);
  if (n2 != n1) return n2;
  if (n1) return i2 < i1;
  return v2 < v1 || (v2 == v1 && i2 < i1);
}

// Integer sort key of a double that is >= +0, +inf or NaN (distances, waits):
// IEEE bit patterns of non-negative doubles order like their values, and NaN
// maps below everything (np.argmin returns the first NaN).  Comparing keys
// keeps the block reductions off the (slow) FP64 pipe.
__device__ __forceinline__ long long argmin_key(double v) {
  const long long b = __double_as_longlong(v);
  return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll ? LLONG_MIN : b;
}

// Per-simulation state.  The "local" arrays live in shared memory when they
// fit (global memory otherwise); the FP64 hole coordinates always live in the
// simulation's global-memory region: the nearest-centre scans read FP32
// copies scaled by the largest box side from the local arrays and touch the
// FP64 values only for the few candidates the FP32 pass cannot exclude.
struct Arrays {
  double *ex, *ey, *ez, *ed;  // electron coordinates, nearest distance
  double* u2;                 // the step's wait uniform of each electron
  float* edf;                 // nearest distance rounded to FP32 (kept in step with ed)
  float* lw;                  // FP32 log-wait of the current step
  int32_t* en;                // nearest hole index
  uint8_t* choice;            // E_loc choice of the current step
  int32_t* mlist;             // electrons to rescan after a removal
  float *exf, *eyf, *ezf;     // electron coordinates / largest box side, FP32
  float *hxf, *hyf, *hzf;     // hole coordinates / largest box side, FP32
  double *hx, *hy, *hz;       // hole coordinates (global memory)
  double inv_l;               // 1 / largest box side
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t local_bytes(int e_cap, int h_cap) {
  return align16(sizeof(double) * 5 * (size_t)e_cap) + align16(sizeof(float) * 2 * (size_t)e_cap) +
         align16(sizeof(int32_t) * (size_t)e_cap) + align16((size_t)e_cap) +
         align16(sizeof(int32_t) * (size_t)e_cap) + align16(sizeof(float) * 3 * (size_t)e_cap) +
         align16(sizeof(float) * 3 * (size_t)h_cap);
}

__host__ __device__ inline size_t hole64_bytes(int h_cap) { return align16(sizeof(double) * 3 * (size_t)h_cap); }

// Bytes of one simulation's global-memory region (at its ws_offset).
__host__ __device__ inline size_t region_bytes(int e_cap, int h_cap, bool local_in_smem) {
  return hole64_bytes(h_cap) + (local_in_smem ? 0 : local_bytes(e_cap, h_cap));
}

__device__ inline Arrays carve(unsigned char* local, int e_cap, int h_cap, unsigned char* region, int h_cap_sim) {
  Arrays A;
  double* d = reinterpret_cast<double*>(local);
  A.ex = d;
  A.ey = d + e_cap;
  A.ez = d + 2 * e_cap;
  A.ed = d + 3 * e_cap;
  A.u2 = d + 4 * e_cap;
  unsigned char* p = local + align16(sizeof(double) * 5 * (size_t)e_cap);
  A.edf = reinterpret_cast<float*>(p);
  A.lw = A.edf + e_cap;
  p += align16(sizeof(float) * 2 * (size_t)e_cap);
  A.en = reinterpret_cast<int32_t*>(p);
  p += align16(sizeof(int32_t) * (size_t)e_cap);
  A.choice = p;
  p += align16((size_t)e_cap);
  A.mlist = reinterpret_cast<int32_t*>(p);
  p += align16(sizeof(int32_t) * (size_t)e_cap);
  float* g = reinterpret_cast<float*>(p);
  A.exf = g;
  A.eyf = g + e_cap;
  A.ezf = g + 2 * e_cap;
  p += align16(sizeof(float) * 3 * (size_t)e_cap);
  float* f = reinterpret_cast<float*>(p);
  A.hxf = f;
  A.hyf = f + h_cap;
  A.hzf = f + 2 * h_cap;
  double* h = reinterpret_cast<double*>(region);
  A.hx = h;
  A.hy = h + h_cap_sim;
  A.hz = h + 2 * h_cap_sim;
  A.inv_l = 1.0;
  return A;
}

// Shared scalars of the CTA.
struct Shared {
  double rv[32];
  int ri[32];
  int ra[32];
  double best_v;
  int best_i;
  int any;
  int n_mask;
  // per-step scalars, computed once (thread 0) instead of by every warp:
  // GB300's FP64 pipe is narrow, so redundant FP64 work costs real time
  double kT, rcb, dt_fill, d1, d2;  // d1, d2: -E_loc_1 / kT, -E_loc_2 / kT
  float c1, c2, lrcb;
  // the electrons whose FP32 log-wait is within the margin of the minimum,
  // and their exponential draws -log(1 - u)
  int n_cand;
  int cand[32];
  double cand_e[32];
  // block minima of floats, one slot per call in rotation (see block_minf)
  int mkey[3];
  int mflags[3];
};

// Order-preserving map of a float to an int (and back): negative floats have
// their magnitude bits flipped.
__device__ __forceinline__ int fkey(float v) {
  const int b = __float_as_int(v);
  return b ^ ((b >> 31) & 0x7fffffff);
}
__device__ __forceinline__ float fkey_inv(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); }

// Block-wide argmin with np.argmin semantics over values >= +0, +inf or NaN
// (compared through argmin_key); also ORs `any`.
template <int BLOCK>
__device__ void block_argmin(Shared& sh, double v, int i, int any, double& out_v, int& out_i, int& out_any) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long k = argmin_key(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long k2 = __shfl_down_sync(0xffffffffu, k, o);
    const double v2 = __shfl_down_sync(0xffffffffu, v, o);
    const int i2 = __shfl_down_sync(0xffffffffu, i, o);
    const int a2 = __shfl_down_sync(0xffffffffu, any, o);
    if (k2 < k || (k2 == k && i2 < i)) {
      k = k2;
      v = v2;
      i = i2;
    }
    any |= a2;
  }
  if (lane == 0) {
    sh.rv[warp] = v;
    sh.ri[warp] = i;
    sh.ra[warp] = any;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int W = BLOCK / 32;
    v = lane < W ? sh.rv[lane] : INFINITY;
    i = lane < W ? sh.ri[lane] : INT_MAX;
    any = lane < W ? sh.ra[lane] : 0;
    k = argmin_key(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long k2 = __shfl_down_sync(0xffffffffu, k, o);
      const double v2 = __shfl_down_sync(0xffffffffu, v, o);
      const int i2 = __shfl_down_sync(0xffffffffu, i, o);
      const int a2 = __shfl_down_sync(0xffffffffu, any, o);
      if (k2 < k || (k2 == k && i2 < i)) {
        k = k2;
        v = v2;
        i = i2;
      }
      any |= a2;
    }
    if (lane == 0) {
      sh.best_v = v;
      sh.best_i = i;
      sh.any = any;
    }
  }
  __syncthreads();
  out_v = sh.best_v;
  out_i = sh.best_i;
  out_any = sh.any;
  __syncthreads();
}

// Block-wide minimum of a float (NaN ignored, +inf if all are) and OR of flags,
// with one CTA barrier: each warp's lane 0 folds its warp's result into slot
// `rot` with atomics.  Call k uses slot k % 3 and, before its barrier, thread
// 0 clears slot (k + 1) % 3, whose last readers (call k - 2) all passed call
// k - 1's barrier; `rot` (the same in every thread) advances per call.
template <int BLOCK>
__device__ void block_minf(Shared& sh, int& rot, float v, int flags, float& out_v, int& out_flags) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    flags |= __shfl_xor_sync(0xffffffffu, flags, o);
  }
  const int r = rot;
  rot = r == 2 ? 0 : r + 1;
  if (threadIdx.x == 0) {
    sh.mkey[rot] = INT_MAX;
    sh.mflags[rot] = 0;
  }
  if (lane == 0) {
    atomicMin(&sh.mkey[r], fkey(v));
    atomicOr(&sh.mflags[r], flags);
  }
  __syncthreads();
  out_v = fkey_inv(sh.mkey[r]);
  out_flags = sh.mflags[r];
}

__device__ __forceinline__ float dsq3f(float ax, float ay, float az, float bx, float by, float bz) {
  const float dx = ax - bx, dy = ay - by, dz = az - bz;
  return (dx * dx + dy * dy) + dz * dz;
}

// FP32 prefilter of the nearest-centre searches.  Coordinates scaled by the
// largest box side lie in [0, 1]; each FP32 coordinate is within 2^-24 of its
// scaled FP64 value, so a scaled FP32 squared distance is within 24 * 2^-24
// of the exact one.  A hole whose FP64 norm could be the minimum therefore
// has an FP32 squared distance at most 48 * 2^-24 above the FP32 minimum; the
// margin kSqMargin = 128 * 2^-24 keeps every such hole, and the exact FP64
// comparison (the reference's order of operations, first index on ties)
// decides among the candidates.
constexpr float kSqMargin = 0x1p-17f;

__device__ __forceinline__ float scaled(double x, double inv_l) { return __double2float_rn(__dmul_rn(x, inv_l)); }

// Nearest hole of point p over holes [0, n_h): exact np.argmin of the norms.
// Pass 1: block minimum of the FP32 squared distances.  Pass 2: per thread a
// running best over its strided candidates in FP64 (sqrt only when the
// squared distance does not exceed the best so far), then the block argmin.
template <int BLOCK>
__device__ void nearest_block(Shared& sh, int& rot, const Arrays& A, int n_h, double px, double py, double pz, float qx,
                              float qy, float qz, double& d_out, int& i_out) {
  float m = INFINITY;
  for (int h = threadIdx.x; h < n_h; h += BLOCK) m = fminf(m, dsq3f(qx, qy, qz, A.hxf[h], A.hyf[h], A.hzf[h]));
  float mv;
  int dummy_a;
  block_minf<BLOCK>(sh, rot, m, 0, mv, dummy_a);
  const float thr = mv + kSqMargin;
  double bsq = INFINITY, bd = INFINITY;
  int bi = INT_MAX;
  for (int h = threadIdx.x; h < n_h; h += BLOCK) {
    if (!(dsq3f(qx, qy, qz, A.hxf[h], A.hyf[h], A.hzf[h]) <= thr)) continue;
    const double sq = dsq3(px, py, pz, A.hx[h], A.hy[h], A.hz[h]);
    if (sq <= bsq) {
      const double d = __dsqrt_rn(sq);
      if (d < bd) {
        bd = d;
        bsq = sq;
        bi = h;
      }
    }
  }
  block_argmin<BLOCK>(sh, bd, bi, 0, d_out, i_out, dummy_a);
}

// ---------------------------------------------------------------------------
// Uniform sources
// ---------------------------------------------------------------------------
struct Source {
  int rng;
  // injected
  const double* u;
  int64_t u_base, u_count;
  // Philox
  uint32_t k0, k1, stream;
  // MT19937 (shared memory)
  uint32_t* mt;    // 624 key words (current state)
  uint32_t* mt2;   // the other state buffer
  uint32_t* ring;  // kRing tempered words
  uint32_t rd, wr;  // ring positions (identical in every thread)
  int64_t pos;     // doubles consumed in this simulation
};

__device__ __forceinline__ uint32_t mt_mix(uint32_t xi, uint32_t xi1, uint32_t xm) {
  const uint32_t y = (xi & 0x80000000u) | (xi1 & 0x7fffffffu);
  return xm ^ (y >> 1) ^ ((xi1 & 1u) ? 0x9908b0dfu : 0u);
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// One MT19937 state transition (Matsumoto & Nishimura 1998) by the whole CTA,
// from `cur` into `nxt` (two buffers, so no read/write hazards inside a
// phase), each new word tempered straight into the output ring at wr + i:
// indices [0,227) read only old words, [227,454) and [454,623) read words
// updated 227 places earlier, 623 reads the new words 0 and 396.  Three
// block barriers per 624 words.
template <int BLOCK>
__device__ void mt_twist(const uint32_t* cur, uint32_t* nxt, uint32_t* ring, uint32_t wr) {
  constexpr int D = kMtN - kMtM;  // 227
  for (int i = threadIdx.x; i < D; i += BLOCK) {
    const uint32_t v = mt_mix(cur[i], cur[i + 1], cur[i + kMtM]);
    nxt[i] = v;
    ring[(wr + i) & (kRing - 1)] = mt_temper(v);
  }
  __syncthreads();
  for (int i = D + threadIdx.x; i < 2 * D; i += BLOCK) {
    const uint32_t v = mt_mix(cur[i], cur[i + 1], nxt[i - D]);
    nxt[i] = v;
    ring[(wr + i) & (kRing - 1)] = mt_temper(v);
  }
  __syncthreads();
  for (int i = 2 * D + threadIdx.x; i < kMtN; i += BLOCK) {
    const uint32_t v = mt_mix(cur[i], i == kMtN - 1 ? nxt[0] : cur[i + 1], nxt[i - D]);
    nxt[i] = v;
    ring[(wr + i) & (kRing - 1)] = mt_temper(v);
  }
  __syncthreads();
}

// Make `n` doubles available (n <= kChunk).  Returns false when an injected
// stream would run out.
template <int BLOCK>
__device__ bool ensure(Source& S, int n) {
  if (S.rng == MCL_RNG_INJECTED) return S.pos + n <= S.u_count;
  if (S.rng != MCL_RNG_MT19937) return true;
  while ((int)(S.wr - S.rd) < 2 * n) {
    mt_twist<BLOCK>(S.mt, S.mt2, S.ring, S.wr);
    uint32_t* t = S.mt;
    S.mt = S.mt2;
    S.mt2 = t;
    S.wr += kMtN;
  }
  return true;
}

__device__ __forceinline__ double value(const Source& S, int k) {
  if (S.rng == MCL_RNG_MT19937) {
    const uint32_t a = S.ring[(S.rd + 2u * k) & (kRing - 1)];
    const uint32_t b = S.ring[(S.rd + 2u * k + 1u) & (kRing - 1)];
    return u53(a, b);
  }
  if (S.rng == MCL_RNG_INJECTED) return S.u[S.u_base + S.pos + k];
  const uint64_t d = (uint64_t)(S.pos + k);
  const uint4 r = philox4x32_10((uint32_t)(d >> 1), S.stream, (uint32_t)(d >> 33), kTagK, S.k0, S.k1);
  return (d & 1) ? u53(r.z, r.w) : u53(r.x, r.y);
}

// The 53-bit integer m of uniform k (value = m * 2^-53 exactly) for the
// generated streams; the injected stream has doubles only.
__device__ __forceinline__ uint64_t bits53(const Source& S, int k) {
  uint32_t a, b;
  if (S.rng == MCL_RNG_MT19937) {
    a = S.ring[(S.rd + 2u * k) & (kRing - 1)];
    b = S.ring[(S.rd + 2u * k + 1u) & (kRing - 1)];
  } else {
    const uint64_t d = (uint64_t)(S.pos + k);
    const uint4 r = philox4x32_10((uint32_t)(d >> 1), S.stream, (uint32_t)(d >> 33), kTagK, S.k0, S.k1);
    a = (d & 1) ? r.z : r.x;
    b = (d & 1) ? r.w : r.y;
  }
  return ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
}

__device__ __forceinline__ void advance(Source& S, int n) {
  S.pos += n;
  if (S.rng == MCL_RNG_MT19937) S.rd += 2u * n;
}

// ---------------------------------------------------------------------------
// One simulation by the whole CTA
// ---------------------------------------------------------------------------
template <int BLOCK>
__device__ int run_sim(const mcl_k_args& a, int si, const mcl_k_sim& sm, const Arrays& A, Shared& sh, int& rot,
                       Source& S) {
  const int tid = threadIdx.x;
  int status = MCL_OK;
  int n_e = sm.e0, n_h = sm.n_h0;
  int n_ev = 0;
  S.pos = 0;

  // ---- seeding (engine.py:124-129): electrons, then holes -----------------
  if (n_e > sm.e_cap || n_h > sm.h_cap) status = MCL_ECAPACITY;
  for (int pass = 0; pass < 2 && status == MCL_OK; ++pass) {
    const int cnt_all = 3 * (pass == 0 ? n_e : n_h);
    double* X = pass == 0 ? A.ex : A.hx;
    double* Y = pass == 0 ? A.ey : A.hy;
    double* Z = pass == 0 ? A.ez : A.hz;
    const double sx = pass == 0 ? sm.L : sm.Lb, sy = pass == 0 ? sm.W : sm.Wb, sz = pass == 0 ? sm.H : sm.Hb;
    for (int c0 = 0; c0 < cnt_all; c0 += kChunk) {
      const int cnt = min(kChunk, cnt_all - c0);
      if (!ensure<BLOCK>(S, cnt)) {
        status = MCL_EBUDGET;
        break;
      }
      for (int k = tid; k < cnt; k += BLOCK) {
        const int idx = c0 + k, p = idx / 3, c = idx - 3 * p;
        const double u = value(S, k);
        const double v = __dmul_rn(u, c == 0 ? sx : (c == 1 ? sy : sz));
        if (c == 0) X[p] = v;
        else if (c == 1) Y[p] = v;
        else Z[p] = v;
        if (pass == 1) (c == 0 ? A.hxf : (c == 1 ? A.hyf : A.hzf))[p] = scaled(v, A.inv_l);
        else (c == 0 ? A.exf : (c == 1 ? A.eyf : A.ezf))[p] = scaled(v, A.inv_l);
      }
      advance(S, cnt);
      __syncthreads();
    }
  }

  // ---- full nearest search (engine.py:113-119) ----------------------------
  if (status == MCL_OK) {
    if (n_e > 0 && n_h == 0) status = MCL_ENOHOLE;
    for (int e = tid; e < n_e && status == MCL_OK; e += BLOCK) {
      const double px = A.ex[e], py = A.ey[e], pz = A.ez[e];
      const float qx = A.exf[e], qy = A.eyf[e], qz = A.ezf[e];
      float m = INFINITY;
      for (int h = 0; h < n_h; ++h) m = fminf(m, dsq3f(qx, qy, qz, A.hxf[h], A.hyf[h], A.hzf[h]));
      const float thr = m + kSqMargin;
      double bsq = INFINITY, bd = INFINITY;
      int bi = INT_MAX;
      for (int h = 0; h < n_h; ++h) {
        if (!(dsq3f(qx, qy, qz, A.hxf[h], A.hyf[h], A.hzf[h]) <= thr)) continue;
        const double sq = dsq3(px, py, pz, A.hx[h], A.hy[h], A.hz[h]);
        if (sq <= bsq) {
          const double d = __dsqrt_rn(sq);
          if (d < bd) {
            bd = d;
            bsq = sq;
            bi = h;
          }
        }
      }
      A.ed[e] = bd;
      A.edf[e] = __double2float_rn(bd);
      A.en[e] = bi;
    }
    __syncthreads();
  }

  // ---- block-collective pieces shared by the loops -------------------------
  const int64_t N = (int64_t)sm.N_e;
  int n_ev_local = 0;
  // Retrap choices and waits at temperature T (tl_trap_lab.py:48-51 with
  // engine.py:65-77): 2n uniforms.  Pass 1 scores every electron with an FP32
  // log-wait log(-log(1-U)) - log(s e^{-E_cb/kT} + b e^{arg}) (absolute error
  // < 5e-5, so a margin of 1e-3 in log space cannot exclude the FP64 minimum);
  // pass 2 evaluates the reference's FP64 wait exactly for the electrons within
  // the margin of the FP32 minimum and takes np.argmin over them.  A
  // non-finite FP32 score or a rate near FP64 over/underflow sends the whole
  // step through the exact FP64 path.  wait != 0 (np.any) holds exactly when
  // some log-wait is above -inf, as -inf means U == 0.
  const float af = __double2float_rn(sm.alpha);
  const float lb = __double2float_rn(log(sm.b));
  const double ls = log(sm.s);
  auto waits = [&](double T, double& wmin, int& emin, int& any) -> int {
    // the step's FP64 scalars, on two warps at once: the conduction-band rate
    // (and its FP32 log for the scores: log s + x equals log(s e^x) to far
    // below the scores' error, except for a subnormal rate, which takes the
    // FP64 log) and the two trap-depth terms
    if (tid == 0) {
      sh.n_cand = 0;
      const double kT0 = __dmul_rn(sm.k_b, T);
      const double x = __ddiv_rn(-sm.E_cb, kT0);
      const double rcb0 = __dmul_rn(sm.s, exp(x));
      sh.kT = kT0;
      sh.rcb = rcb0;
      sh.lrcb = rcb0 >= 0x1p-1022 ? __double2float_rn(ls + x) : rcb0 > 0.0 ? __double2float_rn(log(rcb0))
                                                                          : -INFINITY;
    } else if (tid == 32) {
      const double kT0 = __dmul_rn(sm.k_b, T);
      const double d1 = __ddiv_rn(-sm.E_loc_1, kT0), d2 = __ddiv_rn(-sm.E_loc_2, kT0);
      sh.d1 = d1;
      sh.d2 = d2;
      sh.c1 = __double2float_rn(d1);
      sh.c2 = __double2float_rn(d2);
    }
    __syncthreads();
    const double rcb = sh.rcb, d1 = sh.d1, d2 = sh.d2;
    // Generated streams stay in integers: u < Retrap  <=>  m < ceil(Retrap 2^53)
    // (exact: u = m 2^-53), and the wait uniform is kept as m until the exact
    // pass needs it as a double.
    const bool gen = S.rng != MCL_RNG_INJECTED;
    const uint64_t r53 = sm.Retrap >= 1.0 ? (1ull << 53)
                         : sm.Retrap > 0.0 ? (uint64_t)ceil(__dmul_rn(sm.Retrap, 9007199254740992.0)) : 0ull;
    uint64_t* u2bits = reinterpret_cast<uint64_t*>(A.u2);
    const float c1 = sh.c1, c2 = sh.c2, lrcb = sh.lrcb;
    float lmin = INFINITY;
    int flags = 0;  // bit 0: exact path needed; bit 1: some wait is non-zero
    // the FP32 score of electron e given its choice and wait uniform
    auto score = [&](int e, int choice, float uf) {
      const float arg = (choice ? c2 : c1) - af * A.edf[e];
      const float lrt = lb + arg;
      const float lrate = lrcb > -INFINITY ? fmaxf(lrcb, lrt) + log1pf(expf(-fabsf(lrcb - lrt))) : lrt;
      const float E = -log1pf(-uf);
      const float lw = logf(E) - lrate;
      A.lw[e] = lw;
      // FP64 over/underflow of the rate (life 0 or inf) is left to the exact path
      if (isnan(lw) || lw == INFINITY || lrate > 700.0f || lrt < -700.0f || rcb == INFINITY) flags |= 1;
      if (lw > -INFINITY) flags |= 2;
      lmin = fminf(lmin, lw);
    };
    if (S.rng == MCL_RNG_PHILOX) {
      // uniforms addressed by position: electron e's choice and wait are
      // uniforms 2e and 2e + 1 of this step, the two halves of one Philox
      // block (the step starts on a block boundary); one pass, no barrier
      if (S.pos & 1) advance(S, 1);
      for (int e = tid; e < n_e; e += BLOCK) {
        const uint64_t d = (uint64_t)S.pos + 2u * (uint64_t)e;
        const uint4 r = philox4x32_10((uint32_t)(d >> 1), S.stream, (uint32_t)(d >> 33), kTagK, S.k0, S.k1);
        const int choice = (((uint64_t)(r.x >> 5) << 26) | (uint64_t)(r.y >> 6)) < r53 ? 1 : 0;
        A.choice[e] = choice;
        const uint64_t m = ((uint64_t)(r.z >> 5) << 26) | (uint64_t)(r.w >> 6);
        u2bits[e] = m;
        score(e, choice, __fmul_rn(__ull2float_rn(m), 0x1p-53f));
      }
      advance(S, 2 * n_e);
    } else {
      for (int c0 = 0; c0 < n_e; c0 += kChunk) {
        const int cnt = min(kChunk, n_e - c0);
        if (!ensure<BLOCK>(S, cnt)) return MCL_EBUDGET;
        for (int k = tid; k < cnt; k += BLOCK)
          A.choice[c0 + k] = (gen ? bits53(S, k) < r53 : value(S, k) < sm.Retrap) ? 1 : 0;
        advance(S, cnt);
        __syncthreads();
      }
      for (int c0 = 0; c0 < n_e; c0 += kChunk) {
        const int cnt = min(kChunk, n_e - c0);
        if (!ensure<BLOCK>(S, cnt)) return MCL_EBUDGET;
        for (int k = tid; k < cnt; k += BLOCK) {
          const int e = c0 + k;
          float uf;
          if (gen) {
            const uint64_t m = bits53(S, k);
            u2bits[e] = m;
            uf = __fmul_rn(__ull2float_rn(m), 0x1p-53f);  // = float(m 2^-53), both rounded once
          } else {
            const double u2 = value(S, k);
            A.u2[e] = u2;
            uf = __double2float_rn(u2);
          }
          score(e, A.choice[e], uf);
        }
        advance(S, cnt);
        __syncthreads();
      }
    }
    float lmin_b;
    int allflags;
    block_minf<BLOCK>(sh, rot, lmin, flags, lmin_b, allflags);
    const bool exact_all = (allflags & 1) != 0;
    const float thr = lmin_b + 1e-3f;
    auto draw_e = [&](int e) {  // -log(1 - u) of electron e's wait uniform
      const double u2 = gen ? __dmul_rn(__ull2double_rn(u2bits[e]), 0x1p-53) : A.u2[e];
      return -log(__dadd_rn(1.0, -u2));
    };
    auto lifetime = [&](int e) {
      const double arg = __dadd_rn(A.choice[e] ? d2 : d1, -__dmul_rn(sm.alpha, A.ed[e]));
      const double rate = __dmul_rn(sm.b, exp(arg));
      return __ddiv_rn(1.0, __dadd_rn(rcb, rate));
    };
    if (!exact_all) {
      // The few candidates go to a list; warp 1 evaluates their draws' log
      // while warp 0 evaluates their lifetimes (two FP64 chains at once),
      // then warp 0 takes np.argmin over the list.
      for (int e = tid; e < n_e; e += BLOCK)
        if (A.lw[e] <= thr) {
          const int k = atomicAdd(&sh.n_cand, 1);
          if (k < 32) sh.cand[k] = e;
        }
      __syncthreads();
      const int nc = sh.n_cand;
      if (nc <= 32) {
        const int lane = tid & 31, warp = tid >> 5;
        if (warp == 1 && lane < nc) sh.cand_e[lane] = draw_e(sh.cand[lane]);
        double life = 0.0;
        if (warp == 0 && lane < nc) life = lifetime(sh.cand[lane]);
        __syncthreads();
        if (warp == 0) {
          double v = INFINITY;
          int i = INT_MAX;
          if (lane < nc) {
            v = __dmul_rn(life, sh.cand_e[lane]);
            i = sh.cand[lane];
          }
          long long k = argmin_key(v);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const long long k2 = __shfl_down_sync(0xffffffffu, k, o);
            const double v2 = __shfl_down_sync(0xffffffffu, v, o);
            const int i2 = __shfl_down_sync(0xffffffffu, i, o);
            if (k2 < k || (k2 == k && i2 < i)) {
              k = k2;
              v = v2;
              i = i2;
            }
          }
          if (lane == 0) {
            sh.best_v = v;
            sh.best_i = i;
          }
        }
        __syncthreads();
        wmin = sh.best_v;
        emin = sh.best_i;
        any = (allflags & 2) ? 1 : 0;
        __syncthreads();  // sh.best_* and the list are reused
        return MCL_OK;
      }
    }
    // every electron (exact_all), or more than 32 candidates: each thread
    // evaluates its own and the block takes the argmin
    double bv = INFINITY;
    int bi = INT_MAX, an = 0;
    for (int e = tid; e < n_e; e += BLOCK) {
      if (!exact_all && !(A.lw[e] <= thr)) continue;
      const double w = __dmul_rn(lifetime(e), draw_e(e));
      an |= (w != 0.0);
      if (better(w, e, bv, bi)) {
        bv = w;
        bi = e;
      }
    }
    block_argmin<BLOCK>(sh, bv, bi, an, wmin, emin, any);
    if (!exact_all) any = (allflags & 2) ? 1 : 0;
    return MCL_OK;
  };

  // filling wait (tl_trap_lab.py:53-60): one uniform whenever lambda > 0.
  // fill_draw takes the uniform (every thread reads the same value) and a
  // lower bound of the wait, lb = 0.99 u / lambda <= (1 / lambda)(-log(1 - u))
  // (in FP32: its roundings are far inside the factor 0.99; 0 when lambda is
  // below 1e-30, where the quotient could leave the FP32 range);
  // fill_exact evaluates the wait itself (one thread, FP64), which the
  // simulate loop skips whenever the bound already shows that it is not the
  // minimum.
  const double fill_rate = __ddiv_rn(sm.dose_rate, sm.D0);  // per empty trap
  auto fill_draw = [&](double& lam, double& u, double& lb) -> int {
    if ((int64_t)n_e == N || sm.dose_rate == 0.0) lam = 1e-20;
    else lam = __dmul_rn(fill_rate, (double)(N - (int64_t)n_e));
    u = 0.0;
    lb = 1e20;
    if (lam > 0.0) {
      if (!ensure<BLOCK>(S, 1)) return MCL_EBUDGET;
      u = value(S, 0);
      advance(S, 1);
      lb = lam >= 1e-30 ? (double)(0.99f * __fdiv_rn(__double2float_rn(u), __double2float_rn(lam))) : 0.0;
    }
    return MCL_OK;
  };
  auto fill_exact = [&](double lam, double u) -> double {
    if (!(lam > 0.0)) return 1e20;
    __syncthreads();  // every thread has read the uniform
    if (tid == 0) sh.dt_fill = __dmul_rn(__ddiv_rn(1.0, lam), -log(__dadd_rn(1.0, -u)));
    __syncthreads();
    return sh.dt_fill;
  };
  auto fill_wait = [&](double& dt_fill) -> int {
    double lam, u, lb;
    const int st = fill_draw(lam, u, lb);
    if (st != MCL_OK) return st;
    dt_fill = fill_exact(lam, u);
    return MCL_OK;
  };

  auto log_event = [&](int step, int kind, int e, int h) {
    if (tid == 0 && a.events && n_ev < sm.ev_cap) {
      int32_t* evp = a.events + 4 * (sm.ev_offset + n_ev);
      evp[0] = step;
      evp[1] = kind;
      evp[2] = e;
      evp[3] = h;
    }
    ++n_ev;
  };

  // pair creation (engine.py:133-152)
  auto pair_create = [&](int step) -> int {
    if (!ensure<BLOCK>(S, 6)) return MCL_EBUDGET;
    const double nex = __dmul_rn(value(S, 0), sm.L), ney = __dmul_rn(value(S, 1), sm.W),
                 nez = __dmul_rn(value(S, 2), sm.H);
    const double nhx = __dmul_rn(value(S, 3), sm.Lb), nhy = __dmul_rn(value(S, 4), sm.Wb),
                 nhz = __dmul_rn(value(S, 5), sm.Hb);
    advance(S, 6);
    if (n_h == 0) return MCL_ENOHOLE;
    if (n_e + 1 > sm.e_cap || n_h + 1 > sm.h_cap) return MCL_ECAPACITY;
    double dn;
    int hn;
    const float qx = scaled(nex, A.inv_l), qy = scaled(ney, A.inv_l), qz = scaled(nez, A.inv_l);
    nearest_block<BLOCK>(sh, rot, A, n_h, nex, ney, nez, qx, qy, qz, dn, hn);  // OLD holes only
    if (tid == 0) {
      A.ex[n_e] = nex;
      A.ey[n_e] = ney;
      A.ez[n_e] = nez;
      A.exf[n_e] = qx;
      A.eyf[n_e] = qy;
      A.ezf[n_e] = qz;
      A.ed[n_e] = dn;
      A.edf[n_e] = __double2float_rn(dn);
      A.en[n_e] = hn;
      A.hx[n_h] = nhx;
      A.hy[n_h] = nhy;
      A.hz[n_h] = nhz;
      A.hxf[n_h] = scaled(nhx, A.inv_l);
      A.hyf[n_h] = scaled(nhy, A.inv_l);
      A.hzf[n_h] = scaled(nhz, A.inv_l);
    }
    log_event(step, 0, n_e, n_h);
    ++n_e;
    ++n_h;
    __syncthreads();
    return MCL_OK;
  };

  // recombination (engine.py:154-175)
  auto remove_pair = [&](int step, int e_idx) -> int {
    const int h_idx = A.en[e_idx];
    __syncthreads();
    log_event(step, 1, e_idx, h_idx);
    // np.delete of electron row e_idx and hole h_idx: shift the tails down
    const int ne_tail = n_e - 1 - e_idx, nh_tail = n_h - 1 - h_idx;
    for (int base = 0; base < max(ne_tail, nh_tail); base += BLOCK) {
      const int k = base + tid;
      double x0 = 0, y0 = 0, z0 = 0, d0 = 0, hx0 = 0, hy0 = 0, hz0 = 0;
      float f0 = 0, hxf0 = 0, hyf0 = 0, hzf0 = 0, exf0 = 0, eyf0 = 0, ezf0 = 0;
      int n0 = 0;
      if (k < ne_tail) {
        const int s = e_idx + 1 + k;
        x0 = A.ex[s];
        y0 = A.ey[s];
        z0 = A.ez[s];
        d0 = A.ed[s];
        f0 = A.edf[s];
        n0 = A.en[s];
        exf0 = A.exf[s];
        eyf0 = A.eyf[s];
        ezf0 = A.ezf[s];
      }
      if (k < nh_tail) {
        const int s = h_idx + 1 + k;
        hx0 = A.hx[s];
        hy0 = A.hy[s];
        hz0 = A.hz[s];
        hxf0 = A.hxf[s];
        hyf0 = A.hyf[s];
        hzf0 = A.hzf[s];
      }
      __syncthreads();
      if (k < ne_tail) {
        const int dst = e_idx + k;
        A.ex[dst] = x0;
        A.ey[dst] = y0;
        A.ez[dst] = z0;
        A.ed[dst] = d0;
        A.edf[dst] = f0;
        A.en[dst] = n0;
        A.exf[dst] = exf0;
        A.eyf[dst] = eyf0;
        A.ezf[dst] = ezf0;
      }
      if (k < nh_tail) {
        const int dst = h_idx + k;
        A.hx[dst] = hx0;
        A.hy[dst] = hy0;
        A.hz[dst] = hz0;
        A.hxf[dst] = hxf0;
        A.hyf[dst] = hyf0;
        A.hzf[dst] = hzf0;
      }
      __syncthreads();
    }
    --n_e;
    --n_h;
    if (tid == 0) sh.n_mask = 0;
    __syncthreads();
    for (int e = tid; e < n_e; e += BLOCK) {
      int nn = A.en[e];
      if (nn > h_idx) A.en[e] = --nn;
      if (nn == h_idx) A.mlist[atomicAdd(&sh.n_mask, 1)] = e;
    }
    __syncthreads();
    const int n_mask = sh.n_mask;
    if (n_mask > 0 && n_h == 0) return MCL_ENOHOLE;
    for (int m = 0; m < n_mask; ++m) {
      const int e = A.mlist[m];
      double dn;
      int hn;
      nearest_block<BLOCK>(sh, rot, A, n_h, A.ex[e], A.ey[e], A.ez[e], A.exf[e], A.eyf[e], A.ezf[e], dn, hn);
      if (tid == 0) {
        A.ed[e] = dn;
        A.edf[e] = __double2float_rn(dn);
        A.en[e] = hn;
      }
      __syncthreads();
    }
    return MCL_OK;
  };

  double t = 0.0;
  int i = 0;
  const int64_t out = sm.out_offset;
  if (sm.loop == MCL_LOOP_SIMULATE) {
    // ---- the step loop of simulate() (simulate.py:51-92) ------------------
    while (status == MCL_OK && t <= sm.duration) {
      const double T = __dadd_rn(__dadd_rn(sm.T_start, __dmul_rn(sm.T_rate, t)), 273.15);
      double wmin, dt_fill;
      int emin, any;
      if ((status = waits(T, wmin, emin, any)) != MCL_OK) break;
      double lam, uf, lb;
      if ((status = fill_draw(lam, uf, lb)) != MCL_OK) break;
      // the filling wait matters only if it can be the minimum (uniform
      // over the CTA: wmin, any and the uniform are the same in every thread)
      const bool need_fill = !any || !((wmin < sm.dt_cap ? wmin : sm.dt_cap) < lb);
      dt_fill = need_fill ? fill_exact(lam, uf) : INFINITY;
      const double dt_recomb = any ? wmin : dt_fill;
      double dt = dt_fill;  // Python's min(): the first minimal argument
      if (dt_recomb < dt) dt = dt_recomb;
      if (sm.dt_cap < dt) dt = sm.dt_cap;
      t = __dadd_rn(t, dt);
      if (i >= sm.steps) {  // x_ax[i] would raise IndexError (simulate.py:64)
        status = MCL_EOVERFLOW;
        break;
      }
      if (tid == 0) a.x_ax[out + i] = t;
      double ev = 0.0;
      if (dt == dt_fill) {
        if ((status = pair_create(i)) != MCL_OK) break;
      } else if (dt == dt_recomb) {
        if ((status = remove_pair(i, emin)) != MCL_OK) break;
        ev = 1.0;
      }
      if (tid == 0) {
        a.lum[out + i] = ev;
        a.ratio[out + i] = __ddiv_rn((double)n_e, sm.N_e);
      }
      ++i;
      if (sm.duration != 0.0 && t >= sm.duration) break;
    }
  } else if (status == MCL_OK) {
    // ---- the lab-data loops (tl_trap_lab.py:90-108 and :147-172) ----------
    // T(t) = T_start[K] + T_rate (t + dt) after each event (isothermal: T_rate
    // 0); waits and the fill wait are drawn before the loop and after every
    // event; dt = min(dt_recomb, tf) with no cap; a simulation without
    // electrons (.size == 0) waits for a pair creation.
    const double T0 = __dadd_rn(sm.T_start, 273.15);
    double wmin, tf;
    int emin, any;
    int obs_idx = 0;
    if (sm.loop == MCL_LOOP_LAB_ISO && (!a.obs_time || !a.obs_ratio)) status = MCL_EINVAL;
    if (status == MCL_OK) status = waits(T0, wmin, emin, any);
    if (status == MCL_OK) status = fill_wait(tf);
    while (status == MCL_OK) {
      if (sm.loop == MCL_LOOP_LAB_TL ? !(t < sm.duration) : !(obs_idx < sm.n_obs)) break;
      const double dt_recomb = n_e > 0 ? wmin : tf;
      const double dt = tf < dt_recomb ? tf : dt_recomb;
      const double T_now = __dadd_rn(T0, __dmul_rn(sm.T_rate, __dadd_rn(t, dt)));
      t = __dadd_rn(t, dt);
      if (i >= sm.steps) {
        status = MCL_EOVERFLOW;
        break;
      }
      if (tid == 0) a.x_ax[out + i] = t;
      double ev = 0.0;
      if (dt == tf) {
        if ((status = pair_create(i)) != MCL_OK) break;
      } else {
        if ((status = remove_pair(i, emin)) != MCL_OK) break;
        ev = 1.0;
      }
      if ((status = fill_wait(tf)) != MCL_OK) break;
      if ((status = waits(T_now, wmin, emin, any)) != MCL_OK) break;
      if (tid == 0) {
        a.lum[out + i] = ev;
        a.ratio[out + i] = __ddiv_rn((double)n_e, sm.N_e);
      }
      ++i;
      while (obs_idx < sm.n_obs && t >= a.obs_time[sm.obs_offset + obs_idx]) {
        if (tid == 0) a.obs_ratio[sm.obs_offset + obs_idx] = __ddiv_rn((double)n_e, sm.N_e);
        ++obs_idx;
      }
    }
  }
  (void)n_ev_local;
  if (tid == 0) {
    a.n_steps[si] = i;
    a.n_events[si] = n_ev;
    a.draws[si] = S.pos;
    a.status[si] = status;
  }
  __syncthreads();
  return status;
}

template <int BLOCK, bool SMEM_ARRAYS>
__global__ void __launch_bounds__(BLOCK) kk_kernel(const mcl_k_args a, int e_cap_max, int h_cap_max) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Shared sh;
  Source S;
  S.rng = a.rng;
  S.u = a.uniforms;
  S.k0 = (uint32_t)a.seed;
  S.k1 = (uint32_t)(a.seed >> 32);
  S.mt = reinterpret_cast<uint32_t*>(smem);
  S.mt2 = S.mt + 640;
  S.ring = S.mt + 1280;
  unsigned char* arr_base = smem + sizeof(uint32_t) * (1280 + kRing);
  S.rd = S.wr = 0;
  if (a.rng == MCL_RNG_MT19937) {
    // load the key array and position; queue the untaken words of the current block
    for (int k = threadIdx.x; k < kMtN; k += BLOCK) S.mt[k] = a.mt_state[k];
    __syncthreads();
    const uint32_t p = a.mt_state[kMtN];
    for (int k = threadIdx.x + (int)p; k < kMtN; k += BLOCK) S.ring[k - p] = mt_temper(S.mt[k]);
    S.wr = kMtN - p;
    __syncthreads();
  }
  int rot = 0;  // block_minf's slot rotation
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) {
      sh.mkey[k] = INT_MAX;
      sh.mflags[k] = 0;
    }
  __syncthreads();
  const int first = a.sequential ? 0 : blockIdx.x;
  const int last = a.sequential ? a.n_sims : blockIdx.x + 1;
  for (int si = first; si < last; ++si) {
    const mcl_k_sim sm = a.sims[si];
    S.stream = sm.stream_id;
    if (!a.sequential || si == first) {
      S.u_base = sm.u_offset;
      S.u_count = sm.u_count;
    }
    unsigned char* region = reinterpret_cast<unsigned char*>(a.workspace) + sm.ws_offset;
    unsigned char* local = SMEM_ARRAYS ? arr_base : region + hole64_bytes(sm.h_cap);
    Arrays A = carve(local, SMEM_ARRAYS ? e_cap_max : sm.e_cap, SMEM_ARRAYS ? h_cap_max : sm.h_cap, region,
                     sm.h_cap);
    A.inv_l = 1.0 / fmax(fmax(fmax(sm.L, sm.W), fmax(sm.H, sm.Lb)), fmax(fmax(sm.Wb, sm.Hb), 1e-300));
    if (run_sim<BLOCK>(a, si, sm, A, sh, rot, S) != MCL_OK && a.sequential) break;
    // sequential runs share one injected stream: the next simulation starts
    // where this one stopped (like the reference's global RandomState)
    S.u_base += S.pos;
    S.u_count -= S.pos;
  }
  if (a.rng == MCL_RNG_MT19937 && a.sequential) {
    // the unread ring words all come from the last block: position = 624 - left
    for (int k = threadIdx.x; k < kMtN; k += BLOCK) a.mt_state[k] = S.mt[k];
    if (threadIdx.x == 0) a.mt_state[kMtN] = (uint32_t)(kMtN - (int)(S.wr - S.rd));
  }
}

constexpr size_t kFixedSmem = sizeof(uint32_t) * (1280 + kRing);
constexpr size_t kMaxSmem = 220 * 1024;

}  // namespace
}  // namespace mcl

using namespace mcl;

extern "C" int mcl_k_validate(const mcl_k_sim* sims, int32_t n_sims, int32_t rng, int32_t block,
                              int64_t n_uniforms, int32_t* arrays_in_smem, int64_t* workspace_bytes,
                              int32_t* e_cap_max, int32_t* h_cap_max) {
  if (n_sims < 0 || (n_sims > 0 && !sims)) return MCL_EINVAL;
  if (rng != MCL_RNG_PHILOX && rng != MCL_RNG_INJECTED && rng != MCL_RNG_MT19937) return MCL_EINVAL;
  if (block != 256 && block != 512) return MCL_EINVAL;
  int e_max = 0, h_max = 0;
  int64_t ws = 0;
  for (int32_t i = 0; i < n_sims; ++i) {
    const mcl_k_sim& s = sims[i];
    if (s.e0 < 0 || s.n_h0 < 0 || s.e_cap < s.e0 || s.h_cap < s.n_h0 || s.steps < 0) return MCL_EINVAL;
    if (s.ev_cap < 0 || s.ev_offset < 0 || s.out_offset < 0 || s.ws_offset < 0) return MCL_EINVAL;
    if (s.loop < MCL_LOOP_SIMULATE || s.loop > MCL_LOOP_LAB_ISO || s.n_obs < 0 || s.obs_offset < 0)
      return MCL_EINVAL;
    if (s.loop == MCL_LOOP_LAB_ISO && s.n_obs == 0) return MCL_EINVAL;
    if (!(s.N_e > 0) || !std::isfinite(s.duration) || !std::isfinite(s.T_rate)) return MCL_EINVAL;
    if (rng == MCL_RNG_INJECTED && (s.u_offset < 0 || s.u_count < 0 || s.u_offset + s.u_count > n_uniforms))
      return MCL_ECAPACITY;
    if (s.ws_offset % 16) return MCL_EINVAL;
    e_max = s.e_cap > e_max ? s.e_cap : e_max;
    h_max = s.h_cap > h_max ? s.h_cap : h_max;
  }
  const bool fits = kFixedSmem + local_bytes(e_max, h_max) <= kMaxSmem;
  for (int32_t i = 0; i < n_sims; ++i) {
    const int64_t end = sims[i].ws_offset + (int64_t)region_bytes(sims[i].e_cap, sims[i].h_cap, fits);
    ws = end > ws ? end : ws;
  }
  if (arrays_in_smem) *arrays_in_smem = fits ? 1 : 0;
  if (workspace_bytes) *workspace_bytes = ws;
  if (e_cap_max) *e_cap_max = e_max;
  if (h_cap_max) *h_cap_max = h_max;
  return MCL_OK;
}

extern "C" int64_t mcl_k_region_bytes(int32_t e_cap, int32_t h_cap, int32_t arrays_in_smem) {
  if (e_cap < 0 || h_cap < 0) return -1;
  return (int64_t)region_bytes(e_cap, h_cap, arrays_in_smem != 0);
}

extern "C" int32_t mcl_k_arrays_fit_smem(int32_t e_cap_max, int32_t h_cap_max) {
  return kFixedSmem + local_bytes(e_cap_max, h_cap_max) <= kMaxSmem ? 1 : 0;
}

namespace {
template <int BLOCK>
int launch_k(const mcl_k_args& a, cudaStream_t s) {
  const bool in_smem = a.arrays_in_smem != 0;
  const size_t smem = kFixedSmem + (in_smem ? local_bytes(a.e_cap_max, a.h_cap_max) : 0);
  if (smem > kMaxSmem) return MCL_ECAPACITY;
  if (!a.workspace) return MCL_EINVAL;
  auto fn = in_smem ? kk_kernel<BLOCK, true> : kk_kernel<BLOCK, false>;
  MCL_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = a.sequential ? 1 : a.n_sims;
  fn<<<grid, BLOCK, smem, s>>>(a, a.e_cap_max, a.h_cap_max);
  MCL_CUDA_TRY(cudaGetLastError());
  return MCL_OK;
}
}  // namespace

extern "C" int mcl_k_run(const mcl_k_args* args, void* stream) {
  if (!args) return MCL_EINVAL;
  const mcl_k_args& a = *args;
  if (a.n_sims == 0) return MCL_OK;
  if (a.n_sims < 0 || !a.sims || !a.x_ax || !a.lum || !a.ratio || !a.n_events || !a.n_steps ||
      !a.draws || !a.status)
    return MCL_EINVAL;
  if (a.rng == MCL_RNG_INJECTED && !a.uniforms) return MCL_EINVAL;
  if (a.rng == MCL_RNG_MT19937 && (!a.mt_state || !a.sequential)) return MCL_EINVAL;
  if (a.rng != MCL_RNG_PHILOX && a.rng != MCL_RNG_INJECTED && a.rng != MCL_RNG_MT19937) return MCL_EINVAL;
  if (a.e_cap_max < 0 || a.h_cap_max < 0) return MCL_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (a.block == 256) return launch_k<256>(a, s);
  if (a.block == 512) return launch_k<512>(a, s);
  return MCL_EINVAL;
}
