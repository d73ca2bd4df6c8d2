// Device code of the Bernoulli kernels, shared by the translation units that
// instantiate them (one per FP32 launch shape and one for FP64, compiled in
// parallel).
// The method is described at the top of kinetics_b.cu.
#pragma once

#include <algorithm>

#include "common.cuh"
namespace mcl {
namespace {

constexpr int kChunk = 256;       // steps per shared-memory chunk of (c_j, q_j)
constexpr int kHeaderBytes = 256;  // workspace header (ticket)

struct Header {
  int32_t ticket;
};

// Kernel parameters: the public launch arguments plus the Philox key
// schedule k + r*W (r = 0..9), which lands in the constant parameter bank.
struct KParams {
  mcl_b_args a;
  uint32_t ks0[10];
  uint32_t ks1[10];
};

// Philox4x32-10 with a precomputed key schedule.
__device__ __forceinline__ uint4 philox_ks(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                           const KParams& p) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)kPhiloxM0 * c0;
    const uint64_t p1 = (uint64_t)kPhiloxM1 * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ p.ks0[r];
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ p.ks1[r];
    c1 = (uint32_t)p1;
    c3 = (uint32_t)p0;
    c0 = n0;
    c2 = n2;
  }
  return make_uint4(c0, c1, c2, c3);
}

// c_j and q_j of local step j of segment sg (FP64 without contraction, in the
// oracle's evaluation order).
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

// Extents of set st against the sizes the launch declares (a C caller may
// pass sets whose offsets disagree with them).  Returns the set's step count
// (the sum of its segments' n_steps, which is what the kernels index with),
// or -1 if a segment, table row, bin, slot or injected uniform of the set
// would fall outside its buffer.  Every thread of a CTA evaluates it for the
// same set, so the answer is uniform over the CTA.
__device__ __forceinline__ int64_t checked_steps(const mcl_b_args& a, const mcl_set& st) {
  if (st.seg_begin < 0 || st.seg_count < 0 || (int64_t)st.seg_begin + st.seg_count > a.n_segs) return -1;
  if (st.n_slots < 0 || st.n_filled < 0 || st.n_filled > st.n_slots) return -1;
  if (st.n_bins < 0 || st.n_bins > a.max_bins || st.bin_offset < 0 || st.bin_offset + st.n_bins > a.n_bins_total)
    return -1;
  if (st.slot_offset < 0 || st.slot_offset + st.n_slots > a.n_slots_total) return -1;
  int64_t steps = 0;
  for (int g = 0; g < st.seg_count; ++g) {
    const mcl_segment& sg = a.segs[st.seg_begin + g];
    if (sg.n_steps < 0 || sg.steps_per_bin < 1 || sg.bin_offset < 0) return -1;
    if ((int64_t)sg.bin_offset + ((int64_t)sg.n_steps + sg.steps_per_bin - 1) / sg.steps_per_bin > st.n_bins)
      return -1;
    steps += sg.n_steps;
  }
  if (steps > 0x7fffffff || st.step_offset < 0 || st.step_offset + steps > a.table_steps) return -1;
  if (a.rng == MCL_RNG_INJECTED &&
      (st.u_offset < 0 || st.u_offset + (int64_t)st.n_slots * (1 + steps) > a.n_uniforms))
    return -1;
  return steps;
}

// The item's set, or -1 (with the status word set) if the item or its set
// fails the extent checks.
__device__ __forceinline__ int checked_item(const mcl_b_args& a, const mcl_item& item) {
  if (item.set < 0 || item.set >= a.n_sets) {
    report(a.status, MCL_EINVAL);
    return -1;
  }
  const mcl_set& st = a.sets[item.set];
  if (item.slot_begin < 0 || item.slot_begin >= st.n_slots) {
    report(a.status, MCL_EINVAL);
    return -1;
  }
  if (checked_steps(a, st) < 0) {
    report(a.status, MCL_ECAPACITY);
    return -1;
  }
  return item.set;
}

// Pre-pass: one CTA per set fills its rows of the (c_j, q_j) table (none if
// the set's rows would leave the table).
template <typename T>
__global__ void __launch_bounds__(256) kb_tables(const mcl_b_args a) {
  const int s = blockIdx.x;
  if (s >= a.n_sets) return;
  const mcl_set st = a.sets[s];
  if (checked_steps(a, st) < 0) {
    if (threadIdx.x == 0) report(a.status, MCL_ECAPACITY);
    return;
  }
  T* tab = reinterpret_cast<T*>(reinterpret_cast<char*>(a.workspace) + kHeaderBytes) + 2 * st.step_offset;
  int64_t base = 0;
  for (int g = 0; g < st.seg_count; ++g) {
    const mcl_segment sg = a.segs[st.seg_begin + g];
    for (int j = threadIdx.x; j < sg.n_steps; j += blockDim.x) {
      double c, q;
      step_constants(st, sg, j, c, q);
      tab[2 * (base + j)] = (T)c;
      tab[2 * (base + j) + 1] = (T)q;
    }
    base += sg.n_steps;
  }
}

__device__ __forceinline__ float r_prime_f(float u) { return cbrtf(-log1pf(-u)); }
__device__ __forceinline__ double r_prime_d(double u) { return cbrt(-log1p(-u)); }

// Exact FP32-mode tests, kept out of line: they run on ~2e-5 of the trials.
// The 32-bit uniform of a trial is (h << 16) | lo16: h is the 16-bit field the
// fast test used, lo16 the low half of word 0 of philox(step, slot, set,
// TAG_LO).  An event happens iff u32 < T, T = ceil(prob 2^32) (2^32 when
// prob >= 1).  When every lo16 gives the same answer -- (h + 1) 2^16 <= T or
// h 2^16 >= T -- the low half is not drawn: only h == T >> 16 needs it.  The
// counter-based stream makes skipping a draw invisible to every other draw.
__device__ __forceinline__ uint64_t threshold_u32(float prob) {
  return prob >= 1.0f ? (1ull << 32) : (uint64_t)__float2uint_ru(__fmul_rn(prob, 4294967296.0f));
}

__device__ __noinline__ bool u32_below(uint32_t h, uint64_t T, uint32_t kstep, uint32_t slot, uint32_t set_id,
                                       const KParams& P) {
  const uint64_t lo_edge = (uint64_t)h << 16;
  if (T >= lo_edge + 65536u) return true;
  if (T <= lo_edge) return false;
  const uint4 r = philox_ks(kstep, slot, set_id, kTagLow, P);
  return (lo_edge | (r.x & 0xffffu)) < T;
}

// p = -expm1f(-c w) for an escape
__device__ __noinline__ bool escape_exact(uint32_t h, float c, float w, uint32_t kstep, uint32_t slot,
                                          uint32_t set_id, const KParams& P) {
  return u32_below(h, threshold_u32(-expm1f(-__fmul_rn(c, w))), kstep, slot, set_id, P);
}

__device__ __noinline__ bool threshold_exact(uint32_t h, float q, uint32_t kstep, uint32_t slot,
                                             uint32_t set_id, const KParams& P) {
  return u32_below(h, threshold_u32(q), kstep, slot, set_id, P);
}

__device__ __noinline__ float refill_w(uint32_t word, float alpha) {
  const float u = (float)(word >> 8) * 0x1p-24f;
  return expf(-alpha * r_prime_f(u));
}

// Sum `v` over the warp and add it to *dst from lane 0 (skipped if all zero).
__device__ __forceinline__ void warp_flush(uint32_t v, uint32_t* dst) {
  if (__any_sync(0xffffffffu, v != 0)) {
    const uint32_t tot = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) atomicAdd(dst, tot);
  }
}

// The CTA's bins: `copies` copies of the recombination counts, max_bins
// apart, and one of the filled counts.
template <int BLOCK>
__device__ __forceinline__ void zero_bins(uint32_t* s_lum, uint32_t* s_alive, int n_bins, int copies = 1,
                                          int stride = 0) {
  for (int b = threadIdx.x; b < n_bins; b += BLOCK) {
    for (int c = 0; c < copies; ++c) s_lum[c * stride + b] = 0;
    if (s_alive) s_alive[b] = 0;
  }
}

template <int BLOCK>
__device__ __forceinline__ void flush_bins(const mcl_b_args& a, const mcl_set& st, const uint32_t* s_lum,
                                           const uint32_t* s_alive, int copies = 1, int stride = 0) {
  for (int b = threadIdx.x; b < st.n_bins; b += BLOCK) {
    uint32_t v = s_lum[b];
    for (int c = 1; c < copies; ++c) v += s_lum[c * stride + b];
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

// Step t (0..7) of a Philox block uses the 16-bit field h of word t&3: the
// word's upper half for t < 4, its lower half for t >= 4.  field_f returns the
// float 2^23 + h with one byte permute (h becomes the low mantissa bits under
// the exponent of 2^23).
template <int T>
__device__ __forceinline__ float field_f(uint32_t word) {
  return __uint_as_float(__byte_perm(word, 0x4B000000u, (T < 4) ? 0x7432 : 0x7410));
}

template <int T>
__device__ __forceinline__ uint32_t field16(uint32_t word) {
  return (T < 4) ? (word >> 16) : (word & 0xffffu);
}

// Per-step float test of the FP32 mode (run for the traps the integer
// prefilter below flags).  The shared-memory step table holds
// c16 = c * 2^16 and q16 = q * 2^16 (exact power-of-two scalings).  For a
// filled trap d = fl(2^23 + h - c16 w) (one FFMA), for an empty trap of a
// filling segment d = fl(2^23 + h - q16).  An event needs u32 < ceil(p 2^32)
// with u32 = h 2^16 + lo16, hence h < p 2^16 <= c16 w (1 + 2^-21) < c16 w + 2^-5
// when c w < 1, so the exact value of d is below 2^23 + 2^-5 and d rounds to
// at most 2^23; d >= kCand = 2^23 + 1 therefore proves that nothing happens.
// (For c w >= 1, d <= 2^23 + 65535 - 65536 and the trial is always a
// candidate.)  The test admits h <= c16 w + 1/2, i.e. about c w + 2^-16 of the
// trials, which go to the exact test.
constexpr float kCand = 8388609.0f;  // 2^23 + 1
constexpr float kInv16 = 0x1p-16f;

// Per-thread state of the FP32 kernel for one work item.
template <int EPT>
struct SlotState {
  float w[EPT];        // w of a filled trap, 0 for an empty one
  uint32_t slot[EPT];  // slot index within the set
  uint32_t filled;     // bit i: slot i holds an electron
};

// Block-level integer prefilter.  When the CTA stages a chunk of the step
// table it also stores, per 8-step block, cm = RU(max_t c16_t (1 + 2^-20))
// and (filling segments) qm = RU(max_t q16_t (1 + 2^-20)).  For a filled
// trap b = bits(RN(2^23 + 1 + cm w)) = 0x4B000000 + TI with TI = 1 +
// rint(cm w) while cm w < 2^23 - 1; an empty trap of a filling segment uses
// b = bits(RN(2^23 + 1 + qm)).  An escape at step t needs h < p 2^16 <=
// c16_t w (1 + 2^-22) <= cm w (the tests above), a refill h < q16_t <= qm,
// hence h <= floor(bound) < TI.  With TI <= 0x7FFF (b <= kHotBits) both
// 16-bit fields of a Philox word are tested by one subtraction r = word -
// TI (2^16 + 1): bit 15 of r & ~word is set iff lo < TI, bit 31 iff
// hi < TI + [lo < TI] (a borrow only adds the case hi == TI); a field with
// its top bit set is never below TI.  TI (2^16 + 1) is one byte permute of b,
// whose low 16 bits are TI.  A trap with b > kHotBits (p or q near 1/2 or
// more, or a non-finite rate) flags every trap of its thread's block.
constexpr uint32_t kHotBits = 0x4B007FFFu;
constexpr float kCmScale = 1.0f + 0x1p-20f;
constexpr int kBlocksPerChunk = kChunk / 8;

// Nonzero iff one of the 8 fields of Philox block r is below TI, b =
// 0x4B000000 + TI.
__device__ __forceinline__ uint32_t field_flags(const uint4& r, uint32_t b) {
  const uint32_t tt = __byte_perm(b, 0u, 0x1010);  // TI * 0x10001 (TI < 2^16)
  return (((r.x - tt) & ~r.x) | ((r.y - tt) & ~r.y) | ((r.z - tt) & ~r.z) | ((r.w - tt) & ~r.w)) &
         0x80008000u;
}

// Alive counts at the bin ends inside a block of n steps (the block's first
// step is seg_left steps before the segment's end).  to_flush counts the
// steps up to and including the one that ends the current bin; alive_at(t)
// is the thread's filled count after step t.
template <typename AliveAt>
__device__ __forceinline__ void flush_block_bins(int n, uint32_t* s_alive, int& bin, int& to_flush, int spb,
                                                 int seg_left, AliveAt alive_at) {
  if (to_flush > n) {
    to_flush -= n;
    return;
  }
  int t = to_flush - 1;  // block step that ends the current bin
  for (;;) {
    if (s_alive) warp_flush(alive_at(t), &s_alive[bin]);
    ++bin;
    const int next = min(spb, seg_left - t - 1);
    if (next == 0) {  // the segment's last step
      to_flush = 0;
      return;
    }
    if (t + next >= n) {
      to_flush = t + next - n + 1;
      return;
    }
    t += next;
  }
}

// Bin of block step t (the current bin ends at step to_flush - 1).
__device__ __forceinline__ int bin_of_step(int bin, int to_flush, int spb, int t) {
  for (int tf = to_flush; t >= tf; tf += spb) ++bin;
  return bin;
}

// Per-step tests of one filled trap over a Philox block of a segment without
// filling (steps 0..nq-1): the Philox block is drawn again (the fast pass
// keeps only a flag per trap), each step applies the FP32 test d = 2^23 + h -
// c16 w < kCand and then the exact test.  Returns the step of the escape, or
// -1.  A trap's fate depends only on its own uniforms, so testing the flagged
// traps one after another gives the same escapes as testing step by step.
__device__ __noinline__ int first_escape(const KParams& P, uint32_t set_id, uint32_t slot, float w, uint32_t blk,
                                         const float* c16, int nq, int64_t kstep) {
  const uint4 r = philox_ks(blk, slot, set_id, kTagStep, P);
#define MCL_T(T)                                                                                  \
  if ((T) < nq) {                                                                                 \
    const uint32_t word = word_of(r, (T) & 3);                                                    \
    const float c = c16[T];                                                                       \
    if (__fmaf_rn(-c, w, field_f<T>(word)) < kCand &&                                             \
        escape_exact(field16<T>(word), c * kInv16, w, (uint32_t)(kstep + (T)), slot, set_id, P))  \
      return (T);                                                                                 \
  }
  MCL_T(0) MCL_T(1) MCL_T(2) MCL_T(3) MCL_T(4) MCL_T(5) MCL_T(6) MCL_T(7)
#undef MCL_T
  return -1;
}

// The steps of one Philox block of a segment without filling (8 steps; fewer
// at the segment's end when FULL is false).  Traps only empty here, so flags
// computed with the state at the block's start can only over-report: the
// fast pass runs the integer prefilter over the 8 steps of each slot (one
// subtraction and one LOP3 per word, i.e. per two trials) and keeps one flag
// bit per slot; one branch per block sends the flagged filled traps to
// first_escape.  The bin bookkeeping then runs for the whole block: alive
// counts at bin ends inside the block subtract the escapes up to that step,
// which dcount holds as 4-bit counts per step (prefix sums by one multiply;
// EPT <= 8 keeps every nibble below 16, as a trap escapes at most once here).
template <int EPT, bool FULL>
__device__ __forceinline__ void block_nofill(const KParams& P, const mcl_set& st, SlotState<EPT>& S,
                                             uint32_t blk, const float* s_c, const float* s_cm, int jq, int nq,
                                             int64_t kstep, uint32_t* s_lum, uint32_t* s_alive, int& bin,
                                             int& to_flush, int spb, int seg_left) {
  static_assert(EPT <= 8, "per-step escape counts are 4-bit fields");
  const float cm = s_cm[jq >> 3];
  uint32_t mask = 0, hmax = 0;
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const uint4 r = philox_ks(blk, S.slot[i], st.set_id, kTagStep, P);
    // an empty trap (w = 0) gets TI = 1 here; the mask drops it below
    const uint32_t b = __float_as_uint(__fmaf_rn(cm, S.w[i], kCand));
    hmax = max(hmax, b);
    if (field_flags(r, b)) mask |= 1u << i;
  }
  if (hmax > kHotBits) mask = ~0u;
  mask &= S.filled;
  const uint32_t alive0 = (uint32_t)__popc(S.filled);
  uint32_t dcount = 0;
  if (mask) {
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      if ((mask >> i) & 1u) {
        const int t = first_escape(P, st.set_id, S.slot[i], S.w[i], blk, s_c + jq, FULL ? 8 : nq, kstep);
        if (t >= 0) {
          S.filled &= ~(1u << i);
          S.w[i] = 0.0f;
          atomicAdd(&s_lum[bin_of_step(bin, to_flush, spb, t)], 1u);
          if (P.a.fates) P.a.fates[st.slot_offset + S.slot[i]] = (int32_t)(kstep + t);
          dcount += 1u << (4 * t);
        }
      }
    }
  }
  const uint32_t cum = dcount * 0x11111111u;  // nibble t: escapes in steps 0..t
  flush_block_bins(FULL ? 8 : nq, s_alive, bin, to_flush, spb, seg_left,
                   [&](int t) { return alive0 - ((cum >> (4 * t)) & 0xfu); });
}

// Events of one trap over a Philox block of a filling segment (steps
// 0..nq-1), step by step: a filled trap may escape (FP32 test, then the
// exact test), an empty one in a real slot may be refilled (threshold q,
// then a fresh w from its refill counter) -- the tests of the per-step
// filling path, applied to one trap.  ev bits 0-7: escape steps; bits 8-15:
// refill steps; bit 16: filled at the end; w: the trap's w at the end.
struct FillEvents {
  uint32_t ev;
  float w;
};

__device__ __noinline__ FillEvents fill_events(const KParams& P, uint32_t set_id, uint32_t slot, bool real,
                                               bool filled, float w, uint32_t blk, const float* c16,
                                               const float* q16, int nq, int64_t kstep, float alpha) {
  const uint4 r = philox_ks(blk, slot, set_id, kTagStep, P);
  uint32_t ev = 0;
#define MCL_T(T)                                                                                          \
  if ((T) < nq) {                                                                                         \
    const uint32_t word = word_of(r, (T) & 3);                                                            \
    const float f = field_f<T>(word);                                                                     \
    const uint32_t ks = (uint32_t)(kstep + (T));                                                          \
    if (filled) {                                                                                         \
      const float c = c16[T];                                                                             \
      if (__fmaf_rn(-c, w, f) < kCand && escape_exact(field16<T>(word), c * kInv16, w, ks, slot, set_id, P)) { \
        filled = false;                                                                                   \
        w = 0.0f;                                                                                         \
        ev |= 1u << (T);                                                                                  \
      }                                                                                                   \
    } else if (real) {                                                                                    \
      const float q = q16[T];                                                                             \
      if (__fsub_rn(f, q) < kCand && threshold_exact(field16<T>(word), q * kInv16, ks, slot, set_id, P)) { \
        const uint4 rr = philox_ks(ks, slot, set_id, kTagRefill, P);                                      \
        w = refill_w(rr.x, alpha);                                                                        \
        filled = true;                                                                                    \
        ev |= 0x100u << (T);                                                                              \
      }                                                                                                   \
    }                                                                                                     \
  }
  MCL_T(0) MCL_T(1) MCL_T(2) MCL_T(3) MCL_T(4) MCL_T(5) MCL_T(6) MCL_T(7)
#undef MCL_T
  return FillEvents{ev | (filled ? 0x10000u : 0u), w};
}

// The steps of one Philox block of a filling segment (8 steps; fewer at the
// segment's end when FULL is false).  A trap that is not flagged by the
// prefilter (filled: escape bound cm w; empty: refill bound qm) has no event
// in the block, so it keeps its state and every later step of the block is
// covered by the same test; a flagged trap goes to fill_events, which runs
// all of the block's steps for it in order.  Refill and escape counts per step
// (8-bit fields; at most EPT events per step and 4 EPT per block) give the
// alive counts at bin ends inside the block.
template <int EPT, bool FULL>
__device__ __forceinline__ void block_fill(const KParams& P, const mcl_set& st, SlotState<EPT>& S,
                                           uint32_t blk, const float* s_c, const float* s_q, const float* s_cm,
                                           const float* s_qm, int jq, int nq, int64_t kstep, uint32_t* s_lum,
                                           uint32_t* s_alive, int& bin, int& to_flush, int spb, int seg_left,
                                           float alpha) {
  const float cm = s_cm[jq >> 3];
  const uint32_t bq = __float_as_uint(__fadd_rn(s_qm[jq >> 3], kCand));
  uint32_t mask = 0, hmax = bq;
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const uint4 r = philox_ks(blk, S.slot[i], st.set_id, kTagStep, P);
    const uint32_t b = ((S.filled >> i) & 1u) ? __float_as_uint(__fmaf_rn(cm, S.w[i], kCand)) : bq;
    hmax = max(hmax, b);
    if (field_flags(r, b)) mask |= 1u << i;
  }
  if (hmax > kHotBits) mask = ~0u;
  const uint32_t alive0 = (uint32_t)__popc(S.filled);
  uint64_t ecnt = 0, rcnt = 0;
  if (mask) {
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const bool filled = (S.filled >> i) & 1u;
      const bool real = S.slot[i] < (uint32_t)st.n_slots;
      if (((mask >> i) & 1u) && (filled || real)) {
        const FillEvents o = fill_events(P, st.set_id, S.slot[i], real, filled, S.w[i], blk, s_c + jq, s_q + jq,
                                         FULL ? 8 : nq, kstep, alpha);
        if (o.ev & 0xffffu) {
          S.w[i] = o.w;
          S.filled = (o.ev & 0x10000u) ? (S.filled | (1u << i)) : (S.filled & ~(1u << i));
          uint32_t esc = o.ev & 0xffu, ref = (o.ev >> 8) & 0xffu;
          if (esc && P.a.fates)  // the last escape of the block
            P.a.fates[st.slot_offset + S.slot[i]] = (int32_t)(kstep + (31 - __clz(esc)));
          while (esc) {
            const int t = __ffs(esc) - 1;
            esc &= esc - 1;
            atomicAdd(&s_lum[bin_of_step(bin, to_flush, spb, t)], 1u);
            ecnt += 1ull << (8 * t);
          }
          while (ref) {
            const int t = __ffs(ref) - 1;
            ref &= ref - 1;
            rcnt += 1ull << (8 * t);
          }
        }
      }
    }
  }
  uint64_t ecum = 0, rcum = 0;  // byte t: events in steps 0..t
  if (ecnt | rcnt) {
    ecum = ecnt * 0x0101010101010101ull;
    rcum = rcnt * 0x0101010101010101ull;
  }
  flush_block_bins(FULL ? 8 : nq, s_alive, bin, to_flush, spb, seg_left, [&](int t) {
    return alive0 + (uint32_t)((rcum >> (8 * t)) & 0xffu) - (uint32_t)((ecum >> (8 * t)) & 0xffu);
  });
}

// One segment of one work item (FP32).  s_bm holds the per-block bounds of
// the prefilter: cm at [0, kBlocksPerChunk), qm after it.
template <int BLOCK, int EPT, bool FILL>
__device__ __forceinline__ void segment_f32(const KParams& P, const mcl_set& st, const mcl_segment& sg,
                                            SlotState<EPT>& S, const float2* tab, float* s_c, float* s_q,
                                            float* s_bm, uint32_t* s_lum, uint32_t* s_alive, uint32_t bbase,
                                            int64_t kglob, float alpha) {
  const int spb = sg.steps_per_bin;
  int bin = sg.bin_offset;
  int to_flush = min(spb, sg.n_steps);
  float* s_cm = s_bm;
  float* s_qm = s_bm + kBlocksPerChunk;
  for (int j0 = 0; j0 < sg.n_steps; j0 += kChunk) {
    const int nj = min(kChunk, sg.n_steps - j0);
    __syncthreads();
    // The trip count is uniform, so whole warps take part in the shuffles
    // (a warp's lanes 8k..8k+7 hold one 8-step block).
    for (int j = 0; j < nj; j += BLOCK) {
      const int jj = j + (int)threadIdx.x;
      float c16 = 0.0f, q16 = 0.0f;
      if (jj < nj) {
        const float2 cq = tab[j0 + jj];
        c16 = __fmul_rn(cq.x, 65536.0f);
        s_c[jj] = c16;
        if (FILL) {
          q16 = __fmul_rn(cq.y, 65536.0f);
          s_q[jj] = q16;
        }
      }
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        c16 = fmaxf(c16, __shfl_xor_sync(0xffffffffu, c16, o));
        if (FILL) q16 = fmaxf(q16, __shfl_xor_sync(0xffffffffu, q16, o));
      }
      if ((jj & 7) == 0 && jj < nj) {
        s_cm[jj >> 3] = __fmul_ru(c16, kCmScale);
        if (FILL) s_qm[jj >> 3] = __fmul_ru(q16, kCmScale);
      }
    }
    __syncthreads();
    int jq = 0;
    for (; jq + 8 <= nj; jq += 8) {
      const uint32_t blk = bbase + (uint32_t)((j0 + jq) >> 3);
      if (FILL)
        block_fill<EPT, true>(P, st, S, blk, s_c, s_q, s_cm, s_qm, jq, 8, kglob + j0 + jq, s_lum, s_alive, bin,
                              to_flush, spb, sg.n_steps - (j0 + jq), alpha);
      else
        block_nofill<EPT, true>(P, st, S, blk, s_c, s_cm, jq, 8, kglob + j0 + jq, s_lum, s_alive, bin, to_flush,
                                spb, sg.n_steps - (j0 + jq));
    }
    if (jq < nj) {  // the segment's last, partial Philox block
      const uint32_t blk = bbase + (uint32_t)((j0 + jq) >> 3);
      if (FILL)
        block_fill<EPT, false>(P, st, S, blk, s_c, s_q, s_cm, s_qm, jq, nj - jq, kglob + j0 + jq, s_lum, s_alive,
                               bin, to_flush, spb, sg.n_steps - (j0 + jq), alpha);
      else
        block_nofill<EPT, false>(P, st, S, blk, s_c, s_cm, jq, nj - jq, kglob + j0 + jq, s_lum, s_alive, bin,
                                 to_flush, spb, sg.n_steps - (j0 + jq));
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 / Philox kernel
// ---------------------------------------------------------------------------
// FILLS = false builds the kernel without the filling path (fewer
// registers, more resident warps) for batches whose segments never fill.
template <int BLOCK, int EPT, bool FILLS>
__device__ __forceinline__ void kb_f32_body(const KParams& P) {
  extern __shared__ __align__(16) unsigned char smem[];
  const mcl_b_args& a = P.a;
  float* s_c = reinterpret_cast<float*>(smem);
  float* s_q = s_c + kChunk;
  uint32_t* s_lum = reinterpret_cast<uint32_t*>(s_q + kChunk);
  const int copies = a.bin_copies;  // 1, 2 or 4 (the launcher normalises it)
  uint32_t* s_alive = a.alive ? s_lum + copies * a.max_bins : nullptr;
  uint32_t* s_lum_w = s_lum + ((int)(threadIdx.x >> 5) % copies) * a.max_bins;  // this warp's copy
  __shared__ int s_item;
  __shared__ float s_bm[2 * kBlocksPerChunk];

  Header* hdr = reinterpret_cast<Header*>(a.workspace);
  const float2* table = reinterpret_cast<const float2*>(reinterpret_cast<const char*>(a.workspace) + kHeaderBytes);
  const int tid = threadIdx.x;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(&hdr->ticket, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= a.n_items) break;
    const mcl_item item = a.items[it];
    if (checked_item(a, item) < 0) {  // host validation makes this unreachable
      __syncthreads();
      continue;
    }
    const mcl_set st = a.sets[item.set];
    zero_bins<BLOCK>(s_lum, s_alive, st.n_bins, copies, a.max_bins);

    const float alpha = (float)st.alpha;
    SlotState<EPT> S;
    S.filled = 0;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = item.slot_begin + i * BLOCK + tid;
      S.slot[i] = (uint32_t)e;
      S.w[i] = 0.0f;
      if (e < st.n_filled) {
        const uint4 r0 = philox_ks(0u, (uint32_t)e, st.set_id, kTagInit, P);
        S.w[i] = refill_w(r0.x, alpha);
        S.filled |= 1u << i;
      }
    }

    int64_t kglob = 0;  // global step of the set (fates, refill counters)
    uint32_t bbase = 0;  // Philox blocks used by earlier segments
    const float2* tab = table + st.step_offset;
    for (int g = 0; g < st.seg_count; ++g) {
      const mcl_segment sg = a.segs[st.seg_begin + g];
      if (sg.fill_rate > 0.0) {
        if constexpr (FILLS)
          segment_f32<BLOCK, EPT, true>(P, st, sg, S, tab + kglob, s_c, s_q, s_bm, s_lum_w, s_alive, bbase, kglob,
                                        alpha);
        else  // the caller promised no filling segment (mcl_b_args.no_fill)
          report(a.status, MCL_EINVAL);
      } else
        segment_f32<BLOCK, EPT, false>(P, st, sg, S, tab + kglob, s_c, s_q, s_bm, s_lum_w, s_alive, bbase, kglob,
                                       alpha);
      bbase += (uint32_t)((sg.n_steps + 7) >> 3);
      kglob += sg.n_steps;
    }
    __syncthreads();
    flush_bins<BLOCK>(a, st, s_lum, s_alive, copies, a.max_bins);
    __syncthreads();
  }
}

template <int BLOCK, int EPT, bool FILLS>
__global__ void __launch_bounds__(BLOCK) kb_f32(const KParams P) {
  kb_f32_body<BLOCK, EPT, FILLS>(P);
}

// The same kernel compiled for MINB resident CTAs per SM (fewer registers).
template <int BLOCK, int EPT, int MINB, bool FILLS>
__global__ void __launch_bounds__(BLOCK, MINB) kb_f32_occ(const KParams P) {
  kb_f32_body<BLOCK, EPT, FILLS>(P);
}

// ---------------------------------------------------------------------------
// FP64 kernel (Philox or injected uniforms): the oracle-parity mode
// ---------------------------------------------------------------------------
template <int BLOCK, int EPT, bool INJ>
__global__ void __launch_bounds__(BLOCK) kb_f64(const KParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  const mcl_b_args& a = P.a;
  double* s_c = reinterpret_cast<double*>(smem);
  double* s_q = s_c + kChunk;
  uint32_t* s_lum = reinterpret_cast<uint32_t*>(s_q + kChunk);
  uint32_t* s_alive = a.alive ? s_lum + a.max_bins : nullptr;
  __shared__ int s_item;

  Header* hdr = reinterpret_cast<Header*>(a.workspace);
  const double2* table = reinterpret_cast<const double2*>(reinterpret_cast<const char*>(a.workspace) + kHeaderBytes);
  const int tid = threadIdx.x;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(&hdr->ticket, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= a.n_items) break;
    const mcl_item item = a.items[it];
    if (checked_item(a, item) < 0) {
      __syncthreads();
      continue;
    }
    const mcl_set st = a.sets[item.set];
    zero_bins<BLOCK>(s_lum, s_alive, st.n_bins);

    double w[EPT];
    float wf[EPT];  // w rounded up to FP32 (the prefilter's bound)
    uint32_t slot[EPT];
    uint32_t filled = 0;
    const int64_t n = st.n_slots;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = item.slot_begin + i * BLOCK + tid;
      slot[i] = (uint32_t)e;
      w[i] = 0.0;
      wf[i] = 0.0f;
      if (e < st.n_slots) {
        double u;
        if (INJ) {
          u = a.uniforms[st.u_offset + e];
        } else {
          const uint4 r = philox_ks(0u, (uint32_t)e, st.set_id, kTagInit, P);
          u = u53(r.x, r.y);
        }
        w[i] = exp(__dmul_rn(-st.alpha, r_prime_d(u)));
        wf[i] = __double2float_ru(w[i]);
        if (e < st.n_filled) filled |= 1u << i;
      }
    }

    int64_t kglob = 0;
    uint32_t pbase = 0;
    const double2* tab = table + st.step_offset;
    for (int g = 0; g < st.seg_count; ++g) {
      const mcl_segment sg = a.segs[st.seg_begin + g];
      const bool fill_on = sg.fill_rate > 0.0;
      const int spb = sg.steps_per_bin;
      int to_flush = min(spb, sg.n_steps);
      int bin = sg.bin_offset;
      for (int j0 = 0; j0 < sg.n_steps; j0 += kChunk) {
        const int nj = min(kChunk, sg.n_steps - j0);
        __syncthreads();
        for (int jj = tid; jj < nj; jj += BLOCK) {
          const double2 cq = tab[kglob + j0 + jj];
          s_c[jj] = cq.x;
          s_q[jj] = cq.y;
        }
        __syncthreads();
        uint4 r[EPT];
        for (int jj = 0; jj < nj; ++jj) {
          const int j = j0 + jj;
          const int64_t k = kglob + j;
          if (!INJ && (j & 1) == 0) {
#pragma unroll
            for (int i = 0; i < EPT; ++i)
              r[i] = philox_ks(pbase + (uint32_t)(j >> 1), slot[i], st.set_id, kTagStep, P);
          }
          const double c = s_c[jj];
          const double qv = s_q[jj];
          // FP32 prefilter (GB300 runs FP64 at ~1/64 of the FP32 rate): uf <= u
          // (the top 24 bits of the 53-bit uniform, or the injected double
          // rounded down) and xf >= p (c and w rounded up, product rounded up,
          // times 1 + 2^-20 for expm1's last bit, as p = 1 - e^{-cw} <= cw);
          // uf > xf proves u >= p, so the exact FP64 test runs only otherwise.
          const float cf = __fmul_ru(__double2float_ru(c), 1.0f + 0x1p-20f);
          const float qf = __double2float_ru(qv);
#pragma unroll
          for (int i = 0; i < EPT; ++i) {
            if (slot[i] >= (uint32_t)st.n_slots) continue;
            const bool full = (filled >> i) & 1u;
            if (!full && !(!INJ && fill_on)) continue;
            float uf;
            double uinj = 0.0;
            if (INJ) {
              uinj = a.uniforms[st.u_offset + n + k * n + slot[i]];
              uf = __double2float_rd(uinj);
            } else {
              uf = __fmul_rn(__uint2float_rz(((j & 1) ? r[i].z : r[i].x) >> 8), 0x1p-24f);
            }
            if (uf > (full ? __fmul_ru(cf, wf[i]) : qf)) continue;
            const double u = INJ ? uinj : ((j & 1) ? u53(r[i].z, r[i].w) : u53(r[i].x, r[i].y));
            if (full) {
              const double p = -expm1(__dmul_rn(-c, w[i]));
              if (u < p) {
                filled &= ~(1u << i);
                atomicAdd(&s_lum[bin], 1u);
                if (a.fates) a.fates[st.slot_offset + slot[i]] = (int32_t)k;
              }
            } else if (u < qv) {
              const uint4 rr = philox_ks((uint32_t)k, slot[i], st.set_id, kTagRefill, P);
              w[i] = exp(__dmul_rn(-st.alpha, r_prime_d(u53(rr.x, rr.y))));
              wf[i] = __double2float_ru(w[i]);
              filled |= 1u << i;
            }
          }
          if (--to_flush == 0) {
            if (s_alive) warp_flush((uint32_t)__popc(filled), &s_alive[bin]);
            ++bin;
            to_flush = min(spb, sg.n_steps - j - 1);
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

using KernelFn = void (*)(const KParams);

}  // namespace

// Kernel getters, one per translation unit.  `occupancy` 0 selects the
// default build; another value selects the build compiled for that many
// resident CTAs per SM (fewer registers), where one exists.  `fills` false
// selects the build without the filling path.  nullptr = no such kernel.
KernelFn b_f32_128_e2(int occupancy, bool fills);
KernelFn b_f32_128_e4(int occupancy, bool fills);
KernelFn b_f32_128_e8(int occupancy, bool fills);
KernelFn b_f32_256_e2(int occupancy, bool fills);
KernelFn b_f32_256_e4(int occupancy, bool fills);
KernelFn b_f32_256_e8(int occupancy, bool fills);
KernelFn b_pick_f64(int block, int ept, bool injected);

}  // namespace mcl

