/*
 * mclum.h -- C ABI of the GB300 (sm_103a) Monte Carlo trap-kinetics library.
 *
 * Plain C: pointers, sizes and POD structs only; no CUDA or torch types.
 * Device pointers are caller-owned (e.g. torch tensors); streams are passed as
 * `void*` holding a cudaStream_t (NULL = the legacy default stream).  Every
 * entry point returns MCL_OK (0) or a negative MCL_E* code; kernels report
 * problems they detect on the device through a caller-provided int32 status
 * word (0 = fine), never by trapping.
 *
 * The reference is a Python program (no native code, no FFI).  Each entry
 * point below replaces one piece of its simulation call stack, cited by file
 * and line in the reference project:
 *
 *   mcl_k_*  the event-driven kinetics loop of simulate()
 *            src/class/simulate.py:36-92 over TLTrapSim / Box / Physics
 *            (src/class/tl_trap_lab.py:27-60, src/class/engine.py:44-188).
 *   mcl_b_*  the fixed-dt Bernoulli kinetics over ragged batches of parameter
 *            sets (the dilute limit of the same physics; no single reference
 *            function -- it replaces the per-set loop that
 *            src/class/optimizer.py:68-84 and simulate.py:36-48 run serially).
 *   mcl_graph_*  CUDA-graph capture/replay of a packed batch (no reference
 *            counterpart; the reference re-enters Python per step).
 */
#ifndef MCLUM_H
#define MCLUM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCL_ABI_VERSION 3

/* ---- return / status codes ------------------------------------------- */
#define MCL_OK 0
#define MCL_EINVAL (-1)     /* bad argument (host-side validation)          */
#define MCL_ECAPACITY (-2)  /* an output table or on-chip buffer too small   */
#define MCL_EBUDGET (-3)    /* a step / iteration budget ran out             */
#define MCL_ECUDA (-4)      /* a CUDA runtime call failed                    */
#define MCL_ENODEV (-5)     /* no usable sm_103 device                        */
#define MCL_ENOHOLE (-6)    /* a nearest-centre search over zero centres      */
#define MCL_EOVERFLOW (-7)  /* more steps than rows in an output table        */

/* ---- precision / RNG selectors ---------------------------------------- */
#define MCL_FP32 0          /* FP32 arithmetic, 32-bit Philox uniforms        */
#define MCL_FP64 1          /* FP64 arithmetic, 53-bit Philox uniforms        */
#define MCL_RNG_PHILOX 0    /* counter-based Philox4x32-10 keyed by seed      */
#define MCL_RNG_INJECTED 1  /* caller-supplied uniforms (FP64 only)           */
#define MCL_RNG_MT19937 2   /* numpy's legacy RandomState stream (MT19937)    */

/* ---- Bernoulli-mode schedule ------------------------------------------ */
#define MCL_SEG_THERMAL 1   /* add s*exp(-E/(k_b*T)) to the segment's rate   */

/* One phase of a set's schedule (TL ramp, isothermal hold, irradiation,
 * fading, optical stimulation).  Step j of the segment has length
 * dt*g^j (g = dt_growth), starts at time t_j = sum of earlier lengths, at
 * temperature T0 + beta*t_j, with escape rate
 *     A_j = rate_const + [flags&THERMAL] s*exp(-E/(k_b*T))
 * scaled per trap by exp(-alpha*r'), and fill probability
 * 1-exp(-dt_j*fill_rate) for empty traps.  Events of step j count into bin
 * bin_offset + j/steps_per_bin of the set.                          64 B */
typedef struct mcl_segment {
  int32_t n_steps;
  int32_t steps_per_bin;
  int32_t bin_offset;
  int32_t flags;
  double dt;
  double dt_growth;
  double T0;
  double beta;
  double rate_const;
  double fill_rate;
} mcl_segment;

/* One parameter set: n_slots traps, the first n_filled of them occupied at
 * the start, segments [seg_begin, seg_begin+seg_count).  step_offset is the
 * set's first entry in the per-step rate table kept in the workspace; sets
 * must be laid out back to back (step_offset = sum of earlier total_steps). 96 B */
typedef struct mcl_set {
  int32_t n_slots;
  int32_t n_filled;
  int32_t seg_begin;
  int32_t seg_count;
  int32_t n_bins;
  uint32_t set_id;      /* Philox counter word 2 (the set's identity)        */
  int64_t bin_offset;   /* first bin of this set in lum[] / alive[]          */
  int64_t slot_offset;  /* first slot of this set in fates[]                  */
  int64_t u_offset;     /* injected mode: first uniform of this set           */
  int64_t total_steps;  /* sum of the segments' n_steps                       */
  int64_t step_offset;  /* first step of this set in the rate table           */
  double E;             /* trap depth, eV                                     */
  double s;             /* frequency factor, 1/s                              */
  double alpha;         /* tunnelling coefficient on the dimensionless r'     */
  double k_b;           /* Boltzmann constant, eV/K                            */
} mcl_set;

/* A work item: slots [slot_begin, slot_begin + slots_per_item) of one set. */
typedef struct mcl_item {
  int32_t set;
  int32_t slot_begin;
} mcl_item;

/* Arguments of one Bernoulli launch (all pointers are device pointers).
 * The kernels check every set against the sizes declared here before they
 * touch a buffer: segments within n_segs, the set's steps (the sum of its
 * segments' n_steps) within table_steps from step_offset, bins within
 * n_bins_total and max_bins, slots within n_slots_total, injected uniforms
 * within n_uniforms, and every item's set and first slot.  A set or item
 * that fails writes MCL_ECAPACITY (MCL_EINVAL for a bad item) to the status
 * word and is skipped: nothing is read or written outside the buffers. */
typedef struct mcl_b_args {
  const mcl_set* sets;
  const mcl_segment* segs;
  const mcl_item* items;
  uint32_t* lum;           /* [n_bins_total] recombinations per bin           */
  uint32_t* alive;         /* [n_bins_total] filled traps at bin end, or NULL */
  int32_t* fates;          /* [n_slots_total] step of last recombination, or NULL */
  const double* uniforms;  /* injected mode only                              */
  int32_t* status;         /* [1] device status word                          */
  void* workspace;         /* device scratch: ticket + per-step rate table      */
  int64_t workspace_bytes; /* >= mcl_b_workspace_size(sets, n_sets, precision) */
  int64_t table_steps;     /* sum of total_steps over all sets (table rows)    */
  int64_t n_bins_total;
  int64_t n_slots_total;
  int64_t n_uniforms;      /* injected mode: elements of uniforms[]            */
  uint64_t seed;
  int32_t n_sets;
  int32_t n_segs;
  int32_t n_items;
  int32_t slots_per_item;  /* block * ept                                      */
  int32_t max_bins;        /* largest n_bins of any set                        */
  int32_t precision;       /* MCL_FP32 | MCL_FP64                               */
  int32_t rng;             /* MCL_RNG_PHILOX | MCL_RNG_INJECTED                 */
  int32_t block;           /* threads per CTA: 128, 256 or 512                  */
  int32_t ept;             /* slots per thread: 1, 2, 4 or 8                    */
  int32_t grid;            /* persistent CTAs; 0 = SM count x occupancy         */
  int32_t zero_outputs;    /* 1: clear lum/alive/fates/status before the launch */
  int32_t occupancy;       /* FP32 build: 0 = default; else resident CTAs per
                              SM the build targets (fewer registers): 4 at
                              block 256 / 8 at block 128 with ept 2, 3 at
                              block 256 / 6 at block 128 with ept 4, 2 at
                              block 256 / 4 at block 128 with ept 8           */
  int32_t no_fill;         /* 1: no segment has fill_rate > 0; the FP32 launch
                              then uses its build without the filling path
                              (fewer registers), and a filling segment sets
                              MCL_EINVAL in the status word                   */
  int32_t bin_copies;      /* FP32: copies of the set's bins each CTA keeps in
                              shared memory (1, 2 or 4; 0 = 1): warp w adds its
                              events to copy w % bin_copies, which spreads the
                              shared-memory atomics of hot bins; the copies are
                              summed when the CTA flushes.  Results do not
                              depend on it.  FP64 keeps one copy.            */
  int32_t reserved;
} mcl_b_args;

/* ---- reference-kinetics (event-driven) mode ----------------------------- */
#define MCL_LOOP_SIMULATE 0  /* simulate.py:51-92: waits, fill wait, dt cap, one event      */
#define MCL_LOOP_LAB_TL 1    /* TL_lab (tl_trap_lab.py:90-108): heat until `duration`       */
#define MCL_LOOP_LAB_ISO 2   /* ISO_lab (tl_trap_lab.py:147-172): until the last obs time  */
/* One simulation: one (run, sim) pair of src/class/simulate.py:36-92, with
 * the run's parameters already read the way simulate.py:39-45 and
 * tl_trap_lab.py:27-43 read them (box sides computed on the host in FP64).  */
typedef struct mcl_k_sim {
  double alpha, b, s, E_cb, E_loc_1, E_loc_2, D0, Retrap, k_b;
  double dose_rate;     /* simulate.py:42 reads physics_fp.dose_rate         */
  double T_start;       /* degC                                               */
  double T_rate;        /* K/s                                                */
  double dt_cap;        /* max_dt / T_rate, or 1e20 when T_rate == 0          */
  double duration;      /* s                                                  */
  double N_e;           /* trap count (electron_ratio = n / N_e)              */
  double L, W, H;       /* core box sides                                     */
  double Lb, Wb, Hb;    /* boundary box sides (x boundary_factor)             */
  int32_t e0;           /* initial electrons int(N_e * e_ratio_start)         */
  int32_t n_h0;         /* initial holes int(holes * bf^3)                    */
  int32_t e_cap;        /* electron capacity (e0 + pair creations allowed)   */
  int32_t h_cap;        /* hole capacity                                      */
  int32_t steps;        /* rows of the output tables                          */
  uint32_t stream_id;   /* Philox stream of this simulation                   */
  int64_t out_offset;   /* first row of this simulation in the tables         */
  int64_t u_offset;     /* injected: first uniform (sequential mode: sim 0 only; */
  int64_t u_count;      /*   later sims continue the stream); uniforms available */
  int64_t ws_offset;    /* bytes into the workspace (arrays in global memory) */
  int64_t ev_offset;    /* first event slot in events[] (4 int32 per event)   */
  int64_t ev_cap;       /* event slots of this simulation                     */
  int32_t loop;         /* MCL_LOOP_*                                         */
  int32_t n_obs;        /* MCL_LOOP_LAB_ISO: observation times                */
  int64_t obs_offset;   /* first observation in obs_time[] / obs_ratio[]      */
} mcl_k_sim;

typedef struct mcl_k_args {
  const mcl_k_sim* sims;
  double* x_ax;            /* [rows] time after each step, zero padded        */
  double* lum;             /* [rows] 1.0 on recombination steps               */
  double* ratio;           /* [rows] electrons / N_e after each step          */
  int32_t* events;         /* [4 * slots] step, kind(0 pair created, 1 recombination), e, h; or NULL */
  int32_t* n_events;       /* [n_sims]                                         */
  int32_t* n_steps;        /* [n_sims] steps taken                             */
  int64_t* draws;          /* [n_sims] uniforms consumed                       */
  int32_t* status;         /* [n_sims] 0 or a negative MCL_E* code            */
  const double* uniforms;  /* MCL_RNG_INJECTED                                 */
  uint32_t* mt_state;      /* MCL_RNG_MT19937: [625] key words + position, in/out */
  const double* obs_time;  /* MCL_LOOP_LAB_ISO: observation times (s), ascending */
  double* obs_ratio;       /* MCL_LOOP_LAB_ISO: electrons / N_e at each observation */
  void* workspace;         /* per-simulation regions at ws_offset (FP64 hole
                              coordinates; all arrays when they exceed shared
                              memory); >= workspace_bytes of mcl_k_validate   */
  int64_t workspace_bytes;
  uint64_t seed;           /* MCL_RNG_PHILOX key                               */
  int32_t n_sims;
  int32_t rng;
  int32_t sequential;      /* 1: one CTA runs the simulations in order on one stream */
  int32_t block;           /* 256 or 512                                       */
  int32_t e_cap_max;       /* largest e_cap / h_cap (from mcl_k_validate)      */
  int32_t h_cap_max;
  int32_t arrays_in_smem;  /* 1: per-electron arrays and FP32 hole copies in shared memory (from mcl_k_validate) */
  int32_t reserved;
} mcl_k_args;

/* ---- library ------------------------------------------------------------ */
int mcl_abi_version(void);
const char* mcl_status_string(int code);
/* Text of the last CUDA error seen by this thread's calls ("" if none). */
const char* mcl_last_error(void);
/* sizeof(mcl_segment), sizeof(mcl_set), sizeof(mcl_item), sizeof(mcl_b_args),
 * sizeof(mcl_k_sim), sizeof(mcl_k_args), written to out[0..5], so bindings
 * can check their struct layouts. */
int mcl_struct_sizes(size_t* out);
/* SM count and compute capability of the current device. */
int mcl_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);

/* ---- Bernoulli mode ----------------------------------------------------- */
/* Host-side validation of a packed batch (host arrays). */
int mcl_b_validate(const mcl_set* sets, int32_t n_sets, const mcl_segment* segs,
                   int32_t n_segs, int64_t n_bins_total, int64_t n_slots_total,
                   int32_t precision, int32_t rng, int64_t n_uniforms);
/* Ragged packer: split every set into items of slots_per_item slots, ordered
 * longest-first (steps x slots) for the persistent ticket scheduler.  Writes
 * at most items_cap items and returns the item count (or a negative code). */
int64_t mcl_b_pack_items(const mcl_set* sets, int32_t n_sets, int32_t slots_per_item,
                         mcl_item* items_out, int64_t items_cap);
/* Bytes of device workspace one launch needs (host set array): a 256-byte
 * header (the work ticket) plus one table entry per step of every set
 * (c_j and q_j: 8 bytes in FP32 mode, 16 in FP64 mode). */
size_t mcl_b_workspace_size(const mcl_set* sets, int32_t n_sets, int32_t precision);
/* Largest block/ept-independent dynamic shared memory (bytes) for max_bins. */
size_t mcl_b_smem_bytes(int32_t max_bins, int32_t precision, int32_t want_alive);
/* Launch on `stream` (stream-ordered, no host synchronisation). */
int mcl_b_run(const mcl_b_args* args, void* stream);

/* Size of the library's own scratch array used by mcl_b_run_static. */
#define MCL_B_STATIC_SCRATCH_BYTES (16 * 1024 * 1024)

/* mcl_b_run without a caller-provided workspace (no counterpart in the
 * reference).  For callers that may not allocate device memory -- e.g. a host
 * application or plugin framework that owns all GPU memory through its own
 * pool and forbids cudaMalloc, which can stall on work already queued.  The
 * caller passes inputs and outputs exactly as for mcl_b_run; args->workspace
 * and workspace_bytes are ignored.  Scratch comes from a static device array
 * of MCL_B_STATIC_SCRATCH_BYTES held by every GPU that loads the library, so
 * table_steps may be at most (MCL_B_STATIC_SCRATCH_BYTES - 256) / 8 (FP32) or
 * / 16 (FP64); larger batches return MCL_ECAPACITY without launching.  The
 * first call on a device looks up the array's device address (once per
 * device, with that device current) and should come before any stream
 * capture.  Calls share the array: ones that overlap on the GPU race, so
 * issue them on one stream.  Allocates nothing. */
int mcl_b_run_static(const mcl_b_args* args, void* stream);

/* Roofline microbenchmark (no reference counterpart): `grid` CTAs of 256
 * threads each generate iters x 4 Philox4x32-10 blocks with the Bernoulli
 * kernel's counter layout and write one folded word per thread to
 * sink[grid*256].  Blocks/s of this kernel x 8 bounds FP32 trials/s. */
int mcl_bench_philox(uint32_t* sink, int32_t grid, int32_t iters, uint64_t seed, void* stream);

/* ---- reference-kinetics mode ----------------------------------------------- */
/* Host validation; also reports whether the per-electron arrays of the
 * largest simulation fit in shared memory (*arrays_in_smem), the workspace
 * bytes needed (*workspace_bytes: the end of the last region, each of
 * mcl_k_region_bytes at its ws_offset) and the largest capacities, all to be
 * copied into mcl_k_args. */
int mcl_k_validate(const mcl_k_sim* sims, int32_t n_sims, int32_t rng, int32_t block,
                   int64_t n_uniforms, int32_t* arrays_in_smem, int64_t* workspace_bytes,
                   int32_t* e_cap_max, int32_t* h_cap_max);
/* Launch (stream-ordered).  Per-simulation problems land in status[]:
 * MCL_ECAPACITY when the output table is too short (the reference raises
 * IndexError, simulate.py:64) or a capacity is exceeded, MCL_EBUDGET when an
 * injected stream runs out, MCL_ENOHOLE for a nearest search over no holes. */
int mcl_k_run(const mcl_k_args* args, void* stream);
/* Bytes of simulation i's global-memory region at sims[i].ws_offset (the FP64
 * hole coordinates, plus the per-electron arrays unless they live in shared
 * memory); offsets must be multiples of 16.  mcl_k_arrays_fit_smem tells
 * whether the per-electron arrays of the largest simulation fit in shared
 * memory, which mcl_k_validate reports as arrays_in_smem. */
int64_t mcl_k_region_bytes(int32_t e_cap, int32_t h_cap, int32_t arrays_in_smem);
int32_t mcl_k_arrays_fit_smem(int32_t e_cap_max, int32_t h_cap_max);

/* ---- step-level operations of the event-driven loop ------------------------ */
/* For callers that drive the loop one step at a time through the reference's
 * TLTrapSim / Box surface (src/class/simulate.py:51-92); mcl_k_run keeps the
 * whole loop on the device and is the throughput path.  Coordinates are
 * device arrays [n][3] (FP64, row-major).
 * mcl_k_box_nearest replaces Box._rebuild / the incremental searches of
 * Box.add_electron and Box.remove_pair (src/class/engine.py:113-119, 147-152,
 * 170-175): for each electron index in rows[0..n_rows) (all n_e electrons
 * when rows is NULL and n_rows == n_e), the minimum over the n_h holes of
 * sqrt((dx*dx + dy*dy) + dz*dz), dx = e.x - h.x (numpy's np.linalg.norm
 * association, no contraction) into min_d[row] and its first argmin into
 * nearest[row]; a NaN distance counts as the minimum, as in numpy; row
 * indices outside [0, n_e) are skipped.  n_h == 0
 * with n_rows > 0 returns MCL_ENOHOLE (numpy raises ValueError there). */
int mcl_k_box_nearest(const double* electrons, int32_t n_e, const double* holes, int32_t n_h,
                      const int32_t* rows, int32_t n_rows, double* min_d, int64_t* nearest, void* stream);
/* TLTrapSim._update_lifetimes (src/class/tl_trap_lab.py:48-51 over
 * src/class/engine.py:65-77) given its uniforms: E_loc = E_loc_2 if
 * u_retrap[i] < Retrap else E_loc_1; lifetime[i] = 1 / (s exp(-E_cb/(k_b T))
 * + b exp(-E_loc/(k_b T) - alpha min_d[i])); wait[i] = lifetime[i] *
 * (-log(1 - u_wait[i])) (numpy's legacy exponential).  The physics fields of
 * *phys (a host struct) are read; the rest of it is ignored. */
int mcl_k_box_waits(const mcl_k_sim* phys, double T, const double* min_d, const double* u_retrap,
                    const double* u_wait, int32_t n, double* lifetime, double* wait, void* stream);
/* Box.distances (src/class/engine.py:180-183): out[i*n_h + j] = the distance
 * of electron i to hole j, as mcl_k_box_nearest evaluates it. */
int mcl_k_box_distances(const double* electrons, int32_t n_e, const double* holes, int32_t n_h, double* out,
                        void* stream);

/* ---- surrogate network (no counterpart in the reference) ------------------ */
/* The reference fits parameters by running the Monte Carlo for every
 * candidate (src/class/optimizer.py:93-111); these kernels train and run a
 * small MLP (6 -> 256 -> 256 -> 256 -> 256 -> 200, GELU) that proposes
 * candidates instead.  bf16 tensors are passed as void* (2-byte elements).  */
#define MCL_EPI_F32 0        /* C = A B^T                                      */
#define MCL_EPI_BIAS 1       /* C = A B^T + bias                               */
#define MCL_EPI_BIAS_GELU 2  /* C = A B^T + bias; Y = gelu(C) (bf16), Yt = Y^T */
/* C[M][N] (fp32) = sum_k A[m][k] B[n][k] with BF16 operands (k contiguous),
 * FP32 accumulation on the tensor cores and a fused epilogue.  M, N multiples
 * of 64, K of 32; leading dimensions in elements, multiples of 8. */
int mcl_gemm_nt(int32_t epilogue, int32_t M, int32_t N, int32_t K, const void* A, int32_t lda,
                const void* B, int32_t ldb, const float* bias, float* C, int32_t ldc, void* Y,
                int32_t ldy, void* Yt, int32_t ldyt, void* stream);
/* The same GEMM on the tcgen05 tensor cores (accumulator in tensor memory):
 * M multiple of 128, N of 64, K of 64.  *err is set to 1 if a completion wait
 * times out (the kernel then skips its epilogue and still frees its tensor
 * memory). */
int mcl_gemm_nt_tc(int32_t epilogue, int32_t M, int32_t N, int32_t K, const void* A, int32_t lda,
                   const void* B, int32_t ldb, const float* bias, float* C, int32_t ldc, void* Y,
                   int32_t ldy, void* Yt, int32_t ldyt, int32_t* err, void* stream);
/* The whole network in one persistent launch: a thread-block cluster of
 * `split` CTAs (1, 2 or 4) per 128-row tile of the batch keeps the tile's
 * activations in shared memory (each CTA a full copy, which the CTAs write
 * into each other's shared memory) and its accumulator in tensor memory from
 * layer to layer; CTA q computes output columns [q 256/split, (q+1)
 * 256/split) of every layer (tcgen05 MMAs with M 128, N 256/split, K 16),
 * copying its slice of the next weights from L2 while the current epilogue
 * runs.  split 0 lets the library pick the one with the fewest waves for
 * this batch on this device.  Forward: bias + GELU epilogues, the last
 * layer's outputs to `out`.  Training adds, in the same launch and per
 * tile, the loss and its gradient (mcl_mse_loss's), then the input-gradient
 * chain dY_{l-1} = dZ_l W_l with dZ = dY * GELU'(pre-activation) fused into
 * the epilogues (mcl_act_backward's), writing what the weight gradients
 * need (the transposed activations and dZ) and adding the bias gradients.
 * The weight gradients then take one mcl_gemm_nt_tc_grouped launch.  The
 * network shape is fixed: 6 inputs (padded to 64), four hidden layers of
 * 256, 200 outputs (padded to 256). */
typedef struct mcl_mlp_layer {
  const void* W;        /* bf16 [256][k] (k = 64 for layer 0, else 256)        */
  const void* Wt;       /* bf16 [k][256] (training, layers 1..4)               */
  const float* bias;    /* [256]                                               */
  float* grad_b;        /* [256] += bias gradient (training; caller clears)    */
  void* dZt;            /* bf16 [256][batch] d loss / d pre-activation, transposed (training) */
  float* gelu_grad;     /* batch x 256 floats: GELU' of the pre-activation, in a layout
                           private to the kernel (training scratch, layers 0..3)  */
  void* Yt;             /* bf16 [256][batch] activation, transposed (training, layers 0..3) */
} mcl_mlp_layer;

typedef struct mcl_mlp_args {
  mcl_mlp_layer layer[5];
  const float* x;       /* [*][6] standardized inputs                           */
  const int64_t* idx;   /* [batch] rows of x and target to use, or NULL (rows 0..batch-1) */
  const float* target;  /* [*][target_ld], 200 used per row (training)          */
  float* out;           /* [batch][256] last layer's outputs, or NULL           */
  void* xt;             /* bf16 [64][batch] transposed inputs (training; rows 6..63 stay zero) */
  float* loss;          /* [1] += squared error over the 200 outputs (training; caller clears) */
  int32_t* err;         /* [1] set to 1 if a completion wait timed out          */
  float loss_scale;     /* loss gradient 2 (out - target) * loss_scale          */
  int32_t batch;        /* multiple of 128                                      */
  int32_t training;
  int32_t target_ld;    /* elements between target rows (>= 200)               */
  int32_t split;        /* CTAs per 128-row tile: 1, 2, 4, or 0 = pick          */
  int32_t reserved;
} mcl_mlp_args;
int mcl_mlp_fused(const mcl_mlp_args* args, void* stream);

/* Several plain GEMMs C = A B^T (fp32 output, as mcl_gemm_nt_tc with
 * MCL_EPI_F32) in ONE launch, each with its K split over a thread-block
 * cluster of `splits` CTAs (1, 2, 4 or 8; K a multiple of 64 * splits, and
 * at least two 64-wide slabs per CTA when split): the surrogate's weight
 * gradients of all layers at once.  Up to 8 GEMMs. */
typedef struct mcl_gemm_desc {
  const void* A;  /* bf16 [M][lda] */
  const void* B;  /* bf16 [N][ldb] */
  float* C;       /* fp32 [M][ldc] */
  int32_t M, N, K, lda, ldb, ldc;
} mcl_gemm_desc;
int mcl_gemm_nt_tc_grouped(const mcl_gemm_desc* gemms, int32_t n, int32_t splits, int32_t* err, void* stream);

/* The weight gradients dW = dZt Xt^T of every layer and one Adam step on
 * every weight and bias, in ONE launch: each 128 x 64 tile of dW on a
 * cluster of 4 CTAs splitting the batch, operands streamed by TMA, the
 * partial tiles summed in distributed shared memory in rank order, then
 * Adam with the arithmetic of mcl_adam_multi_dev (learning rate *lr, step
 * *step_base + step_offset counting from 1), the bf16 copies W and Wt
 * refreshed.  The bias gradients gb come summed already (mcl_mlp_fused).
 * batch: a multiple of 256; out: a multiple of 128; in: a multiple of 64; at
 * most 8 layers and 64 tiles.  *err is set to 1 if a completion wait timed
 * out (the launch then changes no weight of the affected tile). */
typedef struct mcl_wgrad_layer {
  const void* dZt;     /* bf16 [out][ld] d loss / d pre-activation, transposed */
  const void* Xt;      /* bf16 [in][ld] the layer's input, transposed          */
  float* W;            /* fp32 [out][in] master weights (updated)              */
  float* m1;           /* fp32 [out][in] Adam first moment (updated)           */
  float* m2;           /* fp32 [out][in] Adam second moment (updated)          */
  void* Wb;            /* bf16 [out][in] copy of W, or NULL                    */
  void* Wt;            /* bf16 [in][out] transposed copy of W, or NULL         */
  float* gW;           /* fp32 [out][in] the gradient, or NULL                 */
  float* b;            /* fp32 [out] bias (updated)                            */
  const float* gb;     /* fp32 [out] bias gradient                             */
  float* mb;           /* fp32 [out] bias first moment (updated)               */
  float* vb;           /* fp32 [out] bias second moment (updated)              */
  int32_t out, in, ld; /* ld >= batch, a multiple of 8                         */
  int32_t reserved;
} mcl_wgrad_layer;
int mcl_wgrad_adam(const mcl_wgrad_layer* layers, int32_t n, int32_t batch, const float* lr,
                   const int32_t* step_base, int32_t step_offset, float b1, float b2, float eps, int32_t* err,
                   void* stream);
/* dZ = dY * gelu'(Z) (or dY when gelu_on == 0) as bf16 in [M][N] and [N][M];
 * db[n] += sum_m dZ[m][n] (db must be cleared by the caller). */
int mcl_act_backward(int32_t M, int32_t N, const float* dY, int32_t lddy, const float* Z, int32_t ldz,
                     int32_t gelu_on, void* dZ, int32_t lddz, void* dZt, int32_t lddzt, float* db,
                     void* stream);
/* *loss += sum over columns < n_valid of (out - target)^2;
 * dout = 2 (out - target) * scale (0 in the padding columns). */
int mcl_mse_loss(int32_t M, int32_t N, int32_t n_valid, const float* out, int32_t ldo,
                 const float* target, int32_t ldt, float scale, float* dout, int32_t ldd, float* loss,
                 void* stream);
/* Adam step on fp32 master weights p[rows][cols]; refreshes the bf16 copies
 * W[rows][cols] and Wt[cols][rows] when non-null.  step counts from 1. */
int mcl_adam(int32_t rows, int32_t cols, float* p, const float* g, float* m1, float* m2, float lr,
             float b1, float b2, float eps, int32_t step, void* W, void* Wt, void* stream);
/* The same Adam step for up to 16 tensors in one launch (the arrays are
 * host memory holding device pointers; W / Wt may be NULL). */
typedef struct mcl_adam_tensor {
  float* p;
  const float* g;
  float* m1;
  float* m2;
  void* W;
  void* Wt;
  int32_t rows;
  int32_t cols;
} mcl_adam_tensor;
int mcl_adam_multi(const mcl_adam_tensor* tensors, int32_t n, float lr, float b1, float b2, float eps,
                   int32_t step, void* stream);
/* The same with the learning rate (*lr) and the step (*step_base +
 * step_offset, counting from 1) read on the device, so that a captured
 * graph of several training steps replays with fresh values. */
int mcl_adam_multi_dev(const mcl_adam_tensor* tensors, int32_t n, const float* lr, const int32_t* step_base,
                       int32_t step_offset, float b1, float b2, float eps, void* stream);
int mcl_f32_to_bf16(int64_t n, const float* x, void* y, void* stream);

/* ---- CUDA graphs -------------------------------------------------------- */
/* Capture mcl_b_run(args) (with its output clearing) into a graph. */
int mcl_b_graph_create(const mcl_b_args* args, void* stream, void** graph_out);
int mcl_graph_launch(void* graph, void* stream);
int mcl_graph_destroy(void* graph);

/* ---- presentation binning and smoothing --------------------------------- */
/* The glow curves src/class/plots.py:52-74 (plot_TL) draws from simulate()'s
 * tables x_ax, lum [steps][sims][runs] (device, FP64): per run the steps with
 * x_ax[:, 0, r] > 0 at T = T_start[r] + T_rate[r] * t, histogrammed into
 * bin_width-wide bins from 0 (hist_and_smooth, plots.py:39-47).
 * mcl_glow_extent writes per run the number of bin edges,
 * ceil((max T + bin_width) / bin_width), or -1 if no step has t > 0 (the
 * reference raises there).  mcl_glow_hist fills hist (bin_offsets[runs+1]
 * from those counts: n_edges - 1 bins per run) with the replica-mean event
 * count per bin divided by bin_width; counts is scratch of n_bins_total
 * words; *status becomes MCL_EINVAL if a lum entry is not a 0/1 flag. */
int mcl_glow_extent(const double* x_ax, int32_t steps, int32_t sims, int32_t runs,
                    const double* T_start, const double* T_rate, double bin_width, int64_t* n_edges,
                    void* stream);
int mcl_glow_hist(const double* x_ax, const double* lum, int32_t steps, int32_t sims, int32_t runs,
                  const double* T_start, const double* T_rate, double bin_width,
                  const int64_t* bin_offsets, int64_t n_bins_total, uint32_t* counts, double* hist,
                  int32_t* status, void* stream);
/* running_mean (plots.py:19-21) of every curve: out = 'valid' boxcar of width
 * k over in / divisor.  in_type 0 = double, 1 = uint32 (e.g. Bernoulli bins);
 * curves are [in_offsets[c], in_offsets[c+1]); out_offsets must give
 * n - k + 1 outputs per curve of n >= k values and k - n + 1 (all equal to
 * the curve's sum / k) for 0 < n < k; max_out = largest output count. */
int mcl_running_mean(int32_t in_type, const void* in, const int64_t* in_offsets, int32_t n_curves,
                     int32_t k, double divisor, const int64_t* out_offsets, int64_t max_out, double* out,
                     void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MCLUM_H */
