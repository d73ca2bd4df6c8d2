"""Roofline arithmetic for the kinetics kernels.

The Bernoulli kernel reads only descriptors and a per-step rate table (a few
hundred MB at most, L2-resident per set) and writes only bins, so neither HBM
nor tensor cores bound it: it is bound by SM instruction issue on the integer
(ALU) and FMA-heavy pipes, which execute the Philox rounds.

Two denominators are reported:

* ``issue``: the algorithmic operation count per electron-step trial -- one
  eighth of a Philox4x32-10 block (10 rounds of two 32x32->64 multiplies and
  two 3-input XORs = 40 operations per block of 8 trials = 5) plus three
  for the Bernoulli test itself (scale, compare, select) = 8, a fixed count
  of the algorithm's work (the kernel's integer prefilter spends about one
  instruction per trial on the test) -- against the issue peak of 4
  sub-partitions x 32 lanes x SM clock x SMs.  The ALU pipe (XORs, the
  prefilter's subtractions and LOP3s) issues at half that rate and
  a 32x32->64 multiply takes about four FMA-heavy cycles per warp, so this
  peak is above what any Philox4x32-10 kernel reaches;
* ``philox``: the measured rate of a kernel that only generates Philox blocks
  in the same counter layout (``mcl_bench_philox``); eight trials per block
  is the most this design can reach.

The event-driven kernel (one CTA per simulation) has no algorithmic
operation count of its own: per step it scores every electron, takes a
block-wide argmin, and on an event shifts arrays and rescans the holes, with
about twenty block barriers in between.  Its roofline is warp-instruction
issue: warp instructions per electron-step, counted by ncu
(smsp__inst_executed.sum) over the parallel TL12 launch (1,216 simulations
of 2,000 electrons and 3,455 centres heated at 5 K/s, Philox streams), times
the measured electron-steps per second, against one warp instruction per
cycle per sub-partition (4 per SM).
"""
from __future__ import annotations

OPS_PER_TRIAL_FP32 = 8
SMS = 152
LANES_PER_SM = 128
# 6.5504e10 warp instructions / 2.9025e9 electron-steps, counted by ncu over
# the parallel TL12 launch (kk_kernel<512>, 1,216 CTAs)
KK_WARP_INSTR_PER_ESTEP = 22.57


def issue_peak_gops(sm_mhz) -> float:
    return SMS * LANES_PER_SM * float(sm_mhz) * 1e6 / 1e9


def bernoulli_fp32(trials: int, seconds: float, sm_mhz=None, traffic=None) -> dict:
    mhz = sm_mhz or 2070.0
    achieved = trials * OPS_PER_TRIAL_FP32 / seconds / 1e9
    peak = issue_peak_gops(mhz)
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gop/s",
            "frac": achieved / peak, "traffic": traffic,
            "ops_per_trial": OPS_PER_TRIAL_FP32, "trials_per_s": trials / seconds,
            "peak_basis": f"{SMS} SMs x {LANES_PER_SM} lanes x {mhz:.0f} MHz "
                          "(median SM clock sampled during the timed region)"
                          if sm_mhz else "max SM clock 2070 MHz"}


def measure_philox_peak(iters: int = 4096, reps: int = 3) -> float:
    """Philox4x32-10 blocks per second on the current GPU (CUDA events)."""
    import ctypes as C
    import torch
    from . import _lib
    lib = _lib.load()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    grid = sms * 8
    sink = torch.empty(grid * 256, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream()
    _lib.check(lib.mcl_bench_philox(C.c_void_p(sink.data_ptr()), grid, 64, 1, C.c_void_p(s.cuda_stream)),
               "mcl_bench_philox")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        _lib.check(lib.mcl_bench_philox(C.c_void_p(sink.data_ptr()), grid, iters, 1,
                                        C.c_void_p(s.cuda_stream)), "mcl_bench_philox")
    e1.record(s)
    e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / reps
    return grid * 256 * 4 * iters / sec


def kk_issue(electron_steps: float, seconds: float, sm_mhz=None, sms: int = SMS) -> dict:
    mhz = sm_mhz or 2070.0
    achieved = electron_steps / seconds * KK_WARP_INSTR_PER_ESTEP
    peak = 4 * sms * mhz * 1e6
    return {"bound": "issue", "unit": "warp instructions/s", "achieved": achieved, "peak": peak,
            "frac": achieved / peak, "warp_instr_per_electron_step": KK_WARP_INSTR_PER_ESTEP,
            "peak_basis": f"4 schedulers x {sms} SMs x {mhz:.0f} MHz",
            "limiter": "block barriers (one CTA per simulation, ~20 barriers per step)"}
