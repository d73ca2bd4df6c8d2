"""Roofline arithmetic for the kinetics kernels.

The Bernoulli kernel reads only descriptors and writes only bins, so it is not
bound by HBM or by tensor cores but by SM instruction issue: every
electron-step trial needs a quarter of a Philox4x32-10 block (10 rounds of two
32x32->64 multiplies and two three-input XORs = 40 operations per 4 uniforms)
plus the three-operation fast test (form f from the uniform's top bits, one
FMA, one compare): 13 algorithmic operations per trial.  The issue peak is
4 sub-partitions x 32 lanes x SM clock x SMs thread-operations per second.
"""
from __future__ import annotations

OPS_PER_TRIAL_FP32 = 13
SMS = 152
LANES_PER_SM = 128


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
