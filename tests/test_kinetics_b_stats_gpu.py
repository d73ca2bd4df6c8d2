"""FP32 native-Philox glow curves against the exact expected curves.

The FP32 mode has no draw-for-draw oracle at scale: its statistical contract
is that every binned curve agrees with the FP64 expectation within 3 Monte
Carlo standard errors per bin, and within 0.5 % on the integrated signal and
the peak temperature where the run resolves 0.5 %.  The expected curves come
from ``oracle.bernoulli.expected_curves`` (quadrature over r', no sampling; a
linear two-state chain where traps fill).  Covered here:

* the first 64 sets of the signal-bearing variant of the batched TL +
  isothermal workload (alpha = 5; full schedules, real trap counts), half TL
  ramps and half isothermal holds;
* isothermal holds with many replicas (per-bin and integrated precision);
* irradiation -> fading -> IR stimulation with many replicas, with the
  workload's own alpha (all of its signal is fading) and with a
  signal-bearing alpha in both phases.

Per-bin test: bins with an expected count above 25 are converted to z-scores
(binomial SE); at most as many may exceed 3 in magnitude as a correct sampler
exceeds with probability 1e-3 (binomial quantile of the 0.27 % two-sided
rate), and the chi-square of those bins lies within its 1e-3..1 - 1e-3 band.
"""
import copy

import numpy as np
import pytest
from scipy import stats

from mcluminescence_gb300 import schedule, simulate_batch
from oracle import bernoulli as ob

pytestmark = pytest.mark.gpu


def per_bin_check(obs, exp, n_traps):
    """3-SE per bin with a multiple-comparison allowance, and chi-square."""
    p = np.clip(exp / n_traps, 0.0, 1.0)
    se = np.sqrt(n_traps * p * (1 - p))
    big = exp > 25
    n = int(big.sum())
    z = (obs[big] - exp[big]) / se[big]
    allowed = stats.binom.ppf(0.999, n, 2 * stats.norm.sf(3.0))
    assert np.sum(np.abs(z) > 3) <= allowed, np.sort(np.abs(z))[-5:]
    chi2 = float(np.sum(z ** 2))
    assert stats.chi2.ppf(1e-3, n) < chi2 < stats.chi2.ppf(1 - 1e-3, n), (chi2, n)
    return n


def integrated_check(obs, exp, n_traps):
    """Integrated signal within 4 SE, and within 0.5 % where 3 SE < 0.5 %."""
    P = exp.sum() / n_traps
    se = np.sqrt(n_traps * P * (1 - P))
    assert abs(obs.sum() - exp.sum()) <= 4 * se + 1, (obs.sum(), exp.sum(), se)
    if 3 * se < 0.005 * exp.sum():
        assert abs(obs.sum() - exp.sum()) / exp.sum() < 0.005
        return True
    return False


def peak_check(obs, exp, T0_K, bin_K):
    """Peak temperature after the reference's 50-bin boxcar (1 degC bins:
    50 degC, src/class/plots.py:39-47) within 0.5 % (K)."""
    k = np.ones(50) / 50
    t_peak = np.argmax(np.convolve(obs, k, "valid"))
    e_peak = np.argmax(np.convolve(exp, k, "valid"))
    Tt, Te = T0_K + bin_K * t_peak, T0_K + bin_K * e_peak
    assert abs(Tt - Te) / Te < 0.005, (Tt, Te)


def test_signal_bearing_batch_first_sets():
    specs = schedule.batch_tl_iso(4096, alpha=5.0)[:64]
    res = simulate_batch(specs, precision="fp32", seed=20261203)
    obs_all, exp_all, n_all = [], [], []
    resolved = peaks = 0
    for i, sp in enumerate(specs):
        obs = res.lum_of(i).astype(np.float64)
        exp = ob.expected_lum(sp.to_dict(), n_u=20000)
        resolved += integrated_check(obs, exp, sp.n_slots)
        if sp.kind == "tl" and exp.sum() > 4e4:
            peak_check(obs, exp, sp.segments[0].T0, 1.0)
            peaks += 1
        obs_all.append(obs)
        exp_all.append(exp)
        n_all.append(np.full(obs.size, sp.n_slots, dtype=np.float64))
    n = per_bin_check(np.concatenate(obs_all), np.concatenate(exp_all), np.concatenate(n_all))
    assert n > 2000 and resolved >= 10 and peaks >= 4, (n, resolved, peaks)


@pytest.mark.parametrize("set_index", [5, 11, 15])
def test_isothermal_hold_replicas(set_index):
    """Isothermal holds of the signal-bearing batch (set 5: 282 degC, nearly
    every trap empties; set 11: 204 degC, 46 %; set 15: 236 degC, 8 %),
    4,096 replicas of 2,000 traps each."""
    base = copy.deepcopy(schedule.batch_tl_iso(4096, alpha=5.0)[set_index])
    assert base.kind == "iso"
    base.n_slots = base.n_filled = 2000
    R = 4096
    specs = []
    for r in range(R):
        s = copy.deepcopy(base)
        s.set_id = 50000 + r
        specs.append(s.finalize())
    res = simulate_batch(specs, precision="fp32", seed=99)
    tot = res.lum.reshape(R, base.n_bins).sum(axis=0).astype(np.float64)
    exp = ob.expected_lum(base.finalize().to_dict(), n_u=200000) * R
    N = R * base.n_slots
    assert per_bin_check(tot, exp, N) > 20
    assert integrated_check(tot, exp, N)


@pytest.mark.parametrize("variant", ["own_alpha", "alpha5"])
def test_dose_fade_irsl_replicas(variant):
    """Irradiation -> fading -> IR stimulation, 1,024 replicas of 2,000
    traps starting empty: the per-bin test over all three phases, the filled
    count after the dose, and the integrated signal of each phase."""
    if variant == "own_alpha":
        base = copy.deepcopy(schedule.batch_dose_fade_irsl(8)[2])
    else:
        base = copy.deepcopy(schedule.batch_dose_fade_irsl(8, alpha=5.0, s_tun=1e-4)[5])
    base.n_slots = 2000
    base.n_filled = 0
    base.finalize()
    R = 1024
    specs = []
    for r in range(R):
        s = copy.deepcopy(base)
        s.set_id = 70000 + r
        specs.append(s.finalize())
    res = simulate_batch(specs, precision="fp32", seed=31)
    lum = res.lum.reshape(R, base.n_bins).sum(axis=0).astype(np.float64)
    alive = res.alive.reshape(R, base.n_bins).sum(axis=0).astype(np.float64)
    e_lum, e_alive = ob.expected_curves(base.to_dict(), n_u=20000)
    N = R * base.n_slots
    per_bin_check(lum, e_lum * R, N)
    nb = [g.n_bins for g in base.segments]
    b1, b2 = nb[0], nb[0] + nb[1]
    pa = e_alive[b1 - 1] / base.n_slots          # filled after the dose
    assert abs(alive[b1 - 1] - N * pa) <= 4 * np.sqrt(N * pa * (1 - pa))
    for lo, hi in ((b1, b2), (b2, base.n_bins)):   # fading, then stimulation
        if e_lum[lo:hi].sum() * R > 100:
            integrated_check(lum[lo:hi], e_lum[lo:hi] * R, N)
    if variant == "alpha5":
        assert e_lum[b2:].sum() * R > 2e4        # the stimulation phase carries signal
