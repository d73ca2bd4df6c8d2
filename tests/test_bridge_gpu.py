"""Dilute-limit bridge between the two kinetics modes.

The event-driven kernel reproduces the reference draw for draw; the batched
Bernoulli kernel restates the same rates as per-step escape probabilities
p = 1 - exp(-dt s e^{-E/kT} e^{-alpha d}).  With far more recombination
centres than electrons (holes = 100 N_e), a recombination barely changes the
other electrons' nearest centres, so every electron escapes independently at
the rate b e^{-E/kT} e^{-alpha d} with d its initial nearest distance, and the
event-driven glow curve must follow the Bernoulli expectation
E[S(t_k) - S(t_{k+1})], S(t) = exp(-e^{-alpha d} Lambda(t)), with
Lambda(t) = sum over 0.1 s steps of dt b e^{-E/kT_j} (temperature frozen per
step as both kernels do).  The expectation uses the distance distribution of
the reference's own box geometry (electrons in [0, L)^3, centres in
[0, bf L)^3, sampled here), so box edges do not bias the comparison.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_E, HOLES, BF, RHO_P = 200, 20000, 1.2, 1e-3
E, B, KB, BETA, DT = 1.45, 3.5e12, 8.617343e-5, 1.0, 0.1


def mode_k_cfg():
    from mcluminescence_gb300.config import default_config
    cfg = default_config()
    mc, ph = cfg["exp_type_fp"], cfg["physics_fp"]
    mc.update({"T_start": [0], "T_rate": [BETA], "duration": [500], "max_dt": DT * BETA, "sims": 1,
               "N_e": N_E, "holes": HOLES, "e_ratio_start": 1, "rho_prime": RHO_P,
               "boundary_factor": [BF], "steps": 6000})
    ph.update({"E_loc_1": E, "E_loc_2": E, "b": B, "E_cb": 1000, "k_b": KB, "D": 0})
    return cfg


def alpha_d_samples(n_boxes=40, per_box=20000, seed=3):
    """alpha * nearest-centre distance for electrons of the reference's box:
    alpha L = (4 pi holes / (3 rho'))^(1/3) (tl_trap_lab.py:33-35)."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    aL = (4 * math.pi * HOLES / (3 * RHO_P)) ** (1 / 3)
    n_h = int(HOLES * BF ** 3)
    out = []
    for _ in range(n_boxes):
        holes = rng.random((n_h, 3)) * BF
        el = rng.random((per_box, 3))
        d, _ = cKDTree(holes).query(el)
        out.append(aL * d)
    return np.concatenate(out)


def expected_per_bin(n_electrons, ad):
    """Expected events per 1 degC bin (0..499) for n_electrons."""
    steps = int(round(500 / (BETA * DT)))
    T = 273.15 + BETA * DT * np.arange(steps)
    lam = np.concatenate([[0.0], np.cumsum(DT * B * np.exp(-E / (KB * T)))])   # Lambda at step edges
    edges = lam[::int(round(1 / (BETA * DT)))]                                  # at each 1 degC
    # E over the w distribution: histogram of log w, fine enough to be exact to <1e-3
    logw = -ad
    h, be = np.histogram(logw, bins=4000)
    w = np.exp(0.5 * (be[1:] + be[:-1]))
    pw = h / h.sum()
    S = np.array([np.dot(pw, np.exp(-w * L)) for L in edges])
    return n_electrons * (S[:-1] - S[1:])


def test_event_driven_matches_bernoulli_expectation_in_the_dilute_limit():
    from mcluminescence_gb300 import kinetics as K
    from mcluminescence_gb300.config import initialize_runs
    cfg = mode_k_cfg()
    rp = K.run_params(initialize_runs(cfg)[0])
    n_sims = 1216
    res, _ = K.run_kinetics([rp] * n_sims, 6000, rng="philox", seed=2026, want_events=False)
    assert np.all(res.status == 0), res.status[:8]
    x = res.x_ax.reshape(6000, n_sims)
    lum = res.lum.reshape(6000, n_sims)
    t_ev = x[lum > 0.5]
    obs = np.bincount(np.floor(BETA * t_ev).astype(np.int64), minlength=500)[:500].astype(float)
    exp = expected_per_bin(N_E * n_sims, alpha_d_samples())
    assert obs.sum() > 50000
    # integrated signal within 1 %, per-bin agreement within 3 standard errors
    # (binomial allowance for the number of bins tested), and chi^2 / dof near 1
    assert abs(obs.sum() / exp.sum() - 1) < 0.01, (obs.sum(), exp.sum())
    m = exp > 20
    z = (obs[m] - exp[m]) / np.sqrt(exp[m])
    from scipy.stats import binom
    allowed = int(binom.ppf(0.999, int(m.sum()), 0.0027))
    assert int(np.count_nonzero(np.abs(z) > 3)) <= allowed, np.sort(np.abs(z))[-5:]
    chi2 = float(np.sum(z ** 2)) / int(m.sum())
    assert chi2 < 1.5, chi2
    # peak temperature within 0.5 % (K) after the reference's 50 degC boxcar
    # (src/class/plots.py:39-47); the smoothed top is flat, so its argmax
    # moves by a few degrees with the Monte Carlo noise
    k = np.ones(50) / 50
    t_peak = np.argmax(np.convolve(obs, k, "valid")) + 273.15
    e_peak = np.argmax(np.convolve(exp, k, "valid")) + 273.15
    assert abs(t_peak - e_peak) / e_peak < 0.005, (t_peak, e_peak)
