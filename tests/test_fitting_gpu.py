"""Batched fitting: what the trained surrogate gains over plain Monte Carlo
fitting at the same Monte-Carlo-verified acceptance criterion."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_surrogate_fitting_needs_far_less_monte_carlo():
    from mcluminescence_gb300 import fitting as Fm, surrogate as S
    P, Cn = S.generate_dataset(250000, seed=21)
    m = S.SurrogateMLP(batch=2048, seed=1)
    S.train(m, P, Cn, steps=4000)
    prob = Fm.make_problem(64, seed=22)
    plain = Fm.fit_plain_mc(prob, pop=32, max_gens=40, seed=3)
    sur = Fm.fit_surrogate(prob, m, pop=32, seed=3)
    Fm.reverify(prob, plain)
    Fm.reverify(prob, sur)
    # same acceptance criterion (MC-verified MSE within 1.5x the noise floor)
    assert sur.accepted >= 0.9 * plain.accepted
    assert sur.accepted >= 0.8 * prob.floor.numel()
    # the surrogate does the search; Monte Carlo only verifies
    assert sur.mc_trials * 3 <= plain.mc_trials, (sur.mc_trials, plain.mc_trials)
    # the answers hold up under a fresh, independent Monte Carlo run
    assert sur.reverified_ratio_median < 1.5
    assert plain.reverified_ratio_median < 1.5


def test_plain_fit_recovers_hidden_parameters_on_easy_targets():
    """Sanity of the objective: DE on Monte Carlo alone reaches the noise floor
    and lands near the hidden trap depth for most fits.  E and log s trade off
    along the peak position (and alpha against rho'), so E is checked to a
    tenth of an eV, not to the Monte Carlo precision of the curve."""
    from mcluminescence_gb300 import fitting as Fm, surrogate as S
    prob = Fm.make_problem(32, seed=23)
    rep = Fm.fit_plain_mc(prob, pop=32, max_gens=40, seed=4)
    assert rep.final_ratio_median < 1.5
    x = S.LOW[:4] + (S.HIGH[:4] - S.LOW[:4]) * rep.best_x.cpu().numpy()
    dE = np.abs(x[:, 0] - prob.hidden[:, 0])
    assert np.median(dE) < 0.12
