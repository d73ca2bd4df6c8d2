"""Internal consistency of the Bernoulli oracle (CPU only)."""
import numpy as np

from mcluminescence_gb300 import schedule
from oracle import bernoulli as ob
from oracle.philox import TAG_INIT, TAG_STEP, philox4x32, seed_key, u53


def _philox_as_injected(st, seed):
    """The f64 Philox stream of a single-segment set laid out as an injected array."""
    n = st["n_slots"]
    steps = ob.total_steps(st)
    e = np.arange(n, dtype=np.uint64)
    k = seed_key(seed)
    w = philox4x32(0, e, st["set_id"], TAG_INIT, *k)
    u = [u53(w[0], w[1])]
    for j in range(steps):
        w = philox4x32(j >> 1, e, st["set_id"], TAG_STEP, *k)
        h = 2 * (j & 1)
        u.append(u53(w[h], w[h + 1]))
    return np.concatenate(u)


def test_injected_layout_equals_philox_layout():
    st = schedule.single_tl_set(alpha=3.0, n_slots=64, T_end_C=400.0, set_id=5).to_dict()
    a = ob.run_set(st, layout="f64", seed=99, want_fates=True)
    b = ob.run_set(st, layout="injected", uniforms=_philox_as_injected(st, 99), want_fates=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_sampled_curve_matches_expectation():
    """Many replicas of the oracle's sampled curve against the exact expected
    curve: integrated signal within 3 standard errors."""
    base = schedule.single_tl_set(alpha=5.0, n_slots=500, T_end_C=450.0)
    exp = ob.expected_lum(base.to_dict())
    tot = np.zeros_like(exp)
    R = 8
    for r in range(R):
        st = base.to_dict()
        st["set_id"] = 100 + r
        lum, _, _ = ob.run_set(st, layout="f64", seed=7)
        tot += lum
    N = R * 500
    p = exp.sum() / 500
    se = np.sqrt(N * p * (1 - p))
    assert abs(tot.sum() - R * exp.sum()) < 3 * se + 1


def test_fill_saturation():
    """Irradiation alone fills traps to 1 - exp(-D/D0) (binomial check)."""
    sp = schedule.SetSpec(n_slots=4000, n_filled=0, E=2.5, s=1e5, alpha=50.0, set_id=3,
                          segments=[schedule.irradiate(200.0, 0.2, 250.0, 1.0,
                                                       bin_seconds=1000.0)]).finalize()
    _, alive, _ = ob.run_set(sp.to_dict(), layout="f64", seed=3)
    p = 1 - np.exp(-200.0 / 250.0)
    assert abs(alive[-1] - 4000 * p) < 4 * np.sqrt(4000 * p * (1 - p))


def test_expected_curve_mass():
    st = schedule.single_tl_set(alpha=0.0, n_slots=1000).to_dict()
    exp = ob.expected_lum(st)
    assert abs(exp.sum() - 1000.0) < 1e-6   # alpha = 0: everything recombines by 500 C


def _short_dose_fade_irsl(alpha, n_slots, set_id=0):
    S = schedule
    return S.SetSpec(n_slots=n_slots, n_filled=0, E=1.45, s=3e12, alpha=alpha, set_id=set_id,
                     segments=[S.irradiate(150.0, 0.1, 200.0, 1.0, bin_seconds=100.0),
                               S.fade(1e5, 60, 3e-4, dt0=1.0, steps_per_bin=6),
                               S.optical(1.0, 100.0, 0.1, T_C=50.0, bin_seconds=2.0)]).finalize()


def test_expected_fill_alone_is_the_saturating_occupancy():
    """Irradiation with escapes switched off (a trap depth no temperature
    reaches): the expected filled count is N (1 - prod(1 - q_j))."""
    sp = schedule.SetSpec(n_slots=1000, n_filled=0, E=50.0, s=1e12, alpha=5.0,
                          segments=[schedule.irradiate(300.0, 0.2, 250.0, 1.0, bin_seconds=50.0)]).finalize()
    lum, alive = ob.expected_curves(sp.to_dict(), n_u=2000)
    _, q = ob.segment_constants(sp.to_dict(), sp.segments[0].to_dict())
    assert np.all(lum == 0)
    assert abs(alive[-1] - 1000 * (1 - np.prod(1 - q))) < 1e-9


def test_expected_curves_agree_with_the_closed_form_without_filling():
    """The stepped chain and the closed-form survival give the same curve on
    a schedule without filling (the stepped path forced by a tiny fill rate
    on traps that are all filled)."""
    S = schedule
    sp = S.SetSpec(n_slots=500, E=1.3, s=1e11, alpha=4.0,
                   segments=[S.isothermal(180.0, 300.0, 1.0, 10.0)]).finalize()
    closed, alive = ob.expected_curves(sp.to_dict(), n_u=4000)
    st = sp.to_dict()
    st["segments"][0]["fill_rate"] = 1e-300     # q = 0 exactly, stepped path
    stepped, alive2 = ob.expected_curves(st, n_u=4000)
    np.testing.assert_allclose(stepped, closed, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(alive2, alive, rtol=1e-12)


def test_expected_curves_with_filling_match_the_sampled_oracle():
    """Dose -> fading -> IR stimulation: 400 replicas of the sampled oracle
    (numpy stream) against the expected curve, per bin within 4 SE for bins
    with enough counts, and the filled count after the dose within 4 SE."""
    base = _short_dose_fade_irsl(5.0, 500)
    lum_e, alive_e = ob.expected_curves(base.to_dict(), n_u=20000)
    R = 400
    tot = np.zeros_like(lum_e)
    alive_dose = 0
    nb0 = base.segments[0].n_bins
    for r in range(R):
        st = base.to_dict()
        st["set_id"] = 500 + r
        lum, alive, _ = ob.run_set(st, layout="numpy", seed=11)
        tot += lum
        alive_dose += alive[nb0 - 1]
    N = R * base.n_slots
    exp = R * lum_e
    p = exp / N
    se = np.sqrt(N * p * (1 - p))
    big = exp > 25
    assert big.sum() > 20
    assert np.all(np.abs(tot[big] - exp[big]) < 4 * se[big])
    pa = alive_e[nb0 - 1] / base.n_slots
    assert abs(alive_dose - N * pa) < 4 * np.sqrt(N * pa * (1 - pa))
    assert abs(tot.sum() - exp.sum()) < 4 * np.sqrt(exp.sum()) + 1
