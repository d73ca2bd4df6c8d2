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
