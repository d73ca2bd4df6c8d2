"""The event-driven (reference) kinetics kernel against the reference's own
outputs (golden fixtures made by running the unmodified reference)."""
import numpy as np
import pytest

from golden_io import k_case, k_case_names, load_k
from mcluminescence_gb300 import run_kinetics, run_params, simulate
from mcluminescence_gb300.config import initialize_runs

pytestmark = pytest.mark.gpu

DATA = load_k()
CASES = [c for c in k_case_names(DATA) if c not in ("box_ops", "lab_tl", "lab_iso")]


def _check_against_golden(case, x_ax, lum, ratio, res):
    # integer outcomes exactly; times to the last bits of exp/log
    assert np.array_equal(lum, case["lum"])
    assert np.array_equal(ratio, case["electron_ratio"])
    np.testing.assert_allclose(x_ax, case["x_ax"], rtol=1e-12, atol=0)
    assert list(res.n_steps) == list(case["steps_taken"])
    assert list(res.draws) == list(case["draws"])
    for got, want in zip(res.events, case["events"]):
        assert np.array_equal(got, want)


@pytest.mark.parametrize("name", CASES)
def test_simulate_matches_reference_draw_for_draw(name):
    """np.random.seed(k); simulate(cfg) on the GPU == the reference's simulate(cfg)."""
    case = k_case(DATA, name)
    np.random.seed(case["seed"])
    if case["error"]:
        with pytest.raises(IndexError):
            simulate(case["cfg"])
        return
    (x_ax, lum, ratio, configs), res = simulate(case["cfg"], return_result=True)
    _check_against_golden(case, x_ax, lum, ratio, res)
    # numpy's global stream is left where the reference leaves it
    after = np.random.random_sample(3)
    rs = np.random.RandomState(case["seed"])
    rs.random_sample(int(np.sum(case["draws"])))
    assert np.array_equal(after, rs.random_sample(3))


@pytest.mark.parametrize("name", ["tl12_small", "lab_physics", "cold_isothermal", "isothermal"])
def test_injected_stream_equals_mt_stream(name):
    """The same draws handed over as an injected array give the same results."""
    case = k_case(DATA, name)
    cfg = case["cfg"]
    sims = int(cfg["exp_type_fp"]["sims"])
    params = []
    for r in initialize_runs(cfg).values():
        params += [run_params(r)] * sims
    u = np.random.RandomState(case["seed"]).random_sample(int(np.sum(case["draws"])))
    steps = int(cfg["exp_type_fp"]["steps"])
    res, _ = run_kinetics(params, steps, rng="injected", uniforms=u)
    assert list(res.status) == [0] * len(params)
    assert list(res.draws) == list(case["draws"])
    for got, want in zip(res.events, case["events"]):
        assert np.array_equal(got, want)


def test_injected_stream_too_short_is_reported():
    case = k_case(DATA, "tl12_small")
    cfg = case["cfg"]
    params = [run_params(initialize_runs(cfg)[0])]
    u = np.random.RandomState(0).random_sample(1000)
    res, _ = run_kinetics(params, int(cfg["exp_type_fp"]["steps"]), rng="injected", uniforms=u)
    from mcluminescence_gb300 import _lib
    assert res.status[0] == _lib.MCL_EBUDGET


def test_philox_parallel_statistics_and_determinism():
    """Independent Philox streams, all simulations in parallel, against the
    reference's own method: 192 simulations per run on numpy's stream (the
    mode that is bit-exact with the reference) and 192 on Philox streams have
    the same distribution of event counts (two-sample Kolmogorov-Smirnov
    test, and means within 4 standard errors of their difference) and of
    event times (mean time of an event within 4 SE); Philox runs repeat
    exactly."""
    from scipy import stats
    case = k_case(DATA, "tl12_small")
    cfg = dict(case["cfg"])
    R = 192
    cfg["exp_type_fp"] = dict(cfg["exp_type_fp"], sims=R)
    x1, l1, r1, _ = simulate(cfg, rng="philox", seed=3, write_csv=False)
    x2, l2, r2, _ = simulate(cfg, rng="philox", seed=3, write_csv=False)
    assert np.array_equal(l1, l2) and np.array_equal(x1, x2) and np.array_equal(r1, r2)
    np.random.seed(11)
    xm, lm, _, _ = simulate(cfg, write_csv=False)      # numpy's stream, as the reference
    # sanity: both agree with the reference's own two simulations per run
    ref = case["lum"].sum(axis=0)                       # (2, 3)
    for r in range(3):
        cp, cm = l1[:, :, r].sum(axis=0), lm[:, :, r].sum(axis=0)   # events per simulation
        se = np.sqrt(cp.var(ddof=1) / R + cm.var(ddof=1) / R)
        assert abs(cp.mean() - cm.mean()) < 4 * se + 1e-9, (r, cp.mean(), cm.mean())
        assert stats.ks_2samp(cp, cm).pvalue > 1e-3, r
        assert abs(ref[:, r].mean() - cm.mean()) < 4 * cm.std(ddof=1) + 1
        # times of the events
        tp = x1[:, :, r][l1[:, :, r] > 0]
        tm = xm[:, :, r][lm[:, :, r] > 0]
        se_t = np.sqrt(tp.var(ddof=1) / tp.size + tm.var(ddof=1) / tm.size)
        assert abs(tp.mean() - tm.mean()) < 4 * se_t, (r, tp.mean(), tm.mean())


def test_philox_parallel_results_do_not_depend_on_block_size():
    """One CTA per simulation with 256 or 512 threads: the same draws, the
    same events, the same curves."""
    from mcluminescence_gb300 import kinetics as K
    from mcluminescence_gb300.config import initialize_runs
    case = k_case(DATA, "tl12_small")
    runs = initialize_runs(dict(case["cfg"]))
    params = [K.run_params(runs[r]) for r in runs] * 6
    a, _ = K.run_kinetics(params, 20000, rng="philox", seed=17, block=256, want_events=True)
    b, _ = K.run_kinetics(params, 20000, rng="philox", seed=17, block=512, want_events=True)
    assert np.array_equal(a.n_steps, b.n_steps) and np.array_equal(a.draws, b.draws)
    assert np.array_equal(a.lum, b.lum) and np.array_equal(a.x_ax, b.x_ax) and np.array_equal(a.electron_ratio, b.electron_ratio)
    for ea, eb in zip(a.events, b.events):
        assert np.array_equal(ea, eb)


@pytest.mark.parametrize("kind", ["tl", "iso"])
def test_lab_objectives_match_reference(kind):
    """np.random.seed(k); TLTrapSim(run).TL_lab / ISO_lab on the GPU == the
    reference on the same (synthetic) lab table."""
    import json
    from mcluminescence_gb300 import TLTrapSim
    name = f"lab_{kind}"
    cfg = json.loads(bytes(DATA[f"{name}/cfg"]).decode())
    table = json.loads(bytes(DATA[f"{name}/table"]).decode())
    np.random.seed(int(DATA[f"{name}/seed"]))
    sim = TLTrapSim(initialize_runs(cfg)[0])
    mse = sim.TL_lab(table) if kind == "tl" else sim.ISO_lab(table)
    assert mse == float(DATA[f"{name}/mse"])
    assert list(sim.last.draws) == list(DATA[f"{name}/draws"])
    for i, ev in enumerate(sim.last.events):
        assert np.array_equal(ev, DATA[f"{name}/events{i}"])


def test_batched_lab_objective_and_optimizer():
    """All DE candidates x lab rows in one launch; DE lowers the lab MSE."""
    import json
    from mcluminescence_gb300 import optimizer as O
    cfg = json.loads(bytes(DATA["lab_tl/cfg"]).decode())
    table = json.loads(bytes(DATA["lab_tl/table"]).decode())
    run = initialize_runs(cfg)[0]
    rng = np.random.default_rng(0)
    lo = np.array([b[0] for b in O.DEFAULT_BOUNDS])
    hi = np.array([b[1] for b in O.DEFAULT_BOUNDS])
    cands = lo + (hi - lo) * rng.random((40, 10))
    f1 = O.lab_objective_batch(run, cands, table, "tl", seed=5)
    f2 = O.lab_objective_batch(run, cands, table, "tl", seed=5)
    assert np.array_equal(f1, f2) and np.all(np.isfinite(f1))
    best, mse, hist = O.optimize(run, table, "tl", gens=4, popsize=4, seed=1)
    assert hist[-1] <= hist[0]
    assert mse == hist[-1]
