"""The FP64 oracle of the event-driven kinetics against the reference's own
outputs (golden fixtures made by running the unmodified reference)."""
import numpy as np
import pytest

from golden_io import k_case, k_case_names, load_k
from mcluminescence_gb300.config import initialize_runs
from oracle import kinetics_k as ok

DATA = load_k()
CASES = [c for c in k_case_names(DATA) if c not in ("box_ops", "lab_tl", "lab_iso")]
FAST = CASES


def _run(case):
    cfg = case["cfg"]
    runs = [ok.run_from_cfg(r) for r in initialize_runs(cfg).values()]
    stream = ok.UniformStream(np.random.RandomState(case["seed"]))
    steps = int(cfg["exp_type_fp"]["steps"])
    sims = int(cfg["exp_type_fp"]["sims"])
    return ok.simulate_runs(runs, stream, steps, sims)


@pytest.mark.parametrize("name", FAST)
def test_oracle_matches_reference(name):
    case = k_case(DATA, name)
    if case["error"]:
        with pytest.raises(IndexError):
            _run(case)
        return
    x_ax, lum, ratio, results = _run(case)
    assert np.array_equal(x_ax, case["x_ax"])
    assert np.array_equal(lum, case["lum"])
    assert np.array_equal(ratio, case["electron_ratio"])
    assert [r.draws for r in results] == list(case["draws"])
    assert [r.n_steps for r in results] == list(case["steps_taken"])
    for r, ev in zip(results, case["events"]):
        assert np.array_equal(r.events, ev)


def test_box_ops_quirks():
    """Pair creation/removal bookkeeping, op by op (engine.py:133-175)."""
    seed = int(DATA["box_ops/seed"])
    stream = ok.UniformStream(np.random.RandomState(seed))
    geom = (1.0, 30, int(25 * 1.2 ** 3), (1.0, 1.0, 1.0), (1.2, 1.2, 1.2))
    sim = ok.KSim(None, stream, geometry=geom)
    sim.nearest()
    lens = DATA["box_ops/lens"]
    offs = np.concatenate([[0], np.cumsum(lens)])
    for k, (kind, e, h) in enumerate(DATA["box_ops/ops"]):
        if kind == 0:
            sim.add_electron()
        else:
            sim.remove_pair(int(e), int(h))
        d, n = sim.nearest()
        assert np.array_equal(d, DATA["box_ops/d_min"][offs[k]:offs[k + 1]])
        assert np.array_equal(n, DATA["box_ops/nearest"][offs[k]:offs[k + 1]])


def test_initialize_runs_divisibility():
    cfg = {"exp_type_fp": {"a": [1, 2, 3], "b": [1, 2]}, "physics_fp": {}}
    with pytest.raises(ValueError, match="not divisible"):
        initialize_runs(cfg)
    runs = initialize_runs({"exp_type_fp": {"a": [1, 2, 3, 4], "b": [7, 8]},
                            "physics_fp": {"c": 5}})
    assert [r["exp_type_fp"]["b"] for r in runs.values()] == [7, 8, 7, 8]
    assert all(r["physics_fp"]["c"] == 5 for r in runs.values())


@pytest.mark.parametrize("kind", ["tl", "iso"])
def test_lab_objectives_match_reference(kind):
    """TL_lab / ISO_lab restated: same MSE, event logs and draws as the
    reference on synthetic lab tables (tl_trap_lab.py:65-179)."""
    import json
    name = f"lab_{kind}"
    cfg = json.loads(bytes(DATA[f"{name}/cfg"]).decode())
    table = json.loads(bytes(DATA[f"{name}/table"]).decode())
    r = ok.run_from_cfg(initialize_runs(cfg)[0])
    stream = ok.UniformStream(np.random.RandomState(int(DATA[f"{name}/seed"])))
    stream.take(int(DATA[f"{name}/init_draws"]))
    if kind == "tl":
        mse, _, events, draws = ok.tl_lab(r, stream, table, D=float(cfg["physics_fp"]["D"]))
    else:
        mse, _, events, draws = ok.iso_lab(r, stream, table)
    assert mse == float(DATA[f"{name}/mse"])
    assert draws == list(DATA[f"{name}/draws"])
    for i, ev in enumerate(events):
        assert np.array_equal(ev, DATA[f"{name}/events{i}"])
