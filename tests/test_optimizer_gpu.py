"""The optimiser drop-in on the reference's own lab data (GPU).

The golden case ``replay_tl_clbr`` is the reference's optimiser in replay
mode: the minimum-MSE row of its results/lab_sims/result_tl_clbr.csv scored
by its ``objective`` (TLTrapSim.TL_lab) against
data/processed/CLBR_IRSL50_0.25KperGy.csv, after np.random.seed(41).
"""
import json
import os

import numpy as np
import pytest

from golden_io import load_k
from mcluminescence_gb300 import optimizer as O

pytestmark = pytest.mark.gpu

DATA = load_k()
NAME = "replay_tl_clbr"
TABLE = "CLBR_IRSL50_0.25KperGy"


@pytest.fixture
def project(tmp_path, monkeypatch):
    """A project root holding the lab table (data/processed) and a result
    file (results/lab_sims) in the reference's formats."""
    tb = json.loads(bytes(DATA[f"{NAME}/table"]).decode())
    dd = tmp_path / "data" / "processed"
    dd.mkdir(parents=True)
    cols = list(tb)
    with open(dd / f"{TABLE}.csv", "w") as f:
        f.write(",".join(cols) + "\n")
        for i in range(len(tb[cols[0]])):
            f.write(",".join(repr(float(tb[c][i])) for c in cols) + "\n")
    rd = tmp_path / "results" / "lab_sims"
    rd.mkdir(parents=True)
    best = DATA[f"{NAME}/best_params"]
    with open(rd / "result_tl_clbr.csv", "w") as f:
        f.write(",".join([f"param_{i}" for i in range(10)] + ["mse", "rmse"]) + "\n")
        f.write(",".join(["0.5"] * 10 + ["0.2", ""]) + "\n")
        f.write(",".join("" if np.isnan(v) else repr(float(v)) for v in best)
                + "," + repr(float(np.nanmin(DATA[f"{NAME}/results_mse"]))) + ",\n")
        f.write(",".join(["0.7"] * 7 + ["", "", ""] + ["0.09", ""]) + "\n")
    monkeypatch.setenv("MCL_PROJECT_ROOT", str(tmp_path))
    monkeypatch.delenv("MCL_DATA_DIR", raising=False)
    return tmp_path


def _cfg():
    return json.loads(bytes(DATA[f"{NAME}/cfg"]).decode())


def _stream_after(seed, draws):
    rs = np.random.RandomState(seed)
    rs.random_sample(int(np.sum(draws)))
    return rs.random_sample(3)


def test_replay_reproduces_the_reference(project):
    seed = int(DATA[f"{NAME}/seed"])
    np.random.seed(seed)
    mse = O.main(_cfg(), task="replay", exp="tl_clbr")
    assert mse == float(DATA[f"{NAME}/mse"])
    assert np.array_equal(np.random.random_sample(3), _stream_after(seed, DATA[f"{NAME}/draws"]))


def test_batched_objective_equals_tl_lab_under_the_reference_stream(project):
    """One candidate through the batched objective with numpy's stream
    scores exactly what the reference's TL_lab scored."""
    from mcluminescence_gb300.config import initialize_runs
    seed = int(DATA[f"{NAME}/seed"])
    base = initialize_runs(_cfg())[0]
    np.random.seed(seed)
    f = O.lab_objective_batch(base, DATA[f"{NAME}/best_params"][None, :], TABLE, "tl", rng="numpy")
    assert f[0] == float(DATA[f"{NAME}/mse"])
    assert np.array_equal(np.random.random_sample(3), _stream_after(seed, DATA[f"{NAME}/draws"]))


def test_batched_de_on_the_lab_data_then_replay(project):
    """train: the batched DE over the reference's ten bounds on the real lab
    table (150 candidates x 11 rows per launch); the best MSE never rises
    over generations, the result row is appended in the reference's format,
    and replay scores that row once more."""
    from mcluminescence_gb300.config import initialize_runs
    base = initialize_runs(_cfg())[0]
    x, f, hist = O.optimize(base, TABLE, "tl", gens=4, popsize=15, seed=3)
    assert np.all(np.diff(hist) <= 0) and np.isfinite(f)
    assert all(lo <= v <= hi for v, (lo, hi) in zip(x, O.DEFAULT_BOUNDS))
    path = str(project / "results" / "lab_sims" / "result_tl_fresh.csv")
    O.append_result(path, x, f)
    got, m = O.best_result(path)
    assert m == f and np.array_equal(got, x)
    cfg = _cfg()
    s = O.main(cfg, task="train", exp="tl_clbr", gens=2, pop=4, seed=5)
    assert np.isfinite(s)
    assert O.best_result(O.result_path("tl_clbr"))[1] <= 0.09
    assert np.isfinite(O.main(cfg, task="replay", exp="tl_clbr"))
