"""Host side of the optimiser drop-in: the result file format and the row
that replay mode picks (src/class/optimizer.py:113-133).  No GPU needed."""
import os

import numpy as np

from golden_io import load_k
from mcluminescence_gb300 import optimizer as O


def test_append_then_best_row_round_trip(tmp_path):
    p = str(tmp_path / "result_tl_clbr.csv")
    rows = [(np.linspace(0.1, 1.0, 10) * (k + 1), m) for k, m in enumerate([0.5, 0.02, 0.3])]
    for x, m in rows:
        O.append_result(p, x, m)
    text = open(p, newline="").read()
    lines = text.split(os.linesep)
    assert lines[0] == ",".join([f"param_{i}" for i in range(10)] + ["mse"])
    assert len(lines) == 5 and lines[-1] == ""
    best, mse = O.best_result(p)
    assert mse == 0.02 and np.array_equal(best, rows[1][0])


def test_best_row_of_a_mixed_format_file(tmp_path):
    """The reference's own result files mix rows with fewer parameters, empty
    cells and an extra trailing column; pandas reads empty cells as NaN and
    idxmin skips NaN MSEs.  The golden replay case stores the reference's
    MSE column and the parameters of its best row."""
    d = load_k()
    mse_col = d["replay_tl_clbr/results_mse"]
    best_p = d["replay_tl_clbr/best_params"]
    i_best = int(np.nanargmin(mse_col))
    p = tmp_path / "r.csv"
    with open(p, "w") as f:
        f.write(",".join([f"param_{i}" for i in range(10)] + ["mse", "rmse"]) + "\n")
        for i, m in enumerate(mse_col):
            x = best_p if i == i_best else np.full(10, 1.0 + i)
            cells = ["" if np.isnan(v) else repr(float(v)) for v in x]
            if i != i_best and i % 3 == 0:
                cells[7:] = ["", "", ""]          # an older row with fewer parameters
            f.write(",".join(cells + ["" if np.isnan(m) else repr(float(m)), ""]) + "\n")
        f.write(",,,,,,,,,,,\n")                   # a row with nothing in it
    got, m = O.best_result(str(p))
    assert m == float(mse_col[i_best])
    assert np.array_equal(np.isnan(got), np.isnan(best_p))
    assert np.array_equal(got[~np.isnan(got)], best_p[~np.isnan(best_p)])


def test_cfg_with_params_keeps_nan_cells():
    """A NaN parameter (an empty cell of the result file) reaches the
    configuration as NaN, as float(nan) does in the reference."""
    base = {"exp_type_fp": {"rho_prime": 1e-4, "holes": 100}, "physics_fp": {"Retrap": 0.5}}
    x = np.arange(10, dtype=float) + 1.0
    x[9] = np.nan
    cfg = O.cfg_with_params(base, x)
    assert np.isnan(cfg["physics_fp"]["Retrap"]) and base["physics_fp"]["Retrap"] == 0.5
    assert cfg["exp_type_fp"]["holes"] == 9.0 and isinstance(cfg["exp_type_fp"]["holes"], float)
