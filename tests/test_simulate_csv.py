"""The long-format CSV side effect of ``simulate()`` (src/class/simulate.py:95-110).

The reference always writes ``results/simulations/exp_{tag}.csv``.  The golden
files in ``tests/golden/simulate_csv.npz`` are the reference's own output,
written by its unmodified ``simulate()`` (``tests/golden/make_golden_csv.py``,
through a stand-in pandas that restates pandas' ``to_csv`` text rules).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from mcluminescence_gb300.kinetics import write_table

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("tl12_small", "cold_isothermal", "lab_physics")


def _golden():
    return (np.load(os.path.join(HERE, "golden", "kinetics_k.npz")),
            np.load(os.path.join(HERE, "golden", "simulate_csv.npz")))


@pytest.mark.parametrize("case", CASES)
def test_writer_reproduces_the_reference_file_from_its_tables(case, tmp_path):
    """The reference's own tables through write_table give its file byte for
    byte (no GPU needed)."""
    g, c = _golden()
    p = tmp_path / "t.csv"
    write_table(str(p), g[f"{case}/lum"], g[f"{case}/electron_ratio"])
    data = p.read_bytes()
    assert hashlib.sha256(data).hexdigest() == str(c[f"{case}/sha256"])
    assert data == bytes(c[f"{case}/csv"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_simulate_writes_the_reference_file(case, tmp_path, monkeypatch):
    """np.random.seed(seed); simulate(cfg) with cfg.tag set writes
    exp_{tag}.csv into the results directory, identical to the reference's."""
    from mcluminescence_gb300 import simulate
    g, c = _golden()
    cfg = json.loads(bytes(g[f"{case}/cfg"]).decode())
    cfg["tag"] = case
    monkeypatch.setenv("MCL_RESULTS_DIR", str(tmp_path / "results" / "simulations"))
    np.random.seed(int(c[f"{case}/seed"]))
    simulate(cfg)
    data = (tmp_path / "results" / "simulations" / f"exp_{case}.csv").read_bytes()
    assert data == bytes(c[f"{case}/csv"])


@pytest.mark.gpu
def test_simulate_csv_opt_out_and_explicit_path(tmp_path, monkeypatch):
    from mcluminescence_gb300 import simulate
    g, c = _golden()
    cfg = json.loads(bytes(g["cold_isothermal/cfg"]).decode())
    monkeypatch.setenv("MCL_RESULTS_DIR", str(tmp_path / "r"))
    simulate(cfg, write_csv=False)
    assert not (tmp_path / "r").exists()
    np.random.seed(int(c["cold_isothermal/seed"]))
    simulate(cfg, csv_path=str(tmp_path / "x.csv"))
    assert (tmp_path / "x.csv").read_bytes() == bytes(c["cold_isothermal/csv"])
