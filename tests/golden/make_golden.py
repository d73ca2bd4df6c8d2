"""Generate the golden fixtures by running the UNMODIFIED reference.

Run where the reference checkout is available, with ``MCL_REFERENCE``
naming its root::

    MCL_REFERENCE=<checkout> python tests/golden/make_golden.py   # writes tests/golden/kinetics_k.npz

What it does
* puts the stand-in ``omegaconf``/``hydra``/``pandas``/``matplotlib`` modules
  of ``tests/golden/refshim`` first on ``sys.path`` and imports the reference's
  ``src/class`` modules unchanged;
* wraps (without changing behaviour) ``Box.add_electron``, ``Box.remove_pair``,
  ``TLTrapSim.__init__`` and ``TLTrapSim._update_lifetimes`` to log, per
  simulation, the step index and the array indices of every pair creation and
  recombination, and ``np.random.rand`` / ``np.random.exponential`` to count
  the uniforms each simulation consumes;
* seeds numpy's global legacy ``RandomState`` and calls ``simulate(cfg)``;
* stores the returned ``x_ax, Lum, electron_ratio`` tables, the event logs and
  the draw counts per case.

The GPU parity tests regenerate the same uniform stream with
``np.random.RandomState(seed).random_sample`` (numpy's legacy stream is fixed
across versions and platforms), so no reference code is needed where they run.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from refpath import reference_root  # noqa: E402

REF = reference_root()

sys.path.insert(0, os.path.join(HERE, "refshim"))
sys.path.insert(0, os.path.join(REF, "src", "class"))
sys.path.insert(0, REPO)

from mcluminescence_gb300.config import compose  # noqa: E402

import engine as ref_engine  # noqa: E402
import tl_trap_lab as ref_tl  # noqa: E402
import simulate as ref_sim  # noqa: E402
from omegaconf import OmegaConf  # noqa: E402  (the stand-in)

# --------------------------------------------------------------------------
# instrumentation (behaviour-preserving wrappers)
# --------------------------------------------------------------------------
LOG = {"sims": []}
_draws = [0]

_orig_rand = np.random.rand
_orig_exp = np.random.exponential


def _rand(*shape):
    _draws[0] += int(np.prod(shape)) if shape else 1
    return _orig_rand(*shape)


def _exponential(scale=1.0, size=None):
    _draws[0] += int(np.size(scale)) if size is None else int(np.prod(size))
    return _orig_exp(scale, size)


np.random.rand = _rand
np.random.exponential = _exponential

_orig_init = ref_tl.TLTrapSim.__init__
_orig_upd = ref_tl.TLTrapSim._update_lifetimes
_orig_add = ref_engine.Box.add_electron
_orig_rm = ref_engine.Box.remove_pair


def _init(self, cfg, *, e_ratio_start=None):
    LOG["sims"].append({"events": [], "step": -1, "draw0": _draws[0]})
    return _orig_init(self, cfg, e_ratio_start=e_ratio_start)


def _upd(self, T):
    LOG["sims"][-1]["step"] += 1
    return _orig_upd(self, T)


def _add(self):
    r = _orig_add(self)
    s = LOG["sims"][-1]
    s["events"].append((s["step"], 0, self.electrons.shape[0] - 1, self.holes.shape[0] - 1))
    return r


def _rm(self, e_idx, h_idx):
    s = LOG["sims"][-1]
    s["events"].append((s["step"], 1, int(e_idx), int(h_idx)))
    return _orig_rm(self, e_idx, h_idx)


ref_tl.TLTrapSim.__init__ = _init
ref_tl.TLTrapSim._update_lifetimes = _upd
ref_engine.Box.add_electron = _add
ref_engine.Box.remove_pair = _rm

# --------------------------------------------------------------------------
# cases
# --------------------------------------------------------------------------
CONF = os.path.join(REF, "conf")

CASES = {
    # TL12 physics, small box, three heating rates, two sims each
    "tl12_small": dict(seed=11, overrides=[
        "exp_type_fp.N_e=200", "exp_type_fp.holes=200", "exp_type_fp.sims=2",
        "exp_type_fp.T_rate=[1,5,20]", "exp_type_fp.duration=[800,160,40]",
        "exp_type_fp.steps=3000"]),
    # TL12 defaults at full size (2,000 electrons, 3,455 holes), two rates
    "tl12_full": dict(seed=0, overrides=[
        "exp_type_fp.sims=1", "exp_type_fp.T_rate=[5,20]",
        "exp_type_fp.duration=[160,40]"]),
    # the single-set TL shape (2,000 e, 0->500 C at 1 K/s, dt cap 0.1 s,
    # E=1.45 eV, b=3.5e12, conduction band off) at rho'=1e-3
    "config1_shape": dict(seed=20261203, overrides=[
        "exp_type_fp.sims=1", "exp_type_fp.T_rate=[1]", "exp_type_fp.duration=[500]",
        "exp_type_fp.max_dt=0.1", "exp_type_fp.rho_prime=1e-3",
        "exp_type_fp.steps=8000", "physics_fp.E_loc_1=1.45", "physics_fp.E_loc_2=1.45",
        "physics_fp.b=3.5e12", "physics_fp.E_cb=1000"]),
    # two localisation depths chosen by Retrap, conduction band open
    "lab_physics": dict(seed=7, overrides=[
        "physics_fp=lab_TL", "exp_type_fp.N_e=100", "exp_type_fp.holes=100",
        "exp_type_fp.sims=1", "exp_type_fp.rho_prime=1e-4",
        "exp_type_fp.T_start=[150]", "exp_type_fp.T_rate=[1]",
        "exp_type_fp.duration=[400]", "exp_type_fp.e_ratio_start=0.8",
        "exp_type_fp.steps=4000", "physics_fp.E_loc_2=1.25", "physics_fp.Retrap=0.3",
        "physics_fp.E_cb=1.6"]),
    # isothermal hold: no heating, so the dt cap is 1e20
    "isothermal": dict(seed=3, overrides=[
        "exp_type_fp.N_e=120", "exp_type_fp.holes=120", "exp_type_fp.sims=1",
        "exp_type_fp.T_start=[250]", "exp_type_fp.T_rate=[0]",
        "exp_type_fp.duration=[3000]", "exp_type_fp.steps=500"]),
    # empty start: no electrons, so wait.any() is False and dt_recomb = dt_fill
    "empty_start": dict(seed=9, overrides=[
        "exp_type_fp.N_e=60", "exp_type_fp.holes=60", "exp_type_fp.sims=1",
        "exp_type_fp.T_rate=[5]", "exp_type_fp.duration=[100]",
        "exp_type_fp.e_ratio_start=0", "exp_type_fp.steps=2000"]),
    # cold isothermal hold: lifetimes ~1e37 s exceed the 1e20 s filling wait
    # (lambda = 1e-20 because the dose rate is 0), so pairs are CREATED even
    # with a full trap population (tl_trap_lab.py:53-60, simulate.py:57-72)
    "cold_isothermal": dict(seed=4, overrides=[
        "exp_type_fp.N_e=40", "exp_type_fp.holes=40", "exp_type_fp.sims=2",
        "exp_type_fp.T_start=[-150]", "exp_type_fp.T_rate=[0]",
        "exp_type_fp.duration=[6e20]", "exp_type_fp.steps=200"]),
    # zero duration: exactly one step is taken
    "zero_duration": dict(seed=1, overrides=[
        "exp_type_fp.N_e=50", "exp_type_fp.holes=50", "exp_type_fp.sims=1",
        "exp_type_fp.T_rate=[1]", "exp_type_fp.duration=[0]", "exp_type_fp.steps=10"]),
    # the output table is too short: the reference raises IndexError
    "step_overflow": dict(seed=2, overrides=[
        "exp_type_fp.N_e=80", "exp_type_fp.holes=80", "exp_type_fp.sims=1",
        "exp_type_fp.T_rate=[20]", "exp_type_fp.duration=[40]", "exp_type_fp.steps=25"]),
}


def run_case(name, spec):
    cfg_plain = compose(CONF, spec["overrides"])
    cfg = OmegaConf.create(cfg_plain)
    LOG["sims"] = []
    _draws[0] = 0
    np.random.seed(spec["seed"])
    t0 = time.time()
    err = None
    try:
        x_ax, lum, ratio, _ = ref_sim.simulate(cfg)
    except IndexError as e:
        err = "IndexError"
        x_ax = lum = ratio = np.zeros((0, 0, 0))
    wall = time.time() - t0
    sims = LOG["sims"]
    draws = []
    for i, s in enumerate(sims):
        end = sims[i + 1]["draw0"] if i + 1 < len(sims) else _draws[0]
        draws.append(end - s["draw0"])
    out = {
        f"{name}/cfg": np.frombuffer(json.dumps(cfg_plain).encode(), dtype=np.uint8),
        f"{name}/seed": np.array(spec["seed"]),
        f"{name}/error": np.frombuffer((err or "").encode(), dtype=np.uint8),
        f"{name}/x_ax": x_ax, f"{name}/lum": lum, f"{name}/electron_ratio": ratio,
        f"{name}/n_sims": np.array(len(sims)),
        f"{name}/draws": np.array(draws, dtype=np.int64),
        f"{name}/steps_taken": np.array([s["step"] + 1 for s in sims], dtype=np.int64),
        f"{name}/wall_s": np.array(wall),
    }
    for i, s in enumerate(sims):
        out[f"{name}/events{i}"] = np.array(s["events"], dtype=np.int64).reshape(-1, 4)
    nev = [len(s["events"]) for s in sims]
    print(f"{name}: {len(sims)} sims, events {nev}, draws {draws}, {wall:.1f}s"
          + (f", error {err}" if err else ""), flush=True)
    return out


def run_box_ops(seed=123, n_ops=80):
    """Scripted pair creations/removals on the reference ``Box``.

    Records ``(d_min, nearest)`` after every operation, which pins the
    bookkeeping quirks of engine.py:133-175 independently of the rates.
    """
    ops_rs = np.random.RandomState(seed + 1)
    np.random.seed(seed)
    box = ref_engine.Box(1.0, 1.0, 1.0, 1.2)
    box.seed(30, 25)
    box.nearest()
    ops, dmins, nears = [], [], []
    LOG["sims"] = [{"events": [], "step": 0, "draw0": 0}]
    for _ in range(n_ops):
        n_e = box.electrons.shape[0]
        if n_e < 3 or ops_rs.random_sample() < 0.4:
            box.add_electron()
            ops.append((0, -1, -1))
        else:
            e = int(ops_rs.randint(n_e))
            # mostly the physical pairing, sometimes an arbitrary hole
            h = int(box.nearest()[1][e]) if ops_rs.random_sample() < 0.7 else \
                int(ops_rs.randint(box.holes.shape[0]))
            box.remove_pair(e, h)
            ops.append((1, e, h))
        d, n = box.nearest()
        dmins.append(d.copy())
        nears.append(n.copy())
    lens = np.array([len(d) for d in dmins], dtype=np.int64)
    print(f"box_ops: {n_ops} ops, final {box.electrons.shape[0]} e / {box.holes.shape[0]} h")
    return {"box_ops/seed": np.array(seed), "box_ops/ops": np.array(ops, dtype=np.int64),
            "box_ops/lens": lens, "box_ops/d_min": np.concatenate(dmins),
            "box_ops/nearest": np.concatenate(nears).astype(np.int64)}


# synthetic lab tables with the columns of data/processed/*.csv
LAB_TL = {"Duration": [800.0, 1600.0, 2400.0, 3200.0, 1200.0, 2000.0],
          "T_start": [300.0] * 6, "T_end": [275.0, 250.0, 225.0, 200.0, 290.0, 260.0],
          "Fill": [0.05, 0.15, 0.30, 0.45, 0.10, 0.20], "e_ratio": [0.0, 0.0, 0.0, 0.0, 0.2, 0.0]}
LAB_ISO = {"exp_no": [0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2],
           "e_ratio": [0.0, 0.20, 0.35, 0.50, 0.0, 0.10, 0.20, 0.25, 0.3, 0.25, 0.2],
           "temp": [15.0] * 4 + [120.0] * 4 + [200.0] * 3,
           "dose": [0.092] * 4 + [0.092] * 4 + [0.05] * 3,
           "time": [0.0, 500.0, 1000.0, 2500.0, 0.0, 300.0, 900.0, 1800.0, 0.0, 200.0, 600.0],
           "L": [0.0] * 11}
LAB_CFG = ["physics_fp=lab_TL", "exp_type_fp=TLlab", "physics_fp.E_loc_2=1.3",
           "physics_fp.Retrap=0.4"]


def run_lab(kind, seed):
    import pandas as stub_pd
    stub_pd.register_table("synthetic_tl", LAB_TL)
    stub_pd.register_table("synthetic_iso", LAB_ISO)
    cfg_plain = compose(CONF, LAB_CFG)
    cfg = OmegaConf.create(cfg_plain)
    runs = ref_engine.initialize_runs(cfg)
    LOG["sims"] = []
    _draws[0] = 0
    np.random.seed(seed)
    sim = ref_tl.TLTrapSim(runs[0])
    init_draws = _draws[0]      # the constructor seeds a box before TL_lab re-initialises
    LOG["sims"] = []
    _draws[0] = 0
    t0 = time.time()
    mse = sim.TL_lab("synthetic_tl") if kind == "tl" else sim.ISO_lab("synthetic_iso")
    wall = time.time() - t0
    sims = LOG["sims"]
    draws = []
    for i, s in enumerate(sims):
        end = sims[i + 1]["draw0"] if i + 1 < len(sims) else _draws[0]
        draws.append(end - s["draw0"])
    name = f"lab_{kind}"
    table = LAB_TL if kind == "tl" else LAB_ISO
    out = {f"{name}/cfg": np.frombuffer(json.dumps(cfg_plain).encode(), dtype=np.uint8),
           f"{name}/table": np.frombuffer(json.dumps(table).encode(), dtype=np.uint8),
           f"{name}/seed": np.array(seed), f"{name}/mse": np.array(mse),
           f"{name}/n_sims": np.array(len(sims)), f"{name}/draws": np.array(draws, dtype=np.int64),
           f"{name}/init_draws": np.array(init_draws)}
    for i, s in enumerate(sims):
        out[f"{name}/events{i}"] = np.array(s["events"], dtype=np.int64).reshape(-1, 4)
    print(f"{name}: mse {mse:.6g}, {len(sims)} sims, events {[len(s['events']) for s in sims]}, "
          f"draws {draws}, {wall:.1f}s", flush=True)
    return out


def _read_columns(path):
    """A CSV of numbers as {column: float array}, empty cells as NaN (what
    pandas' read_csv gives for these files)."""
    import csv
    with open(path, newline="") as f:
        rows = list(csv.DictReader(f))
    return {k: np.array([float(r[k]) if r[k] not in ("", None) else np.nan for r in rows])
            for k in rows[0] if k}


# The reference's optimiser in replay mode on its own lab data: the
# min-MSE row of results/lab_sims/result_tl_clbr.csv (optimizer.py:124-132)
# scored by the reference's objective (optimizer.py:82-84 -> run_one_sim ->
# TLTrapSim.TL_lab) against data/processed/CLBR_IRSL50_0.25KperGy.csv, with
# the lab configuration groups.
REAL_LAB = {"replay_tl_clbr": ("tl_clbr", "CLBR_IRSL50_0.25KperGy", "result_tl_clbr.csv", 41)}


def run_lab_real(name):
    import pandas as stub_pd
    import optimizer as ref_opt
    exp, table_name, result_name, seed = REAL_LAB[name]
    table = _read_columns(os.path.join(REF, "data", "processed", table_name + ".csv"))
    stub_pd.register_table(table_name, table)
    res_cols = _read_columns(os.path.join(REF, "results", "lab_sims", result_name))
    mse_col = res_cols["mse"]
    best = int(np.nanargmin(mse_col))   # pandas idxmin: the first minimum, NaN skipped
    best_p = np.array([res_cols[f"param_{i}"][best] for i in range(10)], dtype=np.float64)
    cfg_plain = compose(CONF, ["physics_fp=lab_TL", "exp_type_fp=TLlab"])
    cfg = OmegaConf.create(cfg_plain)
    LOG["sims"] = []
    _draws[0] = 0
    np.random.seed(seed)
    t0 = time.time()
    mse = ref_opt.objective(best_p, cfg, exp)
    wall = time.time() - t0
    sims = LOG["sims"]          # the first is the objective's TLTrapSim constructor
    draws = []
    for i, s in enumerate(sims):
        end = sims[i + 1]["draw0"] if i + 1 < len(sims) else _draws[0]
        draws.append(end - s["draw0"])
    out = {f"{name}/cfg": np.frombuffer(json.dumps(cfg_plain).encode(), dtype=np.uint8),
           f"{name}/table": np.frombuffer(json.dumps({k: v.tolist() for k, v in table.items()}).encode(),
                                          dtype=np.uint8),
           f"{name}/results_mse": mse_col.astype(np.float64), f"{name}/best_params": best_p,
           f"{name}/exp": np.array(exp), f"{name}/seed": np.array(seed), f"{name}/mse": np.array(mse),
           f"{name}/n_sims": np.array(len(sims)), f"{name}/draws": np.array(draws, dtype=np.int64),
           f"{name}/wall_s": np.array(wall)}
    for i, s in enumerate(sims):
        out[f"{name}/events{i}"] = np.array(s["events"], dtype=np.int64).reshape(-1, 4)
    print(f"{name}: mse {mse:.6g}, {len(sims)} sims, events {[len(s['events']) for s in sims]}, "
          f"draws {draws}, {wall:.1f}s", flush=True)
    return out


def main(argv):
    names = argv[1:] or list(CASES) + ["box_ops", "lab_tl", "lab_iso"] + list(REAL_LAB)
    path = os.path.join(HERE, "kinetics_k.npz")
    data = dict(np.load(path)) if os.path.exists(path) else {}
    for n in names:
        data = {k: v for k, v in data.items() if not k.startswith(n + "/")}
        if n == "box_ops":
            data.update(run_box_ops())
        elif n in ("lab_tl", "lab_iso"):
            data.update(run_lab(n[4:], seed=31 if n == "lab_tl" else 32))
        elif n in REAL_LAB:
            data.update(run_lab_real(n))
        else:
            data.update(run_case(n, CASES[n]))
    np.savez_compressed(path, **data)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv)
