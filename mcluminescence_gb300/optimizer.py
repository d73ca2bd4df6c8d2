"""Batched lab-data parameter estimation (the reference's optimiser, batched).

The reference (src/class/optimizer.py) runs scipy's differential evolution over
ten parameters (``DEFAULT_BOUNDS``, optimizer.py:32-43), building a config per
candidate (``cfg_with_params``, optimizer.py:49-65) and scoring it with one
``TL_lab`` or ``ISO_lab`` call (optimizer.py:68-84) -- one simulation per lab
row, one candidate after another (or in a 4-process pool).  Here every
candidate of a generation and every lab row run in ONE launch of the
event-driven kernel (one CTA per simulation, independent Philox streams), and
the DE itself (randtobest1bin, mutation 0.5, recombination 0.3, the reference's
settings) advances on the GPU.  scipy's exact DE trajectory (sobol
initialisation, polishing) is not reproduced; the objective is.
"""
from __future__ import annotations

import copy
import csv
import os
from typing import Any, Dict, List, Sequence, Tuple

import numpy as np

from . import _lib
from .kinetics import TLTrapSim, read_table, run_kinetics, _raise_for

DEFAULT_BOUNDS: List[Tuple[float, float]] = [
    (1e-8, 1e-3),     # rho_prime
    (1.9, 2.4),       # E_cb
    (1.2, 1.7),       # E_loc_1
    (1.0, 1.5),       # E_loc_2
    (1e2, 4e2),       # D0
    (1e12, 1e14),     # s
    (1e10, 1e13),     # b
    (1e9, 5e10),      # alpha
    (1e2, 7.5e2),     # holes
    (0.0, 1.0),       # retrap
]


def cfg_with_params(base: Any, params: Sequence[float]) -> Dict[str, Any]:
    """A copy of ``base`` with the ten fitted parameters replaced (optimizer.py:49-65)."""
    cfg = copy.deepcopy({"exp_type_fp": dict(base["exp_type_fp"]), "physics_fp": dict(base["physics_fp"])})
    (rho_prime, E_cb, E_loc_1, E_loc_2, D0, s, b, alpha, holes, retrap) = params
    cfg["exp_type_fp"]["rho_prime"] = float(rho_prime)
    cfg["exp_type_fp"]["holes"] = float(holes)
    cfg["physics_fp"]["E_cb"] = float(E_cb)
    cfg["physics_fp"]["E_loc_1"] = float(E_loc_1)
    cfg["physics_fp"]["E_loc_2"] = float(E_loc_2)
    cfg["physics_fp"]["D0"] = float(D0)
    cfg["physics_fp"]["s"] = float(s)
    cfg["physics_fp"]["b"] = float(b)
    cfg["physics_fp"]["alpha"] = float(alpha)
    cfg["physics_fp"]["Retrap"] = float(retrap)
    return cfg


def _lab_sims(cfg, table: Dict[str, np.ndarray], kind: str):
    """Simulation parameters of one candidate's lab objective, and its targets."""
    sim = TLTrapSim(cfg, rng="philox")
    params, targets = [], []
    if kind == "tl":
        for k in range(len(table["Duration"])):
            params.append(sim._params(table["e_ratio"][k], table["T_start"][k],
                                      (table["T_end"][k] - table["T_start"][k]) / table["Duration"][k],
                                      table["Duration"][k], sim.D, _lib.MCL_LOOP_LAB_TL))
            targets.append(table["Fill"][k])
    else:
        order = []
        for v in table["exp_no"]:
            if v not in order:
                order.append(v)
        for exp_no in sorted(order):
            m = table["exp_no"] == exp_no
            sub = {k: v[m] for k, v in table.items()}
            obs = sub["time"].astype(np.float64)
            params.append(sim._params(sub["e_ratio"][0], sub["temp"][0], 0.0, 0.0, sub["dose"][0],
                                      _lib.MCL_LOOP_LAB_ISO, obs))
            targets.append(np.array([sub["e_ratio"][sub["time"] == o][0] for o in obs]))
    return params, targets


def lab_objective_batch(base_cfg: Any, candidates: np.ndarray, table, kind: str = "tl",
                        seed: int = 0, steps: int = 4096) -> np.ndarray:
    """MSE of every candidate (rows of ``candidates``, the ten parameters in
    DEFAULT_BOUNDS order) against the lab table: all candidates and rows in
    one launch."""
    tb = read_table(table)
    all_params, spans, targets = [], [], []
    for c in candidates:
        p, t = _lab_sims(cfg_with_params(base_cfg, c), tb, kind)
        spans.append((len(all_params), len(p)))
        all_params += p
        targets.append(t)
    while True:
        res, _ = run_kinetics(all_params, steps, rng="philox", seed=seed, want_events=False)
        if np.any(res.status == _lib.MCL_EOVERFLOW) and steps < 1 << 22:
            steps *= 4
            continue
        break
    _raise_for(res.status, steps)
    out = np.empty(len(candidates))
    for ci, (o, n) in enumerate(spans):
        if kind == "tl":
            finals = np.array([res.electron_ratio[int(res.n_steps[o + j]) - 1, o + j] for j in range(n)])
            out[ci] = np.mean((finals - np.asarray(targets[ci])) ** 2)
        else:
            err = np.concatenate([res.obs_ratio[o + j] - targets[ci][j] for j in range(n)])
            out[ci] = np.mean(err ** 2)
    return out


def optimize(base_cfg: Any, table, kind: str = "tl", gens: int = 7, popsize: int = 15,
             seed: int = 0, bounds: Sequence[Tuple[float, float]] = DEFAULT_BOUNDS,
             mutation: float = 0.5, recombination: float = 0.3):
    """Differential evolution (randtobest1bin) over ``bounds`` with the whole
    population scored per launch; population = popsize x dimensions like
    scipy.  Returns (best parameters, best MSE, best MSE per generation)."""
    rng = np.random.default_rng(seed)
    lo = np.array([b[0] for b in bounds])
    hi = np.array([b[1] for b in bounds])
    D = len(bounds)
    P = popsize * D
    x = rng.random((P, D))
    f = lab_objective_batch(base_cfg, lo + (hi - lo) * x, table, kind, seed=seed)
    hist = [float(f.min())]
    for g in range(gens):
        best = int(np.argmin(f))
        trial = np.empty_like(x)
        for i in range(P):
            r0, r1, r2 = rng.choice([j for j in range(P) if j != i], 3, replace=False)
            mutant = x[r0] + mutation * (x[best] - x[r0]) + mutation * (x[r1] - x[r2])
            cross = rng.random(D) < recombination
            cross[rng.integers(D)] = True
            t = np.where(cross, mutant, x[i])
            bad = (t < 0) | (t > 1)
            t[bad] = rng.random(int(bad.sum()))
            trial[i] = t
        ft = lab_objective_batch(base_cfg, lo + (hi - lo) * trial, table, kind, seed=seed + g + 1)
        better = ft <= f
        x[better] = trial[better]
        f[better] = ft[better]
        hist.append(float(f.min()))
    best = int(np.argmin(f))
    return lo + (hi - lo) * x[best], float(f[best]), hist


def append_result(csv_path: str, params: Sequence[float], mse: float) -> None:
    """Append one result row as optimizer.py:113-117 does (param_0..param_9, mse)."""
    exists = os.path.exists(csv_path)
    with open(csv_path, "a", newline="") as f:
        w = csv.writer(f)
        if not exists:
            w.writerow([f"param_{i}" for i in range(len(params))] + ["mse"])
        w.writerow([repr(float(p)) for p in params] + [repr(float(mse))])
