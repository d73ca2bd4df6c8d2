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

The reference's entry point (optimizer.py:89-136) is ``main``: ``task="train"``
runs the batched DE and appends the best row to
``results/lab_sims/result_{exp}.csv`` (param_0..param_9, mse);
``task="replay"`` reads that file, takes its minimum-MSE row and scores it
again with one ``TL_lab`` / ``ISO_lab`` call.  Lab tables are found by name as
the reference finds them (``data/processed/<name>.csv``, optimizer.py:73-78).
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


# optimizer.py:68-80: the lab experiment behind each ``exp`` label
EXPERIMENTS = {"iso": ("iso", "CLBR_IR50_ISO"),
               "tl_clbr": ("tl", "CLBR_IRSL50_0.25KperGy"),
               "tl_fsm-13": ("tl", "FSM-13_IRSL50_0.25KperGy")}


def project_root() -> str:
    """The directory ``results/`` and ``data/`` hang from (the reference's
    PROJECT_ROOT, src/class/paths.py): ``MCL_PROJECT_ROOT`` if set, else the
    current directory."""
    return os.environ.get("MCL_PROJECT_ROOT") or os.getcwd()


def result_path(exp: str) -> str:
    """results/lab_sims/result_{exp}.csv (optimizer.py:99)."""
    return os.path.join(project_root(), "results", "lab_sims", f"result_{exp}.csv")


def run_one_sim(cfg: Any, exp: str, plot: bool = False, rng: str = "numpy") -> float:
    """MSE of one parameter set on one lab experiment (optimizer.py:68-80):
    the first run of ``cfg`` in a ``TLTrapSim``, then ``ISO_lab`` or
    ``TL_lab`` on the experiment's table."""
    from .config import initialize_runs
    if exp not in EXPERIMENTS:
        raise ValueError(f"Unknown exp '{exp}'")
    kind, name = EXPERIMENTS[exp]
    sim = TLTrapSim(initialize_runs(cfg)[0], rng=rng)
    return sim.ISO_lab(name, plot=plot) if kind == "iso" else sim.TL_lab(name, plot=plot)


def objective(p: Sequence[float], cfg: Any, exp: str) -> float:
    """optimizer.py:82-84: the MSE of parameter vector ``p`` (DEFAULT_BOUNDS order)."""
    return run_one_sim(cfg_with_params(cfg, p), exp)


def read_results(csv_path: str) -> Dict[str, np.ndarray]:
    """A result table as float columns, empty cells as NaN (how the
    reference's pandas reads them; its files mix rows with fewer parameters
    and an extra trailing column)."""
    with open(csv_path, newline="") as f:
        rows = list(csv.DictReader(f))
    if not rows:
        raise ValueError(f"{csv_path} has no result rows")
    return {k: np.array([float(r[k]) if r.get(k) not in ("", None) else np.nan for r in rows])
            for k in rows[0] if k}


def best_result(csv_path: str) -> Tuple[np.ndarray, float]:
    """The parameters and MSE of the row with the smallest MSE (the first one
    on ties, NaN rows skipped), as optimizer.py:128-130 picks it: every
    ``param_*`` column in order, NaN where the row left a cell empty."""
    cols = read_results(csv_path)
    mse = cols["mse"]
    if np.all(np.isnan(mse)):
        raise ValueError(f"{csv_path} has no row with an MSE")
    i = int(np.nanargmin(mse))
    names = sorted((k for k in cols if k.startswith("param_")), key=lambda k: int(k.split("_")[1]))
    return np.array([cols[k][i] for k in names], dtype=np.float64), float(mse[i])


def replay(cfg: Any, exp: str, csv_path: str = None, plot: bool = False) -> float:
    """``task=replay`` (optimizer.py:124-133): score the best row of the
    experiment's result file once more; returns the MSE."""
    path = csv_path or result_path(exp)
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    best_p, _ = best_result(path)
    return run_one_sim(cfg_with_params(cfg, best_p), exp, plot=plot)


def main(cfg: Any, task: str = None, exp: str = None, gens: int = None, pop: int = None,
         seed: int = 0) -> float:
    """The reference's dispatcher (optimizer.py:89-136) with its defaults
    (task "train", exp "tl_clbr", gens 7, pop 15, read from ``cfg`` like the
    reference's command-line overrides).  ``train`` runs the batched DE,
    appends the best row to ``result_path(exp)`` and scores it once more;
    ``replay`` re-scores the file's best row.  Returns that score."""
    task = task or _get_key(cfg, "task", "train")
    exp = exp or _get_key(cfg, "exp", "tl_clbr")
    gens = int(gens if gens is not None else _get_key(cfg, "gens", 7))
    pop = int(pop if pop is not None else _get_key(cfg, "pop", 15))
    path = result_path(exp)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    if task == "train":
        from .config import initialize_runs
        kind, name = EXPERIMENTS[exp]
        x, f, _ = optimize(initialize_runs(cfg)[0], name, kind, gens=gens, popsize=pop, seed=seed)
        append_result(path, x, f)
        return run_one_sim(cfg_with_params(cfg, x), exp)
    if task == "replay":
        return replay(cfg, exp, path)
    raise ValueError("task must be 'train' or 'replay'")


def _get_key(cfg, k, default):
    try:
        return cfg.get(k, default)
    except AttributeError:
        return getattr(cfg, k, default)


def _lab_sims(cfg, table: Dict[str, np.ndarray], kind: str, rng: str = "philox"):
    """Simulation parameters of one candidate's lab objective, and its
    targets.  With ``rng="numpy"`` the candidate's TLTrapSim constructor
    draws its box from numpy's global stream, as the reference's does."""
    sim = TLTrapSim(cfg, rng=rng)
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


def _mse_of(kind, res, o, n, targets):
    if kind == "tl":
        finals = np.array([res.electron_ratio[int(res.n_steps[o + j]) - 1, o + j] for j in range(n)])
        return float(np.mean((finals - np.asarray(targets)) ** 2))
    err = np.concatenate([res.obs_ratio[o + j] - targets[j] for j in range(n)])
    return float(np.mean(err ** 2))


def lab_objective_batch(base_cfg: Any, candidates: np.ndarray, table, kind: str = "tl",
                        seed: int = 0, steps: int = 4096, rng: str = "philox") -> np.ndarray:
    """MSE of every candidate (rows of ``candidates``, the ten parameters in
    DEFAULT_BOUNDS order) against the lab table.

    ``rng="philox"``: all candidates and rows in one launch, each simulation
    on its own counter-based stream keyed by ``seed``.  ``rng="numpy"``: the
    reference's stream -- candidate after candidate, each one's constructor
    draws, then its rows in one launch continuing numpy's global stream -- so
    one candidate scores exactly as ``TLTrapSim(cfg).TL_lab(table)`` (or
    ``ISO_lab``) does after the same ``np.random.seed``."""
    tb = read_table(table)
    if rng == "numpy":
        out = np.empty(len(candidates))
        for ci, c in enumerate(candidates):
            p, t = _lab_sims(cfg_with_params(base_cfg, c), tb, kind, rng="numpy")
            n_steps = steps
            while True:
                state0 = np.random.get_state()
                res, new_state = run_kinetics(p, n_steps, rng="mt19937", mt_state=state0, want_events=False)
                if np.any(res.status == _lib.MCL_EOVERFLOW) and n_steps < 1 << 24:
                    n_steps *= 4
                    continue
                break
            np.random.set_state(("MT19937", new_state[1], new_state[2], state0[3], state0[4]))
            _raise_for(res.status, n_steps)
            out[ci] = _mse_of(kind, res, 0, len(p), t)
        return out
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
        out[ci] = _mse_of(kind, res, o, n, targets[ci])
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
    """Append one result row as optimizer.py:113-117 does: columns
    param_0..param_{n-1}, mse, the header only when the file is new, values as
    the reference's pandas writes float64 (shortest round-trip repr),
    ``os.linesep`` line ends."""
    exists = os.path.exists(csv_path)
    vals = np.array([float(p) for p in params] + [float(mse)], dtype=np.float64).astype(str)
    with open(csv_path, "a", newline="") as f:
        if not exists:
            f.write(",".join([f"param_{i}" for i in range(len(params))] + ["mse"]) + os.linesep)
        f.write(",".join(vals) + os.linesep)
