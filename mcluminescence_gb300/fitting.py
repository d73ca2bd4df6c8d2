"""Batched parameter estimation: many glow-curve fits at once on one GPU.

The reference fits one parameter set at a time with scipy's differential
evolution (src/class/optimizer.py:93-111: strategy randtobest1bin, mutation
0.5, recombination 0.3), evaluating every candidate with a full Monte Carlo
simulation (``objective``, optimizer.py:82-84).  Here all fits and all
candidates of a generation are evaluated together:

* ``fit_plain_mc``     the same DE, every candidate scored by the batched
                       Monte Carlo kernel;
* ``fit_surrogate``    the DE runs on the learned surrogate (no Monte Carlo),
                       its best candidates are re-simulated by the Monte
                       Carlo and accepted only if their MSE is within the
                       Monte Carlo noise floor; fits that fail continue with
                       Monte-Carlo-scored DE from the surrogate's population.

Both methods stop each fit on the same criterion: the first Monte Carlo
evaluation at or below ``accept_factor`` x the fit's noise floor (1.0 by
default: the expected MSE of the true parameters).  An accepted fit is frozen
and costs no further Monte Carlo.

The objective is the mean squared difference of area-normalised curves over
the 200 bins, for the four free parameters (E, log10 s, alpha, log10 rho');
dose and heating rate are the known experimental conditions.  Targets are
Monte Carlo curves at hidden parameters scaled to a peak of ~1e4 counts with
Poisson counting noise.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Dict

import numpy as np

from . import _lib
from . import surrogate as S

FREE = 4  # E, log10 s, alpha, log10 rho'


def pack_curves(params: np.ndarray, n_traps: int, id0: int = 0):
    """Packed host arrays of the surrogate's curve family (one TL segment per
    set), built column-wise: ``surrogate.pack_curves``."""
    return S.pack_curves(params, id0, n_traps)


def mc_curves(params: np.ndarray, n_traps: int, seed: int, id0: int = 0):
    """Monte Carlo curves (counts) as a float32 device tensor [n][200]."""
    from .batch import BernoulliBatch
    b = BernoulliBatch(None, packed=pack_curves(params, n_traps, id0), precision="fp32", seed=seed,
                       want_alive=False, block=128, ept=8)
    b.launch()
    st = b.status()
    if st:
        raise _lib.MclError(st, "kinetics kernel reported", detail=False)
    return b.d_lum[:len(params) * S.N_BINS].view(len(params), S.N_BINS).float()


def normalized(c):
    return c / c.sum(dim=-1, keepdim=True).clamp_min(1e-30)


def mse(curves, target_norm):
    """Mean over bins of the squared difference of area-normalised curves,
    scaled by n_bins^2 so a perfect shape match is O(noise)."""
    return ((normalized(curves) - target_norm) ** 2).mean(dim=-1) * S.N_BINS ** 2


@dataclass
class Problem:
    hidden: np.ndarray          # [F][4] true free parameters
    known: np.ndarray           # [F][2] log10 dose, log10 beta
    target: object              # device [F][200] counts (Poisson)
    target_norm: object         # device [F][200]
    floor: object               # device [F] expected MSE at the truth (Poisson + MC noise)
    n_traps_eval: int


def make_problem(n_fits: int, seed: int, n_traps_eval: int = 20000, n_traps_target: int = 200000,
                 peak: float = 1e4) -> Problem:
    """Targets: Monte Carlo at hidden parameters (drawn from the surrogate's
    ranges, curves with a visible peak only) with Poisson noise at ~peak counts."""
    import torch
    rng = np.random.default_rng(seed)
    out_h, out_k = [], []
    while sum(len(h) for h in out_h) < n_fits:
        p = S.sample_params(4 * n_fits, rng)
        curves = mc_curves(p, 4000, seed=seed + 1, id0=50_000_000).cpu().numpy()
        tot = curves.sum(axis=1)
        pk = curves.argmax(axis=1)
        ok = (tot > 400) & (pk > 10) & (pk < S.N_BINS - 10)
        out_h.append(p[ok, :FREE])
        out_k.append(p[ok, FREE:])
    hidden = np.concatenate(out_h)[:n_fits]
    known = np.concatenate(out_k)[:n_fits]
    full = np.concatenate([hidden, known], axis=1)
    clean = mc_curves(full, n_traps_target, seed=seed + 2, id0=60_000_000)
    scale = peak / clean.max(dim=1, keepdim=True).values.clamp_min(1.0)
    g = torch.Generator(device=clean.device).manual_seed(seed + 3)
    target = torch.poisson(clean * scale, generator=g)
    tn = normalized(target)
    lam = target.sum(dim=1)
    # expected events of an evaluation curve at the truth
    n_ev = clean.sum(dim=1) * (n_traps_eval / n_traps_target)
    floor = (tn * (1 - tn) * (1.0 / lam[:, None] + 1.0 / n_ev.clamp_min(1.0)[:, None])).mean(dim=1) * S.N_BINS ** 2
    return Problem(hidden, known, target, tn, floor, n_traps_eval)


def to_params(u, known):
    """Unit-cube free parameters [F][P][4] + known [F][2] -> full [F*P][6] (host)."""
    lo, hi = S.LOW[:FREE], S.HIGH[:FREE]
    F, P, _ = u.shape
    x = lo + (hi - lo) * u
    k = np.broadcast_to(known[:, None, :], (F, P, 2))
    return np.concatenate([x, k], axis=2).reshape(F * P, 6)


class DE:
    """Batched differential evolution (randtobest1bin: mutant = x_r0 +
    F (x_best - x_r0) + F (x_r1 - x_r2), binomial crossover with one forced
    dimension), all fits advancing together.  Unit-cube coordinates;
    out-of-bounds trial coordinates are redrawn uniformly."""

    def __init__(self, n_fits: int, pop: int, dim: int, seed: int, mutation: float = 0.5,
                 recombination: float = 0.3, init=None):
        import torch
        self.t = torch
        self.g = torch.Generator(device="cuda").manual_seed(seed)
        self.F, self.P, self.D = n_fits, pop, dim
        self.mut, self.cr = mutation, recombination
        self.x = init if init is not None else torch.rand(n_fits, pop, dim, device="cuda", generator=self.g)
        self.f = None

    def trials(self):
        t, F, P, D = self.t, self.F, self.P, self.D
        best = self.f.argmin(dim=1)
        xb = self.x[t.arange(F, device="cuda"), best][:, None, :]
        keys = t.rand(F, P, P, device="cuda", generator=self.g)
        keys[:, t.arange(P), t.arange(P)] = 2.0          # exclude the target vector itself
        r = keys.argsort(dim=2)[:, :, :3]
        gather = lambda idx: t.gather(self.x, 1, idx[..., None].expand(F, P, D))
        x0, x1, x2 = gather(r[..., 0]), gather(r[..., 1]), gather(r[..., 2])
        mutant = x0 + self.mut * (xb - x0) + self.mut * (x1 - x2)
        cross = t.rand(F, P, D, device="cuda", generator=self.g) < self.cr
        jr = t.randint(0, D, (F, P), device="cuda", generator=self.g)
        cross.scatter_(2, jr[..., None], True)
        trial = t.where(cross, mutant, self.x)
        bad = (trial < 0) | (trial > 1)
        trial = t.where(bad, t.rand(F, P, D, device="cuda", generator=self.g), trial)
        return trial

    def select(self, trial, f_trial):
        better = f_trial <= self.f
        self.x = self.t.where(better[..., None], trial, self.x)
        self.f = self.t.where(better, f_trial, self.f)


def _quartiles(r) -> list:
    r = np.asarray(r, dtype=np.float64)
    return [float(q) for q in np.quantile(r, [0.25, 0.5, 0.75])] if r.size else []


@dataclass
class FitReport:
    method: str
    seconds: float
    accepted: int
    n_fits: int
    mc_curves: int
    mc_trials: float
    final_ratio_median: float     # MC-verified MSE / noise floor, median over fits
    accepted_ratio_median: float
    history: list = field(default_factory=list)
    best_x: object = None         # [F][4] unit-cube parameters of each fit's answer
    reverified_ratio_median: float = float("nan")   # fresh, independent MC of the answers
    final_ratios: object = None   # [F] MC-verified MSE / floor of each answer
    reverified_ratios: object = None
    accept_factor: float = 1.0

    @property
    def fits_per_s(self) -> float:
        return self.accepted / self.seconds if self.seconds > 0 else 0.0

    def as_dict(self) -> Dict:
        return {"method": self.method, "seconds": self.seconds, "accepted": self.accepted,
                "n_fits": self.n_fits, "fits_per_s": self.fits_per_s, "mc_curves": self.mc_curves,
                "mc_trials": self.mc_trials, "accept_factor": self.accept_factor,
                "final_mse_over_floor_median": self.final_ratio_median,
                "final_mse_over_floor_quartiles": _quartiles(self.final_ratios if self.final_ratios is not None else []),
                "accepted_mse_over_floor_median": self.accepted_ratio_median,
                "reverified_mse_over_floor_median": self.reverified_ratio_median,
                "reverified_mse_over_floor_quartiles": _quartiles(
                    self.reverified_ratios if self.reverified_ratios is not None else [])}


def _mc_eval(prob: Problem, u, seed: int, id0: int):
    F, P, _ = u.shape
    full = to_params(u.cpu().numpy(), prob.known)
    c = mc_curves(full, prob.n_traps_eval, seed=seed, id0=id0)
    tn = prob.target_norm.repeat_interleave(P, dim=0)
    trials = float(prob.n_traps_eval) * float(np.sum(_steps(full)))
    return mse(c, tn).view(F, P), trials


def _steps(full):
    beta = 10.0 ** full[:, 5]
    k = np.maximum(1, np.ceil(S.BIN_C / (beta * 0.1) - 1e-9))
    return S.N_BINS * k


def _mc_de(prob: Problem, de: DE, thr, max_gens: int, seed: int, id0: int, hist: list, hist_base: int = 0):
    """Monte-Carlo-scored DE generations until every fit has a member at or
    below ``thr`` (or ``max_gens``).  A fit that gets there is frozen: its
    population stops evolving and costs no further Monte Carlo.  ``de.f``
    must hold the population's Monte Carlo scores.  Returns (curves, trials)."""
    import torch
    F, P = de.F, de.P
    n_curves, n_trials = 0, 0.0
    done = de.f.min(dim=1).values <= thr
    for g in range(max_gens):
        hist.append(hist_base + int(done.sum()))
        if bool(done.all()):
            break
        trial = de.trials()
        idx = (~done).nonzero().flatten()
        f_sub, tr = _mc_eval(_subproblem(prob, idx), trial[idx], seed + 17 * (g + 1), id0=id0 + g * F * P)
        f_trial = torch.full_like(de.f, float("inf"))
        f_trial[idx] = f_sub
        n_curves += len(idx) * P
        n_trials += tr
        de.select(trial, f_trial)
        done = done | (de.f.min(dim=1).values <= thr)
    return n_curves, n_trials


def fit_plain_mc(prob: Problem, pop: int = 32, max_gens: int = 60, seed: int = 0,
                 accept_factor: float = 1.0) -> FitReport:
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    F = len(prob.known)
    de = DE(F, pop, FREE, seed)
    de.f, n_trials = _mc_eval(prob, de.x, seed, id0=1_000_000)
    n_curves = F * pop
    thr = accept_factor * prob.floor
    hist = []
    c, t = _mc_de(prob, de, thr, max_gens, seed, 2_000_000, hist)
    n_curves += c
    n_trials += t
    best = de.f.min(dim=1).values
    best_x = de.x[torch.arange(F, device="cuda"), de.f.argmin(dim=1)]
    acc = best <= thr
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    ratio = (best / prob.floor).cpu().numpy()
    return FitReport("plain_mc", secs, int(acc.sum()), F, n_curves, n_trials,
                     float(np.median(ratio)), float(np.median(ratio[acc.cpu().numpy()])) if bool(acc.any()) else float("nan"),
                     hist, best_x, final_ratios=ratio, accept_factor=accept_factor)


def _surrogate_curves(model, u, known_t):
    """Area-normalised surrogate curves of unit-cube candidates u [F][P][4]."""
    import torch
    F, P, _ = u.shape
    lo = S.dev_const("LOW_FREE", S.LOW[:FREE], torch.float32, u.device)
    hi = S.dev_const("HIGH_FREE", S.HIGH[:FREE], torch.float32, u.device)
    x = lo + (hi - lo) * u
    full = torch.cat([x, known_t[:, None, :].expand(F, P, 2)], dim=2).reshape(F * P, 6)
    y = S.predict_t(model, full)
    return normalized((10.0 ** y - S.EPS_Y).clamp_min(0.0)).view(F, P, S.N_BINS)


def _surrogate_eval(model: "S.SurrogateMLP", prob: Problem, u, known_t, delta=None):
    """Surrogate MSE of unit-cube candidates, all on the device.  ``delta``
    [F][200] is a per-fit correction of the normalised curve: the Monte Carlo
    minus surrogate residual at a verified point (space mapping), which
    removes most of the surrogate's local bias."""
    c = _surrogate_curves(model, u, known_t)
    if delta is not None:
        c = c + delta[:, None, :]
    return ((c - prob.target_norm[:, None, :]) ** 2).mean(dim=-1) * S.N_BINS ** 2


def _surrogate_round(model, prob, known_t, pop, gens, seed, init=None, delta=None):
    de = DE(len(prob.known), pop, FREE, seed, init=init)
    de.f = _surrogate_eval(model, prob, de.x, known_t, delta)
    for _ in range(gens):
        trial = de.trials()
        de.select(trial, _surrogate_eval(model, prob, trial, known_t, delta))
    return de


def _subproblem(prob: Problem, idx):
    i = idx.cpu().numpy()
    return Problem(prob.hidden[i], prob.known[i], prob.target[idx], prob.target_norm[idx],
                   prob.floor[idx], prob.n_traps_eval)


def fit_surrogate(prob: Problem, model: "S.SurrogateMLP", pop: int = 32, sur_gens: int = 120,
                  refine_gens: int = 60, verify_top: int = 8, rounds: int = 6, max_mc_gens: int = 60,
                  seed: int = 0, accept_factor: float = 1.0) -> FitReport:
    """Surrogate-proposed, Monte-Carlo-verified fitting.

    Round 1: DE on the surrogate for ``sur_gens`` generations, the
    ``verify_top`` best candidates of each fit re-simulated by the Monte Carlo;
    a fit is accepted when one of them is within ``accept_factor`` x its noise
    floor.  Later rounds (fits still open only) continue the surrogate DE for
    ``refine_gens`` generations with the surrogate corrected by the Monte
    Carlo residual at the fit's best verified candidate, then verify again.
    Fits still open after ``rounds`` rounds continue with Monte-Carlo-scored
    DE (the plain method) for at most ``max_mc_gens`` generations."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    F = len(prob.known)
    model = model.inference_copy(F * pop)   # every candidate of a generation in one forward pass
    thr = accept_factor * prob.floor
    best = torch.full((F,), float("inf"), device="cuda")
    open_idx = torch.arange(F, device="cuda")
    known_all = torch.tensor(prob.known, dtype=torch.float32, device="cuda")
    pop_x = None
    delta = None
    best_x = torch.zeros(F, FREE, device="cuda")
    n_curves, n_trials, hist = 0, 0.0, []
    for r in range(rounds):
        sub = _subproblem(prob, open_idx)
        known_t = known_all[open_idx]
        de = _surrogate_round(model, sub, known_t, pop, sur_gens if r == 0 else refine_gens,
                              seed + 101 * r, init=pop_x, delta=delta)
        order = de.f.argsort(dim=1)[:, :verify_top]
        cand = torch.gather(de.x, 1, order[..., None].expand(len(open_idx), verify_top, FREE))
        full = to_params(cand.cpu().numpy(), sub.known)
        curves = mc_curves(full, prob.n_traps_eval, seed=seed + 5 + r, id0=3_000_000 + r * 1_000_000)
        n_curves += len(open_idx) * verify_top
        n_trials += float(prob.n_traps_eval) * float(np.sum(_steps(full)))
        cn = normalized(curves).view(len(open_idx), verify_top, S.N_BINS)
        f_mc = ((cn - sub.target_norm[:, None, :]) ** 2).mean(dim=-1) * S.N_BINS ** 2
        jbest = f_mc.argmin(dim=1)
        b = f_mc.min(dim=1).values
        ar = torch.arange(len(open_idx), device="cuda")
        improved = b < best[open_idx]
        best_x[open_idx[improved]] = cand[ar, jbest][improved]
        best[open_idx] = torch.minimum(best[open_idx], b)
        still = best[open_idx] > thr[open_idx]
        # residual at each fit's best verified candidate, for the next round
        xbest = cand[ar, jbest][:, None, :]
        sbest = _surrogate_curves(model, xbest, known_t)[:, 0, :]
        delta = (cn[ar, jbest] - sbest)[still]
        pop_x = de.x[still]
        open_idx = open_idx[still]
        hist.append(F - len(open_idx))
        if len(open_idx) == 0:
            break
    if len(open_idx):
        sub = _subproblem(prob, open_idx)
        de2 = DE(len(open_idx), pop, FREE, seed + 1, init=pop_x.clone())
        de2.f, tr = _mc_eval(sub, de2.x, seed + 7, id0=8_000_000)
        n_curves += len(open_idx) * pop
        n_trials += tr
        c, t = _mc_de(sub, de2, thr[open_idx], max_mc_gens, seed + 14, 9_000_000, hist,
                      hist_base=F - len(open_idx))
        n_curves += c
        n_trials += t
        b2 = de2.f.min(dim=1).values
        x2 = de2.x[torch.arange(len(open_idx), device="cuda"), de2.f.argmin(dim=1)]
        improved = b2 < best[open_idx]
        best_x[open_idx[improved]] = x2[improved]
        best[open_idx] = torch.minimum(best[open_idx], b2)
    acc = best <= thr
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    ratio = (best / prob.floor).cpu().numpy()
    return FitReport("surrogate_mc", secs, int(acc.sum()), F, n_curves, n_trials,
                     float(np.median(ratio)), float(np.median(ratio[acc.cpu().numpy()])) if bool(acc.any()) else float("nan"),
                     hist, best_x, final_ratios=ratio, accept_factor=accept_factor)


def reverify(prob: Problem, rep: FitReport, seed: int = 999) -> FitReport:
    """Score every fit's answer once more with a fresh, independent Monte
    Carlo run (the minimum over a DE population is biased low by the noise of
    the evaluations it was selected on); fills ``reverified_ratio_median``."""
    f, _ = _mc_eval(prob, rep.best_x[:, None, :], seed, id0=90_000_000)
    rep.reverified_ratios = (f[:, 0] / prob.floor).cpu().numpy()
    rep.reverified_ratio_median = float(np.median(rep.reverified_ratios))
    return rep
