"""Parameter sets and their time schedules for the batched (Bernoulli) mode.

A *set* is one sample of trap physics -- trap depth E, frequency factor s,
tunnelling coefficient alpha on the dimensionless centre distance r', a number
of trap slots -- run through a schedule of *segments*: TL ramps, isothermal
holds, irradiation, fading, optical stimulation.  Events are counted into the
set's bins (1 degC bins for a TL ramp, fixed time bins otherwise).

The physics is the dilute limit of the reference's kinetics:
``b * exp(-E_loc/(k_b T) - alpha*d)`` (src/class/engine.py:69-73) with
``alpha*d = rho'^(-1/3) * r'`` for the box geometry of
src/class/tl_trap_lab.py:33-35, so ``alpha_dimless = rho'^(-1/3)`` unless a set
gives its own.  Temperatures are evaluated at the start of each step, like
``T_now`` in src/class/simulate.py:53-55.

Workload builders reproduce the shapes of the benchmark configurations:
``single_tl_set`` (one TL set: 2,000 traps, E = 1.45 eV, s = 3.5e12 /s,
rho' = 1e-6, 0 -> 500 degC at 1 K/s, dt = 0.1 s), ``batch_tl_iso`` (4,096 sets,
half TL ramps and half isothermal holds, ragged 1e3..1e5 traps) and
``batch_dose_fade_irsl`` (2,048 irradiation -> fading -> IR stimulation sets).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import numpy as np

K_B = 8.617333262145e-5   # eV/K (src/class/engine.py:60)
C_TO_K = 273.15


@dataclass
class Segment:
    n_steps: int
    dt: float
    steps_per_bin: int
    T0: float = C_TO_K            # K at the segment start
    beta: float = 0.0             # K/s
    thermal: bool = True          # include s*exp(-E/(k_b T))
    rate_const: float = 0.0       # optical sigma*Phi or ground-state s_tun, 1/s
    fill_rate: float = 0.0        # dose rate / D0, 1/s
    dt_growth: float = 1.0        # geometric growth of dt per step
    bin_offset: int = 0           # assigned by SetSpec.finalize()

    @property
    def n_bins(self) -> int:
        return -(-int(self.n_steps) // int(self.steps_per_bin))

    def to_dict(self) -> dict:
        return dict(n_steps=int(self.n_steps), dt=float(self.dt),
                    steps_per_bin=int(self.steps_per_bin), T0=float(self.T0),
                    beta=float(self.beta), thermal=bool(self.thermal),
                    rate_const=float(self.rate_const), fill_rate=float(self.fill_rate),
                    dt_growth=float(self.dt_growth), bin_offset=int(self.bin_offset))


@dataclass
class SetSpec:
    n_slots: int
    E: float
    s: float
    alpha: float
    segments: List[Segment]
    n_filled: Optional[int] = None    # default: all slots filled
    set_id: int = 0
    k_b: float = K_B
    kind: str = ""

    def finalize(self) -> "SetSpec":
        b = 0
        for sg in self.segments:
            sg.bin_offset = b
            b += sg.n_bins
        if self.n_filled is None:
            self.n_filled = self.n_slots
        return self

    @property
    def n_bins(self) -> int:
        return int(sum(sg.n_bins for sg in self.segments))

    @property
    def total_steps(self) -> int:
        return int(sum(int(sg.n_steps) for sg in self.segments))

    @property
    def trials(self) -> int:
        """Electron-step trials one run performs (slots x steps)."""
        return int(self.n_slots) * self.total_steps

    def to_dict(self) -> dict:
        self.finalize()
        return dict(n_slots=int(self.n_slots), n_filled=int(self.n_filled), E=float(self.E),
                    s=float(self.s), alpha=float(self.alpha), k_b=float(self.k_b),
                    set_id=int(self.set_id), n_bins=self.n_bins,
                    segments=[sg.to_dict() for sg in self.segments])


# ---------------------------------------------------------------------------
# segment builders
# ---------------------------------------------------------------------------
def tl_ramp(T_start_C: float, T_end_C: float, beta: float, dt: float,
            bin_width_C: float = 1.0) -> Segment:
    """Linear heating; bins of ``bin_width_C`` degC (an integer number of steps)."""
    n = int(round((T_end_C - T_start_C) / (beta * dt)))
    spb = int(round(bin_width_C / (beta * dt)))
    if spb < 1 or abs(spb * beta * dt - bin_width_C) > 1e-9 * max(1.0, bin_width_C):
        raise ValueError("the bin width must be a whole number of steps")
    return Segment(n_steps=n, dt=dt, steps_per_bin=spb, T0=T_start_C + C_TO_K, beta=beta)


def isothermal(T_C: float, duration: float, dt: float, bin_seconds: float) -> Segment:
    n = int(round(duration / dt))
    spb = int(round(bin_seconds / dt))
    return Segment(n_steps=n, dt=dt, steps_per_bin=max(spb, 1), T0=T_C + C_TO_K, beta=0.0)


def irradiate(dose_Gy: float, dose_rate: float, D0: float, dt: float, T_C: float = 20.0,
              bin_seconds: Optional[float] = None) -> Segment:
    """Filling at dose rate D (Gy/s): empty traps fill with rate D/D0, giving the
    saturating occupancy 1 - exp(-dose/D0) (src/class/tl_trap_lab.py:53-60)."""
    duration = dose_Gy / dose_rate
    n = max(1, int(round(duration / dt)))
    spb = n if bin_seconds is None else max(1, int(round(bin_seconds / dt)))
    return Segment(n_steps=n, dt=duration / n, steps_per_bin=spb, T0=T_C + C_TO_K,
                   fill_rate=dose_rate / D0)


def fade(duration: float, n_steps: int, s_tun: float, dt0: float = 1.0, T_C: float = 20.0,
         steps_per_bin: int = 10) -> Segment:
    """Ground-state tunnelling (anomalous fading) at rate s_tun*exp(-alpha r')
    (src/est_params/functions.py:108-112) with geometrically growing steps
    whose lengths sum to ``duration``."""
    g = _growth_for(duration, dt0, n_steps)
    return Segment(n_steps=n_steps, dt=dt0, dt_growth=g, steps_per_bin=steps_per_bin,
                   T0=T_C + C_TO_K, thermal=False, rate_const=s_tun)


def optical(sigma_phi: float, duration: float, dt: float, T_C: float = 50.0,
            bin_seconds: float = 1.0, thermal: bool = True) -> Segment:
    """Constant optical stimulation (IRSL/OSL) at rate sigma*Phi per trap,
    scaled by exp(-alpha r'), plus the thermal rate at T_C."""
    n = int(round(duration / dt))
    return Segment(n_steps=n, dt=dt, steps_per_bin=max(1, int(round(bin_seconds / dt))),
                   T0=T_C + C_TO_K, thermal=thermal, rate_const=sigma_phi)


def _growth_for(duration: float, dt0: float, n: int) -> float:
    """g with dt0 * (g^n - 1) / (g - 1) = duration (bisection)."""
    if abs(dt0 * n - duration) <= 1e-12 * duration:
        return 1.0
    lo, hi = (1.0 + 1e-12, 2.0) if duration > dt0 * n else (1e-6, 1.0 - 1e-12)
    f = lambda g: dt0 * (g ** n - 1.0) / (g - 1.0) - duration
    while f(hi) < 0:
        hi *= 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if f(mid) > 0:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def single_tl_set(alpha: float = 100.0, n_slots: int = 2000, E: float = 1.45, s: float = 3.5e12,
                  beta: float = 1.0, dt: float = 0.1, T_end_C: float = 500.0,
                  set_id: int = 0) -> SetSpec:
    """One TL set: 2,000 traps, 0 -> 500 degC at 1 K/s, dt = 0.1 s (5,000 steps),
    1 degC bins.  ``alpha`` multiplies r'; rho' = 1e-6 gives rho'^(-1/3) = 100."""
    return SetSpec(n_slots=n_slots, E=E, s=s, alpha=alpha, set_id=set_id, kind="tl",
                   segments=[tl_ramp(0.0, T_end_C, beta, dt, 1.0)]).finalize()


def batch_tl_iso(n_sets: int = 4096, seed: int = 20261203, n_min: int = 1000,
                 n_max: int = 100000, alpha_from_rho: bool = True,
                 alpha: Optional[float] = None) -> List[SetSpec]:
    """Batched TL + isothermal workload.

    E ~ U[1.2, 1.8] eV, log10 s ~ U[10, 14], rho' log-uniform [1e-7, 1e-5],
    traps per set log-uniform [1e3, 1e5] (ragged); even set ids are TL ramps
    (beta in {0.5, 1, 2, 5} K/s, 0 -> 500 degC, dt = 0.1 s, 1 degC bins), odd
    ids isothermal holds (T ~ U[150, 300] degC, 1e4 s, dt = 1 s, 20 s bins).
    alpha = rho'^(-1/3) (46..215 over the batch: most traps stay filled),
    10 with ``alpha_from_rho=False``, or the given ``alpha`` for every set
    (the signal-bearing variant uses 5: most TL sets empty by 500 degC).  The
    other parameters do not depend on the choice, so the variants share them.
    """
    rng = np.random.default_rng(seed)
    E = rng.uniform(1.2, 1.8, n_sets)
    s = 10.0 ** rng.uniform(10.0, 14.0, n_sets)
    rho = 10.0 ** rng.uniform(-7.0, -5.0, n_sets)
    n = np.rint(10.0 ** rng.uniform(np.log10(n_min), np.log10(n_max), n_sets)).astype(np.int64)
    betas = rng.choice(np.array([0.5, 1.0, 2.0, 5.0]), n_sets)
    T_iso = rng.uniform(150.0, 300.0, n_sets)
    out = []
    for i in range(n_sets):
        a_i = alpha if alpha is not None else (rho[i] ** (-1.0 / 3.0) if alpha_from_rho else 10.0)
        if i % 2 == 0:
            seg = tl_ramp(0.0, 500.0, float(betas[i]), 0.1, 1.0)
            kind = "tl"
        else:
            seg = isothermal(float(T_iso[i]), 1e4, 1.0, 20.0)
            kind = "iso"
        out.append(SetSpec(n_slots=int(n[i]), E=float(E[i]), s=float(s[i]), alpha=float(a_i),
                           segments=[seg], set_id=i, kind=kind).finalize())
    return out


def batch_dose_fade_irsl(n_sets: int = 2048, seed: int = 20261204, n_min: int = 1000,
                         n_max: int = 100000, fade_steps: int = 200,
                         s_tun: float = 3e15, alpha: Optional[float] = None) -> List[SetSpec]:
    """Irradiation -> fading -> IRSL sequences (uneven step counts per set).

    dose rate ~ U[0.05, 0.2] Gy/s to dose log-uniform [1, 1000] Gy with
    D0 ~ U[100, 500] Gy (fill steps of ~1 s), ground-state tunnelling fading over
    1e5 s in ``fade_steps`` geometric steps, then IR stimulation at 50 degC with
    sigma*Phi log-uniform [1e-3, 1e-1] /s for 1,000 s at dt = 0.1 s.  Traps
    start empty.  E, s, rho' and alpha as in ``batch_tl_iso``, or the given
    ``alpha`` for every set.  With alpha = rho'^(-1/3) and s_tun = 3e15 /s
    the fading empties every trap with alpha r' < ln(3e15 * 1e5) = 48, which
    includes every trap the stimulation could empty (alpha r' < ln(100)), so
    the IRSL phase of that workload has no events; a small alpha with a small
    s_tun (e.g. 5 and 1e-4 /s) gives signal in both phases.
    """
    rng = np.random.default_rng(seed)
    E = rng.uniform(1.2, 1.8, n_sets)
    s = 10.0 ** rng.uniform(10.0, 14.0, n_sets)
    rho = 10.0 ** rng.uniform(-7.0, -5.0, n_sets)
    n = np.rint(10.0 ** rng.uniform(np.log10(n_min), np.log10(n_max), n_sets)).astype(np.int64)
    rate = rng.uniform(0.05, 0.2, n_sets)
    dose = 10.0 ** rng.uniform(0.0, 3.0, n_sets)
    D0 = rng.uniform(100.0, 500.0, n_sets)
    sphi = 10.0 ** rng.uniform(-3.0, -1.0, n_sets)
    out = []
    for i in range(n_sets):
        a_i = alpha if alpha is not None else rho[i] ** (-1.0 / 3.0)
        segs = [irradiate(float(dose[i]), float(rate[i]), float(D0[i]), dt=1.0, T_C=20.0),
                fade(1e5, fade_steps, s_tun, dt0=1.0, T_C=20.0, steps_per_bin=10),
                optical(float(sphi[i]), 1000.0, 0.1, T_C=50.0, bin_seconds=1.0)]
        out.append(SetSpec(n_slots=int(n[i]), n_filled=0, E=float(E[i]), s=float(s[i]),
                           alpha=float(a_i), segments=segs, set_id=i,
                           kind="dose_fade_irsl").finalize())
    return out
