"""FP64 CPU restatement of the reference's event-driven KMC step (the oracle).

Test infrastructure only: the GPU library never imports this module.  It
restates, operation for operation, what the reference computes, so that it is
bit-exact with the reference when both consume the same uniform stream
(numpy's legacy MT19937 ``RandomState``, or an injected array of its draws):

* box geometry and initial fill      src/class/tl_trap_lab.py:27-43
* carrier seeding                    src/class/engine.py:124-129
* nearest-hole search                src/class/engine.py:113-119, 185-188
  (``np.linalg.norm`` sums the squared components left to right:
  ``sqrt((dx*dx + dy*dy) + dz*dz)``; ``argmin`` keeps the first index)
* pair creation quirks               src/class/engine.py:133-152
  (a new electron searches the OLD holes only; existing electrons are not
  re-pointed to the new hole)
* pair removal quirks                src/class/engine.py:154-175
  (hole indices above the removed one shift down BEFORE the mask
  ``nearest == h`` is taken, so owners of the former ``h+1`` are rescanned)
* rates and lifetimes                src/class/engine.py:65-77
* waits: legacy ``exponential(scale) = scale * -log(1 - U)`` with the C
  library ``log`` (numpy's vectorised ``log`` differs in the last bit)
                                     src/class/tl_trap_lab.py:48-60
* the simulation loop and output tables  src/class/simulate.py:36-92

Instead of the reference's dense electron x hole distance matrix (whose
``np.delete`` costs 94 % of its run time) the oracle keeps per electron the
nearest distance and hole index and recomputes a row only when the reference
would read it; the values are identical because every matrix entry is the same
norm expression of the same coordinates.

Unlike the reference this module also returns the event log
``(step, kind, e_idx, h_idx)`` in current-array indices, which is what the
GPU kernel's parity tests compare exactly.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

K_B_DEFAULT = 8.617333262145e-5  # src/class/engine.py:60

_mlog = np.frompyfunc(math.log, 1, 1)


def libm_log(x: np.ndarray) -> np.ndarray:
    """Element-wise C-library ``log`` (what numpy's legacy exponential calls)."""
    x = np.asarray(x, dtype=np.float64)
    if x.size == 0:
        return np.empty(x.shape, dtype=np.float64)
    return _mlog(x).astype(np.float64)


class UniformStream:
    """Sequential U[0,1) doubles: a legacy ``RandomState`` or a recorded array."""

    def __init__(self, source):
        if isinstance(source, np.random.RandomState):
            self._rs = source
            self._arr = None
        else:
            self._rs = None
            self._arr = np.ascontiguousarray(source, dtype=np.float64)
        self.consumed = 0

    def take(self, n: int) -> np.ndarray:
        n = int(n)
        if self._rs is not None:
            out = self._rs.random_sample(n)
        else:
            if self.consumed + n > self._arr.size:
                raise IndexError("injected uniform stream exhausted")
            out = self._arr[self.consumed:self.consumed + n].copy()
        self.consumed += n
        return out


@dataclass
class KRun:
    """One sweep point (a run) in flat form; see ``run_from_cfg``."""
    alpha: float
    b: float
    s: float
    E_cb: float
    E_loc_1: float
    E_loc_2: float
    D0: float
    Retrap: float
    k_b: float
    rho_prime: float
    holes: float
    N_e: float
    boundary_factor: float
    e_ratio_start: float
    duration: float
    dose_rate: float
    T_rate: float
    max_dt: float
    T_start: float


def run_from_cfg(run_cfg) -> KRun:
    """Read one run's parameters the way src/class/simulate.py:37-45 does.

    ``dose_rate`` is read from the physics group under that key (default 0),
    exactly like simulate.py:42 -- the YAML key ``D`` is NOT used there.
    """
    mc = run_cfg["exp_type_fp"]
    ph = run_cfg["physics_fp"]
    g = (lambda d, k, dflt: d.get(k, dflt))
    return KRun(
        alpha=float(ph["alpha"]), b=float(ph["b"]), s=float(ph["s"]),
        E_cb=float(ph["E_cb"]), E_loc_1=float(ph["E_loc_1"]),
        E_loc_2=float(ph["E_loc_2"]), D0=float(ph["D0"]),
        Retrap=float(ph["Retrap"]), k_b=float(g(ph, "k_b", K_B_DEFAULT)),
        rho_prime=float(mc["rho_prime"]), holes=float(mc["holes"]),
        N_e=float(mc["N_e"]), boundary_factor=float(mc["boundary_factor"]),
        e_ratio_start=float(g(mc, "e_ratio_start", 0.0)),
        duration=float(g(mc, "duration", 0.0)),
        dose_rate=float(g(ph, "dose_rate", 0.0)),
        T_rate=float(g(mc, "T_rate", 0.0)),
        max_dt=float(g(mc, "max_dt", 0.5)),
        T_start=float(g(mc, "T_start", 0)),
    )


def box_geometry(r: KRun):
    """Cube side and carrier counts (src/class/tl_trap_lab.py:33-39, engine.py:127)."""
    rho = r.rho_prime * (3 / (4 * np.pi) * r.alpha ** 3)
    d = (r.holes / rho) ** (1 / 3)
    e0 = int(r.N_e * r.e_ratio_start)
    total_h = int(r.holes * r.boundary_factor ** 3)
    core = (d, d, d)
    bound = (d * r.boundary_factor, d * r.boundary_factor, d * r.boundary_factor)
    return d, e0, total_h, core, bound


def _dist(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    """``np.linalg.norm(p - q, axis=-1)`` in its exact summation order."""
    x = p - q
    return np.sqrt((x[..., 0] * x[..., 0] + x[..., 1] * x[..., 1]) + x[..., 2] * x[..., 2])


class KSim:
    """State of one simulation (electrons, holes, nearest bookkeeping)."""

    def __init__(self, r: KRun, stream: UniformStream, geometry=None):
        self.r = r
        self.stream = stream
        _, e0, total_h, core, bound = geometry or box_geometry(r)
        self.core = np.array(core)
        self.bound = np.array(bound)
        self.electrons = stream.take(e0 * 3).reshape(e0, 3) * self.core
        self.holes = stream.take(total_h * 3).reshape(total_h, 3) * self.bound
        self.d_min = None
        self.nearest_idx = None

    # engine.py:113-119 (lazily, on the first nearest() call)
    def nearest(self):
        if self.d_min is None:
            n = self.electrons.shape[0]
            self.d_min = np.empty(n)
            self.nearest_idx = np.empty(n, dtype=np.int64)
            for i in range(n):
                row = _dist(self.electrons[i], self.holes)
                self.d_min[i] = np.min(row)
                self.nearest_idx[i] = int(np.argmin(row))
        return self.d_min, self.nearest_idx

    # tl_trap_lab.py:48-51 with engine.py:65-77
    def recomb_wait(self, T: float) -> np.ndarray:
        r = self.r
        d, _ = self.nearest()
        u_loc = self.stream.take(d.shape[0])
        E_loc = np.where(u_loc < r.Retrap, r.E_loc_2, r.E_loc_1)
        rate_cb = r.s * np.exp(-r.E_cb / (r.k_b * T))
        rate_tn = r.b * np.exp(-E_loc / (r.k_b * T) - r.alpha * d)
        lifetime = 1.0 / (rate_cb + rate_tn)
        u_w = self.stream.take(d.shape[0])
        return lifetime * -libm_log(1.0 - u_w)

    # tl_trap_lab.py:53-60
    def filling_time(self, D: float) -> float:
        e = self.electrons.shape[0]
        N = int(self.r.N_e)
        if e == N or D == 0:
            lam = 1e-20
        else:
            lam = (D / self.r.D0) * (N - e)
        if lam > 0:
            u = self.stream.take(1)[0]
            return (1 / lam) * -math.log(1.0 - u)
        return 1e20

    # engine.py:133-152
    def add_electron(self) -> None:
        new_e = self.stream.take(3).reshape(1, 3) * self.core
        new_h = self.stream.take(3).reshape(1, 3) * self.bound
        old_holes = self.holes
        self.electrons = np.vstack([self.electrons, new_e])
        self.holes = np.vstack([self.holes, new_h])
        if self.d_min is None:
            self.nearest()
            return
        row = _dist(new_e[0], old_holes)
        self.d_min = np.append(self.d_min, np.min(row))
        self.nearest_idx = np.append(self.nearest_idx, int(np.argmin(row)))

    # engine.py:154-175
    def remove_pair(self, e_idx: int, h_idx: int) -> None:
        self.electrons = np.delete(self.electrons, e_idx, axis=0)
        self.holes = np.delete(self.holes, h_idx, axis=0)
        if self.d_min is None:
            return
        self.d_min = np.delete(self.d_min, e_idx)
        self.nearest_idx = np.delete(self.nearest_idx, e_idx)
        self.nearest_idx[self.nearest_idx > h_idx] -= 1
        for i in np.nonzero(self.nearest_idx == h_idx)[0]:
            row = _dist(self.electrons[i], self.holes)
            self.d_min[i] = np.min(row)
            self.nearest_idx[i] = int(np.argmin(row))


@dataclass
class KResult:
    x_ax: np.ndarray          # (steps,) time after each step, zero padded
    lum: np.ndarray           # (steps,) 1.0 on recombination steps
    electron_ratio: np.ndarray
    n_steps: int              # steps actually taken
    events: np.ndarray        # (n_events, 4) int64: step, kind(0 fill,1 recomb), e_idx, h_idx
    draws: int                # uniforms consumed by this sim
    final_electrons: int


def run_sim(r: KRun, stream: UniformStream, steps: int) -> KResult:
    """One simulation of src/class/simulate.py:46-92."""
    start = stream.consumed
    sim = KSim(r, stream)
    x_ax = np.zeros(steps)
    lum = np.zeros(steps)
    ratio = np.zeros(steps)
    events = []
    dt_cap = r.max_dt / r.T_rate if r.T_rate else 1e20
    duration = r.duration
    t_cur = 0.0
    i = 0
    while t_cur <= duration:
        T_now = r.T_start + r.T_rate * t_cur + 273.15
        wait = sim.recomb_wait(T_now)
        dt_fill = sim.filling_time(r.dose_rate)
        dt_recomb = np.min(wait) if wait.any() else dt_fill
        dt = min(dt_fill, dt_recomb, dt_cap)
        t_cur += dt
        if i >= steps:
            raise IndexError(f"step {i} exceeds the {steps}-step output table")
        x_ax[i] = t_cur
        if dt == dt_fill:
            sim.add_electron()
            events.append((i, 0, sim.electrons.shape[0] - 1, sim.holes.shape[0] - 1))
            ev = 0
        elif dt == dt_recomb:
            e_idx = int(np.argmin(wait))
            _, nearest = sim.nearest()
            h_idx = int(nearest[e_idx])
            sim.remove_pair(e_idx, h_idx)
            events.append((i, 1, e_idx, h_idx))
            ev = 1
        else:
            ev = 0
        lum[i] = ev
        ratio[i] = sim.electrons.shape[0] / r.N_e
        i += 1
        if duration and t_cur >= duration:
            break
    ev_arr = np.array(events, dtype=np.int64).reshape(-1, 4)
    return KResult(x_ax, lum, ratio, i, ev_arr, stream.consumed - start,
                   sim.electrons.shape[0])


def simulate_runs(runs, stream: UniformStream, steps: int, sims: int):
    """Mirror of simulate(): every (run, sim) in order on one shared stream.

    Returns ``(x_ax, Lum, electron_ratio)`` shaped ``(steps, sims, runs)`` and
    the per-(run, sim) ``KResult`` list (src/class/simulate.py:30-32, 36-92).
    """
    n_runs = len(runs)
    x_ax = np.zeros((steps, sims, n_runs))
    lum = np.zeros((steps, sims, n_runs))
    ratio = np.zeros((steps, sims, n_runs))
    results = []
    for ri, r in enumerate(runs):
        for j in range(sims):
            res = run_sim(r, stream, steps)
            x_ax[:, j, ri] = res.x_ax
            lum[:, j, ri] = res.lum
            ratio[:, j, ri] = res.electron_ratio
            results.append(res)
    return x_ax, lum, ratio, results


# ---------------------------------------------------------------------------
# lab-data objectives (src/class/tl_trap_lab.py:65-179)
# ---------------------------------------------------------------------------
def _lab_sim(r: KRun, stream: UniformStream, e_ratio: float):
    rr = KRun(**{**r.__dict__, "e_ratio_start": float(e_ratio)})
    return KSim(rr, stream)


def _lab_step(sim: KSim, wait, tf):
    """One iteration's event: pair creation when the fill wait is not longer
    than the shortest recombination wait (min(dt_recomb, tf) keeps dt_recomb
    on a tie, and dt == tf then picks the fill)."""
    dt_recomb = np.min(wait) if wait.size else tf
    dt = min(dt_recomb, tf)
    if dt == tf:
        sim.add_electron()
        ev = (0, sim.electrons.shape[0] - 1, sim.holes.shape[0] - 1)
    else:
        e_idx = int(np.argmin(wait))
        _, nearest = sim.nearest()
        h_idx = int(nearest[e_idx])
        sim.remove_pair(e_idx, h_idx)
        ev = (1, e_idx, h_idx)
    return dt, ev


def tl_lab(r: KRun, stream: UniformStream, table: dict, D: float):
    """TLTrapSim.TL_lab (tl_trap_lab.py:65-123): one fresh simulation per
    table row, heating linearly from T_start to T_end over Duration with
    filling at dose rate D; returns (mse, per-row final ratio, per-row events,
    per-row draws)."""
    n_rows = len(table["Duration"])
    finals, events, draws, se = [], [], [], []
    for k in range(n_rows):
        start = stream.consumed
        sim = _lab_sim(r, stream, table["e_ratio"][k])
        T_start = table["T_start"][k] + 273.15
        T_rate = (table["T_end"][k] - table["T_start"][k]) / table["Duration"][k]
        wait = sim.recomb_wait(T_start)
        tf = sim.filling_time(D)
        t_cur, i, ev_log, ratio = 0.0, 0, [], None
        while t_cur < table["Duration"][k]:
            dt_recomb = np.min(wait) if wait.size else tf
            dt = min(dt_recomb, tf)
            T_now = T_start + T_rate * (t_cur + dt)
            t_cur += dt
            _, ev = _lab_step(sim, wait, tf)
            ev_log.append((i,) + ev)
            tf = sim.filling_time(D)
            wait = sim.recomb_wait(T_now)
            ratio = sim.electrons.shape[0] / r.N_e
            i += 1
        err = ratio - table["Fill"][k]
        se.append(err ** 2)
        finals.append(ratio)
        events.append(np.array(ev_log, dtype=np.int64).reshape(-1, 4))
        draws.append(stream.consumed - start)
    return float(np.mean(se)), finals, events, draws


def iso_lab(r: KRun, stream: UniformStream, table: dict):
    """TLTrapSim.ISO_lab (tl_trap_lab.py:125-179): one simulation per
    experiment number (sorted), held at its temperature with filling at its
    dose rate, scored against e_ratio at each observation time; returns
    (mse, per-experiment observed ratios, events, draws)."""
    exp = np.asarray(table["exp_no"])
    order = []
    for v in exp:
        if v not in order:
            order.append(v)
    se, obs_out, events, draws = [], [], [], []
    for exp_no in sorted(order):
        m = exp == exp_no
        sub = {k: np.asarray(v)[m] for k, v in table.items()}
        start = stream.consumed
        sim = _lab_sim(r, stream, float(sub["e_ratio"][0]))
        T_iso = float(sub["temp"][0]) + 273.15
        D = float(sub["dose"][0])
        wait = sim.recomb_wait(T_iso)
        tf = sim.filling_time(D)
        t_cur, i, ev_log, obs_idx, got = 0.0, 0, [], 0, []
        obs = sub["time"]
        while obs_idx < len(obs):
            dt_recomb = np.min(wait) if wait.size else tf
            dt = min(dt_recomb, tf)
            t_cur += dt
            _, ev = _lab_step(sim, wait, tf)
            ev_log.append((i,) + ev)
            tf = sim.filling_time(D)
            wait = sim.recomb_wait(T_iso)
            i += 1
            while obs_idx < len(obs) and t_cur >= obs[obs_idx]:
                fill = sim.electrons.shape[0] / r.N_e
                target = sub["e_ratio"][sub["time"] == obs[obs_idx]][0]
                se.append((fill - target) ** 2)
                got.append(fill)
                obs_idx += 1
        obs_out.append(got)
        events.append(np.array(ev_log, dtype=np.int64).reshape(-1, 4))
        draws.append(stream.consumed - start)
    return float(np.mean(se)), obs_out, events, draws
