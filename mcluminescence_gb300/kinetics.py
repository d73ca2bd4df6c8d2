"""Drop-in for the reference's ``simulate(cfg)``: the event-driven kinetics on the GPU.

``simulate(cfg)`` takes the same configuration (a dict or an OmegaConf
``DictConfig`` with ``exp_type_fp`` / ``physics_fp`` groups), expands it with
``initialize_runs`` (src/class/engine.py:13-38), reads each run's parameters the
way src/class/simulate.py:39-45 and src/class/tl_trap_lab.py:27-43 do, runs every
(run, sim) on the GPU (``mcl_k_run``) and returns ``(x_ax, Lum,
electron_ratio, configs)`` shaped ``(steps, sims, runs)`` like
src/class/simulate.py:30-32,112.

Random numbers: by default the kernel draws from numpy's *global* legacy
``RandomState`` (MT19937): its state is read before the call and advanced
after it, exactly as the reference's ``np.random`` calls would advance it, so
``np.random.seed(k); simulate(cfg)`` gives the reference's result for the same
seed (up to the last bit of ``exp``/``log``, which can differ between numpy's
and CUDA's implementations and, very rarely, flip a near-tie).  The
simulations then run one after another on one CTA, as they share that stream.
``rng="philox"`` gives each simulation its own counter-based stream and runs
them all in parallel (one CTA each).

Errors follow the reference: unknown or missing physics keys raise
``TypeError`` (``Physics(**cfg.physics_fp)``, tl_trap_lab.py:30), more steps
than table rows raise ``IndexError`` (simulate.py:64), a nearest search over no
holes raises ``ValueError`` (numpy's empty ``min``).
"""
from __future__ import annotations

import csv
import ctypes as C
import os
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Sequence

import numpy as np

from . import _lib
from .config import initialize_runs

K_B_DEFAULT = 8.617333262145e-5  # src/class/engine.py:60
PHYSICS_FIELDS = ("alpha", "b", "s", "E_cb", "E_loc_1", "E_loc_2", "D0", "Retrap",
                  "name", "D", "rho_trap", "k_b")
PHYSICS_REQUIRED = PHYSICS_FIELDS[:8]

K_SIM_DTYPE = _lib.K_SIM_DTYPE
KArgs = _lib.KArgs


def _get(d: Any, k: str, default: Any = None) -> Any:
    try:
        return d.get(k, default)
    except AttributeError:
        return getattr(d, k, default)


def physics(ph: Any) -> Dict[str, float]:
    """The checks ``Physics(**cfg.physics_fp)`` performs (engine.py:44-60)."""
    keys = list(ph.keys())
    for k in keys:
        if k not in PHYSICS_FIELDS:
            raise TypeError(f"Physics.__init__() got an unexpected keyword argument '{k}'")
    missing = [k for k in PHYSICS_REQUIRED if k not in keys]
    if missing:
        raise TypeError(f"Physics.__init__() missing {len(missing)} required positional "
                        f"argument{'s' if len(missing) > 1 else ''}: "
                        + ", ".join(f"'{m}'" for m in missing))
    out = {k: float(ph[k]) for k in PHYSICS_REQUIRED}
    out["k_b"] = float(_get(ph, "k_b", K_B_DEFAULT))
    return out


@dataclass
class RunParams:
    """One run's parameters, read as simulate.py:39-48 and tl_trap_lab.py:27-43 read them."""
    phys: Dict[str, float]
    duration: float
    e_ratio_start: float
    dose_rate: float
    T_rate: float
    dt_cap: float
    T_start: float
    N_e: float
    L: float
    Lb: float
    e0: int
    n_h0: int
    loop: int = 0                 # MCL_LOOP_*
    obs: Optional[np.ndarray] = None   # lab isothermal: observation times


def run_params(run_cfg: Any, dose_rate: Optional[float] = None) -> RunParams:
    mc = run_cfg["exp_type_fp"]
    ph = run_cfg["physics_fp"]
    duration = float(_get(mc, "duration", 0.0))
    e_ratio_start = float(_get(mc, "e_ratio_start", 0.0))
    # simulate.py:42 reads the key "dose_rate" (the YAML files call it "D");
    # Physics(**physics_fp) would reject that key, so only the keyword
    # argument of this function can switch filling on.
    dr = float(_get(ph, "dose_rate", 0.0)) if dose_rate is None else float(dose_rate)
    T_rate = float(_get(mc, "T_rate", 0.0))
    max_dt = float(_get(mc, "max_dt", 0.5))
    dt_cap = max_dt / T_rate if T_rate else 1e20
    p = physics(ph)
    T_start = _get(mc, "T_start", 0)
    rho = mc["rho_prime"] * (3 / (4 * np.pi) * p["alpha"] ** 3)
    d = (mc["holes"] / rho) ** (1 / 3)
    bf = mc["boundary_factor"]
    e0 = int(mc["N_e"] * e_ratio_start)
    n_h0 = int(mc["holes"] * bf ** 3)
    return RunParams(p, duration, e_ratio_start, dr, T_rate, dt_cap, float(T_start),
                     float(mc["N_e"]), float(d), float(d * bf), e0, n_h0)


@dataclass
class KResult:
    x_ax: np.ndarray              # (steps, n_sims)
    lum: np.ndarray
    electron_ratio: np.ndarray
    n_steps: np.ndarray           # (n_sims,)
    draws: np.ndarray
    status: np.ndarray
    events: List[np.ndarray]      # per simulation (n, 4): step, kind, e_idx, h_idx
    obs_ratio: Optional[List[np.ndarray]] = None   # lab isothermal loop: ratio at each observation


def _fill_sims(params: Sequence[RunParams], steps: int, extra: int):
    sims = np.zeros(len(params), dtype=K_SIM_DTYPE)
    for i, rp in enumerate(params):
        r = sims[i]
        for k, v in rp.phys.items():
            r[k] = v
        r["dose_rate"], r["T_start"], r["T_rate"] = rp.dose_rate, rp.T_start, rp.T_rate
        r["dt_cap"], r["duration"], r["N_e"] = rp.dt_cap, rp.duration, rp.N_e
        r["L"] = r["W"] = r["H"] = rp.L
        r["Lb"] = r["Wb"] = r["Hb"] = rp.Lb
        r["e0"], r["n_h0"] = rp.e0, rp.n_h0
        e_cap = max(rp.e0, int(rp.N_e)) + extra
        r["e_cap"] = e_cap
        r["h_cap"] = rp.n_h0 + (e_cap - rp.e0)
        r["steps"] = steps
        r["stream_id"] = i
        r["out_offset"] = i * steps
        r["ev_offset"] = i * steps
        r["ev_cap"] = steps
        r["loop"] = rp.loop
    return sims


def _ws_offsets(lib, sims: np.ndarray) -> int:
    """Place each simulation's global-memory region (sizes from the library)
    back to back in the workspace; returns the total bytes."""
    if len(sims) == 0:
        return 0
    fit = int(lib.mcl_k_arrays_fit_smem(int(sims["e_cap"].max()), int(sims["h_cap"].max())))
    off = 0
    for r in sims:
        r["ws_offset"] = off
        nb = int(lib.mcl_k_region_bytes(int(r["e_cap"]), int(r["h_cap"]), fit))
        if nb < 0:
            raise ValueError("negative capacity")
        off += nb
    return off


def run_kinetics(params: Sequence[RunParams], steps: int, *, rng: str = "philox", seed: int = 0,
                 mt_state=None, uniforms: Optional[np.ndarray] = None, sequential: Optional[bool] = None,
                 block: Optional[int] = None, extra_capacity: int = 64, want_events: bool = True,
                 timing=None):
    """Run simulations on the GPU.  ``rng``: "philox" (independent streams,
    parallel), "mt19937" (one shared stream continuing from ``mt_state``, a
    numpy legacy state tuple, sequential) or "injected" (``uniforms``; shared
    and sequential unless ``sequential=False``, then each simulation starts
    at ``u_offset``).  ``timing``: an optional pair of CUDA events (timing
    enabled) recorded just before and after the kernel launch.  Returns
    (KResult, final mt_state or None)."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required (the library has no CPU path)")
    lib = _lib.load()
    code = {"philox": _lib.MCL_RNG_PHILOX, "injected": _lib.MCL_RNG_INJECTED,
            "mt19937": _lib.MCL_RNG_MT19937}[rng]
    if sequential is None:
        sequential = rng != "philox"
    if block is None:
        # more threads per barrier-separated phase: 512 beats 256 both for one
        # CTA walking the simulations in order and for one CTA per simulation
        # (1,216 TL12 simulations: 238.6 ms against 259.4 ms, same events)
        block = 512
    n = len(params)
    sims = _fill_sims(params, steps, extra_capacity)
    n_u = 0
    if rng == "injected":
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        n_u = int(u.size)
        if sequential:
            sims["u_offset"][0] = 0
            sims["u_count"][0] = n_u
    obs_list = [np.asarray(rp.obs, dtype=np.float64) if rp.obs is not None else np.zeros(0) for rp in params]
    n_obs_tot = int(sum(len(o) for o in obs_list))
    off = 0
    for i, o in enumerate(obs_list):
        sims[i]["n_obs"] = len(o)
        sims[i]["obs_offset"] = off
        off += len(o)
    smem_flag, ws_need = C.c_int32(), C.c_int64()
    e_max, h_max = C.c_int32(), C.c_int32()
    ws_bytes = _ws_offsets(lib, sims)
    _lib.check(lib.mcl_k_validate(_lib.ptr(sims), n, code, block, n_u, C.byref(smem_flag),
                                  C.byref(ws_need), C.byref(e_max), C.byref(h_max)), "mcl_k_validate")
    if ws_need.value > ws_bytes:
        raise RuntimeError("workspace layout disagrees with the library")
    dev = torch.device("cuda")
    d_sims = torch.from_numpy(sims.view(np.uint8)).to(dev)
    rows = max(n * steps, 1)
    x_ax = torch.zeros(rows, dtype=torch.float64, device=dev)
    lum = torch.zeros_like(x_ax)
    ratio = torch.zeros_like(x_ax)
    events = torch.zeros(max(4 * n * steps, 4), dtype=torch.int32, device=dev) if want_events else None
    n_ev = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    n_st = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    draws = torch.zeros(max(n, 1), dtype=torch.int64, device=dev)
    status = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    d_u = torch.from_numpy(u).to(dev) if rng == "injected" else None
    d_mt = None
    if rng == "mt19937":
        name, keys, pos = mt_state[0], mt_state[1], mt_state[2]
        if name != "MT19937":
            raise ValueError("expected a legacy MT19937 state")
        st = np.zeros(625, dtype=np.uint32)
        st[:624] = np.asarray(keys, dtype=np.uint32)
        st[624] = int(pos)
        d_mt = torch.from_numpy(st.view(np.int32)).to(dev)
    d_ws = torch.empty(max(ws_need.value, 16), dtype=torch.uint8, device=dev)
    d_obs_t = d_obs_r = None
    if n_obs_tot:
        d_obs_t = torch.from_numpy(np.concatenate(obs_list)).to(dev)
        d_obs_r = torch.full((n_obs_tot,), float("nan"), dtype=torch.float64, device=dev)
    a = KArgs()
    a.sims, a.x_ax, a.lum, a.ratio = _lib.ptr(d_sims), _lib.ptr(x_ax), _lib.ptr(lum), _lib.ptr(ratio)
    a.events, a.n_events, a.n_steps = _lib.ptr(events), _lib.ptr(n_ev), _lib.ptr(n_st)
    a.draws, a.status, a.uniforms = _lib.ptr(draws), _lib.ptr(status), _lib.ptr(d_u)
    a.mt_state, a.workspace = _lib.ptr(d_mt), _lib.ptr(d_ws)
    a.obs_time, a.obs_ratio = _lib.ptr(d_obs_t), _lib.ptr(d_obs_r)
    a.workspace_bytes = int(d_ws.numel()) if d_ws is not None else 0
    a.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    a.n_sims, a.rng, a.sequential, a.block = n, code, int(bool(sequential)), block
    a.e_cap_max, a.h_cap_max, a.arrays_in_smem = e_max.value, h_max.value, smem_flag.value
    s = torch.cuda.current_stream()
    if timing is not None:
        timing[0].record(s)
    _lib.check(lib.mcl_k_run(C.byref(a), C.c_void_p(s.cuda_stream)), "mcl_k_run")
    if timing is not None:
        timing[1].record(s)
    s.synchronize()
    st_h = status.cpu().numpy()[:n]
    nst = n_st.cpu().numpy()[:n]
    nev = n_ev.cpu().numpy()[:n]
    ev_h = events.cpu().numpy().reshape(-1, 4) if want_events else None
    evs = []
    for i in range(n):
        if want_events:
            k = min(int(nev[i]), steps)
            evs.append(ev_h[i * steps:i * steps + k].astype(np.int64))
        else:
            evs.append(None)
    # rows past the longest simulation stay zero on the device: copy only the
    # rows any simulation wrote (a failing step may write row n_steps)
    used = min(steps, int(nst.max()) + 1) if n else 0

    def table(d):
        h = np.zeros((steps, n), dtype=np.float64)
        if used:
            h[:used] = d.view(n, steps)[:, :used].cpu().numpy().T
        return h

    res = KResult(table(x_ax), table(lum), table(ratio), nst, draws.cpu().numpy()[:n], st_h, evs)
    if n_obs_tot:
        o = d_obs_r.cpu().numpy()
        res.obs_ratio = [o[int(sims[i]["obs_offset"]):int(sims[i]["obs_offset"]) + len(obs_list[i])]
                         for i in range(n)]
    new_state = None
    if d_mt is not None:
        st = d_mt.cpu().numpy().view(np.uint32)
        new_state = ("MT19937", st[:624].copy(), int(st[624]))
    return res, new_state


def _raise_for(status: np.ndarray, steps: int):
    for code in status:
        code = int(code)
        if code == _lib.MCL_EOVERFLOW:
            raise IndexError(f"index {steps} is out of bounds for axis 0 with size {steps}")
        if code == _lib.MCL_ENOHOLE:
            raise ValueError("zero-size array to reduction operation minimum which has no identity")
        if code != _lib.MCL_OK:
            raise _lib.MclError(code, "event-driven kinetics kernel", detail=False)


def results_dir() -> str:
    """Where ``simulate`` writes its table: ``MCL_RESULTS_DIR`` if set, else
    ``results/simulations`` under the current directory (the reference
    writes under its project root, src/class/simulate.py:110)."""
    return os.environ.get("MCL_RESULTS_DIR") or os.path.join(os.getcwd(), "results", "simulations")


def simulate(cfg: Any, *, rng: str = "numpy", seed: Optional[int] = None,
             dose_rate: Optional[float] = None, write_csv: bool = True, csv_path: Optional[str] = None,
             block: Optional[int] = None, return_result: bool = False):
    """GPU replacement of src/class/simulate.py:simulate.

    ``rng="numpy"`` continues numpy's global legacy RandomState (seeded with
    ``seed`` first when given); ``rng="philox"`` uses independent Philox
    streams keyed by ``seed``.  ``dose_rate`` switches trap filling on (the
    reference reads it from ``physics_fp.dose_rate``, a key its Physics class
    rejects).  Like the reference, the call writes the long table of
    simulate.py:95-110 to ``exp_{tag}.csv`` (``tag`` = ``cfg.tag``, default
    "") in ``results_dir()``, creating the directory; ``csv_path`` gives
    another file, ``write_csv=False`` turns the side effect off.
    """
    configs = initialize_runs(cfg)
    n_runs = len(configs)
    mc0 = configs[0]["exp_type_fp"]
    steps = int(mc0["steps"])
    sims = int(mc0["sims"])
    params = []
    for ri in range(n_runs):
        rp = run_params(configs[ri], dose_rate)
        params += [rp] * sims
    extra = 64
    while True:
        if rng == "numpy":
            if seed is not None:
                np.random.seed(seed)
            state0 = np.random.get_state()
            res, new_state = run_kinetics(params, steps, rng="mt19937", mt_state=state0, block=block,
                                          extra_capacity=extra)
        else:
            res, new_state = run_kinetics(params, steps, rng="philox", seed=seed or 0, block=block,
                                          extra_capacity=extra)
        if np.any(res.status == _lib.MCL_ECAPACITY) and extra < 1 << 20:
            extra *= 8    # more pair creations than provisioned: run again with room
            continue
        break
    if rng == "numpy":
        np.random.set_state(("MT19937", new_state[1], new_state[2], state0[3], state0[4]))
    _raise_for(res.status, steps)
    x_ax = res.x_ax.reshape(steps, n_runs, sims).transpose(0, 2, 1).copy()
    lum = res.lum.reshape(steps, n_runs, sims).transpose(0, 2, 1).copy()
    ratio = res.electron_ratio.reshape(steps, n_runs, sims).transpose(0, 2, 1).copy()
    if write_csv or csv_path:
        if not csv_path:
            os.makedirs(results_dir(), exist_ok=True)
            csv_path = os.path.join(results_dir(), f"exp_{_get(cfg, 'tag', '')}.csv")
        write_table(csv_path, lum, ratio)
    out = (x_ax, lum, ratio, configs)
    return (out, res) if return_result else out


def write_table(path: str, lum: np.ndarray, ratio: np.ndarray) -> None:
    """The long table of src/class/simulate.py:95-110, byte for byte: columns
    run,sim,step,lum,electron_ratio, rows ordered run, then sim, then step
    (the tables transposed to (runs, sims, steps) and flattened), written the
    way the reference's ``DataFrame.to_csv(path, index=False)`` writes them
    (pandas 2.2.3, requirements.txt:14): integers as ``str``, float64 values
    as numpy's shortest round-trip repr (``astype(str)``), commas, and
    ``os.linesep`` after every line including the header."""
    steps, sims, runs = lum.shape
    cols = (np.repeat(np.arange(runs), sims * steps).astype(str),
            np.tile(np.repeat(np.arange(sims), steps), runs).astype(str),
            np.tile(np.arange(steps), runs * sims).astype(str),
            np.ascontiguousarray(lum.transpose(2, 1, 0)).ravel().astype(str),
            np.ascontiguousarray(ratio.transpose(2, 1, 0)).ravel().astype(str))
    comma = np.array(",")
    rows = cols[0]
    for c in cols[1:]:
        rows = np.char.add(np.char.add(rows, comma), c)
    nl = os.linesep
    with open(path, "w", newline="") as f:
        f.write("run,sim,step,lum,electron_ratio" + nl)
        if rows.size:
            f.write(nl.join(rows.tolist()) + nl)


# ---------------------------------------------------------------------------
# lab-data objectives: the TLTrapSim drop-in (tl_trap_lab.py:24-179)
# ---------------------------------------------------------------------------
def data_dir() -> str:
    """Where lab tables named without a path are found: ``MCL_DATA_DIR`` if
    set, else ``data/processed`` under the project root (``MCL_PROJECT_ROOT``
    or the current directory), as the reference reads
    ``PROJECT_ROOT/data/processed/<name>.csv`` (tl_trap_lab.py:67, 127)."""
    root = os.environ.get("MCL_PROJECT_ROOT") or os.getcwd()
    return os.environ.get("MCL_DATA_DIR") or os.path.join(root, "data", "processed")


def read_table(src) -> Dict[str, np.ndarray]:
    """A lab table as columns: a dict of columns, a CSV path, or a table
    name (no directory, no extension) looked up in ``data_dir()`` like the
    reference's ``TL_lab(csv_name)``."""
    if isinstance(src, dict):
        return {k: np.asarray(v) for k, v in src.items()}
    src = str(src)
    if os.sep not in src and not src.endswith(".csv"):
        src = os.path.join(data_dir(), src + ".csv")
    with open(src, newline="") as f:
        rows = list(csv.DictReader(f))
    out = {}
    for k in rows[0].keys():
        vals = [r[k] for r in rows]
        try:
            out[k] = np.array([float(v) for v in vals])
        except ValueError:
            out[k] = np.array(vals)
    return out


class _Attr(dict):
    """A config group or the physics constants with attribute access
    (``sim.mc.N_e``, ``sim.phys.D0``), as the reference's DictConfig and
    Physics objects give it."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e


def _empty_min():
    return ValueError("zero-size array to reduction operation minimum which has no identity")


class Box:
    """GPU-backed drop-in of src/class/engine.py:Box (electrons, recombination
    centres and the nearest-centre bookkeeping), for callers that step the
    simulation themselves.

    Coordinates are drawn from ``rng`` (numpy's global legacy stream unless
    another ``RandomState`` is given) in the reference's order and kept as
    host arrays ``electrons`` / ``holes`` like the reference's.  Every
    distance is evaluated on the GPU (``mcl_k_box_nearest``,
    ``mcl_k_box_distances``) exactly as np.linalg.norm evaluates it, and the
    bookkeeping follows engine.py:113-188 step for step, quirks included:
    ``seed`` invalidates the distance cache but not the nearest arrays; a new
    electron's nearest centre is searched over the centres that existed
    before its own (engine.py:147,151-152) and existing electrons ignore the
    new centre; ``remove_pair`` shifts the nearest indices above the removed
    centre before it masks the owners of that index, so the former owners of
    the next centre are searched again too (engine.py:167-175); without a
    cache ``remove_pair`` only deletes coordinates.  The full distance
    matrix is not kept: every search recomputes the distances it needs,
    which gives the values the reference caches.
    """

    def __init__(self, L: float, W: float, H: float, boundary_factor: float, rng=None):
        self.L, self.W, self.H, self.boundary_factor = L, W, H, boundary_factor
        self._rs = rng if rng is not None else np.random
        self.electrons = np.zeros((0, 3))
        self.holes = np.zeros((0, 3))
        self._cached = False      # the reference's `_d is not None`
        self._min_d = None
        self._nearest = None

    @property
    def core_shape(self):
        return self.L, self.W, self.H

    @property
    def boundary_shape(self):
        bf = self.boundary_factor
        return self.L * bf, self.W * bf, self.H * bf

    @staticmethod
    def _dev(a):
        import torch
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()

    def _search(self, electrons, holes, rows=None):
        """(min distance, first argmin) over ``holes`` of the listed rows of
        ``electrons`` (all rows if None), on the GPU."""
        import torch
        lib = _lib.load()
        n_e, n_h = int(electrons.shape[0]), int(holes.shape[0])
        rows = np.arange(n_e) if rows is None else np.asarray(rows)
        if rows.size == 0:
            return np.zeros(0), np.zeros(0, dtype=np.int64)
        if n_h == 0:
            raise _empty_min()
        d_e, d_h = self._dev(electrons), self._dev(holes)
        d_rows = torch.from_numpy(rows.astype(np.int32)).cuda()
        md = torch.empty(n_e, dtype=torch.float64, device="cuda")
        nn = torch.empty(n_e, dtype=torch.int64, device="cuda")
        st = torch.cuda.current_stream()
        _lib.check(lib.mcl_k_box_nearest(_lib.ptr(d_e), n_e, _lib.ptr(d_h), n_h, _lib.ptr(d_rows), int(rows.size),
                                         _lib.ptr(md), _lib.ptr(nn), C.c_void_p(st.cuda_stream)),
                   "mcl_k_box_nearest")
        return md.cpu().numpy()[rows], nn.cpu().numpy()[rows]

    def _rebuild(self) -> None:
        self._min_d, self._nearest = self._search(self.electrons, self.holes)
        self._cached = True

    def seed(self, n_e: int, n_h: int) -> None:
        self.electrons = self._rs.rand(n_e, 3) * self.core_shape
        total_h = int(n_h * self.boundary_factor ** 3)
        self.holes = self._rs.rand(total_h, 3) * self.boundary_shape
        self._cached = False

    def add_electron(self) -> None:
        new_e = self._rs.rand(1, 3) * self.core_shape
        new_h = self._rs.rand(1, 3) * self.boundary_shape
        old_holes = self.holes
        self.electrons = np.vstack([self.electrons, new_e])
        self.holes = np.vstack([self.holes, new_h])
        if not self._cached:
            self._rebuild()
            return
        md, nn = self._search(new_e, old_holes)
        self._min_d = np.append(self._min_d, md)
        self._nearest = np.append(self._nearest, nn)

    def remove_pair(self, e_idx: int, h_idx: int) -> None:
        self.electrons = np.delete(self.electrons, e_idx, axis=0)
        self.holes = np.delete(self.holes, h_idx, axis=0)
        if not self._cached:
            return
        self._min_d = np.delete(self._min_d, e_idx)
        self._nearest = np.delete(self._nearest, e_idx)
        self._nearest[self._nearest > h_idx] -= 1
        mask = self._nearest == h_idx
        if mask.any():
            md, nn = self._search(self.electrons, self.holes, np.nonzero(mask)[0])
            self._min_d[mask] = md
            self._nearest[mask] = nn

    def distances(self) -> np.ndarray:
        """The electron x centre distance matrix (computed on the GPU)."""
        import torch
        if not self._cached:
            self._rebuild()
        n_e, n_h = self.electrons.shape[0], self.holes.shape[0]
        out = torch.empty(n_e * n_h, dtype=torch.float64, device="cuda")
        if n_e * n_h:
            # the device copies stay referenced until the result is read back
            d_e, d_h = self._dev(self.electrons), self._dev(self.holes)
            _lib.check(_lib.load().mcl_k_box_distances(
                _lib.ptr(d_e), n_e, _lib.ptr(d_h), n_h, _lib.ptr(out),
                C.c_void_p(torch.cuda.current_stream().cuda_stream)), "mcl_k_box_distances")
        return out.cpu().numpy().reshape(n_e, n_h)

    def nearest(self):
        if self._min_d is None:
            self._rebuild()
        return self._min_d, self._nearest


class TLTrapSim:
    """GPU drop-in of src/class/tl_trap_lab.py:TLTrapSim.

    The constructor performs the reference's checks (``Physics(**physics_fp)``),
    sizes the box as tl_trap_lab.py:33-35 does and seeds it (engine.py:124-129)
    from numpy's global stream (``rng="numpy"``), so ``np.random.seed(k);
    TLTrapSim(run).TL_lab(table)`` matches the reference.  ``TL_lab`` and
    ``ISO_lab`` take a lab table (dict of columns or a CSV path with the
    reference's columns) and return the MSE like the reference; they run the
    whole loop in one launch.

    The step-level surface that the reference's ``simulate()`` loop drives
    (simulate.py:51-92) is here too: ``box`` (a GPU-backed ``Box``),
    ``_update_lifetimes(T)`` (lifetimes and waits on the GPU from the
    reference's draws), ``_filling_time(D)``, ``_lifetime``,
    ``_recomb_wait``, ``mc`` and ``phys`` with attribute access.  It takes
    one GPU round trip per call; ``simulate(cfg)`` runs the same loop in one
    launch and is the throughput path.  With ``rng="philox"`` the box and the
    step-level draws use a private numpy generator seeded with ``seed``.
    """

    def __init__(self, cfg: Any, *, e_ratio_start: Optional[float] = None, rng: str = "numpy",
                 seed: Optional[int] = None, block: Optional[int] = None):
        self.cfg = cfg
        mc = cfg["exp_type_fp"]
        self.mc = _Attr(mc) if isinstance(mc, dict) else mc
        self.phys = _Attr(physics(cfg["physics_fp"]))
        self.D = _get(cfg["physics_fp"], "D", None)
        self.rng, self.seed, self.block = rng, seed, block
        self.last = None
        if rng == "numpy":
            if seed is not None:
                np.random.seed(seed)
            self._rs = np.random
        else:
            self._rs = np.random.RandomState(seed or 0)
        rho = self.mc["rho_prime"] * (3 / (4 * np.pi) * self.phys["alpha"] ** 3)
        d = (self.mc["holes"] / rho) ** (1 / 3)
        self.box = Box(d, d, d, self.mc["boundary_factor"], rng=self._rs)
        e0 = int(self.mc["N_e"] * (e_ratio_start if e_ratio_start is not None else 0))
        self.box.seed(e0, self.mc["holes"])
        self._lifetime = None
        self._recomb_wait = None
        self._k_phys = None

    def _update_lifetimes(self, T: float) -> None:
        """tl_trap_lab.py:48-51: fresh lifetimes at temperature T (K) and an
        exponential wait per electron.  The uniforms come from the stream in
        the reference's order -- the Retrap choices (engine.py:72), then the
        waits' -- and the arithmetic runs on the GPU (mcl_k_box_waits)."""
        import torch
        d_min, _ = self.box.nearest()
        n = int(d_min.shape[0])
        u_r = self._rs.random_sample(n)
        u_w = self._rs.random_sample(n)
        if self._k_phys is None:
            self._k_phys = np.zeros(1, dtype=K_SIM_DTYPE)
            for k, v in self.phys.items():
                self._k_phys[0][k] = v
        if n == 0:
            self._lifetime, self._recomb_wait = np.zeros(0), np.zeros(0)
            return
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
        d_d, d_r, d_w = dev(d_min), dev(u_r), dev(u_w)
        lt = torch.empty(n, dtype=torch.float64, device="cuda")
        wt = torch.empty(n, dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().mcl_k_box_waits(
            _lib.ptr(self._k_phys), float(T), _lib.ptr(d_d), _lib.ptr(d_r), _lib.ptr(d_w), n, _lib.ptr(lt),
            _lib.ptr(wt), C.c_void_p(torch.cuda.current_stream().cuda_stream)), "mcl_k_box_waits")
        self._lifetime = lt.cpu().numpy()
        self._recomb_wait = wt.cpu().numpy()

    def _filling_time(self, D: float) -> float:
        """tl_trap_lab.py:53-60: the wait for the next filling event (one
        draw from the stream on every call)."""
        e = self.box.electrons.shape[0]
        N = int(self.mc["N_e"])
        if e == N or D == 0:
            lam = 1e-20
        else:
            lam = (D / self.phys["D0"]) * (N - e)
        return self._rs.exponential(1 / lam) if lam > 0 else 1e20

    def _params(self, e_ratio, T_start_C, T_rate, duration, D, loop, obs=None) -> RunParams:
        run = {"exp_type_fp": dict(self.mc), "physics_fp": dict(self.cfg["physics_fp"])}
        run["exp_type_fp"]["e_ratio_start"] = float(e_ratio)
        run["physics_fp"].pop("dose_rate", None)
        rp = run_params(run, dose_rate=0.0 if D is None else float(D))
        rp.T_start, rp.T_rate, rp.duration, rp.dt_cap = float(T_start_C), float(T_rate), float(duration), 1e20
        rp.loop = loop
        rp.obs = obs
        return rp

    def _run(self, params, steps=4096):
        while True:
            if self.rng == "numpy":
                state0 = np.random.get_state()
                res, new_state = run_kinetics(params, steps, rng="mt19937", mt_state=state0, block=self.block)
            else:
                res, new_state = run_kinetics(params, steps, rng="philox", seed=self.seed or 0,
                                              block=self.block)
            if np.any(res.status == _lib.MCL_EOVERFLOW) and steps < 1 << 24:
                steps *= 4        # more events than rows provisioned: run again with room
                continue
            break
        if self.rng == "numpy":
            np.random.set_state(("MT19937", new_state[1], new_state[2], state0[3], state0[4]))
        _raise_for(res.status, steps)
        self.last = res
        return res

    def TL_lab(self, table, *, plot: bool = False) -> float:
        """tl_trap_lab.py:65-123: per row, heat from T_start to T_end over
        Duration with filling at physics D; MSE of the final fill ratio."""
        tb = read_table(table)
        if self.D is None:
            raise TypeError("unsupported operand type(s) for /: 'NoneType' and 'float'")
        params = [self._params(tb["e_ratio"][k], tb["T_start"][k],
                               (tb["T_end"][k] - tb["T_start"][k]) / tb["Duration"][k],
                               tb["Duration"][k], self.D, _lib.MCL_LOOP_LAB_TL)
                  for k in range(len(tb["Duration"]))]
        res = self._run(params)
        finals = np.array([res.electron_ratio[int(res.n_steps[j]) - 1, j] for j in range(len(params))])
        self.finals = finals
        return float(np.mean((finals - tb["Fill"]) ** 2))

    def ISO_lab(self, table, *, plot: bool = False) -> float:
        """tl_trap_lab.py:125-179: per experiment number, hold at its
        temperature with filling at its dose rate; MSE over observation times."""
        tb = read_table(table)
        order = []
        for v in tb["exp_no"]:
            if v not in order:
                order.append(v)
        params, targets = [], []
        for exp_no in sorted(order):
            m = tb["exp_no"] == exp_no
            sub = {k: v[m] for k, v in tb.items()}
            obs = sub["time"].astype(np.float64)
            params.append(self._params(sub["e_ratio"][0], sub["temp"][0], 0.0, 0.0, sub["dose"][0],
                                       _lib.MCL_LOOP_LAB_ISO, obs))
            targets.append(np.array([sub["e_ratio"][sub["time"] == o][0] for o in obs]))
        res = self._run(params)
        err = np.concatenate([r - tgt for r, tgt in zip(res.obs_ratio, targets)])
        return float(np.mean(err ** 2))
