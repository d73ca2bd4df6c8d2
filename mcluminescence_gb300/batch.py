"""Batched Bernoulli-mode simulation: pack, launch, capture, read back.

``BernoulliBatch`` packs a list of ``SetSpec`` into the C structs of
include/mclum.h, validates them (``mcl_b_validate``), splits every set into
work items longest-first (``mcl_b_pack_items``), places descriptors and
outputs in device memory (torch tensors; the library never allocates), and
launches the persistent kernel on a CUDA stream -- directly or through a
captured CUDA graph.  ``simulate_batch`` is the one-call form that takes host
specs and returns host arrays.

No reference function corresponds one-to-one: this replaces the serial
per-parameter-set loops of src/class/simulate.py:36-48 and
src/class/optimizer.py:68-84 with one launch over all sets.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .schedule import SetSpec

_PREC = {"fp32": _lib.MCL_FP32, "fp64": _lib.MCL_FP64}
_RNG = {"philox": _lib.MCL_RNG_PHILOX, "injected": _lib.MCL_RNG_INJECTED}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required (the library has no CPU path)")
    return torch


def pack_host(specs: Sequence[SetSpec]):
    """Host struct arrays for ``specs``: (sets, segs, bin_offsets, slot_offsets,
    u_offsets).  Column-wise numpy assignment, so packing thousands of sets
    costs milliseconds."""
    n_sets = len(specs)
    for sp in specs:
        sp.finalize()
    seg_counts = np.array([len(sp.segments) for sp in specs], dtype=np.int64)
    n_segs = int(seg_counts.sum())
    sets = np.zeros(n_sets, dtype=_lib.SET_DTYPE)
    segs = np.zeros(n_segs, dtype=_lib.SEG_DTYPE)
    all_segs = [sg for sp in specs for sg in sp.segments]
    if n_segs:
        col = lambda name, dt: np.fromiter((getattr(sg, name) for sg in all_segs), dtype=dt, count=n_segs)
        segs["n_steps"] = col("n_steps", np.int32)
        segs["steps_per_bin"] = col("steps_per_bin", np.int32)
        segs["bin_offset"] = col("bin_offset", np.int32)
        segs["flags"] = np.where(col("thermal", bool), _lib.MCL_SEG_THERMAL, 0)
        for name in ("dt", "dt_growth", "T0", "beta", "rate_const", "fill_rate"):
            segs[name] = col(name, np.float64)
    seg_steps = segs["n_steps"].astype(np.int64)
    seg_bins = -(-seg_steps // np.maximum(segs["steps_per_bin"].astype(np.int64), 1))
    seg_begin = np.concatenate([[0], np.cumsum(seg_counts)[:-1]]) if n_sets else np.zeros(0, np.int64)
    owner = np.repeat(np.arange(n_sets), seg_counts)
    total_steps = np.bincount(owner, weights=seg_steps, minlength=n_sets).astype(np.int64)
    n_bins = np.bincount(owner, weights=seg_bins, minlength=n_sets).astype(np.int64)
    sc = lambda name, dt: np.fromiter((getattr(sp, name) for sp in specs), dtype=dt, count=n_sets)
    n_slots = sc("n_slots", np.int64)
    sets["n_slots"] = n_slots
    sets["n_filled"] = sc("n_filled", np.int64)
    sets["seg_begin"] = seg_begin
    sets["seg_count"] = seg_counts
    sets["n_bins"] = n_bins
    sets["set_id"] = sc("set_id", np.int64) & 0xFFFFFFFF
    b_off = np.concatenate([[0], np.cumsum(n_bins)]).astype(np.int64)
    s_off = np.concatenate([[0], np.cumsum(n_slots)]).astype(np.int64)
    u_off = np.concatenate([[0], np.cumsum(n_slots * (1 + total_steps))]).astype(np.int64)
    sets["bin_offset"] = b_off[:-1]
    sets["slot_offset"] = s_off[:-1]
    sets["u_offset"] = u_off[:-1]
    sets["total_steps"] = total_steps
    sets["step_offset"] = np.concatenate([[0], np.cumsum(total_steps)[:-1]]) if n_sets else 0
    for name in ("E", "s", "alpha", "k_b"):
        sets[name] = sc(name, np.float64)
    return sets, segs, b_off, s_off, u_off


@dataclass
class BatchResult:
    lum: np.ndarray             # (n_bins_total,) uint32 events per bin, all sets
    alive: Optional[np.ndarray]  # (n_bins_total,) filled traps at bin end
    fates: Optional[np.ndarray]  # (n_slots_total,) last recombination step or -1
    bin_offsets: np.ndarray     # (n_sets+1,)
    slot_offsets: np.ndarray    # (n_sets+1,)

    def lum_of(self, i: int) -> np.ndarray:
        return self.lum[self.bin_offsets[i]:self.bin_offsets[i + 1]]

    def alive_of(self, i: int) -> np.ndarray:
        return self.alive[self.bin_offsets[i]:self.bin_offsets[i + 1]]

    def fates_of(self, i: int) -> np.ndarray:
        return self.fates[self.slot_offsets[i]:self.slot_offsets[i + 1]]


class BernoulliBatch:
    """A packed batch resident on the GPU, ready to launch or replay."""

    def __init__(self, specs: Optional[Sequence[SetSpec]], *, precision: str = "fp32",
                 rng: str = "philox", seed: int = 0, block: int = 256, ept: int = 4,
                 grid: int = 0, want_alive: bool = True, want_fates: bool = False,
                 uniforms: Optional[np.ndarray] = None, device: str = "cuda", packed=None,
                 occupancy: int = 0, bin_copies: int = 1):
        """``specs`` (a list of SetSpec) or ``packed`` = (sets, segs, bin_offsets,
        slot_offsets, u_offsets) host arrays as returned by ``pack_host``.
        ``occupancy`` picks a register-capped FP32 build by the resident CTAs
        per SM it targets (ept 2: 4 at block 256, 8 at block 128; ept 4: 3 at
        block 256, 6 at block 128); 0 is the default build.  ``bin_copies``
        (1, 2 or 4) is how many copies of its set's bins each FP32 CTA keeps in
        shared memory; results do not depend on it."""
        if int(bin_copies) not in (1, 2, 4):
            raise ValueError(f"bin_copies must be 1, 2 or 4, not {bin_copies}")
        torch = _torch()
        self.lib = _lib.load()
        self.specs = list(specs) if specs is not None else None
        self.precision = _PREC[precision]
        self.rng = _RNG[rng]
        if self.precision == _lib.MCL_FP64 and block != 256:
            block = 256
        if self.precision == _lib.MCL_FP64 and ept not in (1, 2):
            ept = 2
        self.block, self.ept, self.grid = int(block), int(ept), int(grid)
        self.occupancy = int(occupancy) if self.precision == _lib.MCL_FP32 else 0
        self.bin_copies = int(bin_copies) if self.precision == _lib.MCL_FP32 else 1
        sets, segs, b_off, s_off, u_off = packed if packed is not None else pack_host(self.specs)
        self.bin_offsets, self.slot_offsets, self.u_offsets = b_off, s_off, u_off
        self.n_bins_total = int(b_off[-1])
        self.n_slots_total = int(s_off[-1])
        n_u = int(u_off[-1]) if self.rng == _lib.MCL_RNG_INJECTED else 0
        if self.rng == _lib.MCL_RNG_INJECTED:
            if uniforms is None or uniforms.size < n_u:
                raise ValueError(f"injected mode needs {n_u} uniforms")
        _lib.check(self.lib.mcl_b_validate(_lib.ptr(sets), len(sets), _lib.ptr(segs), len(segs),
                                           self.n_bins_total, self.n_slots_total,
                                           self.precision, self.rng,
                                           int(uniforms.size) if uniforms is not None else 0),
                   "mcl_b_validate")
        spi = self.block * self.ept
        n_slots = sets["n_slots"].astype(np.int64)
        cap = int(np.sum((n_slots + spi - 1) // spi))
        items = np.zeros(max(cap, 1), dtype=_lib.ITEM_DTYPE)
        n_items = self.lib.mcl_b_pack_items(_lib.ptr(sets), len(sets), spi, _lib.ptr(items), cap)
        if n_items < 0:
            _lib.check(int(n_items), "mcl_b_pack_items")
        self.n_items = int(n_items)
        self.max_bins = int(sets["n_bins"].max()) if len(sets) else 0
        self.host_sets, self.host_segs, self.host_items = sets, segs, items[:self.n_items]
        # batches that never fill run the FP32 build without the filling path
        self.no_fill = int(not np.any(segs["fill_rate"] > 0.0)) if len(segs) else 1
        self._trials = int(np.sum(n_slots * sets["total_steps"].astype(np.int64)))
        dev = torch.device(device)
        u8 = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8)).to(dev)
        self.d_sets = u8(sets) if len(sets) else torch.empty(8, dtype=torch.uint8, device=dev)
        self.d_segs = u8(segs) if len(segs) else torch.empty(8, dtype=torch.uint8, device=dev)
        self.d_items = u8(self.host_items) if self.n_items else torch.empty(8, dtype=torch.uint8, device=dev)
        self.d_lum = torch.zeros(max(self.n_bins_total, 1), dtype=torch.int32, device=dev)
        self.d_alive = torch.zeros_like(self.d_lum) if want_alive else None
        self.d_fates = (torch.full((max(self.n_slots_total, 1),), -1, dtype=torch.int32, device=dev)
                        if want_fates else None)
        self.d_u = (torch.from_numpy(np.ascontiguousarray(uniforms[:n_u], dtype=np.float64)).to(dev)
                    if self.rng == _lib.MCL_RNG_INJECTED else None)
        self.n_uniforms = n_u
        self.d_status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.table_steps = int(np.sum(sets["total_steps"]))
        self.ws_bytes = int(self.lib.mcl_b_workspace_size(_lib.ptr(sets), len(sets), self.precision))
        self.d_ws = torch.zeros(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self._graph = None
        self.args = self._make_args(zero_outputs=1)

    # -- launch ---------------------------------------------------------------
    def _make_args(self, zero_outputs: int) -> _lib.BArgs:
        a = _lib.BArgs()
        a.sets, a.segs, a.items = _lib.ptr(self.d_sets), _lib.ptr(self.d_segs), _lib.ptr(self.d_items)
        a.lum, a.alive, a.fates = _lib.ptr(self.d_lum), _lib.ptr(self.d_alive), _lib.ptr(self.d_fates)
        a.uniforms = _lib.ptr(self.d_u)
        a.status, a.workspace = _lib.ptr(self.d_status), _lib.ptr(self.d_ws)
        a.workspace_bytes, a.table_steps = self.ws_bytes, self.table_steps
        a.n_bins_total, a.n_slots_total, a.seed = self.n_bins_total, self.n_slots_total, self.seed
        a.n_uniforms = self.n_uniforms
        a.n_sets, a.n_segs, a.n_items = len(self.host_sets), len(self.host_segs), self.n_items
        a.slots_per_item, a.max_bins = self.block * self.ept, self.max_bins
        a.precision, a.rng, a.block, a.ept, a.grid = self.precision, self.rng, self.block, self.ept, self.grid
        a.occupancy, a.no_fill, a.bin_copies = self.occupancy, self.no_fill, self.bin_copies
        a.zero_outputs = zero_outputs
        return a

    @staticmethod
    def _stream_ptr(stream) -> int:
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream()
        return int(s.cuda_stream)

    def launch(self, stream=None) -> None:
        """Enqueue one full run (outputs cleared first) on ``stream``."""
        _lib.check(self.lib.mcl_b_run(C.byref(self.args), C.c_void_p(self._stream_ptr(stream))),
                   "mcl_b_run")

    def capture(self, stream=None) -> None:
        """Capture one full run into a CUDA graph (replayed by ``replay``)."""
        torch = _torch()
        s = stream if stream is not None else torch.cuda.Stream()
        self._graph_stream = s
        if self._graph is not None:  # re-capture: release the previous graph
            torch.cuda.synchronize()  # after its replays have finished
            self.lib.mcl_graph_destroy(self._graph)
            self._graph = None
        g = C.c_void_p()
        _lib.check(self.lib.mcl_b_graph_create(C.byref(self.args), C.c_void_p(int(s.cuda_stream)),
                                               C.byref(g)), "mcl_b_graph_create")
        self._graph = g

    def replay(self, stream=None) -> None:
        if self._graph is None:
            self.capture()
        _lib.check(self.lib.mcl_graph_launch(self._graph, C.c_void_p(self._stream_ptr(stream))),
                   "mcl_graph_launch")

    def __del__(self):
        g = getattr(self, "_graph", None)
        if g is not None and getattr(self, "lib", None) is not None:
            try:
                self.lib.mcl_graph_destroy(g)
            except Exception:
                pass

    # -- results ---------------------------------------------------------------
    def status(self) -> int:
        return int(self.d_status.item())

    def result(self) -> BatchResult:
        st = self.status()
        if st != 0:
            raise _lib.MclError(st, "kinetics kernel reported", detail=False)
        lum = self.d_lum.cpu().numpy().view(np.uint32)[:self.n_bins_total]
        alive = self.d_alive.cpu().numpy().view(np.uint32)[:self.n_bins_total] if self.d_alive is not None else None
        fates = self.d_fates.cpu().numpy()[:self.n_slots_total] if self.d_fates is not None else None
        return BatchResult(lum, alive, fates, self.bin_offsets, self.slot_offsets)

    @property
    def trials(self) -> int:
        """Electron-step trials of one run: sum over sets of slots x steps."""
        return self._trials


def simulate_batch(specs: Sequence[SetSpec], **kw) -> BatchResult:
    """One call: host specs in, host bins out (synchronises the stream)."""
    torch = _torch()
    b = BernoulliBatch(specs, **kw)
    b.launch()
    torch.cuda.current_stream().synchronize()
    return b.result()
