"""Launch-shape autotuner for the Bernoulli kernel.

Times each (threads per CTA, traps per thread, register-capped build)
candidate with CUDA events (best of three passes) on a deterministic sample
of the batch (about 512 evenly strided sets, so the ragged size and step mix
is kept), then the bins-per-CTA knob (how many copies of its sets' bins a CTA
keeps in shared memory) on the winning shape, and caches the winner per
(device, precision, shape bucket, with or without filling segments) in a JSON
file next to the library.
"""
from __future__ import annotations

import json
import math
import os
from typing import NamedTuple, Sequence

from . import build as _build
from .schedule import SetSpec

CANDIDATES = {
    "fp32": [(256, 4, 0), (256, 2, 0), (128, 4, 0), (128, 2, 0), (256, 8, 0), (128, 8, 0),
             (256, 8, 2), (128, 8, 4), (256, 4, 3), (128, 4, 6), (256, 2, 4), (128, 2, 8)],
    "fp64": [(256, 1, 0), (256, 2, 0)],
}
BIN_COPIES = (1, 2, 4)
CACHE = os.path.join(_build.LIBDIR, "autotune.json")


class Shape(NamedTuple):
    """Launch shape of the Bernoulli kernel; ``BernoulliBatch(**shape._asdict())``."""
    block: int
    ept: int
    occupancy: int = 0
    bin_copies: int = 1


def _no_fill(specs: Sequence[SetSpec]) -> bool:
    return all(g.fill_rate <= 0.0 for s in specs for g in s.segments)


def _bucket(specs: Sequence[SetSpec], precision: str) -> str:
    import torch
    mb = max(s.n_bins for s in specs)
    steps = sum(s.total_steps for s in specs) / max(len(specs), 1)
    slots = sum(s.n_slots for s in specs) / max(len(specs), 1)
    return (f"{torch.cuda.get_device_name()}|{precision}|bins{2 ** math.ceil(math.log2(max(mb, 1)))}"
            f"|steps{2 ** round(math.log2(max(steps, 1)))}|slots{2 ** round(math.log2(max(slots, 1)))}"
            f"|{'nofill' if _no_fill(specs) else 'fill'}")


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def time_shape(specs, precision, block, ept, occupancy=0, reps=3, bin_copies=1) -> float:
    import torch
    from .batch import BernoulliBatch
    b = BernoulliBatch(specs, precision=precision, seed=1, block=block, ept=ept, want_alive=True,
                       occupancy=occupancy, bin_copies=bin_copies)
    s = torch.cuda.Stream()
    b.capture(s)
    b.replay(s)
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        b.replay(s)
        e1.record(s)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def pick_bernoulli(specs: Sequence[SetSpec], precision: str = "fp32",
                   use_cache: bool = True) -> Shape:
    """The fastest launch shape for this batch shape."""
    key = _bucket(specs, precision)
    cache = _load() if use_cache else {}
    if key in cache and len(cache[key]["best"]) == 4:
        return Shape(*cache[key]["best"])
    # about 512 sets: enough work items per CTA that the launch's tail does
    # not decide the ranking
    sample = list(specs[::max(1, len(specs) // 512)]) or list(specs)
    cands = CANDIDATES[precision]
    if _no_fill(specs):
        # the builds without the filling path already use 54-80 registers: the
        # register-capped builds only matter when the filling path is compiled in
        cands = [c for c in cands if c[2] == 0]
    times = {}
    for blk, ept, occ in cands:
        times[(blk, ept, occ)] = time_shape(sample, precision, blk, ept, occ)
    blk, ept, occ = min(times, key=times.get)
    ms = {f"{b}x{e}/{o}": t for (b, e, o), t in times.items()}
    copies, t_best = 1, times[(blk, ept, occ)]
    if precision == "fp32":
        for c in BIN_COPIES[1:]:
            t = time_shape(sample, precision, blk, ept, occ, bin_copies=c)
            ms[f"{blk}x{ept}/{occ}/bins{c}"] = t
            if t < t_best:
                copies, t_best = c, t
    best = Shape(blk, ept, occ, copies)
    cache = _load()
    cache[key] = {"best": list(best), "ms": ms}
    try:  # write-then-rename: processes sharing the library never see a torn file
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = f"{CACHE}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, CACHE)
    except OSError:
        pass
    return best
