"""Bernoulli kernel at the benchmark's full sizes and on the benchmark's own
parameter sets.

* The first 64 sets of the batched TL + isothermal workload (the sets the FP64
  oracle mode covers) with the trap count capped so the CPU oracle finishes:
  FP64 Philox runs are bit-exact against the oracle, FP32 fates agree with the
  oracle's evaluation of the same 32-bit integers.
* The full 4,096-set batch and the 2,048-set dose -> fade -> IRSL batch,
  checked through size-independent invariants: in a segment without filling
  every escape empties one trap, so the filled count at each bin end equals
  the count before the segment minus the escapes so far; launch shapes give
  identical results.
"""
import copy

import numpy as np
import pytest

from mcluminescence_gb300 import schedule, simulate_batch
from oracle import bernoulli as ob

pytestmark = pytest.mark.gpu


def first_sets(n_sets=64, cap=192, alpha=None):
    specs = schedule.batch_tl_iso(4096)[:n_sets]
    out = []
    for sp in specs:
        sp = copy.deepcopy(sp)
        sp.n_slots = min(sp.n_slots, cap)
        sp.n_filled = sp.n_slots
        if alpha is not None:
            sp.alpha = alpha
        out.append(sp.finalize())
    return out


@pytest.mark.parametrize("alpha", [None, 6.0])
def test_fp64_philox_bit_exact_on_first_sets_of_the_batch(alpha):
    specs = first_sets(64 if alpha is None else 24, alpha=alpha)
    res = simulate_batch(specs, precision="fp64", seed=123, want_fates=True)
    events = 0
    for i, sp in enumerate(specs):
        lum, alive, fates = ob.run_set(sp.to_dict(), layout="f64", seed=123, want_fates=True)
        assert np.array_equal(res.lum_of(i), lum), i
        assert np.array_equal(res.alive_of(i), alive), i
        assert np.array_equal(res.fates_of(i), fates), i
        events += int(lum.sum())
    if alpha is not None:
        assert events > 500


def test_fp32_fates_on_first_sets_of_the_batch():
    specs = first_sets(24, alpha=6.0)
    res = simulate_batch(specs, precision="fp32", seed=7, want_fates=True)
    mism = ev = 0
    for i, sp in enumerate(specs):
        lum, alive, fates = ob.run_set(sp.to_dict(), layout="f32", seed=7, want_fates=True)
        mism += int(np.count_nonzero(res.fates_of(i) != fates))
        ev += int(lum.sum())
    assert ev > 500
    assert mism <= 2


def check_conservation(specs, res):
    checked = 0
    for i, sp in enumerate(specs):
        lum = res.lum_of(i).astype(np.int64)
        alive = res.alive_of(i).astype(np.int64)
        before = int(sp.n_filled)
        for sg in sp.segments:
            b0, b1 = sg.bin_offset, sg.bin_offset + sg.n_bins
            if sg.fill_rate == 0.0:
                assert np.array_equal(alive[b0:b1], before - np.cumsum(lum[b0:b1])), (i, b0)
                checked += 1
            before = int(alive[b1 - 1]) if b1 > b0 else before
    return checked


def test_full_batch_conservation_and_shape_invariance():
    specs = schedule.batch_tl_iso(4096)
    a = simulate_batch(specs, precision="fp32", seed=20261203, block=256, ept=8)
    assert check_conservation(specs, a) == 4096
    assert int(a.lum.sum()) > 0
    b = simulate_batch(specs, precision="fp32", seed=20261203, block=128, ept=4)
    assert np.array_equal(a.lum, b.lum)
    assert np.array_equal(a.alive, b.alive)


def test_dose_fade_irsl_batch_conservation():
    specs = schedule.batch_dose_fade_irsl(2048)
    res = simulate_batch(specs, precision="fp32", seed=5, block=128, ept=8)
    assert check_conservation(specs, res) == 2 * 2048   # fading and IRSL segments
    # the irradiation fills traps: the filled count after it is positive for most sets
    after_dose = [int(res.alive_of(i)[sp.segments[0].n_bins - 1]) for i, sp in enumerate(specs)]
    assert np.mean(np.array(after_dose) > 0) > 0.9
