"""Bernoulli kernel at the benchmark's full sizes and on the benchmark's own
parameter sets.

* The first 64 sets of the batched TL + isothermal workload with their real
  trap counts (1,037 to 95,734 traps, 1.44 million in all), in the FP64
  injected-uniform mode (the oracle-parity mode), bit-exact against the FP64
  oracle fed the same uniforms: bins, filled counts at bin ends and every
  trap's fate.  The CPU oracle cannot walk these sets' full schedules (1e10
  trials), so each set runs a 256-step window of its own schedule: its first
  256 steps, or the 256 steps from the onset of escapes, with the workload's
  own alpha = rho'^(-1/3) and with the signal-bearing alpha = 5.  The FP32
  mode's fates on the same windows agree with the oracle's evaluation of the
  same 32-bit integers.
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
from mcluminescence_gb300.batch import pack_host
from oracle import bernoulli as ob

pytestmark = pytest.mark.gpu

WINDOW = 256


def window(sp, n_steps, r_quantile=None):
    """``n_steps`` consecutive steps of a single-segment set's schedule.
    With ``r_quantile`` None: its first steps.  Otherwise from the first step
    at which a trap at that quantile of r' escapes with probability >= 1e-3
    per step (the last steps if no step gets there); a TL ramp then starts at
    that step's temperature.  Trap counts, parameters and ids are kept."""
    s = copy.deepcopy(sp)
    seg = s.segments[0]
    j0 = 0
    if r_quantile is not None:
        c, _ = ob.segment_constants(s.to_dict(), seg.to_dict())
        w = np.exp(-s.alpha * (-np.log1p(-r_quantile)) ** (1.0 / 3.0))
        hit = np.nonzero(-np.expm1(-c * w) >= 1e-3)[0]
        j0 = int(hit[0]) if hit.size else seg.n_steps - n_steps
        j0 = max(0, min(j0, seg.n_steps - n_steps))
    seg.T0 = seg.T0 + seg.beta * seg.dt * j0
    seg.n_steps = min(n_steps, seg.n_steps)
    return s.finalize()


VARIANTS = {
    # name: (alpha of the batch, r' quantile of the window's onset, events at least)
    "own_alpha_first_steps": (None, None, 1),
    "own_alpha_onset": (None, 0.01, 1000),
    "alpha5_onset": (5.0, 0.5, 100000),
}


def window_batch(variant):
    alpha, q, _ = VARIANTS[variant]
    return [window(sp, WINDOW, q) for sp in schedule.batch_tl_iso(4096, alpha=alpha)[:64]]


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_fp64_injected_bit_exact_on_first_sets_of_the_batch(variant):
    specs = window_batch(variant)
    assert sum(sp.n_slots for sp in specs) == 1441510
    u_off = pack_host(specs)[4]
    u = np.random.default_rng(64).random(int(u_off[-1]))
    res = simulate_batch(specs, precision="fp64", rng="injected", uniforms=u, seed=0, want_fates=True)
    events = 0
    for i, sp in enumerate(specs):
        lum, alive, fates = ob.run_set(sp.to_dict(), layout="injected", uniforms=u[u_off[i]:u_off[i + 1]],
                                       want_fates=True)
        assert np.array_equal(res.lum_of(i), lum), i
        assert np.array_equal(res.alive_of(i), alive), i
        assert np.array_equal(res.fates_of(i), fates), i
        events += int(lum.sum())
    assert events >= VARIANTS[variant][2], events


@pytest.mark.parametrize("variant", ["own_alpha_onset", "alpha5_onset"])
def test_fp32_fates_on_first_sets_of_the_batch(variant):
    """FP32 native-Philox mode on the same windows: per-trap fates equal the
    oracle's FP64 evaluation of the same 32-bit integers, up to a few flips
    where p differs in its last float bit."""
    specs = window_batch(variant)
    res = simulate_batch(specs, precision="fp32", seed=7, want_fates=True)
    mism = ev = 0
    for i, sp in enumerate(specs):
        lum, alive, fates = ob.run_set(sp.to_dict(), layout="f32", seed=7, want_fates=True)
        mism += int(np.count_nonzero(res.fates_of(i) != fates))
        ev += int(lum.sum())
    assert ev >= VARIANTS[variant][2]
    assert mism <= 2 + ev // 100000


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
