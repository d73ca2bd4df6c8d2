"""Bernoulli-mode CUDA kernel against the FP64 oracle (GPU)."""
import numpy as np
import pytest

from mcluminescence_gb300 import BernoulliBatch, schedule, simulate_batch
from oracle import bernoulli as ob

pytestmark = pytest.mark.gpu


def mixed_specs():
    """Small sets covering every segment kind and ragged sizes/step counts."""
    S = schedule
    specs = [
        S.single_tl_set(alpha=5.0, n_slots=300, set_id=11, T_end_C=350.0),
        S.SetSpec(n_slots=257, E=1.25, s=3e11, alpha=6.0, set_id=12,
                  segments=[S.isothermal(210.0, 800.0, 1.0, 20.0)]),
        # irradiation from empty -> geometric fading -> IR stimulation
        S.SetSpec(n_slots=130, n_filled=0, E=1.4, s=1e12, alpha=4.0, set_id=13,
                  segments=[S.irradiate(60.0, 0.2, 80.0, 1.0, bin_seconds=10.0),
                            S.fade(1e4, 41, 1e6, dt0=1.0, steps_per_bin=7),
                            S.optical(0.05, 100.0, 0.1, T_C=50.0, bin_seconds=2.0)]),
        # step count not a multiple of 4, bins that do not divide the steps
        S.SetSpec(n_slots=33, E=1.1, s=1e12, alpha=2.0, set_id=14,
                  segments=[S.Segment(n_steps=1003, dt=0.05, steps_per_bin=7, T0=400.0, beta=1.5),
                            S.Segment(n_steps=1, dt=2.0, steps_per_bin=5, T0=450.0, beta=0.0),
                            S.Segment(n_steps=6, dt=1.0, steps_per_bin=6, T0=300.0, thermal=False,
                                      rate_const=0.3)]),
        # empty set and a set with traps but none filled and no filling
        S.SetSpec(n_slots=0, E=1.3, s=1e12, alpha=5.0, set_id=15,
                  segments=[S.isothermal(100.0, 10.0, 1.0, 5.0)]),
        S.SetSpec(n_slots=50, n_filled=0, E=1.3, s=1e12, alpha=5.0, set_id=16,
                  segments=[S.isothermal(100.0, 10.0, 1.0, 5.0)]),
        # a set spanning several work items
        S.single_tl_set(alpha=8.0, n_slots=2600, set_id=17, T_end_C=420.0, beta=2.0),
    ]
    return [s.finalize() for s in specs]


def oracle_all(specs, layout, seed, uniforms=None, u_off=None):
    out = []
    for i, sp in enumerate(specs):
        u = None
        if uniforms is not None:
            u = uniforms[u_off[i]:u_off[i + 1]]
        out.append(ob.run_set(sp.to_dict(), layout=layout, seed=seed, uniforms=u, want_fates=True))
    return out


def test_fp64_philox_bit_exact():
    specs = mixed_specs()
    res = simulate_batch(specs, precision="fp64", seed=2024, want_fates=True)
    for i, (lum, alive, fates) in enumerate(oracle_all(specs, "f64", 2024)):
        assert np.array_equal(res.lum_of(i), lum), i
        assert np.array_equal(res.alive_of(i), alive), i
        assert np.array_equal(res.fates_of(i), fates), i


def test_fp64_injected_bit_exact():
    specs = [s for s in mixed_specs() if all(g.fill_rate == 0 for g in s.segments)]
    from mcluminescence_gb300.batch import pack_host
    *_, u_off = pack_host(specs)
    u = np.random.RandomState(77).random_sample(int(u_off[-1]))
    res = simulate_batch(specs, precision="fp64", rng="injected", uniforms=u, want_fates=True)
    for i, (lum, alive, fates) in enumerate(oracle_all(specs, "injected", 0, u, u_off)):
        assert np.array_equal(res.lum_of(i), lum), i
        assert np.array_equal(res.alive_of(i), alive), i
        assert np.array_equal(res.fates_of(i), fates), i


def test_fp32_fates_match_fp64_oracle_on_same_stream():
    """FP32 mode draws the same 32-bit integers as the oracle's f32 layout; only
    a last-bit difference in p can flip a fate (expected ~1e-6 per event)."""
    specs = mixed_specs()
    res = simulate_batch(specs, precision="fp32", seed=99, want_fates=True)
    total_mism, total_ev = 0, 0
    for i, (lum, alive, fates) in enumerate(oracle_all(specs, "f32", 99)):
        total_mism += int(np.count_nonzero(res.fates_of(i) != fates))
        total_ev += int(lum.sum())
        assert abs(int(res.lum_of(i).sum()) - int(lum.sum())) <= 2
    assert total_ev > 1000
    assert total_mism <= 2


@pytest.mark.parametrize("block,ept,occ", [(128, 2, 0), (256, 2, 0), (256, 8, 0), (128, 8, 0),
                                            (256, 8, 2), (128, 8, 4), (256, 4, 3), (128, 4, 6),
                                            (256, 2, 4), (128, 2, 8)])
def test_fp32_launch_shape_invariance(block, ept, occ):
    specs = mixed_specs()
    ref = simulate_batch(specs, precision="fp32", seed=5, want_fates=True, block=256, ept=4)
    got = simulate_batch(specs, precision="fp32", seed=5, want_fates=True, block=block, ept=ept,
                         occupancy=occ)
    assert np.array_equal(ref.lum, got.lum)
    assert np.array_equal(ref.alive, got.alive)
    assert np.array_equal(ref.fates, got.fates)


def test_recapture_replaces_the_graph():
    import torch
    specs = mixed_specs()[:3]
    b = BernoulliBatch(specs, precision="fp32", seed=17)
    s = torch.cuda.Stream()
    b.capture(s)
    b.replay(s)
    s.synchronize()
    first = b.result().lum.copy()
    b.capture(s)
    b.replay(s)
    s.synchronize()
    assert np.array_equal(b.result().lum, first)


def test_graph_replay_is_deterministic():
    import torch
    specs = mixed_specs()
    b = BernoulliBatch(specs, precision="fp32", seed=31, want_fates=True)
    b.launch()
    torch.cuda.synchronize()
    first = b.result()
    lum0, alive0, fates0 = first.lum.copy(), first.alive.copy(), first.fates.copy()
    s = torch.cuda.Stream()
    b.capture(s)
    for _ in range(3):
        b.replay(s)
        s.synchronize()
        r = b.result()
        assert np.array_equal(r.lum, lum0)
        assert np.array_equal(r.alive, alive0)
        assert np.array_equal(r.fates, fates0)


@pytest.mark.parametrize("alpha", [5.0, 10.0, 100.0])
def test_glow_curve_statistics(alpha):
    """The single-set TL shape (2,000 traps, E = 1.45 eV, s = 3.5e12 /s,
    0 -> 500 degC at 1 K/s, dt = 0.1 s, 1 degC bins), R independent replicas in
    FP32 native-Philox mode, against the exact FP64 expected curve: bins with
    enough counts within 3 MC standard errors, allowing only as many bins
    outside as a correct sampler exceeds with probability 1e-3 (binomial
    quantile of the 0.27 % two-sided 3-sigma rate), the chi-square of those
    bins within its 1e-3..1-1e-3 band, the integrated signal within 0.5 %
    and 4 SE, and the peak temperature within 0.5 % (K)."""
    from scipy import stats
    R = 4096
    base = schedule.single_tl_set(alpha=alpha)
    specs = []
    for r in range(R):
        s = schedule.single_tl_set(alpha=alpha, set_id=1000 + r)
        specs.append(s)
    res = simulate_batch(specs, precision="fp32", seed=20261203)
    tot = np.zeros(base.n_bins)
    for i in range(R):
        tot += res.lum_of(i)
    exp = ob.expected_lum(base.to_dict()) * R
    N = R * base.n_slots
    p = exp / N
    se = np.sqrt(N * p * (1 - p))
    big = exp > 25
    if big.any():
        z = (tot[big] - exp[big]) / se[big]
        n = int(big.sum())
        allowed = stats.binom.ppf(0.999, n, 2 * stats.norm.sf(3.0))
        assert np.sum(np.abs(z) > 3) <= allowed, np.sort(np.abs(z))[-5:]
        chi2 = float(np.sum(z ** 2))
        assert stats.chi2.ppf(1e-3, n) < chi2 < stats.chi2.ppf(1 - 1e-3, n), chi2 / n
    P = exp.sum() / N
    se_tot = np.sqrt(N * P * (1 - P))
    assert abs(tot.sum() - exp.sum()) <= 4 * se_tot + 1
    # 0.5 % on the integrated signal is only testable where 3 SE < 0.5 %
    if exp.sum() > 4e5:
        assert abs(tot.sum() - exp.sum()) / exp.sum() < 0.005
        # peak of the curves after the reference's presentation smoothing
        # (50 degC boxcar, src/class/plots.py:39-47); bins start at 0 degC
        k = np.ones(50) / 50
        t_peak = np.argmax(np.convolve(tot, k, "valid")) + 273.15
        e_peak = np.argmax(np.convolve(exp, k, "valid")) + 273.15
        assert abs(t_peak - e_peak) / e_peak < 0.005


def test_fill_fade_irsl_sequence_fp64():
    specs = schedule.batch_dose_fade_irsl(6, seed=4, n_min=200, n_max=900, fade_steps=30)
    for s in specs:   # shorten the stimulation to keep the oracle quick
        s.segments[2] = schedule.optical(s.segments[2].rate_const, 200.0, 0.1, T_C=50.0,
                                         bin_seconds=1.0)
        s.finalize()
    res = simulate_batch(specs, precision="fp64", seed=8, want_fates=True)
    for i, (lum, alive, fates) in enumerate(oracle_all(specs, "f64", 8)):
        assert np.array_equal(res.lum_of(i), lum), i
        assert np.array_equal(res.alive_of(i), alive), i
        assert np.array_equal(res.fates_of(i), fates), i


def test_fill_fade_irsl_sequence_fp32_fates():
    """The filling path of the FP32 kernel (empty traps filled at the dose
    rate, then fading and optical stimulation) against the oracle on the same
    Philox integers."""
    specs = schedule.batch_dose_fade_irsl(6, seed=9, n_min=200, n_max=900, fade_steps=30)
    for s in specs:
        s.segments[2] = schedule.optical(s.segments[2].rate_const, 200.0, 0.1, T_C=50.0,
                                         bin_seconds=1.0)
        s.finalize()
    res = simulate_batch(specs, precision="fp32", seed=21, want_fates=True)
    mism, ev = 0, 0
    for i, (lum, alive, fates) in enumerate(oracle_all(specs, "f32", 21)):
        mism += int(np.count_nonzero(res.fates_of(i) != fates))
        ev += int(lum.sum())
        assert abs(int(res.alive_of(i)[-1]) - int(alive[-1])) <= 2
    assert ev > 100
    assert mism <= 2


@pytest.mark.parametrize("block,ept,occ,copies", [(256, 4, 0, 2), (256, 4, 0, 4), (128, 8, 4, 4),
                                                   (128, 2, 8, 2)])
def test_fp32_bin_copies_invariance(block, ept, occ, copies):
    """Keeping 2 or 4 copies of the bins per CTA changes only where the
    shared-memory atomics land: bins, alive counts and fates are identical."""
    specs = mixed_specs()
    ref = simulate_batch(specs, precision="fp32", seed=5, want_fates=True, block=block, ept=ept,
                         occupancy=occ)
    got = simulate_batch(specs, precision="fp32", seed=5, want_fates=True, block=block, ept=ept,
                         occupancy=occ, bin_copies=copies)
    assert np.array_equal(ref.lum, got.lum)
    assert np.array_equal(ref.alive, got.alive)
    assert np.array_equal(ref.fates, got.fates)


def test_fp32_bin_copies_over_shared_memory_is_refused():
    """12,000 bins: one copy (plus the filled counts) fits in shared memory,
    four copies do not, and the launcher says so instead of launching."""
    S = schedule
    spec = S.SetSpec(n_slots=64, E=1.3, s=1e12, alpha=5.0, set_id=1,
                     segments=[S.isothermal(150.0, 12000.0, 1.0, 1.0)]).finalize()
    assert spec.n_bins == 12000
    simulate_batch([spec], precision="fp32", seed=3)
    with pytest.raises(Exception, match="too small"):
        simulate_batch([spec], precision="fp32", seed=3, bin_copies=4)


def test_fp32_unknown_register_capped_build_is_rejected():
    with pytest.raises(Exception, match="invalid argument|EINVAL|MCL_EINVAL"):
        simulate_batch(mixed_specs()[:2], precision="fp32", seed=5, block=256, ept=8, occupancy=3)


@pytest.mark.parametrize("block,ept", [(128, 8), (256, 4)])
def test_no_fill_build_matches_general_build(block, ept):
    """Batches that never fill run the build without the filling path; it
    gives the same bins and fates as the general build."""
    import torch
    specs = [s for s in mixed_specs() if all(g.fill_rate == 0 for g in s.segments)]
    lean = BernoulliBatch(specs, precision="fp32", seed=41, block=block, ept=ept, want_fates=True)
    full = BernoulliBatch(specs, precision="fp32", seed=41, block=block, ept=ept, want_fates=True)
    assert lean.no_fill == 1
    full.args.no_fill = 0
    lean.launch()
    full.launch()
    torch.cuda.synchronize()
    a, b = lean.result(), full.result()
    assert lean.status() == 0 and full.status() == 0
    assert np.array_equal(a.lum, b.lum)
    assert np.array_equal(a.alive, b.alive)
    assert np.array_equal(a.fates, b.fates)


def test_no_fill_build_reports_a_filling_segment():
    """A launch that promises no filling segment but has one reports
    MCL_EINVAL in its status word."""
    import torch
    from mcluminescence_gb300 import _lib
    specs = [s for s in mixed_specs() if any(g.fill_rate > 0 for g in s.segments)]
    b = BernoulliBatch(specs, precision="fp32", seed=3, block=256, ept=4)
    assert b.no_fill == 0
    b.args.no_fill = 1
    b.launch()
    torch.cuda.synchronize()
    assert b.status() == _lib.MCL_EINVAL


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("what", ["table_steps", "n_bins_total", "n_slots_total", "n_segs", "item_set",
                                  "item_slot"])
def test_device_refuses_sets_outside_the_declared_sizes(precision, what):
    """A C caller whose sets disagree with the sizes it declares in
    mcl_b_args gets a status code instead of reads and writes past its
    buffers.  Every buffer here is allocated for the sets' real extents, so a
    missed check could not leave its allocation."""
    import ctypes as C
    import torch
    from mcluminescence_gb300 import _lib
    lib = _lib.load()
    specs = mixed_specs()
    b = BernoulliBatch(specs, precision=precision, seed=5, want_fates=True)
    a = b._make_args(zero_outputs=1)
    want = _lib.MCL_ECAPACITY
    keep = None
    if what == "table_steps":      # the last set's rows end one past the table
        a.table_steps -= 1
    elif what == "n_bins_total":
        a.n_bins_total -= 1
    elif what == "n_slots_total":
        a.n_slots_total -= 1
    elif what == "n_segs":
        a.n_segs -= 1
    else:
        items = b.host_items.copy()
        if what == "item_set":
            items["set"][0] = len(specs)
        else:
            items["slot_begin"][0] = -256
        keep = torch.from_numpy(items.view(np.uint8)).cuda()
        a.items = keep.data_ptr()
        want = _lib.MCL_EINVAL
    rc = lib.mcl_b_run(C.byref(a), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert b.status() == want


def test_device_refuses_too_few_injected_uniforms():
    import ctypes as C
    import torch
    from mcluminescence_gb300 import _lib
    lib = _lib.load()
    specs = [s for s in mixed_specs() if all(g.fill_rate == 0 for g in s.segments)]
    from mcluminescence_gb300.batch import pack_host
    n_u = int(pack_host(specs)[4][-1])
    u = np.random.default_rng(3).random(n_u)
    b = BernoulliBatch(specs, precision="fp64", rng="injected", uniforms=u, seed=0)
    a = b._make_args(zero_outputs=1)
    a.n_uniforms -= 1
    assert lib.mcl_b_run(C.byref(a), C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    torch.cuda.synchronize()
    assert b.status() == _lib.MCL_ECAPACITY
