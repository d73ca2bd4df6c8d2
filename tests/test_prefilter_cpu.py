"""The integer prefilter of the FP32 Bernoulli kernel, modelled in numpy with
the same 32-bit arithmetic as the device code (kinetics_b_device.cuh:
field_flags and the threshold b = bits(RN(2^23 + 1 + cm w))).

The kernel's results do not depend on the prefilter as long as it flags
every trial the exact test can accept; these checks cover that property
(and that it flags little else) over all 16-bit field values."""
import numpy as np

K_HOT = 0x4B007FFF
K_CAND = np.float32(8388609.0)  # 2^23 + 1


def field_flags(words: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per word: bit 15 / bit 31 flags of its low / high 16-bit field."""
    words = words.astype(np.uint32)
    ti = (b.astype(np.uint32) & np.uint32(0xFFFF))
    tt = ti | (ti << np.uint32(16))  # __byte_perm(b, 0, 0x1010)
    r = (words - tt).astype(np.uint32)
    return r & ~words & np.uint32(0x80008000)


def test_flags_cover_every_field_below_the_threshold():
    rng = np.random.default_rng(5)
    his = np.arange(65536, dtype=np.uint32)
    for ti in [0, 1, 2, 3, 17, 255, 256, 4096, 0x7FFE, 0x7FFF] + list(rng.integers(0, 0x8000, 20)):
        ti = np.uint32(ti)
        b = np.full(his.size, 0x4B000000 + int(ti), dtype=np.uint32)
        for lo in [0, 1, int(ti) - 1 if ti else 0, int(ti), int(ti) + 1, 0x7FFF, 0x8000, 0xFFFF]:
            lo = np.uint32(lo & 0xFFFF)
            words = (his << np.uint32(16)) | lo
            f = field_flags(words, b)
            lo_flag = (f & np.uint32(0x8000)) != 0
            hi_flag = (f & np.uint32(0x80000000)) != 0
            # the low field: exactly lo < TI
            assert np.all(lo_flag == (lo < ti))
            # the high field: hi < TI always flagged; at most hi == TI extra (a borrow)
            assert np.all(hi_flag[his < ti])
            extra = hi_flag & (his >= ti)
            assert np.all(his[extra] == ti) and (lo < ti or not extra.any())


def test_threshold_from_the_float_bound():
    """b = bits(RN(2^23 + 1 + y)) gives TI = b - 0x4B000000 > floor(y) for
    every y below the hot limit; above it b exceeds kHotBits."""
    rng = np.random.default_rng(7)
    y = np.concatenate([rng.uniform(0, 0x7FFF, 200000).astype(np.float32),
                        np.arange(0, 0x7FFF, dtype=np.float32) + np.float32(0.5),
                        np.arange(0, 0x7FFF, dtype=np.float32)])
    # FFMA(cm, w, 2^23 + 1) rounds once; with cm w = y exactly, float64 holds
    # 2^23 + 1 + y exactly and one rounding to float32 is the FFMA result
    r = (np.float64(K_CAND) + y.astype(np.float64)).astype(np.float32)
    b = r.view(np.uint32).astype(np.int64)
    cold = b <= K_HOT
    ti = b - 0x4B000000
    assert np.all(ti[cold] > np.floor(y[cold]))
    assert np.all(ti[cold] <= np.floor(y[cold]) + 2)
    assert np.all(y[~cold] > 0x7FFE - 1)
    for big in (np.float32(0x8000), np.float32(1e6), np.float32(np.inf)):
        rb = (np.float64(K_CAND) + np.float64(big)).astype(np.float32).view(np.uint32)
        assert int(rb) > K_HOT


def test_accepted_trials_are_flagged():
    """End to end on the model: for p = c w (the largest escape probability
    the float rounding allows, times 1 + 2^-22) every h with h 2^16 <
    ceil(p 2^32) sits below TI built from cm = c16 (1 + 2^-20)."""
    rng = np.random.default_rng(11)
    c16w = np.concatenate([rng.uniform(0, 1, 5000), rng.uniform(0, 64, 5000),
                           rng.uniform(0, 30000, 5000)])
    p16 = c16w * (1 + 2.0 ** -22)
    h_max = np.ceil(p16 * 65536.0) / 65536.0  # h 2^16 < ceil(p 2^32)  =>  h < this
    cm_w = np.float32(c16w * (1 + 2.0 ** -20))
    r = (np.float64(K_CAND) + cm_w.astype(np.float64)).astype(np.float32)
    b = r.view(np.uint32).astype(np.int64)
    ti = b - 0x4B000000
    cold = b <= K_HOT
    largest_h = np.ceil(h_max) - 1  # the largest integer below h_max
    assert np.all(largest_h[cold] < ti[cold])
