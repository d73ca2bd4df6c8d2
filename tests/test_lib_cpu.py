"""The C-ABI library loads without a GPU, exports every declared symbol, and
its host-side entry points (validation, packing) behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mcluminescence_gb300 import _lib, schedule
from mcluminescence_gb300.batch import pack_host

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mclum.h")


@pytest.fixture(scope="module")
def lib():
    from mcluminescence_gb300 import build
    build.build()
    return _lib.load()


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mcl_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), f"{n} declared in mclum.h but not exported"
    assert set(names) <= set(_lib.EXPORTS) | set(getattr(_lib, "EXPORTS_K", ()))


def test_struct_layout(lib):
    sizes = (C.c_size_t * 6)()
    assert lib.mcl_struct_sizes(sizes) == 0
    assert tuple(sizes) == (64, 96, 8, C.sizeof(_lib.BArgs), _lib.K_SIM_DTYPE.itemsize,
                            C.sizeof(_lib.KArgs))


def test_device_info_without_gpu(lib):
    a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
    rc = lib.mcl_device_info(C.byref(a), C.byref(b), C.byref(c))
    assert rc in (0, _lib.MCL_ENODEV)


def _packed(specs):
    sets, segs, b_off, s_off, u_off = pack_host(specs)
    return sets, segs, int(b_off[-1]), int(s_off[-1]), int(u_off[-1])


def test_validate_accepts_workloads(lib):
    specs = schedule.batch_tl_iso(64, seed=1) + schedule.batch_dose_fade_irsl(16, seed=2)
    sets, segs, nb, ns, nu = _packed(specs)
    assert lib.mcl_b_validate(_lib.ptr(sets), len(sets), _lib.ptr(segs), len(segs), nb, ns,
                              _lib.MCL_FP32, _lib.MCL_RNG_PHILOX, 0) == 0


@pytest.mark.parametrize("mutate,code", [
    (lambda st, sg: st.__setitem__(("n_filled", 0), st[0]["n_slots"] + 1), _lib.MCL_EINVAL),
    (lambda st, sg: sg.__setitem__(("dt", 0), 0.0), _lib.MCL_EINVAL),
    (lambda st, sg: sg.__setitem__(("dt", 0), np.nan), _lib.MCL_EINVAL),
    (lambda st, sg: sg.__setitem__(("steps_per_bin", 0), 1), _lib.MCL_ECAPACITY),
    (lambda st, sg: st.__setitem__(("total_steps", 0), 7), _lib.MCL_EINVAL),
    (lambda st, sg: sg.__setitem__(("T0", 0), -5.0), _lib.MCL_EINVAL),
    (lambda st, sg: st.__setitem__(("alpha", 0), -1.0), _lib.MCL_EINVAL),
])
def test_validate_rejects(lib, mutate, code):
    sets, segs, nb, ns, nu = _packed([schedule.single_tl_set(alpha=5.0, n_slots=100)])
    sets = sets.copy()
    segs = segs.copy()
    # structured-array field assignment helpers
    st = {}
    sg = {}

    class View:
        def __init__(self, arr):
            self.arr = arr

        def __getitem__(self, i):
            return self.arr[i]

        def __setitem__(self, key, val):
            name, i = key
            self.arr[name][i] = val

    mutate(View(sets), View(segs))
    assert lib.mcl_b_validate(_lib.ptr(sets), len(sets), _lib.ptr(segs), len(segs), nb, ns,
                              _lib.MCL_FP32, _lib.MCL_RNG_PHILOX, 0) == code


def test_validate_injected_rules(lib):
    sp = [schedule.single_tl_set(alpha=5.0, n_slots=10, T_end_C=5.0)]
    sets, segs, nb, ns, nu = _packed(sp)
    args = (_lib.ptr(sets), 1, _lib.ptr(segs), len(segs), nb, ns)
    assert lib.mcl_b_validate(*args, _lib.MCL_FP32, _lib.MCL_RNG_INJECTED, nu) == _lib.MCL_EINVAL
    assert lib.mcl_b_validate(*args, _lib.MCL_FP64, _lib.MCL_RNG_INJECTED, nu - 1) == _lib.MCL_ECAPACITY
    assert lib.mcl_b_validate(*args, _lib.MCL_FP64, _lib.MCL_RNG_INJECTED, nu) == 0
    fill = [schedule.SetSpec(n_slots=10, n_filled=0, E=1.3, s=1e12, alpha=5.0,
                             segments=[schedule.irradiate(10.0, 0.1, 100.0, 1.0)]).finalize()]
    sets, segs, nb, ns, nu = _packed(fill)
    assert lib.mcl_b_validate(_lib.ptr(sets), 1, _lib.ptr(segs), 1, nb, ns, _lib.MCL_FP64,
                              _lib.MCL_RNG_INJECTED, nu) == _lib.MCL_EINVAL


def test_pack_items_longest_first(lib):
    specs = schedule.batch_tl_iso(200, seed=3, n_min=10, n_max=3000)
    sets, segs, nb, ns, nu = _packed(specs)
    spi = 256
    cap = sum(-(-s.n_slots // spi) for s in specs)
    items = np.zeros(cap, dtype=_lib.ITEM_DTYPE)
    n = lib.mcl_b_pack_items(_lib.ptr(sets), len(sets), spi, _lib.ptr(items), cap)
    assert n == cap
    # every slot covered exactly once
    cover = {}
    for it in items:
        cover.setdefault(int(it["set"]), []).append(int(it["slot_begin"]))
    for i, s in enumerate(specs):
        assert sorted(cover[i]) == list(range(0, s.n_slots, spi))
    cost = np.array([specs[int(it["set"])].total_steps for it in items])
    assert np.all(np.diff(cost) <= 0)
    assert lib.mcl_b_pack_items(_lib.ptr(sets), len(sets), spi, _lib.ptr(items), cap - 1) == _lib.MCL_ECAPACITY


def test_status_strings(lib):
    for code in (0, -1, -2, -3, -4, -5, -6):
        assert lib.mcl_status_string(code)


@pytest.mark.parametrize("split,batch", [(3, 128), (8, 128), (-1, 128), (1, 100)])
def test_mlp_fused_rejects_bad_split_and_batch(lib, split, batch):
    """Host-side validation: returns MCL_EINVAL before any device call."""
    x = np.zeros(6 * 128, dtype=np.float32)
    err = np.zeros(1, dtype=np.int32)
    a = _lib.MlpArgs()
    a.x, a.err, a.batch, a.split = x.ctypes.data, err.ctypes.data, batch, split
    assert lib.mcl_mlp_fused(C.byref(a), None) == _lib.MCL_EINVAL


@pytest.mark.parametrize("batch", [4096 + 128, 0, 100])
def test_wgrad_adam_refuses_batches_it_does_not_tile(lib, batch):
    """Host-side validation: returns MCL_EINVAL before any device call."""
    lr = np.ones(1, dtype=np.float32)
    base = np.zeros(1, dtype=np.int32)
    err = np.zeros(1, dtype=np.int32)
    arr = (_lib.WgradLayer * 1)(_lib.WgradLayer())
    rc = lib.mcl_wgrad_adam(C.cast(arr, C.c_void_p), 1, batch, lr.ctypes.data, base.ctypes.data, 1,
                            C.c_float(0.9), C.c_float(0.999), C.c_float(1e-8), err.ctypes.data, None)
    assert rc == _lib.MCL_EINVAL
