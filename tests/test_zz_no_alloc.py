"""The Bernoulli launch that allocates nothing (``mcl_b_run_static``).

Some callers may not allocate GPU memory at all -- a host application that
owns every byte of device memory through its own pool, or a plugin framework
that forbids cudaMalloc because it can stall on queued work.  For them the
library offers one launch that takes only inputs and outputs and keeps its
scratch (work ticket and per-step rate table) in a fixed array of its own.
These tests call it through the C ABI and check that it returns exactly what
the workspace-based ``mcl_b_run`` returns, twice in a row (the array keeps the
previous call's contents, which must not leak into the next), and that an
oversized batch is refused before anything runs.  The file is named to be
collected last.
"""
import ctypes as C

import numpy as np
import pytest

from mcluminescence_gb300 import _lib, schedule


def _specs():
    S = schedule
    return [s.finalize() for s in [
        S.single_tl_set(alpha=5.0, n_slots=700, set_id=41, T_end_C=380.0),
        S.SetSpec(n_slots=333, E=1.25, s=3e11, alpha=6.0, set_id=42,
                  segments=[S.isothermal(210.0, 900.0, 1.0, 20.0)]),
        S.SetSpec(n_slots=150, n_filled=0, E=1.4, s=1e12, alpha=4.0, set_id=43,
                  segments=[S.irradiate(60.0, 0.2, 80.0, 1.0, bin_seconds=10.0),
                            S.fade(1e4, 41, 1e6, dt0=1.0, steps_per_bin=7),
                            S.optical(0.05, 100.0, 0.1, T_C=50.0, bin_seconds=2.0)]),
    ]]


def _snapshot(b):
    return (b.d_lum.cpu().numpy().copy(), b.d_alive.cpu().numpy().copy(),
            b.d_fates.cpu().numpy().copy(), int(b.d_status.item()))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_static_scratch_matches_workspace_launch(precision):
    import torch
    from mcluminescence_gb300 import BernoulliBatch
    b = BernoulliBatch(_specs(), precision=precision, seed=777, want_fates=True)
    stream = torch.cuda.current_stream()
    b.launch(stream)
    torch.cuda.synchronize()
    ref = _snapshot(b)
    assert ref[3] == 0 and ref[0].sum() > 0
    lib = _lib.load()
    args = b._make_args(zero_outputs=1)
    args.workspace = None
    args.workspace_bytes = 0
    for _ in range(2):
        b.d_lum.fill_(12345)   # outputs are cleared by the call itself
        rc = lib.mcl_b_run_static(C.byref(args), C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.mcl_status_string(rc)
        torch.cuda.synchronize()
        got = _snapshot(b)
        assert got[3] == 0
        for x, y in zip(got[:3], ref[:3]):
            assert np.array_equal(x, y)


@pytest.mark.gpu
def test_static_scratch_refuses_sets_beyond_the_declared_table():
    """Sets whose rate-table rows run past the declared table_steps are
    refused on the device (status MCL_ECAPACITY), so they cannot write past
    the shared array.  The sets' real rows fit the array many times over, so a
    missed check could not leave it either."""
    import torch
    from mcluminescence_gb300 import BernoulliBatch
    b = BernoulliBatch(_specs(), precision="fp32", seed=3)
    args = b._make_args(zero_outputs=1)
    args.table_steps = 100
    lib = _lib.load()
    rc = lib.mcl_b_run_static(C.byref(args), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert b.status() == _lib.MCL_ECAPACITY


# The static array holds 16 MiB: a 256-byte ticket header, then 8-byte (FP32)
# or 16-byte (FP64) table rows.
CAPACITY = {_lib.MCL_FP32: 2_097_120, _lib.MCL_FP64: 1_048_560}


def test_static_scratch_capacity_boundary():
    """Refused on the host one row over the capacity, before any device work;
    a batch of exactly the capacity passes the host check (it then fails for
    other reasons here: no outputs, and no GPU on a CPU-only machine).  No GPU
    needed."""
    lib = _lib.load(auto_build=True)
    for prec, cap in CAPACITY.items():
        entry = 16 if prec == _lib.MCL_FP64 else 8
        assert cap == (16 * 1024 * 1024 - 256) // entry
        a = _lib.BArgs()
        a.precision = prec
        a.table_steps = cap + 1
        assert lib.mcl_b_run_static(C.byref(a), None) == _lib.MCL_ECAPACITY
        assert b"static scratch" in lib.mcl_last_error()
        a.table_steps = cap
        assert lib.mcl_b_run_static(C.byref(a), None) != _lib.MCL_ECAPACITY
