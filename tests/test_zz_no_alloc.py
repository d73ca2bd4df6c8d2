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


def test_static_scratch_rejects_oversized_batch():
    """Refused on the host, before any device work (no GPU needed)."""
    lib = _lib.load(auto_build=True)
    a = _lib.BArgs()
    a.precision = _lib.MCL_FP32
    a.table_steps = (16 * 1024 * 1024 - 256) // 8 + 1
    assert lib.mcl_b_run_static(C.byref(a), None) == _lib.MCL_ECAPACITY
    a.precision = _lib.MCL_FP64
    a.table_steps = (16 * 1024 * 1024 - 256) // 16 + 1
    assert lib.mcl_b_run_static(C.byref(a), None) == _lib.MCL_ECAPACITY
