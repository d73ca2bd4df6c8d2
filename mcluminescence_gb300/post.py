"""Glow curves for presentation and fitting: binning and boxcar smoothing on
the GPU (``csrc/post.cu``).

* ``tl_glow_curves(x_ax, lum, T_start, T_rate)`` -- the curves the
  reference's ``plot_TL`` draws from ``simulate()``'s tables
  (src/class/plots.py:52-74 with ``hist_and_smooth``, :39-47): per run the
  first replica's time axis, the replica-mean events, steps with t > 0,
  histogrammed by temperature and smoothed over ``win_deg``.
* ``running_mean(curves, k)`` -- src/class/plots.py:19-21 over many curves.
* ``smooth_batch(result, k)`` -- the same boxcar over every set's bins of a
  Bernoulli batch (for fitting on smoothed curves).

Inputs may be numpy arrays (uploaded) or CUDA tensors; results come back as
lists of numpy arrays.  Like the reference, an empty curve raises
``ValueError``.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .batch import BatchResult


def _torch():
    import torch
    return torch


def _dev(x, dtype):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def _stream():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _out_counts(n: np.ndarray, k: int) -> np.ndarray:
    return np.where(n >= k, n - k + 1, k - n + 1)


def running_mean_offsets(values, offsets: np.ndarray, k: int, divisor: float = 1.0) -> List[np.ndarray]:
    """Boxcar of width k over the curves [offsets[c], offsets[c+1]) of
    ``values`` (float64 or uint32, host or device), each divided by
    ``divisor`` first."""
    torch = _torch()
    lib = _lib.load()
    offsets = np.asarray(offsets, dtype=np.int64)
    n = np.diff(offsets)
    if k < 1:
        raise ValueError("k must be >= 1")
    if np.any(n <= 0):
        raise ValueError("v cannot be empty")  # numpy.convolve's complaint for an empty curve
    if isinstance(values, torch.Tensor) and values.dtype in (torch.int32, torch.uint32) or \
            (isinstance(values, np.ndarray) and values.dtype == np.uint32):
        d_in, kind = _dev(values.view(torch.int32) if isinstance(values, torch.Tensor)
                          else values.view(np.int32), torch.int32), 1
    else:
        d_in, kind = _dev(values, torch.float64), 0
    counts = _out_counts(n, k)
    out_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    d_ioff = _dev(offsets, torch.int64)
    d_ooff = _dev(out_off, torch.int64)
    d_out = torch.empty(int(out_off[-1]), dtype=torch.float64, device="cuda")
    for c0 in range(0, len(n), 65535):
        c1 = min(c0 + 65535, len(n))
        _lib.check(lib.mcl_running_mean(kind, _lib.ptr(d_in), _lib.ptr(d_ioff[c0:]), c1 - c0, int(k),
                                        float(divisor), _lib.ptr(d_ooff[c0:]), int(counts[c0:c1].max()),
                                        _lib.ptr(d_out), _stream()), "mcl_running_mean")
    host = d_out.cpu().numpy()
    return [host[out_off[c]:out_off[c + 1]] for c in range(len(n))]


def running_mean(curves: Sequence, k: int) -> List[np.ndarray]:
    """src/class/plots.py:19-21 for a list of curves."""
    arrs = [np.asarray(c, dtype=np.float64).ravel() for c in curves]
    off = np.concatenate([[0], np.cumsum([a.size for a in arrs])]).astype(np.int64)
    flat = np.concatenate(arrs) if arrs else np.zeros(0)
    return running_mean_offsets(flat, off, k)


def tl_glow_curves(x_ax, lum, T_start: Sequence[float], T_rate: Sequence[float],
                   bin_width: float = 1.0, win_deg: float = 50.0) -> List[np.ndarray]:
    """The smoothed TL curve per run that plot_TL draws (y values; x is the
    bin index, i.e. degC for 1-degree bins)."""
    torch = _torch()
    lib = _lib.load()
    steps, sims, runs = (int(v) for v in (lum.shape if hasattr(lum, "shape") else np.shape(lum)))
    if tuple(x_ax.shape) != (steps, sims, runs):
        raise ValueError("x_ax and lum must have the same (steps, sims, runs) shape")
    if len(T_start) != runs or len(T_rate) != runs:
        raise ValueError("one T_start and T_rate per run")
    d_x, d_l = _dev(x_ax, torch.float64), _dev(lum, torch.float64)
    d_t0 = _dev(np.asarray(T_start, np.float64), torch.float64)
    d_rate = _dev(np.asarray(T_rate, np.float64), torch.float64)
    d_edges = torch.empty(runs, dtype=torch.int64, device="cuda")
    s = _stream()
    _lib.check(lib.mcl_glow_extent(_lib.ptr(d_x), steps, sims, runs, _lib.ptr(d_t0), _lib.ptr(d_rate),
                                   float(bin_width), _lib.ptr(d_edges), s), "mcl_glow_extent")
    edges = d_edges.cpu().numpy()
    if np.any(edges < 0):
        raise ValueError("zero-size array to reduction operation maximum which has no identity")
    n_bins = edges - 1
    if np.any(n_bins < 1):
        raise ValueError("v cannot be empty")
    b_off = np.concatenate([[0], np.cumsum(n_bins)]).astype(np.int64)
    d_boff = _dev(b_off, torch.int64)
    d_counts = torch.empty(max(int(b_off[-1]), 1), dtype=torch.int32, device="cuda")
    d_hist = torch.empty(max(int(b_off[-1]), 1), dtype=torch.float64, device="cuda")
    d_status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(lib.mcl_glow_hist(_lib.ptr(d_x), _lib.ptr(d_l), steps, sims, runs, _lib.ptr(d_t0),
                                 _lib.ptr(d_rate), float(bin_width), _lib.ptr(d_boff), int(b_off[-1]),
                                 _lib.ptr(d_counts), _lib.ptr(d_hist), _lib.ptr(d_status), s),
               "mcl_glow_hist")
    st = int(d_status.item())
    if st != 0:
        raise _lib.MclError(st, "mcl_glow_hist (lum entries must be 0/1 event flags)", detail=False)
    k = max(1, int(win_deg / bin_width))
    return running_mean_offsets(d_hist, b_off, k)


def tl_glow_curves_from_configs(x_ax, lum, configs, bin_width: float = 1.0,
                                win_deg: float = 50.0) -> List[np.ndarray]:
    """``tl_glow_curves`` with T_start / T_rate read from the per-run configs
    that ``simulate`` returns (plots.py:58-60)."""
    runs = len(configs)
    t0 = [float(configs[r]["exp_type_fp"]["T_start"]) for r in range(runs)]
    rate = [float(configs[r]["exp_type_fp"]["T_rate"]) for r in range(runs)]
    return tl_glow_curves(x_ax, lum, t0, rate, bin_width, win_deg)


def smooth_batch(res: BatchResult, k: int, divisor: float = 1.0,
                 sets: Optional[Sequence[int]] = None) -> List[np.ndarray]:
    """Boxcar of width k over every set's event bins of a Bernoulli batch
    (divided by ``divisor``, the bin width in degC for TL bins)."""
    if sets is None:
        return running_mean_offsets(res.lum, res.bin_offsets, k, divisor)
    curves = [np.asarray(res.lum_of(i), dtype=np.uint32) for i in sets]
    off = np.concatenate([[0], np.cumsum([c.size for c in curves])]).astype(np.int64)
    flat = np.concatenate(curves) if curves else np.zeros(0, np.uint32)
    return running_mean_offsets(flat, off, k, divisor)
