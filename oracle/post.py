"""CPU restatement of the reference's presentation binning and smoothing.

Test infrastructure only (the product computes these curves in
``csrc/post.cu``).  Follows src/class/plots.py of the reference:

* ``running_mean``     plots.py:19-21 -- numpy's 'valid' convolution with a
                       k-wide kernel of 1/k (for fewer than k values numpy
                       swaps the operands: k - n + 1 copies of sum / k);
* ``hist_and_smooth``  plots.py:39-47 -- histogram over edges
                       0, bw, 2 bw, ... (arange up to max + bw, exclusive),
                       bin j = [j bw, (j+1) bw), the last bin closed, values
                       below 0 dropped; divided by bw; running_mean with
                       k = max(1, int(win / bw));
* ``tl_curves``        plots.py:52-67 -- the data plot_TL feeds to it: the
                       first replica's time axis, the replica-mean events,
                       steps with t > 0, T = T_start + T_rate t.

Pinned against the reference's own functions by ``tests/golden/post.npz``
(``tests/golden/make_golden_post.py``).
"""
from __future__ import annotations

import math

import numpy as np


def running_mean(a, k: int) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    n = a.size
    if n == 0 or k < 1:
        raise ValueError("running_mean needs a non-empty curve and k >= 1")
    inv = 1.0 / k
    if n < k:
        return np.full(k - n + 1, float(np.sum(a * inv)))
    c = np.concatenate([[0.0], np.cumsum(a * inv)])
    # window sums; exact sums are not needed (callers compare with a tolerance)
    return np.array([np.sum(a[j:j + k] * inv) for j in range(n - k + 1)]) if n * k <= 4_000_000 \
        else c[k:] - c[:-k]


def edge_count(t_max: float, bw: float) -> int:
    """len(np.arange(0, t_max + bw, bw))."""
    return max(int(math.ceil((t_max + bw) / bw)), 0)


def histogram(t, w, bw: float) -> np.ndarray:
    t = np.asarray(t, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    n_edges = edge_count(float(t.max()), bw)
    if n_edges < 2:
        raise ValueError("fewer than two bin edges")
    edges = np.arange(n_edges, dtype=np.float64) * bw
    j = np.searchsorted(edges, t, side="right") - 1
    j[t == edges[-1]] = n_edges - 2
    keep = (j >= 0) & (j < n_edges - 1)
    hist = np.zeros(n_edges - 1)
    np.add.at(hist, j[keep], w[keep])
    return hist


def hist_and_smooth(t, w, bw: float = 1.0, win: float = 50.0) -> np.ndarray:
    return running_mean(histogram(t, w, bw) / bw, max(1, int(win / bw)))


def tl_curves(x_ax, lum, T_start, T_rate, bw: float = 1.0, win: float = 50.0):
    out = []
    for r in range(lum.shape[-1]):
        t = x_ax[:, 0, r]
        L = lum[:, :, r].mean(axis=1)
        m = t > 0
        out.append(hist_and_smooth(T_start[r] + T_rate[r] * t[m], L[m], bw, win))
    return out
