"""Golden vectors of the reference's presentation binning and smoothing.

Runs the UNMODIFIED reference functions ``hist_and_smooth`` / ``running_mean``
(src/class/plots.py:19-47) and the data path of ``plot_TL``
(src/class/plots.py:52-74, with a recording stand-in for the matplotlib axes)
on synthetic inputs and on the tables of the ``tl12_small`` golden case, and
writes ``tests/golden/post.npz``::

    MCL_REFERENCE=<checkout> python tests/golden/make_golden_post.py

Needs the reference checkout (``MCL_REFERENCE`` names its root) and the
stand-in modules of ``tests/golden/refshim``.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from refpath import reference_root  # noqa: E402

REF = reference_root()
sys.path.insert(0, os.path.join(HERE, "refshim"))
sys.path.insert(0, os.path.join(REF, "src", "class"))

import plots as ref_plots  # noqa: E402
from omegaconf import OmegaConf  # noqa: E402  (the stand-in)

# the stand-in pyplot has no colour maps; plot_TL only iterates over colours
ref_plots.plt.cm = type("cm", (), {"rainbow": staticmethod(lambda x: [None] * len(x))})


class RecordingAxes:
    """Collects the y data of every ``plot`` call; ignores the rest."""

    def __init__(self):
        self.curves = []

    def plot(self, x, y, **kw):
        self.curves.append(np.asarray(y, dtype=np.float64).copy())

    def __getattr__(self, name):
        return lambda *a, **k: None


def synthetic_cases():
    rng = np.random.default_rng(5)
    cases = []
    # (t_axis, events, bin_width, win_deg)
    t = np.sort(rng.uniform(0.0, 480.0, 3000))
    cases.append((t, rng.integers(0, 2, t.size).astype(np.float64), 1.0, 50.0))
    cases.append((t, rng.integers(0, 3, t.size) / 2.0, 1.0, 50.0))
    cases.append((t, rng.integers(0, 4, t.size) / 3.0, 2.5, 50.0))
    cases.append((t, rng.random(t.size), 0.7, 5.0))
    # values exactly on bin edges, the maximum on an edge, negatives dropped
    e = np.array([-3.0, -0.5, 0.0, 1.0, 1.0, 2.0, 2.5, 7.0, 7.0, 12.0])
    cases.append((e, np.arange(1.0, 11.0), 1.0, 3.0))
    cases.append((e, np.arange(1.0, 11.0), 2.0, 1.0))
    # fewer bins than the window (numpy's convolve swaps its operands)
    cases.append((np.array([0.2, 3.7, 9.9]), np.array([1.0, 2.0, 0.5]), 1.0, 50.0))
    cases.append((np.array([4.0]), np.array([1.0]), 1.0, 50.0))
    # unsorted input, large weights
    u = rng.uniform(0.0, 200.0, 5000)
    cases.append((u, rng.integers(0, 100, u.size).astype(np.float64), 1.0, 50.0))
    return cases


def main():
    out = {}
    for i, (t, w, bw, win) in enumerate(synthetic_cases()):
        out[f"hs{i}/t"] = t
        out[f"hs{i}/w"] = w
        out[f"hs{i}/params"] = np.array([bw, win])
        out[f"hs{i}/out"] = ref_plots.hist_and_smooth(t, w, bin_width=bw, win_deg=win)
    for i, (n, k) in enumerate([(100, 5), (7, 7), (3, 10), (1, 1), (60, 50)]):
        a = np.random.default_rng(100 + i).random(n) * 10
        out[f"rm{i}/a"] = a
        out[f"rm{i}/k"] = np.array(k)
        out[f"rm{i}/out"] = ref_plots.running_mean(a, k=k)
    # plot_TL's data path on the tables the reference's simulate() produced
    g = np.load(os.path.join(HERE, "kinetics_k.npz"))
    for case in ("tl12_small", "tl12_full"):
        cfg_plain = json.loads(bytes(g[f"{case}/cfg"]).decode())
        x_ax, lum, ratio = g[f"{case}/x_ax"], g[f"{case}/lum"], g[f"{case}/electron_ratio"]
        runs = lum.shape[-1]
        base = cfg_plain
        configs = {}
        for r in range(runs):
            rc = json.loads(json.dumps(base))
            for key, v in base["exp_type_fp"].items():
                if isinstance(v, list):
                    rc["exp_type_fp"][key] = v[r % len(v)]
            configs[r] = OmegaConf.create(rc)
        ax = RecordingAxes()
        ref_plots.plot_TL(OmegaConf.create(base), ax, x_ax, lum, ratio, configs)
        out[f"tl/{case}/n"] = np.array(len(ax.curves))
        out[f"tl/{case}/T_start"] = np.array([configs[r].exp_type_fp.T_start for r in range(runs)], float)
        out[f"tl/{case}/T_rate"] = np.array([configs[r].exp_type_fp.T_rate for r in range(runs)], float)
        for r, c in enumerate(ax.curves):
            out[f"tl/{case}/smooth{r}"] = c
    np.savez_compressed(os.path.join(HERE, "post.npz"), **out)
    print("wrote", os.path.join(HERE, "post.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
