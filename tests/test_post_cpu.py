"""The oracle's presentation binning/smoothing against the reference's own
functions (golden vectors from tests/golden/make_golden_post.py)."""
import os

import numpy as np
import pytest

from oracle import post as op

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "post.npz"))


def close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * max(1.0, float(np.abs(b).max(initial=0))))


@pytest.mark.parametrize("i", range(9))
def test_hist_and_smooth_matches_reference(i):
    bw, win = G[f"hs{i}/params"]
    close(op.hist_and_smooth(G[f"hs{i}/t"], G[f"hs{i}/w"], bw, win), G[f"hs{i}/out"])


@pytest.mark.parametrize("i", range(5))
def test_running_mean_matches_reference(i):
    close(op.running_mean(G[f"rm{i}/a"], int(G[f"rm{i}/k"])), G[f"rm{i}/out"])


@pytest.mark.parametrize("case", ["tl12_small", "tl12_full"])
def test_plot_tl_data_path_matches_reference(case):
    k = np.load(os.path.join(os.path.dirname(__file__), "golden", "kinetics_k.npz"))
    curves = op.tl_curves(k[f"{case}/x_ax"], k[f"{case}/lum"], G[f"tl/{case}/T_start"], G[f"tl/{case}/T_rate"])
    assert len(curves) == int(G[f"tl/{case}/n"])
    for r, c in enumerate(curves):
        close(c, G[f"tl/{case}/smooth{r}"])


def test_empty_inputs_raise_like_the_reference():
    with pytest.raises(ValueError):
        op.running_mean([], 3)
    with pytest.raises(ValueError):
        op.histogram(np.array([-5.0]), np.array([1.0]), 1.0)
