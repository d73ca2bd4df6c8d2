"""Device binning/smoothing against the reference's plot_TL curves (golden)
and the oracle."""
import os

import numpy as np
import pytest

from oracle import post as op

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(__file__)
G = np.load(os.path.join(HERE, "golden", "post.npz"))
K = np.load(os.path.join(HERE, "golden", "kinetics_k.npz"))


def close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * max(1.0, float(np.abs(b).max(initial=0))))


@pytest.mark.parametrize("case", ["tl12_small", "tl12_full"])
def test_tl_glow_curves_match_reference_plot_tl(case):
    from mcluminescence_gb300 import post
    curves = post.tl_glow_curves(K[f"{case}/x_ax"], K[f"{case}/lum"], G[f"tl/{case}/T_start"],
                                 G[f"tl/{case}/T_rate"])
    assert len(curves) == int(G[f"tl/{case}/n"])
    for r, c in enumerate(curves):
        close(c, G[f"tl/{case}/smooth{r}"])


@pytest.mark.parametrize("bw,win", [(1.0, 50.0), (2.5, 20.0), (0.7, 5.0), (1.0, 1.0)])
def test_tl_glow_curves_match_oracle_other_bins(bw, win):
    from mcluminescence_gb300 import post
    x, lum = K["tl12_small/x_ax"], K["tl12_small/lum"]
    t0, rate = G["tl/tl12_small/T_start"], G["tl/tl12_small/T_rate"]
    for got, want in zip(post.tl_glow_curves(x, lum, t0, rate, bw, win), op.tl_curves(x, lum, t0, rate, bw, win)):
        close(got, want)


def test_running_mean_matches_reference():
    from mcluminescence_gb300 import post
    arrs = [G[f"rm{i}/a"] for i in range(5)]
    for i, a in enumerate(arrs):
        (got,) = post.running_mean([a], int(G[f"rm{i}/k"]))
        close(got, G[f"rm{i}/out"])


def test_smooth_batch_matches_oracle():
    from mcluminescence_gb300 import post, schedule, simulate_batch
    specs = [schedule.single_tl_set(alpha=a, n_slots=3000, set_id=40 + j, T_end_C=400.0)
             for j, a in enumerate((3.0, 5.0, 8.0))]
    res = simulate_batch(specs, precision="fp32", seed=3)
    got = post.smooth_batch(res, 50)
    for i, g in enumerate(got):
        close(g, op.running_mean(res.lum_of(i).astype(np.float64), 50))
    sub = post.smooth_batch(res, 10, divisor=2.0, sets=[2])
    close(sub[0], op.running_mean(res.lum_of(2).astype(np.float64) / 2.0, 10))


def test_errors_like_the_reference():
    from mcluminescence_gb300 import _lib, post
    x = np.zeros((5, 1, 1))
    with pytest.raises(ValueError):          # no step with t > 0
        post.tl_glow_curves(x, np.zeros((5, 1, 1)), [0.0], [1.0])
    with pytest.raises(ValueError):
        post.running_mean([np.zeros(0)], 3)
    x[:, 0, 0] = np.arange(1, 6)
    bad = np.full((5, 1, 1), 0.5)
    with pytest.raises(_lib.MclError):       # lum must hold 0/1 event flags
        post.tl_glow_curves(x, bad, [0.0], [10.0])
