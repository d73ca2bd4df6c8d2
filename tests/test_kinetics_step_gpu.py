"""The step-level TLTrapSim / Box surface against the reference's own outputs.

``drive`` below is the reference's ``simulate()`` loop (src/class/simulate.py:
22-92) restated line for line, with the drop-in ``TLTrapSim`` in place of the
reference's: it touches only the surface the reference's driver uses --
``_update_lifetimes``, ``_filling_time``, ``_recomb_wait``, ``box.nearest``,
``box.add_electron``, ``box.remove_pair``, ``box.electrons`` and ``mc.N_e``.
Every golden case (the unmodified reference run with the same seed) must come
out with the same tables (times to the last bits of exp/log), and numpy's
global stream must end where the reference left it.
"""
import numpy as np
import pytest

from golden_io import k_case, k_case_names, load_k
from mcluminescence_gb300 import TLTrapSim
from mcluminescence_gb300.config import initialize_runs

pytestmark = pytest.mark.gpu

DATA = load_k()
CASES = [c for c in k_case_names(DATA) if c not in ("box_ops", "lab_tl", "lab_iso")]


def drive(cfg):
    configs = initialize_runs(cfg)
    n_runs = len(configs)
    mc0 = configs[0]["exp_type_fp"]
    steps = int(mc0["steps"])
    sims = int(mc0["sims"])
    x_ax = np.zeros((steps, sims, n_runs))
    Lum = np.zeros((steps, sims, n_runs))
    electron_ratio = np.zeros((steps, sims, n_runs))
    for run_idx, run_cfg in configs.items():
        mc = run_cfg["exp_type_fp"]
        phys = run_cfg["physics_fp"]
        duration = float(mc.get("duration", 0.0))
        e_ratio_start = float(mc.get("e_ratio_start", 0.0))
        dose_rate = float(phys.get("dose_rate", 0.0))
        T_rate = float(mc.get("T_rate", 0.0))
        MAX_dT = float(mc.get("max_dt", 0.5))
        dt_cap = MAX_dT / T_rate if T_rate else 1e20
        for j in range(sims):
            sim = TLTrapSim(run_cfg, e_ratio_start=e_ratio_start)
            t_cur = 0.0
            i = 0
            while t_cur <= duration:
                T0 = mc.get("T_start", 0)
                T_now = T0 + T_rate * t_cur + 273.15
                sim._update_lifetimes(T_now)
                dt_fill = sim._filling_time(dose_rate)
                dt_recomb = np.min(sim._recomb_wait) if sim._recomb_wait.any() else dt_fill
                dt = min(dt_fill, dt_recomb, dt_cap)
                t_cur += dt
                x_ax[i, j, run_idx] = t_cur
                if dt == dt_fill:
                    sim.box.add_electron()
                    event = 0
                elif dt == dt_recomb:
                    e_idx = int(np.argmin(sim._recomb_wait))
                    _, nearest = sim.box.nearest()
                    h_idx = int(nearest[e_idx])
                    sim.box.remove_pair(e_idx, h_idx)
                    event = 1
                else:
                    event = 0
                Lum[i, j, run_idx] = event
                electron_ratio[i, j, run_idx] = sim.box.electrons.shape[0] / sim.mc.N_e
                i += 1
                if duration and t_cur >= duration:
                    break
    return x_ax, Lum, electron_ratio


@pytest.mark.parametrize("name", CASES)
def test_reference_driver_loop_on_the_step_surface(name):
    case = k_case(DATA, name)
    np.random.seed(case["seed"])
    if case["error"]:
        with pytest.raises(IndexError):
            drive(case["cfg"])
        return
    x_ax, lum, ratio = drive(case["cfg"])
    assert np.array_equal(lum, case["lum"])
    assert np.array_equal(ratio, case["electron_ratio"])
    np.testing.assert_allclose(x_ax, case["x_ax"], rtol=1e-12, atol=0)
    after = np.random.random_sample(3)
    rs = np.random.RandomState(case["seed"])
    rs.random_sample(int(np.sum(case["draws"])))
    assert np.array_equal(after, rs.random_sample(3))


def test_box_operations_match_the_reference_script():
    """The scripted Box sequence of the golden fixtures (Box(1, 1, 1, 1.2)
    seeded with 30 electrons and 25 centres, then 80 pair creations and
    removals -- some removing an arbitrary centre -- on the unmodified
    reference Box): the same nearest distances and indices after every
    operation, and a distance matrix whose row minima agree."""
    from mcluminescence_gb300.kinetics import Box
    ops = DATA["box_ops/ops"]
    lens = DATA["box_ops/lens"]
    ends = np.cumsum(lens)
    np.random.seed(int(DATA["box_ops/seed"]))
    box = Box(1.0, 1.0, 1.0, 1.2)
    box.seed(30, 25)
    box.nearest()
    for k, (kind, e, h) in enumerate(ops):
        if kind == 0:
            box.add_electron()
        else:
            box.remove_pair(int(e), int(h))
        md, nn = box.nearest()
        lo, hi = ends[k] - lens[k], ends[k]
        assert np.array_equal(md, DATA["box_ops/d_min"][lo:hi]), k
        assert np.array_equal(nn, DATA["box_ops/nearest"][lo:hi]), k
    d = box.distances()
    assert d.shape == (box.electrons.shape[0], box.holes.shape[0])
    fresh = Box(1.0, 1.0, 1.0, 1.2)
    fresh.electrons, fresh.holes = box.electrons, box.holes
    fmd, fnn = fresh.nearest()
    assert np.array_equal(np.min(d, axis=1), fmd) and np.array_equal(np.argmin(d, axis=1), fnn)
