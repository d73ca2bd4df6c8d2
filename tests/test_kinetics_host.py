"""Host-side logic of the event-driven drop-in (no GPU needed)."""
import pytest

from golden_io import k_case, load_k
from mcluminescence_gb300.config import initialize_runs
from mcluminescence_gb300.kinetics import physics, run_params
from oracle import kinetics_k as ok

DATA = load_k()


@pytest.mark.parametrize("name", ["tl12_full", "lab_physics", "cold_isothermal", "config1_shape"])
def test_run_params_geometry_matches_oracle(name):
    cfg = k_case(DATA, name)["cfg"]
    for r in initialize_runs(cfg).values():
        rp = run_params(r)
        kr = ok.run_from_cfg(r)
        d, e0, nh, core, bound = ok.box_geometry(kr)
        assert rp.L == d and rp.Lb == bound[0] and rp.e0 == e0 and rp.n_h0 == nh
        assert rp.dt_cap == (kr.max_dt / kr.T_rate if kr.T_rate else 1e20)


def test_physics_keys_behave_like_the_dataclass():
    good = {"alpha": 1.0, "b": 1.0, "s": 1.0, "E_cb": 1.0, "E_loc_1": 1.0, "E_loc_2": 1.0,
            "D0": 1.0, "Retrap": 0.5, "name": "x", "D": 0, "k_b": 8.6e-5}
    assert physics(good)["k_b"] == 8.6e-5
    with pytest.raises(TypeError, match="unexpected keyword argument 'E'"):
        physics(dict(good, E=1.2))                # conf/physics_fp/BG_basic.yaml
    with pytest.raises(TypeError, match="unexpected keyword argument 'dose_rate'"):
        physics(dict(good, dose_rate=0.1))
    bad = dict(good)
    del bad["Retrap"]
    with pytest.raises(TypeError, match="missing 1 required"):
        physics(bad)


def test_default_config_is_the_reference_composition():
    import os
    from mcluminescence_gb300.config import compose, default_config
    conf = os.environ.get("MCL_REFERENCE_CONF", "/nonexistent")
    if not os.path.isdir(conf):
        pytest.skip("reference conf/ not available")
    assert compose(conf) == default_config()


@pytest.mark.parametrize("n_e,holes", [(200, 200), (2000, 2000), (20000, 20000)])
def test_event_workspace_layout_matches_validation(n_e, holes):
    """Host region offsets (library sizes) cover what validation asks for,
    in shared-memory and global-memory modes alike."""
    import ctypes as C
    from mcluminescence_gb300 import _lib
    from mcluminescence_gb300.config import default_config
    from mcluminescence_gb300.kinetics import _fill_sims, _ws_offsets
    lib = _lib.load(auto_build=True)
    cfg = default_config()
    cfg["exp_type_fp"].update({"N_e": n_e, "holes": holes, "e_ratio_start": 1})
    runs = initialize_runs(cfg)
    params = [run_params(runs[r]) for r in runs]
    sims = _fill_sims(params, 100, 64)
    total = _ws_offsets(lib, sims)
    smem, ws, em, hm = C.c_int32(), C.c_int64(), C.c_int32(), C.c_int32()
    assert lib.mcl_k_validate(_lib.ptr(sims), len(sims), _lib.MCL_RNG_PHILOX, 256, 0, C.byref(smem), C.byref(ws),
                              C.byref(em), C.byref(hm)) == 0
    assert ws.value == total
    assert smem.value == lib.mcl_k_arrays_fit_smem(em.value, hm.value)
    offs = sims["ws_offset"].astype(int)
    assert all(o % 16 == 0 for o in offs)
    for i in range(len(sims)):
        end = offs[i] + lib.mcl_k_region_bytes(int(sims[i]["e_cap"]), int(sims[i]["h_cap"]), smem.value)
        assert end <= total
        if i + 1 < len(sims):
            assert end <= offs[i + 1]
    assert (n_e <= 2000) == bool(smem.value)


def test_batches_without_filling_are_recognised():
    """The autotuner and the packer both key the lean (no filling path) build
    on every segment having fill_rate == 0."""
    from mcluminescence_gb300 import autotune, schedule
    from mcluminescence_gb300.batch import pack_host
    tl = schedule.batch_tl_iso(64, seed=1)
    dose = schedule.batch_dose_fade_irsl(16, seed=1)
    assert autotune._no_fill(tl) and not autotune._no_fill(dose)
    assert not (pack_host(tl)[1]["fill_rate"] > 0).any()
    assert (pack_host(dose)[1]["fill_rate"] > 0).any()


def test_bin_copies_must_be_one_two_or_four():
    import pytest
    from mcluminescence_gb300 import BernoulliBatch, schedule
    specs = [schedule.single_tl_set(alpha=5.0, n_slots=10, set_id=1)]
    with pytest.raises(ValueError, match="bin_copies"):
        BernoulliBatch(specs, bin_copies=3, device="cpu")
