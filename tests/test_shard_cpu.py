"""Multi-rank sharding of a batch (host logic), on CPU with gloo.

The per-rank simulation is the oracle here (no GPU): the point is that the
shard assignment covers every set exactly once, stays balanced, and that the
gathered result equals the single-process result bit for bit, because every
draw is keyed by the set's id and not by its position or rank.
"""
import os
import socket

import numpy as np
import pytest

from mcluminescence_gb300 import schedule
from mcluminescence_gb300.batch import BatchResult
from mcluminescence_gb300.shard import assemble, run_sharded, shard_for_rank, shard_indices
from oracle import bernoulli as ob


def small_specs(n=10):
    """Small sets of every segment kind (TL ramp, isothermal hold, irradiation
    then optical stimulation) with ragged sizes and step counts."""
    S = schedule
    specs = []
    for k in range(n):
        if k % 3 == 0:
            sp = S.single_tl_set(alpha=4.0 + 0.3 * k, n_slots=40 + 7 * k, E=1.3, s=1e12, beta=2.0,
                                 dt=0.5, T_end_C=300.0, set_id=100 + k)
        elif k % 3 == 1:
            sp = S.SetSpec(n_slots=30 + 5 * k, E=1.1, s=1e11, alpha=3.0, set_id=100 + k,
                           segments=[S.isothermal(180.0, 80.0, 2.0, 8.0)])
        else:
            sp = S.SetSpec(n_slots=25 + 3 * k, n_filled=0, E=1.4, s=1e12, alpha=2.5, set_id=100 + k,
                           segments=[S.irradiate(6.0, 0.2, 80.0, 1.0, bin_seconds=5.0),
                                     S.optical(0.05, 30.0, 1.0, bin_seconds=5.0)])
        specs.append(sp.finalize())
    return specs


def oracle_runner(seed):
    def run(specs):
        lums, alives, fates = [], [], []
        for sp in specs:
            lum, alive, fate = ob.run_set(sp.to_dict(), layout="f32", seed=seed, want_fates=True)
            lums.append(lum.astype(np.uint32))
            alives.append(alive.astype(np.uint32))
            fates.append(fate.astype(np.int32))
        b_off = np.concatenate([[0], np.cumsum([len(x) for x in lums])]).astype(np.int64)
        s_off = np.concatenate([[0], np.cumsum([len(x) for x in fates])]).astype(np.int64)
        cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0)
        return BatchResult(cat(lums), cat(alives), cat(fates), b_off, s_off)
    return run


def test_shard_indices_cover_once_and_balance():
    w = [5, 1, 9, 3, 3, 7, 2, 8, 1, 4]
    for world in (1, 2, 3, 4, 16):
        shards = shard_indices(w, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(w)))
        loads = [sum(w[i] for i in s) for s in shards]
        if world <= len(w):
            assert max(loads) - min(loads) <= max(w)
    assert shard_indices(w, 3) == shard_indices(w, 3)
    with pytest.raises(ValueError):
        shard_indices(w, 0)


def test_assemble_rejects_gaps_and_duplicates():
    specs = small_specs(3)
    res = oracle_runner(1)(specs)
    parts = [([0, 1], [res.lum_of(0), res.lum_of(1)], None, None)]
    with pytest.raises(ValueError, match="not simulated"):
        assemble(specs, parts)
    parts.append(([1, 2], [res.lum_of(1), res.lum_of(2)], None, None))
    with pytest.raises(ValueError, match="two ranks"):
        assemble(specs, parts)


def test_single_rank_path_matches_direct_run():
    specs = small_specs(6)
    direct = oracle_runner(3)(specs)
    got = run_sharded(specs, oracle_runner(3), rank=0, world=1)
    assert np.array_equal(got.lum, direct.lum)
    assert np.array_equal(got.alive, direct.alive)
    assert np.array_equal(got.fates, direct.fates)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, seed, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        specs = small_specs(10)
        res = run_sharded(specs, oracle_runner(seed))
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), lum=res.lum, alive=res.alive, fates=res.fates,
                 mine=np.array(shard_for_rank(specs, rank, world)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_ranks_reproduce_single_process_result(tmp_path, world):
    import torch.multiprocessing as mp
    seed = 11
    mp.spawn(_worker, args=(world, _free_port(), seed, str(tmp_path)), nprocs=world, join=True)
    specs = small_specs(10)
    ref = oracle_runner(seed)(specs)
    seen = []
    for r in range(world):
        d = np.load(tmp_path / f"r{r}.npz")
        assert np.array_equal(d["lum"], ref.lum)
        assert np.array_equal(d["alive"], ref.alive)
        assert np.array_equal(d["fates"], ref.fates)
        seen += list(d["mine"])
    assert sorted(seen) == list(range(len(specs)))
