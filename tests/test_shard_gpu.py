"""Sharded batch on the GPU: two ranks (gloo for the host-side gather) each
simulate their share with the CUDA kernel on cuda:0; the gathered result is
bit-identical to one process simulating the whole batch.  The ranks'
kernels never wait on each other (the only exchange is the gather of
finished per-set curves on the host)."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def specs():
    from mcluminescence_gb300 import schedule
    out = [schedule.single_tl_set(alpha=4.0 + i, n_slots=500 + 97 * i, set_id=200 + i, T_end_C=350.0)
           for i in range(6)]
    out += schedule.batch_dose_fade_irsl(6, seed=3, n_min=200, n_max=700, fade_steps=30)
    for k, sp in enumerate(out[6:]):
        sp.set_id = 300 + k
    return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        torch.cuda.set_device(0)
        from mcluminescence_gb300 import simulate_batch_sharded
        res = simulate_batch_sharded(specs(), precision="fp32", seed=17, want_fates=True)
        np.savez(os.path.join(out_dir, f"g{rank}.npz"), lum=res.lum, alive=res.alive, fates=res.fates)
    finally:
        dist.destroy_process_group()


def test_two_ranks_on_one_gpu_reproduce_the_single_process_batch(tmp_path):
    import torch.multiprocessing as mp
    from mcluminescence_gb300 import simulate_batch
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    ref = simulate_batch(specs(), precision="fp32", seed=17, want_fates=True)
    for r in range(2):
        d = np.load(tmp_path / f"g{r}.npz")
        assert np.array_equal(d["lum"], ref.lum)
        assert np.array_equal(d["alive"], ref.alive)
        assert np.array_equal(d["fates"], ref.fates)
    assert int(ref.lum.sum()) > 100
