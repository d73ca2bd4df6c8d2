#!/usr/bin/env python
"""Throughput of the batched Monte Carlo trap kinetics (electron-steps/s).

Workload (one "step" = one pass of the kinetics over the whole batch):
4,096 parameter sets, E ~ U[1.2, 1.8] eV, log10 s ~ U[10, 14],
rho' log-uniform [1e-7, 1e-5] (alpha = rho'^(-1/3)), 1e3..1e5 traps per set
(log-uniform, ragged, 8.8e7 traps in all); even sets are TL ramps
(beta in {0.5, 1, 2, 5} K/s, 0 -> 500 degC, dt = 0.1 s, 1 degC bins), odd sets
isothermal holds (150..300 degC, 1e4 s, dt = 1 s, 20 s bins): 6.46e11
electron-step trials per pass, FP32 with native Philox4x32-10 uniforms.

``value``    trials / device time of one pass (CUDA events around the graph
             replay on its stream; L2 flushed between passes).
``e2e``      the same through the public API with host buffers:
             simulate_batch(specs) packs, validates, uploads, launches and
             reads the bins back every step.
``--impl reference``  the CPU restatement of the kinetics (numpy, FP64) on
             the host cores, over a bounded sample of the same sets.

Multi-GPU (torchrun): every rank runs its own 4,096-set batch (weak scaling);
sets are independent, so there is no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_SETS = 4096
WORKLOAD = "batch_tl_iso"
METRIC = "MC electron-steps/s"
UNIT = "electron-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--seed", type=int, default=20261203)
    p.add_argument("--block", type=int, default=0)
    p.add_argument("--ept", type=int, default=0)
    p.add_argument("--occupancy", type=int, default=0,
                   help="register-capped FP32 build (resident CTAs per SM it targets; 0 = default)")
    p.add_argument("--bin-copies", type=int, default=1, help="copies of the bins per FP32 CTA (1, 2, 4)")
    p.add_argument("--sets", type=int, default=N_SETS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fit", action="store_true", help="skip the surrogate training / fitting measurement")
    p.add_argument("--no-k", action="store_true", help="skip the event-driven kinetics measurement")
    p.add_argument("--fits", type=int, default=1024)
    p.add_argument("--plain-fits", type=int, default=128,
                   help="fits run with plain-MC DE (its per-fit cost does not depend on the batch)")
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="CPU work budget of the CPU-baseline sample")
    return p.parse_args()


def measured_peaks() -> dict:
    """The machine's measured peaks (MEASURED_PEAKS.json next to this file),
    else the figures recorded when it was last read."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {k: float(d[k]) for k in ("hbm_gbs", "bf16_tflops", "bf16_tflops_sustained")}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6797.2, "bf16_tflops": 1926.0, "bf16_tflops_sustained": 1735.4}


def measured_hbm_gbs() -> float:
    """Copy bandwidth measured on the GB300s (MEASURED_PEAKS.json next
    to this file), else the same figure recorded when the file was read."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6778.0


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


# ---------------------------------------------------------------------------
# CPU port (the oracle restatement, timed as the baseline)
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    st, seed = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import bernoulli as ob
    t0 = time.perf_counter()
    ob.run_set(st, layout="numpy", seed=seed)
    return time.perf_counter() - t0


def cpu_sample(specs, budget_s):
    """A deterministic sample of the sets whose trials fit ~budget_s of CPU
    work at ~1e8 trials/s/core, spread over the whole batch."""
    cores = os.cpu_count() or 1
    target = budget_s * 1e8 * cores
    order = list(range(0, len(specs), 7)) + [i for i in range(len(specs)) if i % 7]
    pick, tot = [], 0
    for i in order:
        if tot >= target:
            break
        pick.append(i)
        tot += specs[i].trials
    return pick, tot


def run_cpu(specs, pick, seed):
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    jobs = [(specs[i].to_dict(), seed) for i in sorted(pick, key=lambda i: -specs[i].trials)]
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        list(pool.imap_unordered(_cpu_worker, jobs))
    wall = time.perf_counter() - t0
    trials = sum(specs[i].trials for i in pick)
    return trials / wall, wall, trials, cores


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(index)],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def main():
    a = parse()
    rank, world, local = env_rank()
    if a.impl == "reference":
        return main_reference(a, rank, world)
    import torch
    from mcluminescence_gb300 import BernoulliBatch, schedule, simulate_batch
    from mcluminescence_gb300 import autotune

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    specs = schedule.batch_tl_iso(a.sets, seed=a.seed + 7919 * rank)
    for s in specs:
        s.set_id += rank * a.sets
    shape = autotune.Shape(a.block, a.ept, a.occupancy, a.bin_copies)
    if not shape.block or not shape.ept:
        shape = autotune.pick_bernoulli(specs, precision="fp32")
    block, ept, occ, copies = shape
    batch = BernoulliBatch(specs, precision="fp32", seed=a.seed, want_alive=True, **shape._asdict())
    stream = torch.cuda.Stream()
    batch.capture(stream)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    for _ in range(a.warmup):
        batch.replay(stream)
    stream.synchronize()
    assert batch.status() == 0

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    clocks = Clocks(torch.cuda.current_device())
    barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(a.steps)]
    t_wall = time.perf_counter()
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.zero_()                      # evict L2 between passes (untimed)
        ev[k][0].record(stream)
        batch.replay(stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    if batch.status() != 0:
        raise RuntimeError(f"kernel status {batch.status()}")
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / a.steps
    ms_max = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_max = float(t.item())
    trials = batch.trials
    total_trials = trials * world
    value = total_trials / (ms_max / 1e3)
    events_per_pass = int(batch.result().lum.sum())

    # ---- end to end through the public API (host specs in, host bins out) ----
    e2e = None
    if not a.no_e2e:
        res = simulate_batch(specs, precision="fp32", seed=a.seed, **shape._asdict())
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            res = simulate_batch(specs, precision="fp32", seed=a.seed, **shape._asdict())
        torch.cuda.synchronize()
        barrier()
        e2e_s = (time.perf_counter() - t0) / a.steps
        if world > 1:
            t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = batch.host_sets.nbytes + batch.host_segs.nbytes + batch.host_items.nbytes
        d2h = 4 * batch.n_bins_total * 2 + 4
        e2e = {"value": total_trials / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
               "path": "mcluminescence_gb300.simulate_batch (host specs -> host bins)"}

    # ---- roofline of the dominant kernel ------------------------------------
    from mcluminescence_gb300 import roofline
    # DRAM bytes per launch: ncu capture of the 512-set case (31.1 MB, almost
    # all of it the per-step rate table, which grows with the number of sets)
    # scaled by 4096/512 sets.
    traffic = 31.08e6 * a.sets / 512
    roof = roofline.bernoulli_fp32(trials, ms / 1e3, clk.get("sm_mhz"), traffic=traffic)
    roof["hbm_frac_of_measured"] = (traffic / (ms / 1e3)) / (measured_hbm_gbs() * 1e9)
    blocks_per_s = roofline.measure_philox_peak()
    roof["philox_peak_trials_per_s"] = 8 * blocks_per_s
    roof["frac_of_philox_peak"] = (trials / (ms / 1e3)) / (8 * blocks_per_s)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+u32(philox)",
        "data": "synthetic (seeded parameter sets of the batched TL + isothermal shape)",
        "config": {"workload": f"{WORKLOAD}: {a.sets} sets/GPU, ragged 1e3..1e5 traps, "
                               "half TL ramps (0.5-5 K/s to 500 C, dt 0.1 s), half isothermal "
                               "(150-300 C, 1e4 s, dt 1 s)",
                   "alpha": "rho'^(-1/3) of each set (46..215)", "events_per_pass": events_per_pass,
                   "sets_per_gpu": a.sets, "traps_per_gpu": int(sum(s.n_slots for s in specs)),
                   "trials_per_step_per_gpu": int(trials), "precision": "fp32",
                   "rng": "philox4x32-10", "block": block, "ept": ept, "occupancy_build": occ,
                   "bin_copies": copies,
                   "filling_path_built": not batch.no_fill, "n_items": batch.n_items,
                   "l2": "flushed between passes (256 MB write, untimed)",
                   "parallelism": f"replicas x{world} (independent sets, no collective)"},
        # each replayed pass launches the rate-table pre-pass and the kinetics kernel
        "e2e": e2e, "gpu_launches": 2 * a.steps,
        "gpu_launches_per_step": {"kb_tables": 1, "kb_f32": 1}, "clocks": clk, "roofline": roof,
        "wall_s_timed": t_wall,
    }
    out["batch_variants"] = variants_bench(a, rank, specs)
    out["dose_fade_irsl"] = sequence_bench(a, rank)
    out["single_set_tl"] = single_set_bench(a, rank, world)
    if not a.no_k:
        out["reference_kinetics"] = kinetics_k_bench(a, rank, world, clk.get("sm_mhz"))
    if not a.no_fit:
        out["fitting"] = fitting_bench(a, rank)
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        pick, _ = cpu_sample(specs, a.cpu_seconds)
        v, wall, tr, cores = run_cpu(specs, pick, a.seed)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                               "value_per_core": v / max(cores, 1),
                               "sample": f"{len(pick)} of the {a.sets} sets ({tr:.3e} trials, "
                                         f"{wall:.1f} s wall), oracle FP64 numpy restatement, "
                                         f"one process per core"}
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


def variants_bench(a, rank, specs_own):
    """The headline workload in FP64 (the oracle-parity arithmetic, next to
    the FP32 headline) and its signal-bearing variant (the same sets with
    alpha = 5: most TL sets empty by 500 degC) in FP32 and FP64.  Each is the
    full batch replayed from a captured graph, L2 flushed between passes."""
    import torch
    from mcluminescence_gb300 import BernoulliBatch, autotune, schedule
    sig = schedule.batch_tl_iso(a.sets, seed=a.seed + 7919 * rank, alpha=5.0)
    for s in sig:
        s.set_id += rank * a.sets
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    out = {}
    for name, specs in (("own_alpha", specs_own), ("alpha5", sig)):
        for prec in ("fp32", "fp64"):
            if name == "own_alpha" and prec == "fp32":
                continue                      # the headline measurement
            shape = autotune.pick_bernoulli(specs, precision=prec)
            b = BernoulliBatch(specs, precision=prec, seed=a.seed, want_alive=True, **shape._asdict())
            st = torch.cuda.Stream()
            b.capture(st)
            b.replay(st)
            st.synchronize()
            reps = 2 if prec == "fp64" else 3
            ms = []
            for _ in range(reps):
                with torch.cuda.stream(st):
                    flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                b.replay(st)
                e1.record(st)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            if b.status() != 0:
                raise RuntimeError(f"kernel status {b.status()}")
            m = sum(ms) / len(ms)
            out[f"{name}_{prec}"] = {
                "alpha": "rho'^(-1/3) of each set" if name == "own_alpha" else 5.0,
                "precision": prec, "sets": len(specs), "trials_per_pass": b.trials, "ms_per_pass": m,
                "electron_steps_per_s": b.trials / (m / 1e3), "events_per_pass": int(b.result().lum.sum()),
                **shape._asdict()}
            del b
    return out


def single_set_bench(a, rank, world):
    """The plain single-set TL case (2,000 traps, E = 1.45 eV, s = 3.5e12,
    0 -> 500 degC at 1 K/s, dt = 0.1 s, 1 degC bins) for alpha in {5, 10, 100}:
    one launch each on the GPU (FP32 and the FP64 oracle-parity mode, latency
    of a single small set) next to the FP64 CPU restatement on one core."""
    import torch
    from mcluminescence_gb300 import schedule, simulate_batch
    out = {}
    for alpha in (5.0, 10.0, 100.0):
        sp = [schedule.single_tl_set(alpha=alpha, set_id=1 + rank)]
        row = {}
        for prec in ("fp32", "fp64"):
            simulate_batch(sp, precision=prec, seed=a.seed)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = simulate_batch(sp, precision=prec, seed=a.seed)
            torch.cuda.synchronize()
            row[f"{prec}_ms"] = (time.perf_counter() - t0) * 1e3
            row[f"{prec}_events"] = int(res.lum.sum())
        if rank == 0 and world == 1 and not a.no_cpu_baseline:
            from oracle import bernoulli as ob
            t0 = time.perf_counter()
            lum, _, _ = ob.run_set(sp[0].to_dict(), layout="f64", seed=a.seed)
            row["cpu_port_1core_ms"] = (time.perf_counter() - t0) * 1e3
            row["cpu_port_events"] = int(lum.sum())
        out[f"alpha_{alpha:g}"] = row
    out["trials"] = int(sp[0].trials)
    out["timing"] = "wall clock around the public call (pack, upload, launch, read back)"
    return out


def sequence_bench(a, rank):
    """2,048 irradiation -> ground-state fading -> IRSL sets (dose rate
    U[0.05, 0.2] Gy/s to log-uniform 1..1000 Gy, D0 U[100, 500] Gy, 1e5 s of
    fading in 200 geometric steps, 1,000 s of IR stimulation at 50 degC in 0.1 s
    steps, sigma*Phi log-uniform 1e-3..1e-1 /s; traps start empty; uneven step
    counts) replayed from one captured CUDA graph."""
    import torch
    from mcluminescence_gb300 import BernoulliBatch, autotune, schedule
    specs = schedule.batch_dose_fade_irsl(2048, seed=a.seed + 1 + 977 * rank)
    shape = autotune.pick_bernoulli(specs, precision="fp32")
    b = BernoulliBatch(specs, precision="fp32", seed=a.seed, want_alive=True, **shape._asdict())
    st = torch.cuda.Stream()
    b.capture(st)
    for _ in range(2):
        b.replay(st)
    st.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record(st)
    for _ in range(reps):
        b.replay(st)
    e1.record(st)
    e1.synchronize()
    if b.status() != 0:
        raise RuntimeError(f"kernel status {b.status()}")
    ms = e0.elapsed_time(e1) / reps
    steps = [s.total_steps for s in specs]
    return {"sets": len(specs), "trials_per_pass": b.trials, "ms_per_pass": ms,
            **shape._asdict(), "filling_path_built": not b.no_fill,
            "electron_steps_per_s": b.trials / (ms / 1e3), "steps_min": min(steps), "steps_max": max(steps),
            "events_per_pass": int(b.result().lum.sum())}


def _esteps(res, params):
    """Electron-steps of event-driven runs: sum over steps of the electrons
    present at the step's start (what each step evaluates)."""
    tot = 0.0
    for j, rp in enumerate(params):
        n = int(res.n_steps[j])
        r = res.electron_ratio[:n, j] * rp.N_e
        tot += rp.e0 + float(np.sum(r[:-1])) if n else 0.0
    return tot


def kinetics_k_bench(a, rank, world, sm_mhz=None):
    """Event-driven (reference) kinetics: the reference's default TL12
    configuration through the drop-in simulate() (numpy's global stream, runs
    in order), and 1,216 independent TL12-size simulations in parallel
    (Philox); next to the CPU restatement of the same loop on one TL12 run."""
    import numpy as np
    import torch
    from mcluminescence_gb300 import kinetics as K
    from mcluminescence_gb300.config import default_config, initialize_runs
    cfg = default_config()
    np.random.seed(a.seed)
    # CSV side effect off: the reference times recorded with the fixtures
    # exclude it too (its stand-in pandas wrote nothing there)
    K.simulate(cfg, write_csv=False)              # warm-up (module load)
    torch.cuda.synchronize()
    np.random.seed(a.seed)
    t0 = time.perf_counter()
    (x_ax, lum, ratio, configs), res = K.simulate(cfg, return_result=True, write_csv=False)
    torch.cuda.synchronize()
    compat_s = time.perf_counter() - t0
    runs = initialize_runs(cfg)
    params = [K.run_params(runs[r]) for r in runs for _ in range(int(cfg["exp_type_fp"]["sims"]))]
    compat_esteps = _esteps(res, params)
    # throughput: independent simulations of the TL12 rate-5 run, one CTA each
    p5 = K.run_params(runs[2])
    n_par = 8 * 152
    K.run_kinetics([p5] * 8, 20000, rng="philox", seed=1, want_events=False)
    torch.cuda.synchronize()
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    t0 = time.perf_counter()
    rp, _ = K.run_kinetics([p5] * n_par, 20000, rng="philox", seed=a.seed, want_events=False, timing=ev)
    torch.cuda.synchronize()
    par_s = time.perf_counter() - t0
    kern_s = ev[0].elapsed_time(ev[1]) / 1e3
    par_esteps = _esteps(rp, [p5] * n_par)
    from mcluminescence_gb300 import roofline
    props = torch.cuda.get_device_properties(0)
    kk_roof = roofline.kk_issue(par_esteps, kern_s, sm_mhz, props.multi_processor_count)
    out = {"compat_tl12": {"config": "reference default (TL12 x basicTL12: 4 heating rates x 2 sims, "
                                     "2000 traps, 3455 centres)", "seconds": compat_s,
                           "steps": int(np.sum(res.n_steps)), "events": int(lum.sum()),
                           "electron_steps": compat_esteps, "electron_steps_per_s": compat_esteps / compat_s},
           "parallel_tl12_rate5": {"sims": n_par, "seconds": par_s, "kernel_seconds": kern_s,
                                   "electron_steps": par_esteps,
                                   "electron_steps_per_s": par_esteps / par_s,
                                   "kernel_electron_steps_per_s": par_esteps / kern_s,
                                   "events": int(rp.lum.sum()),
                                   "roofline": kk_roof}}
    # the reference's own CPU time on two golden cases (recorded when the
    # fixtures were generated from the unmodified reference, one x86 core):
    # the same inputs through simulate() here, outputs checked bit for bit
    gold = np.load(os.path.join(HERE, "tests", "golden", "kinetics_k.npz"))
    for case in ("tl12_full", "config1_shape"):
        gcfg = json.loads(bytes(gold[f"{case}/cfg"]).decode())
        seed = int(gold[f"{case}/seed"])
        np.random.seed(seed)
        K.simulate(gcfg, write_csv=False)
        torch.cuda.synchronize()
        np.random.seed(seed)
        t0 = time.perf_counter()
        g_x, g_lum, g_ratio, _ = K.simulate(gcfg, write_csv=False)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        ref_s = float(gold[f"{case}/wall_s"])
        out[f"golden_{case}"] = {
            "seconds": secs, "reference_cpu_seconds_recorded": ref_s, "speedup_vs_reference": ref_s / secs,
            "bit_exact": bool(np.array_equal(g_lum, gold[f"{case}/lum"])
                              and np.array_equal(g_ratio, gold[f"{case}/electron_ratio"])),
            "steps": int(np.sum(gold[f"{case}/steps_taken"]))}
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        from oracle import kinetics_k as ok
        kr = ok.run_from_cfg(runs[3])          # the 20 K/s run (~1,200 steps)
        st = ok.UniformStream(np.random.RandomState(a.seed))
        t0 = time.perf_counter()
        r = ok.run_sim(kr, st, 20000)
        cpu_s = time.perf_counter() - t0
        es = r.electron_ratio[:r.n_steps] * kr.N_e
        cpu_esteps = int(kr.N_e * kr.e_ratio_start) + float(np.sum(es[:-1]))
        out["cpu_port_one_run"] = {"seconds": cpu_s, "electron_steps_per_s": cpu_esteps / cpu_s, "cores": 1,
                                   "kind": "port", "sample": "TL12 20 K/s run, oracle FP64 numpy "
                                   "restatement (no dense distance matrix)"}
    return out


def fitting_bench(a, rank):
    """Surrogate training on device-generated Monte Carlo curves (1M curves,
    6 -> 256x4 -> 200 GELU MLP, batch 4096, Adam), then 1,024 simultaneous fits
    of Poisson-noised Monte Carlo targets: surrogate-proposed / MC-verified
    versus plain-MC differential evolution, both stopping each fit at the same
    criterion (MC-verified MSE <= 1.0 x the noise floor)."""
    import numpy as np
    import torch
    from mcluminescence_gb300 import fitting as Fm, surrogate as S
    t0 = time.perf_counter()
    P, Cn = S.generate_dataset(1_000_000, seed=a.seed + 11 + 1000 * rank)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    m = S.SurrogateMLP(batch=4096, seed=0)
    hist = S.train(m, P, Cn, steps=8000, log_every=2000)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    # device time of one training step (graph-replayed) and of one forward
    # pass over the fitting DE's 32,768 candidates, with their tensor roofline
    peaks = measured_peaks()
    step_us = S.time_training_steps(m, P[:200000], Cn[:200000])
    step_flop = S.flops_per_step(m)
    inf = m.inference_copy(32768)
    xs = torch.tensor(S.sample_params(32768, np.random.default_rng(3)), dtype=torch.float32, device="cuda")
    S.predict_t(inf, xs)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        S.predict_t(inf, xs)
    e1.record()
    e1.synchronize()
    inf_us = e0.elapsed_time(e1) * 1e3 / 10
    # the forward kernel alone on inputs already standardized on the device
    inf.set_inputs(torch.tensor(S.standardize(S.sample_params(32768, np.random.default_rng(4))),
                                dtype=torch.float32, device="cuda"))
    inf.forward()
    e0.record()
    for _ in range(10):
        inf.forward()
    e1.record()
    e1.synchronize()
    inf_kernel_us = e0.elapsed_time(e1) * 1e3 / 10
    inf_flop = sum(2.0 * 32768 * k * n for k, n in zip(inf.ins, inf.outs))
    mlp_roof = {
        "bound": "tensor", "unit": "TFLOP/s",
        "train_step_us": step_us, "train_step_flop": step_flop,
        "achieved": step_flop / (step_us * 1e-6) / 1e12, "peak": peaks["bf16_tflops_sustained"],
        "frac": step_flop / (step_us * 1e-6) / 1e12 / peaks["bf16_tflops_sustained"],
        "peak_basis": "bf16_tflops_sustained of measured (a training run is a long loop)",
        "predict_32768_us": inf_us,
        "forward_32768_us": inf_kernel_us,
        "forward_32768_tflops": inf_flop / (inf_kernel_us * 1e-6) / 1e12,
        "forward_32768_frac_of_burst": inf_flop / (inf_kernel_us * 1e-6) / 1e12 / peaks["bf16_tflops"],
        "kernels_per_step": ({"mlp_fused": 1, "wgrad_adam": 1} if m.use_fused and m.use_wgrad_adam else
                             {"mlp_fused": 1, "gemm_nt_tc_grouped": 1, "adam_multi": 1} if m.use_fused else
                             "layer by layer"),
    }
    Ph, Ch = S.generate_dataset(10000, seed=a.seed + 12, id0=10 ** 7)
    pred = S.target_to_curve(S.predict(m, Ph))
    big = Ch > 20
    err_over_se = float(np.sqrt(np.mean((pred[big] - Ch[big]) ** 2 / Ch[big])))
    prob = Fm.make_problem(a.fits, seed=a.seed + 5)
    warm = Fm.make_problem(8, seed=a.seed + 6)            # load every kernel before timing
    Fm.fit_surrogate(warm, m, seed=0, rounds=1, sur_gens=2, max_mc_gens=1)
    Fm.fit_plain_mc(warm, max_gens=1, seed=0)
    sur = Fm.reverify(prob, Fm.fit_surrogate(prob, m, seed=1, accept_factor=1.0))
    sub = Fm._subproblem(prob, torch.arange(min(a.plain_fits, a.fits), device="cuda"))
    plain = Fm.reverify(sub, Fm.fit_plain_mc(sub, pop=32, max_gens=60, seed=1, accept_factor=1.0))
    train_s = t2 - t0
    # the same fits answered by the surrogate path, for a like-for-like median
    sur_sub_rev = float(np.median(sur.reverified_ratios[:sub.floor.numel()]))
    return {
        "surrogate": {"train_curves": len(P), "datagen_s": t1 - t0, "train_steps": 8000,
                      "train_s": t2 - t1, "loss_history": hist,
                      "heldout_curves": len(Ph), "heldout_rms_err_over_mc_se": err_over_se},
        "mlp_roofline": mlp_roof,
        "surrogate_mc": sur.as_dict(), "plain_mc": plain.as_dict(),
        "fits_per_s_ratio": sur.fits_per_s / plain.fits_per_s if plain.fits_per_s else None,
        "mc_trials_per_fit_ratio": (plain.mc_trials / plain.n_fits) / (sur.mc_trials / sur.n_fits),
        "surrogate_fits_per_s_incl_training": sur.accepted / (sur.seconds + train_s),
        "reverified_median_rel_diff": (sur.reverified_ratio_median - plain.reverified_ratio_median)
        / plain.reverified_ratio_median,
        "surrogate_reverified_median_on_plain_fits": sur_sub_rev,
        "acceptance": "both methods stop each fit at its first Monte Carlo evaluation with MSE of "
                      "area-normalised curves <= 1.0 x its noise floor (the expected MSE of the true "
                      "parameters: Poisson at ~1e4 peak counts + 20,000-trap Monte Carlo); "
                      "'reverified' scores each answer again with a fresh, independent Monte Carlo run",
    }


def main_reference(a, rank, world):
    """The CPU restatement of the kinetics (the reference has no compiled or GPU
    path) on this host's cores, on a bounded sample of the same workload."""
    if rank != 0:
        return
    from mcluminescence_gb300 import schedule
    specs = schedule.batch_tl_iso(a.sets, seed=a.seed)
    pick, _ = cpu_sample(specs, a.cpu_seconds)
    times = []
    for k in range(a.warmup + a.steps):
        v, wall, tr, cores = run_cpu(specs, pick, a.seed + k)
        if k >= a.warmup:
            times.append(wall)
    wall = statistics.mean(times)
    value = tr / wall
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": wall * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded parameter sets of the batched TL + isothermal shape)",
        "config": {"workload": f"{WORKLOAD}: sample of {len(pick)} of {a.sets} sets",
                   "trials_per_step": int(tr)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{len(pick)} sets, {tr:.3e} trials per step, oracle FP64 "
                                   "numpy restatement, one process per core"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
