"""Golden copies of the long-format CSV the reference's ``simulate()`` writes.

``simulate()`` ends by writing ``results/simulations/exp_{tag}.csv`` with the
columns run,sim,step,lum,electron_ratio (src/class/simulate.py:95-110).  This
script runs the UNMODIFIED reference ``simulate()`` on three golden
configurations (those of ``kinetics_k.npz``, each given a ``tag``), with the
stand-in pandas of ``tests/golden/refshim`` writing the table for real into a
scratch directory, and stores every file's bytes and SHA-256 in
``tests/golden/simulate_csv.npz``::

    MCL_REFERENCE=<checkout> python tests/golden/make_golden_csv.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from refpath import reference_root  # noqa: E402

REF = reference_root()
sys.path.insert(0, os.path.join(HERE, "refshim"))
sys.path.insert(0, os.path.join(REF, "src", "class"))

import simulate as ref_sim  # noqa: E402
from omegaconf import OmegaConf  # noqa: E402  (the stand-in)

CASES = ("tl12_small", "cold_isothermal", "lab_physics")


def main():
    gold = np.load(os.path.join(HERE, "kinetics_k.npz"))
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        os.environ["MCL_REFSHIM_CSV_DIR"] = tmp
        for name in CASES:
            cfg = json.loads(bytes(gold[f"{name}/cfg"]).decode())
            cfg["tag"] = name
            seed = int(gold[f"{name}/seed"])
            np.random.seed(seed)
            ref_sim.simulate(OmegaConf.create(cfg))
            data = open(os.path.join(tmp, f"exp_{name}.csv"), "rb").read()
            out[f"{name}/csv"] = np.frombuffer(data, dtype=np.uint8)
            out[f"{name}/sha256"] = np.array(hashlib.sha256(data).hexdigest())
            out[f"{name}/seed"] = np.array(seed)
            n_lines = data.count(b"\n")
            print(f"{name}: {len(data)} bytes, {n_lines} lines", flush=True)
    path = os.path.join(HERE, "simulate_csv.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
