"""Readers for the committed golden fixtures (tests/golden/*.npz)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_k():
    return np.load(os.path.join(GOLDEN, "kinetics_k.npz"))


def k_case_names(data):
    """The simulate() cases: those that stored the reference's output tables
    (the lab-objective and replay cases store an MSE instead)."""
    return sorted({k.split("/")[0] for k in data.files if k.endswith("/cfg")
                   and f"{k.split('/')[0]}/x_ax" in data.files})


def k_case(data, name):
    cfg = json.loads(bytes(data[f"{name}/cfg"]).decode())
    out = {"cfg": cfg, "seed": int(data[f"{name}/seed"]),
           "error": bytes(data[f"{name}/error"]).decode(),
           "x_ax": data[f"{name}/x_ax"], "lum": data[f"{name}/lum"],
           "electron_ratio": data[f"{name}/electron_ratio"],
           "draws": data[f"{name}/draws"], "steps_taken": data[f"{name}/steps_taken"]}
    n = int(data[f"{name}/n_sims"])
    out["events"] = [data[f"{name}/events{i}"] for i in range(n)]
    return out
