"""GB300-native (sm_103a) Monte Carlo trap/charge kinetics for luminescence.

Drop-in for the simulation API of MCLuminescence's ``src/class``:
``simulate(cfg)`` / ``TLTrapSim`` run the reference's event-driven kinetics on
the GPU; ``simulate_batch`` runs thousands of parameter sets of the fixed-dt
Bernoulli kinetics in one persistent launch.  All compute runs in the CUDA
library ``lib/libmclum.so`` (C ABI, include/mclum.h); there is no CPU path.
"""
from .config import compose, initialize_runs, read_yaml  # noqa: F401
from .schedule import (SetSpec, Segment, batch_dose_fade_irsl, batch_tl_iso,  # noqa: F401
                       fade, irradiate, isothermal, optical, single_tl_set, tl_ramp)
from .batch import BatchResult, BernoulliBatch, simulate_batch  # noqa: F401

__all__ = [
    "compose", "initialize_runs", "read_yaml", "SetSpec", "Segment", "tl_ramp", "isothermal",
    "irradiate", "fade", "optical", "single_tl_set", "batch_tl_iso", "batch_dose_fade_irsl",
    "BernoulliBatch", "BatchResult", "simulate_batch",
]
from .kinetics import run_kinetics, run_params, simulate, write_table  # noqa: F401,E402

__all__ += ["simulate", "run_kinetics", "run_params", "write_table"]
from .kinetics import TLTrapSim  # noqa: F401,E402

__all__ += ["TLTrapSim"]
from .shard import run_sharded, shard_for_rank, simulate_batch_sharded  # noqa: F401,E402

__all__ += ["simulate_batch_sharded", "run_sharded", "shard_for_rank"]
from .post import running_mean, smooth_batch, tl_glow_curves, tl_glow_curves_from_configs  # noqa: F401,E402

__all__ += ["tl_glow_curves", "tl_glow_curves_from_configs", "running_mean", "smooth_batch"]
