"""ctypes binding of ``libmclum.so`` (the C ABI declared in include/mclum.h).

The library is built in-tree by ``mcluminescence_gb300.build``.  There is no
CPU fallback: if the library is missing or fails to load, every entry point
raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

MCL_OK = 0
MCL_EINVAL = -1
MCL_ECAPACITY = -2
MCL_EBUDGET = -3
MCL_ECUDA = -4
MCL_ENODEV = -5
MCL_ENOHOLE = -6
MCL_EOVERFLOW = -7

ABI_VERSION = 3

MCL_FP32 = 0
MCL_FP64 = 1
MCL_RNG_PHILOX = 0
MCL_RNG_INJECTED = 1
MCL_RNG_MT19937 = 2
MCL_SEG_THERMAL = 1

# numpy mirrors of the C structs (natural alignment, little endian)
SEG_DTYPE = np.dtype([
    ("n_steps", "<i4"), ("steps_per_bin", "<i4"), ("bin_offset", "<i4"), ("flags", "<i4"),
    ("dt", "<f8"), ("dt_growth", "<f8"), ("T0", "<f8"), ("beta", "<f8"),
    ("rate_const", "<f8"), ("fill_rate", "<f8")], align=True)
SET_DTYPE = np.dtype([
    ("n_slots", "<i4"), ("n_filled", "<i4"), ("seg_begin", "<i4"), ("seg_count", "<i4"),
    ("n_bins", "<i4"), ("set_id", "<u4"), ("bin_offset", "<i8"), ("slot_offset", "<i8"),
    ("u_offset", "<i8"), ("total_steps", "<i8"), ("step_offset", "<i8"), ("E", "<f8"), ("s", "<f8"),
    ("alpha", "<f8"), ("k_b", "<f8")], align=True)
ITEM_DTYPE = np.dtype([("set", "<i4"), ("slot_begin", "<i4")], align=True)


class BArgs(C.Structure):
    _fields_ = [
        ("sets", C.c_void_p), ("segs", C.c_void_p), ("items", C.c_void_p),
        ("lum", C.c_void_p), ("alive", C.c_void_p), ("fates", C.c_void_p),
        ("uniforms", C.c_void_p), ("status", C.c_void_p), ("workspace", C.c_void_p),
        ("workspace_bytes", C.c_int64), ("table_steps", C.c_int64), ("n_bins_total", C.c_int64),
        ("n_slots_total", C.c_int64), ("n_uniforms", C.c_int64), ("seed", C.c_uint64),
        ("n_sets", C.c_int32), ("n_segs", C.c_int32), ("n_items", C.c_int32),
        ("slots_per_item", C.c_int32), ("max_bins", C.c_int32), ("precision", C.c_int32),
        ("rng", C.c_int32), ("block", C.c_int32), ("ept", C.c_int32), ("grid", C.c_int32),
        ("zero_outputs", C.c_int32), ("occupancy", C.c_int32), ("no_fill", C.c_int32),
        ("bin_copies", C.c_int32), ("reserved", C.c_int32),
    ]


K_SIM_DTYPE = np.dtype(
    [(n, "<f8") for n in ("alpha", "b", "s", "E_cb", "E_loc_1", "E_loc_2", "D0", "Retrap", "k_b",
                          "dose_rate", "T_start", "T_rate", "dt_cap", "duration", "N_e",
                          "L", "W", "H", "Lb", "Wb", "Hb")]
    + [(n, "<i4") for n in ("e0", "n_h0", "e_cap", "h_cap", "steps")] + [("stream_id", "<u4")]
    + [(n, "<i8") for n in ("out_offset", "u_offset", "u_count", "ws_offset", "ev_offset", "ev_cap")]
    + [("loop", "<i4"), ("n_obs", "<i4"), ("obs_offset", "<i8")],
    align=True)

MCL_LOOP_SIMULATE = 0
MCL_LOOP_LAB_TL = 1
MCL_LOOP_LAB_ISO = 2


class KArgs(C.Structure):
    _fields_ = [
        ("sims", C.c_void_p), ("x_ax", C.c_void_p), ("lum", C.c_void_p), ("ratio", C.c_void_p),
        ("events", C.c_void_p), ("n_events", C.c_void_p), ("n_steps", C.c_void_p),
        ("draws", C.c_void_p), ("status", C.c_void_p), ("uniforms", C.c_void_p),
        ("mt_state", C.c_void_p), ("obs_time", C.c_void_p), ("obs_ratio", C.c_void_p),
        ("workspace", C.c_void_p), ("workspace_bytes", C.c_int64),
        ("seed", C.c_uint64), ("n_sims", C.c_int32), ("rng", C.c_int32), ("sequential", C.c_int32),
        ("block", C.c_int32), ("e_cap_max", C.c_int32), ("h_cap_max", C.c_int32),
        ("arrays_in_smem", C.c_int32), ("reserved", C.c_int32),
    ]


class AdamTensor(C.Structure):
    """mcl_adam_tensor (include/mclum.h)."""
    _fields_ = [("p", C.c_void_p), ("g", C.c_void_p), ("m1", C.c_void_p), ("m2", C.c_void_p),
                ("W", C.c_void_p), ("Wt", C.c_void_p), ("rows", C.c_int32), ("cols", C.c_int32)]


class WgradLayer(C.Structure):
    """mcl_wgrad_layer (include/mclum.h)."""
    _fields_ = [("dZt", C.c_void_p), ("Xt", C.c_void_p), ("W", C.c_void_p), ("m1", C.c_void_p),
                ("m2", C.c_void_p), ("Wb", C.c_void_p), ("Wt", C.c_void_p), ("gW", C.c_void_p),
                ("b", C.c_void_p), ("gb", C.c_void_p), ("mb", C.c_void_p), ("vb", C.c_void_p),
                ("out", C.c_int32), ("in_", C.c_int32), ("ld", C.c_int32), ("reserved", C.c_int32)]


class MlpLayer(C.Structure):
    """mcl_mlp_layer (include/mclum.h)."""
    _fields_ = [("W", C.c_void_p), ("Wt", C.c_void_p), ("bias", C.c_void_p), ("grad_b", C.c_void_p),
                ("dZt", C.c_void_p), ("gelu_grad", C.c_void_p), ("Yt", C.c_void_p)]


class MlpArgs(C.Structure):
    """mcl_mlp_args (include/mclum.h)."""
    _fields_ = [("layer", MlpLayer * 5), ("x", C.c_void_p), ("idx", C.c_void_p), ("target", C.c_void_p),
                ("out", C.c_void_p), ("xt", C.c_void_p), ("loss", C.c_void_p), ("err", C.c_void_p),
                ("loss_scale", C.c_float), ("batch", C.c_int32), ("training", C.c_int32),
                ("target_ld", C.c_int32), ("split", C.c_int32), ("reserved", C.c_int32)]


class GemmDesc(C.Structure):
    """mcl_gemm_desc (include/mclum.h)."""
    _fields_ = [("A", C.c_void_p), ("B", C.c_void_p), ("C", C.c_void_p), ("M", C.c_int32), ("N", C.c_int32),
                ("K", C.c_int32), ("lda", C.c_int32), ("ldb", C.c_int32), ("ldc", C.c_int32)]


class MclError(RuntimeError):
    """A negative status.  ``detail`` appends the library's last error text
    (set by the entry point that just returned ``code``); device status words
    pass ``detail=False``, as no entry point set a text for them."""

    def __init__(self, code: int, what: str, detail: bool = True):
        self.code = code
        lib = _LIB[0]
        msg = lib.mcl_status_string(code).decode() if lib is not None else str(code)
        extra = (lib.mcl_last_error().decode()
                 if (detail and lib is not None and code in (MCL_ECUDA, MCL_ECAPACITY)) else "")
        super().__init__(f"{what}: {msg}" + (f" ({extra})" if extra else ""))


_LIB = [None]
_LOCK = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def _declare(lib):
    vp, i32, i64, u64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_size_t
    sig = {
        "mcl_abi_version": (C.c_int, []),
        "mcl_status_string": (C.c_char_p, [C.c_int]),
        "mcl_last_error": (C.c_char_p, []),
        "mcl_struct_sizes": (C.c_int, [C.POINTER(sz)]),
        "mcl_device_info": (C.c_int, [C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
        "mcl_b_validate": (C.c_int, [vp, i32, vp, i32, i64, i64, i32, i32, i64]),
        "mcl_b_pack_items": (i64, [vp, i32, i32, vp, i64]),
        "mcl_b_workspace_size": (sz, [vp, i32, i32]),
        "mcl_b_smem_bytes": (sz, [i32, i32, i32]),
        "mcl_b_run": (C.c_int, [C.POINTER(BArgs), vp]),
        "mcl_b_graph_create": (C.c_int, [C.POINTER(BArgs), vp, C.POINTER(vp)]),
        "mcl_bench_philox": (C.c_int, [vp, i32, i32, u64, vp]),
        "mcl_b_run_static": (C.c_int, [C.POINTER(BArgs), vp]),
        "mcl_k_validate": (C.c_int, [vp, i32, i32, i32, i64, C.POINTER(i32), C.POINTER(i64),
                                     C.POINTER(i32), C.POINTER(i32)]),
        "mcl_k_run": (C.c_int, [C.POINTER(KArgs), vp]),
        "mcl_gemm_nt": (C.c_int, [i32, i32, i32, i32, vp, i32, vp, i32, vp, vp, i32, vp, i32, vp, i32, vp]),
        "mcl_gemm_nt_tc": (C.c_int, [i32, i32, i32, i32, vp, i32, vp, i32, vp, vp, i32, vp, i32, vp, i32, vp, vp]),
        "mcl_act_backward": (C.c_int, [i32, i32, vp, i32, vp, i32, i32, vp, i32, vp, i32, vp, vp]),
        "mcl_mlp_fused": (C.c_int, [C.POINTER(MlpArgs), vp]),
        "mcl_gemm_nt_tc_grouped": (C.c_int, [vp, i32, i32, vp, vp]),
        "mcl_wgrad_adam": (C.c_int, [vp, i32, i32, vp, vp, i32, C.c_float, C.c_float, C.c_float, vp, vp]),
        "mcl_mse_loss": (C.c_int, [i32, i32, i32, vp, i32, vp, i32, C.c_float, vp, i32, vp, vp]),
        "mcl_adam": (C.c_int, [i32, i32, vp, vp, vp, vp, C.c_float, C.c_float, C.c_float, C.c_float,
                               i32, vp, vp, vp]),
        "mcl_f32_to_bf16": (C.c_int, [i64, vp, vp, vp]),
        "mcl_adam_multi": (C.c_int, [vp, i32, C.c_float, C.c_float, C.c_float, C.c_float, i32, vp]),
        "mcl_adam_multi_dev": (C.c_int, [vp, i32, vp, vp, i32, C.c_float, C.c_float, C.c_float, vp]),
        "mcl_k_box_nearest": (C.c_int, [vp, i32, vp, i32, vp, i32, vp, vp, vp]),
        "mcl_k_box_waits": (C.c_int, [vp, C.c_double, vp, vp, vp, i32, vp, vp, vp]),
        "mcl_k_box_distances": (C.c_int, [vp, i32, vp, i32, vp, vp]),
        "mcl_k_region_bytes": (i64, [i32, i32, i32]),
        "mcl_k_arrays_fit_smem": (i32, [i32, i32]),
        "mcl_glow_extent": (C.c_int, [vp, i32, i32, i32, vp, vp, C.c_double, vp, vp]),
        "mcl_glow_hist": (C.c_int, [vp, vp, i32, i32, i32, vp, vp, C.c_double, vp, i64, vp, vp, vp, vp]),
        "mcl_running_mean": (C.c_int, [i32, vp, vp, i32, i32, C.c_double, vp, i64, vp, vp]),
        "mcl_graph_launch": (C.c_int, [vp, vp]),
        "mcl_graph_destroy": (C.c_int, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


EXPORTS = (
    "mcl_abi_version", "mcl_status_string", "mcl_last_error", "mcl_struct_sizes",
    "mcl_device_info", "mcl_b_validate", "mcl_b_pack_items", "mcl_b_workspace_size",
    "mcl_b_smem_bytes", "mcl_b_run", "mcl_b_graph_create", "mcl_graph_launch",
    "mcl_graph_destroy", "mcl_bench_philox", "mcl_b_run_static", "mcl_k_validate", "mcl_k_run",
    "mcl_gemm_nt", "mcl_gemm_nt_tc", "mcl_act_backward", "mcl_mse_loss", "mcl_adam", "mcl_f32_to_bf16",
    "mcl_glow_extent", "mcl_glow_hist", "mcl_running_mean", "mcl_adam_multi", "mcl_adam_multi_dev",
    "mcl_k_region_bytes", "mcl_k_arrays_fit_smem", "mcl_k_box_nearest", "mcl_k_box_waits",
    "mcl_k_box_distances", "mcl_mlp_fused", "mcl_gemm_nt_tc_grouped", "mcl_wgrad_adam",
)


def load(auto_build: bool = False):
    """Load (optionally building first) the CUDA library; raises if absent."""
    with _LOCK:
        if _LIB[0] is not None:
            return _LIB[0]
        path = lib_path()
        if auto_build:
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(
                f"CUDA library {path} is not built; run `python -c \"import __graft_entry__ as g; "
                f"g.build()\"` or `python -m mcluminescence_gb300.build` (there is no CPU fallback)")
        lib = _declare(C.CDLL(path))
        if lib.mcl_abi_version() != ABI_VERSION:
            raise RuntimeError("libmclum ABI version mismatch; rebuild the library")
        sizes = (C.c_size_t * 6)()
        lib.mcl_struct_sizes(sizes)
        want = (SEG_DTYPE.itemsize, SET_DTYPE.itemsize, ITEM_DTYPE.itemsize, C.sizeof(BArgs),
                K_SIM_DTYPE.itemsize, C.sizeof(KArgs))
        if tuple(sizes) != want:
            raise RuntimeError(f"struct layout mismatch: library {tuple(sizes)} vs binding {want}")
        _LIB[0] = lib
        return lib


def check(code: int, what: str) -> None:
    if code != MCL_OK:
        raise MclError(code, what)


def ptr(arr) -> int:
    """Device (torch tensor) or host (numpy array) data pointer, or 0 for None."""
    if arr is None:
        return 0
    if isinstance(arr, np.ndarray):
        return arr.ctypes.data
    return arr.data_ptr()
