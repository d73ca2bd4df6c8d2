"""Learned surrogate of the Monte Carlo glow curve, trained on the GPU.

A small MLP maps six physics parameters -- trap depth E, log10 s, the
tunnelling coefficient alpha, log10 rho', log10 dose and log10 heating rate --
to the 200-bin log glow curve that the Monte Carlo kernel produces (TL ramp
0 -> 500 degC, 2.5 degC bins, 2,000 traps).  Forward, backward and Adam run in
the library's own kernels (``mcl_gemm_nt_tc``: tcgen05 tensor-core GEMM with
the accumulator in tensor memory and a fused bias+GELU epilogue, BF16
operands, FP32 accumulation, split-K over a thread-block cluster for the
weight gradients; ``mcl_act_backward``, ``mcl_mse_loss``, ``mcl_adam_multi``);
torch only provides device memory and the stream.

The reference has no surrogate: its optimiser (src/class/optimizer.py:93-111)
evaluates every differential-evolution candidate with a full simulation.  Here
the surrogate proposes candidates and the Monte Carlo verifies them.

Physics of the training curves (the batched kernel's Bernoulli mode):
effective tunnelling coefficient alpha_eff = alpha * (1e-6 / rho')^(1/3)
(the centre spacing scales as rho'^(-1/3)), initial fill
N (1 - exp(-dose / D0)) with D0 = 200 Gy, TL ramp from 0 degC at beta K/s.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import _lib
from .schedule import SetSpec, Segment, C_TO_K

DIMS = (6, 256, 256, 256, 256, 200)
IN_PAD = 64
OUT_PAD = 256
N_TRAPS = 2000
D0_GY = 200.0
N_BINS = 200
BIN_C = 2.5
EPS_Y = 1e-4

# parameter ranges: E, log10 s, alpha, log10 rho', log10 dose, log10 beta
LOW = np.array([1.2, 10.0, 2.0, -7.0, 0.0, math.log10(0.5)])
HIGH = np.array([1.8, 14.0, 12.0, -5.0, 3.0, math.log10(5.0)])


def sample_params(n: int, rng: np.random.Generator) -> np.ndarray:
    return LOW + (HIGH - LOW) * rng.random((n, 6))


def standardize(p: np.ndarray) -> np.ndarray:
    """Map each parameter's range to [-1, 1]."""
    return 2.0 * (p - LOW) / (HIGH - LOW) - 1.0


def curve_spec(p: Sequence[float], set_id: int, n_traps: int = N_TRAPS) -> SetSpec:
    """The Monte Carlo set whose glow curve the surrogate learns for parameters p."""
    E, log_s, alpha, log_rho, log_dose, log_beta = (float(x) for x in p)
    beta = 10.0 ** log_beta
    k = max(1, int(math.ceil(BIN_C / (beta * 0.1) - 1e-9)))   # steps per 2.5 degC bin, dt <= 0.1 s
    dt = BIN_C / (beta * k)
    a_eff = alpha * (1e-6 / 10.0 ** log_rho) ** (1.0 / 3.0)
    filled = int(round(n_traps * (1.0 - math.exp(-(10.0 ** log_dose) / D0_GY))))
    seg = Segment(n_steps=N_BINS * k, dt=dt, steps_per_bin=k, T0=C_TO_K, beta=beta)
    return SetSpec(n_slots=n_traps, n_filled=filled, E=E, s=10.0 ** log_s, alpha=a_eff,
                   segments=[seg], set_id=set_id, kind="tl_curve").finalize()


def pack_curves(params: np.ndarray, id0: int = 0, n_traps: int = N_TRAPS):
    """The packed host arrays (as ``batch.pack_host`` returns them) of the
    sets ``curve_spec`` builds, computed column-wise for many parameter
    vectors at once (no per-set Python objects)."""
    from . import _lib as L
    from .schedule import K_B
    p = np.asarray(params, dtype=np.float64).reshape(-1, 6)
    n = p.shape[0]
    E, log_s, alpha, log_rho, log_dose, log_beta = (p[:, i] for i in range(6))
    beta = 10.0 ** log_beta
    k = np.maximum(1, np.ceil(BIN_C / (beta * 0.1) - 1e-9).astype(np.int64))
    dt = BIN_C / (beta * k)
    a_eff = alpha * (1e-6 / 10.0 ** log_rho) ** (1.0 / 3.0)
    filled = np.rint(n_traps * (1.0 - np.exp(-(10.0 ** log_dose) / D0_GY))).astype(np.int64)
    steps = N_BINS * k
    segs = np.zeros(n, dtype=L.SEG_DTYPE)
    segs["n_steps"] = steps
    segs["steps_per_bin"] = k
    segs["bin_offset"] = 0
    segs["flags"] = L.MCL_SEG_THERMAL
    segs["dt"] = dt
    segs["dt_growth"] = 1.0
    segs["T0"] = C_TO_K
    segs["beta"] = beta
    sets = np.zeros(n, dtype=L.SET_DTYPE)
    sets["n_slots"] = n_traps
    sets["n_filled"] = filled
    sets["seg_begin"] = np.arange(n)
    sets["seg_count"] = 1
    sets["n_bins"] = N_BINS
    sets["set_id"] = (id0 + np.arange(n, dtype=np.int64)) & 0xFFFFFFFF
    b_off = np.arange(n + 1, dtype=np.int64) * N_BINS
    s_off = np.arange(n + 1, dtype=np.int64) * n_traps
    u_off = np.concatenate([[0], np.cumsum(n_traps * (1 + steps))]).astype(np.int64)
    sets["bin_offset"] = b_off[:-1]
    sets["slot_offset"] = s_off[:-1]
    sets["u_offset"] = u_off[:-1]
    sets["total_steps"] = steps
    sets["step_offset"] = np.concatenate([[0], np.cumsum(steps)[:-1]]) if n else 0
    sets["E"], sets["s"], sets["alpha"], sets["k_b"] = E, 10.0 ** log_s, a_eff, K_B
    return sets, segs, b_off, s_off, u_off


def simulate_curves(params: np.ndarray, seed: int, id0: int = 0, n_traps: int = N_TRAPS,
                    chunk: int = 65536, precision: str = "fp32") -> np.ndarray:
    """Monte Carlo glow curves (counts per bin, float32 [n][200]) on the GPU."""
    from .batch import BernoulliBatch
    import torch
    out = np.zeros((len(params), N_BINS), dtype=np.float32)
    for c0 in range(0, len(params), chunk):
        sub = params[c0:c0 + chunk]
        b = BernoulliBatch(None, packed=pack_curves(sub, id0 + c0, n_traps), precision=precision, seed=seed,
                           want_alive=False, block=128 if precision == "fp32" else 256,
                           ept=8 if precision == "fp32" else 2)
        b.launch()
        torch.cuda.synchronize()
        out[c0:c0 + len(sub)] = b.result().lum.reshape(len(sub), N_BINS)
    return out


def curve_to_target(counts: np.ndarray, n_traps: int = N_TRAPS) -> np.ndarray:
    return np.log10(counts / n_traps + EPS_Y).astype(np.float32)


def target_to_curve(y: np.ndarray, n_traps: int = N_TRAPS) -> np.ndarray:
    return np.clip(10.0 ** y - EPS_Y, 0.0, None) * n_traps


@dataclass
class Layer:
    W: object      # fp32 master [out][in]
    b: object      # fp32 [out]
    Wb: object     # bf16 [out][in]
    Wt: object     # bf16 [in][out]
    mW: object
    vW: object
    mb: object
    vb: object
    gW: object
    gb: object


class SurrogateMLP:
    """The network with its device buffers for a fixed batch size."""

    def __init__(self, batch: int = 4096, seed: int = 0, device: str = "cuda"):
        import torch
        assert batch % 64 == 0
        self.torch = torch
        self.lib = _lib.load()
        self.B = batch
        self.dev = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.ins = [IN_PAD] + [256] * 4
        self.outs = [256] * 4 + [OUT_PAD]
        self.layers: List[Layer] = []
        for l, (k, n) in enumerate(zip(self.ins, self.outs)):
            fan_in = DIMS[l]
            W = torch.zeros(n, k, dtype=torch.float32)
            W[:DIMS[l + 1], :fan_in] = (torch.rand(DIMS[l + 1], fan_in, generator=g) * 2 - 1) / math.sqrt(fan_in)
            b = torch.zeros(n, dtype=torch.float32)
            W, b = W.to(self.dev), b.to(self.dev)
            z = lambda *s: torch.zeros(*s, dtype=torch.float32, device=self.dev)
            L = Layer(W, b, W.to(torch.bfloat16).contiguous(), W.t().contiguous().to(torch.bfloat16),
                      z(n, k), z(n, k), z(n), z(n), z(n, k), z(n))
            self.layers.append(L)
        B = batch
        bf = lambda *s: torch.zeros(*s, dtype=torch.bfloat16, device=self.dev)
        f32 = lambda *s: torch.zeros(*s, dtype=torch.float32, device=self.dev)
        self.x0 = bf(B, IN_PAD)
        self.x0t = bf(IN_PAD, B)
        self.Z = [f32(B, n) for n in self.outs]
        self.Y = [bf(B, n) for n in self.outs[:-1]]
        self.Yt = [bf(n, B) for n in self.outs[:-1]]
        self.target = f32(B, OUT_PAD)
        self.dOut = f32(B, OUT_PAD)
        self.dY = [f32(B, k) for k in self.ins]
        self.dZ = [bf(B, n) for n in self.outs]
        self.dZt = [bf(n, B) for n in self.outs]
        self.loss = f32(1)
        self.tc_err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.use_tcgen05 = True
        self.training = True      # False: forward only (no transposed copies for backward)
        self.step_count = 0
        # the fused path (mcl_mlp_fused): one launch per forward pass, or per
        # forward + loss + input-gradient chain in training; then one grouped
        # launch for the weight gradients
        self.use_fused = batch % 128 == 0
        self.fused_split = 0      # CTAs per 128-row tile (1, 2, 4); 0: the library picks
        # weight gradients and Adam in one launch (mcl_wgrad_adam) after a
        # fused pass, in the device-step training loops
        self.use_wgrad_adam = batch % 256 == 0
        self._wg = None
        self.x_f32 = f32(B, 6)
        self.G = [f32(B, n) for n in self.outs[:-1]]     # GELU'(pre-activation) per hidden layer
        self.gb_all = f32(sum(self.outs))                  # the bias gradients, cleared together
        o = 0
        for L, n in zip(self.layers, self.outs):
            L.gb = self.gb_all[o:o + n]
            o += n
        self._fused = {}
        self._dw = None

    # -- plumbing -------------------------------------------------------------
    def _s(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    def _gemm(self, epi, M, N, K, A, lda, Bm, ldb, bias, Cm, ldc, Y=None, ldy=0, Yt=None, ldyt=0):
        """tcgen05 GEMM (tensor-memory accumulator) when the shape tiles by
        128 x 64 x 64, the mma.sync kernel otherwise."""
        args = (epi, M, N, K, self._p(A), lda, self._p(Bm), ldb, self._p(bias), self._p(Cm), ldc,
                self._p(Y), ldy, self._p(Yt), ldyt)
        if self.use_tcgen05 and M % 128 == 0 and N % 64 == 0 and K % 64 == 0:
            _lib.check(self.lib.mcl_gemm_nt_tc(*args, self._p(self.tc_err), self._s()), "mcl_gemm_nt_tc")
        else:
            _lib.check(self.lib.mcl_gemm_nt(*args, self._s()), "mcl_gemm_nt")

    def check_errors(self) -> None:
        """Raise if a tcgen05 completion wait timed out in any launch so far."""
        if int(self.tc_err.item()):
            raise RuntimeError("tcgen05 GEMM: a completion wait timed out")

    # -- data -----------------------------------------------------------------
    def set_inputs(self, x_std: "torch.Tensor") -> None:
        """x_std: float tensor [B][6] of standardized parameters (device)."""
        t = self.torch
        if self.use_fused:
            self.x_f32.copy_(x_std)
            return
        x = t.zeros(self.B, IN_PAD, dtype=t.bfloat16, device=self.dev)
        x[:, :6] = x_std.to(t.bfloat16)
        self.x0.copy_(x)
        if self.training:
            self.x0t.copy_(x.t())   # only the first layer's weight gradient reads it

    def set_targets(self, y: "torch.Tensor") -> None:
        self.target[:, :DIMS[-1]].copy_(y)

    # -- fused passes -----------------------------------------------------------
    def _fused_args(self, training: bool, x, idx, target, target_ld: int) -> _lib.MlpArgs:
        key = (training, x.data_ptr(), idx.data_ptr() if idx is not None else 0, target.data_ptr(), target_ld,
               self.fused_split)
        a = self._fused.get(key)
        if a is not None:
            return a
        a = _lib.MlpArgs()
        for l, L in enumerate(self.layers):
            d = a.layer[l]
            d.W, d.Wt, d.bias = L.Wb.data_ptr(), L.Wt.data_ptr(), L.b.data_ptr()
            if training:
                d.grad_b, d.dZt = L.gb.data_ptr(), self.dZt[l].data_ptr()
                if l < len(self.layers) - 1:
                    d.gelu_grad, d.Yt = self.G[l].data_ptr(), self.Yt[l].data_ptr()
        a.x = x.data_ptr()
        a.idx = idx.data_ptr() if idx is not None else None
        a.target = target.data_ptr()
        a.out = self.Z[-1].data_ptr()
        a.xt = self.x0t.data_ptr()
        a.loss = self.loss.data_ptr()
        a.err = self.tc_err.data_ptr()
        a.loss_scale = 1.0 / (self.B * DIMS[-1])
        a.batch = self.B
        a.training = 1 if training else 0
        a.target_ld = target_ld
        a.split = self.fused_split
        self._fused[key] = a
        return a

    def fused_pass(self, x, target=None, idx=None, target_ld: int = OUT_PAD) -> None:
        """One mcl_mlp_fused launch on inputs ``x`` (device fp32 [*][6],
        standardized) and, in training, ``target`` (device fp32 [*][target_ld]);
        ``idx`` (device int64 [B]) picks the rows, else rows 0..B-1.  Training
        clears the bias gradients and the loss first."""
        training = self.training and target is not None
        if training:
            self.gb_all.zero_()
            self.loss.zero_()
        a = self._fused_args(training, x, idx, target if target is not None else x, target_ld)
        _lib.check(self.lib.mcl_mlp_fused(C.byref(a), self._s()), "mcl_mlp_fused")

    def wgrad_adam_dev(self, lr_ptr: int, step_base_ptr: int, step_offset: int, b1: float = 0.9,
                       b2: float = 0.999, eps: float = 1e-8) -> None:
        """All weight gradients and one Adam step on every weight and bias in
        one launch (after a training fused_pass); lr = *lr_ptr and step =
        *step_base_ptr + step_offset are read on the device.  gW is written
        too."""
        if self._wg is None:
            ls = []
            for l, L in enumerate(self.layers):
                Xt = self.Yt[l - 1] if l > 0 else self.x0t
                d = _lib.WgradLayer()
                d.dZt, d.Xt = self.dZt[l].data_ptr(), Xt.data_ptr()
                d.W, d.m1, d.m2 = L.W.data_ptr(), L.mW.data_ptr(), L.vW.data_ptr()
                d.Wb, d.Wt, d.gW = L.Wb.data_ptr(), L.Wt.data_ptr(), L.gW.data_ptr()
                d.b, d.gb, d.mb, d.vb = L.b.data_ptr(), L.gb.data_ptr(), L.mb.data_ptr(), L.vb.data_ptr()
                d.out, d.in_, d.ld = self.outs[l], self.ins[l], self.B
                ls.append(d)
            self._wg = (_lib.WgradLayer * len(ls))(*ls)
        _lib.check(self.lib.mcl_wgrad_adam(C.cast(self._wg, C.c_void_p), len(self._wg), self.B, C.c_void_p(lr_ptr),
                                           C.c_void_p(step_base_ptr), step_offset, C.c_float(b1), C.c_float(b2),
                                           C.c_float(eps), self._p(self.tc_err), self._s()), "mcl_wgrad_adam")

    def train_step_dev(self, X, Y, idx, lr_ptr: int, step_base_ptr: int, step_offset: int) -> None:
        """One training step on rows ``idx`` of (X, Y) with the learning rate
        and step read on the device: the fused pass, then the weight
        gradients and Adam (one launch when use_wgrad_adam, else the grouped
        weight-gradient GEMM and the multi-tensor Adam)."""
        self.fused_pass(X, Y, idx=idx, target_ld=Y.shape[1])
        if self.use_wgrad_adam:
            self.wgrad_adam_dev(lr_ptr, step_base_ptr, step_offset)
        else:
            self.weight_grads()
            self.adam_step_dev(lr_ptr, step_base_ptr, step_offset)

    def weight_grads(self) -> None:
        """All layers' weight gradients dW_l = dZ_l^T X_l in one grouped
        split-K launch (after a training fused_pass)."""
        if self._dw is None:
            descs = []
            for l, L in enumerate(self.layers):
                n, k = self.outs[l], self.ins[l]
                Xt = self.Yt[l - 1] if l > 0 else self.x0t
                descs.append(_lib.GemmDesc(self.dZt[l].data_ptr(), Xt.data_ptr(), L.gW.data_ptr(),
                                           n, k, self.B, self.B, self.B, k))
            self._dw = (_lib.GemmDesc * len(descs))(*descs)
        splits = 8 if self.B % (64 * 8) == 0 else 1
        _lib.check(self.lib.mcl_gemm_nt_tc_grouped(C.cast(self._dw, C.c_void_p), len(self._dw), splits,
                                                   self._p(self.tc_err), self._s()), "mcl_gemm_nt_tc_grouped")

    # -- passes ---------------------------------------------------------------
    def forward(self) -> "torch.Tensor":
        if self.use_fused:
            # training: forward, loss and the input-gradient chain in one launch
            self.fused_pass(self.x_f32, self.target if self.training else None)
            return self.Z[-1][:, :DIMS[-1]]
        B = self.B
        A, lda = self.x0, IN_PAD
        for l, L in enumerate(self.layers):
            n, k = self.outs[l], self.ins[l]
            if l < len(self.layers) - 1:
                self._gemm(_lib_EPI.BIAS_GELU, B, n, k, A, lda, L.Wb, k, L.b, self.Z[l], n,
                           self.Y[l], n, self.Yt[l] if self.training else None, B)
                A, lda = self.Y[l], n
            else:
                self._gemm(_lib_EPI.BIAS, B, n, k, A, lda, L.Wb, k, L.b, self.Z[l], n)
        return self.Z[-1][:, :DIMS[-1]]

    def backward(self, want_input_grad: bool = False) -> None:
        """Gradients of the mean squared error (over batch and 200 bins).  On
        the fused path forward() already ran the loss and the input-gradient
        chain, so only the weight gradients remain (the input gradient needs
        the layer-by-layer path: set ``use_fused = False`` before forward)."""
        if self.use_fused:
            if want_input_grad:
                raise ValueError("input gradients need use_fused = False before forward()")
            self.weight_grads()
            return
        B = self.B
        self.loss.zero_()
        _lib.check(self.lib.mcl_mse_loss(B, OUT_PAD, DIMS[-1], self._p(self.Z[-1]), OUT_PAD,
                                         self._p(self.target), OUT_PAD, C.c_float(1.0 / (B * DIMS[-1])),
                                         self._p(self.dOut), OUT_PAD, self._p(self.loss), self._s()),
                   "mcl_mse_loss")
        dY, lddy = self.dOut, OUT_PAD
        for l in range(len(self.layers) - 1, -1, -1):
            L = self.layers[l]
            n, k = self.outs[l], self.ins[l]
            L.gb.zero_()
            last = l == len(self.layers) - 1
            _lib.check(self.lib.mcl_act_backward(B, n, self._p(dY), lddy, self._p(self.Z[l]), n,
                                                 0 if last else 1, self._p(self.dZ[l]), n,
                                                 self._p(self.dZt[l]), B, self._p(L.gb), self._s()),
                       "mcl_act_backward")
            Xt = self.Yt[l - 1] if l > 0 else self.x0t
            # dW[n][k] = sum_m dZ[m][n] X[m][k]
            self._gemm(_lib_EPI.F32, n, k, B, self.dZt[l], B, Xt, B, None, L.gW, k)
            if l > 0 or want_input_grad:
                # dX[m][k] = sum_n dZ[m][n] W[n][k]
                self._gemm(_lib_EPI.F32, B, k, n, self.dZ[l], n, L.Wt, n, None, self.dY[l], k)
            dY, lddy = self.dY[l], k

    def _adam_tensors(self):
        if getattr(self, "_adam_arr", None) is None:
            ts = []
            for L in self.layers:
                n, k = L.W.shape
                ts.append(_lib.AdamTensor(L.W.data_ptr(), L.gW.data_ptr(), L.mW.data_ptr(), L.vW.data_ptr(),
                                          L.Wb.data_ptr(), L.Wt.data_ptr(), n, k))
                ts.append(_lib.AdamTensor(L.b.data_ptr(), L.gb.data_ptr(), L.mb.data_ptr(), L.vb.data_ptr(),
                                          None, None, 1, n))
            self._adam_arr = (_lib.AdamTensor * len(ts))(*ts)
        return C.cast(self._adam_arr, C.c_void_p), len(self._adam_arr)

    def adam_step(self, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
        """One Adam step on every weight and bias (one launch)."""
        self.step_count += 1
        arr, n = self._adam_tensors()
        _lib.check(self.lib.mcl_adam_multi(arr, n, C.c_float(lr), C.c_float(b1), C.c_float(b2), C.c_float(eps),
                                           self.step_count, self._s()), "mcl_adam_multi")

    def adam_step_dev(self, lr_ptr: int, step_base_ptr: int, step_offset: int, b1: float = 0.9,
                      b2: float = 0.999, eps: float = 1e-8) -> None:
        """Adam with lr = *lr_ptr and step = *step_base_ptr + step_offset read
        on the device (for captured multi-step graphs)."""
        arr, n = self._adam_tensors()
        _lib.check(self.lib.mcl_adam_multi_dev(arr, n, C.c_void_p(lr_ptr), C.c_void_p(step_base_ptr), step_offset,
                                               C.c_float(b1), C.c_float(b2), C.c_float(eps), self._s()),
                   "mcl_adam_multi_dev")

    def state_dict(self) -> dict:
        """FP32 master weights and biases (host tensors), for checkpoints."""
        return {"W": [L.W.cpu() for L in self.layers], "b": [L.b.cpu() for L in self.layers],
                "step": self.step_count}

    def load_state_dict(self, st: dict) -> None:
        t = self.torch
        for L, W, b in zip(self.layers, st["W"], st["b"]):
            L.W.copy_(W.to(self.dev))
            L.b.copy_(b.to(self.dev))
            L.Wb.copy_(L.W.to(t.bfloat16))
            L.Wt.copy_(L.W.t().contiguous().to(t.bfloat16))
        self.step_count = int(st.get("step", 0))

    def inference_copy(self, batch: int) -> "SurrogateMLP":
        """A forward-only model with the same weights and a batch of ``batch``
        rows (rounded up to 128), so that large candidate sets run in one pass."""
        b = -(-int(batch) // 128) * 128
        m = SurrogateMLP(batch=b, seed=0, device=str(self.dev))
        m.load_state_dict(self.state_dict())
        m.training = False
        m.use_fused = self.use_fused
        m.fused_split = self.fused_split
        return m

    def input_grad(self) -> "torch.Tensor":
        """d loss / d standardized input (after backward(want_input_grad=True))."""
        return self.dY[0][:, :6]


class _lib_EPI:
    F32 = 0
    BIAS = 1
    BIAS_GELU = 2


def reference_forward_backward(model: SurrogateMLP, x_std: np.ndarray, y: np.ndarray):
    """The same network in float64 on the CPU (torch autograd) with the
    model's bf16-rounded weights, inputs and hidden activations: loss and
    parameter gradients.  Used by the gradient checks."""
    import torch
    t = torch
    xb = t.tensor(x_std, dtype=t.float32).to(t.bfloat16).to(t.float64)
    h = t.zeros(xb.shape[0], IN_PAD, dtype=t.float64)
    h[:, :6] = xb
    Ws, bs = [], []
    for L in model.layers:
        W = L.Wb.float().cpu().to(t.float64).requires_grad_(True)
        b = L.b.cpu().to(t.float64).requires_grad_(True)
        Ws.append(W)
        bs.append(b)
    for l in range(len(Ws)):
        z = h @ Ws[l].t() + bs[l]
        # hidden activations travel between layers in bf16, as on the GPU
        h = t.nn.functional.gelu(z).to(t.bfloat16).to(t.float64) if l < len(Ws) - 1 else z
    out = h[:, :DIMS[-1]]
    yt = t.tensor(y, dtype=t.float64)
    loss = ((out - yt) ** 2).mean()
    loss.backward()
    return float(loss.detach()), [W.grad.numpy() for W in Ws], [b.grad.numpy() for b in bs], out.detach().numpy()


# ---------------------------------------------------------------------------
# training and inference
# ---------------------------------------------------------------------------
def generate_dataset(n: int, seed: int, id0: int = 0, n_traps: int = N_TRAPS):
    """n parameter draws and their Monte Carlo curves (counts), on the GPU."""
    rng = np.random.default_rng(seed)
    params = sample_params(n, rng)
    counts = simulate_curves(params, seed=seed, id0=id0, n_traps=n_traps)
    return params, counts


def train(model: SurrogateMLP, params: np.ndarray, counts: np.ndarray, steps: int = 4000,
          lr: float = 2e-3, lr_final: float = 5e-5, seed: int = 0, log_every: int = 0,
          n_traps: int = N_TRAPS, use_graph: bool = True, graph_steps: int = 25) -> List[float]:
    """Adam on random mini-batches; cosine decay from lr to lr_final.

    One step (batch gather, forward, loss, backward, Adam) is ~25 small
    kernels, so ``graph_steps`` steps are captured once in a CUDA graph and
    replayed; Adam reads the learning rate and step count from device
    memory.  Returns the loss (mean squared error of the log curve) about
    every log_every steps."""
    t = model.torch
    X = t.tensor(standardize(params), dtype=t.float32, device=model.dev)
    Y = t.tensor(curve_to_target(counts, n_traps), dtype=t.float32, device=model.dev)
    gen = t.Generator(device=model.dev).manual_seed(seed)
    idx = t.zeros(model.B, dtype=t.int64, device=model.dev)
    lrs = [lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * k / max(steps - 1, 1)))
           for k in range(steps)]
    hist = []

    def step_on(ix):
        """One forward/backward pass on rows ``ix`` of the dataset."""
        if model.use_fused:
            # the fused kernel gathers its rows itself: no copies of the batch
            model.fused_pass(X, Y, idx=ix, target_ld=Y.shape[1])
            model.weight_grads()
            return
        model.set_inputs(X.index_select(0, ix))
        model.set_targets(Y.index_select(0, ix))
        model.forward()
        model.backward()

    def body(k):
        step_on(idx)
        model.adam_step(lr=lrs[k])

    if not use_graph:
        for k in range(steps):
            idx.copy_(t.randint(0, X.shape[0], (model.B,), generator=gen, device=model.dev))
            body(k)
            if log_every and (k % log_every == 0 or k == steps - 1):
                hist.append(float(model.loss.item()) / (model.B * DIMS[-1]))
        return hist
    # G steps per graph: batch indices for the G steps are drawn before each
    # replay, and Adam reads its learning rate and step from device memory,
    # so one capture serves the whole run.
    G = max(1, min(graph_steps, steps))
    lr_all = t.tensor(lrs, dtype=t.float32, device=model.dev)
    lr_cur = t.empty(G, dtype=t.float32, device=model.dev)
    base = t.zeros(1, dtype=t.int32, device=model.dev)
    idxs = t.zeros((G, model.B), dtype=t.int64, device=model.dev)
    s = t.cuda.Stream()
    s.wait_stream(t.cuda.current_stream())
    with t.cuda.stream(s):   # one eager forward/backward before the capture
        step_on(idxs[0])
    t.cuda.current_stream().wait_stream(s)
    g = t.cuda.CUDAGraph()
    with t.cuda.graph(g):
        for j in range(G):
            if model.use_fused:
                model.train_step_dev(X, Y, idxs[j], lr_cur[j:].data_ptr(), base.data_ptr(), j + 1)
            else:
                step_on(idxs[j])
                model.adam_step_dev(lr_cur[j:].data_ptr(), base.data_ptr(), j + 1)
    k = 0
    while k + G <= steps:
        idxs.copy_(t.randint(0, X.shape[0], (G, model.B), generator=gen, device=model.dev))
        lr_cur.copy_(lr_all[k:k + G])
        base.fill_(model.step_count)
        g.replay()
        model.step_count += G
        k += G
        if log_every and ((k - 1) // log_every != (k - 1 - G) // log_every or k == steps):
            hist.append(float(model.loss.item()) / (model.B * DIMS[-1]))
    while k < steps:          # the remainder, eagerly
        idx.copy_(t.randint(0, X.shape[0], (model.B,), generator=gen, device=model.dev))
        body(k)
        k += 1
        if log_every and (k % log_every == 0 or k == steps):
            hist.append(float(model.loss.item()) / (model.B * DIMS[-1]))
    model.check_errors()
    return hist


def flops_per_step(model: SurrogateMLP) -> float:
    """Multiply-add FLOPs of one training step: the forward GEMMs, the
    weight-gradient GEMMs and the input-gradient GEMMs of layers 1..4."""
    fwd = sum(2.0 * model.B * k * n for k, n in zip(model.ins, model.outs))
    dx = sum(2.0 * model.B * k * n for k, n in zip(model.ins[1:], model.outs[1:]))
    return 2.0 * fwd + dx


def time_training_steps(model: SurrogateMLP, params: np.ndarray, counts: np.ndarray, graph_steps: int = 25,
                        replays: int = 8, seed: int = 0, n_traps: int = N_TRAPS) -> float:
    """Device time of one training step (forward, loss, backward, Adam on a
    random mini-batch): ``graph_steps`` steps captured in one CUDA graph,
    replayed ``replays`` times between CUDA events.  Returns microseconds per
    step.  The model's weights keep training while it is timed."""
    t = model.torch
    X = t.tensor(standardize(params), dtype=t.float32, device=model.dev)
    Y = t.tensor(curve_to_target(counts, n_traps), dtype=t.float32, device=model.dev)
    gen = t.Generator(device=model.dev).manual_seed(seed)
    idxs = t.randint(0, X.shape[0], (graph_steps, model.B), generator=gen, device=model.dev)
    lr = t.full((graph_steps,), 1e-4, dtype=t.float32, device=model.dev)
    base = t.full((1,), model.step_count, dtype=t.int32, device=model.dev)

    def step(j):
        if model.use_fused:
            model.train_step_dev(X, Y, idxs[j], lr[j:].data_ptr(), base.data_ptr(), j + 1)
            return
        model.set_inputs(X.index_select(0, idxs[j]))
        model.set_targets(Y.index_select(0, idxs[j]))
        model.forward()
        model.backward()
        model.adam_step_dev(lr[j:].data_ptr(), base.data_ptr(), j + 1)

    s = t.cuda.Stream()
    s.wait_stream(t.cuda.current_stream())
    with t.cuda.stream(s):
        step(0)
    t.cuda.current_stream().wait_stream(s)
    g = t.cuda.CUDAGraph()
    with t.cuda.graph(g):
        for j in range(graph_steps):
            step(j)
    g.replay()
    e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(replays):
        g.replay()
    e1.record()
    e1.synchronize()
    model.check_errors()
    return e0.elapsed_time(e1) * 1e3 / (replays * graph_steps)


def predict(model: SurrogateMLP, params: np.ndarray) -> np.ndarray:
    """Predicted log curves [n][200] (float32, host)."""
    t = model.torch
    X = t.tensor(standardize(params), dtype=t.float32, device=model.dev)
    n = X.shape[0]
    out = np.zeros((n, DIMS[-1]), dtype=np.float32)
    for c0 in range(0, n, model.B):
        xb = X[c0:c0 + model.B]
        m = xb.shape[0]
        if m < model.B:
            xb = t.cat([xb, t.zeros(model.B - m, 6, device=model.dev)])
        model.set_inputs(xb)
        out[c0:c0 + m] = model.forward()[:m].float().cpu().numpy()
    return out


_DEV_CONST = {}


def dev_const(name: str, values, dtype, device):
    """A small constant array on the device, uploaded once (a fresh upload from
    pageable host memory would stall the stream on every call)."""
    import torch
    key = (name, dtype, str(device))
    t = _DEV_CONST.get(key)
    if t is None:
        t = torch.tensor(values, dtype=dtype, device=device)
        _DEV_CONST[key] = t
    return t


def standardize_t(p):
    """Device version of ``standardize`` (torch tensor [n][6])."""
    lo = dev_const("LOW", LOW, p.dtype, p.device)
    hi = dev_const("HIGH", HIGH, p.dtype, p.device)
    return 2.0 * (p - lo) / (hi - lo) - 1.0


def predict_t(model: SurrogateMLP, params_t) -> "torch.Tensor":
    """Predicted log curves for a device tensor of parameters [n][6] (float32
    device tensor [n][200]); no host round trip."""
    t = model.torch
    X = standardize_t(params_t.float())
    n = X.shape[0]
    out = t.empty(n, DIMS[-1], dtype=t.float32, device=model.dev)
    for c0 in range(0, n, model.B):
        xb = X[c0:c0 + model.B]
        m = xb.shape[0]
        if m < model.B:
            xb = t.cat([xb, t.zeros(model.B - m, 6, device=model.dev)])
        model.set_inputs(xb)
        out[c0:c0 + m] = model.forward()[:m]
    return out


