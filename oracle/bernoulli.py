"""FP64 CPU restatement of the fixed-dt Bernoulli trap kinetics (the oracle).

Test infrastructure only; the GPU library never imports it.

The reference has no fixed-dt kernel: its event-driven loop
(src/class/simulate.py:51-92) draws one exponential wait per electron per
event.  In the dilute limit (many more recombination centres than electrons,
small dt) that loop is a set of independent electrons, each escaping in a step
of length dt with probability

    p = 1 - exp(-dt * A(T) * w),   w = exp(-alpha * r'),
    A(T) = s * exp(-E / (k_b * T))  [+ an optical or ground-state rate]

where r' is the electron's dimensionless distance to its nearest centre,
distributed as 3 r'^2 exp(-r'^3) (inverse CDF r' = (-ln(1-U))^(1/3)).  This is
the tunnelling rate of src/class/engine.py:69-73 with b = s, E_loc = E and the
conduction-band channel off, and alpha*d = rho'^(-1/3) * r' (the box geometry
of src/class/tl_trap_lab.py:33-35 makes alpha*d exactly that for a Poisson
field of centres).  Trap filling at dose rate D fills an empty trap in a step
with probability 1 - exp(-dt * D / D0) (the per-trap form of
src/class/tl_trap_lab.py:53-60), giving the saturating occupancy
1 - exp(-D t / D0).

A set is a schedule of segments (TL ramp, isothermal hold, irradiation,
fading, optical stimulation).  Recombinations are counted into bins; the
number of filled traps at the end of each bin is reported too.

Uniform streams
---------------
Philox counters restart their step blocks at every segment, so that a segment's
first step always opens a fresh block: with ``P_g`` the blocks used by earlier
segments, local step j of segment g of slot e draws from

``layout="f64"``      Philox4x32-10, two 53-bit doubles per call: words
                      (2(j&1), 2(j&1)+1) of philox(P_g + (j>>1), e, set_id,
                      TAG_STEP), P_g = sum of ceil(n_steps/2); FP64 mode.
``layout="f32"``      Philox4x32-10, eight steps per call: step j takes the
                      16-bit field h of word t&3 of
                      philox(P_g + (j>>3), e, set_id, TAG_STEP), t = j&7,
                      P_g = sum of ceil(n_steps/8): the word's upper half
                      for t < 4, its lower half for t >= 4.  The uniform is
                      u32 = (h << 16) | lo16 with lo16 the low 16 bits of word
                      0 of philox(k, e, set_id, TAG_LOW) (k = the set's global
                      step); an event happens iff u32 < p * 2^32.  The
                      kernel's FP32 mode draws the same integers, so its fates
                      agree with this FP64 evaluation except where p itself
                      differs in the last float bit (expected flips ~1e-6 per
                      event).
``layout="injected"`` doubles from an array: slot e's r' uniform at
                      ``u[e]``, step k's at ``u[n_slots + k*n_slots + e]``.
``layout="numpy"``    numpy's PCG64 generator (used only to time the CPU
                      baseline; not comparable draw by draw).
"""
from __future__ import annotations

import numpy as np

from .philox import TAG_INIT, TAG_LOW, TAG_REFILL, TAG_STEP, philox4x32, seed_key, u53

K_B = 8.617333262145e-5


def segment_constants(st: dict, seg: dict):
    """Per-step hazard scale c_j = dt_j * A_j and fill probability q_j (FP64)."""
    n = int(seg["n_steps"])
    j = np.arange(n, dtype=np.float64)
    dt = float(seg["dt"])
    g = float(seg.get("dt_growth", 1.0))
    if g == 1.0:
        dts = np.full(n, dt)
        t = dt * j
    else:
        gj = np.power(g, j)
        dts = dt * gj
        t = dt * (gj - 1.0) / (g - 1.0)
    T = float(seg.get("T0", 273.15)) + float(seg.get("beta", 0.0)) * t
    A = np.full(n, float(seg.get("rate_const", 0.0)))
    if seg.get("thermal", True):
        A = A + float(st["s"]) * np.exp(-float(st["E"]) / (float(st.get("k_b", K_B)) * T))
    c = dts * A
    fr = float(seg.get("fill_rate", 0.0))
    q = -np.expm1(-dts * fr) if fr > 0 else np.zeros(n)
    return c, q


def _r_prime(u):
    return np.cbrt(-np.log1p(-u))


class _Draws:
    """Uniforms of one set, step by step, in the chosen layout."""

    def __init__(self, st, layout, seed, uniforms):
        self.n = int(st["n_slots"])
        self.sid = int(st.get("set_id", 0))
        self.layout = layout
        self.key = seed_key(seed)
        self.u = uniforms
        self.e = np.arange(self.n, dtype=np.uint64)
        self._blk = None
        self._blk_id = -1
        if layout == "numpy":
            self.gen = np.random.default_rng(seed + self.sid)

    def init(self):
        if self.layout == "f64":
            w = philox4x32(0, self.e, self.sid, TAG_INIT, *self.key)
            return u53(w[0], w[1])
        if self.layout == "f32":
            w = philox4x32(0, self.e, self.sid, TAG_INIT, *self.key)
            return (w[0] >> np.uint64(8)).astype(np.float64) * 2.0 ** -24
        if self.layout == "injected":
            return np.asarray(self.u[:self.n], dtype=np.float64)
        return self.gen.random(self.n)

    def refill(self, k, idx):
        """r' uniforms for slots ``idx`` refilled at step k."""
        if self.layout == "f64":
            w = philox4x32(k, idx.astype(np.uint64), self.sid, TAG_REFILL, *self.key)
            return u53(w[0], w[1])
        if self.layout == "f32":
            w = philox4x32(k, idx.astype(np.uint64), self.sid, TAG_REFILL, *self.key)
            return (w[0] >> np.uint64(8)).astype(np.float64) * 2.0 ** -24
        if self.layout == "injected":
            raise ValueError("the injected layout has no refill draws")
        return self.gen.random(idx.size)

    def block_span(self, n_steps):
        """Philox blocks a segment of n_steps consumes in this layout."""
        if self.layout == "f64":
            return (n_steps + 1) // 2
        if self.layout == "f32":
            return (n_steps + 7) // 8
        return 0

    def step(self, base, j, k, thr=None):
        """Uniforms of local step j (global step k) of the segment whose
        Philox blocks start at ``base``, as doubles.  In the f32 layout the
        low 16 bits are drawn only where the high field lies below the
        per-slot threshold ``thr`` (elsewhere u = h / 2^16 already decides)."""
        if self.layout == "f64":
            b = base + (j >> 1)
            if b != self._blk_id:
                self._blk = philox4x32(b, self.e, self.sid, TAG_STEP, *self.key)
                self._blk_id = b
            h = 2 * (j & 1)
            return u53(self._blk[h], self._blk[h + 1])
        if self.layout == "f32":
            b = base + (j >> 3)
            if b != self._blk_id:
                self._blk = philox4x32(b, self.e, self.sid, TAG_STEP, *self.key)
                self._blk_id = b
            t = j & 7
            word = self._blk[t & 3]
            h = (word >> np.uint64(16)) if t < 4 else (word & np.uint64(0xFFFF))
            u = h.astype(np.float64) * 2.0 ** -16
            cand = np.nonzero(u < thr)[0]
            if cand.size:
                lo = philox4x32(k, cand.astype(np.uint64), self.sid, TAG_LOW, *self.key)[0]
                u32 = (h[cand] << np.uint64(16)) | (lo & np.uint64(0xFFFF))
                u[cand] = u32.astype(np.float64) * 2.0 ** -32
            return u
        if self.layout == "injected":
            o = self.n + k * self.n
            return np.asarray(self.u[o:o + self.n], dtype=np.float64)
        return self.gen.random(self.n)


def run_set(st: dict, *, layout: str = "f64", seed: int = 0, uniforms=None,
            want_fates: bool = False):
    """Simulate one set; returns ``(lum, alive, fates)``.

    ``lum[b]``   recombinations counted in bin b (int64)
    ``alive[b]`` filled traps after the last step of bin b (int64)
    ``fates``    per slot, the global step of its last recombination or -1
                 (only if ``want_fates``)
    """
    n = int(st["n_slots"])
    n_bins = int(st["n_bins"])
    alpha = float(st["alpha"])
    dr = _Draws(st, layout, seed, uniforms)
    filled = np.arange(n) < int(st["n_filled"])
    w = np.exp(-alpha * _r_prime(dr.init()))
    lum = np.zeros(n_bins, dtype=np.int64)
    alive = np.zeros(n_bins, dtype=np.int64)
    fates = np.full(n, -1, dtype=np.int64)
    k = 0
    base = 0
    for seg in st["segments"]:
        c, q = segment_constants(st, seg)
        spb = int(seg["steps_per_bin"])
        b0 = int(seg["bin_offset"])
        fill_on = float(seg.get("fill_rate", 0.0)) > 0
        for j in range(int(seg["n_steps"])):
            p = -np.expm1(-c[j] * w)
            u = dr.step(base, j, k, np.where(filled, p, q[j]) if layout == "f32" else None)
            rec = filled & (u < p)
            b = b0 + j // spb
            nrec = int(np.count_nonzero(rec))
            if nrec:
                lum[b] += nrec
                if want_fates:
                    fates[rec] = k
            if fill_on:
                fil = (~filled) & (u < q[j])
                idx = np.nonzero(fil)[0]
                if idx.size:
                    w[idx] = np.exp(-alpha * _r_prime(dr.refill(k, idx)))
                filled = (filled & ~rec) | fil
            elif nrec:
                filled = filled & ~rec
            if (j + 1) % spb == 0 or j + 1 == int(seg["n_steps"]):
                alive[b] = int(np.count_nonzero(filled))
            k += 1
        base += dr.block_span(int(seg["n_steps"]))
    return lum, alive, (fates if want_fates else None)


def total_steps(st: dict) -> int:
    return int(sum(int(s["n_steps"]) for s in st["segments"]))


def injected_size(st: dict) -> int:
    """Length of the injected uniform block of one set."""
    return int(st["n_slots"]) * (1 + total_steps(st))


def expected_curves(st: dict, n_u: int = 200000):
    """Expected recombinations per bin and expected filled traps at each bin
    end (FP64, no sampling); returns ``(lum, alive)``.

    Every trap is an independent two-state chain (filled with some w, or
    empty), so expectations obey a linear recursion.  The w of a filled trap
    is carried on a quadrature grid: w_i = exp(-alpha r'(u_i)) at the
    midpoints u_i of n_u equal cells of the inverse-CDF variable, each node
    holding the expected number of filled traps with that w.  In a segment
    without filling a filled trap survives to local step k with probability
    exp(-w sum_{j<k} c_j), so each bin's expected escapes follow in closed
    form; in a filling segment the chain is stepped: per step a filled trap
    escapes with p_j(w) = 1 - exp(-c_j w) and an empty one refills with q_j,
    drawing a fresh w from the same distribution (equal weight per node).  A
    trap that escapes in a step is not refilled in it, as in ``run_set``."""
    u = (np.arange(n_u) + 0.5) / n_u
    w = np.exp(-float(st["alpha"]) * _r_prime(u))
    n = int(st["n_slots"])
    n_filled = int(st["n_filled"])
    f = np.full(n_u, n_filled / n_u)      # expected filled traps per node
    e = float(n - n_filled)               # expected empty traps
    n_bins = int(st["n_bins"])
    lum = np.zeros(n_bins)
    alive = np.zeros(n_bins)
    for seg in st["segments"]:
        c, q = segment_constants(st, seg)
        spb = int(seg["steps_per_bin"])
        b0 = int(seg["bin_offset"])
        ns = int(seg["n_steps"])
        if ns == 0:
            continue
        if float(seg.get("fill_rate", 0.0)) > 0:
            for j in range(ns):
                esc = f * -np.expm1(-c[j] * w)
                E = float(esc.sum())
                refill = e * q[j]
                f = f - esc + refill / n_u
                e = e - refill + E
                lum[b0 + j // spb] += E
                if (j + 1) % spb == 0 or j + 1 == ns:
                    alive[b0 + j // spb] = float(f.sum())
            continue
        cum = np.cumsum(c)
        C_prev = 0.0
        S_prev = np.ones_like(w)
        for b in range((ns + spb - 1) // spb):
            C = cum[min((b + 1) * spb, ns) - 1]
            # S_prev - S without cancellation: S_prev * (1 - exp(-w (C - C_prev)))
            d = S_prev * -np.expm1(-w * (C - C_prev))
            lum[b0 + b] = float(np.dot(f, d))
            S_prev = S_prev - d
            C_prev = C
            alive[b0 + b] = float(np.dot(f, S_prev))
        e += float(np.dot(f, 1.0 - S_prev))
        f = f * S_prev
    return lum, alive


def expected_lum(st: dict, n_u: int = 200000) -> np.ndarray:
    """Expected recombinations per bin (``expected_curves``' first output)."""
    return expected_curves(st, n_u)[0]
