"""Philox4x32-10 counter-based generator in vectorised numpy (the oracle's copy).

Restated from the published algorithm: J. K. Salmon, M. A. Moraes, R. O. Dror,
D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11 (the Random123
paper).  Ten rounds of ``(c0, c1, c2, c3) -> (hi(M1*c2)^c1^k0, lo(M1*c2),
hi(M0*c0)^c3^k1, lo(M0*c0))`` with the key bumped by the Weyl constants between
rounds.  ``tests/test_philox.py`` checks it against the paper's known-answer
vectors; the CUDA kernels implement the same function.

Test infrastructure only.
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint64(0x9E3779B9)
W1 = np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
S32 = np.uint64(32)

# counter word 3: which draw of an electron slot this is
TAG_STEP = 0      # per-step Bernoulli uniforms
TAG_INIT = 1      # initial nearest-centre distance r'
TAG_REFILL = 2    # r' of a trap refilled at a given step
TAG_LOW = 3       # low 16 bits of an FP32-layout uniform


def philox4x32(c0, c1, c2, c3, k0, k1, rounds: int = 10):
    """Return the four 32-bit output words (uint64 arrays holding uint32)."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) & MASK for x in (c0, c1, c2, c3))
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    c0, c1, c2, c3 = (np.array(x) for x in (c0, c1, c2, c3))
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    for r in range(rounds):
        if r:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = c0 * M0
        p1 = c2 * M1
        c0, c1, c2, c3 = ((p1 >> S32) ^ c1 ^ k0, p1 & MASK,
                          (p0 >> S32) ^ c3 ^ k1, p0 & MASK)
    return c0, c1, c2, c3


def seed_key(seed: int):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return seed & 0xFFFFFFFF, seed >> 32


def u53(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """53-bit double in [0, 1) from two words: ((a>>5)*2^26 + (b>>6)) / 2^53."""
    a = np.asarray(a, dtype=np.uint64) >> np.uint64(5)
    b = np.asarray(b, dtype=np.uint64) >> np.uint64(6)
    return (a.astype(np.float64) * 67108864.0 + b.astype(np.float64)) / 9007199254740992.0
