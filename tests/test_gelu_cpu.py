"""The fused surrogate kernel's GELU: erf from Abramowitz & Stegun,
Handbook of Mathematical Functions, formula 7.1.26 (published bound
|error| <= 1.5e-7), evaluated in float32 as the kernel evaluates it, against
the exact erf.  The GPU tests compare the fused kernel with the layer-by-layer
kernels, which call CUDA's erff."""
import math

import numpy as np

A = np.float32([0.254829592, -0.284496736, 1.421413741, -1.453152027, 1.061405429])
P = np.float32(0.3275911 * 0.70710678118654752)


def gelu_and_grad(z):
    z = z.astype(np.float32)
    t = np.float32(1.0) / (P * np.abs(z) + np.float32(1.0))
    e = np.exp(np.float32(-0.5) * z * z)
    poly = ((((A[4] * t + A[3]) * t + A[2]) * t + A[1]) * t + A[0]) * t
    h = np.float32(0.5) * poly * e
    cdf = np.where(z < 0, h, np.float32(1.0) - h)
    return z * cdf, cdf + z * (np.float32(0.39894228040143268) * e)


def test_gelu_error_bound():
    z = np.linspace(-10, 10, 200001).astype(np.float32)
    y, g = gelu_and_grad(z)
    zd = z.astype(np.float64)
    cdf = np.array([0.5 * math.erfc(-v / math.sqrt(2.0)) for v in zd])
    pdf = np.exp(-0.5 * zd * zd) / math.sqrt(2 * math.pi)
    # the normal CDF to 1e-6 absolute (formula bound 7.5e-8 plus float32 rounding)
    assert np.max(np.abs(y - zd * cdf) / np.maximum(np.abs(zd), 1.0)) < 1e-6
    assert np.max(np.abs(g - (cdf + zd * pdf))) < 1e-6
    # the lower tail keeps its sign and order of magnitude (no cancellation)
    assert np.all(y[z < -1] <= 0) and np.all(np.abs(y[z < -3] - zd[z < -3] * cdf[z < -3]) < 1e-6)
