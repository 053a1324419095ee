"""The float-float summation of the true residual (k_residp_ff in
andromeda_gb300/csrc/agb_lsqr.cu), restated operation by operation in NumPy
FP32 arithmetic (every operation rounds to nearest, as the kernel's _rn
intrinsics do), against the exactly rounded sum of the same products.

A lane sums products g * x with x = xh + xl split into FP32 parts: every
g * xh is split exactly into the rounded product p and its error pe (the FMA
of the kernel; here g * xh in FP64 is exact for FP32 operands), the p are
summed by TwoSum into (s, er), the pe and the g * xl into a third FP32 sum lo,
and the three move into FP64 every 256 terms.  The error bound the kernel
states is n^2 u^2 / 2 of sum |g x| for n = 256 terms (2^-33); the plain FP32
sum of the same products is ~1e-7 of it.  No GPU needed.
"""
import math

import numpy as np

F = np.float32
TERMS = 256  # kFFTerms of the kernel


def _ff_sum(g, xh, xl):
    """Float-float sums of g[r, j] * (xh[r, j] + xl[r, j]) over j, rows r in parallel."""
    rows, n = g.shape
    acc = np.zeros(rows)
    s = np.zeros(rows, F)
    er = np.zeros(rows, F)
    lo = np.zeros(rows, F)
    for j in range(n):
        gj, hj, lj = g[:, j], xh[:, j], xl[:, j]
        p = (gj * hj).astype(F)  # rounded product
        pe = (gj.astype(np.float64) * hj - p.astype(np.float64)).astype(F)  # its exact error
        t = (s + p).astype(F)  # TwoSum (Knuth)
        bp = (t - s).astype(F)
        e = ((s - (t - bp).astype(F)).astype(F) + (p - bp).astype(F)).astype(F)
        s = t
        er = (er + e).astype(F)
        lo = (gj.astype(np.float64) * lj + (lo + pe).astype(F)).astype(F)  # fma(g, xl, lo + pe)
        if (j + 1) % TERMS == 0 or j == n - 1:
            acc += s.astype(np.float64) + (er.astype(np.float64) + lo.astype(np.float64))
            s[:] = 0
            er[:] = 0
            lo[:] = 0
    return acc


def test_float_float_sum_within_bound_and_far_below_fp32():
    rng = np.random.default_rng(7)
    rows, n = 48, 2048
    # entries of mixed sign and a spread of magnitudes, as in a single-layer row
    g = (rng.standard_normal((rows, n)) * np.exp(rng.uniform(-4, 0, (rows, n)))).astype(F)
    x = rng.standard_normal((rows, n)) * np.exp(rng.uniform(-2, 2, (rows, n)))
    xh = x.astype(F)
    xl = (x - xh.astype(np.float64)).astype(F)
    got = _ff_sum(g, xh, xl)
    plain = np.zeros(rows, F)
    for j in range(n):
        plain = (plain + (g[:, j] * xh[:, j]).astype(F)).astype(F)
    u = 2.0 ** -24
    bound = TERMS ** 2 * u * u / 2
    worst_ff, worst_plain = 0.0, 0.0
    for r in range(rows):
        gd = g[r].astype(np.float64)
        # every g * xh and g * xl is exact in FP64: fsum gives the correctly rounded total
        exact = math.fsum(list(gd * xh[r].astype(np.float64)) + list(gd * xl[r].astype(np.float64)))
        scale = float(np.sum(np.abs(gd * (xh[r].astype(np.float64) + xl[r]))))
        worst_ff = max(worst_ff, abs(got[r] - exact) / scale)
        worst_plain = max(worst_plain, abs(float(plain[r]) - exact) / scale)
    print("float-float", worst_ff, "plain FP32", worst_plain, "bound", bound)
    assert worst_ff <= bound
    assert worst_ff < 2.0 ** -40  # typical rounding stays far below the worst case
    assert worst_plain > 1e4 * worst_ff
