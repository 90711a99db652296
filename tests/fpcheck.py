"""Floating-point parity rule for the GPU tests.

The GPU sums in a different order than the sequential reference, so FP32
results cannot be bit-identical.  The rule: against the FP64 oracle, the GPU
must be at least as accurate as the reference's own FP32 arithmetic (the
oracle, which is bit-exact with the reference's compiled code), within a
factor of 4, plus a floor of 2 FP32 ulps of the largest value:

    |gpu - f64|_inf <= 4 |ref32 - f64|_inf + 2^-22 max|f64|
    |gpu - f64|_1   <= 4 |ref32 - f64|_1   + 2^-22 |f64|_1
"""
import numpy as np

FACTOR = 4.0
FLOOR = 2.0 ** -22


def assert_fp_as_accurate(gpu, ref32, ref64, what=""):
    g = np.asarray(gpu, np.float64)
    r = np.asarray(ref32, np.float64)
    x = np.asarray(ref64, np.float64)
    scale_inf = float(np.abs(x).max()) if x.size else 0.0
    scale_1 = float(np.abs(x).sum())
    ginf, rinf = float(np.abs(g - x).max(initial=0.0)), float(np.abs(r - x).max(initial=0.0))
    g1, r1 = float(np.abs(g - x).sum()), float(np.abs(r - x).sum())
    assert ginf <= FACTOR * rinf + FLOOR * scale_inf, f"{what}: L-inf {ginf:.3e} vs reference {rinf:.3e}"
    assert g1 <= FACTOR * r1 + FLOOR * scale_1, f"{what}: L1 {g1:.3e} vs reference {r1:.3e}"
