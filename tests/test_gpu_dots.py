"""The mixed mode's dot products (FP32 vectors, a double-float sum per
thread on the FP32 pipe, FP64 across threads) against FP64 accumulation and
against the exact value, on vectors of the sigma = 2.0 system.

Every FP32 x FP32 product is exact in FP64 and math.fsum sums exactly, so
the exact dot is known. The bound: the double-float per-thread sums keep
about 44 bits, so the error is within 1e-12 of sum |x_i y_i| (the FP64
per-thread accumulation of the same vectors is held to the same bound)."""
import math

import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import generate

pytestmark = pytest.mark.gpu


def exact_dot(x, y):
    return math.fsum((x.astype(np.float64) * y.astype(np.float64)).tolist())


def test_double_float_dots_match_fp64(built_lib):
    s = generate(60, 60, 20, sigma=2.0, inactive_frac=0.05, fault_frac=0.01, seed=11)
    rng = np.random.default_rng(5)
    A = s.to_scipy()
    b = s.b
    Ab = A @ b
    cases = {
        "(b, b)": (b, b),                       # a residual norm
        "(Ab, b)": (Ab, b),                     # rho-like
        "(Ab, Ab)": (Ab, Ab),                   # (t, t)
        # magnitudes over 12 decades with cancellation: the hard case
        "wide": (rng.standard_normal(s.n) * 10.0 ** rng.uniform(-6, 6, s.n),
                 rng.standard_normal(s.n)),
        "cancel": (np.concatenate([b[: s.n // 2], -b[: s.n // 2]]),
                   np.concatenate([Ab[: s.n // 2], Ab[: s.n // 2]])),
    }
    with GbIlu(device=0, precision="mixed") as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        for name, (x, y) in cases.items():
            x32, y32 = np.float32(x), np.float32(y)
            df, d64 = g.dot_check(x32, y32)
            ex = exact_dot(x32, y32)
            scale = math.fsum(np.abs(x32.astype(np.float64) * y32.astype(np.float64)).tolist())
            print(f"{name}: double-float err {abs(df - ex) / scale:.2e}, "
                  f"FP64 err {abs(d64 - ex) / scale:.2e} (relative to sum |x y|)")
            assert abs(df - ex) <= 1e-12 * scale, name
            assert abs(d64 - ex) <= 1e-12 * scale, name
            assert abs(df - d64) <= 2e-12 * scale, name
