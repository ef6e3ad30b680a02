"""Failure detection of the device waits, without a GPU fault: a grid barrier
that one CTA never reaches and a data-ordered load whose value never
arrives both run out after their poll limit, report TIMEOUT with the kind
of wait in bar_fail, and leave the context usable (a solve right after
succeeds)."""
import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import generate

pytestmark = pytest.mark.gpu

TIMEOUT = 5


@pytest.mark.parametrize("mode,kind", [(0, 1), (1, 3)])
def test_wait_runs_out(built_lib, mode, kind):
    s = generate(12, 10, 5, sigma=1.5, inactive_frac=0.05, fault_frac=0.02, seed=3)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        r = g.wait_probe(mode)
        assert r["bar_fail"] == kind and r["status"] == TIMEOUT
        assert 1.0 < r["ms"] < 20000.0
        x, res = g.solve(s.b, tol=1e-8, maxit=500)
        assert res.status == 0
        assert np.linalg.norm(s.b - s.to_scipy() @ x) <= 1e-8 * np.linalg.norm(s.b) * (1 + 1e-6)
