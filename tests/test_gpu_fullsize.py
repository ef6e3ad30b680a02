"""The 2M-cell system (200x200x50, sigma 1.5, 5 % inactive cells, 1 % fault
connections) through the mixed form and the adjoint, checked by properties
that do not depend on the size: the true FP64 residuals of the forward and
transposed solves (scipy's BSR product, independent of the library), the
gradient dL/dA = -lambda_i x_j^T block by block, and agreement of the mixed
results with the FP64 form's.
"""
import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import CONFIGS, adjoint_selection, make_config

pytestmark = pytest.mark.gpu

NAME = "c5_200x200x50_mixed_adjoint"


@pytest.fixture(scope="module")
def system(built_lib):
    s = make_config(NAME)
    return s, s.to_scipy()


def test_2m_cells_mixed_forward_and_adjoint(system):
    s, A = system
    tol = CONFIGS[NAME]["tol"]
    maxit = CONFIGS[NAME]["maxit"]
    cells, d = adjoint_selection(s.nb)
    idx = (3 * cells[:, None] + np.arange(3)).reshape(-1)
    out = {}
    for prec in ("mixed", "fp64"):
        with GbIlu(device=0, precision=prec) as g:
            g.analyze(s.rowptr, s.colind).factor(s.vals)
            x, r = g.solve(s.b, tol=tol, maxit=maxit)
            assert r.status == 0
            assert np.linalg.norm(s.b - A @ x) <= tol * np.linalg.norm(s.b) * (1 + 1e-6)
            gv = np.zeros(s.n)
            gv[idx] = x[idx] - d
            lam, dA, ra = g.adjoint(gv, x, tol=tol, maxit=maxit)
            assert ra.status == 0
            assert np.linalg.norm(A.T @ lam - gv) <= tol * np.linalg.norm(gv) * (1 + 1e-6)
            # dL/dA on the pattern, in the input block order: -lambda_i x_j^T
            rows = np.repeat(np.arange(s.nb), np.diff(s.rowptr))
            pick = np.random.default_rng(0).choice(s.nnzb, 20000, replace=False)
            li = lam.reshape(-1, 3)[rows[pick]]
            xj = x.reshape(-1, 3)[s.colind[pick]]
            ref = -(li[:, :, None] * xj[:, None, :]).reshape(-1, 9)
            got = dA.reshape(-1, 9)[pick]
            assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()
            out[prec] = (x, lam)
    # the mixed form's results against the FP64 form's (both to 1e-8)
    for k in range(2):
        a, b = out["mixed"][k], out["fp64"][k]
        assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
