"""Edge systems through the CUDA path, against the CPU oracle: one block row,
a block-diagonal matrix (one color: the apply is a single D^-1 step), a 1-D
chain (two colors: no small color steps), and a system whose couplings all
reach the last block row (one row of the highest color). Each in FP64 and
mixed precision, forward solve, adjoint and the two operators.
"""
import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import BlockSystem, generate
from oracle_lib import Prepared

pytestmark = pytest.mark.gpu

KERNEL_TOL = 1e-12


def block_diagonal(nb, seed=0):
    """nb uncoupled, diagonally dominant 3x3 blocks."""
    rng = np.random.default_rng(seed)
    vals = rng.standard_normal((nb, 3, 3)) + 6.0 * np.eye(3)
    return BlockSystem(nb=nb, rowptr=np.arange(nb + 1, dtype=np.int32),
                       colind=np.arange(nb, dtype=np.int32), vals=vals,
                       b=rng.standard_normal(3 * nb), cell_of_row=np.arange(nb),
                       grid=(nb, 1, 1))


def star(nb, seed=0):
    """Block row nb-1 coupled to every other row (symmetric pattern): greedy
    coloring gives the others color 0 and the hub color 1."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(nb - 1):
        rows.append([i, nb - 1])
    rows.append(list(range(nb)))
    rowptr = np.zeros(nb + 1, np.int32)
    rowptr[1:] = np.cumsum([len(r) for r in rows])
    colind = np.concatenate(rows).astype(np.int32)
    vals = 0.1 * rng.standard_normal((len(colind), 3, 3))
    for i in range(nb):
        k = rowptr[i] + rows[i].index(i)
        vals[k] += (4.0 + 0.5 * len(rows[i])) * np.eye(3)
    return BlockSystem(nb=nb, rowptr=rowptr, colind=colind, vals=vals,
                       b=rng.standard_normal(3 * nb), cell_of_row=np.arange(nb), grid=(nb, 1, 1))


def dense(nb, seed=0):
    """Every block row coupled to every other: greedy coloring gives nb colors
    (more than the single-launch apply takes: one launch per color step)."""
    rng = np.random.default_rng(seed)
    rowptr = (np.arange(nb + 1) * nb).astype(np.int32)
    colind = np.tile(np.arange(nb, dtype=np.int32), nb)
    vals = 0.05 * rng.standard_normal((nb * nb, 3, 3))
    for i in range(nb):
        vals[i * nb + i] += (2.0 + 0.1 * nb) * np.eye(3)
    return BlockSystem(nb=nb, rowptr=rowptr, colind=colind, vals=vals,
                       b=rng.standard_normal(3 * nb), cell_of_row=np.arange(nb), grid=(nb, 1, 1))


def random_pattern(nb, p, seed):
    """A random symmetric pattern (density p) with diagonally dominant random
    blocks: color counts from a few to dozens."""
    rng = np.random.default_rng(seed)
    m = rng.random((nb, nb)) < p
    m = m | m.T | np.eye(nb, dtype=bool)
    rows, cols = np.nonzero(m)
    rowptr = np.zeros(nb + 1, np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    vals = 0.1 * rng.standard_normal((len(cols), 3, 3))
    deg = np.diff(rowptr)
    for i in range(nb):
        k = rowptr[i] + int(np.searchsorted(cols[rowptr[i]:rowptr[i + 1]], i))
        vals[k] += (1.0 + 0.5 * deg[i]) * np.eye(3)
    return BlockSystem(nb=nb, rowptr=rowptr, colind=cols.astype(np.int32), vals=vals,
                       b=rng.standard_normal(3 * nb), cell_of_row=np.arange(nb), grid=(nb, 1, 1))


CASES = {
    "one_row": lambda: generate(1, 1, 1, seed=0),
    "random_sparse": lambda: random_pattern(400, 0.01, seed=5),
    "random_mid": lambda: random_pattern(300, 0.08, seed=6),
    "dense_50_colors": lambda: dense(50, seed=4),
    "block_diagonal": lambda: block_diagonal(50, seed=1),
    "chain": lambda: generate(40, 1, 1, sigma=1.0, seed=2),
    "star": lambda: star(33, seed=3),
}


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", params=sorted(CASES))
def edge(request, built_lib):
    s = CASES[request.param]()
    return s, Prepared(s)


@pytest.mark.parametrize("transpose", [False, True])
def test_operators(edge, transpose):
    s, P = edge
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x = np.random.default_rng(4).standard_normal(s.n)
        assert rel(g.spmv(x, transpose), P.spmv(x, transpose)) < KERNEL_TOL
        assert rel(g.ilu_apply(x, transpose), P.ilu_apply(x, transpose)) < KERNEL_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_and_adjoint(edge, precision):
    s, P = edge
    tol = 1e-10
    x_ref, r_ref = P.solve(s.b, tol=tol, maxit=500)
    with GbIlu(device=0, precision=precision) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = g.solve(s.b, tol=tol, maxit=500)
        assert r.status == 0
        if precision == "fp64":
            assert r.half_iters == r_ref.half_iters
        A = s.to_scipy()
        assert np.linalg.norm(s.b - A @ x) <= tol * np.linalg.norm(s.b) * (1 + 1e-6)
        assert rel(x, x_ref) < 1e-6
        gv = np.random.default_rng(5).standard_normal(s.n)
        lam, dA, ra = g.adjoint(gv, x, tol=tol, maxit=500)
        assert ra.status == 0
        assert np.linalg.norm(A.T @ lam - gv) <= tol * np.linalg.norm(gv) * (1 + 1e-6)
        assert np.abs(dA - P.grad_a(lam, x)).max() <= 1e-14 * max(np.abs(dA).max(), 1e-300)


@pytest.mark.parametrize("transpose", [False, True])
def test_apply_input_with_sentinel_bits(built_lib, transpose):
    """The small color steps are ordered by their data: their outputs start
    as a NaN sentinel that consumers wait on. An input vector that carries
    that bit pattern is data like any other (input reads are never waited
    on): the apply returns at once with the oracle's NaN pattern."""
    import time
    s = generate(30, 24, 12, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=7)
    P = Prepared(s)
    p = np.random.default_rng(8).standard_normal(s.n)
    bits = p.view(np.uint64)
    bits[[5, 600, s.n - 4]] = np.uint64(0x7ff4a5a5a5a5a5a5)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        t0 = time.perf_counter()
        z = g.ilu_apply(p, transpose)
        assert time.perf_counter() - t0 < 1.0
    z_ref = P.ilu_apply(p, transpose)
    nan = np.isnan(z_ref)
    assert nan.any() and np.array_equal(np.isnan(z), nan)
    assert rel(z[~nan], z_ref[~nan]) < KERNEL_TOL
