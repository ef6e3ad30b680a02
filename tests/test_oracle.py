"""The CPU oracle against independent references (CPU only).

The reference tree holds no golden vectors or solver tests, so the oracle is
pinned by identities that do not depend on it: the coloring is valid, L*U
equals A on the pattern, the preconditioner apply equals a sparse direct
solve with the same factors, the solution of a small system equals a dense
solve, and the committed golden fixtures (tests/golden/) reproduce bit for
bit.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fpga_gb300.synth import generate, make_config
from oracle_lib import Prepared

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SMALL = {
    "c1": lambda: make_config("c1_20x20x10"),
    "faults": lambda: generate(16, 14, 6, sigma=1.5, inactive_frac=0.05, fault_frac=0.02, seed=9),
}


@pytest.fixture(scope="module", params=sorted(SMALL))
def prep(request):
    return Prepared(SMALL[request.param]())


def lu_matrices(P):
    nb, rp, ci = P.nb, P.rowptr, P.colind
    lu = P.lu.reshape(-1, 3, 3)
    rows = np.repeat(np.arange(nb), np.diff(rp))
    Lb = np.where((ci < rows)[:, None, None], lu, 0)
    Ub = np.where((ci >= rows)[:, None, None], lu, 0)
    L = sp.bsr_matrix((Lb, ci, rp), shape=(3 * nb, 3 * nb)).tocsr() + sp.eye(3 * nb)
    U = sp.bsr_matrix((Ub, ci, rp), shape=(3 * nb, 3 * nb)).tocsr()
    A = sp.bsr_matrix((P.avals.reshape(-1, 3, 3), ci, rp), shape=(3 * nb, 3 * nb)).tocsr()
    return L, U, A


def test_coloring_valid(prep):
    s, P = prep.sys, prep
    for i in range(s.nb):
        for k in range(s.rowptr[i], s.rowptr[i + 1]):
            j = s.colind[k]
            assert j == i or P.color[i] != P.color[j]
    assert np.array_equal(np.sort(P.perm), np.arange(s.nb))
    assert np.all(np.diff(P.color[P.perm]) >= 0)
    assert P.color_ptr[-1] == s.nb
    # inside each color: rows with a higher-colored neighbour (either end)
    # first, then the others, each group in natural order
    higher = np.zeros(s.nb, bool)
    for i in range(s.nb):
        for k in range(s.rowptr[i], s.rowptr[i + 1]):
            j = s.colind[k]
            if P.color[j] > P.color[i]:
                higher[i] = True
            elif P.color[j] < P.color[i]:
                higher[j] = True
    for c in range(P.ncolors):
        rows = P.perm[P.color_ptr[c]:P.color_ptr[c + 1]]
        sp_ = int(P.split[c])
        assert np.all(higher[rows[:sp_]]) and not np.any(higher[rows[sp_:]])
        assert np.all(np.diff(rows[:sp_]) > 0) and np.all(np.diff(rows[sp_:]) > 0)
    assert P.split[-1] == 0


def test_ilu_identity(prep):
    L, U, A = lu_matrices(prep)
    M = (L @ U).tocsr()
    mask = A.copy()
    mask.data[:] = 1.0
    d = abs(M.multiply(mask) - A).max()
    assert d <= 1e-13 * abs(A).max()


def test_ilu_apply_equals_direct_solve(prep):
    L, U, _ = lu_matrices(prep)
    M = (L @ U).tocsc()
    p = np.random.default_rng(0).standard_normal(3 * prep.nb)
    z = prep.to_perm(prep.ilu_apply(p))
    zd = spla.spsolve(M, prep.to_perm(p))
    assert np.linalg.norm(z - zd) <= 1e-13 * np.linalg.norm(zd)
    zt = prep.to_perm(prep.ilu_apply(p, transpose=True))
    ztd = spla.spsolve(M.T.tocsc(), prep.to_perm(p))
    assert np.linalg.norm(zt - ztd) <= 1e-13 * np.linalg.norm(ztd)


def test_spmv_matches_scipy(prep):
    A = prep.sys.to_scipy()
    x = np.random.default_rng(1).standard_normal(3 * prep.nb)
    assert np.allclose(prep.spmv(x), A @ x, rtol=0, atol=1e-12 * np.abs(A @ x).max())
    assert np.allclose(prep.spmv(x, True), A.T @ x, rtol=0, atol=1e-12 * np.abs(A.T @ x).max())


def test_dense_solution_small():
    s = generate(10, 10, 5, sigma=1.0, seed=2)
    P = Prepared(s)
    x, r = P.solve(s.b, tol=1e-13, maxit=500)
    xd = np.linalg.solve(s.dense(), s.b)
    assert r.status == 0
    assert np.linalg.norm(x - xd) <= 1e-10 * np.linalg.norm(xd)
    xt, rt = P.solve(s.b, tol=1e-13, maxit=500, transpose=True)
    xtd = np.linalg.solve(s.dense().T, s.b)
    assert np.linalg.norm(xt - xtd) <= 1e-10 * np.linalg.norm(xtd)


def test_stop_rule_and_counters(prep):
    s = prep.sys
    for tol in (1e-2, 1e-6):
        x, r, hist = prep.solve(s.b, tol=tol, maxit=500, hist_cap=4096)
        assert r.status == 0
        # norm history: initial norm, then one per half iteration
        assert len(hist) == r.half_iters + 2
        assert hist[-1] <= tol * hist[0] < hist[-2]
        assert r.norms[0] == hist[0]
        assert r.last_norm_idx == (r.half_iters % 3) + 1
        true = np.linalg.norm(s.b - s.to_scipy() @ x) / np.linalg.norm(s.b)
        assert abs(true - r.relres) <= 1e-8


def test_maxit_half_iteration(prep):
    s = prep.sys
    for m in range(4):
        x, r = prep.solve(s.b, tol=1e-15, maxit=m)
        assert r.status == 1 and r.half_iters == 2 * m


def test_omp_matches_serial(prep):
    s = prep.sys
    x1, r1 = prep.solve(s.b, tol=1e-6, maxit=500)
    x2, r2 = prep.solve_omp(s.b, tol=1e-6, maxit=500, nthreads=4)
    assert r1.half_iters == r2.half_iters
    assert np.linalg.norm(x1 - x2) <= 1e-10 * np.linalg.norm(x1)


def test_mixed_refinement_reaches_tolerance(prep):
    s = prep.sys
    x, r, outer, inner = prep.mixed(s.b, tol=1e-8, inner_tol=1e-4)
    assert r.status == 0 and outer >= 2
    true = np.linalg.norm(s.b - s.to_scipy() @ x) / np.linalg.norm(s.b)
    assert true <= 1e-8 * (1 + 1e-9)


def test_gradient_finite_differences():
    s = generate(8, 6, 4, sigma=1.0, seed=4)
    P = Prepared(s)
    rng = np.random.default_rng(5)
    W = rng.choice(s.n, 12, replace=False)
    d = rng.standard_normal(12)

    def loss(vals, b):
        from fpga_gb300.synth import BlockSystem
        t = BlockSystem(s.nb, s.rowptr, s.colind, vals, b, s.cell_of_row, s.grid)
        x, _ = Prepared(t).solve(b, tol=1e-14, maxit=500)
        return 0.5 * np.sum((x[W] - d) ** 2), x

    L0, x = loss(s.vals, s.b)
    g = np.zeros(s.n)
    g[W] = x[W] - d
    lam, _ = P.solve(g, tol=1e-14, maxit=500, transpose=True)
    dA = P.grad_a(lam, x)
    eps = 1e-6
    for _ in range(6):
        k, r_, c_ = rng.integers(s.nnzb), rng.integers(3), rng.integers(3)
        vp, vm = s.vals.copy(), s.vals.copy()
        vp[k, r_, c_] += eps
        vm[k, r_, c_] -= eps
        fd = (loss(vp, s.b)[0] - loss(vm, s.b)[0]) / (2 * eps)
        assert abs(fd - dA[k, r_, c_]) <= 1e-5 * max(abs(fd), 1e-8) + 1e-10
        i = rng.integers(s.n)
        bp, bm = s.b.copy(), s.b.copy()
        bp[i] += eps
        bm[i] -= eps
        fd = (loss(s.vals, bp)[0] - loss(s.vals, bm)[0]) / (2 * eps)
        assert abs(fd - lam[i]) <= 1e-5 * max(abs(fd), 1e-8) + 1e-10


def golden_system(f):
    from fpga_gb300.synth import BlockSystem
    nb = f["rowptr"].size - 1
    return BlockSystem(nb, f["rowptr"], f["colind"], f["vals"].reshape(-1, 3, 3), f["b"],
                       np.arange(nb), tuple(int(v) for v in f["grid"]))


@pytest.mark.parametrize("name", ["golden_small.npz", "golden_faults.npz",
                                  "golden_faults_natural.npz"])
def test_golden_fixtures(name):
    f = np.load(os.path.join(GOLDEN, name))
    # the generator reproduces the stored system (structure exactly; values to
    # the last bits, numpy's exp may differ by an ulp across CPU types)
    g = generate(*[int(v) for v in f["grid"]], sigma=float(f["sigma"]),
                 inactive_frac=float(f["inactive"]), fault_frac=float(f["faults"]),
                 seed=int(f["seed"]))
    assert np.array_equal(g.rowptr, f["rowptr"]) and np.array_equal(g.colind, f["colind"])
    assert np.allclose(g.vals.reshape(-1), f["vals"], rtol=1e-14, atol=0)
    s = golden_system(f)
    P = Prepared(s, coloring=str(f["coloring"]))
    assert P.ncolors == int(f["ncolors"])
    assert np.array_equal(P.color, f["color"]) and np.array_equal(P.perm, f["perm"])
    assert np.array_equal(P.split, f["split"])
    assert np.array_equal(P.lu, f["lu"]) and np.array_equal(P.dinv, f["dinv"])
    x = f["x_probe"]
    assert np.array_equal(P.spmv(x), f["spmv"])
    assert np.array_equal(P.ilu_apply(x), f["ilu"])
    assert np.array_equal(P.spmv(x, True), f["spmv_t"])
    assert np.array_equal(P.ilu_apply(x, True), f["ilu_t"])
    xs, r = P.solve(s.b, tol=float(f["tol"]), maxit=500)
    assert r.half_iters == int(f["half_iters"])
    assert np.array_equal(xs, f["x"])


def test_threaded_transposed_solve_matches_sequential(prep):
    """The OpenMP transposed solve (the adjoint's CPU baseline) against the
    sequential transposed solve: same half-iterations, same solution."""
    P = prep
    s = P.sys
    g = np.random.default_rng(4).standard_normal(s.n)
    x1, r1 = P.solve(g, tol=1e-8, maxit=500, transpose=True)
    x2, r2 = P.solve_omp(g, tol=1e-8, maxit=500, nthreads=4, transpose=True)
    assert r1.status == r2.status == 0 and r1.half_iters == r2.half_iters
    assert np.linalg.norm(x1 - x2) <= 1e-10 * np.linalg.norm(x1)
    At = s.to_scipy().T
    assert np.linalg.norm(At @ x2 - g) <= 1e-7 * np.linalg.norm(g)
