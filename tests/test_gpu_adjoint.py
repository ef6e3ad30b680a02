"""The hand-written adjoint: A^T lambda = g with transposed SpMV and U^T/L^T
sweeps reusing the forward factors, dL/dA = -lambda_i x_j^T on the pattern.

Checked against the oracle's transposed solve, central finite differences
(eps = 1e-6, 20 random entries of A and b, 1e-5 relative) and a dense FP64
reference gradient on a 10x10x5 grid, through torch.autograd.
"""
import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import BlockSystem, adjoint_selection, generate, make_config
from oracle_lib import Prepared

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def loss_setup(s, seed=1):
    cells, d = adjoint_selection(s.nb, frac=0.05, seed=seed)
    idx = (3 * cells[:, None] + np.arange(3)).reshape(-1)
    return idx, d


def test_adjoint_matches_oracle(built_lib):
    s = generate(24, 20, 10, sigma=1.0, inactive_frac=0.05, fault_frac=0.01, seed=13)
    P = Prepared(s)
    idx, d = loss_setup(s)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = g.solve(s.b, tol=1e-12, maxit=2000)
        gv = np.zeros(s.n)
        gv[idx] = x[idx] - d
        lam, dA, ra = g.adjoint(gv, x, tol=1e-12, maxit=2000)
    lam_ref, rr = P.solve(gv, tol=1e-12, maxit=2000, transpose=True)
    assert ra.status == rr.status == 0
    assert ra.half_iters == rr.half_iters
    assert np.linalg.norm(lam - lam_ref) <= 1e-6 * np.linalg.norm(lam_ref)
    dA_ref = P.grad_a(lam, x)
    assert np.array_equal(dA, dA_ref) or np.abs(dA - dA_ref).max() <= 1e-15 * np.abs(dA_ref).max()
    At = s.to_scipy().T
    assert np.linalg.norm(At @ lam - gv) <= 1e-11 * np.linalg.norm(gv)


def _torch_loss(s, solver, vals, b, idx, d):
    from fpga_gb300.autograd import solve
    x = solve(vals, b, solver, tol=1e-13, maxit=4000)
    return 0.5 * torch.sum((x[idx] - d) ** 2)


def test_finite_differences(built_lib):
    s = generate(10, 8, 4, sigma=1.0, seed=21)
    idx, d = loss_setup(s, seed=2)
    idx_t = torch.from_numpy(idx)
    d_t = torch.from_numpy(d)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind)
        vals = torch.from_numpy(s.vals.copy()).requires_grad_(True)
        b = torch.from_numpy(s.b.copy()).requires_grad_(True)
        L = _torch_loss(s, g, vals, b, idx_t, d_t)
        L.backward()
    rng = np.random.default_rng(3)
    eps = 1e-6

    def f(v, bb):
        # the loss itself by a sparse direct solve: finite differences of
        # the exact function, free of iterative-solver noise
        import scipy.sparse.linalg as spla
        t = BlockSystem(s.nb, s.rowptr, s.colind, v, bb, s.cell_of_row, s.grid)
        x = spla.spsolve(t.to_scipy().tocsc(), bb)
        return 0.5 * float(np.sum((x[idx] - d) ** 2))

    # 1e-5 relative, relative to the largest sampled gradient entry
    fds, ans = [], []
    for _ in range(20):
        k, r_, c_ = rng.integers(s.nnzb), rng.integers(3), rng.integers(3)
        vp, vm = s.vals.copy(), s.vals.copy()
        vp[k, r_, c_] += eps
        vm[k, r_, c_] -= eps
        fds.append((f(vp, s.b) - f(vm, s.b)) / (2 * eps))
        ans.append(float(vals.grad[k, r_, c_]))
    fds, ans = np.array(fds), np.array(ans)
    assert np.abs(fds - ans).max() <= 1e-5 * np.abs(ans).max(), (fds, ans)
    fds, ans = [], []
    for _ in range(20):
        i = rng.integers(s.n)
        bp, bm = s.b.copy(), s.b.copy()
        bp[i] += eps
        bm[i] -= eps
        fds.append((f(s.vals, bp) - f(s.vals, bm)) / (2 * eps))
        ans.append(float(b.grad[i]))
    fds, ans = np.array(fds), np.array(ans)
    assert np.abs(fds - ans).max() <= 1e-5 * np.abs(ans).max(), (fds, ans)


def test_finite_differences_60x60x30(built_lib):
    """The 60x60x30 adjoint system at its stated size (108,000 cells, sigma
    1.0, W = 1 % of the cells): central differences with eps = 1e-6 on 20
    random entries of A and 20 of b against the adjoint's dL/dA and dL/db,
    forward solve and adjoint to a relative residual of 1e-10.

    Each perturbed solution is x + delta, delta from FP64 GPU solves of
    the perturbed system for the change alone: (A + e E) delta = -e E x
    (for b: A delta = e e_i). Then x + delta solves the perturbed system
    exactly where x solves the unperturbed one, and delta is resolved to
    1e-12 of itself, far below what subtracting two full solves to an
    absolute residual could give. BiCGSTAB stops on its recursive residual,
    which can drift from the true one, so delta is refined in FP64 until
    its true residual (formed on the host with the perturbed matrix) is
    below 1e-12 of the right-hand side. The loss difference is formed as
    (W(d+ - d-)) . (W(x + (d+ + d-)/2) - d), which is
    L(x + d+) - L(x + d-) without the cancellation of two O(1) losses.

    Tolerance: 1e-5 relative, norm-wise over the 20 sampled entries, and per
    entry for the entries at least 1e-3 of the largest sampled one (an
    entry far from every observed cell can be 1e-7 of the largest, below
    what FP64 residuals resolve)."""
    s = make_config("c4_60x60x30_adjoint")
    cells, d = adjoint_selection(s.nb)
    idx = (3 * cells[:, None] + np.arange(3)).reshape(-1)
    rows = np.repeat(np.arange(s.nb), np.diff(s.rowptr))
    rng = np.random.default_rng(4)
    eps = 1e-6
    A = s.to_scipy().tocsr()

    def refined(g, rhs, matvec):
        """delta with ||rhs - A delta|| <= 1e-12 ||rhs|| (true residual)."""
        delta = np.zeros(s.n)
        r = rhs.copy()
        for _ in range(6):
            dd, rr = g.solve(r, tol=1e-9, maxit=4000)
            assert rr.status in (0, 1), rr.status
            delta += dd
            r = rhs - matvec(delta)
            if np.linalg.norm(r) <= 1e-12 * np.linalg.norm(rhs):
                return delta
        raise AssertionError("refinement did not reach 1e-12")

    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = g.solve(s.b, tol=1e-10, maxit=4000)
        assert r.status == 0
        gv = np.zeros(s.n)
        gv[idx] = x[idx] - d
        lam, dA, ra = g.adjoint(gv, x, tol=1e-10, maxit=4000)
        assert ra.status == 0

        def dloss(dp, dm):
            dx = dp - dm
            return float(np.dot(dx[idx], x[idx] + 0.5 * (dp[idx] + dm[idx]) - d))

        def check(fds, ans, what):
            fds, ans = np.array(fds), np.array(ans)
            nrm = np.linalg.norm(fds - ans) / np.linalg.norm(ans)
            big = np.abs(ans) >= 1e-3 * np.abs(ans).max()
            per = np.abs(fds - ans)[big] / np.abs(ans)[big]
            print(f"{what}: norm-wise {nrm:.2e}, per entry max {per.max():.2e} "
                  f"({big.sum()} of {ans.size} entries)")
            for a, b_ in zip(fds, ans):
                print(f"  fd {a:+.10e} adjoint {b_:+.10e}")
            assert nrm <= 1e-5 and per.max() <= 1e-5, (what, fds, ans)

        fds, ans = [], []
        for i in rng.choice(s.n, 20, replace=False):
            e = np.zeros(s.n)
            e[i] = eps
            dp = refined(g, e, lambda v: A @ v)
            dm = refined(g, -e, lambda v: A @ v)
            fds.append(dloss(dp, dm) / (2 * eps))
            ans.append(lam[i])
        check(fds, ans, "dL/db")

        fds, ans = [], []
        for k in rng.choice(s.nnzb, 20, replace=False):
            rr, cc = rng.integers(3), rng.integers(3)
            i, j = rows[k], s.colind[k]
            deltas = []
            for sg in (1.0, -1.0):
                v = s.vals.copy()
                v[k, rr, cc] += sg * eps
                g.factor(v)
                rhs = np.zeros(s.n)
                rhs[3 * i + rr] = -sg * eps * x[3 * j + cc]

                def matvec(vv, sg=sg, i=i, j=j, rr=rr, cc=cc):
                    out = A @ vv
                    out[3 * i + rr] += sg * eps * vv[3 * j + cc]
                    return out
                deltas.append(refined(g, rhs, matvec))
            fds.append(dloss(*deltas) / (2 * eps))
            ans.append(dA[k, rr, cc])
        g.factor(s.vals)
        check(fds, ans, "dL/dA")


def test_dense_reference_gradient(built_lib):
    s = generate(10, 10, 5, sigma=1.0, seed=31)
    idx, d = loss_setup(s, seed=4)
    A = s.dense()
    x = np.linalg.solve(A, s.b)
    gx = np.zeros(s.n)
    gx[idx] = x[idx] - d
    lam = np.linalg.solve(A.T, gx)
    dA_dense = -np.outer(lam, x)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind)
        vals = torch.from_numpy(s.vals.copy()).requires_grad_(True)
        b = torch.from_numpy(s.b.copy()).requires_grad_(True)
        L = _torch_loss(s, g, vals, b, torch.from_numpy(idx), torch.from_numpy(d))
        L.backward()
    assert np.linalg.norm(b.grad.numpy() - lam) <= 1e-8 * np.linalg.norm(lam)
    gv = vals.grad.numpy()
    ref = np.empty_like(gv)
    for i in range(s.nb):
        for k in range(s.rowptr[i], s.rowptr[i + 1]):
            j = s.colind[k]
            ref[k] = dA_dense[3 * i:3 * i + 3, 3 * j:3 * j + 3]
    assert np.linalg.norm(gv - ref) <= 1e-8 * np.linalg.norm(ref)


def test_mixed_adjoint_error_vs_fp64(built_lib):
    """FP32 factor storage, FP64 refinement to 1e-8: gradient error stated
    against the FP64 adjoint of the same system."""
    s = generate(30, 30, 10, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=41)
    idx, d = loss_setup(s, seed=5)
    out = {}
    for prec in ("fp64", "mixed"):
        with GbIlu(device=0, precision=prec) as g:
            g.analyze(s.rowptr, s.colind).factor(s.vals)
            x, r = g.solve(s.b, tol=1e-10 if prec == "fp64" else 1e-8, maxit=4000)
            gv = np.zeros(s.n)
            gv[idx] = x[idx] - d
            lam, dA, ra = g.adjoint(gv, x, tol=1e-10 if prec == "fp64" else 1e-8, maxit=4000)
            assert r.status == 0 and ra.status == 0
            out[prec] = (lam, dA)
    err_l = np.linalg.norm(out["mixed"][0] - out["fp64"][0]) / np.linalg.norm(out["fp64"][0])
    err_a = np.linalg.norm(out["mixed"][1] - out["fp64"][1]) / np.linalg.norm(out["fp64"][1])
    print(f"mixed adjoint: lambda rel err {err_l:.2e}, dA rel err {err_a:.2e}")
    assert err_l < 1e-6 and err_a < 1e-6


def test_adjoint_device_pointers_match_host(built_lib):
    """gbilu_adjoint_device (device arrays, lambda and dL/dA formed without
    leaving the device) gives the same bits as gbilu_adjoint on host
    arrays, with and without the gradient."""
    s = generate(24, 20, 10, sigma=1.0, inactive_frac=0.05, fault_frac=0.01, seed=13)
    idx, d = loss_setup(s)
    dev = torch.device("cuda:0")
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = g.solve(s.b, tol=1e-12, maxit=2000)
        gv = np.zeros(s.n)
        gv[idx] = x[idx] - d
        lam, dA, ra = g.adjoint(gv, x, tol=1e-12, maxit=2000)
        lam0, _, ra0 = g.adjoint(gv, x, tol=1e-12, maxit=2000, want_dA=False)
        gd = torch.from_numpy(gv).to(dev)
        xd = torch.from_numpy(x).to(dev)
        ld = torch.full((s.n,), float("nan"), dtype=torch.float64, device=dev)
        dAd = torch.full((s.nnzb * 9,), float("nan"), dtype=torch.float64, device=dev)
        rd = g.adjoint_device(gd.data_ptr(), xd.data_ptr(), ld.data_ptr(), dAd.data_ptr(),
                              tol=1e-12, maxit=2000)
        assert rd.status == ra.status == 0 and rd.half_iters == ra.half_iters
        assert np.array_equal(ld.cpu().numpy(), lam) and np.array_equal(lam0, lam)
        assert np.array_equal(dAd.cpu().numpy().reshape(-1, 3, 3), dA)
        ld.fill_(float("nan"))
        rd2 = g.adjoint_device(gd.data_ptr(), xd.data_ptr(), ld.data_ptr(), None,
                               tol=1e-12, maxit=2000)
        assert np.array_equal(ld.cpu().numpy(), lam) and rd2.half_iters == ra.half_iters
        assert rd.device_ms > 0 and ra0.device_ms > 0
