"""CUDA path vs the CPU oracle, through the C ABI (libgbilu.so).

Tolerances (norm-wise relative): SpMV and ILU apply 1e-12, solution 1e-6 at
the same stopping rule, identical half-iteration counts. Sizes are ones the
oracle finishes in seconds.
"""
import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import generate, make_config
from oracle_lib import Prepared

pytestmark = pytest.mark.gpu

KERNEL_TOL = 1e-12
SOLUTION_TOL = 1e-6

CASES = {
    "c1": lambda: make_config("c1_20x20x10"),
    "faults": lambda: generate(30, 24, 12, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=7),
    "sigma2": lambda: generate(24, 24, 10, sigma=2.0, inactive_frac=0.05, fault_frac=0.01, seed=11),
    # colors above the shared-memory staging limit (16384 rows): large steps
    # read from global memory around the staged small ones
    "mid": lambda: generate(60, 60, 20, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=5),
}


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request, built_lib):
    s = CASES[request.param]()
    P = Prepared(s)
    g = GbIlu(device=0)
    g.analyze(s.rowptr, s.colind).factor(s.vals)
    yield s, P, g
    g.close()


def test_ordering_matches_oracle(case):
    s, P, g = case
    nc, color, perm, cp = g.ordering()
    assert nc == P.ncolors
    assert np.array_equal(color, P.color) and np.array_equal(perm, P.perm)
    assert np.array_equal(cp, P.color_ptr)
    lu, dinv = g.factors()
    assert np.array_equal(lu, P.lu) and np.array_equal(dinv, P.dinv)


@pytest.mark.parametrize("transpose", [False, True])
def test_spmv(case, transpose):
    s, P, g = case
    x = np.random.default_rng(1).standard_normal(s.n)
    assert rel(g.spmv(x, transpose), P.spmv(x, transpose)) < KERNEL_TOL


@pytest.mark.parametrize("transpose", [False, True])
def test_ilu_apply(case, transpose):
    s, P, g = case
    p = np.random.default_rng(2).standard_normal(s.n)
    assert rel(g.ilu_apply(p, transpose), P.ilu_apply(p, transpose)) < KERNEL_TOL


@pytest.mark.parametrize("tol", [1e-2, 1e-6])
def test_solve(case, tol):
    s, P, g = case
    x_ref, r_ref = P.solve(s.b, tol=tol, maxit=500)
    x, r = g.solve(s.b, tol=tol, maxit=500)
    assert r.status == r_ref.status == 0
    assert r.half_iters == r_ref.half_iters
    assert rel(x, x_ref) < SOLUTION_TOL
    assert abs(r.norm0 - r_ref.norm0) <= 1e-12 * r_ref.norm0
    assert r.last_norm_idx == r_ref.last_norm_idx
    true_res = np.linalg.norm(s.b - s.to_scipy() @ x) / np.linalg.norm(s.b)
    assert true_res <= tol * (1 + 1e-6)


def test_graph_and_host_loop_bit_identical(case):
    s, P, g = case
    x1, r1 = g.solve(s.b, tol=1e-6, maxit=500)
    with GbIlu(device=0, use_graph=False) as h:
        h.analyze(s.rowptr, s.colind).factor(s.vals)
        x2, r2 = h.solve(s.b, tol=1e-6, maxit=500)
    assert r1.half_iters == r2.half_iters
    assert np.array_equal(x1, x2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_and_host_loop_adjoint_bit_identical(case, precision):
    """The CUDA graph with its device-side while loop and host-driven
    launches of the same kernels: identical bits for the forward solve (FP64
    or mixed refinement) and the adjoint (transposed operators)."""
    s, P, g = case
    tol = 1e-8 if precision == "mixed" else 1e-6
    gv = np.random.default_rng(9).standard_normal(s.n)
    out = []
    for graph in (True, False):
        with GbIlu(device=0, precision=precision, use_graph=graph) as h:
            h.analyze(s.rowptr, s.colind).factor(s.vals)
            x, r = h.solve(s.b, tol=tol, maxit=500)
            lam, dA, ra = h.adjoint(gv, x, tol=tol, maxit=500)
            out.append((x, r.half_iters, r.inner_half_iters, lam, ra.half_iters))
    assert out[0][1:3] == out[1][1:3] and out[0][4] == out[1][4]
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][3], out[1][3])


def test_sweep_modes_bit_identical(case):
    """One launch per color and the single cooperative launch compute the
    same rows with the same arithmetic: results agree bit for bit."""
    s, P, g = case
    p = np.random.default_rng(6).standard_normal(s.n)
    x1, r1 = g.solve(s.b, tol=1e-6, maxit=500)
    z1, zt1 = g.ilu_apply(p), g.ilu_apply(p, True)
    with GbIlu(device=0, sweep_mode=0) as h:
        h.analyze(s.rowptr, s.colind).factor(s.vals)
        x2, r2 = h.solve(s.b, tol=1e-6, maxit=500)
        assert np.array_equal(h.ilu_apply(p), z1) and np.array_equal(h.ilu_apply(p, True), zt1)
    assert r1.half_iters == r2.half_iters and np.array_equal(x1, x2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_factorization_bit_identical(case, precision):
    """ILU0 on the GPU (color-parallel) gives the host/oracle factors bit for
    bit, hence identical solves."""
    s, P, g = case
    with GbIlu(device=0, precision=precision, factor_on_device=True) as d, \
            GbIlu(device=0, precision=precision) as h:
        d.analyze(s.rowptr, s.colind).factor(s.vals)
        h.analyze(s.rowptr, s.colind).factor(s.vals)
        lu, dinv = d.factors()
        assert np.array_equal(lu, P.lu) and np.array_equal(dinv, P.dinv)
        x1, r1 = d.solve(s.b, tol=1e-8, maxit=500)
        x2, r2 = h.solve(s.b, tol=1e-8, maxit=500)
        assert r1.status == r2.status and np.array_equal(x1, x2)
        # refactor with new values on the same pattern
        v2 = s.vals * 1.5
        d.factor(v2)
        h.factor(v2)
        assert np.array_equal(d.factors()[0], h.factors()[0])


def test_device_factorization_singular(built_lib):
    from fpga_gb300 import GbIluError
    s = make_config("c1_20x20x10")
    vals = s.vals.copy()
    d = np.nonzero(s.colind[s.rowptr[10]:s.rowptr[11]] == 10)[0][0] + s.rowptr[10]
    vals[d] = 0.0
    msgs = []
    for dev in (True, False):
        with GbIlu(device=0, factor_on_device=dev) as g:
            g.analyze(s.rowptr, s.colind)
            with pytest.raises(GbIluError) as e:
                g.factor(vals)
            assert e.value.code == 7
            msgs.append(str(e.value))
    assert msgs[0] == msgs[1]


@pytest.mark.parametrize("scheme", [0, 1])
def test_mixed_precision_solve(case, scheme):
    """FP32 storage/sweeps with the FP64 residual: reaches relres 1e-8 on the
    FP64 residual; the error against the FP64 oracle solution is stated."""
    s, P, g = case
    x_ref, r_ref = P.solve(s.b, tol=1e-11, maxit=4000)
    with GbIlu(device=0, precision="mixed", mixed_scheme=scheme, inner_tol=1e-3) as m:
        m.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = m.solve(s.b, tol=1e-8, maxit=4000)
        x2, _ = m.solve(s.b, tol=1e-8, maxit=4000)
    true = np.linalg.norm(s.b - s.to_scipy() @ x) / np.linalg.norm(s.b)
    err = rel(x, x_ref)
    print(f"mixed scheme {scheme}: status {r.status} true relres {true:.2e} "
          f"x err vs FP64 {err:.2e} replacements/outer {r.outer_iters} halves {r.inner_half_iters}")
    assert r.status == 0 and true <= 1e-8 * (1 + 1e-6)
    assert abs(r.true_relres - true) <= 1e-3 * true
    assert err < 1e-5
    assert np.array_equal(x, x2)           # deterministic


def test_ilu_trace(case):
    s, P, g = case
    for transpose in (False, True):
        tr = g.ilu_trace(transpose=transpose)
        steps = g.schedule(transpose)
        assert len(tr) == len(steps) and [r for r, _ in tr] == [st["nrows"] for st in steps]
        assert sum(r for r, _ in tr) >= s.nb and all(us >= 0 for _, us in tr)


def test_pinned_host_buffers_bit_identical(case):
    """Page-locked host buffers are read and written in place by the gather
    and scatter kernels; ordinary host memory goes through staging copies.
    Both give the same bits, with x0 = 0, a warm start and an already
    converged right-hand side."""
    torch = pytest.importorskip("torch")
    s, P, g = case
    x0 = np.random.default_rng(3).standard_normal(s.n)
    for b_np, x0_np in ((s.b, np.zeros(s.n)), (s.b, x0), (np.zeros(s.n), x0)):
        x1 = x0_np.copy()
        r1 = g.solve_host_ptr(b_np.ctypes.data, x1.ctypes.data, 1e-6, 500)
        b = torch.from_numpy(b_np.copy()).pin_memory()
        x = torch.from_numpy(x0_np.copy()).pin_memory()
        r2 = g.solve_host_ptr(b.data_ptr(), x.data_ptr(), 1e-6, 500)
        assert r1.status == r2.status and r1.half_iters == r2.half_iters
        assert np.array_equal(x.numpy(), x1)
        x3 = x0_np.copy()      # page-locked b, ordinary x: staging copies
        r3 = g.solve_host_ptr(b.data_ptr(), x3.ctypes.data, 1e-6, 500)
        assert r3.half_iters == r1.half_iters and np.array_equal(x3, x1)
        # device arrays: b permuted by its own kernel instead of inside the
        # initial-residual kernel
        bd, xd = b.cuda(), torch.from_numpy(x0_np.copy()).cuda()
        r4 = g.solve_device(bd.data_ptr(), xd.data_ptr(), 1e-6, 500)
        assert r4.half_iters == r1.half_iters and np.array_equal(xd.cpu().numpy(), x1)
        if r1.status == 2:
            assert np.array_equal(x1, x0_np)


def test_pinned_host_buffers_mixed_bit_identical(case):
    """The mixed form reads b and x0 before its first FP64 residual: from
    page-locked buffers in place, from ordinary memory through staging
    copies; the same bits either way, and the same as device pointers."""
    torch = pytest.importorskip("torch")
    s, P, _ = case
    x0 = np.random.default_rng(4).standard_normal(s.n)
    with GbIlu(device=0, precision="mixed") as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        for x0_np in (np.zeros(s.n), x0):
            x1 = x0_np.copy()
            r1 = g.solve_host_ptr(s.b.ctypes.data, x1.ctypes.data, 1e-8, 500)
            b = torch.from_numpy(s.b.copy()).pin_memory()
            x = torch.from_numpy(x0_np.copy()).pin_memory()
            r2 = g.solve_host_ptr(b.data_ptr(), x.data_ptr(), 1e-8, 500)
            bd, xd = b.cuda(), torch.from_numpy(x0_np.copy()).cuda()
            r3 = g.solve_device(bd.data_ptr(), xd.data_ptr(), 1e-8, 500)
            assert r1.status == r2.status == r3.status == 0
            assert r1.outer_iters == r2.outer_iters == r3.outer_iters
            assert np.array_equal(x.numpy(), x1) and np.array_equal(xd.cpu().numpy(), x1)


def test_deterministic(case):
    s, P, g = case
    x1, _ = g.solve(s.b, tol=1e-6, maxit=500)
    x2, _ = g.solve(s.b, tol=1e-6, maxit=500)
    assert np.array_equal(x1, x2)


@pytest.mark.parametrize("maxit", [0, 1, 2, 3])
def test_maxit_semantics(case, maxit):
    s, P, g = case
    x_ref, r_ref = P.solve(s.b, tol=1e-14, maxit=maxit)
    x, r = g.solve(s.b, tol=1e-14, maxit=maxit)
    assert r_ref.status == 1 and r.status == 1
    assert r.half_iters == r_ref.half_iters == 2 * maxit
    assert rel(x, x_ref) < 1e-10


@pytest.mark.parametrize("scheme", [0, 1])
@pytest.mark.parametrize("use_graph", [True, False])
def test_mixed_maxit_semantics(built_lib, scheme, use_graph):
    """maxit caps the mixed solve's inner half-iterations of all refinement
    steps together at 2*maxit + 1, as the reference caps one run; the
    counter then reads 2*maxit and the status is MAXIT."""
    s = CASES["faults"]()
    with GbIlu(device=0, precision="mixed", mixed_scheme=scheme, use_graph=use_graph) as m:
        m.analyze(s.rowptr, s.colind).factor(s.vals)
        for maxit in (0, 1, 2, 3, 7):
            x, r = m.solve(s.b, tol=1e-14, maxit=maxit)
            assert r.status == 1, (maxit, r.status)
            assert r.half_iters == 2 * maxit, (maxit, r.half_iters)
            assert r.inner_half_iters == 2 * maxit + 1, (maxit, r.inner_half_iters)
            true = np.linalg.norm(s.b - s.to_scipy() @ x) / np.linalg.norm(s.b)
            assert abs(r.true_relres - true) <= 1e-6 * true
        # inner_maxit still caps each refinement step, maxit the total
        if scheme == 0:
            with GbIlu(device=0, precision="mixed", inner_maxit=1, max_outer=50) as m2:
                m2.analyze(s.rowptr, s.colind).factor(s.vals)
                x, r = m2.solve(s.b, tol=1e-14, maxit=4)
                assert r.status == 1 and r.inner_half_iters == 9 and r.outer_iters >= 3


def test_warm_start(case):
    s, P, g = case
    x0 = np.random.default_rng(3).standard_normal(s.n) * 0.1
    x_ref, r_ref = P.solve(s.b, x0=x0, tol=1e-4, maxit=500)
    x, r = g.solve(s.b, x0=x0, tol=1e-4, maxit=500)
    assert r.half_iters == r_ref.half_iters
    assert rel(x, x_ref) < SOLUTION_TOL


def test_already_converged(built_lib):
    s = make_config("c1_20x20x10")
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        # ||r0|| = 0 <= 1e-30: "no results", no iteration
        x, r = g.solve(np.zeros(s.n), x0=np.zeros(s.n), tol=1e-2)
        assert r.status == 2 and r.half_iters == -1 and r.norm0 == 0.0
    with GbIlu(device=0, absolute=True) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        # x untouched when no iteration ran
        x0 = np.full(s.n, 7.0)
        b = s.to_scipy() @ x0 + 1e-9
        x, r = g.solve(b, x0=x0, tol=1e-3)
        assert r.status == 2 and np.array_equal(x, x0)


def test_absolute_tolerance(built_lib):
    s = make_config("c1_20x20x10")
    P = Prepared(s)
    x_ref, r_ref = P.solve(s.b, tol=1.0, maxit=200, absolute=True)
    with GbIlu(device=0, absolute=True) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = g.solve(s.b, tol=1.0, maxit=200)
        assert r.status == 0 and r.norm <= 1.0
        assert r.half_iters == r_ref.half_iters
        assert rel(x, x_ref) < SOLUTION_TOL
        x, r = g.solve(s.b, tol=1e6, maxit=200)   # ||r0|| below the absolute bound
        assert r.status == 2


def test_nonfinite_rhs(built_lib):
    s = make_config("c1_20x20x10")
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        b = s.b.copy()
        b[17] = np.nan
        x, r = g.solve(b, tol=1e-2)
        assert r.status == 4
        # the handle stays usable
        x, r = g.solve(s.b, tol=1e-2)
        assert r.status == 0


def test_timeout_status(built_lib):
    s = generate(40, 40, 20, sigma=2.0, seed=5)
    with GbIlu(device=0, timeout_ms=1e-3) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x, r = g.solve(s.b, tol=1e-14, maxit=100000)
        assert r.status == 5
        x, r = g.solve(s.b, tol=1e-2, maxit=100)
        assert r.status in (0, 5)


def test_config2_size_properties(built_lib):
    """Full 500k-cell system: SpMV parity and the 1e-2 solve against the oracle."""
    s = make_config("c2_100x100x50")
    P = Prepared(s)
    with GbIlu(device=0) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        x = np.random.default_rng(4).standard_normal(s.n)
        assert rel(g.spmv(x), P.spmv(x)) < KERNEL_TOL
        assert rel(g.ilu_apply(x), P.ilu_apply(x)) < KERNEL_TOL
        xs, r = g.solve(s.b, tol=1e-2, maxit=1000)
        xr, rr = P.solve(s.b, tol=1e-2, maxit=1000)
        assert r.half_iters == rr.half_iters and r.status == 0
        assert rel(xs, xr) < SOLUTION_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_staging_off_bit_identical(case, precision):
    """The single-launch apply without shared-memory staging (small steps from
    global memory, grid barriers between them) gives the same bits as with
    staging and data-ordered small steps."""
    s, P, g = case
    p = np.random.default_rng(9).standard_normal(s.n)
    runs = []
    for stage in (True, False):
        with GbIlu(device=0, precision=precision, stage_small_steps=stage) as h:
            h.analyze(s.rowptr, s.colind).factor(s.vals)
            x, r = h.solve(s.b, tol=1e-8, maxit=500)
            runs.append((x, r.half_iters, h.ilu_apply(p), h.ilu_apply(p, True)))
    (x1, k1, z1, t1), (x2, k2, z2, t2) = runs
    assert k1 == k2 and np.array_equal(x1, x2)
    assert np.array_equal(z1, z2) and np.array_equal(t1, t2)


def test_partly_staged_500k_bit_identical(built_lib):
    """A 500k-cell system whose color 2 (17135 rows with the natural-order
    coloring) is above the staging limit: staged runs and global-memory
    (streamed) steps mixed in one apply, against one launch per color step."""
    s = generate(100, 100, 50, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=1)
    p = np.random.default_rng(10).standard_normal(s.n)
    runs = []
    for mode in (1, 0):
        with GbIlu(device=0, sweep_mode=mode, coloring="natural") as h:
            h.analyze(s.rowptr, s.colind).factor(s.vals)
            x, r = h.solve(s.b, tol=1e-6, maxit=500)
            assert r.status == 0
            runs.append((x, r.half_iters, h.ilu_apply(p), h.ilu_apply(p, True)))
    (x1, k1, z1, t1), (x2, k2, z2, t2) = runs
    assert k1 == k2 and np.array_equal(x1, x2)
    assert np.array_equal(z1, z2) and np.array_equal(t1, t2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_off_bit_identical(case, precision):
    """The large color steps streamed through the shared-memory ring by a
    producer warp give the same bits as every warp loading its own rows."""
    s, P, g = case
    p = np.random.default_rng(9).standard_normal(s.n)
    runs = []
    for ring in (True, False):
        with GbIlu(device=0, precision=precision, stream_large_steps=ring) as h:
            h.analyze(s.rowptr, s.colind).factor(s.vals)
            x, r = h.solve(s.b, tol=1e-8, maxit=500)
            runs.append((x, r.half_iters, h.ilu_apply(p), h.ilu_apply(p, True)))
    (x1, k1, z1, t1), (x2, k2, z2, t2) = runs
    assert k1 == k2 and np.array_equal(x1, x2)
    assert np.array_equal(z1, z2) and np.array_equal(t1, t2)


@pytest.mark.parametrize("coloring", ["parity", "natural"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_500k_bit_identical(built_lib, precision, coloring):
    """The 500k-cell system: the single-launch apply with its streamed large
    steps, without the ring, and one launch per color step give the same
    bits (forward and transposed applies, FP64; solves in both precisions);
    the FP64 apply matches the oracle to the kernel tolerance."""
    s = make_config("c2_100x100x50")
    p = np.random.default_rng(12).standard_normal(s.n)
    runs = []
    for kw in (dict(stream_large_steps=True), dict(stream_large_steps=False),
               dict(sweep_mode=0)):
        with GbIlu(device=0, precision=precision, coloring=coloring, **kw) as h:
            h.analyze(s.rowptr, s.colind).factor(s.vals)
            if kw.get("stream_large_steps") and precision == "mixed":
                # the FP32 apply streams its second large step (FP64 slices
                # leave too few stages for a ring)
                st = h.stats()
                assert st["ring_stages"][1] >= 12 and st["apply_smem_bytes"][1] > 0
            x, r = h.solve(s.b, tol=1e-4, maxit=500)
            assert r.status == 0
            runs.append((x, r.half_iters, h.ilu_apply(p), h.ilu_apply(p, True)))
    for x2, k2, z2, t2 in runs[1:]:
        assert k2 == runs[0][1] and np.array_equal(x2, runs[0][0])
        assert np.array_equal(z2, runs[0][2]) and np.array_equal(t2, runs[0][3])
    if precision == "fp64":
        P = Prepared(s, coloring=coloring)
        assert rel(runs[0][2], P.ilu_apply(p)) < KERNEL_TOL
        assert rel(runs[0][3], P.ilu_apply(p, True)) < KERNEL_TOL


def test_zero_start_shortcut(case):
    """From x0 = 0 the initial A x0 is not computed (the gather of x0 finds
    no nonzero entry): -0.0 entries give the same bits as +0.0, and a single
    nonzero entry still takes the full path, matching the oracle."""
    s, P, g = case
    x1, r1 = g.solve(s.b, x0=np.zeros(s.n), tol=1e-6, maxit=500)
    x2, r2 = g.solve(s.b, x0=np.full(s.n, -0.0), tol=1e-6, maxit=500)
    assert r1.half_iters == r2.half_iters and np.array_equal(x1, x2)
    x0 = np.zeros(s.n)
    x0[s.n // 2] = 1e-3
    x_ref, r_ref = P.solve(s.b, x0=x0, tol=1e-6, maxit=500)
    x3, r3 = g.solve(s.b, x0=x0, tol=1e-6, maxit=500)
    assert r3.half_iters == r_ref.half_iters
    assert rel(x3, x_ref) < SOLUTION_TOL
    assert abs(r3.norm0 - r_ref.norm0) <= 1e-12 * r_ref.norm0
