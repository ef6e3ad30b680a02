"""The parity-order coloring computed on the GPU (gbilu_options.
color_on_device) against the host's and the oracle's: the same colors,
hence the same permutation, factors and solves, on grids with faults and
inactive cells and on patterns that are not grids."""
import numpy as np
import pytest

from fpga_gb300 import GbIlu
from fpga_gb300.synth import BlockSystem, generate, make_config
from oracle_lib import lib

pytestmark = pytest.mark.gpu


def random_symmetric(nb, density, seed):
    rng = np.random.default_rng(seed)
    m = rng.random((nb, nb)) < density
    m = m | m.T | np.eye(nb, dtype=bool)
    rowptr = np.concatenate([[0], np.cumsum(m.sum(1))]).astype(np.int32)
    colind = np.concatenate([np.flatnonzero(r) for r in m]).astype(np.int32)
    return rowptr, colind


def chain(nb):
    rows = [[j for j in (i - 1, i, i + 1) if 0 <= j < nb] for i in range(nb)]
    rowptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    return rowptr, np.concatenate(rows).astype(np.int32)


PATTERNS = {
    "c1": lambda: (lambda s: (s.rowptr, s.colind))(make_config("c1_20x20x10")),
    "faults": lambda: (lambda s: (s.rowptr, s.colind))(
        generate(30, 24, 12, sigma=1.5, inactive_frac=0.05, fault_frac=0.02, seed=7)),
    "chain": lambda: chain(1000),
    "rand_sparse": lambda: random_symmetric(300, 0.01, 1),
    "rand_dense": lambda: random_symmetric(120, 0.3, 2),
}


@pytest.mark.parametrize("name", sorted(PATTERNS))
def test_device_coloring_matches_host_and_oracle(built_lib, name):
    rowptr, colind = PATTERNS[name]()
    nb = rowptr.size - 1
    ref = np.empty(nb, np.int32)
    nref = lib().orc_color_parity(nb, rowptr, colind, ref)
    out = {}
    for dev in (False, True):
        with GbIlu(device=0, color_on_device=dev) as g:
            g.analyze(rowptr, colind)
            out[dev] = g.ordering()
            st = g.stats()
            assert st["color_on_device"] == int(dev)
    assert out[True][0] == out[False][0] == nref
    for a, b in zip(out[True][1:], out[False][1:]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[True][1], ref)


def test_device_coloring_500k_solve_bit_identical(built_lib):
    """The 500k-cell system: colors, permutation and the solve itself are
    the same with the coloring on the GPU."""
    s = make_config("c2_100x100x50")
    res = {}
    for dev in (False, True):
        with GbIlu(device=0, color_on_device=dev) as g:
            g.analyze(s.rowptr, s.colind).factor(s.vals)
            nc, color, perm, cp = g.ordering()
            x, r = g.solve(s.b, tol=1e-6, maxit=500)
            res[dev] = (nc, color, perm, x, r.half_iters, g.stats())
    assert res[True][0] == res[False][0] == 3
    for i in (1, 2, 3):
        assert np.array_equal(res[True][i], res[False][i])
    assert res[True][4] == res[False][4]
    print(f"coloring: host {res[False][5]['color_ms']:.1f} ms, "
          f"device {res[True][5]['color_ms']:.1f} ms; analysis host "
          f"{res[False][5]['analyze_ms']:.1f} ms, with device coloring "
          f"{res[True][5]['analyze_ms']:.1f} ms")
