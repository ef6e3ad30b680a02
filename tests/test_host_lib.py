"""libgbilu.so on the CPU: it loads, exports what include/gbilu.h declares,
and its host-side analysis (coloring, permutation, ILU0 factors) matches the
oracle bit for bit. Host-only handles (device = -1) make no CUDA call."""
import ctypes
import os

import numpy as np
import pytest

from fpga_gb300 import GbIlu, GbIluError, native
from fpga_gb300.synth import generate, make_config
from oracle_lib import Prepared

CASES = {
    "c1": lambda: make_config("c1_20x20x10"),
    "faults": lambda: generate(30, 24, 12, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=7),
    "single": lambda: generate(1, 1, 1, seed=0),
    "line": lambda: generate(17, 1, 1, seed=1),
}


def test_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = native.declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name


@pytest.mark.parametrize("coloring", ["parity", "natural"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_host_analysis_matches_oracle(built_lib, name, coloring):
    s = CASES[name]()
    P = Prepared(s, coloring=coloring)
    with GbIlu(device=-1, coloring=coloring) as g:
        g.analyze(s.rowptr, s.colind).factor(s.vals)
        nc, color, perm, cp = g.ordering()
        assert nc == P.ncolors
        assert np.array_equal(color, P.color)
        assert np.array_equal(perm, P.perm)
        assert np.array_equal(cp, P.color_ptr)
        lu, dinv = g.factors()
        assert np.array_equal(lu, P.lu)
        assert np.array_equal(dinv, P.dinv)
        st = g.stats()
        assert st["nnzb_lower"] + st["nnzb_upper"] + st["nb"] == st["nnzb"]
        assert st["slots_a"] * 32 >= st["nnzb"]


def expect(code, fn, *a):
    with pytest.raises(GbIluError) as e:
        fn(*a)
    assert e.value.code == code, str(e.value)


def test_error_behaviour(built_lib):
    s = make_config("c1_20x20x10")
    with GbIlu(device=-1) as g:
        expect(native.NOT_READY, g.factor, s.vals)            # factor before analyze
        bad = s.colind.copy()
        bad[[0, 1]] = bad[[1, 0]]                              # unsorted row 0
        expect(native.BAD_INPUT, g.analyze, s.rowptr, bad)
        bad = s.colind.copy()
        bad[5] = s.nb + 3                                      # out of range
        expect(native.BAD_INPUT, g.analyze, s.rowptr, bad)
        rp = s.rowptr.copy()
        rp[0] = 1
        expect(native.BAD_INPUT, g.analyze, rp, s.colind)
        # a row without its diagonal block
        keep = np.ones(s.nnzb, bool)
        keep[np.nonzero(s.colind[s.rowptr[3]:s.rowptr[4]] == 3)[0][0] + s.rowptr[3]] = False
        rp = np.concatenate([[0], np.cumsum([keep[s.rowptr[i]:s.rowptr[i + 1]].sum() for i in range(s.nb)])])
        expect(native.BAD_INPUT, g.analyze, rp, s.colind[keep])
        # a structurally nonsymmetric pattern: row 3 loses one off-diagonal
        # block whose transpose stays
        keep = np.ones(s.nnzb, bool)
        off = [k for k in range(s.rowptr[3], s.rowptr[4]) if s.colind[k] != 3]
        keep[off[0]] = False
        rp = np.concatenate([[0], np.cumsum([keep[s.rowptr[i]:s.rowptr[i + 1]].sum() for i in range(s.nb)])])
        with pytest.raises(GbIluError, match="structurally symmetric"):
            g.analyze(rp.astype(np.int32), s.colind[keep])
        # empty system; a block-row count whose vector indices overflow int
        # (rejected before the arrays are read)
        with pytest.raises(GbIluError, match="nb must be positive"):
            g.analyze(np.zeros(1, np.int32), np.zeros(0, np.int32))
        rp1, ci1 = np.zeros(2, np.int32), np.zeros(1, np.int32)
        assert g.L.gbilu_analyze(g.h, 2**31 // 9 + 1, rp1, ci1) == native.BAD_INPUT
        assert "nb too large" in g.L.gbilu_last_error(g.h).decode()
        g.analyze(s.rowptr, s.colind)
        vals = s.vals.copy()
        d = np.nonzero(s.colind[s.rowptr[10]:s.rowptr[11]] == 10)[0][0] + s.rowptr[10]
        vals[d] = 0.0                                          # singular pivot
        expect(native.SINGULAR, g.factor, vals)
        g.factor(s.vals)
        expect(native.NO_DEVICE, g.solve, s.b)                 # host-only handle


def test_status_strings(built_lib):
    for code in range(11):
        assert native.status_string(code) != "unknown status"


def random_symmetric(nb, density, seed):
    """A random structurally symmetric pattern with the diagonal."""
    rng = np.random.default_rng(seed)
    m = rng.random((nb, nb)) < density
    m = m | m.T | np.eye(nb, dtype=bool)
    rowptr = np.concatenate([[0], np.cumsum(m.sum(1))]).astype(np.int32)
    colind = np.concatenate([np.flatnonzero(r) for r in m]).astype(np.int32)
    return nb, rowptr, colind


@pytest.mark.parametrize("seed", range(6))
def test_parity_coloring_general_patterns(built_lib, seed):
    """The parity-order coloring on patterns that are not grids (random
    symmetric, from sparse to dense): a valid coloring, identical to the
    oracle's separate implementation."""
    nb, rowptr, colind = random_symmetric(40 + 30 * seed, [0.01, 0.03, 0.1, 0.3, 0.02, 0.05][seed],
                                          seed)
    L = __import__("oracle_lib").lib()
    ref = np.empty(nb, np.int32)
    nref = L.orc_color_parity(nb, rowptr, colind, ref)
    with GbIlu(device=-1) as g:
        g.analyze(rowptr, colind)
        nc, color, perm, cp = g.ordering()
    assert nc == nref and np.array_equal(color, ref)
    rows = np.repeat(np.arange(nb), np.diff(rowptr))
    off = rows != colind
    assert not np.any(color[rows[off]] == color[colind[off]])


def test_parity_coloring_grid_with_faults(built_lib):
    """On the 500k-cell system with fault connections the parity order
    leaves two large colors and one small one; natural order gives five."""
    s = make_config("c2_100x100x50")
    with GbIlu(device=-1) as g:
        g.analyze(s.rowptr, s.colind)
        nc, _, _, cp = g.ordering()
    with GbIlu(device=-1, coloring="natural") as g:
        g.analyze(s.rowptr, s.colind)
        nc_nat = g.ordering()[0]
    sizes = np.diff(cp)
    assert nc == 3 and nc_nat == 5
    assert sizes[2] < 0.01 * s.nb
