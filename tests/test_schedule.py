"""The step schedule of the single-launch ILU apply (gbilu_schedule), checked
on the CPU against the sparsity pattern: every value a step reads was written
in an earlier barrier interval (steps that share an interval are
independent; a CTA barrier between two single-slice steps on one CTA, and
the data ordering of consecutive small steps, count as boundaries), every z
row is written exactly once, every y row at most
once.
Runs on host-only handles (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from fpga_gb300 import GbIlu
from fpga_gb300.synth import generate, make_config

def _dense(nb):
    """Every block row coupled to every other: nb colors, more steps than the
    single-launch apply's fixed list holds (the per-step path)."""
    from fpga_gb300.synth import BlockSystem
    rowptr = (np.arange(nb + 1) * nb).astype(np.int32)
    colind = np.tile(np.arange(nb, dtype=np.int32), nb)
    vals = np.zeros((nb * nb, 3, 3))
    return BlockSystem(nb=nb, rowptr=rowptr, colind=colind, vals=vals, b=np.zeros(3 * nb),
                       cell_of_row=np.arange(nb), grid=(nb, 1, 1))


def _random_pattern(seed):
    """A random symmetric block pattern with its diagonal: from sparse chains
    to dense clusters (many colors)."""
    from fpga_gb300.synth import BlockSystem
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(1, 160))
    p = float(rng.choice([0.0, 0.01, 0.05, 0.3, 0.9]))
    m = rng.random((nb, nb)) < p
    m = m | m.T | np.eye(nb, dtype=bool)
    rows, cols = np.nonzero(m)
    rowptr = np.zeros(nb + 1, np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return BlockSystem(nb=nb, rowptr=rowptr, colind=cols.astype(np.int32),
                       vals=np.zeros((len(cols), 3, 3)), b=np.zeros(3 * nb),
                       cell_of_row=np.arange(nb), grid=(nb, 1, 1))


CASES = {
    "dense60": lambda: _dense(60),
    **{f"random{k}": (lambda k=k: _random_pattern(k)) for k in range(12)},
    "c1": lambda: make_config("c1_20x20x10"),
    "faults": lambda: generate(30, 24, 12, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=7),
    "mid": lambda: generate(60, 60, 20, sigma=1.5, inactive_frac=0.05, fault_frac=0.01, seed=5),
    "sigma2": lambda: generate(40, 40, 16, sigma=2.0, inactive_frac=0.05, fault_frac=0.02, seed=3),
}


def permuted_pattern(s, perm):
    nb = s.nb
    A = sp.csr_matrix((np.ones(len(s.colind)), s.colind, s.rowptr), shape=(nb, nb))
    P = A[perm][:, perm].tocsr()
    P.sort_indices()
    return P


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("transpose", [False, True])
def test_schedule_dependencies(built_lib, name, transpose):
    s = CASES[name]()
    g = GbIlu(device=-1)
    g.analyze(s.rowptr, s.colind)
    P = permuted_pattern(s, g.device_order())   # the numbering the steps use
    low, up = sp.tril(P, -1).tocsr(), sp.triu(P, 1).tocsr()
    if transpose:   # U^T and L^T rows: the pattern's columns, transposed
        first, second = up.T.tocsr(), low.T.tocsr()
    else:
        first, second = low, up
    nb = s.nb
    wy = np.full(nb, -1)
    wh = np.full(nb, -1)
    steps = g.schedule(transpose)
    assert steps and steps[-1]["barrier_after"] in (0, 1)
    # a CTA barrier (2) only links two single-slice steps (both run on CTA 0),
    # so it orders them like a grid barrier would
    # and no barrier (3) links two small steps, whose consumers wait for each
    # value they read: every kind orders the steps
    for st, nxt in zip(steps, steps[1:]):
        if st["barrier_after"] == 2:
            assert st["nrows"] <= 32 and nxt["nrows"] <= 32
            assert st["lane0"] == 0 and nxt["lane0"] == 0
        if st["barrier_after"] == 3:
            assert st["nrows"] <= 16384 and nxt["nrows"] <= 16384
    k = 0
    pend_y, pend_h = [], []
    for st in steps:
        rows = np.arange(st["row0"], st["row0"] + st["nrows"])
        M = second if st["mat"] else first
        sub = M[rows]
        cols = sub.indices
        # own values
        if st["own_y"]:
            assert np.all((wy[rows] >= 0) & (wy[rows] < k)), "own y not ready"
        # neighbours
        from_src = cols < st["src_rows"]
        c = cols[~from_src]
        w = wh[c] if st["nbr_hat"] else wy[c]
        assert np.all((w >= 0) & (w < k)), "neighbour not ready"
        # writes
        if st["to_y"]:
            pend_y.append(rows)
            fin = rows[rows >= st["final0"]]
            pend_h.append(fin)
        else:
            pend_h.append(rows)
        if st["barrier_after"]:
            for r in pend_y:
                assert np.all(wy[r] == -1), "y written twice"
                wy[r] = k
            for r in pend_h:
                assert np.all(wh[r] == -1), "z written twice"
                wh[r] = k
            pend_y, pend_h = [], []
            k += 1
    for r in pend_y:
        assert np.all(wy[r] == -1)
        wy[r] = k
    for r in pend_h:
        assert np.all(wh[r] == -1)
        wh[r] = k
    assert np.all(wh >= 0), "rows without a final value"
    # slice0 / lane0 agree with the layout: a color's slices hold 32
    # consecutive rows from the color's first row on
    _, _, _, cp = g.ordering()
    base = {}
    for st in steps:
        assert 0 <= st["lane0"] < 32
        c = int(np.searchsorted(cp, st["row0"], side="right") - 1)
        off = st["slice0"] * 32 + st["lane0"] - st["row0"]
        assert base.setdefault(c, off) == off
        assert (st["row0"] - cp[c]) % 32 == st["lane0"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_order(built_lib, name):
    """The device numbering permutes rows only inside each color's run of
    split rows and inside its run of other rows, with block counts
    descending in every run."""
    s = CASES[name]()
    g = GbIlu(device=-1)
    g.analyze(s.rowptr, s.colind)
    nc, color, perm, cp = g.ordering()
    order = g.device_order()
    iperm = np.empty(s.nb, np.int64)
    iperm[perm] = np.arange(s.nb)
    width = np.diff(s.rowptr)
    # split run of each color: the rows the permuted order puts first
    A = sp.csr_matrix((np.ones(len(s.colind)), s.colind, s.rowptr), shape=(s.nb, s.nb)).tocoo()
    higher = np.zeros(s.nb, bool)
    higher[A.row[color[A.col] > color[A.row]]] = True
    higher[A.col[color[A.row] > color[A.col]]] = True
    for c in range(nc):
        a, b = cp[c], cp[c + 1]
        k = a + int(higher[perm[a:b]].sum())
        for lo, hi in ((a, k), (k, b)):
            assert sorted(order[lo:hi]) == sorted(perm[lo:hi])
            w = width[order[lo:hi]]
            assert np.all(np.diff(w) <= 0)
            # ties keep the permuted order
            pos = iperm[order[lo:hi]]
            same = np.diff(w) == 0
            assert np.all(np.diff(pos)[same] > 0)
