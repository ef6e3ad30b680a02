"""Seeded synthetic reservoir-like 3x3-block BSR systems.

The reference is benchmarked on linear systems that the Flow simulator hands to
the FPGA backend (README.md:7-11); no such matrices ship with it, so this module
generates stand-ins with the same structure: a structured nx*ny*nz grid of cells
with a 7-point stencil, 3 unknowns per cell, lognormal transmissibilities,
optionally inactive cells and fault-like extra connections inside a k-layer.

Draw order with ``numpy.random.default_rng(seed)`` (fixed, so every machine
produces the same bytes):

1. inactive cells: ``rng.choice(ncells, n_inactive, replace=False)``;
2. fault connections: ``n_faults`` pairs, each drawn as two cell indices in
   one k-layer (``rng.integers``), redrawn until both are active, distinct,
   not face neighbours and not already connected;
3. one transmissibility exponent per undirected connection
   (``rng.standard_normal(E)``), ``t = exp(sigma * z)``;
4. two 3x3 standard-normal matrices per connection
   (``rng.standard_normal((E, 2, 3, 3))``): block (i, j) = -t*(0.1*R0 + I),
   block (j, i) = -t*(0.1*R1 + I), i < j;
5. the right-hand side ``rng.standard_normal(3 * nb)``.

The diagonal block of every row is the negated sum of its off-diagonal blocks
plus 0.5*I (an accumulation term). Off-diagonal blocks carry the sign of a
reservoir flow Jacobian (coupling -t, so the diagonal is +sum(t) + 0.5): with
``offdiag_sign=+1`` the off-diagonals are +t*(0.1*R + I) and the matrix is
0.5*I minus a weighted graph Laplacian, which is indefinite; ILU0-BiCGSTAB
does not reach a relative residual of 1e-2 on it within 400 iterations, so
the default is ``offdiag_sign=-1``.
Connections are ordered x-faces, y-faces, z-faces (each in natural cell order)
followed by the fault connections.
"""
from __future__ import annotations

import dataclasses
import numpy as np


@dataclasses.dataclass
class BlockSystem:
    """A 3x3-block BSR matrix plus right-hand side.

    rowptr[nb+1] (int32), colind[nnzb] (int32, sorted within each row, diagonal
    included), vals[nnzb, 3, 3] (float64, row-major blocks), b[3*nb] (float64).
    cell_of_row maps each block row to its grid cell (inactive cells removed).
    """
    nb: int
    rowptr: np.ndarray
    colind: np.ndarray
    vals: np.ndarray
    b: np.ndarray
    cell_of_row: np.ndarray
    grid: tuple

    @property
    def n(self) -> int:
        return 3 * self.nb

    @property
    def nnzb(self) -> int:
        return int(self.rowptr[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.bsr_matrix((self.vals, self.colind, self.rowptr),
                             shape=(self.n, self.n)).tocsr()

    def dense(self) -> np.ndarray:
        a = np.zeros((self.n, self.n))
        for i in range(self.nb):
            for k in range(self.rowptr[i], self.rowptr[i + 1]):
                j = self.colind[k]
                a[3 * i:3 * i + 3, 3 * j:3 * j + 3] = self.vals[k]
        return a


def _face_pairs(nx, ny, nz):
    idx = np.arange(nx * ny * nz).reshape(nz, ny, nx)
    out = []
    out.append(np.stack([idx[:, :, :-1].ravel(), idx[:, :, 1:].ravel()], 1))
    out.append(np.stack([idx[:, :-1, :].ravel(), idx[:, 1:, :].ravel()], 1))
    out.append(np.stack([idx[:-1, :, :].ravel(), idx[1:, :, :].ravel()], 1))
    return out


def generate(nx: int, ny: int, nz: int, sigma: float = 1.0,
             inactive_frac: float = 0.0, fault_frac: float = 0.0,
             seed: int = 0, offdiag_sign: float = -1.0) -> BlockSystem:
    """Build one synthetic system (see the module docstring for the recipe)."""
    rng = np.random.default_rng(seed)
    ncells = nx * ny * nz
    active = np.ones(ncells, dtype=bool)
    n_inactive = int(round(inactive_frac * ncells))
    if n_inactive:
        active[rng.choice(ncells, n_inactive, replace=False)] = False
    new_id = np.full(ncells, -1, dtype=np.int64)
    cell_of_row = np.nonzero(active)[0]
    nb = cell_of_row.size
    new_id[cell_of_row] = np.arange(nb)

    pairs = []
    for fp in _face_pairs(nx, ny, nz):
        keep = active[fp[:, 0]] & active[fp[:, 1]]
        pairs.append(fp[keep])
    faces = np.concatenate(pairs, 0)

    n_faults = int(round(fault_frac * nb))
    fault = np.zeros((0, 2), dtype=np.int64)
    if n_faults:
        existing = set(map(tuple, np.sort(faces, 1).tolist()))
        layer = nx * ny
        got = []
        while len(got) < n_faults:
            k = int(rng.integers(nz))
            a, c = (int(v) + k * layer for v in rng.integers(layer, size=2))
            if a == c or not (active[a] and active[c]):
                continue
            lo, hi = min(a, c), max(a, c)
            d = hi - lo
            if d == 1 and lo % nx != nx - 1 or d == nx:
                continue            # a face neighbour already
            if (lo, hi) in existing:
                continue
            existing.add((lo, hi))
            got.append((lo, hi))
        fault = np.array(got, dtype=np.int64)
    edges = np.concatenate([faces, fault], 0)
    ei, ej = new_id[edges[:, 0]], new_id[edges[:, 1]]
    E = edges.shape[0]

    t = np.exp(sigma * rng.standard_normal(E))
    R = rng.standard_normal((E, 2, 3, 3))
    eye = np.eye(3)
    blk_ij = offdiag_sign * t[:, None, None] * (0.1 * R[:, 0] + eye)
    blk_ji = offdiag_sign * t[:, None, None] * (0.1 * R[:, 1] + eye)
    b = rng.standard_normal(3 * nb)

    rows = np.concatenate([ei, ej, np.arange(nb)])
    cols = np.concatenate([ej, ei, np.arange(nb)])
    diag = 0.5 * np.broadcast_to(eye, (nb, 3, 3)).copy()
    np.subtract.at(diag, ei, blk_ij)
    np.subtract.at(diag, ej, blk_ji)
    blocks = np.concatenate([blk_ij, blk_ji, diag], 0)
    order = np.lexsort((cols, rows))
    rows, cols, blocks = rows[order], cols[order], blocks[order]
    rowptr = np.zeros(nb + 1, dtype=np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return BlockSystem(nb=nb, rowptr=rowptr, colind=cols.astype(np.int32),
                       vals=np.ascontiguousarray(blocks), b=b,
                       cell_of_row=cell_of_row.astype(np.int64),
                       grid=(nx, ny, nz))


# The five workloads the solver is measured on (grid, sigma, inactive and
# fault fractions, stopping tolerance).
CONFIGS = {
    "c1_20x20x10": dict(grid=(20, 20, 10), sigma=1.0, inactive=0.0, faults=0.0, tol=1e-2, maxit=200),
    "c2_100x100x50": dict(grid=(100, 100, 50), sigma=1.5, inactive=0.05, faults=0.01, tol=1e-2, maxit=1000),
    "c3_100x100x50_mixed": dict(grid=(100, 100, 50), sigma=2.0, inactive=0.05, faults=0.01, tol=1e-8, maxit=2000),
    "c4_60x60x30_adjoint": dict(grid=(60, 60, 30), sigma=1.0, inactive=0.0, faults=0.0, tol=1e-10, maxit=2000),
    "c5_200x200x50_mixed_adjoint": dict(grid=(200, 200, 50), sigma=1.5, inactive=0.05, faults=0.01, tol=1e-8, maxit=2000),
}


def make_config(name: str, seed: int = 0) -> BlockSystem:
    c = CONFIGS[name]
    return generate(*c["grid"], sigma=c["sigma"], inactive_frac=c["inactive"],
                    fault_frac=c["faults"], seed=seed)


def adjoint_selection(nb: int, frac: float = 0.01, seed: int = 1):
    """W (cells picked, sorted) and data d for L = 0.5*||W x - d||^2."""
    rng = np.random.default_rng(seed)
    m = max(1, int(round(frac * nb)))
    cells = np.sort(rng.choice(nb, m, replace=False))
    d = rng.standard_normal(3 * m)
    return cells, d
