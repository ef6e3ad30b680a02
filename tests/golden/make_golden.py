"""Regenerates the golden fixtures of the CPU oracle (tests/golden/*.npz).

Each fixture stores a small seeded system (generator parameters and the
generated arrays) with the oracle's outputs on it: coloring, permutation
(with the split of each color; parity-order coloring, and once the
natural-order one),
ILU0 factors, one SpMV and one ILU apply of a probe vector, and a solve
(half-iteration count and solution). test_oracle.py checks that the oracle
reproduces them bit for bit. The oracle is compiled with -ffp-contract=off
and uses only IEEE-exact operations, so the bits do not depend on the host.

Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from fpga_gb300.synth import generate  # noqa: E402
from oracle_lib import Prepared  # noqa: E402

CASES = {
    "golden_small.npz": dict(grid=(8, 6, 4), sigma=1.0, inactive=0.0, faults=0.0, seed=0, tol=1e-6,
                             coloring="parity"),
    "golden_faults.npz": dict(grid=(12, 10, 5), sigma=1.5, inactive=0.05, faults=0.02, seed=3,
                              tol=1e-4, coloring="parity"),
    "golden_faults_natural.npz": dict(grid=(12, 10, 5), sigma=1.5, inactive=0.05, faults=0.02,
                                      seed=3, tol=1e-4, coloring="natural"),
}

if __name__ == "__main__":
    for name, c in CASES.items():
        s = generate(*c["grid"], sigma=c["sigma"], inactive_frac=c["inactive"],
                     fault_frac=c["faults"], seed=c["seed"])
        P = Prepared(s, coloring=c["coloring"])
        xp = np.random.default_rng(100).standard_normal(s.n)
        x, r = P.solve(s.b, tol=c["tol"], maxit=500)
        np.savez_compressed(
            os.path.join(HERE, name), grid=np.array(c["grid"]), sigma=c["sigma"],
            inactive=c["inactive"], faults=c["faults"], seed=c["seed"], tol=c["tol"],
            coloring=c["coloring"],
            rowptr=s.rowptr, colind=s.colind, vals=s.vals.reshape(-1), b=s.b,
            ncolors=P.ncolors, color=P.color, perm=P.perm, split=P.split, lu=P.lu, dinv=P.dinv,
            x_probe=xp, spmv=P.spmv(xp), ilu=P.ilu_apply(xp), spmv_t=P.spmv(xp, True),
            ilu_t=P.ilu_apply(xp, True), half_iters=r.half_iters, x=x)
        print(name, s.nb, P.ncolors, r.half_iters)
